"""Generates tests/golden/mmc_*.npz: MiniMC results of the reference NCrystal
library itself (oracle/_ref/libNCrystal.so, built from the NCrystal sources by
oracle/ref.mk), through its C entry point ncrystal_jsonquery with
["mmc","run",...] queries (ncrystal.cc:2463-2473, NCMMC_Query.cc:60-100).

Each fixture holds the query entries, the tallied histograms (content and
error^2 of the total and of each breakdown, under/overflow included) and the
metadata counts.  The device engine runs the same queries; its results are
compared statistically (different random streams).  mmc_scenarios.npz holds
the reference's own decoding of scenario strings (["mmc","scenario",...]).

Run from the repository root where the NCrystal sources exist:
    python tests/golden/make_mmc_golden.py
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import ncrystal_gb300._build as B  # noqa: E402
import ncrystal_gb300.workloads as W  # noqa: E402

GROUPS = ["NOSCAT", "SINGLESCAT_ELAS", "SINGLESCAT_INELAS", "MULTISCAT_PUREELAS", "MULTISCAT_OTHER"]

# name: (cfg, geomcfg, srccfg, enginecfg) -- or (cfg, scenario, enginecfg)
RUNS = {
    # polyethylene sphere, pencil beam at the thermal energy (S(alpha,beta), ElInc, absorption)
    "mmc_pe_sphere": (W.PE293, "sphere;r=0.01", "constant;ekin=0.0253;z=-0.01;n=1e7",
                      "seed=11;nthreads=8;tally=theta,mu,e,nscat,w"),
    # aluminium, the reference's default scenario (0.8 x Bragg threshold, circular beam on a 1 mfp sphere)
    "mmc_al_default": (W.AL, "1e7 times", "seed=12;nthreads=8;tally=theta,l,nscat_uw"),
    # water slab with an isotropic source inside (unbounded geometry, per-neutron reference directions,
    # free-gas oxygen)
    "mmc_water_slab": (W.WATER, "slab;dz=0.002", "isotropic;ekin=0.0253;n=1e7",
                       "seed=13;nthreads=8;tally=theta,mu,e,de"),
    # corundum box, log-normal wavelengths, single scattering only, reference = the source's means
    "mmc_al2o3_box": (W.AL2O3, "box;dx=0.01;dy=0.02;dz=0.005", "constant;wl=2+-0.3;z=-0.02;n=1e7",
                      "seed=14;nthreads=8;tally=theta,q,de,l;nscatlimit=1;tallyref=src;roulette=0.5,0.05,3"),
    # polyethylene cylinder hit by a wider circular beam from the side (propagation to the volume, misses)
    "mmc_pe_cyl": (W.PE293, "cyl;r=0.005;dy=0.02", "circular;x=-0.03;ux=1;uy=0;uz=0;r=0.008;ekin=0.1;n=1e7",
                   "seed=15;nthreads=8;tally=theta,nscat;absorption=0"),
}

SCENARIOS = [
    (W.AL, ""), (W.PE293, ""), (W.PE293, "1.8Aa on 1mfp sphere"), (W.AL, "2Aa pencil on 5mm sphere"),
    (W.WATER, "25meV on 2mm slab 1e5 times"), (W.AL2O3, "0.5BT"), (W.PE293, "1kT on 0.5mfp"),
    (W.AL, "0.05eV on 1cm"), (W.AL, "1e7 times"),
]


def _lib():
    path = os.path.join(B.REF_OUT, "libNCrystal.so")
    L = ctypes.CDLL(path)
    L.ncrystal_jsonquery.restype = ctypes.c_void_p
    L.ncrystal_jsonquery.argtypes = [ctypes.c_char_p]
    L.ncrystal_dealloc_string.argtypes = [ctypes.c_void_p]
    return L


def query(L, *entries):
    raw = L.ncrystal_jsonquery("\x07".join(entries).encode())
    if not raw:
        raise RuntimeError("reference query failed: %r" % (entries,))
    txt = ctypes.cast(raw, ctypes.c_char_p).value.decode()
    L.ncrystal_dealloc_string(raw)
    return json.loads(txt)


def flatten(res):
    out = {}
    for name, t in res["output"]["tally"].items():
        parts = [("total", t["total"])] + [(g, t["breakdown"][g]) for g in GROUPS if g in t["breakdown"]]
        for part, h in parts:
            b = h["bindata"]
            key = "%s.%s" % (name, part)
            out[key + ".content"] = np.array([b["underflow"]] + b["content"] + [b["overflow"]])
            out[key + ".errorsq"] = np.array([b["underflow_errorsq"]] + b["errorsq"] + [b["overflow_errorsq"]])
            out[key + ".range"] = np.array([b["xmin"], b["xmax"], b["nbins"]], dtype=float)
            s = h["stats"]
            out[key + ".stats"] = np.array([s["integral"]] + [np.nan if s[k] is None else s[k]
                                                               for k in ("mean", "rms", "minfilled", "maxfilled")])
    md = res["output"]["metadata"]
    for k in ("provided", "miss", "tallied"):
        out["meta.%s" % k] = np.array([md[k]["count"], md[k]["weight"]], dtype=float)
    return out


def main():
    B.build_reference()
    L = _lib()
    os.environ.setdefault("NCRYSTAL_FACTORY_THREADS", "1")
    for name, spec in RUNS.items():
        entries = ["mmc", "run"] + list(spec)
        res = query(L, *entries)
        data = flatten(res)
        data["query"] = np.array("\x07".join(entries))
        data["geomcfg"] = np.array(res["input"]["geom"]["cfgstr"])
        data["srccfg"] = np.array(res["input"]["src"]["cfgstr"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, res["output"]["metadata"])
    sc = []
    for cfg, scen in SCENARIOS:
        d = query(L, "mmc", "scenario", cfg, scen)
        sc.append((cfg, scen, d["geomcfg"], d["srccfg"]))
        print(cfg, repr(scen), d)
    np.savez_compressed(os.path.join(HERE, "mmc_scenarios.npz"), rows=np.array(sc))


if __name__ == "__main__":
    main()
