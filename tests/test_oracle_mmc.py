"""The CPU MiniMC engine of the oracle (oracle/ncgb_oracle_mmc.c) against the
reference's own MiniMC, run live on the queries of tests/golden/mmc_*.npz
with the same (smaller) number of histories on both sides, every tally
histogram compared by a two-sample chi-square (the criteria of the device
engine's tests).  Equal sample sizes matter: some tallies are dominated by
rare heavy-weight events (a first collision near the exit, then a small-angle
scatter), whose sums a smaller sample underestimates.  Pins the CPU engine
that bench.py times as the MiniMC workload's CPU baseline."""
import ctypes
import os

import numpy as np
import pytest

import ncrystal_gb300.minimc as M
from conftest import bundle_path
from mmc_stats import GROUPS, chi2_compare, hist_from_result
from oracle import pyoracle as P
from ncrystal_gb300.bundle.reader import read_bundle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
WL2E = 0.081804209605330899


def test_cfg_struct_layout_matches_c():
    L = P.oracle_lib()
    L.ncgb_oracle_mmc_cfg_size.restype = ctypes.c_int64
    assert L.ncgb_oracle_mmc_cfg_size() == ctypes.sizeof(P.OraMmcCfg)


def _energy(srccfg):
    for part in srccfg.split(";"):
        if part.startswith("ekin="):
            return float(part[5:])
        if part.startswith("wl="):
            return WL2E / float(part[3:]) ** 2
    raise ValueError(srccfg)


@pytest.mark.parametrize("name,nhist", [("mmc_pe_sphere", 300000), ("mmc_al_default", 300000),
                                        ("mmc_water_slab", 300000), ("mmc_pe_cyl", 300000)])
def test_oracle_mmc_matches_reference(name, nhist):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    q = str(g["query"]).split("\x07")
    cfg, enginecfg = q[2], q[-1]
    geomcfg, srccfg = str(g["geomcfg"]), str(g["srccfg"])
    path = bundle_path(cfg)
    geom = M.decode_cfgstr(geomcfg, "geom")["decoded"]
    src = M.decode_cfgstr(srccfg, "src")["decoded"]
    src["energy_ev"] = _energy(srccfg)
    eng = M.decode_cfgstr(enginecfg, "engine")["decoded"]
    tallies = sorted({k.split(".")[0] for k in g.files if k.endswith(".total.content")})
    binnings = {t: (int(g["%s.total.range" % t][2]), g["%s.total.range" % t][0], g["%s.total.range" % t][1])
                for t in tallies}
    srcn = ";".join(p for p in srccfg.split(";") if not p.startswith("n=")) + ";n=%d" % nhist
    ref = P.reference_mmc(["mmc", "run", cfg, geomcfg, srcn, enginecfg])
    if ref is None:
        pytest.skip("the reference library is not built here")
    m = P.HostMaterial(path)
    c, nstat, nbuf = P.mmc_config(m, read_bundle(path), geom, src, eng, binnings, seed=7)
    buf, cnt = P.mmc_run(m, c, nbuf, 0, nhist, threads=os.cpu_count() or 1)
    assert cnt[4] == 0
    n_ref = nhist
    md = ref["output"]["metadata"]
    comps = []
    for t in tallies:
        for part in ["total"] + GROUPS:
            if part != "total" and part not in ref["output"]["tally"][t]["breakdown"]:
                continue
            rc, re_, rng = hist_from_result(ref, t, part)
            assert rng[2] == binnings[t][0]
            oc, oe = P.mmc_hist(c, buf, t, part)
            x, ndf, p, worst = chi2_compare(rc, re_, n_ref, oc, oe, nhist)
            assert len(worst) == 0, (t, part, worst)
            comps.append((p, t, part, x, ndf))
    pmin = min(cc[0] for cc in comps)
    msg = "; ".join("%s/%s chi2=%.1f ndf=%d p=%.2e" % (t, part, x, ndf, p) for p, t, part, x, ndf in sorted(comps)[:4])
    assert pmin > 1e-3 / len(comps), msg
    # misses and tallied weight per history
    pm = md["miss"]["count"] / n_ref
    assert abs(cnt[2] / nhist - pm) < 5 * np.sqrt(2 * pm * (1 - pm) / nhist) + 1e-12
    assert abs(cnt[1] / nhist - md["tallied"]["weight"] / n_ref) < 5e-3
