"""Generates the golden fixtures tests/golden/*.npz from the reference NCrystal
library itself (oracle/_ref, built from the NCrystal sources by oracle/ref.mk).

For each material, the reference's own ncrystal_crosssection_nonoriented and
ncrystal_samplescatterisotropic are run on seeded energies, with the random
source replaced by the per-neutron Philox streams of include/ncgb_philox.h
(oracle/refpin.c).  The fixture holds, per neutron: E, the cross-section, E',
mu, the number of random numbers the reference consumed and whether it raised
an error.  Neutron i uses stream (SEED, i, 0, 0).

dir_*.npz: the same for the reference's ncrystal_samplescatter (scatters with
incoming and outgoing directions).  abs_xs.npz: the reference's absorption
cross-sections (ncrystal_create_absorption) for several materials.

Run from the repository root where the NCrystal sources exist:
    python tests/golden/make_golden.py [--dirs-only | --abs-only]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import ncrystal_gb300._build as B  # noqa: E402
import ncrystal_gb300.workloads as W  # noqa: E402
from oracle import pyoracle  # noqa: E402
from ncrystal_gb300.bundle.reader import read_bundle  # noqa: E402

SEED = 0x5EEDF00D
N_RANDOM = 1500

GOLDEN = {
    "al": (W.AL, lambda n: W.al_wavelength_energies(n, 101)),
    "al2o3": (W.AL2O3, lambda n: W.loguniform_energies(n, 1e-4, 1.0, 102)),
    "pe293": (W.PE293, lambda n: W.loguniform_energies(n, 1e-4, 1.0, 103)),
    "pe320": ("Polyethylene_CH2.ncmat;temp=320K", lambda n: W.loguniform_energies(n, 1e-5, 2.0, 104)),
    "water": (W.WATER, lambda n: W.loguniform_energies(n, 1e-5, 2.0, 105)),
    "cu77": ("Cu_sg225.ncmat;temp=77K", lambda n: W.loguniform_energies(n, 1e-4, 1.0, 106)),
    "zno400": ("ZnO_sg186_ZincOxide.ncmat;temp=400K", lambda n: W.loguniform_energies(n, 1e-4, 1.0, 107)),
    "kat_ni": ("Ni_sg225.ncmat;dcutoff=0.6;vdoslux=2", lambda n: W.loguniform_energies(n, 1e-4, 1.0, 108)),
    # above the S(alpha,beta) grids' Emax (free-gas extender) and free-gas O in water
    "al_highe": (W.AL, lambda n: W.loguniform_energies(n, 4.0, 60.0, 109)),
    "water_highe": (W.WATER, lambda n: W.loguniform_energies(n, 1e-3, 60.0, 110)),
}


# Scatters with directions (ncrystal_samplescatter): energies and directions
# per material; directions random, every other one not normalised.
DIR_GOLDEN = {
    "dir_al": (W.AL, 201),
    "dir_pe293": (W.PE293, 202),
    "dir_water": (W.WATER, 203),
    "dir_cu77": ("Cu_sg225.ncmat;temp=77K", 204),
}
N_DIR = 1000

# Absorption cross-sections (ncrystal_create_absorption).
ABS_CFGS = [W.AL, W.AL2O3, W.PE293, W.WATER, "Cu_sg225.ncmat;temp=77K",
            "ZnO_sg186_ZincOxide.ncmat;temp=400K", "Ni_sg225.ncmat;dcutoff=0.6;vdoslux=2"]


def dir_inputs(seed):
    rng = np.random.default_rng(seed)
    e = np.concatenate([W.loguniform_energies(N_DIR, 1e-5, 20.0, seed), [-1.0, 1e-300, 0.0253]])
    d = rng.normal(size=(len(e), 3))
    d[::2] /= np.linalg.norm(d[::2], axis=1)[:, None]
    return e, d


def edge_energies(bundle):
    """Energies on and next to table edges: Bragg thresholds and plane edges,
    SAB energy-grid points, Emax, and a few extremes."""
    e = [1e-12, 1e-9, 1e-7, 1e-6]
    for ic in range(int(bundle["ncomp"][0])):
        p = "c%d." % ic
        t = bundle[p + "type"]
        if t == "PowderBragg":
            a = bundle[p + "two_dE"]
            for x in list(a[:6]) + list(a[-3:]):
                e += [x, np.nextafter(x, 0.0), np.nextafter(x, np.inf)]
        elif t == "SABScatter":
            g = bundle[p + "egrid"]
            for x in list(g[:3]) + list(g[::37]) + list(g[-3:]):
                e += [x, np.nextafter(x, 0.0), np.nextafter(x, np.inf), x * 1.05, x / 1.05]
    return np.array([x for x in e if x > 0], dtype=np.float64)


def main():
    if not B.build_reference():
        sys.exit("the NCrystal sources are needed to generate golden fixtures")
    B.build_library()
    cfgs = [c for c, _ in GOLDEN.values()]
    paths = B.export_bundles(cfgs)
    only = [a for a in sys.argv[1:] if a.endswith("-only")]
    for key, (cfg, gen) in ([] if only else GOLDEN.items()):
        b = read_bundle(paths[cfg])
        ekin = np.concatenate([gen(N_RANDOM), edge_energies(b)])
        r = pyoracle.reference_run(cfg, ekin, SEED)
        out = os.path.join(HERE, key + ".npz")
        np.savez_compressed(out, cfg=np.array(cfg), seed=np.array(SEED, dtype=np.uint64), ekin=ekin,
                            xs=r["xs"], ekin_final=r["ekin_final"], mu=r["mu"], ndraws=r["ndraws"],
                            status=r["status"])
        print("%-8s %-55s n=%d errors=%d -> %s" % (key, cfg, len(ekin), int(r["status"].sum()), out))
    B.export_bundles([c for c, _ in DIR_GOLDEN.values()])
    for key, (cfg, seed) in (DIR_GOLDEN.items() if not only or "--dirs-only" in only else []):
        e, d = dir_inputs(seed)
        r = pyoracle.reference_run_dir(cfg, e, d, SEED)
        out = os.path.join(HERE, key + ".npz")
        np.savez_compressed(out, cfg=np.array(cfg), seed=np.array(SEED, dtype=np.uint64), ekin=e, direction=d,
                            ekin_final=r["ekin_final"], direction_final=r["direction"], ndraws=r["ndraws"],
                            status=r["status"])
        print("%-10s %-45s n=%d errors=%d -> %s" % (key, cfg, len(e), int(r["status"].sum()), out))
    if not only or "--abs-only" in only:
        B.export_bundles(ABS_CFGS)
        e = np.concatenate([W.loguniform_energies(500, 1e-6, 100.0, 301), [0.0, 1e-300, 0.0253, 1e10]])
        xs = np.stack([pyoracle.reference_abs_xs(c, e) for c in ABS_CFGS])
        out = os.path.join(HERE, "abs_xs.npz")
        np.savez_compressed(out, cfgs=np.array(ABS_CFGS), ekin=e, xs=xs)
        print("abs_xs %d materials x %d energies -> %s" % (len(ABS_CFGS), len(e), out))


if __name__ == "__main__":
    main()
