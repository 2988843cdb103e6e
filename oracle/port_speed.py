"""Single-thread speed of the CPU oracle against the reference NCrystal library
itself, on the same host and the same energies: cross-section plus one
isotropic scatter per neutron.  TEST INFRASTRUCTURE: it tells whether the
oracle, which stands in for NCrystal as the timed CPU baseline where the
reference cannot be built, is a fair stand-in.

Reference side: NCrystal's own batched C entry points
(ncrystal_crosssection_nonoriented_many, ncrystal_samplescatterisotropic_many,
ncrystal.cc:1107-1141, :1201-1245) on a handle with its built-in generator,
from the reference build in oracle/_ref/ (needs the NCrystal sources).
Oracle side: ncgb_oracle_xs_many + ncgb_oracle_scatter_many on the same
energies.  Each timing is the best of three runs.

    python -m oracle.port_speed [n]
"""
import ctypes as C
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


class _H(C.Structure):
    _fields_ = [("internal", C.c_void_p)]


def _reference_lib():
    import ncrystal_gb300._build as B
    L = C.CDLL(os.path.join(B.REF_OUT, "libNCrystal.so"))
    L.ncrystal_create_scatter_builtinrng.restype = _H
    L.ncrystal_create_scatter_builtinrng.argtypes = [C.c_char_p, C.c_ulong]
    L.ncrystal_cast_scat2proc.restype = _H
    L.ncrystal_cast_scat2proc.argtypes = [_H]
    L.ncrystal_crosssection_nonoriented_many.argtypes = [_H, C.c_void_p, C.c_ulong, C.c_ulong, C.c_void_p]
    L.ncrystal_samplescatterisotropic_many.argtypes = [_H, C.c_void_p, C.c_ulong, C.c_ulong, C.c_void_p,
                                                       C.c_void_p]
    return L


def _best(fn, reps=3):
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best


def compare(cfg, e, seed=1234):
    """-> (reference scatters/s, oracle scatters/s) on one thread."""
    import ncrystal_gb300._build as B
    from oracle.pyoracle import HostMaterial
    L = _reference_lib()
    e = np.ascontiguousarray(e, dtype=np.float64)
    n = len(e)
    sc = L.ncrystal_create_scatter_builtinrng(cfg.encode(), seed)
    pr = L.ncrystal_cast_scat2proc(sc)
    xs, ef, mu = np.empty(n), np.empty(n), np.empty(n)
    P = (lambda a: a.ctypes.data_as(C.c_void_p))

    def ref():
        L.ncrystal_crosssection_nonoriented_many(pr, P(e), n, 1, P(xs))
        L.ncrystal_samplescatterisotropic_many(sc, P(e), n, 1, P(ef), P(mu))
    m = HostMaterial(os.path.join(B.BUNDLES, B.bundle_file_name(cfg)))

    def ora():
        m.xs(e)
        m.scatter(e, seed)
    return n / _best(ref), n / _best(ora)


def main(n=1 << 20):
    import ncrystal_gb300.workloads as W
    cases = [(W.AL, W.al_wavelength_energies(n, 0x5EED0001)),
             (W.AL2O3, W.loguniform_energies(n, 1e-4, 1.0, 0x5EED0002)),
             (W.PE293, W.loguniform_energies(n, 1e-4, 1.0, 0x5EED0004))]
    print("| material | NCrystal (scatters/s, 1 thread) | oracle | oracle / NCrystal |")
    print("|---|---|---|---|")
    for cfg, e in cases:
        r, o = compare(cfg, e)
        print("| %s | %.3g | %.3g | %.2f |" % (cfg, r, o, o / r))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 1 << 20)
