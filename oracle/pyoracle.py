"""ctypes wrapper of the CPU oracle (oracle/ncgb_oracle.c) and of the
reference-driving harness (oracle/refpin.c).  TEST INFRASTRUCTURE ONLY: used by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to check and
time beside the GPU path; the library never imports it.

The oracle reads the flat tables built by the library's host-only table
loader (ncgb_tables_load), i.e. exactly the tables the kernels read.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
VIEW_BYTES = 1 << 16  # >= sizeof(ncgb_material_view)

_ora = None
_refpin = None


def _P(a):
    return a.ctypes.data_as(C.c_void_p)


def oracle_lib():
    global _ora
    if _ora is None:
        import ncrystal_gb300._build as B
        path = B.oracle_path()
        if not os.path.exists(path):
            B.build_oracle()
        L = C.CDLL(path)
        L.ncgb_oracle_xs.restype = C.c_double
        L.ncgb_oracle_xs.argtypes = [C.c_void_p, C.c_double]
        L.ncgb_oracle_xs_many.restype = None
        L.ncgb_oracle_xs_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        L.ncgb_oracle_abs_xs_many.restype = None
        L.ncgb_oracle_abs_xs_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        L.ncgb_oracle_scatter_dir_many.restype = C.c_int64
        L.ncgb_oracle_scatter_dir_many.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_uint64,
                                                   C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                                   C.c_void_p]
        L.ncgb_oracle_scatter_many.restype = C.c_int64
        L.ncgb_oracle_scatter_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_uint64, C.c_uint32,
                                               C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p]
        _ora = L
    return _ora


class HostMaterial:
    """A material's flat tables in host memory (built by the library's host
    table loader from a bundle file)."""

    def __init__(self, bundle_path):
        from ncrystal_gb300.core import lib
        L = lib()
        self._L = L
        h = L.ncgb_tables_load(bundle_path.encode())
        if not h:
            raise RuntimeError("could not load %s: %s" % (bundle_path, L.ncgb_tables_lasterror().decode()))
        self._h = h
        self.view = C.create_string_buffer(VIEW_BYTES)
        L.ncgb_tables_view(C.c_void_p(h), self.view)

    def __del__(self):
        try:
            self._L.ncgb_tables_free(C.c_void_p(self._h))
        except Exception:
            pass

    def nbytes(self):
        return self._L.ncgb_tables_bytes(C.c_void_p(self._h))

    def array(self, comp, name, dtype):
        p = C.c_void_p()
        n = C.c_ulong()
        if self._L.ncgb_tables_array(C.c_void_p(self._h), comp, name.encode(), C.byref(p), C.byref(n)):
            raise KeyError(name)
        dt = np.dtype(dtype)
        if n.value == 0:
            return np.zeros(0, dt)
        raw = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_char)), shape=(n.value * dt.itemsize,))
        return raw.view(dt).copy()

    def scalar(self, comp, name):
        v = C.c_double()
        if self._L.ncgb_tables_scalar(C.c_void_p(self._h), comp, name.encode(), C.byref(v)):
            raise KeyError(name)
        return v.value

    # ---- learned beta proposal tables -----------------------------------------
    LP_HDR = np.dtype([("c1", "<f8"), ("c1_thr", "<u4"), ("accept", "<f4"), ("enabled", "<i4"), ("pad", "<i4")])
    LP_SLOT = np.dtype([("aprob", "<f4"), ("alias", "<i4")])
    LP_CELL = np.dtype([("q", "<f8"), ("h", "<f8"), ("env", "<f4"), ("seg_lo", "<i4"), ("seg_n", "<i4"),
                        ("pad", "<i4")])
    LP_SEG = np.dtype([("w0", "<u4"), ("y0", "<f4"), ("slope", "<f4"), ("bin", "<i4")])
    LP_K = 126

    def build_proposal(self, comp, knots, allowed=None, min_accept=0.5):
        """The library's proposal tables from knots[ne, 62] (asinh(beta)):
        -> (hdr[ne], slot[ne, K], cell[ne, K], seg[nseg]) structured arrays."""
        k = np.ascontiguousarray(knots, dtype=np.float32)
        ne = k.shape[0]
        al = None if allowed is None else np.ascontiguousarray(allowed, dtype=np.uint8)
        nseg = C.c_ulong(0)
        args = (C.c_void_p(self._h), comp, _P(k), None if al is None else _P(al), float(min_accept))
        rc = self._L.ncgb_tables_build_proposal(*args, None, None, None, None, C.byref(nseg))
        if rc != 2:
            raise RuntimeError(self._L.ncgb_tables_lasterror().decode())
        hdr = np.zeros(ne, dtype=self.LP_HDR)
        slot = np.zeros((ne, self.LP_K), dtype=self.LP_SLOT)
        cell = np.zeros((ne, self.LP_K), dtype=self.LP_CELL)
        seg = np.zeros(max(1, nseg.value), dtype=self.LP_SEG)
        if self._L.ncgb_tables_build_proposal(*args, _P(hdr), _P(slot), _P(cell), _P(seg), C.byref(nseg)):
            raise RuntimeError(self._L.ncgb_tables_lasterror().decode())
        return hdr, slot, cell, seg[:nseg.value]

    def set_proposal(self, comp, tables):
        """Make the oracle sample component 'comp' with these proposal tables
        ((hdr, slot, cell, seg) from build_proposal, or None to remove them)."""
        if tables is None:
            rc = self._L.ncgb_tables_set_proposal(C.c_void_p(self._h), comp, None, None, None, None, 0)
        else:
            hdr, slot, cell, seg = (np.ascontiguousarray(a, dtype=d) for a, d in
                                    zip(tables, (self.LP_HDR, self.LP_SLOT, self.LP_CELL, self.LP_SEG)))
            rc = self._L.ncgb_tables_set_proposal(C.c_void_p(self._h), comp, _P(hdr), _P(slot), _P(cell), _P(seg),
                                                  len(seg))
        if rc:
            raise RuntimeError("ncgb_tables_set_proposal failed")
        self._L.ncgb_tables_view(C.c_void_p(self._h), self.view)

    # ---- oracle evaluation ----------------------------------------------------
    def xs(self, ekin):
        e = np.ascontiguousarray(ekin, dtype=np.float64)
        out = np.empty(len(e))
        oracle_lib().ncgb_oracle_xs_many(self.view, _P(e), len(e), _P(out))
        return out

    def scatter(self, ekin, seed, index_offset=0, callseq=0, stream=0):
        """Per neutron i: stream (seed, i+index_offset, callseq, stream).
        Returns (ekin_final, mu, status, ndraws)."""
        e = np.ascontiguousarray(ekin, dtype=np.float64)
        n = len(e)
        ef = np.empty(n)
        mu = np.empty(n)
        st = np.empty(n, dtype=np.int32)
        nd = np.empty(n, dtype=np.int32)
        oracle_lib().ncgb_oracle_scatter_many(self.view, _P(e), n, seed, index_offset, callseq, stream,
                                              _P(ef), _P(mu), _P(st), _P(nd))
        return ef, mu, st, nd


def _scatter_dir(self, ekin, direction, seed, index_offset=0, callseq=0, stream=0):
    """Scatters with directions (ProcComposition::sampleScatter): per neutron
    i, stream (seed, i+index_offset, callseq, stream).  Returns (ekin_final,
    direction_final[n, 3], status)."""
    e = np.ascontiguousarray(ekin, dtype=np.float64)
    d = np.ascontiguousarray(direction, dtype=np.float64).reshape(len(e), 3)
    n = len(e)
    ef = np.empty(n)
    do = np.empty((n, 3))
    st = np.empty(n, dtype=np.int32)
    oracle_lib().ncgb_oracle_scatter_dir_many(self.view, _P(e), _P(d), n, seed, index_offset, callseq, stream,
                                              _P(ef), _P(do), _P(st))
    return ef, do, st


HostMaterial.scatter_dir = _scatter_dir


def _abs_xs(self, ekin):
    """Absorption cross-sections (AbsOOV) of the material."""
    e = np.ascontiguousarray(ekin, dtype=np.float64)
    out = np.empty(len(e))
    oracle_lib().ncgb_oracle_abs_xs_many(self.view, _P(e), len(e), _P(out))
    return out


HostMaterial.abs_xs = _abs_xs


def refpin_lib():
    """The harness around the reference library (only where it was built)."""
    global _refpin
    if _refpin is None:
        path = os.path.join(HERE, "_ref", "librefpin.so")
        if not os.path.exists(path):
            return None
        L = C.CDLL(path)
        L.refpin_abs_xs.restype = C.c_int
        L.refpin_abs_xs.argtypes = [C.c_char_p, C.c_void_p, C.c_int64, C.c_void_p]
        L.refpin_run_dir.restype = C.c_int
        L.refpin_run_dir.argtypes = [C.c_char_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                     C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.refpin_run.restype = C.c_int
        L.refpin_run.argtypes = [C.c_char_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p, C.c_int64,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _refpin = L
    return _refpin


def reference_run(cfg, ekin, seed, callseq=0, stream=0):
    """Run the reference library on the same per-neutron Philox streams.
    Returns dict(xs, ekin_final, mu, ndraws, status)."""
    L = refpin_lib()
    if L is None:
        raise RuntimeError("reference harness not built")
    e = np.ascontiguousarray(ekin, dtype=np.float64)
    n = len(e)
    out = dict(xs=np.empty(n), ekin_final=np.empty(n), mu=np.empty(n),
               ndraws=np.empty(n, dtype=np.int32), status=np.empty(n, dtype=np.int32))
    rc = L.refpin_run(cfg.encode(), seed, callseq, stream, _P(e), n, _P(out["xs"]), _P(out["ekin_final"]),
                      _P(out["mu"]), _P(out["ndraws"]), _P(out["status"]))
    if rc:
        raise RuntimeError("reference could not create %r" % cfg)
    return out


def reference_run_dir(cfg, ekin, direction, seed, callseq=0, stream=0):
    """The reference's ncrystal_samplescatter on the same per-neutron streams.
    Returns dict(ekin_final, direction[n, 3], ndraws, status)."""
    L = refpin_lib()
    if L is None:
        raise RuntimeError("reference harness not built")
    e = np.ascontiguousarray(ekin, dtype=np.float64)
    n = len(e)
    d = np.ascontiguousarray(direction, dtype=np.float64).reshape(n, 3)
    out = dict(ekin_final=np.empty(n), direction=np.empty((n, 3)), ndraws=np.empty(n, dtype=np.int32),
               status=np.empty(n, dtype=np.int32))
    rc = L.refpin_run_dir(cfg.encode(), seed, callseq, stream, _P(e), _P(d), n, _P(out["ekin_final"]),
                          _P(out["direction"]), _P(out["ndraws"]), _P(out["status"]))
    if rc:
        raise RuntimeError("reference could not create %r" % cfg)
    return out


def reference_abs_xs(cfg, ekin):
    """The reference's absorption cross-sections for cfg."""
    L = refpin_lib()
    if L is None:
        raise RuntimeError("reference harness not built")
    e = np.ascontiguousarray(ekin, dtype=np.float64)
    out = np.empty(len(e))
    if L.refpin_abs_xs(cfg.encode(), _P(e), len(e), _P(out)):
        raise RuntimeError("reference could not create absorption for %r" % cfg)
    return out
