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


# ---- CPU MiniMC engine (oracle/ncgb_oracle_mmc.c) --------------------------------------

MMC_TALLIES = ["theta", "mu", "nscat", "nscat_uw", "w", "e", "l", "de", "q"]
MMC_GROUPS = ["NOSCAT", "SINGLESCAT_ELAS", "SINGLESCAT_INELAS", "MULTISCAT_PUREELAS", "MULTISCAT_OTHER"]


class OraMmcCfg(C.Structure):
    _fields_ = [("geom", C.c_int32), ("unbounded", C.c_int32), ("r", C.c_double), ("dx", C.c_double),
                ("dy", C.c_double), ("dz", C.c_double),
                ("src", C.c_int32), ("might_be_outside", C.c_int32),
                ("sx", C.c_double), ("sy", C.c_double), ("sz", C.c_double), ("sux", C.c_double),
                ("suy", C.c_double), ("suz", C.c_double), ("sr", C.c_double), ("energy", C.c_double),
                ("ax", C.c_double), ("ay", C.c_double), ("az", C.c_double), ("bx", C.c_double),
                ("by", C.c_double), ("bz", C.c_double),
                ("macro", C.c_double), ("abs_c", C.c_double), ("psurv", C.c_double), ("wthr", C.c_double),
                ("nscatthr", C.c_int32), ("nscatlimit", C.c_int32), ("has_abs", C.c_int32), ("has_scat", C.c_int32),
                ("ignore_miss", C.c_int32), ("breakdown", C.c_int32),
                ("seed", C.c_uint64), ("scatter_seed", C.c_uint64), ("scatter_stream", C.c_uint32), ("pad", C.c_uint32),
                ("fixed_dir", C.c_int32), ("fixed_e", C.c_int32),
                ("d0x", C.c_double), ("d0y", C.c_double), ("d0z", C.c_double), ("e0", C.c_double),
                ("enabled", C.c_int32 * 9), ("nbins", C.c_int32 * 9), ("xmin", C.c_double * 9),
                ("xmax", C.c_double * 9), ("off", C.c_int64 * 9), ("soff", C.c_int64 * 9)]


def mmc_config(material, bundle, geom, src, engine, binnings, seed=1, scatter_seed=2, scatter_stream=0):
    """The engine's configuration from a run's decoded input (the 'decoded'
    dicts of a MiniMC results document: geometry, source with a fixed energy
    in eV under 'energy_ev', engine) and the tally binnings
    {name: (nbins, xmin, xmax)}; bundle: the material's bundle records
    (info.numdens, abs_c)."""
    c = OraMmcCfg()
    kinds = {"sphere": 0, "box": 1, "slab": 2, "cyl": 3}
    c.geom = kinds[geom["name"]]
    c.r = geom.get("r", 0.0)
    c.dx = geom.get("dx", 0.0)
    c.dy = geom.get("dy", 0.0)
    c.dz = geom.get("dz", 0.0)
    c.unbounded = int(c.geom == 2 or (c.geom == 3 and c.dy == 0.0))
    sk = {"constant": 0, "circular": 1, "isotropic": 2}[src["name"]]
    c.src = sk
    c.sx, c.sy, c.sz = src.get("x", 0.0), src.get("y", 0.0), src.get("z", 0.0)
    c.sux, c.suy, c.suz = src.get("ux", 0.0), src.get("uy", 0.0), src.get("uz", 1.0)
    c.sr = src.get("r", 0.0)
    c.energy = src["energy_ev"]
    def inside(x, y, z):
        if c.geom == 0:
            return x * x + y * y + z * z <= c.r * c.r
        if c.geom == 1:
            return abs(x) <= c.dx and abs(y) <= c.dy and abs(z) <= c.dz
        if c.geom == 2:
            return abs(z) <= c.dz
        return x * x + z * z <= c.r * c.r and (c.dy == 0.0 or abs(y) <= c.dy)
    c.might_be_outside = int((sk == 1 and c.sr > 0) or not inside(c.sx, c.sy, c.sz))
    if sk == 1 and c.sr > 0:
        d = np.array([c.sux, c.suy, c.suz])
        a = np.array([1.0, 0.0, 0.0])
        if a @ d > 0.8:
            a = np.array([0.0, 1.0, 0.0])
        if a @ d > 0.8:
            a = np.array([0.0, 0.0, 1.0])
        va = np.cross(d, a); va /= np.linalg.norm(va)
        vb = np.cross(d, va); vb /= np.linalg.norm(vb)
        c.ax, c.ay, c.az = va * c.sr
        c.bx, c.by, c.bz = vb * c.sr
    nd = float(bundle["info.numdens"][0])
    c.macro = 100.0 * nd
    absc = float(bundle["abs_c"][0]) if "abs_c" in bundle else 0.0
    c.has_abs = int(bool(engine.get("absorption", True)) and absc > 0.0 and c.macro > 0.0)
    c.abs_c = absc if c.has_abs else 0.0
    c.has_scat = int(c.macro > 0.0 and int(bundle["ncomp"][0]) > 0)
    rl = engine.get("roulette", {"psurvival": 0.1, "weight_threshold": 0.01, "nscat_threshold": 2})
    c.psurv, c.wthr, c.nscatthr = rl["psurvival"], rl["weight_threshold"], rl["nscat_threshold"]
    c.nscatlimit = -1 if engine.get("nscatlimit") is None else int(engine["nscatlimit"])
    c.ignore_miss = int(bool(engine.get("ignoremiss", False)))
    c.breakdown = int(bool(engine.get("tallybreakdown", True)))
    c.seed, c.scatter_seed, c.scatter_stream = seed, scatter_seed, scatter_stream
    src_src = engine.get("tallyref", "truth") == "src"
    if sk in (0, 1):
        c.fixed_dir = 1
        c.d0x, c.d0y, c.d0z = c.sux, c.suy, c.suz
    c.fixed_e = 1
    c.e0 = c.energy
    del src_src
    off = 0
    for k, name in enumerate(MMC_TALLIES):
        if name in binnings:
            c.enabled[k] = 1
            c.soff[k] = off
            off += 6 * 5
    nstat = off
    for k, name in enumerate(MMC_TALLIES):
        if name in binnings:
            nb, lo, hi = binnings[name]
            c.nbins[k], c.xmin[k], c.xmax[k] = int(nb), lo, hi
            c.off[k] = off
            off += 6 * (int(nb) + 2) * 2
    return c, nstat, off


def mmc_empty_buffer(c, nbuf):
    buf = np.zeros(nbuf, dtype=np.float64)
    k = buf.view(np.int64)
    for t in range(9):
        if c.enabled[t]:
            for g in range(6):
                k[c.soff[t] + g * 5 + 3] = np.iinfo(np.int64).max
                k[c.soff[t] + g * 5 + 4] = np.iinfo(np.int64).min
    return buf


def mmc_run(material, c, nbuf, first_id, count, threads=1):
    """Histories [first_id, first_id+count) on `threads` host threads.
    Returns (tally buffer, counts[tallied, tallied_w, miss, miss_w, nfail, steps])."""
    from concurrent.futures import ThreadPoolExecutor
    L = oracle_lib()
    if not hasattr(L, "_mmc_ready"):
        L.ncgb_oracle_mmc_run.restype = C.c_int
        L.ncgb_oracle_mmc_run.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p]
        L._mmc_ready = True
    parts = max(1, min(threads, count))
    edges = np.linspace(first_id, first_id + count, parts + 1).astype(np.uint64)
    bufs = [mmc_empty_buffer(c, nbuf) for _ in range(parts)]
    cnts = [np.zeros(6) for _ in range(parts)]

    def work(i):
        L.ncgb_oracle_mmc_run(material.view, C.byref(c), int(edges[i]), int(edges[i + 1] - edges[i]),
                              _P(bufs[i]), _P(cnts[i]))

    with ThreadPoolExecutor(max_workers=parts) as ex:
        list(ex.map(work, range(parts)))
    out = mmc_empty_buffer(c, nbuf)
    ko = out.view(np.int64)
    for b in bufs:
        kb = b.view(np.int64)
        for t in range(9):
            if not c.enabled[t]:
                continue
            for g in range(6):
                s0 = c.soff[t] + g * 5
                out[s0:s0 + 3] += b[s0:s0 + 3]
                ko[s0 + 3] = min(ko[s0 + 3], kb[s0 + 3])
                ko[s0 + 4] = max(ko[s0 + 4], kb[s0 + 4])
        nstat_end = min(c.off[t] for t in range(9) if c.enabled[t])
        out[nstat_end:] += b[nstat_end:]
    return out, np.sum(cnts, axis=0)


def mmc_hist(c, buf, name, part="total"):
    """(content, errorsq) with under/overflow of one tally group."""
    k = MMC_TALLIES.index(name)
    g = 0 if part == "total" else 1 + MMC_GROUPS.index(part)
    nb = c.nbins[k]
    b = buf[c.off[k] + g * (nb + 2) * 2: c.off[k] + (g + 1) * (nb + 2) * 2].reshape(-1, 2)
    return b[:, 0].copy(), b[:, 1].copy()


def reference_mmc(entries):
    """The reference library's own MiniMC (ncrystal_jsonquery of
    oracle/_ref/libNCrystal.so, where the NCrystal sources were built) for a
    query ["mmc", "run", ...]; None when that library is absent."""
    import json
    import ncrystal_gb300._build as B
    path = os.path.join(B.REF_OUT, "libNCrystal.so")
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    L.ncrystal_jsonquery.restype = C.c_void_p
    L.ncrystal_jsonquery.argtypes = [C.c_char_p]
    L.ncrystal_dealloc_string.argtypes = [C.c_void_p]
    raw = L.ncrystal_jsonquery("\x07".join(entries).encode())
    if not raw:
        raise RuntimeError("reference MiniMC query failed: %r" % (entries,))
    txt = C.cast(raw, C.c_char_p).value.decode()
    L.ncrystal_dealloc_string(raw)
    return json.loads(txt)
