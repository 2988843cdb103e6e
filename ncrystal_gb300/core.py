"""Python face of the GPU scattering path, shaped like NCrystal's own Python
API for non-oriented materials (ncrystal_python/src/NCrystal/core.py:
createScatter, Process.crossSectionIsotropic, Scatter.sampleScatterIsotropic,
Scatter.clone; _chooks.py:499-560 for the array handling).

Everything goes through the C ABI of libncrystal_gb300.so (ctypes); the
per-neutron work runs in its CUDA kernels.  If the library is not built, or no
GPU is present, calls fail with an exception: there is no CPU fallback.
"""
import ctypes as _C
import os as _os

import numpy as _np

from . import _build


class NCException(RuntimeError):
    """Base error (mirrors NCrystal.exceptions.NCException)."""


class NCFileNotFound(NCException):
    pass


class NCBadInput(NCException):
    pass


class NCCalcError(NCException):
    pass


class NCLogicError(NCException):
    pass


_ERRTYPES = {"FileNotFound": NCFileNotFound, "BadInput": NCBadInput,
             "CalcError": NCCalcError, "LogicError": NCLogicError}

_lib = None


class _Handle(_C.Structure):
    _fields_ = [("internal", _C.c_void_p)]


_dblp = _C.POINTER(_C.c_double)


def lib():
    """The loaded C library (built on first use if sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.library_path()
    if not _os.path.exists(path):
        raise ImportError("libncrystal_gb300.so is not built (run __graft_entry__.build()); "
                          "the GPU scattering path has no CPU fallback")
    L = _C.CDLL(path)
    H = _Handle
    sig = {
        "ncrystal_create_scatter": (H, [_C.c_char_p]),
        "ncrystal_create_scatter_builtinrng": (H, [_C.c_char_p, _C.c_ulong]),
        "ncrystal_clone_scatter": (H, [H]),
        "ncrystal_clone_scatter_rngbyidx": (H, [H, _C.c_ulong]),
        "ncrystal_clone_scatter_rngforcurrentthread": (H, [H]),
        "ncrystal_cast_scat2proc": (H, [H]),
        "ncrystal_create_absorption": (H, [_C.c_char_p]),
        "ncrystal_clone_absorption": (H, [H]),
        "ncrystal_cast_abs2proc": (H, [H]),
        "ncrystal_cast_proc2abs": (H, [H]),
        "ncrystal_cast_proc2scat": (H, [H]),
        "ncgb_xs_abs_scatter_device": (_C.c_int, [H, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p, _C.c_void_p,
                                                  _C.c_void_p, _C.c_void_p, _C.c_void_p]),
        "ncrystal_unref": (None, [_C.c_void_p]),
        "ncrystal_refcount": (_C.c_int, [_C.c_void_p]),
        "ncrystal_valid": (_C.c_int, [_C.c_void_p]),
        "ncrystal_name": (_C.c_char_p, [H]),
        "ncrystal_domain": (None, [H, _dblp, _dblp]),
        "ncrystal_isnonoriented": (_C.c_int, [H]),
        "ncrystal_crosssection_nonoriented": (None, [H, _C.c_double, _dblp]),
        "ncrystal_crosssection_nonoriented_many": (None, [H, _C.c_void_p, _C.c_ulong, _C.c_ulong, _C.c_void_p]),
        "ncrystal_samplescatterisotropic": (None, [H, _C.c_double, _dblp, _dblp]),
        "ncrystal_samplescatterisotropic_many": (None, [H, _C.c_void_p, _C.c_ulong, _C.c_ulong,
                                                        _C.c_void_p, _C.c_void_p]),
        "ncrystal_genscatter_nonoriented_many": (None, [H, _C.c_void_p, _C.c_ulong, _C.c_ulong,
                                                        _C.c_void_p, _C.c_void_p]),
        "ncrystal_sethaltonerror": (_C.c_int, [_C.c_int]),
        "ncrystal_setquietonerror": (_C.c_int, [_C.c_int]),
        "ncrystal_error": (_C.c_int, []),
        "ncrystal_lasterror": (_C.c_char_p, []),
        "ncrystal_lasterrortype": (_C.c_char_p, []),
        "ncrystal_clearerror": (None, []),
        "ncrystal_version": (_C.c_int, []),
        "ncgb_bundle_path": (_C.c_int, [_C.c_char_p, _C.c_char_p, _C.c_ulong]),
        "ncgb_bundle_cache_dir": (_C.c_int, [_C.c_char_p, _C.c_ulong]),
        "ncgb_create_scatter_bundle": (H, [_C.c_char_p, _C.c_ulong]),
        "ncgb_samplescatterisotropic_keyed": (_C.c_int, [H, _C.c_double, _C.c_ulonglong,
                                                         _C.POINTER(_C.c_double), _C.POINTER(_C.c_double)]),
        "ncgb_sab_phase_profile": (_C.c_int, [H, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p, _C.c_void_p,
                                              _C.c_void_p]),
        "ncgb_scatter_device": (_C.c_int, [H, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p,
                                           _C.c_void_p, _C.c_void_p, _C.c_void_p]),
        "ncgb_scatter_device_f32": (_C.c_int, [H, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p,
                                               _C.c_void_p, _C.c_void_p, _C.c_void_p]),
        "ncgb_crosssection_nonoriented_many_f32": (None, [H, _C.c_void_p, _C.c_ulong, _C.c_void_p]),
        "ncgb_samplescatterisotropic_many_f32": (None, [H, _C.c_void_p, _C.c_ulong, _C.c_void_p,
                                                        _C.c_void_p]),
        "ncgb_xs_scatter_many": (None, [H, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p, _C.c_void_p]),
        "ncgb_xs_scatter_many_f32": (None, [H, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p,
                                            _C.c_void_p]),
        "ncgb_last_nfailed": (_C.c_ulong, []),
        "ncgb_batch_create": (_Handle, [_C.POINTER(_Handle), _C.c_ulong]),
        "ncgb_batch_destroy": (None, [_C.c_void_p]),
        "ncgb_batch_scatter_device": (_C.c_int, [_Handle, _C.c_void_p, _C.c_void_p, _C.c_ulong, _C.c_void_p,
                                                 _C.c_void_p, _C.c_void_p, _C.c_void_p, _C.c_void_p]),
        "ncgb_batch_graph_launch": (_C.c_int, [_Handle, _C.c_void_p, _C.c_void_p, _C.c_ulong, _C.c_void_p,
                                               _C.c_void_p, _C.c_void_p, _C.c_void_p, _C.c_void_p]),
        "ncgb_batch_autotune": (_C.c_int, [_Handle, _C.c_void_p, _C.c_void_p, _C.c_ulong, _C.c_void_p,
                                           _C.c_void_p, _C.c_void_p, _C.c_void_p]),
        "ncgb_batch_config": (_C.c_int, [_Handle, _C.POINTER(_C.c_int), _C.POINTER(_C.c_int)]),
        "ncgb_batch_split_lists": (_C.c_int, [_Handle, _C.POINTER(_C.c_int)]),
        "ncgb_batch_set_split_lists": (_C.c_int, [_Handle, _C.c_int]),
        "ncgb_batch_set_mode": (_C.c_int, [_Handle, _C.c_int]),
        "ncrystal_samplescatter": (None, [H, _C.c_double, _C.POINTER(_C.c_double * 3), _dblp,
                                          _C.POINTER(_C.c_double * 3)]),
        "ncrystal_samplescatter_many": (None, [H, _C.c_double, _C.POINTER(_C.c_double * 3), _C.c_ulong, _C.c_void_p,
                                               _C.c_void_p, _C.c_void_p, _C.c_void_p]),
        "ncgb_scatter_dir_device": (_C.c_int, [H, _C.c_void_p, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p,
                                               _C.c_void_p, _C.c_void_p]),
        "ncgb_batch_set_sampler": (_C.c_int, [_Handle, _C.c_int]),
        "ncgb_set_sampler": (_C.c_int, [H, _C.c_int]),
        "ncgb_get_sampler": (_C.c_int, [H]),
        "ncgb_material_info": (_C.c_int, [H, _C.POINTER(_C.c_int), _dblp]),
        "ncgb_component_info": (_C.c_int, [H, _C.c_int, _C.POINTER(_C.c_int), _dblp, _C.POINTER(_C.c_ulong)]),
        "ncgb_sab_egrid": (_C.c_int, [H, _C.c_int, _C.c_void_p]),
        "ncgb_sab_sample_device": (_C.c_int, [H, _C.c_int, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p,
                                              _C.c_void_p, _C.c_void_p]),
        "ncgb_mlp_create": (_Handle, [_C.c_ulonglong]),
        "ncgb_mlp_destroy": (None, [_C.c_void_p]),
        "ncgb_mlp_nparams": (_C.c_ulong, []),
        "ncgb_mlp_get_params": (_C.c_int, [_Handle, _C.c_void_p]),
        "ncgb_mlp_set_params": (_C.c_int, [_Handle, _C.c_void_p]),
        "ncgb_mlp_set_ranges": (_C.c_int, [_Handle, _C.c_double, _C.c_double, _C.c_double, _C.c_double]),
        "ncgb_mlp_gradients": (_C.c_int, [_Handle, _C.c_void_p, _C.c_void_p, _C.c_void_p, _C.c_ulong, _C.c_void_p,
                                          _C.POINTER(_C.c_float), _C.c_void_p]),
        "ncgb_mlp_train": (_C.c_int, [_Handle, _C.c_void_p, _C.c_void_p, _C.c_void_p, _C.c_ulong, _C.c_ulong,
                                      _C.c_uint, _C.c_float, _C.c_ulonglong, _C.c_void_p, _C.c_ulong, _C.c_void_p]),
        "ncgb_mlp_knots": (_C.c_int, [_Handle, _C.c_void_p, _C.c_void_p, _C.c_ulong, _C.c_void_p, _C.c_void_p]),
        "ncgb_attach_proposal": (_C.c_int, [H, _C.c_int, _Handle, _C.c_double, _dblp]),
        "ncgb_attach_proposal_knots": (_C.c_int, [H, _C.c_int, _C.c_void_p, _C.c_double, _dblp]),
        "ncgb_detach_proposal": (_C.c_int, [H, _C.c_int]),
        "ncgb_proposal_acceptance": (_C.c_int, [H, _C.c_int, _C.c_void_p, _C.c_void_p]),
        "ncgb_tables_build_proposal": (_C.c_int, [_C.c_void_p, _C.c_int, _C.c_void_p, _C.c_void_p, _C.c_double,
                                                  _C.c_void_p, _C.c_void_p, _C.c_void_p, _C.c_void_p,
                                                  _C.POINTER(_C.c_ulong)]),
        "ncgb_tables_set_proposal": (_C.c_int, [_C.c_void_p, _C.c_int, _C.c_void_p, _C.c_void_p, _C.c_void_p,
                                                _C.c_void_p, _C.c_ulong]),
        "ncgb_set_mode": (_C.c_int, [H, _C.c_int]),
        "ncgb_get_mode": (_C.c_int, [H]),
        "ncgb_batch_xs_scatter_many": (None, [_Handle, _C.c_void_p, _C.c_void_p, _C.c_ulong, _C.c_void_p,
                                              _C.c_void_p, _C.c_void_p]),
        "ncgb_phase_timing": (None, [_C.c_int]),
        "ncgb_phase_times": (_C.c_int, [_dblp, _dblp, _C.POINTER(_C.c_ulong), _C.POINTER(_C.c_ulong)]),
        "ncgb_device_bytes": (_C.c_ulong, [H]),
        "ncgb_sab_derive_compare": (_C.c_int, [_C.c_char_p, _C.c_int, _dblp, _C.POINTER(_C.c_longlong),
                                               _C.POINTER(_C.c_longlong), _dblp, _dblp]),
        "ncgb_sab_derive_compare_many": (_C.c_int, [_C.POINTER(_C.c_char_p), _C.c_ulong, _dblp,
                                                    _C.POINTER(_C.c_longlong), _C.POINTER(_C.c_longlong),
                                                    _C.POINTER(_C.c_longlong), _dblp, _dblp]),
        "ncgb_create_scatters": (_C.c_int, [_C.POINTER(_C.c_char_p), _C.c_ulong, _C.c_ulong, _C.POINTER(H)]),
        "ncrystal_jsonquery": (_C.c_void_p, [_C.c_char_p]),
        "ncrystal_dealloc_string": (None, [_C.c_void_p]),
        "ncgb_mmc_run": (_C.c_void_p, [H, _C.c_char_p, _C.c_char_p, _C.c_char_p]),
        "ncgb_tables_load": (_C.c_void_p, [_C.c_char_p]),
        "ncgb_tables_lasterror": (_C.c_char_p, []),
        "ncgb_tables_view": (_C.c_int, [_C.c_void_p, _C.c_void_p]),
        "ncgb_tables_bytes": (_C.c_ulong, [_C.c_void_p]),
        "ncgb_tables_free": (None, [_C.c_void_p]),
        "ncgb_tables_array": (_C.c_int, [_C.c_void_p, _C.c_int, _C.c_char_p, _C.POINTER(_C.c_void_p),
                                         _C.POINTER(_C.c_ulong)]),
        "ncgb_tables_scalar": (_C.c_int, [_C.c_void_p, _C.c_int, _C.c_char_p, _dblp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    # Errors become Python exceptions, as in NCrystal's Python layer.
    L.ncrystal_sethaltonerror(0)
    L.ncrystal_setquietonerror(1)
    _lib = L
    return L


def _check():
    L = lib()
    if L.ncrystal_error():
        msg = (L.ncrystal_lasterror() or b"").decode()
        typ = (L.ncrystal_lasterrortype() or b"").decode()
        L.ncrystal_clearerror()
        raise _ERRTYPES.get(typ, NCException)("%s [%s]" % (msg, typ) if typ else msg)


def _prepare_many(ekin, repeat):
    """Same conventions as NCrystal's _chooks.py:499-507."""
    if repeat is None and not hasattr(ekin, "__len__"):
        return None
    repeat = 1 if repeat is None else int(repeat)
    arr = _np.ascontiguousarray(_np.asarray(ekin, dtype=_np.float64).reshape(-1)) \
        if hasattr(ekin, "__len__") else _np.ones(1) * float(ekin)
    return arr, len(arr), repeat


class Process:
    """A material's scattering process on the GPU (non-oriented)."""

    def __init__(self, handle, cfgstr):
        self._h = handle
        self._cfg = cfgstr

    def __del__(self):
        try:
            if self._h is not None and self._h.internal:
                lib().ncrystal_unref(_C.byref(self._h))
        except Exception:
            pass

    @property
    def cfgstr(self):
        return self._cfg

    @property
    def name(self):
        return lib().ncrystal_name(self._h).decode()

    def domain(self):
        a, b = _C.c_double(), _C.c_double()
        lib().ncrystal_domain(self._h, _C.byref(a), _C.byref(b))
        _check()
        return a.value, b.value

    def isNonOriented(self):
        return True

    def isOriented(self):
        return False

    def crossSectionIsotropic(self, ekin, repeat=None):
        """Cross-sections in barn (NCrystal core.py:1277); arrays in, arrays out."""
        L = lib()
        many = _prepare_many(ekin, repeat)
        if many is None:
            r = _C.c_double()
            L.ncrystal_crosssection_nonoriented(self._h, float(ekin), _C.byref(r))
            _check()
            return r.value
        arr, n, rep = many
        out = _np.empty(n * rep, dtype=_np.float64)
        if n * rep:
            L.ncrystal_crosssection_nonoriented_many(self._h, arr.ctypes.data, n, rep, out.ctypes.data)
            _check()
        return out

    def xsect(self, ekin=None, wl=None, repeat=None):
        if (ekin is None) == (wl is None):
            raise NCBadInput("xsect: give exactly one of ekin and wl")
        if wl is not None:
            w = _np.asarray(wl, dtype=_np.float64)
            ekin = 0.081804209605330899 / (w * w)
            if w.ndim == 0:
                ekin = float(ekin)
        return self.crossSectionIsotropic(ekin, repeat)

    def device_bytes(self):
        return lib().ncgb_device_bytes(self._h)


MODES = {"exact": 0, "mixed": 1}
SAMPLERS = {"plain": 0, "learned": 1}
COMP_SAB = 3


def _mode_code(mode):
    if mode not in MODES:
        raise NCBadInput("mode must be one of %s" % sorted(MODES))
    return MODES[mode]


class Scatter(Process):
    """A scattering process with its own random streams (NCrystal core.py:1411-1520)."""

    @property
    def mode(self):
        """Arithmetic mode, "exact" (FP64 throughout) or "mixed" (FP32 for the
        incoherent-elastic exponentials and the alpha inversion)."""
        m = lib().ncgb_get_mode(self._h)
        _check()
        return {v: k for k, v in MODES.items()}[m]

    def set_mode(self, mode):
        if lib().ncgb_set_mode(self._h, _mode_code(mode)):
            _check()
        return self

    # ---- learned beta proposal ----------------------------------------------
    @property
    def sampler(self):
        """"plain" (percentile inversion) or "learned" (attached proposals)."""
        m = lib().ncgb_get_sampler(self._h)
        _check()
        return {v: k for k, v in SAMPLERS.items()}[m]

    def set_sampler(self, sampler):
        if sampler not in SAMPLERS:
            raise NCBadInput("sampler must be one of %s" % sorted(SAMPLERS))
        if lib().ncgb_set_sampler(self._h, SAMPLERS[sampler]):
            _check()
        return self

    def material_info(self):
        """-> (ncomp, temperature K, [(type, scale, ne), ...])."""
        L = lib()
        nc, T = _C.c_int(), _C.c_double()
        if L.ncgb_material_info(self._h, _C.byref(nc), _C.byref(T)):
            _check()
        comps = []
        for c in range(nc.value):
            t, sc, ne = _C.c_int(), _C.c_double(), _C.c_ulong()
            if L.ncgb_component_info(self._h, c, _C.byref(t), _C.byref(sc), _C.byref(ne)):
                _check()
            comps.append((t.value, sc.value, ne.value))
        return nc.value, T.value, comps

    def sab_components(self):
        return [i for i, (t, _, _) in enumerate(self.material_info()[2]) if t == COMP_SAB]

    def sab_egrid(self, comp):
        ne = self.material_info()[2][comp][2]
        out = _np.empty(ne)
        if lib().ncgb_sab_egrid(self._h, comp, out.ctypes.data):
            _check()
        return out

    SAB_PHASES = ("claim", "beta", "alpha", "accept", "convert", "idle")

    def sab_phase_profile(self, ekin, xs=None, ekin_final=None, mu=None):
        """One scatter batch on the float64 CUDA tensor 'ekin' (synchronous)
        with the S(alpha,beta) pass's phase clocks (ncgb_sab_phase_profile):
        -> ({phase: summed lane cycles}, Alg.1 attempts)."""
        out = (_C.c_ulonglong * (len(self.SAB_PHASES) + 1))()
        p = (lambda t: 0 if t is None else t.data_ptr())
        if lib().ncgb_sab_phase_profile(self._h, ekin.data_ptr(), ekin.numel(), p(xs), p(ekin_final), p(mu),
                                        _C.cast(out, _C.c_void_p)):
            _check()
        return dict(zip(self.SAB_PHASES, [int(v) for v in out[:-1]])), int(out[-1])

    def sample_keyed(self, ekin, key):
        """One isotropic scatter at 'ekin' on the random stream of a 64-bit
        key (ncgb_samplescatterisotropic_keyed): -> (E', mu)."""
        ef, mu = _C.c_double(), _C.c_double()
        if lib().ncgb_samplescatterisotropic_keyed(self._h, float(ekin), int(key) & 0xFFFFFFFFFFFFFFFF,
                                                   _C.byref(ef), _C.byref(mu)):
            _check()
        return ef.value, mu.value

    def sab_sample_device(self, comp, ekin, alpha, beta, status=None, stream=None):
        """(alpha, beta) of S(alpha,beta) component 'comp' at the energies of the
        float64 CUDA tensor 'ekin' (ncgb_sab_sample_device)."""
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(ekin.device)
        if lib().ncgb_sab_sample_device(self._h, comp, ekin.data_ptr(), ekin.numel(), alpha.data_ptr(),
                                        beta.data_ptr(), 0 if status is None else status.data_ptr(),
                                        stream.cuda_stream):
            _check()

    def attach_proposal(self, comp, net, min_accept=0.5):
        """Attach network 'net' (an MLP) as the beta proposal of component
        'comp'; returns the mean envelope acceptance of the enabled egrid points."""
        a = _C.c_double()
        if lib().ncgb_attach_proposal(self._h, comp, net._h, float(min_accept), _C.byref(a)):
            _check()
        return a.value

    def attach_proposal_knots(self, comp, knots, min_accept=0.5):
        k = _np.ascontiguousarray(knots, dtype=_np.float32)
        a = _C.c_double()
        if lib().ncgb_attach_proposal_knots(self._h, comp, k.ctypes.data, float(min_accept), _C.byref(a)):
            _check()
        return a.value

    def detach_proposal(self, comp):
        if lib().ncgb_detach_proposal(self._h, comp):
            _check()

    def proposal_acceptance(self, comp):
        """-> (acceptance[ne] float32, enabled[ne] bool) per egrid point."""
        ne = self.material_info()[2][comp][2]
        acc = _np.zeros(ne, dtype=_np.float32)
        en = _np.zeros(ne, dtype=_np.int32)
        if lib().ncgb_proposal_acceptance(self._h, comp, acc.ctypes.data, en.ctypes.data):
            _check()
        return acc, en.astype(bool)

    def sampleScatterIsotropic(self, ekin, repeat=None):
        """Returns (ekin_final, mu) -- NCrystal core.py:1492."""
        L = lib()
        many = _prepare_many(ekin, repeat)
        if many is None:
            ef, mu = _C.c_double(), _C.c_double()
            L.ncrystal_samplescatterisotropic(self._h, float(ekin), _C.byref(ef), _C.byref(mu))
            _check()
            return ef.value, mu.value
        arr, n, rep = many
        ef = _np.empty(n * rep, dtype=_np.float64)
        mu = _np.empty(n * rep, dtype=_np.float64)
        if n * rep:
            L.ncrystal_samplescatterisotropic_many(self._h, arr.ctypes.data, n, rep, ef.ctypes.data,
                                                   mu.ctypes.data)
            _check()
        return ef, mu

    def sampleScatter(self, ekin, direction, repeat=None):
        """NCrystal core.py:1478: (ekin_final, (ux, uy, uz)) for one neutron, or
        arrays (ekin_final, (ux, uy, uz)) of 'repeat' scatters of it."""
        L = lib()
        cdir = (_C.c_double * 3)(*[float(x) for x in direction])
        if not repeat:
            ef = _C.c_double()
            out = (_C.c_double * 3)(0.0, 0.0, 0.0)
            L.ncrystal_samplescatter(self._h, float(ekin), _C.byref(cdir), _C.byref(ef), _C.byref(out))
            _check()
            return ef.value, (out[0], out[1], out[2])
        n = int(repeat)
        ef, ux, uy, uz = (_np.empty(n) for _ in range(4))
        L.ncrystal_samplescatter_many(self._h, float(ekin), _C.byref(cdir), n, ef.ctypes.data, ux.ctypes.data,
                                      uy.ctypes.data, uz.ctypes.data)
        _check()
        return ef, (ux, uy, uz)

    def xs_abs_scatter_device(self, ekin, xs=None, xs_abs=None, ekin_final=None, mu=None, status=None,
                              stream=None):
        """One pass over float64 CUDA tensors: scattering cross-section,
        absorption cross-section (1/v) and one isotropic scatter per neutron."""
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(ekin.device)
        p = (lambda t: 0 if t is None else t.data_ptr())
        if lib().ncgb_xs_abs_scatter_device(self._h, ekin.data_ptr(), ekin.numel(), p(xs), p(xs_abs),
                                            p(ekin_final), p(mu), p(status), stream.cuda_stream):
            _check()

    def scatter_dir_device(self, ekin, direction, ekin_final, direction_final, status=None, stream=None):
        """Scatters with directions on CUDA tensors: ekin (n,) and direction
        (n, 3) float64 in, ekin_final (n,) and direction_final (n, 3) out."""
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(ekin.device)
        if lib().ncgb_scatter_dir_device(self._h, ekin.data_ptr(), direction.data_ptr(), ekin.numel(),
                                         ekin_final.data_ptr(), direction_final.data_ptr(),
                                         0 if status is None else status.data_ptr(), stream.cuda_stream):
            _check()

    def minimc_run(self, geomcfg, srccfg, enginecfg=None):
        """MiniMC on the device with this handle's material, mode, sampler
        and random stream (ncgb_mmc_run); returns the results dictionary."""
        from .minimc import _take_json
        raw = lib().ncgb_mmc_run(self._h, geomcfg.encode(), srccfg.encode(),
                                 None if enginecfg is None else enginecfg.encode())
        return _take_json(raw)

    def genScatterNonOriented(self, ekin, repeat=None):
        """Obsolete NCrystal call: returns (angle, delta_ekin) arrays."""
        arr, n, rep = _prepare_many(ekin if hasattr(ekin, "__len__") else [ekin], repeat)
        ang = _np.zeros(n * rep, dtype=_np.float64)
        de = _np.zeros(n * rep, dtype=_np.float64)
        if n * rep:
            lib().ncrystal_genscatter_nonoriented_many(self._h, arr.ctypes.data, n, rep, ang.ctypes.data,
                                                       de.ctypes.data)
            _check()
        return ang, de

    def clone(self, rng_stream_index=None, for_current_thread=False):
        L = lib()
        if rng_stream_index is not None:
            h = L.ncrystal_clone_scatter_rngbyidx(self._h, int(rng_stream_index))
        elif for_current_thread:
            h = L.ncrystal_clone_scatter_rngforcurrentthread(self._h)
        else:
            h = L.ncrystal_clone_scatter(self._h)
        _check()
        return Scatter(h, self._cfg)

    # ---- device-resident batches (torch CUDA tensors or raw pointers) --------
    def scatter_device(self, ekin, xs=None, ekin_final=None, mu=None, status=None, stream=None):
        """Fused cross-section + scatter on device arrays.  'ekin' and outputs are
        torch CUDA tensors (float64, or all float32) or None.  Asynchronous on
        'stream' (a torch.cuda.Stream, default: torch's current stream)."""
        import torch
        n = ekin.numel()
        f32 = ekin.dtype == torch.float32
        p = (lambda t: 0 if t is None else t.data_ptr())
        if stream is None:
            stream = torch.cuda.current_stream(ekin.device)
        fn = lib().ncgb_scatter_device_f32 if f32 else lib().ncgb_scatter_device
        rc = fn(self._h, ekin.data_ptr(), n, p(xs), p(ekin_final), p(mu), p(status), stream.cuda_stream)
        if rc:
            _check()
        return xs, ekin_final, mu

    def scatter_device_ptr(self, d_ekin, n, d_xs, d_ef, d_mu, d_status, cuda_stream, f32=False):
        fn = lib().ncgb_scatter_device_f32 if f32 else lib().ncgb_scatter_device
        rc = fn(self._h, d_ekin, n, d_xs, d_ef, d_mu, d_status, cuda_stream)
        if rc:
            _check()

    def xs_scatter_host_ptr(self, ekin_ptr, n, xs_ptr, ef_ptr, mu_ptr, f32=False):
        """Fused xs + scatter on host arrays given as raw pointers (pinned
        memory makes the chunked copies asynchronous)."""
        fn = lib().ncgb_xs_scatter_many_f32 if f32 else lib().ncgb_xs_scatter_many
        fn(self._h, ekin_ptr, n, xs_ptr, ef_ptr, mu_ptr)
        _check()

    def xs_scatter(self, ekin):
        """Fused xs + scatter on a numpy array (float64 or float32):
        returns (xs, ekin_final, mu); neutron i uses stream index i."""
        arr = _np.ascontiguousarray(ekin)
        f32 = arr.dtype == _np.float32
        if not f32:
            arr = arr.astype(_np.float64, copy=False)
        n = len(arr)
        xs, ef, mu = (_np.empty(n, dtype=arr.dtype) for _ in range(3))
        self.xs_scatter_host_ptr(arr.ctypes.data, n, xs.ctypes.data, ef.ctypes.data, mu.ctypes.data, f32)
        return xs, ef, mu

    def crossSectionIsotropic_f32(self, ekin):
        arr = _np.ascontiguousarray(ekin, dtype=_np.float32)
        out = _np.empty(len(arr), dtype=_np.float32)
        lib().ncgb_crosssection_nonoriented_many_f32(self._h, arr.ctypes.data, len(arr), out.ctypes.data)
        _check()
        return out

    def sampleScatterIsotropic_f32(self, ekin):
        arr = _np.ascontiguousarray(ekin, dtype=_np.float32)
        ef = _np.empty(len(arr), dtype=_np.float32)
        mu = _np.empty(len(arr), dtype=_np.float32)
        lib().ncgb_samplescatterisotropic_many_f32(self._h, arr.ctypes.data, len(arr), ef.ctypes.data,
                                                   mu.ctypes.data)
        _check()
        return ef, mu


class Absorption(Process):
    """A material's absorption process (NCrystal core.py's Absorption): the
    1/v model, cross-sections evaluated on the GPU."""

    def clone(self):
        h = lib().ncrystal_clone_absorption(self._h)
        _check()
        return Absorption(h, self._cfg)


def createAbsorption(cfgstr):
    """NCrystal.createAbsorption on the GPU path."""
    h = lib().ncrystal_create_absorption(cfgstr.encode())
    _check()
    if not h.internal:
        raise NCException("could not create absorption for %r" % cfgstr)
    return Absorption(h, cfgstr)


class Batch:
    """A ragged multi-material batch (ncgb_batch_*): neutrons [offsets[k],
    offsets[k+1]) belong to scatters[k].  Device entry points take torch CUDA
    tensors (ekin float64, offsets int64)."""

    def __init__(self, scatters):
        L = lib()
        self._scatters = list(scatters)   # keep the handles alive
        arr = (_Handle * len(self._scatters))(*[sc._h for sc in self._scatters])
        self._h = L.ncgb_batch_create(arr, len(self._scatters))
        _check()
        if not self._h.internal:
            raise NCException("could not create the batch")

    def __del__(self):
        try:
            if self._h is not None and self._h.internal:
                lib().ncgb_batch_destroy(_C.byref(self._h))
        except Exception:
            pass

    @property
    def nmat(self):
        return len(self._scatters)

    def set_mode(self, mode):
        """Arithmetic mode of the batch: "exact" or "mixed" (see Scatter.mode)."""
        if lib().ncgb_batch_set_mode(self._h, _mode_code(mode)):
            _check()
        return self

    def set_sampler(self, sampler):
        """"plain" or "learned" (proposals attached before the batch was made)."""
        if sampler not in SAMPLERS:
            raise NCBadInput("sampler must be one of %s" % sorted(SAMPLERS))
        if lib().ncgb_batch_set_sampler(self._h, SAMPLERS[sampler]):
            _check()
        return self

    def _args(self, ekin, offsets, xs, ef, mu, status, stream):
        import torch
        p = (lambda t: 0 if t is None else t.data_ptr())
        if stream is None:
            stream = torch.cuda.current_stream(ekin.device)
        return (self._h, ekin.data_ptr(), offsets.data_ptr(), ekin.numel(), p(xs), p(ef), p(mu), p(status),
                stream.cuda_stream)

    def scatter_device(self, ekin, offsets, xs=None, ekin_final=None, mu=None, status=None, stream=None):
        if lib().ncgb_batch_scatter_device(*self._args(ekin, offsets, xs, ekin_final, mu, status, stream)):
            _check()

    def graph_launch(self, ekin, offsets, xs=None, ekin_final=None, mu=None, status=None, stream=None):
        if lib().ncgb_batch_graph_launch(*self._args(ekin, offsets, xs, ekin_final, mu, status, stream)):
            _check()

    def autotune(self, ekin, offsets, xs, ekin_final, mu, stream=None):
        a = self._args(ekin, offsets, xs, ekin_final, mu, None, stream)
        if lib().ncgb_batch_autotune(*(a[:7] + a[8:])):
            _check()
        pb, sb = _C.c_int(), _C.c_int()
        lib().ncgb_batch_config(self._h, _C.byref(pb), _C.byref(sb))
        return pb.value, sb.value

    def split_lists(self):
        """Whether the batch's S(alpha,beta) queue uses two lists (the
        autotuner's choice)."""
        v = _C.c_int()
        if lib().ncgb_batch_split_lists(self._h, _C.byref(v)):
            _check()
        return bool(v.value)

    def set_split_lists(self, split):
        if lib().ncgb_batch_set_split_lists(self._h, 1 if split else 0):
            _check()
        return self

    def xs_scatter_host(self, ekin, offsets):
        e = _np.ascontiguousarray(ekin, dtype=_np.float64)
        off = _np.ascontiguousarray(offsets, dtype=_np.int64)
        n = len(e)
        xs, ef, mu = (_np.empty(n) for _ in range(3))
        lib().ncgb_batch_xs_scatter_many(self._h, e.ctypes.data, off.ctypes.data, n, xs.ctypes.data,
                                         ef.ctypes.data, mu.ctypes.data)
        _check()
        return xs, ef, mu

    def xs_scatter_host_ptr(self, ekin_ptr, offsets_ptr, n, xs_ptr, ef_ptr, mu_ptr):
        lib().ncgb_batch_xs_scatter_many(self._h, ekin_ptr, offsets_ptr, n, xs_ptr, ef_ptr, mu_ptr)
        _check()


class MLP:
    """The proposal network (ncgb_mlp_*): 4 hidden layers of 128, trained and
    evaluated on the current CUDA device by the library's own kernels."""

    def __init__(self, seed=1, emin=1e-5, emax=2.0, tmin=250.0, tmax=350.0):
        L = lib()
        self._h = L.ncgb_mlp_create(int(seed))
        _check()
        if not self._h.internal:
            raise NCException("could not create the network")
        self.ranges = (emin, emax, tmin, tmax)
        if L.ncgb_mlp_set_ranges(self._h, emin, emax, tmin, tmax):
            _check()

    def __del__(self):
        try:
            if self._h is not None and self._h.internal:
                lib().ncgb_mlp_destroy(_C.byref(self._h))
        except Exception:
            pass

    @staticmethod
    def nparams():
        return int(lib().ncgb_mlp_nparams())

    def params(self):
        out = _np.empty(self.nparams(), dtype=_np.float32)
        if lib().ncgb_mlp_get_params(self._h, out.ctypes.data):
            _check()
        return out

    def set_params(self, p):
        p = _np.ascontiguousarray(p, dtype=_np.float32)
        assert p.size == self.nparams()
        if lib().ncgb_mlp_set_params(self._h, p.ctypes.data):
            _check()

    def gradients(self, loge, temp, target):
        """(mean pinball loss, flat gradient) on float32 CUDA tensors."""
        g = _np.empty(self.nparams(), dtype=_np.float32)
        loss = _C.c_float()
        if lib().ncgb_mlp_gradients(self._h, loge.data_ptr(), temp.data_ptr(), target.data_ptr(), loge.numel(),
                                    g.ctypes.data, _C.byref(loss), None):
            _check()
        return loss.value, g

    def train(self, loge, temp, target, steps, batch=8192, lr=2e-3, seed=7, trace_every=0):
        ntr = steps // trace_every if trace_every else 0
        tr = _np.zeros(max(1, ntr), dtype=_np.float32)
        if lib().ncgb_mlp_train(self._h, loge.data_ptr(), temp.data_ptr(), target.data_ptr(), loge.numel(),
                                int(steps), int(batch), float(lr), int(seed), tr.ctypes.data if ntr else None,
                                int(trace_every), None):
            _check()
        return tr[:ntr]

    def knots(self, loge, temp):
        """(n, 62) asinh(beta) knots at float32 CUDA tensors (log E, T)."""
        import torch
        out = torch.empty((loge.numel(), 62), dtype=torch.float32, device=loge.device)
        if lib().ncgb_mlp_knots(self._h, loge.data_ptr(), temp.data_ptr(), loge.numel(), out.data_ptr(), None):
            _check()
        torch.cuda.synchronize()
        return out


def phase_timing(enable):
    """Switch CUDA-event timing of the two scatter kernels on or off."""
    lib().ncgb_phase_timing(1 if enable else 0)


def phase_times():
    """(ms in the pick pass, ms in the S(alpha,beta) pass, batches, SAB queue
    length of the last batch) since the last call; waits for the events."""
    a, b = _C.c_double(), _C.c_double()
    n, q = _C.c_ulong(), _C.c_ulong()
    if lib().ncgb_phase_times(_C.byref(a), _C.byref(b), _C.byref(n), _C.byref(q)):
        _check()
    return a.value, b.value, n.value, q.value


def bundle_path(cfgstr):
    """Path of the material bundle of a cfg-string (ncgb_bundle_path): found
    in the bundle directories, or exported there on demand through NCrystal's
    own material loading where an exporter library is available."""
    buf = _C.create_string_buffer(8192)
    if lib().ncgb_bundle_path(cfgstr.encode(), buf, len(buf)):
        _check()
    return buf.value.decode()


def createScatterFromBundle(path, seed=0):
    """A Scatter for the material of an explicit bundle file
    (ncgb_create_scatter_bundle)."""
    h = lib().ncgb_create_scatter_bundle(path.encode(), int(seed))
    _check()
    if not h.internal:
        raise NCException("could not create scatter from %r" % path)
    return Scatter(h, path)


def createScatter(cfgstr, seed=None):
    """NCrystal.createScatter (core.py:1602) on the GPU path.  'seed' selects
    the Philox key (ncrystal_create_scatter_builtinrng)."""
    L = lib()
    if seed is None:
        h = L.ncrystal_create_scatter(cfgstr.encode())
    else:
        h = L.ncrystal_create_scatter_builtinrng(cfgstr.encode(), int(seed))
    _check()
    if not h.internal:
        raise NCException("could not create scatter for %r" % cfgstr)
    return Scatter(h, cfgstr)


# Philox key of handles made without a seed (ncrystal_create_scatter).
_DEFAULT_SEED = 0x4e43727973746c21


def createScatters(cfgstrs, seed=None):
    """Scatter objects for many cfg-strings at once (ncgb_create_scatters):
    the S(alpha,beta) samplers of all the materials (a temperature grid, a
    set of crystals) are derived in one batched device derivation."""
    L = lib()
    cfgstrs = list(cfgstrs)
    n = len(cfgstrs)
    arr = (_C.c_char_p * max(n, 1))(*[c.encode() for c in cfgstrs])
    out = (_Handle * max(n, 1))()
    seed = _DEFAULT_SEED if seed is None else int(seed)
    if L.ncgb_create_scatters(arr, n, seed, out):
        _check()
        raise NCException("could not create scatters")
    return [Scatter(out[i], cfgstrs[i]) for i in range(n)]


def sab_derive_compare_many(bundle_paths):
    """ncgb_sab_derive_compare over every S(alpha,beta) component of many
    bundles, the device side as one batched derivation: dict with
    max_rel_diff, n_double_diff, n_int_mismatch, ncomp, ms_host, ms_device."""
    L = lib()
    paths = list(bundle_paths)
    arr = (_C.c_char_p * max(len(paths), 1))(*[p.encode() for p in paths])
    mr, ms_h, ms_d = _C.c_double(), _C.c_double(), _C.c_double()
    nd, ni, nc = _C.c_longlong(), _C.c_longlong(), _C.c_longlong()
    if L.ncgb_sab_derive_compare_many(arr, len(paths), _C.byref(mr), _C.byref(nd), _C.byref(ni), _C.byref(nc),
                                      _C.byref(ms_h), _C.byref(ms_d)):
        raise NCCalcError(L.ncgb_tables_lasterror().decode())
    return {"max_rel_diff": mr.value, "n_double_diff": nd.value, "n_int_mismatch": ni.value,
            "ncomp": nc.value, "ms_host": ms_h.value, "ms_device": ms_d.value}


def sab_derive_compare(bundle_path, comp):
    """Host- and device-derived S(alpha,beta) sampling tables of one
    component compared (ncgb_sab_derive_compare): dict with max_rel_diff,
    n_double_diff, n_int_mismatch, ms_host, ms_device."""
    L = lib()
    mr, ms_h, ms_d = _C.c_double(), _C.c_double(), _C.c_double()
    nd, ni = _C.c_longlong(), _C.c_longlong()
    if L.ncgb_sab_derive_compare(bundle_path.encode(), int(comp), _C.byref(mr), _C.byref(nd), _C.byref(ni),
                                 _C.byref(ms_h), _C.byref(ms_d)):
        raise NCCalcError(L.ncgb_tables_lasterror().decode())
    return {"max_rel_diff": mr.value, "n_double_diff": nd.value, "n_int_mismatch": ni.value,
            "ms_host": ms_h.value, "ms_device": ms_d.value}


def createProcess(cfgstr):
    return createScatter(cfgstr)
