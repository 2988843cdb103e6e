"""The learned beta proposal: training set, training and attachment.

The training set is drawn by the plain GPU sampler of one S(alpha,beta)
component (ncgb_sab_sample_device) over instances of a material at several
temperatures; the network (ncgb_mlp_*) learns the quantiles of asinh(beta) at
62 levels as a function of (log E, T) by quantile regression.  Attached to a
component, the network is evaluated once per sampler energy (egrid point) of
the instance's temperature, and its knots become the intervals of an exact
rejection envelope for beta (see include/ncrystal_gb300.h, Part 3).

    nets = train_proposals(pe_cfg, TRAIN_TEMPS)        # {component: MLP}
    sc = NC.createScatter(pe_cfg(293))
    attach(sc, nets); sc.set_sampler("learned")
"""
import ctypes as _C
import os
import time

import numpy as np

from . import core
from . import _build
from .workloads import PE_TRAIN_TEMPS as TRAIN_TEMPS, pe_cfg

# Energy range (eV) of the training energies (log-uniform).
TRAIN_EMIN, TRAIN_EMAX = 1e-5, 2.0


def training_cfgs(cfg_of_t=pe_cfg, temps=TRAIN_TEMPS):
    return [cfg_of_t(T) for T in temps]


def training_set(cfgs, comp, n_total, emin=TRAIN_EMIN, emax=TRAIN_EMAX, seed=0x7EA1):
    """Device tensors (log E, T, asinh(beta)) of n_total samples of component
    'comp', split evenly over the material instances 'cfgs'.  Samples whose
    sampling failed are dropped."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    per = n_total // len(cfgs)
    loge, temp, tgt = [], [], []
    rng = np.random.default_rng(seed)
    for k, cfg in enumerate(cfgs):
        sc = core.createScatter(cfg, seed=seed + 101 * k)
        T = sc.material_info()[1]
        e = torch.from_numpy(np.exp(rng.uniform(np.log(emin), np.log(emax), per))).to(dev)
        a = torch.empty_like(e)
        b = torch.empty_like(e)
        st = torch.empty(per, dtype=torch.int32, device=dev)
        sc.sab_sample_device(comp, e, a, b, st)
        ok = st == 0
        loge.append(torch.log(e[ok]).float())
        temp.append(torch.full((int(ok.sum()),), T, dtype=torch.float32, device=dev))
        tgt.append(torch.asinh(b[ok]).float())
        del sc
    torch.cuda.synchronize()
    return torch.cat(loge), torch.cat(temp), torch.cat(tgt)


def train_component(cfgs, comp, n_total=1 << 26, steps=6000, batch=8192, lr=2e-3, seed=11,
                    emin=TRAIN_EMIN, emax=TRAIN_EMAX, trace_every=500):
    """-> (MLP, info dict) for component 'comp' of the material instances."""
    import torch
    t0 = time.perf_counter()
    loge, temp, tgt = training_set(cfgs, comp, n_total, emin, emax, seed=seed * 7919)
    t1 = time.perf_counter()
    temps = sorted({float(t) for t in temp[:: max(1, temp.numel() // 4096)].cpu().numpy()})
    net = core.MLP(seed=seed, emin=emin, emax=emax, tmin=min(temps), tmax=max(temps))
    trace = net.train(loge, temp, tgt, steps=steps, batch=batch, lr=lr, seed=seed, trace_every=trace_every)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    info = {"samples": int(loge.numel()), "steps": steps, "batch": batch, "sample_s": t1 - t0, "train_s": t2 - t1,
            "loss_trace": [float(x) for x in trace]}
    del loge, temp, tgt
    return net, info


def train_proposals(cfg_of_t=pe_cfg, temps=TRAIN_TEMPS, **kw):
    """One network per S(alpha,beta) component of the material:
    -> ({component index: MLP}, {component index: info})."""
    cfgs = training_cfgs(cfg_of_t, temps)
    probe = core.createScatter(cfgs[0])
    nets, infos = {}, {}
    for comp in probe.sab_components():
        nets[comp], infos[comp] = train_component(cfgs, comp, **kw)
    return nets, infos


def attach(sc, nets, min_accept=0.5):
    """Attach {component: MLP} to the handle's material; -> {component: mean
    envelope acceptance}."""
    return {comp: sc.attach_proposal(comp, net, min_accept) for comp, net in nets.items()}


# ---- reference partitions (for comparisons with the network) --------------------
class _Tables:
    """Host copy of a material's tables through the library's host API."""

    def __init__(self, cfg):
        L = core.lib()
        L.ncgb_tables_load.restype = _C.c_void_p
        path = os.path.join(_build.BUNDLES, _build.bundle_file_name(cfg))
        self.h = L.ncgb_tables_load(path.encode())
        if not self.h:
            raise core.NCFileNotFound(L.ncgb_tables_lasterror().decode())

    def array(self, comp, name, dtype):
        L = core.lib()
        p, n = _C.c_void_p(), _C.c_ulong()
        if L.ncgb_tables_array(self.h, comp, name.encode(), _C.byref(p), _C.byref(n)):
            raise KeyError(name)
        return np.ctypeslib.as_array(_C.cast(p, _C.POINTER(np.ctypeslib.as_ctypes_type(dtype))),
                                     (n.value,)).copy()

    def __del__(self):
        try:
            core.lib().ncgb_tables_free(_C.c_void_p(self.h))
        except Exception:
            pass


def reference_knots(cfg, comp, kind):
    """(ne, 62) asinh(beta) knots without the network: 'uniform' (equal-width
    intervals over each sampler's regular beta range) or 'quantile' (the exact
    quantiles of the sampler's own beta distribution)."""
    t = _Tables(cfg)
    off = t.array(comp, "smp_offset", np.int64)
    nb = t.array(comp, "smp_nbeta", np.int32)
    kind_ = t.array(comp, "smp_kind", np.int32)
    fbkep = t.array(comp, "smp_fbkep", np.float64)
    bx = t.array(comp, "bx", np.float64)
    bcdf = t.array(comp, "bcdf", np.float64)
    ne = len(off)
    out = np.zeros((ne, 62), dtype=np.float32)
    levels = np.arange(1, 63) / 63.0
    for i in range(ne):
        if kind_[i] == 0 or nb[i] < 3:
            continue
        x = bx[off[i]:off[i] + nb[i]]
        c = bcdf[off[i]:off[i] + nb[i]]
        fr = 1 if fbkep[i] <= 0 else 0
        lo, hi = x[fr], x[-1]
        if kind == "uniform":
            q = lo + (hi - lo) * levels
        elif kind == "quantile":
            cc = (c[fr:] - c[fr]) / max(c[-1] - c[fr], 1e-300)
            q = np.interp(levels, cc, x[fr:])
        else:
            raise ValueError(kind)
        out[i] = np.arcsinh(q).astype(np.float32)
    return out
