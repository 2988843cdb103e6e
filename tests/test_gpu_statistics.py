"""Statistical parity at 1e8 events: GPU-sampled (E', mu) against the CPU
oracle's (a restatement of the reference sampler, pinned to it neutron by
neutron), with independent random streams.

Cases: fixed incident energies, and the benchmark workloads' own energy
distribution (log-uniform in [1e-4, 1] eV; the GPU and the oracle each draw
their own 1e8 energies from it, so the two samples are independent draws of
the same joint distribution of (E, E', mu)).

Binned chi-square on (E', mu) histograms (Pearson two-sample statistic, as
NCrystal's hist.Hist.check_compat does for its tests, hist.py:810-903) and
exact two-sample Kolmogorov-Smirnov on E' and mu over all events (the two
empirical CDFs compared at every sample point), p > 0.01 with a Bonferroni
correction over all comparisons of the module."""
import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.workloads as W
from conftest import bundle_path
from oracle.pyoracle import HostMaterial

pytestmark = pytest.mark.gpu

N = 10 ** 8
CASES = [(W.PE293, 0.001), (W.PE293, 0.0253), (W.PE293, 0.5), (W.AL2O3, 0.0253), (W.AL2O3, 0.2)]
# the mixed-precision mode must sample the same distributions
CASES_MIXED = [(W.PE293, 0.0253), (W.AL2O3, 0.0253)]
# the benchmark workloads' energy distribution: polyethylene (FP64 I/O) in both
# modes, Al2O3 with dcutoff 0.2 through the FP32 entry point in the mixed mode
LOGU = (1e-4, 1.0)
CASES_LOGU = [(W.PE293, "exact", False), (W.PE293, "mixed", False), (W.AL2O3, "mixed", True)]
# comparisons per case: chi-square, KS on E', KS on mu
NTESTS = 3 * (len(CASES) + len(CASES_MIXED) + len(CASES_LOGU))
ALPHA = 0.01 / NTESTS


def scatter_device(sc, e):
    """(E', mu) on the device for the device array e (FP64, or FP32 through
    the FP32 entry point); no neutron may fail."""
    import torch
    ef = torch.empty_like(e)
    mu = torch.empty_like(e)
    st = torch.empty(e.shape, dtype=torch.int32, device=e.device)
    sc.scatter_device(e, None, ef, mu, st)
    torch.cuda.synchronize()
    assert int((st != 0).sum()) == 0
    return ef.double(), mu.double()


def gpu_samples(cfg, e0, n, seed, mode="exact"):
    import torch
    sc = NC.createScatter(cfg, seed=seed).set_mode(mode)
    e = torch.full((n,), e0, dtype=torch.float64, device="cuda")
    ef, mu = scatter_device(sc, e)
    return ef.cpu().numpy(), mu.cpu().numpy()


def oracle_samples(cfg, e0, n, seed, energies=None):
    """The oracle's (E', mu) at the fixed energy e0, or at energies[i] for
    neutron i; all host threads, neutron i on stream i whatever the split."""
    m = HostMaterial(bundle_path(cfg))
    nt = os.cpu_count() or 4
    chunks = np.array_split(np.arange(n), nt * 4)

    def work(idx):
        e = np.full(len(idx), e0) if energies is None else np.ascontiguousarray(energies[idx[0]:idx[-1] + 1])
        ef, mu, st, _ = m.scatter(e, seed, index_offset=int(idx[0]))
        assert np.all(st == 0)
        return ef, mu
    with ThreadPoolExecutor(max_workers=nt) as ex:
        res = list(ex.map(work, chunks))
    return np.concatenate([r[0] for r in res]), np.concatenate([r[1] for r in res])


def chi2_two_sample(a, b):
    """Pearson chi-square for two histograms of (possibly) different totals."""
    from scipy.stats import chi2
    na, nb = a.sum(), b.sum()
    m = (a + b) > 0
    a, b = a[m].astype(float), b[m].astype(float)
    ka, kb = np.sqrt(nb / na), np.sqrt(na / nb)
    stat = np.sum((ka * a - kb * b) ** 2 / (a + b))
    dof = int(m.sum()) - 1
    return stat, dof, chi2.sf(stat, dof)


def ks_two_sample(x, y, chunk=1 << 24):
    """Exact two-sample KS statistic over all points of both samples (sorted
    on the GPU; the empirical CDFs compared at every sample point, ties
    included), with scipy's asymptotic p-value for it (ks_2samp's 'asymp'
    method: the Kolmogorov distribution at n_eff = n m / (n + m))."""
    import torch
    from scipy.stats import kstwo
    xs = torch.sort(torch.as_tensor(np.asarray(x, dtype=np.float64), device="cuda"))[0]
    ys = torch.sort(torch.as_tensor(np.asarray(y, dtype=np.float64), device="cuda"))[0]
    n, m = xs.numel(), ys.numel()
    d = 0.0
    for pts in (xs, ys):
        for s in range(0, pts.numel(), chunk):
            p = pts[s:s + chunk]
            fx = torch.searchsorted(xs, p, right=True).double() / n
            fy = torch.searchsorted(ys, p, right=True).double() / m
            d = max(d, float((fx - fy).abs().max()))
    del xs, ys
    torch.cuda.empty_cache()
    en = n * m / (n + m)
    return d, float(kstwo.sf(d, round(en)))


def check_same_distribution(gef, gmu, oef, omu, e_ref, alpha, ge=None, oe=None):
    """chi-square on (log E'/E, mu) [x log E bins when the energies vary] and
    exact KS on E' and mu; e_ref: the fixed energy, or None with ge/oe the
    incident energies of the two samples."""
    gr = np.log(np.maximum(gef, 1e-30) / (e_ref if ge is None else ge))
    orr = np.log(np.maximum(oef, 1e-30) / (e_ref if oe is None else oe))
    r_edges = np.unique(np.quantile(np.concatenate([gr[:10 ** 6], orr[:10 ** 6]]), np.linspace(0, 1, 61)))
    mu_edges = np.linspace(-1, 1, 51)
    if ge is None:
        hg, _ = np.histogramdd((gr, gmu), bins=[r_edges, mu_edges])
        ho, _ = np.histogramdd((orr, omu), bins=[r_edges, mu_edges])
    else:
        le = np.linspace(math.log(LOGU[0]), math.log(LOGU[1]), 11)
        r_edges = np.unique(np.quantile(np.concatenate([gr[:10 ** 6], orr[:10 ** 6]]), np.linspace(0, 1, 41)))
        mu_edges = np.linspace(-1, 1, 26)
        hg, _ = np.histogramdd((np.log(ge), gr, gmu), bins=[le, r_edges, mu_edges])
        ho, _ = np.histogramdd((np.log(oe), orr, omu), bins=[le, r_edges, mu_edges])
    stat, dof, p = chi2_two_sample(hg.ravel(), ho.ravel())
    assert p > alpha, "chi2=%.1f dof=%d p=%.3g" % (stat, dof, p)
    d1, p1 = ks_two_sample(gef, oef)
    assert p1 > alpha, "KS on E': D=%.3g p=%.3g" % (d1, p1)
    d2, p2 = ks_two_sample(gmu, omu)
    assert p2 > alpha, "KS on mu: D=%.3g p=%.3g" % (d2, p2)
    return {"chi2_p": p, "ks_ef": (d1, p1), "ks_mu": (d2, p2)}


ALL = [(c, e, "exact") for c, e in CASES] + [(c, e, "mixed") for c, e in CASES_MIXED]


@pytest.mark.parametrize("cfg,e0,mode", ALL, ids=["%s@%g-%s" % (c.split(".")[0], e, m) for c, e, m in ALL])
def test_gpu_vs_oracle_distributions(cfg, e0, mode):
    pytest.importorskip("scipy")
    bundle_path(cfg)
    gef, gmu = gpu_samples(cfg, e0, N, seed=1001, mode=mode)
    oef, omu = oracle_samples(cfg, e0, N, seed=2002)
    print(check_same_distribution(gef, gmu, oef, omu, e0, ALPHA))


@pytest.mark.parametrize("cfg,mode,f32", CASES_LOGU,
                         ids=["%s-loguniform-%s%s" % (c.split(".")[0], m, "-f32" if f else "")
                              for c, m, f in CASES_LOGU])
def test_gpu_vs_oracle_workload_distribution(cfg, mode, f32):
    """1e8 neutrons at the benchmark workloads' energy distribution; the FP32
    case rounds its energies to FP32 first (the oracle gets the same rounded
    values' distribution)."""
    pytest.importorskip("scipy")
    import torch
    bundle_path(cfg)
    ge = W.loguniform_energies(N, LOGU[0], LOGU[1], 0x57A7001)
    oe = W.loguniform_energies(N, LOGU[0], LOGU[1], 0x57A7002)
    if f32:
        ge = ge.astype(np.float32).astype(np.float64)
        oe = oe.astype(np.float32).astype(np.float64)
    sc = NC.createScatter(cfg, seed=1003).set_mode(mode)
    e = torch.as_tensor(ge.astype(np.float32) if f32 else ge, device="cuda")
    gef, gmu = scatter_device(sc, e)
    gef, gmu = gef.cpu().numpy(), gmu.cpu().numpy()
    del e
    oef, omu = oracle_samples(cfg, None, N, seed=2004, energies=oe)
    if f32:
        # the GPU returns FP32 results: compare like with like
        oef = oef.astype(np.float32).astype(np.float64)
        omu = omu.astype(np.float32).astype(np.float64)
    print(check_same_distribution(gef, gmu, oef, omu, None, ALPHA, ge=ge, oe=oe))
