"""Statistical parity at 1e8 events: GPU-sampled (E', mu) against the CPU
oracle's (a restatement of the reference sampler, pinned to it neutron by
neutron), with independent random streams, at fixed incident energies.

Binned chi-square on 2D (E', mu) histograms (Pearson two-sample statistic, as
NCrystal's hist.Hist.check_compat does for its tests, hist.py:810-903) and
two-sample Kolmogorov-Smirnov on E' and mu (scipy), p > 0.01 with a
Bonferroni correction over all comparisons of the module."""
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
NTESTS = 3 * (len(CASES) + len(CASES_MIXED))
ALPHA = 0.01 / NTESTS


def gpu_samples(cfg, e0, n, seed, mode="exact"):
    import torch
    sc = NC.createScatter(cfg, seed=seed).set_mode(mode)
    e = torch.full((n,), e0, dtype=torch.float64, device="cuda")
    ef = torch.empty_like(e)
    mu = torch.empty_like(e)
    st = torch.empty((n,), dtype=torch.int32, device="cuda")
    sc.scatter_device(e, None, ef, mu, st)
    torch.cuda.synchronize()
    assert int((st != 0).sum()) == 0
    return ef.cpu().numpy(), mu.cpu().numpy()


def oracle_samples(cfg, e0, n, seed):
    m = HostMaterial(bundle_path(cfg))
    nt = os.cpu_count() or 4
    chunks = np.array_split(np.arange(n), nt * 4)

    def work(idx):
        e = np.full(len(idx), e0)
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


def ks_two_sample_large(x, y, nsub=2_000_000, seed=0):
    """KS on random subsamples (scipy's exact two-sample KS on 1e8 points is
    needlessly slow; the chi-square uses all events)."""
    from scipy.stats import ks_2samp
    r = np.random.default_rng(seed)
    return ks_2samp(x[r.integers(0, len(x), nsub)], y[r.integers(0, len(y), nsub)]).pvalue


ALL = [(c, e, "exact") for c, e in CASES] + [(c, e, "mixed") for c, e in CASES_MIXED]


@pytest.mark.parametrize("cfg,e0,mode", ALL, ids=["%s@%g-%s" % (c.split(".")[0], e, m) for c, e, m in ALL])
def test_gpu_vs_oracle_distributions(cfg, e0, mode):
    pytest.importorskip("scipy")
    bundle_path(cfg)
    gef, gmu = gpu_samples(cfg, e0, N, seed=1001, mode=mode)
    oef, omu = oracle_samples(cfg, e0, N, seed=2002)
    # 2D histogram in (log E'/E, mu): 60 x 50 bins, edges from the pooled range
    lg = np.log(np.maximum(gef, 1e-30) / e0)
    lo = np.log(np.maximum(oef, 1e-30) / e0)
    lo_edges = np.quantile(np.concatenate([lg[:10 ** 6], lo[:10 ** 6]]), np.linspace(0, 1, 61))
    lo_edges = np.unique(lo_edges)
    mu_edges = np.linspace(-1, 1, 51)
    hg, _, _ = np.histogram2d(lg, gmu, bins=[lo_edges, mu_edges])
    ho, _, _ = np.histogram2d(lo, omu, bins=[lo_edges, mu_edges])
    stat, dof, p = chi2_two_sample(hg.ravel(), ho.ravel())
    assert p > ALPHA, "chi2=%.1f dof=%d p=%.3g" % (stat, dof, p)
    assert ks_two_sample_large(gef, oef) > ALPHA
    assert ks_two_sample_large(gmu, omu, seed=1) > ALPHA
