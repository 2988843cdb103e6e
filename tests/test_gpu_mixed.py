"""Mixed-precision mode (NCGB_MODE_MIXED): FP32 incoherent-elastic
exponentials and FP32 log-linear alpha inversion, FP64 elsewhere.

Cross-sections are compared with the CPU oracle (FP64) at a stated relative
tolerance; per-neutron samples on the same random streams must agree with the
oracle to FP32-level tolerances for nearly every neutron (a rejection decision
or a table-bin choice within ~1e-7 of its edge may flip).  The sampled
distributions are checked at 1e8 events in test_gpu_statistics.py."""
import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.workloads as W
from conftest import bundle_path
from oracle.pyoracle import HostMaterial

pytestmark = pytest.mark.gpu

# The bar the mixed mode is held to: 1e-6 relative to the FP64 oracle.  Its
# FP32 terms (one expm1f per incoherent-elastic element, the S(alpha,beta)
# interpolation, the composition sum) each carry a few ulp of 2^-24 (~2e-7).
XS_RTOL_MIXED = 1e-6
# Sampled E' and mu carry the FP32 error of the alpha inversion (relative
# ~1e-7 in alpha, amplified by at most a few in E' and mu).
VAL_RTOL_MIXED = 1e-5
MU_ATOL_MIXED = 1e-5
MIN_AGREE_MIXED = 0.99

CFGS = [W.AL, W.AL2O3, W.PE293, W.WATER, "Cu_sg225.ncmat;temp=77K"]


def _mixed(cfg, seed):
    return NC.createScatter(cfg, seed=seed).set_mode("mixed")


@pytest.mark.parametrize("cfg", CFGS, ids=[c.split(".")[0] for c in CFGS])
def test_mixed_xs_within_tolerance(cfg):
    m = HostMaterial(bundle_path(cfg))
    e = np.concatenate([W.loguniform_energies(200000, 1e-6, 5.0, 61), W.al_wavelength_energies(20000, 62)])
    xs = _mixed(cfg, 1).crossSectionIsotropic(e)
    np.testing.assert_allclose(xs, m.xs(e), rtol=XS_RTOL_MIXED, atol=0)


def test_mixed_xs_f32_io_within_tolerance():
    """The FP32 entry point of the large Al2O3 workload (energies and results
    in FP32): cross-sections against the oracle's FP64 values at the same
    FP32-rounded energies, within the same bar."""
    import torch
    m = HostMaterial(bundle_path(W.AL2O3))
    e = W.loguniform_energies(300000, 1e-4, 1.0, 66).astype(np.float32)
    sc = _mixed(W.AL2O3, 2)
    d_e = torch.as_tensor(e, device="cuda")
    xs = torch.empty_like(d_e)
    sc.scatter_device(d_e, xs, None, None, None)
    torch.cuda.synchronize()
    np.testing.assert_allclose(xs.cpu().numpy().astype(np.float64), m.xs(e.astype(np.float64)),
                               rtol=XS_RTOL_MIXED, atol=0)


@pytest.mark.parametrize("cfg", CFGS, ids=[c.split(".")[0] for c in CFGS])
def test_mixed_samples_vs_oracle(cfg):
    m = HostMaterial(bundle_path(cfg))
    e = np.concatenate([W.loguniform_energies(100000, 1e-5, 3.0, 63), W.al_wavelength_energies(20000, 64)])
    ef, mu = _mixed(cfg, 99).sampleScatterIsotropic(e)
    oef, omu, ost, _ = m.scatter(e, 99)
    assert np.all(ost == 0)
    assert np.all(np.isfinite(ef)) and np.all(ef >= 0)
    assert np.all(np.abs(mu) <= 1.0)
    ok = np.isclose(ef, oef, rtol=VAL_RTOL_MIXED, atol=1e-300) & np.isclose(mu, omu, rtol=0, atol=MU_ATOL_MIXED)
    assert ok.mean() >= MIN_AGREE_MIXED, ok.mean()


def test_mode_switch_and_inheritance():
    sc = NC.createScatter(W.PE293, seed=5)
    assert sc.mode == "exact"
    sc.set_mode("mixed")
    assert sc.mode == "mixed"
    assert sc.clone(rng_stream_index=3).mode == "mixed"
    with pytest.raises(NC.NCBadInput):
        sc.set_mode("half")
    sc.set_mode("exact")
    e = W.loguniform_energies(5000, 1e-4, 1.0, 65)
    exact = NC.createScatter(W.PE293, seed=5)
    np.testing.assert_array_equal(sc.crossSectionIsotropic(e), exact.crossSectionIsotropic(e))


def test_mixed_batch_matches_mixed_single_calls():
    import torch
    cfgs = [W.AL2O3, W.PE293]
    counts = [30000, 50000]
    energies = [W.loguniform_energies(n, 1e-4, 1.0, 70 + k) for k, n in enumerate(counts)]
    e_all = torch.as_tensor(np.concatenate(energies), device="cuda")
    off = torch.as_tensor(np.concatenate([[0], np.cumsum(counts)]), dtype=torch.int64, device="cuda")
    batch = NC.Batch([NC.createScatter(c, seed=21 + k) for k, c in enumerate(cfgs)]).set_mode("mixed")
    xs, ef, mu = (torch.empty_like(e_all) for _ in range(3))
    batch.scatter_device(e_all, off, xs, ef, mu)
    torch.cuda.synchronize()
    o = np.concatenate([[0], np.cumsum(counts)])
    for k, c in enumerate(cfgs):
        sxs, sef, smu = _mixed(c, 21 + k).xs_scatter(energies[k])
        np.testing.assert_array_equal(xs[o[k]:o[k + 1]].cpu().numpy(), sxs)
        np.testing.assert_array_equal(ef[o[k]:o[k + 1]].cpu().numpy(), sef)
        np.testing.assert_array_equal(mu[o[k]:o[k + 1]].cpu().numpy(), smu)
