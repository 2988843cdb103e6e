"""The fused host-array calls (ncgb_xs_scatter_many, _f32, and the ragged
batch's ncgb_batch_xs_scatter_many) on pinned host memory, where the kernels
read and write the caller's arrays directly over NVLink-C2C, give the same
results as the chunked-copy path on pageable arrays (same random streams:
neutron i of a call uses stream index i).  NCGB_ZERO_COPY=1 forces the
zero-copy path (by default only the FP32 call takes it)."""
import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.workloads as W
from conftest import bundle_path

pytestmark = pytest.mark.gpu


def _pinned(n, dtype):
    import torch
    return torch.empty(n, dtype=dtype).pin_memory()


@pytest.fixture(autouse=True)
def _zero_copy_on(monkeypatch):
    monkeypatch.setenv("NCGB_ZERO_COPY", "1")


@pytest.mark.parametrize("f32", [False, True])
def test_zero_copy_equals_copy_path(f32):
    import torch
    cfg = W.PE293
    bundle_path(cfg)
    n = (1 << 23) + 12345           # larger than one copy chunk (2^22)
    e = W.loguniform_energies(n, 1e-4, 1.0, 11).astype(np.float32 if f32 else np.float64)
    # pageable arrays: the chunked copy path
    xs1, ef1, mu1 = NC.createScatter(cfg, seed=5).xs_scatter(e)
    # pinned arrays: zero-copy
    dt = torch.float32 if f32 else torch.float64
    he = torch.from_numpy(e).pin_memory()
    hx, hf, hm = _pinned(n, dt), _pinned(n, dt), _pinned(n, dt)
    NC.createScatter(cfg, seed=5).xs_scatter_host_ptr(he.data_ptr(), n, hx.data_ptr(), hf.data_ptr(),
                                                      hm.data_ptr(), f32)
    np.testing.assert_array_equal(hx.numpy(), xs1)
    np.testing.assert_array_equal(hf.numpy(), ef1)
    np.testing.assert_array_equal(hm.numpy(), mu1)


def test_zero_copy_batch_equals_copy_path():
    import torch
    cfgs = [W.PE293, W.AL, W.WATER]
    for c in cfgs:
        bundle_path(c)
    counts = [300000, 5000000, 123457]
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    n = int(offs[-1])
    e = W.loguniform_energies(n, 1e-5, 2.0, 12)
    out = {}
    for pinned in (False, True):
        b = NC.Batch([NC.createScatter(c, seed=9) for c in cfgs])
        if pinned:
            he, ho = torch.from_numpy(e).pin_memory(), torch.from_numpy(offs).pin_memory()
            arrs = [_pinned(n, torch.float64) for _ in range(3)]
            b.xs_scatter_host_ptr(he.data_ptr(), ho.data_ptr(), n, *(a.data_ptr() for a in arrs))
            out[pinned] = [a.numpy().copy() for a in arrs]
        else:
            arrs = [np.empty(n) for _ in range(3)]
            b.xs_scatter_host_ptr(e.ctypes.data, offs.ctypes.data, n, *(a.ctypes.data for a in arrs))
            out[pinned] = arrs
    for a, b_ in zip(out[False], out[True]):
        np.testing.assert_array_equal(a, b_)
