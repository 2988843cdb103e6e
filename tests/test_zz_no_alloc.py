"""The allocation-free device entry point (ncgb_scatter_device_noalloc).

It serves callers that may not allocate device memory while they run (a
transport code inside a framework that owns all device memory, or one that
cannot take cudaMalloc's synchronisation in its loop).  Called through the C
ABI, it must give the same results as ncgb_scatter_device on the same random
streams, on two calls in a row (its fixed working memory keeps the previous
call's contents), must not change the device's free memory, and must refuse
batches above its fixed capacity.

This file is collected last, so that a run stopping at the first failure has
run every other test already.
"""
import ctypes as C

import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.workloads as W
from conftest import bundle_path

pytestmark = pytest.mark.gpu

XS_RTOL = 1e-12
SEED = 31337


def _lib():
    L = NC.lib()
    f = L.ncgb_scatter_device_noalloc
    f.restype = C.c_int
    f.argtypes = [NC.core._Handle, C.c_void_p, C.c_ulong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    return L


def _outputs(torch, n):
    return (torch.empty(n, dtype=torch.float64, device="cuda"),
            torch.empty(n, dtype=torch.float64, device="cuda"),
            torch.empty(n, dtype=torch.float64, device="cuda"),
            torch.empty(n, dtype=torch.int32, device="cuda"))


@pytest.mark.parametrize("cfg", [W.AL2O3, W.PE293])
def test_noalloc_matches_allocating_entry_point(cfg):
    import torch
    bundle_path(cfg)
    L = _lib()
    n = 300000
    e = torch.as_tensor(W.loguniform_energies(n, 1e-4, 1.0, 77), dtype=torch.float64, device="cuda")
    ref = NC.createScatter(cfg, seed=SEED)   # uses ncgb_scatter_device
    na = NC.createScatter(cfg, seed=SEED)    # uses ncgb_scatter_device_noalloc
    stream = torch.cuda.current_stream().cuda_stream
    rx, ref_ef, rm, rs = _outputs(torch, n)
    ax, af, am, ast = _outputs(torch, n)
    for call in range(2):
        assert L.ncgb_scatter_device(ref._h, e.data_ptr(), n, rx.data_ptr(), ref_ef.data_ptr(), rm.data_ptr(),
                                     rs.data_ptr(), stream) == 0
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.ncgb_scatter_device_noalloc(na._h, e.data_ptr(), n, ax.data_ptr(), af.data_ptr(), am.data_ptr(),
                                           ast.data_ptr(), stream)
        assert rc == 0, L.ncrystal_lasterror()
        torch.cuda.synchronize()
        if call == 1:
            # set-up is done by the first call; later calls must not allocate
            assert torch.cuda.mem_get_info()[0] == free_before
        assert torch.equal(ast, rs) and int((ast != 0).sum()) == 0
        np.testing.assert_allclose(ax.cpu().numpy(), rx.cpu().numpy(), rtol=XS_RTOL, atol=0)
        np.testing.assert_allclose(af.cpu().numpy(), ref_ef.cpu().numpy(), rtol=XS_RTOL, atol=0)
        np.testing.assert_allclose(am.cpu().numpy(), rm.cpu().numpy(), rtol=0, atol=1e-12)


def test_noalloc_follows_mode_and_skips_empty_calls():
    """A handle in the mixed mode gets the mixed mode here too, and an empty
    call consumes no call sequence number: after one, the next call draws the
    same random streams as the allocating entry point's first call."""
    import torch
    bundle_path(W.PE293)
    L = _lib()
    n = 100000
    e = torch.as_tensor(W.loguniform_energies(n, 1e-4, 1.0, 78), dtype=torch.float64, device="cuda")
    ref = NC.createScatter(W.PE293, seed=SEED).set_mode("mixed")
    na = NC.createScatter(W.PE293, seed=SEED).set_mode("mixed")
    stream = torch.cuda.current_stream().cuda_stream
    rx, ref_ef, rm, rs = _outputs(torch, n)
    ax, af, am, ast = _outputs(torch, n)
    assert L.ncgb_scatter_device_noalloc(na._h, e.data_ptr(), 0, None, None, None, None, stream) == 0
    assert L.ncgb_scatter_device(ref._h, e.data_ptr(), n, rx.data_ptr(), ref_ef.data_ptr(), rm.data_ptr(),
                                 rs.data_ptr(), stream) == 0
    assert L.ncgb_scatter_device_noalloc(na._h, e.data_ptr(), n, ax.data_ptr(), af.data_ptr(), am.data_ptr(),
                                         ast.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert torch.equal(ast, rs) and int((ast != 0).sum()) == 0
    assert torch.equal(ax, rx) and torch.equal(af, ref_ef) and torch.equal(am, rm)


def test_noalloc_refuses_batches_above_capacity():
    import torch
    bundle_path(W.AL)
    L = _lib()
    cap = 1048576
    sc = NC.createScatter(W.AL, seed=1)
    e = torch.full((cap + 1,), 0.025, dtype=torch.float64, device="cuda")
    ef = torch.empty_like(e)
    mu = torch.empty_like(e)
    rc = L.ncgb_scatter_device_noalloc(sc._h, e.data_ptr(), cap + 1, None, ef.data_ptr(), mu.data_ptr(), None,
                                       torch.cuda.current_stream().cuda_stream)
    assert rc != 0
    assert L.ncrystal_lasterrortype() == b"BadInput"
    assert b"1048576" in L.ncrystal_lasterror()
    L.ncrystal_clearerror()
    # a batch at the capacity runs
    rc = L.ncgb_scatter_device_noalloc(sc._h, e.data_ptr(), cap, None, ef.data_ptr(), mu.data_ptr(), None,
                                       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == 0
    assert float(mu[:cap].abs().max()) <= 1.0
