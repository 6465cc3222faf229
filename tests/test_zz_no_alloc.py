"""The allocation-free Hogbom entry point, called through the C ABI.

cr_hogbom_noalloc serves callers that may not allocate device memory while
they run (a fixed device-memory budget reserved at start-up, or a process in
which another allocator holds the device's memory).  Its scratch is a fixed
array in the library's device memory, shared by every call on the device.
This test runs it twice in a row on different inputs and checks each call
against the ordinary entry point, cr_hogbom, bit for bit (the Hogbom path's
tolerance): a second call must not see the first call's barrier, candidates
or components.  It also checks that a call leaves both the context's
workspaces and the device's free memory unchanged, that a budget of exactly
16384 components (the scratch's limit) runs, and that a budget beyond it is
rejected.  The file sorts last so that a run stopping at the first failure
has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import casars_cuda as cc
from casars_cuda import _lib

pytestmark = pytest.mark.gpu


def _inputs(seed, shape):
    rng = np.random.default_rng(seed)
    nx, ny = shape
    x = np.arange(nx)[:, None] - nx // 2
    y = np.arange(ny)[None, :] - ny // 2
    psf = np.exp(-(x * x + y * y) / 15.0).astype(np.float32)
    psf += (0.02 * rng.normal(size=shape)).astype(np.float32)
    psf[nx // 2, ny // 2] = 1.0
    res = (0.01 * rng.normal(size=shape)).astype(np.float32)
    for _ in range(10):
        px, py = rng.integers(8, nx - 8), rng.integers(8, ny - 8)
        res[px, py] += rng.uniform(0.1, 1.0)
    mask = (rng.uniform(size=shape) > 0.03).astype(np.uint8)
    return res, psf, mask


def _run(ctx, name, res, psf, mask, niter, gain=0.1, threshold=0.002):
    nx, ny = res.shape
    dev = torch.device("cuda", 0)
    model_t = torch.zeros((nx, ny), dtype=torch.float32, device=dev)
    res_t = torch.as_tensor(res, device=dev).clone()
    psf_t = torch.as_tensor(psf, device=dev)
    mask_t = torch.as_tensor(mask, device=dev)
    cap = niter + 1
    cx, cy = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
    cp, cf = np.zeros(cap, np.float32), np.zeros(cap, np.float32)
    actual, reported, stop = C.c_int64(), C.c_int64(), C.c_int32()
    torch.cuda.synchronize()
    ctx.use_own_stream()
    common = (model_t.data_ptr(), res_t.data_ptr(), psf_t.data_ptr(), mask_t.data_ptr(), nx, ny)
    tail = (gain, threshold, 0.0, 0.0, niter, 1, cx.ctypes.data, cy.ctypes.data, cp.ctypes.data,
            cf.ctypes.data, C.byref(actual), C.byref(reported), C.byref(stop))
    if name == "cr_hogbom":
        _lib.call(name, ctx.handle, *common, _lib.CR_DEVICE, *tail)
    else:
        _lib.call(name, ctx.handle, *common, *tail)
    ctx.synchronize()
    k = actual.value
    return dict(model=model_t.cpu().numpy(), residual=res_t.cpu().numpy(), x=cx[:k], y=cy[:k],
                peak=cp[:k], flux=cf[:k], actual=k, reported=reported.value, stop=stop.value)


def test_noalloc_matches_cr_hogbom_on_two_calls_in_a_row():
    ctx = cc.Context(0)
    try:
        for seed, shape, niter in ((5, (160, 128), 400), (6, (96, 96), 150)):
            res, psf, mask = _inputs(seed, shape)
            ref = _run(ctx, "cr_hogbom", res, psf, mask, niter)
            got = _run(ctx, "cr_hogbom_noalloc", res, psf, mask, niter)
            assert got["actual"] == ref["actual"] > 0
            assert got["reported"] == ref["reported"] and got["stop"] == ref["stop"]
            for key in ("x", "y", "peak", "flux", "model", "residual"):
                np.testing.assert_array_equal(got[key], ref[key])
    finally:
        ctx.close()


def test_noalloc_rejects_budget_beyond_its_scratch():
    ctx = cc.Context(0)
    try:
        res, psf, mask = _inputs(7, (32, 32))
        with pytest.raises(cc.CasarsCudaError) as e:
            _run(ctx, "cr_hogbom_noalloc", res, psf, mask, 16384)
        assert e.value.kind == "InvalidRequest" and "16384" in str(e.value)
    finally:
        ctx.close()


def test_noalloc_allocates_nothing():
    """A fresh context holds no workspace; a call through the C ABI with all
    buffers already in place leaves the context's workspaces empty and the
    device's free memory (cudaMemGetInfo) unchanged."""
    ctx = cc.Context(0)
    try:
        res, psf, mask = _inputs(8, (128, 128))
        nx, ny = res.shape
        dev = torch.device("cuda", 0)
        model_t = torch.zeros((nx, ny), dtype=torch.float32, device=dev)
        res_t = torch.as_tensor(res, device=dev).clone()
        psf_t = torch.as_tensor(psf, device=dev)
        mask_t = torch.as_tensor(mask, device=dev)
        cap = 301
        cx, cy = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
        cp, cf = np.zeros(cap, np.float32), np.zeros(cap, np.float32)
        actual, reported, stop = C.c_int64(), C.c_int64(), C.c_int32()
        ctx.use_own_stream()
        torch.cuda.synchronize()

        def call():
            _lib.call("cr_hogbom_noalloc", ctx.handle, model_t.data_ptr(), res_t.data_ptr(),
                      psf_t.data_ptr(), mask_t.data_ptr(), nx, ny, 0.1, 0.0, 0.0, 0.0, 300, 1,
                      cx.ctypes.data, cy.ctypes.data, cp.ctypes.data, cf.ctypes.data,
                      C.byref(actual), C.byref(reported), C.byref(stop))
            ctx.synchronize()

        assert ctx.workspace_bytes == 0
        free0, _ = torch.cuda.mem_get_info(0)
        call()
        free1, _ = torch.cuda.mem_get_info(0)
        call()
        free2, _ = torch.cuda.mem_get_info(0)
        assert actual.value == 301
        assert ctx.workspace_bytes == 0
        assert free0 == free1 == free2
    finally:
        ctx.close()


def test_noalloc_runs_a_budget_of_exactly_its_limit():
    """cycle_niter 16383 with the inclusive budget: 16384 components, the
    scratch's capacity, bit-identical to cr_hogbom."""
    ctx = cc.Context(0)
    try:
        res, psf, mask = _inputs(9, (48, 40))
        ref = _run(ctx, "cr_hogbom", res, psf, mask, 16383, threshold=0.0)
        got = _run(ctx, "cr_hogbom_noalloc", res, psf, mask, 16383, threshold=0.0)
        assert got["actual"] == ref["actual"] == 16384
        assert got["reported"] == ref["reported"] == 16383
        for key in ("x", "y", "peak", "flux", "model", "residual"):
            np.testing.assert_array_equal(got[key], ref[key])
    finally:
        ctx.close()
