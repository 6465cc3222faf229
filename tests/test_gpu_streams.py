"""Calls on device tensors run on torch's current stream.

Torch's default stream is CUDA's legacy default stream (handle 0); the
binding passes it as cudaStreamLegacy, because a null handle selects the
context's own non-blocking stream, which is not ordered with torch's work.
With the per-call stage timings off the calls return as soon as their work
is queued, so torch work queued right after them must still see their
results: checked here by reading the outputs with torch immediately, against
the same calls with the timings on (which wait for their work).
"""
import ctypes as C

import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import _lib

from gpu_common import random_batch

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.set_timings(True)
    c.close()


def _stream_of(ctx):
    return _lib.load().cr_ctx_stream(ctx.handle) or 0


def test_stream_handles(ctx):
    ctx.use_torch_stream()
    assert _stream_of(ctx) == cc.imaging.CUDA_STREAM_LEGACY
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx.use_torch_stream()
        assert _stream_of(ctx) == s.cuda_stream
    ctx.use_own_stream()
    own = _stream_of(ctx)
    assert own not in (0, cc.imaging.CUDA_STREAM_LEGACY, s.cuda_stream)


@pytest.mark.parametrize("side_stream", [False, True])
def test_async_calls_ordered_with_torch(ctx, side_stream):
    rng = np.random.default_rng(41)
    nx, cell = 512, 2e-5
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    gw = cc.WProjector(gg, 2000.0, planes=16, sampling=8, support_law=(8, 24))
    u, v, w, wt, vis = random_batch(rng, 1 << 20, gg.grid_shape()[0], gg.info.du, margin=32,
                                    w_max=2000.0)
    dev = torch.device("cuda", 0)
    s = torch.cuda.Stream() if side_stream else torch.cuda.current_stream()

    def run():
        with torch.cuda.stream(s):
            # inputs made by torch on the stream, the calls queued behind them,
            # the outputs reduced by torch right after
            b = cc.VisibilityBatch(*(torch.as_tensor(a).to(dev, non_blocking=True)
                                     for a in (u, v, vis, wt, w)))
            grid = torch.complex(torch.ones(gg.grid_shape(), device=dev),
                                 torch.zeros(gg.grid_shape(), device=dev)) * 0.5
            plan = cc.Plan(gg, b, gw)
            psf, dirty = plan.grid_dirty()
            pred = plan.degrid(grid)
            out = (psf.abs().sum(), dirty.real.sum(), pred.real.clone())
            plan.close()
        torch.cuda.synchronize()
        return [o.cpu().numpy() for o in out]

    ctx.set_timings(True)
    ref = run()
    ctx.set_timings(False)
    try:
        got = run()
    finally:
        ctx.set_timings(True)
    # degridding is a deterministic gather; the grid sums agree to float32
    # atomics' order
    assert np.array_equal(got[2], ref[2])
    assert np.allclose(got[0], ref[0], rtol=1e-5) and np.allclose(got[1], ref[1], rtol=1e-4)
