"""The float-pair image transforms (cr_dfft.cu) against cuFFT FP64.

The single-plane calls run their FP64-grade image transforms as float-pair
kernels by default ("auto"); "cufft" runs cuFFT FP64 as before.  Both compute
the same exact DFT to far better than float32, so the float32 images and
model grids they return may differ only where the last rounding to float32
falls on the other side: within four float32 ulps of each value (plus 1e-10
of the peak for values near zero).  Checked for standard and W-projection
geometries (sinc division and the adjoint's sinc product), the PSF's
real-grid input, odd image sizes (the transforms take image rows two at a
time), and the headline 4096^2 image on its 5000^2 grid.  The
oracle-parity tests of the other files run on the float-pair default.
"""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

from gpu_common import peak_norm_err, random_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if np.iscomplexobj(b):
        return _close(a.real, b.real) and _close(a.imag, b.imag)
    peak = float(np.max(np.abs(b)))
    bound = 4 * np.spacing(np.abs(b).astype(np.float32)) + 1e-10 * peak
    bad = np.abs(a - b) > bound
    if bad.any():
        k = np.argmax(np.abs(a - b) - bound)
        print("worst", a.flat[k], b.flat[k], bound.flat[k])
    return not bad.any()


def _engines(ctx, fn):
    ctx.set_image_fft_engine("cufft")
    try:
        ref = fn()
    finally:
        ctx.set_image_fft_engine("auto")
    return fn(), ref


def _random_grid(rng, shape):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)


@pytest.mark.parametrize("nx", [64, 75, 96, 101, 250, 512])   # odd nx: a last row unpaired
def test_grid_to_image_and_back(ctx, nx):
    rng = np.random.default_rng(nx)
    cell = 2e-5
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx + 6, cell, cell), 100)
    gs = gg.grid_shape()
    grid = _random_grid(rng, gs)
    img, ref = _engines(ctx, lambda: cc.grid_to_image(gg, grid, 0.37))
    assert _close(img, ref)
    model = rng.normal(size=(nx, nx + 6)).astype(np.float32)
    mg, mref = _engines(ctx, lambda: cc.image_to_grid(gg, model))
    assert _close(mg, mref)


def test_wproj_image_stage(ctx):
    rng = np.random.default_rng(7)
    nx, cell = 128, 2e-5
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    gw = cc.WProjector(gg, 2000.0, planes=8, sampling=8, support_law=(4, 8))
    grid = _random_grid(rng, gg.grid_shape())
    img, ref = _engines(ctx, lambda: cc.grid_to_image(gg, grid, 1.0, gw))     # sinc division
    assert _close(img, ref)
    model = rng.normal(size=(nx, nx)).astype(np.float32)
    mg, mref = _engines(ctx, lambda: cc.image_to_grid(gg, model, gw))         # sinc product
    assert _close(mg, mref)
    u, v, w, wt, vis = random_batch(rng, 5000, gg.grid_shape()[0], gg.info.du, margin=16,
                                    w_max=2000.0)
    batch = cc.VisibilityBatch(u, v, vis, wt, w)
    # the adjoint grids the batch on each call (float32 sums in a run-dependent
    # order), so its two images agree to the gridder's tolerance, not to ulps
    adj, aref = _engines(ctx, lambda: cc.adjoint(gg, batch, gw))               # adjoint's sinc
    assert peak_norm_err(adj, aref) <= 1e-6


def test_dirty_image_on_float_pairs_matches_oracle(ctx):
    rng = np.random.default_rng(17)
    nx, cell = 96, 5e-5
    og = O.StdGridder(O.Geometry(nx, nx, cell, cell), 100)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    u, v, w, wt, vis = random_batch(rng, 30000, og.gnx, og.du, margin=2)
    p, d, acc = og.grid_dirty(u, v, wt, vis)
    psf_o, res_o, peak_o = og.dirty_products(p, d, acc)
    (psf, res, st, _), (psf_c, res_c, st_c, _) = _engines(
        ctx, lambda: cc.dirty_image(gg, cc.VisibilityBatch(u, v, vis, wt)))
    for p_, r_ in ((psf, res), (psf_c, res_c)):
        assert peak_norm_err(p_, psf_o) <= 1e-5 and peak_norm_err(r_, res_o) <= 1e-5
    # each call grids the batch again (float32 sums in a run-dependent order:
    # two runs of one engine differ by about 2e-6 of the peak on this
    # noise-like residual)
    assert peak_norm_err(psf, psf_c) <= 5e-6 and peak_norm_err(res, res_c) <= 5e-6
    assert st.psf_peak == pytest.approx(st_c.psf_peak, rel=1e-6)


def test_headline_grid_size(ctx):
    """The 4096^2 image of the W-projection benchmark on its 5000^2 grid."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    nx, cell = 4096, 1.5e-6
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    assert gg.grid_shape() == (5000, 5000)
    dev = torch.device("cuda", 0)
    grid = torch.complex(torch.randn((5000, 5000), device=dev),
                         torch.randn((5000, 5000), device=dev))
    img, ref = _engines(ctx, lambda: cc.grid_to_image(gg, grid, 1.0))
    assert _close(img.cpu().numpy(), ref.cpu().numpy())
    model = torch.randn((nx, nx), device=dev)
    mg, mref = _engines(ctx, lambda: cc.image_to_grid(gg, model))
    assert _close(mg.cpu().numpy(), mref.cpu().numpy())
