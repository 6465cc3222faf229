"""Image-stage FFT precision of the single-plane calls (the dirty-product
policy's F32 / F64 choice) on the GPU against the FP64 oracle.

The image correction divides by grdsf (and by sinc for W-projection), which
amplifies the float32 transform's rounding near the image edge: on the
noise-like dirty images here the FP32 stage lands at 0.9-1.2e-5 of the
oracle's peak, so its images are held to 3e-5 (the FP64 default meets
1e-5 in the other tests).  Model grids and the forward/adjoint pair carry
no such amplification and stay within 1e-5.  "auto" runs FP64.
"""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

from gpu_common import arcsec, peak_norm_err, random_batch

pytestmark = pytest.mark.gpu
TOL = 1e-5
TOL_F32_IMAGE = 3e-5


@pytest.fixture()
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def test_precision_setting_validates(ctx):
    assert ctx.image_fft_precision == "f64"
    ctx.set_image_fft_precision("f32")
    assert ctx.image_fft_precision == "f32"
    ctx.set_image_fft_precision("auto")
    assert ctx.image_fft_precision == "f64"
    with pytest.raises(ValueError):
        ctx.set_image_fft_precision(16)


def test_standard_f32_images_match_oracle(ctx):
    ctx.set_image_fft_precision("f32")
    rng = np.random.default_rng(41)
    nx, cell = 96, 5e-5
    geom = O.Geometry(nx, nx, cell, cell)
    og = O.StdGridder(geom, 100)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    u, v, w, wt, vis = random_batch(rng, 30000, og.gnx, og.du, margin=2)
    psf_og, dirty_og, acc = og.grid_dirty(u, v, wt, vis)
    psf_o, res_o, peak_o = og.dirty_products(psf_og, dirty_og, acc)
    psf_g, res_g, state, _ = cc.dirty_image(gg, cc.VisibilityBatch(u, v, vis, wt))
    assert peak_norm_err(psf_g, psf_o) <= TOL_F32_IMAGE
    assert peak_norm_err(res_g, res_o) <= TOL_F32_IMAGE
    assert abs(state.psf_peak - peak_o) <= 1e-5 * peak_o
    model = np.zeros((nx, nx), np.float32)
    model[40, 50] = 1.0
    model[60, 33] = -0.4
    assert peak_norm_err(cc.image_to_grid(gg, model), og.model_grid(model)) <= TOL


def test_wproj_f32_images_match_oracle(ctx):
    ctx.set_image_fft_precision("f32")
    nx, cell, max_w = 256, arcsec(15.0), 3000.0
    geom = O.Geometry(nx, nx, cell, cell)
    og = O.StdGridder(geom, 100)
    ow = O.WProjector(geom, og, max_w, planes=16, sampling=8, support_min=4, support_max=12)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    gw = cc.WProjector(gg, max_w, planes=16, sampling=8, support_law=(4, 12))
    rng = np.random.default_rng(43)
    margin = int(ow.support.max()) + 2
    u, v, w, wt, vis = random_batch(rng, 8000, og.gnx, og.du, margin=margin, w_max=max_w)
    psf_og, dirty_og, acc = ow.grid_dirty(u, v, w, wt, vis)
    psf_o, res_o, _ = ow.dirty_products(psf_og, dirty_og, acc)
    psf_g, res_g, _, _ = cc.dirty_image(gg, cc.VisibilityBatch(u, v, vis, wt, w), gw)
    assert peak_norm_err(psf_g, psf_o) <= TOL_F32_IMAGE
    assert peak_norm_err(res_g, res_o) <= TOL_F32_IMAGE


@pytest.mark.parametrize("wproj", [False, True])
def test_f32_forward_adjoint_pair(ctx, wproj):
    """The FP32 stage keeps predict and adjoint an adjoint pair and within
    1e-5 of the FP64 stage's outputs."""
    rng = np.random.default_rng(47)
    nx = 128
    cell = 1e-4 if not wproj else 1.2e-4
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell))
    gw = cc.WProjector(gg, 500.0, planes=8, sampling=4, support_law=(4, 10)) if wproj else None
    du = 1.0 / (gg.grid_shape()[0] * cell)
    u, v, w, wt, vis = random_batch(rng, 20000, gg.grid_shape()[0], du, margin=14, w_max=500.0,
                                    weights=False)
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    x = rng.normal(size=(nx, nx)).astype(np.float32)
    ax64, aty64 = cc.predict(gg, b, x, gw), cc.adjoint(gg, b, gw)
    ctx.set_image_fft_precision("f32")
    ax, aty = cc.predict(gg, b, x, gw), cc.adjoint(gg, b, gw)
    assert peak_norm_err(ax, ax64) <= TOL
    assert peak_norm_err(aty, aty64) <= TOL
    lhs = np.sum(np.conj(ax.astype(np.complex128)) * vis.astype(np.complex128)).real
    rhs = np.sum(x.astype(np.float64) * aty.astype(np.float64))
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))


def test_run_imaging_precision_is_scoped(ctx):
    rng = np.random.default_rng(53)
    nx, cell = 64, 1e-4
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    du = 1.0 / (gg.grid_shape()[0] * cell)
    u, v, w, wt, vis = random_batch(rng, 5000, gg.grid_shape()[0], du, margin=2)
    b = cc.VisibilityBatch(u, v, vis, wt)
    ref = cc.run_imaging(ctx, cc.ImagingRequest(cc.ImageGeometry(nx, nx, cell, cell), [b]))
    got = cc.run_imaging(ctx, cc.ImagingRequest(cc.ImageGeometry(nx, nx, cell, cell), [b],
                                                fft_precision="f32"))
    assert ctx.image_fft_precision == "f64"
    assert peak_norm_err(np.asarray(got.residual), np.asarray(ref.residual)) <= TOL_F32_IMAGE
