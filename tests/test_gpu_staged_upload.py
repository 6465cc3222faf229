"""Host batches of 2^20 samples or more are uploaded in pieces on a second
stream while the plan kernel works through the pieces already copied
(StagedBatch, csrc/cr_core.cu; the peak readback and the PSF image's
download in cr_dirty_image overlap the residual transform too).  The calls
must return what they return for the same batch held on the device: the same
sums and bit-identical predictions (degridding is a deterministic gather),
images within 5e-6 of the peak (the run-to-run spread of float32 atomics in a
run-dependent order: about 1e-6 for the W-projection PSF of 2^20 samples),
and images within 1e-5 of the FP64 oracle.
"""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

from gpu_common import peak_norm_err, random_batch

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# above the staging threshold and not a multiple of the four pieces
N = (1 << 20) + 12345


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def _batches(rng, gnx, du, cell, w_max=0.0):
    u, v, w, wt, _ = random_batch(rng, N, gnx, du, margin=16, w_max=w_max)
    wt[rng.random(N) < 0.01] = 0.0                 # some samples not gridded
    # two point sources and a little noise: images with a real peak, so that
    # the float32 sums' order-dependent spread stays far below the bounds
    vis = np.zeros(N, np.complex128)
    for amp, l, m in ((1.0, 11 * cell, -7 * cell), (0.4, -23 * cell, 30 * cell)):
        vis += amp * np.exp(-2j * np.pi * (u * l + v * m))
    vis = (vis + 0.01 * (rng.normal(size=N) + 1j * rng.normal(size=N))).astype(np.complex64)
    pinned = [torch.as_tensor(a).pin_memory() for a in (u, v, vis, wt, w)]
    host = cc.VisibilityBatch(*pinned)
    dev = cc.VisibilityBatch(*(t.cuda() for t in pinned))
    return (u, v, w, wt, vis), host, dev


def _same_sums(a, b):
    assert a.gridded_samples == b.gridded_samples
    assert a.normalization_sumwt == pytest.approx(b.normalization_sumwt, rel=1e-12)


def test_standard_dirty_image_and_predict(ctx):
    rng = np.random.default_rng(23)
    nx, cell = 128, 5e-5
    og = O.StdGridder(O.Geometry(nx, nx, cell, cell), 100)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    (u, v, w, wt, vis), host, dev = _batches(rng, og.gnx, og.du, cell)
    psf_h, res_h, st_h, s_h = cc.dirty_image(gg, host)
    psf_d, res_d, st_d, s_d = cc.dirty_image(gg, dev)
    _same_sums(s_h, s_d)
    assert st_h.psf_peak == pytest.approx(st_d.psf_peak, rel=1e-6)
    psf_d, res_d = psf_d.cpu().numpy(), res_d.cpu().numpy()
    assert peak_norm_err(psf_h, psf_d) <= 1e-6 and peak_norm_err(res_h, res_d) <= 5e-6
    p, d, acc = og.grid_dirty(u, v, wt, vis)
    psf_o, res_o, _ = og.dirty_products(p, d, acc)
    assert s_h.gridded_samples == acc.gridded
    assert peak_norm_err(psf_h, psf_o) <= 1e-5 and peak_norm_err(res_h, res_o) <= 1e-5

    model = np.zeros((nx, nx), np.float32)
    model[40, 70], model[90, 33] = 1.0, -0.25
    pred_h = cc.predict(gg, host, torch.as_tensor(model).pin_memory())
    pred_d = cc.predict(gg, dev, torch.as_tensor(model).cuda()).cpu().numpy()
    assert np.array_equal(np.asarray(pred_h), pred_d)


def test_wproj_dirty_image_residual_and_adjoint(ctx):
    rng = np.random.default_rng(29)
    nx, cell = 128, 2e-5
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    gw = cc.WProjector(gg, 2000.0, planes=8, sampling=8, support_law=(4, 8))
    (u, v, w, wt, vis), host, dev = _batches(rng, gg.grid_shape()[0], gg.info.du, cell,
                                             w_max=2000.0)
    psf_h, res_h, st_h, s_h = cc.dirty_image(gg, host, gw)
    psf_d, res_d, st_d, s_d = cc.dirty_image(gg, dev, gw)
    _same_sums(s_h, s_d)
    assert peak_norm_err(psf_h, psf_d.cpu().numpy()) <= 5e-6
    assert peak_norm_err(res_h, res_d.cpu().numpy()) <= 5e-6
    model = np.zeros((nx, nx), np.float32)
    model[64, 64], model[20, 100] = 0.5, 0.125
    r_h, rs_h = cc.residual_image(gg, host, torch.as_tensor(model).pin_memory(), st_h, gw)
    r_d, rs_d = cc.residual_image(gg, dev, torch.as_tensor(model).cuda(), st_d, gw)
    _same_sums(rs_h, rs_d)
    assert peak_norm_err(r_h, r_d.cpu().numpy()) <= 5e-6
    a_h = cc.adjoint(gg, host, gw)
    a_d = cc.adjoint(gg, dev, gw).cpu().numpy()
    assert peak_norm_err(a_h, a_d) <= 5e-6


def test_plan_and_accumulator(ctx):
    rng = np.random.default_rng(31)
    nx, cell = 96, 5e-5
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    (u, v, w, wt, vis), host, dev = _batches(rng, gg.grid_shape()[0], gg.info.du, cell)
    ph, pd = cc.Plan(gg, host), cc.Plan(gg, dev)
    _same_sums(ph.sums, pd.sums)
    grid = torch.complex(torch.randn(gg.grid_shape()), torch.randn(gg.grid_shape()))
    assert np.array_equal(np.asarray(ph.degrid(grid.pin_memory())),
                          pd.degrid(grid.cuda()).cpu().numpy())
    ph.close()
    pd.close()
    ah, ad = cc.DirtyAccumulator(gg), cc.DirtyAccumulator(gg)
    _same_sums(ah.add(host), ad.add(dev))
    (psf_h, res_h, _), (psf_d, res_d, _) = ah.finish()[:3], ad.finish()[:3]
    assert peak_norm_err(np.asarray(psf_h), _np(psf_d)) <= 5e-6
    assert peak_norm_err(np.asarray(res_h), _np(res_d)) <= 5e-6
    ah.close()
    ad.close()


def _np(x):
    return x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x)
