"""W-projection at the benchmark's shape against the FP64 oracle.

The benchmark grids a 4096^2 image (5000^2 grid) with 128 w-planes whose
support grows linearly from 8 to 64 pixels, at oversampling 8.  These cases
run that shape and its neighbours through every code path the benchmark
takes, and compare each stage with the oracle:

* the kernel construction at conv_size 5000 (all 128 planes), the support
  table and the (plane, offset) normalisation table;
* gridding (PSF and dirty grids), where supports up to 64 make the output
  tiles gather candidates from home tiles up to two tiles away, and up to 76
  (1250^2 grid) three tiles away;
* degridding, whose windows of 17..129 columns use every register-chunk
  width of the row-pair path (2..9 chunks of 16 lanes), and windows of 153
  columns the flat fallback;
* the dirty image and the residual refresh of a model image.

Tolerances: kernels within 1e-5 of the kernel peak; grids, model
visibilities and images within 1e-5 of the oracle's peak; supports, counts
and plane choice exact; sums of weights within 1e-5 relative.
"""
import math
import os

import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import oracle as O

from gpu_common import arcsec, peak_norm_err

pytestmark = pytest.mark.gpu
TOL = 1e-5
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def chunks_of_support(s):
    """Register-chunk count of the degridder's row-pair path for support s
    (16-lane chunks covering a 2s+1 window); above 9 the flat path runs."""
    return (2 * s + 1 + 15) // 16


def samples_on_every_plane(rng, ow, og, per_plane, margin):
    """Samples whose |w| selects each plane in turn, both signs of w,
    positions uniform over the usable grid."""
    P = ow.planes
    p = np.repeat(np.arange(P), per_plane).astype(np.float64)
    frac = rng.uniform(-0.35, 0.35, len(p))
    wabs = np.clip(p + frac, 0.0, None) ** 2 / ow.w_scale
    w = wabs * rng.choice([-1.0, 1.0], len(p))
    half = (og.gnx / 2 - margin) * og.du
    u = rng.uniform(-half, half, len(p))
    v = rng.uniform(-half, half, len(p))
    return u, v, w


def planes_hit(ow, u, v, w):
    out = []
    for a, b, c in zip(u, v, w):
        pl = ow.plan(float(a), float(b), float(c))
        if pl is not None:
            out.append(pl["plane"])
    return np.array(out, np.int64)


def build_pair(ctx, nx, cell, planes, law, max_w):
    geom = O.Geometry(nx, nx, cell, cell)
    og = O.StdGridder(geom, 100)
    ow = O.WProjector(geom, og, max_w, planes=planes, sampling=8, support_min=law[0],
                      support_max=law[1], threads=THREADS)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    gw = cc.WProjector(gg, max_w, planes=planes, sampling=8, support_law=law)
    return og, ow, gg, gw


def check_kernels(gw, ow):
    assert gw.planes == ow.planes and gw.sampling == ow.sampling == 8
    assert gw.w_scale == pytest.approx(ow.w_scale, rel=1e-15)
    support, kern, norm = gw.tables()
    np.testing.assert_array_equal(support, ow.support)
    assert kern.shape[1] == ow.width
    scale = float(np.max(np.abs(ow.kernels)))
    # plane by plane, so no full-size complex128 difference is held at once
    worst = max(float(np.max(np.abs(kern[p] - ow.kernels[p]))) for p in range(ow.planes))
    assert worst <= TOL * scale, worst / scale
    assert np.max(np.abs(norm - ow.norm)) <= 1e-5 * np.max(np.abs(ow.norm))
    return support


def check_grid_degrid(gg, gw, og, ow, u, v, w, wt, vis, rng):
    psf_o, dirty_o, acc = ow.grid_dirty(u, v, w, wt, vis, threads=THREADS)
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    psf_g, dirty_g, sums = cc.grid_dirty(gg, b, gw)
    assert sums.gridded_samples == acc.gridded and sums.skipped_samples == acc.skipped
    assert abs(sums.normalization_sumwt - acc.normalization_sumwt) <= 1e-5 * acc.normalization_sumwt
    assert peak_norm_err(psf_g, psf_o) <= TOL
    assert peak_norm_err(dirty_g, dirty_o) <= TOL
    del psf_o, dirty_o, psf_g, dirty_g
    grid = (rng.standard_normal((og.gnx, og.gny), np.float32)
            + 1j * rng.standard_normal((og.gnx, og.gny), np.float32)).astype(np.complex64)
    pred_o = ow.degrid(grid, u, v, w, threads=THREADS)
    pred_g = cc.degrid(gg, b, grid, gw)
    assert peak_norm_err(pred_g, pred_o) <= TOL
    return acc


def check_images(gg, gw, og, ow, u, v, w, wt, vis, nx):
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    psf_og, dirty_og, acc = ow.grid_dirty(u, v, w, wt, vis, threads=THREADS)
    psf_o, res_o, _ = ow.dirty_products(psf_og, dirty_og, acc)
    del psf_og, dirty_og
    psf_g, res_g, _, _ = cc.dirty_image(gg, b, gw)
    assert peak_norm_err(psf_g, psf_o) <= TOL
    assert peak_norm_err(res_g, res_o) <= TOL
    # residual refresh of a model with a few components
    model = np.zeros((nx, nx), np.float32)
    model[nx // 2, nx // 2] = 1.0
    model[nx // 3, 2 * nx // 3] = 0.3
    model[nx // 5 + 7, nx // 4] = -0.05
    mg_o = ow.model_grid(model)
    mg_g = cc.image_to_grid(gg, model, gw)
    assert peak_norm_err(mg_g, mg_o) <= TOL
    res_grid_o, _ = ow.residual(mg_o, u, v, w, wt, vis, threads=THREADS)
    res_grid_g, _ = cc.grid_residual(gg, b, mg_g, gw)
    assert peak_norm_err(res_grid_g, res_grid_o) <= TOL


def test_full_size_grid_128_planes(ctx):
    """The benchmark's own geometry: 4096^2 image, 5000^2 grid, cell from the
    21 km layout at 1.4 GHz, 128 planes, support 8..64, oversampling 8.
    Inputs: every 3000th row of the benchmark observation plus samples placed
    on each of the 128 planes."""
    obs = S.wproj_4096_observation(2)
    og, ow, gg, gw = build_pair(ctx, obs.nx, obs.cell, 128, (8, 64), float(np.abs(obs.w).max()))
    assert (og.gnx, og.gny) == (5000, 5000)
    support = check_kernels(gw, ow)
    assert int(support.min()) == 8 and int(support.max()) == 64
    rng = np.random.default_rng(40)
    sl = slice(0, None, 3000)
    u1, v1, w1 = obs.u[sl], obs.v[sl], obs.w[sl]
    u2, v2, w2 = samples_on_every_plane(rng, ow, og, 6, margin=70)
    u = np.concatenate([u1, u2]); v = np.concatenate([v1, v2]); w = np.concatenate([w1, w2])
    n = len(u)
    wt = rng.uniform(0.5, 2.0, n).astype(np.float32)
    vis = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    hit = planes_hit(ow, u, v, w)
    assert set(hit.tolist()) == set(range(128))
    assert {chunks_of_support(int(s)) for s in ow.support[hit]} == set(range(2, 10))
    check_grid_degrid(gg, gw, og, ow, u, v, w, wt, vis, rng)
    check_images(gg, gw, og, ow, u, v, w, wt, vis, obs.nx)


def test_2048_image_32_planes(ctx):
    """2048^2 image (2500^2 grid), 32 planes with supports 8..64: a few
    thousand samples on every plane, some repeated exactly (deduplicated
    records), some at the edge of the usable grid."""
    nx, cell = 2048, arcsec(1.0)
    og, ow, gg, gw = build_pair(ctx, nx, cell, 32, (8, 64), 0.25 / cell)
    check_kernels(gw, ow)
    rng = np.random.default_rng(41)
    u, v, w = samples_on_every_plane(rng, ow, og, 100, margin=66)
    # the windows of the last plane (support 64) at the grid edge from both
    # sides: 65.6 cells in fit, 62.6 cells in are rejected
    inside, outside = (og.gnx / 2 - 65.6) * og.du, (og.gnx / 2 - 62.6) * og.du
    u[-40:-30], u[-30:-20] = inside, -inside
    u[-20:-10], u[-10:] = outside, -outside
    # repeated samples: deduplicated into records with summed values
    u, v, w = (np.concatenate([a, a[300:600]]) for a in (u, v, w))
    n = len(u)
    wt = rng.uniform(0.5, 2.0, n).astype(np.float32)
    vis = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    hit = planes_hit(ow, u, v, w)
    assert set(hit.tolist()) == set(range(32))
    assert {chunks_of_support(int(s)) for s in ow.support[hit]} == set(range(2, 10))
    acc = check_grid_degrid(gg, gw, og, ow, u, v, w, wt, vis, rng)
    assert acc.skipped > 0 and acc.gridded > 0
    check_images(gg, gw, og, ow, u, v, w, wt, vis, nx)


def test_support_76_neighbourhood_three_tiles(ctx):
    """1024^2 image (1250^2 grid), 16 planes with supports 8..76: windows up
    to 153 wide reach output tiles three tiles from their home tile, and the
    degridder's flat path takes the widest."""
    nx, cell = 1024, arcsec(2.0)
    og, ow, gg, gw = build_pair(ctx, nx, cell, 16, (8, 76), 0.25 / cell)
    support = check_kernels(gw, ow)
    assert int(support.max()) == 76 and (31 + 76) // 32 == 3
    rng = np.random.default_rng(42)
    u, v, w = samples_on_every_plane(rng, ow, og, 120, margin=78)
    n = len(u)
    wt = rng.uniform(0.5, 2.0, n).astype(np.float32)
    vis = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    hit = planes_hit(ow, u, v, w)
    chunks = {chunks_of_support(int(s)) for s in ow.support[hit]}
    assert 10 in chunks and 2 in chunks
    check_grid_degrid(gg, gw, og, ow, u, v, w, wt, vis, rng)
    check_images(gg, gw, og, ow, u, v, w, wt, vis, nx)
