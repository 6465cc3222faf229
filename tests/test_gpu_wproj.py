"""W-projection on the GPU against the FP64 oracle.

The oracle builds its kernels from FP64 screens with a direct FP64 DFT; the
GPU uses FP64 phases, FP32 screens and cuFFT.  Kernels agree to 1e-5 of the
kernel peak; grids, model visibilities and images to 1e-5 of the oracle's
peak; supports, w_scale, plane choice and counts exactly.
"""
import math

import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

from gpu_common import arcsec, peak_norm_err, random_batch

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


# (image, cell arcsec, planes, sampling, support law, max |w|)
CASES = [
    (128, 30.0, 8, None, None, 1500.0),     # reference rules: sampling 4, threshold support
    (256, 15.0, 16, 8, (4, 12), 3000.0),    # benchmark-style law at oversampling 8
]


def build(ctx, nx, cell_as, planes, sampling, law, max_w):
    cell = arcsec(cell_as)
    geom = O.Geometry(nx, nx, cell, cell)
    og = O.StdGridder(geom, 100)
    ow = O.WProjector(geom, og, max_w, planes=planes, sampling=sampling,
                      support_min=law[0] if law else 0, support_max=law[1] if law else 0)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
    gw = cc.WProjector(gg, max_w, planes=planes, sampling=sampling, support_law=law)
    return og, ow, gg, gw


@pytest.mark.parametrize("case", CASES)
def test_kernels_match_oracle(ctx, case):
    nx, cell_as, planes, sampling, law, wmax = case
    og, ow, gg, gw = build(ctx, nx, cell_as, planes, sampling, law, wmax)
    assert gw.planes == ow.planes and gw.sampling == ow.sampling
    assert gw.w_scale == pytest.approx(ow.w_scale, rel=1e-15)
    support, kern, norm = gw.tables()
    np.testing.assert_array_equal(support, ow.support)
    W = min(kern.shape[1], ow.width)
    assert kern.shape[1] == ow.width
    err = np.max(np.abs(kern - ow.kernels)) / np.max(np.abs(ow.kernels))
    assert err <= TOL
    assert np.max(np.abs(norm - ow.norm)) <= 1e-5 * np.max(np.abs(ow.norm))


@pytest.mark.parametrize("case", CASES)
def test_grid_and_degrid_match_oracle(ctx, case):
    nx, cell_as, planes, sampling, law, wmax = case
    og, ow, gg, gw = build(ctx, nx, cell_as, planes, sampling, law, wmax)
    rng = np.random.default_rng(21)
    margin = int(ow.support.max()) + 2
    u, v, w, wt, vis = random_batch(rng, 6000, og.gnx, og.du, margin=margin, w_max=wmax)
    # repeat some samples exactly so deduplication merges them
    u[1000:1500], v[1000:1500], w[1000:1500] = u[:500], v[:500], w[:500]
    psf_o, dirty_o, acc = ow.grid_dirty(u, v, w, wt, vis)
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    psf_g, dirty_g, sums = cc.grid_dirty(gg, b, gw)
    assert sums.gridded_samples == acc.gridded and sums.skipped_samples == acc.skipped
    assert sums.unique_records < sums.gridded_samples
    assert abs(sums.normalization_sumwt - acc.normalization_sumwt) <= 1e-5 * acc.normalization_sumwt
    assert peak_norm_err(psf_g, psf_o) <= TOL
    assert peak_norm_err(dirty_g, dirty_o) <= TOL
    grid = (rng.normal(size=(og.gnx, og.gny)) + 1j * rng.normal(size=(og.gnx, og.gny))).astype(np.complex64)
    pred_o = ow.degrid(grid, u, v, w)
    pred_g = cc.degrid(gg, b, grid, gw)
    assert peak_norm_err(pred_g, pred_o) <= TOL


def _around(x):
    """x and the doubles one and two ulps either side of it."""
    lo1 = np.nextafter(x, -np.inf)
    hi1 = np.nextafter(x, np.inf)
    return [np.nextafter(lo1, -np.inf), lo1, x, hi1, np.nextafter(hi1, np.inf)]


@pytest.mark.parametrize("case", CASES)
def test_plan_decisions_at_rounding_boundaries(ctx, case):
    """The plan's anchor, oversampling offset and plane decisions for samples
    on and a few ulps either side of each kind of rounding boundary equal
    the oracle's FP64 ones: the degridded value of every sample (which
    selects its kernel by exactly those decisions) matches, and the same
    samples are accepted."""
    nx, cell_as, planes, sampling, law, wmax = case
    og, ow, gg, gw = build(ctx, nx, cell_as, planes, sampling, law, wmax)
    s = ow.sampling
    G = og.gnx
    rng = np.random.default_rng(77)
    us, vs, ws = [], [], []
    base_w = rng.uniform(-0.5 * wmax, 0.5 * wmax)
    for k in rng.integers(G // 4, 3 * G // 4, 6):
        # anchor boundaries x = k + 1/2 and offset boundaries x = k + (j + 1/2)/s
        for frac in [0.5] + [(j + 0.5) / s for j in range(-s // 2, s // 2)]:
            for du in _around((k + frac - G / 2) * og.du):
                us.append(du)
                vs.append(rng.uniform(-0.2, 0.2) * G * og.du)
                ws.append(base_w)
                us.append(rng.uniform(-0.2, 0.2) * G * og.du)
                vs.append(-du)
                ws.append(-base_w)
    # plane boundaries |w| w_scale = (k + 1/2)^2
    for k in range(planes):
        for wv in _around((k + 0.5) ** 2 / ow.w_scale):
            for sign in (1.0, -1.0):
                us.append(rng.uniform(-0.2, 0.2) * G * og.du)
                vs.append(rng.uniform(-0.2, 0.2) * G * og.du)
                ws.append(sign * wv)
    u, v, w = np.array(us), np.array(vs), np.array(ws)
    n = len(u)
    wt = np.ones(n, np.float32)
    vis = np.ones(n, np.complex64)
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    _, _, acc = ow.grid_dirty(u, v, w, wt, vis)
    _, _, sums = cc.grid_dirty(gg, b, gw)
    assert sums.gridded_samples == acc.gridded and sums.skipped_samples == acc.skipped
    grid = (rng.normal(size=(og.gnx, og.gny)) + 1j * rng.normal(size=(og.gnx, og.gny))) \
        .astype(np.complex64)
    pred_o = ow.degrid(grid, u, v, w)
    pred_g = cc.degrid(gg, b, grid, gw)
    scale = np.maximum(np.abs(pred_o), 1e-3 * np.max(np.abs(pred_o)))
    assert np.max(np.abs(pred_g - pred_o) / scale) <= 1e-3


def test_plane_choice_and_conjugation(ctx):
    og, ow, gg, gw = build(ctx, *CASES[0][:5], CASES[0][5])
    # a single sample with w > 0 uses the conjugated kernel (lib.rs:95167);
    # |w| past the largest planned |w| clamps to the last plane
    for wv in (-1200.0, 1200.0, 0.0, 1e-9, 4500.0, -9000.0):
        u = np.array([3.3 * og.du]); v = np.array([-5.7 * og.du]); w = np.array([wv])
        psf_o, dirty_o, acc = ow.grid_dirty(u, v, w, np.ones(1, np.float32), np.ones(1, np.complex64))
        psf_g, dirty_g, sums = cc.grid_dirty(gg, cc.VisibilityBatch(u, v, np.ones(1, np.complex64),
                                                                    np.ones(1, np.float32), w), gw)
        assert peak_norm_err(dirty_g, dirty_o) <= TOL


def test_dirty_image_matches_oracle(ctx):
    og, ow, gg, gw = build(ctx, *CASES[1][:5], CASES[1][5])
    rng = np.random.default_rng(5)
    margin = int(ow.support.max()) + 2
    u, v, w, wt, vis = random_batch(rng, 8000, og.gnx, og.du, margin=margin, w_max=CASES[1][5])
    psf_og, dirty_og, acc = ow.grid_dirty(u, v, w, wt, vis)
    psf_o, res_o, peak_o = ow.dirty_products(psf_og, dirty_og, acc)
    psf_g, res_g, state, sums = cc.dirty_image(gg, cc.VisibilityBatch(u, v, vis, wt, w), gw)
    assert peak_norm_err(psf_g, psf_o) <= TOL
    assert peak_norm_err(res_g, res_o) <= TOL


def test_residual_refresh_matches_oracle(ctx):
    og, ow, gg, gw = build(ctx, *CASES[1][:5], CASES[1][5])
    rng = np.random.default_rng(9)
    margin = int(ow.support.max()) + 2
    u, v, w, wt, vis = random_batch(rng, 6000, og.gnx, og.du, margin=margin, w_max=CASES[1][5])
    model = np.zeros((256, 256), np.float32)
    model[70, 90] = 1.0
    model[100, 60] = 0.25
    mg_o = ow.model_grid(model)
    mg_g = cc.image_to_grid(gg, model, gw)
    assert peak_norm_err(mg_g, mg_o) <= TOL
    res_o, acc = ow.residual(mg_o, u, v, w, wt, vis)
    res_g, sums = cc.grid_residual(gg, cc.VisibilityBatch(u, v, vis, wt, w), mg_g, gw)
    assert peak_norm_err(res_g, res_o) <= TOL


def test_footprints_at_the_grid_edge(ctx):
    """Samples whose W-kernel footprint would leave the grid are rejected
    (counted as skipped) exactly as the oracle rejects them; those just
    inside are gridded."""
    og, ow, gg, gw = build(ctx, *CASES[0][:5], CASES[0][5])
    s_max = int(ow.support.max())
    half = og.gnx // 2
    xs = np.arange(half - s_max - 4, half + 1, dtype=np.float64)   # cells from the centre
    u = np.concatenate([xs, -xs]) * og.du + 0.3 * og.du
    v = np.full(len(u), 2.2 * og.du)
    w = np.linspace(-1500.0, 1500.0, len(u))
    wt = np.ones(len(u), np.float32)
    vis = np.ones(len(u), np.complex64)
    psf_o, dirty_o, acc = ow.grid_dirty(u, v, w, wt, vis)
    psf_g, dirty_g, sums = cc.grid_dirty(gg, cc.VisibilityBatch(u, v, vis, wt, w), gw)
    assert acc.skipped > 0 and acc.gridded > 0
    assert sums.gridded_samples == acc.gridded and sums.skipped_samples == acc.skipped
    assert peak_norm_err(dirty_g, dirty_o) <= TOL
