"""Standard (PSWF) gridder on the GPU against the FP64 oracle.

Tolerances: grids and images within 1e-5 of the oracle's peak (FP32 bulk
arithmetic against FP64); sums of weights within 1e-10 relative (FP64 on
both sides); single-sample footprints, tap rows and counts bit-exact.
"""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

from gpu_common import peak_norm_err, random_batch

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def make(ctx, nx=64, cell=1e-4, os_=100):
    geom = O.Geometry(nx, nx, cell, cell)
    og = O.StdGridder(geom, os_)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), os_)
    return geom, og, gg


@pytest.mark.parametrize("os_", [100, 128])
def test_tables_and_shape_match(ctx, os_):
    geom, og, gg = make(ctx, 512, 1e-5, os_)
    assert gg.grid_shape() == (og.gnx, og.gny) == (640, 640)
    assert gg.image_grid_origin() == (og.blc_x, og.blc_y)
    taps, cx, cy = gg.tables()
    np.testing.assert_array_equal(taps, og.taps)
    np.testing.assert_array_equal(cx, og.corr_x)


@pytest.mark.parametrize("os_", [100, 128])
def test_grid_matches_oracle(ctx, os_):
    rng = np.random.default_rng(7 + os_)
    geom, og, gg = make(ctx, 64, 1e-4, os_)
    u, v, w, wt, vis = random_batch(rng, 20000, og.gnx, og.du, margin=2)
    f = rng.uniform(0.5, 2.0, len(u)).astype(np.float32)
    gridable = (rng.uniform(size=len(u)) > 0.1).astype(np.uint8)
    # a few samples off the grid and a non-finite visibility (PSF only)
    u[:5] = 1e9
    vis[10] = np.nan
    psf_o, dirty_o, acc = og.grid_dirty(u, v, wt, vis, f, gridable)
    b = cc.VisibilityBatch(u, v, vis, wt, None, f, gridable)
    psf_g, dirty_g, sums = cc.grid_dirty(gg, b)
    assert sums.gridded_samples == acc.gridded
    assert sums.skipped_samples == acc.skipped
    assert abs(sums.normalization_sumwt - acc.normalization_sumwt) <= 1e-10 * acc.normalization_sumwt
    assert peak_norm_err(psf_g, psf_o) <= TOL
    assert peak_norm_err(dirty_g, dirty_o) <= TOL
    assert sums.unique_records <= sums.gridded_samples


def test_single_sample_footprint_bit_exact(ctx):
    """Cell, oversampling row and tap values of one sample equal the oracle's,
    including coordinates that sit on rounding boundaries."""
    geom, og, gg = make(ctx, 64, 1e-4, 100)
    du = og.du
    cases = [(0.0, 0.0), (0.5 * du, -0.5 * du), (1.5 * du, 2.5 * du), (-0.005 * du, 0.005 * du),
             (3.0049999 * du, -7.0050001 * du), (12.345 * du, -20.995 * du), (-0.125 * du, 0.375 * du)]
    for (u, v) in cases:
        plan = og.plan(u, v)
        b = cc.VisibilityBatch(np.array([u]), np.array([v]), np.array([1 + 0j], np.complex64),
                               np.array([1.0], np.float32))
        psf_g, _, sums = cc.grid_dirty(gg, b)
        nz = np.argwhere(psf_g.real != 0)
        x0, y0, wx, wy = plan
        assert nz[:, 0].min() >= x0 and nz[:, 0].max() <= x0 + 6
        assert nz[:, 1].min() >= y0 and nz[:, 1].max() <= y0 + 6
        expect = np.outer(og.taps[wx], og.taps[wy])  # float32 products
        expect = (og.taps[wx][:, None] * og.taps[wy][None, :]).astype(np.float32)
        got = psf_g.real[x0:x0 + 7, y0:y0 + 7].astype(np.float32)
        np.testing.assert_array_equal(got, expect)


def test_degrid_matches_oracle(ctx):
    rng = np.random.default_rng(11)
    geom, og, gg = make(ctx, 64, 1e-4, 100)
    u, v, w, wt, vis = random_batch(rng, 5000, og.gnx, og.du, margin=2)
    grid = (rng.normal(size=(og.gnx, og.gny)) + 1j * rng.normal(size=(og.gnx, og.gny))).astype(np.complex64)
    pred_o = og.degrid(grid, u, v)
    pred_g = cc.degrid(gg, cc.VisibilityBatch(u, v, vis, wt), grid)
    assert peak_norm_err(pred_g, pred_o) <= TOL


def test_constant_grid_degrids_to_constant(ctx):
    geom, og, gg = make(ctx, 32, 1e-4, 100)
    grid = np.full(gg.grid_shape(), 2.5 - 1.0j, np.complex64)
    p = cc.degrid(gg, cc.VisibilityBatch(np.array([55.0]), np.array([-40.0]),
                                         np.array([0j], np.complex64)), grid)[0]
    assert abs(p.real - 2.5) < 1e-4 and abs(p.imag + 1.0) < 1e-4


def test_residual_grid_matches_oracle(ctx):
    rng = np.random.default_rng(13)
    geom, og, gg = make(ctx, 64, 1e-4, 100)
    u, v, w, wt, vis = random_batch(rng, 8000, og.gnx, og.du, margin=2)
    model = np.zeros((64, 64), np.float32)
    model[30, 33] = 1.0
    model[20, 41] = -0.5
    mg_o = og.model_grid(model)
    mg_g = cc.image_to_grid(gg, model)
    assert peak_norm_err(mg_g, mg_o) <= TOL
    res_o, pred_o, acc = og.residual(mg_o, u, v, wt, vis)
    res_g, sums = cc.grid_residual(gg, cc.VisibilityBatch(u, v, vis, wt), mg_g)
    assert peak_norm_err(res_g, res_o) <= TOL


def test_dirty_image_matches_oracle(ctx):
    rng = np.random.default_rng(17)
    geom, og, gg = make(ctx, 96, 5e-5, 100)
    u, v, w, wt, vis = random_batch(rng, 30000, og.gnx, og.du, margin=2)
    psf_o_g, dirty_o_g, acc = og.grid_dirty(u, v, wt, vis)
    psf_o, res_o, peak_o = og.dirty_products(psf_o_g, dirty_o_g, acc)
    psf_g, res_g, state, sums = cc.dirty_image(gg, cc.VisibilityBatch(u, v, vis, wt))
    assert peak_norm_err(psf_g, psf_o) <= TOL
    assert peak_norm_err(res_g, res_o) <= TOL
    assert abs(state.psf_peak - peak_o) <= 1e-5 * peak_o


def test_no_usable_samples_raises(ctx):
    geom, og, gg = make(ctx, 32, 1e-4, 100)
    b = cc.VisibilityBatch(np.array([1e12]), np.array([0.0]), np.array([1 + 0j], np.complex64))
    with pytest.raises(cc.CasarsCudaError) as e:
        cc.dirty_image(gg, b)
    assert e.value.kind == "NoUsableSamples"
    empty = cc.VisibilityBatch(np.zeros(0), np.zeros(0), np.zeros(0, np.complex64))
    psf, dirty, sums = cc.grid_dirty(gg, empty)
    assert sums.gridded_samples == 0 and not np.any(psf) and not np.any(dirty)


@pytest.mark.parametrize("device", [False, True])
def test_dirty_accumulator_matches_one_batch(device):
    """StandardMfsDirtyAccumulator: three chunks added one after another give
    the images of the whole batch (cr_dirty_image) and of the oracle, within
    1e-5 of the peak, with summed counts and sums of weights."""
    import casars_cuda as cc
    from casars_cuda import synthetic as S
    from oracle import oracle as O
    from gpu_common import peak_norm_err
    ctx = cc.Context(0)
    nx = 128
    obs = S.observation(1000.0, 1.0, 60.0, 1.4e9, nx, 8, 0.1, 1.0, 21, "acc")
    rng = np.random.default_rng(21)
    obs.vis = S.visibilities(obs.u, obs.v, np.zeros_like(obs.w), obs.sky, nx, nx, obs.cell,
                             0.01, rng, w_term=False)
    wt = rng.uniform(0.5, 2.0, obs.rows).astype(np.float32)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, obs.cell, obs.cell), 100)
    if device:
        import torch
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    else:
        t = lambda a: np.ascontiguousarray(a)
    acc = cc.DirtyAccumulator(gg)
    cuts = [0, obs.rows // 3, 2 * obs.rows // 3, obs.rows]
    for a, b in zip(cuts[:-1], cuts[1:]):
        acc.add(cc.VisibilityBatch(t(obs.u[a:b]), t(obs.v[a:b]), t(obs.vis[a:b]), t(wt[a:b])))
    psf, res, state, sums = acc.finish()
    psf1, res1, state1, sums1 = cc.dirty_image(gg, cc.VisibilityBatch(t(obs.u), t(obs.v),
                                                                      t(obs.vis), t(wt)))
    get = (lambda x: x.cpu().numpy()) if device else np.asarray
    assert sums.gridded_samples == sums1.gridded_samples
    assert abs(sums.normalization_sumwt - sums1.normalization_sumwt) <= \
        1e-12 * sums1.normalization_sumwt
    # float32 grids summed in another order (and records merged per chunk)
    assert peak_norm_err(get(psf), get(psf1)) <= 1e-5
    assert peak_norm_err(get(res), get(res1)) <= 1e-5
    og = O.StdGridder(O.Geometry(nx, nx, obs.cell, obs.cell), 100)
    p, d, oacc = og.grid_dirty(obs.u, obs.v, wt, obs.vis, threads=8)
    psf_o, res_o, _ = og.dirty_products(p, d, oacc)
    assert peak_norm_err(get(res), res_o) <= 1e-5
    acc.close()
    ctx.close()


def test_pinned_host_inputs_give_pinned_outputs(ctx):
    """Page-locked torch host inputs: the call copies them like numpy
    arrays and returns its images in page-locked torch tensors."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(29)
    geom, og, gg = make(ctx, 64, 1e-4, 100)
    u, v, w, wt, vis = random_batch(rng, 6000, og.gnx, og.du, margin=2)
    psf, res, state, _ = cc.dirty_image(gg, cc.VisibilityBatch(u, v, vis, wt))
    pin = lambda a: torch.as_tensor(a).pin_memory()
    psf_p, res_p, state_p, _ = cc.dirty_image(
        gg, cc.VisibilityBatch(pin(u), pin(v), pin(vis), pin(wt)))
    assert isinstance(res_p, torch.Tensor) and res_p.is_pinned() and not res_p.is_cuda
    assert peak_norm_err(psf_p.numpy(), psf) <= TOL
    assert peak_norm_err(res_p.numpy(), res) <= TOL
    assert state_p.psf_peak == pytest.approx(state.psf_peak, rel=1e-6)


def _around(x):
    """x and the doubles one and two ulps either side of it."""
    lo1 = np.nextafter(x, -np.inf)
    hi1 = np.nextafter(x, np.inf)
    return [np.nextafter(lo1, -np.inf), lo1, x, hi1, np.nextafter(hi1, np.inf)]


@pytest.mark.parametrize("os_", [100, 128])
def test_plan_decisions_at_rounding_boundaries(ctx, os_):
    """The standard plan takes its anchor and tap-row decisions on float32
    pairs and falls back to the reference's FP64 operations near a rounding
    boundary.  Samples on and a few ulps either side of each anchor boundary
    (x = k + 1/2) and tap-row boundary (x = k + (j + 1/2)/os) must get the
    oracle's FP64 decisions: the same samples accepted, and degridded values
    (which select the taps by exactly those decisions) that match; the grid
    edges (anchors 3 cells from either end) too."""
    geom, og, gg = make(ctx, 256, 2e-5, os_)
    G = og.gnx
    rng = np.random.default_rng(91 + os_)
    us, vs = [], []
    ks = list(rng.integers(G // 4, 3 * G // 4, 4)) + [3, G - 4]
    for k in ks:
        for frac in [0.5] + [(j + 0.5) / os_ for j in range(-os_ // 2, os_ // 2, 7)]:
            for du in _around((k + frac - G / 2) * og.du):
                us.append(du)
                vs.append(rng.uniform(-0.2, 0.2) * G * og.du)
                us.append(rng.uniform(-0.2, 0.2) * G * og.du)
                vs.append(-du)
    u, v = np.array(us), np.array(vs)
    n = len(u)
    wt = np.ones(n, np.float32)
    vis = np.ones(n, np.complex64)
    _, _, acc = og.grid_dirty(u, v, wt, vis)
    _, _, sums = cc.grid_dirty(gg, cc.VisibilityBatch(u, v, vis, wt))
    assert sums.gridded_samples == acc.gridded and sums.skipped_samples == acc.skipped
    grid = (rng.normal(size=(G, G)) + 1j * rng.normal(size=(G, G))).astype(np.complex64)
    pred_o = og.degrid(grid, u, v)
    pred_g = cc.degrid(gg, cc.VisibilityBatch(u, v, vis, wt), grid)
    scale = np.maximum(np.abs(pred_o), 1e-3 * np.max(np.abs(pred_o)))
    assert np.max(np.abs(pred_g - pred_o) / scale) <= 1e-3
