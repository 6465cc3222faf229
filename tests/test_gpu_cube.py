"""The batched spectral cube against the oracle, channel by channel.

A small cube (8 channels over 1-2 GHz, 128 x 128 image, seeded per-channel
flag fractions up to 60 %) is planned, weighted and gridded in one batched
call.  Per channel the oracle builds the batch the reference's imager would
(u_lambda = u_m * f/c, flagged samples left out), weights it with the
PerPlane density and grids / degrids it in FP64.

* the per-sample plan (start cells, tap rows) is bit-exact, and so is the
  imaging weight (unit input weights make every density sum exact);
* PSF and dirty grids agree within 1e-5 of each channel's peak, sums of
  weights to 1e-12 relative, gridded counts exactly;
* the batched grids agree with the plain single-channel GPU path run
  channel by channel (cr_apply_weighting_plane + cr_grid_dirty);
* degridding agrees within 1e-5 of each channel's largest prediction;
* samples placed on and next to every rounding boundary take the same
  decisions as the oracle (the integer fast path hands them to FP64).
"""
import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import oracle as O

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu

OS = 128


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def cube():
    obs = S.cube_observation(channels=8, nx=128, hours=1.0, dump_s=60.0, n_sources=6, seed=9)
    flags = S.cube_flags(obs)
    vis = S.cube_visibilities(obs)
    return obs, flags, vis


def _oracle_channel(obs, flags, vis, c, mode, robust):
    geom = O.Geometry(obs.nx, obs.nx, obs.cell, obs.cell)
    og = O.StdGridder(geom, OS)
    keep = ~flags[c]
    ls = obs.lambda_scale[c]
    u, v = obs.u_m[keep] * ls, obs.v_m[keep] * ls
    w0 = np.ones(len(u), np.float32)
    wt, _, _ = O.apply_weighting(geom, u, v, w0, mode, robust, convention=1)
    return og, keep, u, v, wt


@pytest.mark.parametrize("mode,robust", [("natural", 0.0), ("uniform", 0.0), ("briggs", 0.5)])
def test_cube_plan_and_weights_bit_exact(ctx, cube, mode, robust):
    obs, flags, vis = cube
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), OS)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, np.ones(vis.shape, np.float32),
                      flags)
    sx, sy, rx, ry, wt = cc.cube_sample_taps(gg, cb, mode, robust)
    for c in range(obs.channels):
        og, keep, u, v, wo = _oracle_channel(obs, flags, vis, c, mode, robust)
        ox, oy, orx, ory = og.plan_many(u, v)
        ok = (ox >= 0) & (wo > 0)
        exp = [np.where(ok, a, -1) for a in (ox, oy, orx, ory)]
        for got, want in zip((sx, sy, rx, ry), exp):
            np.testing.assert_array_equal(got[c][keep], want)
        assert np.all(sx[c][~keep] == -1)
        np.testing.assert_array_equal(wt[c][keep], np.where(ok, wo, 0.0).astype(np.float32))


@pytest.mark.parametrize("mode,robust", [("natural", 0.0), ("briggs", 0.5)])
def test_cube_grids_match_oracle_and_plain_loop(ctx, cube, mode, robust):
    obs, flags, vis = cube
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), OS)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    psf, dirty, sums = cc.cube_grid_dirty(gg, cb, mode, robust)
    assert psf.shape == (obs.channels,) + gg.grid_shape()
    for c in range(obs.channels):
        og, keep, u, v, wo = _oracle_channel(obs, flags, vis, c, mode, robust)
        p_o, d_o, acc = og.grid_dirty(u, v, wo, vis[c][keep], threads=8)
        assert sums[c].gridded_samples == acc.gridded
        assert abs(sums[c].normalization_sumwt - acc.normalization_sumwt) <= \
            1e-12 * acc.normalization_sumwt
        assert peak_norm_err(psf[c], p_o.real) <= 1e-5
        assert peak_norm_err(dirty[c], d_o) <= 1e-5
        # the plain single-channel GPU path on the same channel batch
        b = cc.VisibilityBatch(u, v, vis[c][keep], np.ones(len(u), np.float32))
        w1, _ = cc.apply_weighting(gg, b, mode, robust, per_plane=True)
        np.testing.assert_array_equal(w1, wo)
        pg, dg, s1 = cc.grid_dirty(gg, cc.VisibilityBatch(u, v, vis[c][keep], w1))
        assert s1.gridded_samples == acc.gridded
        assert peak_norm_err(psf[c], pg.real) <= 1e-5
        assert peak_norm_err(dirty[c], dg) <= 1e-5


def test_cube_degrid_matches_oracle(ctx, cube):
    obs, flags, vis = cube
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), OS)
    rng = np.random.default_rng(3)
    gs = (obs.channels,) + gg.grid_shape()
    model = (rng.normal(size=gs) + 1j * rng.normal(size=gs)).astype(np.complex64)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    psf, dirty, pred, sums = cc.cube_grid_degrid(gg, cb, model)
    pred2 = cc.cube_degrid(gg, cb, model)
    np.testing.assert_array_equal(pred, pred2)
    for c in range(obs.channels):
        og, keep, u, v, wo = _oracle_channel(obs, flags, vis, c, "natural", 0.0)
        po = og.degrid(model[c], u, v)
        ox, _, _, _ = og.plan_many(u, v)
        po = np.where(ox >= 0, po, 0.0)
        got = pred[c][keep]
        assert float(np.max(np.abs(got - po))) <= 1e-5 * float(np.max(np.abs(po)))
        assert np.all(pred[c][~keep] == 0)


def test_cube_degrid_footprint_paths_agree(ctx, cube):
    """Model footprints arrive by tensor-map copies when the model grids are
    16-byte aligned and by plain loads otherwise (here an 8-byte offset
    view); both feed the same arithmetic, so predictions agree bit for bit."""
    torch = pytest.importorskip("torch")
    obs, flags, vis = cube
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), OS)
    rng = np.random.default_rng(4)
    gs = (obs.channels,) + gg.grid_shape()
    model = (rng.normal(size=gs) + 1j * rng.normal(size=gs)).astype(np.complex64)
    dev = torch.device("cuda", 0)
    u, v, vs, fl = (torch.as_tensor(a).to(dev) for a in (obs.u_m, obs.v_m, vis, flags))
    cb = cc.CubeBatch(u, v, obs.lambda_scale, vs, None, fl)
    aligned = torch.as_tensor(model).to(dev)
    assert aligned.data_ptr() % 16 == 0
    store = torch.zeros(model.size + 1, dtype=torch.complex64, device=dev)
    offset = store[1:].view(gs)
    offset.copy_(aligned)
    assert offset.data_ptr() % 16 == 8
    a = cc.cube_degrid(gg, cb, aligned)
    b = cc.cube_degrid(gg, cb, offset)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_cube_boundary_samples_take_the_oracle_decisions(ctx):
    nx = 256
    cell = 2.0e-5
    geom = O.Geometry(nx, nx, cell, cell)
    og = O.StdGridder(geom, OS)
    ls = np.array([1.0e9, 1.37e9, 1.9e9]) / S.C_LIGHT
    xs = [b + k * 2.0 ** -9 for k in range(-3, 4) for b in (10.5, 100.5, og.gnx - 3.5, 3.5, 2.5)]
    xs += [150.0 - (j + 0.5) / OS for j in range(-66, 66)]
    um = []
    for x in xs:
        base = (x - og.gnx / 2.0) * og.du / ls[1]
        for d in range(-2, 3):
            um.append(base)
            base = np.nextafter(base, np.inf)
    um = np.array(um)
    vm = um[::-1].copy()
    um = np.concatenate([um, [np.nan, np.inf, 1e300, -0.0, 0.0, 5e-324]])
    vm = np.concatenate([vm, [0.0, 0.0, 0.0, -0.0, 0.0, 0.0]])
    R = len(um)
    vis = np.ones((len(ls), R), np.complex64)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), OS)
    sx, sy, rx, ry, wt = cc.cube_sample_taps(gg, cc.CubeBatch(um, vm, ls, vis))
    for c in range(len(ls)):
        ox, oy, orx, ory = og.plan_many(um * ls[c], vm * ls[c])
        np.testing.assert_array_equal(sx[c], ox)
        np.testing.assert_array_equal(sy[c], oy)
        np.testing.assert_array_equal(rx[c], orx)
        np.testing.assert_array_equal(ry[c], ory)


@pytest.mark.parametrize("nx,os_,cell", [(100, 100, 3.1e-5), (150, 100, 2.2e-5), (96, 64, 4.4e-5)])
def test_cube_plan_other_oversampling_and_sizes(ctx, nx, os_, cell):
    """Oversampling 100 (offset boundaries that are not dyadic) and grids whose
    halves are not whole multiples of the tile: the integer path still takes
    the oracle's decisions for every sample."""
    rng = np.random.default_rng(nx)
    geom = O.Geometry(nx, nx, cell, cell)
    og = O.StdGridder(geom, os_)
    ls = np.array([1.0e9, 1.23e9, 1.7e9, 2.0e9]) / S.C_LIGHT
    half = (og.gnx / 2 - 4) * og.du / ls[-1]
    um = rng.uniform(-half, half, 30000)
    vm = rng.uniform(-half, half, 30000)
    vis = np.ones((len(ls), len(um)), np.complex64)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), os_)
    for mode in ("natural", "uniform"):
        sx, sy, rx, ry, wt = cc.cube_sample_taps(gg, cc.CubeBatch(um, vm, ls, vis), mode)
        for c in range(len(ls)):
            u, v = um * ls[c], vm * ls[c]
            wo, _, _ = O.apply_weighting(geom, u, v, np.ones(len(u), np.float32), mode,
                                         convention=1)
            ox, oy, orx, ory = og.plan_many(u, v)
            ok = (ox >= 0) & (wo > 0)
            np.testing.assert_array_equal(sx[c], np.where(ok, ox, -1))
            np.testing.assert_array_equal(sy[c], np.where(ok, oy, -1))
            np.testing.assert_array_equal(rx[c], np.where(ok, orx, -1))
            np.testing.assert_array_equal(ry[c], np.where(ok, ory, -1))
            np.testing.assert_array_equal(wt[c], np.where(ok, wo, 0.0).astype(np.float32))


def test_cube_graph_replay_matches_eager_calls(ctx, cube):
    """All-device calls repeated with the same arrays run eagerly once, are
    captured on the second call and replayed afterwards: each call reads the
    arrays' current contents (new visibilities, new baselines) and agrees
    with an eager call on the same data, with the same kernel count."""
    import torch
    obs, flags, vis = cube
    dev = torch.device("cuda", 0)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), OS)
    gs = (obs.channels,) + gg.grid_shape()
    rng = np.random.default_rng(11)
    model = torch.as_tensor((rng.normal(size=gs) + 1j * rng.normal(size=gs)).astype(np.complex64),
                            device=dev)
    um = torch.as_tensor(obs.u_m, device=dev)
    vm = torch.as_tensor(obs.v_m, device=dev)
    vd = torch.as_tensor(vis, device=dev)
    wd = torch.ones(vis.shape, dtype=torch.float32, device=dev)
    fd = torch.as_tensor(flags, device=dev)
    cb = cc.CubeBatch(um, vm, obs.lambda_scale, vd, wd, fd)
    outs = (torch.empty(gs, dtype=torch.float32, device=dev),
            torch.empty(gs, dtype=torch.complex64, device=dev),
            torch.empty((obs.channels, obs.rows), dtype=torch.complex64, device=dev))

    ctx_e = cc.Context(0)
    ctx_e.set_cube_graphs(False)
    gg_e = cc.StandardGridder(ctx_e, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), OS)

    def eager():
        n0 = ctx_e.launch_count
        p, d, pr, s = cc.cube_grid_degrid(gg_e, cb, model, "briggs", 0.5)
        return p.clone(), d.clone(), pr.clone(), s, ctx_e.launch_count - n0

    ctx.set_cube_graphs(True)
    eager()   # the eager context's first call tunes its chunk size
    for call in range(5):
        if call == 3:
            vd.mul_(1.5)
            um.mul_(1.01)
        n0 = ctx.launch_count
        p, d, pr, s = cc.cube_grid_degrid(gg, cb, model, "briggs", 0.5, out=outs)
        n = ctx.launch_count - n0
        assert p.data_ptr() == outs[0].data_ptr()
        got = (p.clone(), d.clone(), pr.clone(), s)
        ep, ed, epr, es, en = eager()
        if call >= 1:
            assert n == en
        for c in range(obs.channels):
            assert got[3][c].gridded_samples == es[c].gridded_samples
            assert abs(got[3][c].normalization_sumwt - es[c].normalization_sumwt) <= \
                1e-12 * es[c].normalization_sumwt
            assert peak_norm_err(got[0][c].cpu().numpy(), ep[c].cpu().numpy()) <= 1e-6
            assert peak_norm_err(got[1][c].cpu().numpy(), ed[c].cpu().numpy()) <= 1e-6
            assert peak_norm_err(got[2][c].cpu().numpy(), epr[c].cpu().numpy()) <= 1e-6
        t = ctx.last_timings()
        assert t["grid_ms"] > 0
    gg_e.close()
    ctx_e.close()


def test_cube_density_boundary_samples_take_the_oracle_cells(ctx):
    """Samples on and one ulp around density-cell boundaries (odd image
    size, so the centre is a half-integer): uniform weights, which divide by
    each sample's density cell, agree bit-exactly with the oracle."""
    nx = 129
    cell = 2.0e-5
    geom = O.Geometry(nx, nx, cell, cell)
    ls = np.array([1.0e9, 1.37e9, 1.9e9]) / S.C_LIGHT
    dus = nx * cell
    xs = [b + k * 2.0 ** -20 for k in (-1, 0, 1) for b in (5.5, 40.5, 64.0, 90.5, nx - 1.5)]
    um = []
    for x in xs:
        base = (x - nx / 2.0) / (ls[1] * dus)
        for _ in range(3):
            um.append(base)
            base = np.nextafter(base, np.inf)
    um = np.array(um)
    rng = np.random.default_rng(2)
    um = np.concatenate([um, rng.uniform(-0.4, 0.4, 200) / (ls[1] * cell)])
    vm = np.random.default_rng(3).permutation(um)
    R = len(um)
    vis = np.ones((len(ls), R), np.complex64)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), OS)
    sx, sy, rx, ry, wt = cc.cube_sample_taps(gg, cc.CubeBatch(um, vm, ls, vis), "uniform")
    og = O.StdGridder(geom, OS)
    for c in range(len(ls)):
        u, v = um * ls[c], vm * ls[c]
        wo, _, _ = O.apply_weighting(geom, u, v, np.ones(R, np.float32), "uniform", 0.0,
                                     convention=1)
        ox, _, _, _ = og.plan_many(u, v)
        np.testing.assert_array_equal(wt[c], np.where((ox >= 0) & (wo > 0), wo, 0.0)
                                      .astype(np.float32))


def test_cube_edge_cases(ctx, cube):
    """No rows at all: empty grids and zero sums.  A channel whose samples
    are all flagged: empty grids for it, and the other channels as in the
    run without that flag (PerPlane density keeps channels apart)."""
    obs, flags, vis = cube
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), OS)
    C = obs.channels
    empty = cc.CubeBatch(np.zeros(0), np.zeros(0), obs.lambda_scale,
                         np.zeros((C, 0), np.complex64), None, np.zeros((C, 0), np.uint8))
    psf, dirty, sums = cc.cube_grid_dirty(gg, empty, "briggs", 0.5)
    assert not np.any(psf) and not np.any(dirty)
    assert all(s.gridded_samples == 0 and s.normalization_sumwt == 0.0 for s in sums)

    ref_psf, ref_dirty, ref_sums = cc.cube_grid_dirty(
        gg, cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags), "briggs", 0.5)
    f2 = flags.copy()
    f2[3] = 1
    psf, dirty, sums = cc.cube_grid_dirty(
        gg, cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, f2), "briggs", 0.5)
    assert not np.any(psf[3]) and not np.any(dirty[3]) and sums[3].gridded_samples == 0
    for c in range(C):
        if c == 3:
            continue
        assert sums[c].gridded_samples == ref_sums[c].gridded_samples
        assert sums[c].normalization_sumwt == ref_sums[c].normalization_sumwt
        # tiles shared by several work items add with atomics in any order
        assert peak_norm_err(psf[c], ref_psf[c]) <= 1e-6
        assert peak_norm_err(dirty[c], ref_dirty[c]) <= 1e-6
