"""run_imaging over the library: the request's pieces composed as the
reference's entry point composes them.

* niter 0 gives cr_dirty_image's PSF and residual (and the oracle's within
  1e-5 of the peak), the image being the residual;
* Hogbom with natural weighting over two batches equals run_cotton_schwab on
  the concatenated batch;
* Clark with uniform weighting equals apply_weighting followed by
  run_clark_cotton_schwab.
"""
import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import oracle as O

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    ctx = cc.Context(0)
    nx = 128
    obs = S.observation(1000.0, 1.0, 60.0, 1.4e9, nx, 8, 0.1, 1.0, 31, "run")
    rng = np.random.default_rng(31)
    obs.vis = S.visibilities(obs.u, obs.v, np.zeros_like(obs.w), obs.sky, nx, nx, obs.cell,
                             0.0, rng, w_term=False)
    wt = np.ones(obs.rows, np.float32)
    yield ctx, obs, wt
    ctx.close()


def _geom(obs):
    return cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell)


def test_dirty_only(setup):
    ctx, obs, wt = setup
    b = cc.VisibilityBatch(obs.u, obs.v, obs.vis, wt)
    r = cc.run_imaging(ctx, cc.ImagingRequest(_geom(obs), [b]))
    gg = cc.StandardGridder(ctx, _geom(obs), 100)
    psf, res, state, _ = cc.dirty_image(gg, b)
    # the grids' float32 atomics add in a different order from run to run
    assert peak_norm_err(r.psf, psf) <= 1e-5
    assert peak_norm_err(r.residual, res) <= 1e-5
    np.testing.assert_array_equal(r.image, r.residual)
    assert r.sumwt == state.reported_sumwt and r.beam is not None
    og = O.StdGridder(O.Geometry(obs.nx, obs.nx, obs.cell, obs.cell), 100)
    p, d, acc = og.grid_dirty(obs.u, obs.v, wt, obs.vis, threads=8)
    psf_o, res_o, _ = og.dirty_products(p, d, acc)
    assert peak_norm_err(r.residual, res_o) <= 1e-5


def test_hogbom_two_batches(setup):
    ctx, obs, wt = setup
    h = obs.rows // 2
    parts = [cc.VisibilityBatch(obs.u[a:b], obs.v[a:b], obs.vis[a:b], wt[a:b])
             for a, b in ((0, h), (h, obs.rows))]
    cfg = cc.CleanConfig(niter=150, gain=0.1, minor_cycle_length=50)
    r = cc.run_imaging(ctx, cc.ImagingRequest(_geom(obs), parts, cfg))
    gg = cc.StandardGridder(ctx, _geom(obs), 100)
    ref = cc.run_cotton_schwab(gg, cc.VisibilityBatch(obs.u, obs.v, obs.vis, wt), cfg)
    assert r.minor_iterations == ref.minor_iterations > 0
    assert r.stop_reason == ref.stop_reason and r.major_cycles == ref.major_cycles
    assert [c[0] for c in r.components] == [c[0] for c in ref.components]
    assert peak_norm_err(r.residual, ref.residual) <= 1e-5
    assert peak_norm_err(r.image, ref.restored) <= 1e-5


def test_clark_uniform(setup):
    ctx, obs, wt = setup
    b = cc.VisibilityBatch(obs.u, obs.v, obs.vis, wt)
    cfg = cc.CleanConfig(niter=120, gain=0.1, minor_cycle_length=60)
    r = cc.run_imaging(ctx, cc.ImagingRequest(_geom(obs), [b], cfg, weighting="uniform",
                                              deconvolver="clark"))
    gg = cc.StandardGridder(ctx, _geom(obs), 100)
    w, _ = cc.apply_weighting(gg, b, "uniform")
    ref = cc.run_clark_cotton_schwab(gg, cc.VisibilityBatch(obs.u, obs.v, obs.vis, w), cfg)
    assert r.minor_iterations == ref.minor_iterations > 0
    assert [c[0] for c in r.components] == [c[0] for c in ref.components]
    assert peak_norm_err(r.residual, ref.residual) <= 1e-5


def test_dirty_grid_plan_then_finish(setup):
    """run_standard_mfs_dirty_grid_plan over three blocks with Briggs
    weighting, then finish_standard_mfs_dirty_grid_result, against
    run_imaging (niter 0) on the same request."""
    ctx, obs, wt = setup
    cuts = [0, obs.rows // 3, 2 * obs.rows // 3, obs.rows]
    blocks = [cc.VisibilityBatch(obs.u[a:b], obs.v[a:b], obs.vis[a:b], wt[a:b])
              for a, b in zip(cuts[:-1], cuts[1:])]
    req = cc.ImagingRequest(_geom(obs), blocks, weighting="briggs", robust=0.5)
    raw = cc.run_standard_mfs_dirty_grid_plan(ctx, req)
    assert len(raw.block_sums) == 3
    psf, res, state = cc.finish_standard_mfs_dirty_grid_result(ctx, raw)
    ref = cc.run_imaging(ctx, req)
    assert raw.gridded_samples + raw.skipped_samples == obs.rows
    assert peak_norm_err(psf, ref.psf) <= 1e-5
    assert peak_norm_err(res, ref.residual) <= 1e-5
    assert abs(state.reported_sumwt - ref.sumwt) <= 1e-6 * ref.sumwt
    with pytest.raises(ValueError):
        cc.run_standard_mfs_plan(ctx, cc.ImagingRequest(_geom(obs), blocks,
                                                        w_term_mode="wproject"))
