"""Materialised plans (cr_plan): one plan serves gridding, degridding and
residual refreshes with the same results as the one-shot calls."""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

from gpu_common import arcsec, peak_norm_err, random_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("wproj", [False, True])
def test_plan_reuse_matches_one_shot_calls(ctx, wproj):
    nx, cell = 256, arcsec(15.0)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell))
    gw = cc.WProjector(gg, 3000.0, planes=16, sampling=8, support_law=(4, 12)) if wproj else None
    rng = np.random.default_rng(31)
    du = gg.grid_spacing_lambda()[0]
    u, v, w, wt, vis = random_batch(rng, 20000, gg.grid_shape()[0], du, margin=16, w_max=3000.0)
    u[5000:9000], v[5000:9000], w[5000:9000] = u[:4000], v[:4000], w[:4000]
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    plan = cc.Plan(gg, b, gw)
    psf1, dirty1, sums = cc.grid_dirty(gg, b, gw)
    assert plan.sums.gridded_samples == sums.gridded_samples
    assert plan.sums.unique_records == sums.unique_records
    psf2, dirty2 = plan.grid_dirty()
    assert peak_norm_err(psf2, psf1) <= 1e-6 and peak_norm_err(dirty2, dirty1) <= 1e-6
    shape = gg.grid_shape()
    for seed in (1, 2):
        g = np.random.default_rng(seed)
        grid = (g.normal(size=shape) + 1j * g.normal(size=shape)).astype(np.complex64)
        p1 = cc.degrid(gg, b, grid, gw)
        p2 = plan.degrid(grid)
        np.testing.assert_array_equal(p1, p2)
        r1, _ = cc.grid_residual(gg, b, grid, gw)
        r2 = plan.grid_residual(grid)
        assert peak_norm_err(r2, r1) <= 1e-6
    plan.close()
