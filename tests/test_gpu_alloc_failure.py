"""Allocation failure, simulated on the host (cr_ctx_set_alloc_limit).

A context given a device-memory budget smaller than a call's workspaces
fails that call the way a failed device allocation does: a CasarsCudaError
of kind "Cuda" naming the workspace, before any work, with nothing of the
call left running.  The context stays usable: once the budget is lifted
the same call runs and matches the oracle, and calls that fit a budget run
under it.
"""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

from gpu_common import peak_norm_err, random_batch

pytestmark = pytest.mark.gpu


def test_dirty_image_fails_then_recovers():
    ctx = cc.Context(0)
    try:
        rng = np.random.default_rng(31)
        nx, cell = 96, 5e-5
        og = O.StdGridder(O.Geometry(nx, nx, cell, cell), 100)
        gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell), 100)
        u, v, w, wt, vis = random_batch(rng, 20000, og.gnx, og.du, margin=4)
        batch = cc.VisibilityBatch(u, v, vis, wt)
        assert ctx.workspace_bytes == 0
        ctx.set_alloc_limit(64 * 1024)
        with pytest.raises(cc.CasarsCudaError) as e:
            cc.dirty_image(gg, batch)
        assert e.value.kind == "Cuda" and "allocation limit" in str(e.value)
        assert ctx.workspace_bytes <= 64 * 1024
        ctx.set_alloc_limit(0)
        psf, res, state, sums = cc.dirty_image(gg, batch)
        p, d, acc = og.grid_dirty(u, v, wt, vis)
        psf_o, res_o, _ = og.dirty_products(p, d, acc)
        assert sums.gridded_samples == acc.gridded
        assert peak_norm_err(psf, psf_o) <= 1e-5 and peak_norm_err(res, res_o) <= 1e-5
        # a budget the call's workspaces fit in: the same images again
        held = ctx.workspace_bytes
        ctx.set_alloc_limit(held)
        psf2, res2, _, _ = cc.dirty_image(gg, batch)
        assert ctx.workspace_bytes == held
        assert peak_norm_err(res2, res_o) <= 1e-5
        with pytest.raises(ValueError):
            ctx.set_alloc_limit(-1)
    finally:
        ctx.close()


def test_cube_call_fails_then_recovers():
    ctx = cc.Context(0)
    try:
        from casars_cuda import synthetic as S
        obs = S.cube_observation(channels=4, nx=64, hours=1.0, dump_s=120.0, n_sources=3,
                                 seed=5)
        rng = np.random.default_rng(6)
        vis = (rng.normal(size=(4, obs.rows)) + 1j * rng.normal(size=(4, obs.rows))) \
            .astype(np.complex64)
        flags = (rng.random((4, obs.rows)) < 0.2).astype(np.uint8)
        gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), 128)
        cube = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
        ctx.set_alloc_limit(4096)
        with pytest.raises(cc.CasarsCudaError) as e:
            cc.cube_grid_dirty(gg, cube, "briggs", 0.5)
        assert e.value.kind == "Cuda"
        ctx.set_alloc_limit(0)
        psf_a, dirty_a, sums_a = cc.cube_grid_dirty(gg, cube, "briggs", 0.5)
        psf_b, dirty_b, sums_b = cc.cube_grid_dirty(gg, cube, "briggs", 0.5)
        assert [s.gridded_samples for s in sums_a] == [s.gridded_samples for s in sums_b]
        assert np.max(np.abs(np.asarray(dirty_a) - np.asarray(dirty_b))) <= \
            1e-5 * np.max(np.abs(np.asarray(dirty_b)))
    finally:
        ctx.close()
