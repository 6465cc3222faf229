"""The bounded device waits give up cleanly, and the context stays usable.

Every wait in the library's kernels is bounded: the Hogbom grid barrier
(blocks of the cooperative launch waiting for each other) and the cube
kernels' waits on bulk copies into shared memory.  With the bound set to
zero through cr_ctx_set_wait_limits, a wait gives up at once: the kernel
records CR_TIMEOUT and returns (a cube block first lets its copies in
flight land, under the default bound), and the call reports the timeout.
The next call, with the default bounds restored, must give the oracle's
answer on the same context.  Nothing here faults or hangs the device: the
waits that run out are ordinary bounded loops.
"""
import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from casars_cuda._lib import CR_TIMEOUT
from oracle import oracle as O

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu


@pytest.fixture()
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def hogbom_inputs(nx=256, ny=256):
    rng = np.random.default_rng(17)
    x = np.arange(nx)[:, None] - nx // 2
    y = np.arange(ny)[None, :] - ny // 2
    psf = np.exp(-(x * x + y * y) / 18.0).astype(np.float32)
    psf[nx // 2, ny // 2] = 1.0
    res = (0.01 * rng.normal(size=(nx, ny))).astype(np.float32)
    for _ in range(10):
        px, py = rng.integers(10, nx - 10), rng.integers(10, ny - 10)
        res[px, py] += rng.uniform(0.1, 1.0)
    return res, psf


def test_hogbom_barrier_timeout_then_normal_call(ctx):
    res, psf = hogbom_inputs()
    # 256 x 256 pixels run on 128 blocks: all but the last to arrive wait
    ctx.set_wait_limits(barrier_polls=0)
    with pytest.raises(cc.CasarsCudaError) as e:
        cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res), res, psf, 0.1, 200)
    assert e.value.code == CR_TIMEOUT and e.value.kind == "Timeout"
    ctx.set_wait_limits()
    ref = O.hogbom(res, psf, 0.1, 200)
    out = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res), res, psf, 0.1, 200)
    assert out.actual_updates == ref["actual"]
    np.testing.assert_array_equal(out.positions[:, 0], ref["x"])
    np.testing.assert_array_equal(out.positions[:, 1], ref["y"])
    np.testing.assert_array_equal(out.residual, ref["residual"])
    np.testing.assert_array_equal(out.model, ref["model"])


def test_hogbom_planes_barrier_timeout_then_normal_call(ctx):
    import torch
    res, psf = hogbom_inputs(128, 128)
    res2 = np.stack([res, res[::-1].copy()])
    psf2 = np.stack([psf, psf])
    dev = torch.device("cuda", 0)

    def run():
        m = torch.zeros(res2.shape, dtype=torch.float32, device=dev)
        r = torch.as_tensor(res2, device=dev).contiguous()
        p = torch.as_tensor(psf2, device=dev).contiguous()
        cc.run_hogbom_planes(ctx, m, r, p, [0, 1], 0.1, 50)
        return m.cpu().numpy(), r.cpu().numpy()

    ctx.set_wait_limits(barrier_polls=0)
    with pytest.raises(cc.CasarsCudaError) as e:
        run()
    assert e.value.code == CR_TIMEOUT
    ctx.set_wait_limits()
    m, r = run()
    for k in range(2):
        ref = O.hogbom(res2[k], psf2[k], 0.1, 50)
        np.testing.assert_array_equal(r[k], ref["residual"])
        np.testing.assert_array_equal(m[k], ref["model"])


@pytest.fixture(scope="module")
def cube():
    obs = S.cube_observation(channels=4, nx=128, hours=1.0, dump_s=60.0, n_sources=4, seed=12)
    return obs, S.cube_flags(obs), S.cube_visibilities(obs)


def test_cube_copy_waits_timeout_then_normal_call(ctx, cube):
    """The cube gridder's tap-table wait and the degridder's footprint waits
    (tensor-map copies: the 160 x 160 grid meets the tensor-map rules)."""
    obs, flags, vis = cube
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), 128)
    assert gg.grid_shape()[1] % 2 == 0
    rng = np.random.default_rng(4)
    gs = (obs.channels,) + gg.grid_shape()
    model = (rng.normal(size=gs) + 1j * rng.normal(size=gs)).astype(np.complex64)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    ctx.set_wait_limits(mbar_polls=0)
    for fn in (lambda: cc.cube_grid_dirty(gg, cb, "natural", 0.0),
               lambda: cc.cube_degrid(gg, cb, model)):
        with pytest.raises(cc.CasarsCudaError) as e:
            fn()
        assert e.value.code == CR_TIMEOUT
    ctx.set_wait_limits()
    psf, dirty, sums = cc.cube_grid_dirty(gg, cb, "natural", 0.0)
    pred = cc.cube_degrid(gg, cb, model)
    geom = O.Geometry(obs.nx, obs.nx, obs.cell, obs.cell)
    og = O.StdGridder(geom, 128)
    for c in range(obs.channels):
        keep = ~flags[c]
        ls = obs.lambda_scale[c]
        u, v = obs.u_m[keep] * ls, obs.v_m[keep] * ls
        wt = np.ones(len(u), np.float32)
        p_o, d_o, acc = og.grid_dirty(u, v, wt, vis[c][keep])
        assert sums[c].gridded_samples == acc.gridded
        assert peak_norm_err(psf[c], p_o.real) <= 1e-5
        assert peak_norm_err(dirty[c], d_o) <= 1e-5
        ox, _, _, _ = og.plan_many(u, v)
        po = np.where(ox >= 0, og.degrid(model[c], u, v), 0.0)
        assert float(np.max(np.abs(pred[c][keep] - po))) <= 1e-5 * float(np.max(np.abs(po)))
