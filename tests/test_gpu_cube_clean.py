"""Persistent cube plans and cube CLEAN on the device against the oracle.

A small cube (6 channels over 1-2 GHz, 128 x 128 image, point sources,
seeded per-channel flags) is planned once (cr_cube_plan_create) and replayed:

* plan gridding and degridding agree with the one-shot cube calls;
* residual grids (degrid the model grids, grid w (vis - pred)) of the
  selected planes agree with the oracle's FP64 residual gridding within
  1e-5 of each channel's peak, and unselected planes are left untouched;
* PSF and residual images with their PSF states agree with the oracle's
  dirty products per channel, and model -> residual images with the
  oracle's major-cycle refresh, within 1e-5 of the peak, with float32 or
  FP64 image transforms;
* run_cube_clean (batched refreshes, cr_hogbom per plane) agrees with the
  oracle's run_standard_mfs_cube_clean restatement (each plane refreshed in
  turn): component positions exactly, fluxes within 1e-5 relative, the same
  passes, active planes, budgets and stop reasons.
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
    obs = S.cube_observation(channels=6, nx=128, hours=1.0, dump_s=60.0, n_sources=4, seed=21)
    flags = S.cube_flags(obs)
    vis = S.cube_visibilities(obs)
    return obs, flags, vis


def _oracle_planes(obs, flags, vis, mode="natural", robust=0.0):
    geom = O.Geometry(obs.nx, obs.nx, obs.cell, obs.cell)
    og = O.StdGridder(geom, OS)
    out = []
    for c in range(obs.channels):
        keep = ~flags[c]
        ls = obs.lambda_scale[c]
        u, v = obs.u_m[keep] * ls, obs.v_m[keep] * ls
        w0 = np.ones(len(u), np.float32)
        wt, _, _ = O.apply_weighting(geom, u, v, w0, mode, robust, convention=1)
        vc = vis[c][keep]
        p, d, acc = og.grid_dirty(u, v, wt, vc, threads=8)
        psf, res, peak = og.dirty_products(p, d, acc)

        def refresh(model, u=u, v=v, wt=wt, vc=vc, acc=acc, peak=peak):
            rg, _, _ = og.residual(og.model_grid(model.astype(np.float64)), u, v, wt, vc,
                                   threads=8)
            return (og.corrected_image(O.centered_ifft2(rg)) / acc.normalization_sumwt /
                    peak).astype(np.float32)
        out.append(dict(og=og, u=u, v=v, wt=wt, vis=vc, acc=acc, psf=psf, residual=res,
                        peak=peak, refresh=refresh))
    return out


def _gridder(ctx, obs):
    return cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), OS)


def test_cube_plan_replays_the_one_shot_calls(ctx, cube):
    obs, flags, vis = cube
    gg = _gridder(ctx, obs)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    plan = cc.CubePlan(gg, cb, "briggs", 0.5)
    psf, dirty, sums = cc.cube_grid_dirty(gg, cb, "briggs", 0.5)
    for k in range(2):   # the plan replays any number of times
        p2, d2 = plan.grid_dirty()
        for c in range(obs.channels):
            assert peak_norm_err(p2[c], psf[c]) <= 1e-6
            assert peak_norm_err(d2[c], dirty[c]) <= 1e-6
    for a, b in zip(plan.sums, sums):
        assert a.gridded_samples == b.gridded_samples
        assert a.normalization_sumwt == b.normalization_sumwt
    rng = np.random.default_rng(4)
    gs = (obs.channels,) + gg.grid_shape()
    model = (rng.normal(size=gs) + 1j * rng.normal(size=gs)).astype(np.complex64)
    np.testing.assert_array_equal(plan.degrid(model), cc.cube_degrid(gg, cb, model, "briggs", 0.5))
    plan.close()


def test_cube_plan_residual_grids_match_oracle(ctx, cube):
    obs, flags, vis = cube
    gg = _gridder(ctx, obs)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    plan = cc.CubePlan(gg, cb)
    ref = _oracle_planes(obs, flags, vis)
    rng = np.random.default_rng(6)
    gs = (obs.channels,) + gg.grid_shape()
    model = (rng.normal(size=gs) + 1j * rng.normal(size=gs)).astype(np.complex64)
    sentinel = np.full(gs, 7.0 + 3.0j, np.complex64)
    planes = np.array([1, 0, 1, 1, 0, 1], np.uint8)
    for sel in (None, planes):
        out = sentinel.copy()
        res = plan.grid_residual(model, planes=sel, out=out)
        assert res is out
        for c in range(obs.channels):
            if sel is not None and not sel[c]:
                np.testing.assert_array_equal(res[c], sentinel[c])
                continue
            r = ref[c]
            rg, _, _ = r["og"].residual(model[c].astype(np.complex128), r["u"], r["v"], r["wt"],
                                        r["vis"], threads=8)
            assert peak_norm_err(res[c], rg) <= 1e-5
    plan.close()


@pytest.mark.parametrize("mode,robust,bits", [("natural", 0.0, 32), ("briggs", 0.5, 32),
                                              ("briggs", 0.5, 64)])
def test_cube_plan_images_match_oracle(ctx, cube, mode, robust, bits):
    """Float32 (default) and FP64 image-stage transforms."""
    obs, flags, vis = cube
    gg = _gridder(ctx, obs)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    plan = cc.CubePlan(gg, cb, mode, robust, fft_bits=bits)
    ref = _oracle_planes(obs, flags, vis, mode, robust)
    psf, res, states = plan.dirty_images()
    models = np.zeros((obs.channels, obs.nx, obs.nx), np.float32)
    rng = np.random.default_rng(8)
    for c in range(obs.channels):
        r = ref[c]
        assert peak_norm_err(psf[c], r["psf"]) <= 1e-5
        assert peak_norm_err(res[c], r["residual"]) <= 1e-5
        assert abs(states[c].psf_peak - r["peak"]) <= 1e-6 * r["peak"]
        assert abs(states[c].normalization_sumwt - r["acc"].normalization_sumwt) <= \
            1e-6 * r["acc"].normalization_sumwt
        for _ in range(5):
            models[c, rng.integers(10, 118), rng.integers(10, 118)] = rng.uniform(0.1, 1.0)
    sel = np.array([0, 1, 1, 0, 1, 1], np.uint8)
    out = res.copy()
    got = plan.residual_images(models, states, planes=sel, out=out)
    for c in range(obs.channels):
        if not sel[c]:
            np.testing.assert_array_equal(got[c], res[c])
            continue
        want = ref[c]["refresh"](models[c])
        assert peak_norm_err(got[c], want) <= 1e-5
    plan.close()


@pytest.mark.parametrize("device", [False, True])
def test_cube_clean_matches_oracle(ctx, cube, device):
    obs, flags, vis = cube
    vis = vis.copy()
    vis[3] *= np.float32(0.2)    # a faint plane that joins in a later pass
    gg = _gridder(ctx, obs)
    if device:
        import torch
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        cb = cc.CubeBatch(t(obs.u_m), t(obs.v_m), obs.lambda_scale, t(vis), None,
                          t(flags.astype(np.uint8)))
    else:
        cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    ref_planes = _oracle_planes(obs, flags, vis)
    sl = 0.2
    kw = dict(gain=0.1, threshold=0.01, minor_cycle_length=40)
    for p in ref_planes:
        p["sidelobe"] = sl
    ref = O.cube_clean(ref_planes, 400, **kw)
    assert ref["major_cycles"] >= 2
    cfg = cc.CleanConfig(niter=400, gain=0.1, threshold_jy_per_beam=0.01, minor_cycle_length=40)
    out = cc.run_cube_clean(gg, cb, cfg, max_psf_sidelobe=sl)
    assert out.major_cycles == ref["major_cycles"]
    assert out.active_planes == ref["active"]
    np.testing.assert_allclose(out.cycle_thresholds, ref["thresholds"], rtol=1e-5)
    assert out.plane_iterations == ref["plane_iterations"]
    assert out.minor_iterations == ref["minor_iterations"]
    assert out.plane_stop_reasons == ref["plane_stops"]
    to_np = (lambda a: a.cpu().numpy()) if device else np.asarray
    for c in range(obs.channels):
        pos = [tuple(p) for p, _ in out.components[c]]
        assert pos == [tuple(p) for p, _ in ref["components"][c]]
        if pos:
            fl = np.array([f for _, f in out.components[c]])
            fo = np.array([f for _, f in ref["components"][c]])
            assert float(np.max(np.abs(fl - fo) / np.abs(fo))) <= 1e-5
        assert peak_norm_err(to_np(out.residuals[c]), ref["residuals"][c]) <= 1e-5
        assert peak_norm_err(to_np(out.models[c]), ref["models"][c]) <= 1e-5
        assert out.beams[c] is not None
    assert out.restored is not None


def test_hogbom_planes_equals_single_plane_calls(ctx, cube):
    """cr_hogbom_planes on a subset of planes gives each listed plane exactly
    what cr_hogbom gives it alone, and leaves the other planes untouched."""
    import torch
    obs, flags, vis = cube
    gg = _gridder(ctx, obs)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    plan = cc.CubePlan(gg, cb)
    psf, res, states = plan.dirty_images()
    plan.close()
    P = obs.channels
    psf_d = torch.as_tensor(psf).cuda().contiguous()
    res_d = torch.as_tensor(res).cuda().contiguous()
    mod_d = torch.zeros_like(res_d)
    planes = [4, 0, 2, 5]
    outs = cc.run_hogbom_planes(ctx, mod_d, res_d, psf_d, planes, 0.1, 60,
                                cycle_threshold=0.05)
    for s, c in enumerate(planes):
        one = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res[c]), res[c], psf[c], 0.1, 60,
                                        cycle_threshold=0.05)
        o = outs[s]
        assert o.actual_updates == one.actual_updates > 0
        assert o.reported_updates == one.reported_updates
        assert o.stop_reason == one.stop_reason
        np.testing.assert_array_equal(o.positions, one.positions)
        np.testing.assert_array_equal(o.fluxes, one.fluxes)
        np.testing.assert_array_equal(res_d[c].cpu().numpy(), one.residual)
        np.testing.assert_array_equal(mod_d[c].cpu().numpy(), one.model)
    for c in set(range(P)) - set(planes):
        np.testing.assert_array_equal(res_d[c].cpu().numpy(), res[c])
        assert float(mod_d[c].abs().max()) == 0.0


def test_cube_clean_nsigma_matches_oracle(ctx, cube):
    """The per-plane n-sigma threshold (nsigma * the plane's robust RMS, all
    active planes in one batched cr_robust_rms call) in the cube loop: the
    same passes, budgets and stop reasons as the oracle's loop, most planes
    stopping at their n-sigma threshold."""
    import torch
    obs, flags, vis = cube
    vis = vis.copy()
    vis[3] *= np.float32(0.2)
    gg = _gridder(ctx, obs)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    cb = cc.CubeBatch(t(obs.u_m), t(obs.v_m), obs.lambda_scale, t(vis), None,
                      t(flags.astype(np.uint8)))
    ref_planes = _oracle_planes(obs, flags, vis)
    for p in ref_planes:
        p["sidelobe"] = 0.2
    dirty_peak = [float(np.max(np.abs(p["residual"]))) for p in ref_planes]
    kw = dict(gain=0.1, threshold=0.0, minor_cycle_length=40, nsigma=10.0)
    ref = O.cube_clean(ref_planes, 1000, **kw)
    assert ref["plane_stops"].count("NsigmaThresholdReached") >= 4
    cfg = cc.CleanConfig(niter=1000, gain=0.1, minor_cycle_length=40, nsigma=10.0)
    out = cc.run_cube_clean(gg, cb, cfg, max_psf_sidelobe=0.2, restore=False)
    assert out.major_cycles == ref["major_cycles"]
    assert out.active_planes == ref["active"]
    assert out.plane_iterations == ref["plane_iterations"]
    assert out.plane_stop_reasons == ref["plane_stops"]
    for c in range(obs.channels):
        assert [tuple(p) for p, _ in out.components[c]] == \
            [tuple(p) for p, _ in ref["components"][c]]
        # residual errors scale with the plane's image before cleaning (float32
        # sums of full-amplitude visibilities, in a run-dependent order), not
        # with the small residual left at the 10-sigma stop
        err = float(np.max(np.abs(out.residuals[c].cpu().numpy() - ref["residuals"][c])))
        assert err <= 1e-5 * dirty_peak[c]
        assert err <= 1e-4 * float(np.max(np.abs(ref["residuals"][c])))


def test_hogbom_planes_per_plane_nsigma(ctx, cube):
    """cr_hogbom_planes with one n-sigma threshold per listed plane equals
    cr_hogbom on each plane with its own threshold."""
    import torch
    obs, flags, vis = cube
    gg = _gridder(ctx, obs)
    cb = cc.CubeBatch(obs.u_m, obs.v_m, obs.lambda_scale, vis, None, flags)
    plan = cc.CubePlan(gg, cb)
    psf, res, states = plan.dirty_images()
    plan.close()
    psf_d = torch.as_tensor(psf).cuda().contiguous()
    res_d = torch.as_tensor(res).cuda().contiguous()
    mod_d = torch.zeros_like(res_d)
    planes = [1, 3, 4]
    peaks = [float(np.max(np.abs(res[c]))) for c in planes]
    nsig = [0.5 * peaks[0], 0.05 * peaks[1], 0.3 * peaks[2]]
    outs = cc.run_hogbom_planes(ctx, mod_d, res_d, psf_d, planes, 0.1, 200,
                                nsigma_threshold=nsig)
    for s, c in enumerate(planes):
        one = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res[c]), res[c], psf[c], 0.1, 200,
                                        nsigma_threshold=nsig[s])
        assert outs[s].actual_updates == one.actual_updates > 0
        assert outs[s].stop_reason == one.stop_reason
        np.testing.assert_array_equal(outs[s].positions, one.positions)
        np.testing.assert_array_equal(res_d[c].cpu().numpy(), one.residual)
    assert outs[0].stop_reason == "NsigmaThresholdReached"
