"""Cube CLEAN control on the CPU: casars_cuda.clean.cube_clean_loop (the
control of run_standard_mfs_cube_clean, casa-imaging lib.rs:3026-3210, with
the residual refreshes of a pass batched) against the oracle's restatement
of the same controller with each plane refreshed in turn.  Both drive the
oracle's Hogbom and FP64 residual refresh on a small 4-channel cube, so their
decisions (active planes, cube thresholds, per-plane budgets and stop
reasons) and images must agree exactly."""
import numpy as np
import pytest

from casars_cuda import clean as CL
from casars_cuda import synthetic as S
from oracle import oracle as O


class _Out:
    def __init__(self, d):
        self.model, self.residual = d["model"], d["residual"]
        self.positions = np.stack([d["x"], d["y"]], 1)
        self.fluxes = d["flux"]
        self.actual_updates, self.reported_updates = d["actual"], d["reported"]
        self.stop_reason = O._STOP_NAMES[d["stop_reason"]]


def _planes(obs, flags, vis, os_=64):
    geom = O.Geometry(obs.nx, obs.nx, obs.cell, obs.cell)
    og = O.StdGridder(geom, os_)
    planes = []
    for c in range(obs.channels):
        keep = ~flags[c]
        ls = obs.lambda_scale[c]
        u, v = obs.u_m[keep] * ls, obs.v_m[keep] * ls
        w = np.ones(len(u), np.float32)
        vc = vis[c][keep]
        p, d, acc = og.grid_dirty(u, v, w, vc, threads=4)
        psf, res, peak = og.dirty_products(p, d, acc)

        def refresh(model, u=u, v=v, w=w, vc=vc, acc=acc, peak=peak):
            rg, _, _ = og.residual(og.model_grid(model.astype(np.float64)), u, v, w, vc,
                                   threads=4)
            return (og.corrected_image(O.centered_ifft2(rg)) / acc.normalization_sumwt /
                    peak).astype(np.float32)
        planes.append(dict(residual=res.astype(np.float32), psf=psf.astype(np.float32),
                           refresh=refresh, sidelobe=0.15 + 0.02 * c))
    return planes


# (niter, minor cycle length, major-cycle limit, threshold, weak plane scale,
# nsigma): several passes on every plane, a budget that one pass exceeds, a
# pass limit, a global threshold with a faint plane that joins late, and the
# n-sigma threshold of each plane's robust RMS.
@pytest.mark.parametrize("niter,mcl,limit,thr,weak,nsigma", [
    (120, 25, None, 0.0, 1.0, 0.0), (40, 1000, None, 0.0, 1.0, 0.0), (200, 30, 2, 0.0, 1.0, 0.0),
    (600, 40, None, 0.02, 0.15, 0.0), (2000, 30, None, 0.0, 0.3, 6.0)])
def test_cube_clean_loop_matches_oracle(niter, mcl, limit, thr, weak, nsigma):
    obs = S.cube_observation(channels=4, nx=64, hours=1.0, dump_s=120.0, n_sources=3, seed=5)
    flags = S.cube_flags(obs)
    vis = S.cube_visibilities(obs)
    vis[2] *= np.float32(weak)
    planes = _planes(obs, flags, vis)
    kw = dict(gain=0.1, threshold=thr, minor_cycle_length=mcl, major_cycle_limit=limit)
    ref = O.cube_clean(planes, niter, nsigma=nsigma, **kw)
    if weak < 1.0 and nsigma == 0.0:
        assert 2 not in ref["active"][0] and any(2 in a for a in ref["active"])
        assert "GlobalThresholdReached" in ref["plane_stops"]
    if nsigma > 0.0:
        assert "NsigmaThresholdReached" in ref["plane_stops"]

    cfg = CL.CleanConfig(niter=niter, gain=0.1, threshold_jy_per_beam=thr,
                         minor_cycle_length=mcl, major_cycle_limit=limit, nsigma=nsigma)
    res = np.stack([p["residual"] for p in planes])
    psfs = np.stack([p["psf"] for p in planes])
    models = np.zeros_like(res)

    def hogbom(model, residual, psf, n, threshold, cycle_threshold, nsigma_threshold):
        return _Out(O.hogbom(residual, psf, 0.1, n, threshold=threshold,
                             cycle_threshold=cycle_threshold,
                             nsigma_threshold=nsigma_threshold, model=model, inclusive=True))

    def refresh(cs):
        for c in cs:
            res[c] = planes[c]["refresh"](models[c])

    def nsigma_fn(cs):
        return [O.nsigma_threshold(res[c], nsigma) for c in cs]

    out = CL.cube_clean_loop(res, psfs, models, [p["sidelobe"] for p in planes], cfg, hogbom,
                             refresh, nsigma_fn=nsigma_fn)
    assert out["major_cycles"] == ref["major_cycles"] and out["major_cycles"] > 0
    assert out["minor_iterations"] == ref["minor_iterations"]
    assert out["active"] == ref["active"]
    assert out["thresholds"] == ref["thresholds"]
    assert out["plane_iterations"] == ref["plane_iterations"]
    assert out["plane_stops"] == ref["plane_stops"]
    assert out["final_cycle_threshold"] == ref["final_cycle_threshold"]
    assert out["planes_at_or_below_initial_threshold"] == \
        ref["planes_at_or_below_initial_threshold"]
    assert out["initial_peak"] == ref["initial_peak"]
    for c in range(obs.channels):
        assert [tuple(p) for p, _ in out["components"][c]] == \
            [tuple(p) for p, _ in ref["components"][c]]
        np.testing.assert_array_equal(models[c], ref["models"][c])
        np.testing.assert_array_equal(res[c], ref["residuals"][c])
