"""Cotton-Schwab major/minor loop on the device against the oracle's loop.

The device loop (casars_cuda.clean.run_cotton_schwab: cr_hogbom minor cycles,
cr_plan_residual_image refreshes) and the oracle loop (oracle.cotton_schwab:
the C Hogbom and the FP64 residual) run on the same noise-free point-source
observation.  Every component position matches, fluxes agree within 1e-5
relative, the cycle thresholds, major-cycle count and stop reason agree, and
the final residual is within 1e-5 of the oracle's peak; the restored image
(fitted beam, model convolved plus residual) agrees with the oracle's.
"""
import math

import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import oracle as O

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def _obs(seed, nx, w_term):
    obs = S.observation(1000.0, 1.0, 30.0, 1.4e9, nx, 8, 0.1, 1.0, seed, "loop")
    rng = np.random.default_rng(seed)
    w = obs.w if w_term else np.zeros_like(obs.w)
    obs.vis = S.visibilities(obs.u, obs.v, w, obs.sky, nx, nx, obs.cell, 0.0, rng,
                             w_term=w_term)
    return obs


def _compare(out, ref):
    assert out.stop_reason == ref["stop_reason"]
    assert out.major_cycles == ref["major_cycles"]
    assert out.reported_iterations == ref["reported"]
    assert out.minor_iterations == ref["actual"]
    np.testing.assert_allclose(out.cycle_thresholds, ref["thresholds"], rtol=1e-5)
    pos = [c[0] for c in out.components]
    pos_o = [tuple(c[0]) for c in ref["components"]]
    assert pos == pos_o
    fl = np.array([c[1] for c in out.components])
    fl_o = np.array([c[1] for c in ref["components"]])
    assert float(np.max(np.abs(fl - fl_o) / np.abs(fl_o))) <= 1e-5
    assert peak_norm_err(out.residual, ref["residual"]) <= 1e-5
    assert peak_norm_err(out.model, ref["model"]) <= 1e-5


@pytest.mark.parametrize("host", [True, False])
def test_standard_loop_matches_oracle(ctx, host):
    nx = 256
    obs = _obs(11, nx, False)
    wt = np.ones(obs.rows, np.float32)
    og = O.StdGridder(O.Geometry(nx, nx, obs.cell, obs.cell), 128)
    p, d, acc = og.grid_dirty(obs.u, obs.v, wt, obs.vis, threads=8)
    psf_o, res_o, peak_o = og.dirty_products(p, d, acc)

    def refresh(model):
        rg, _, _ = og.residual(og.model_grid(model.astype(np.float64)), obs.u, obs.v, wt,
                               obs.vis, threads=8)
        return og.corrected_image(O.centered_ifft2(rg)) / acc.normalization_sumwt / peak_o

    kw = dict(niter=300, gain=0.1, minor_cycle_length=60)
    ref = O.cotton_schwab(res_o, psf_o, refresh, sidelobe=0.2, **kw)

    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, obs.cell, obs.cell), 128)
    if host:
        b = cc.VisibilityBatch(obs.u, obs.v, obs.vis, wt)
    else:
        import torch
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        b = cc.VisibilityBatch(t(obs.u), t(obs.v), t(obs.vis), t(wt))
    out = cc.run_cotton_schwab(gg, b, cc.CleanConfig(**kw), max_psf_sidelobe=0.2)
    if not host:
        out.residual = out.residual.cpu().numpy()
        out.model = out.model.cpu().numpy()
        out.restored = out.restored.cpu().numpy()
    assert ref["major_cycles"] >= 3
    _compare(out, ref)
    # the restored image: the oracle's beam fit of its PSF, restoration of its
    # model plus residual
    from oracle import beam as OB
    cell = (obs.cell, obs.cell)
    ob, _, _ = OB.fit_beam(psf_o.astype(np.float32), cell, 0.35)
    assert out.beam is not None
    for a, b2 in ((out.beam.major_fwhm_rad, ob.major_fwhm_rad),
                  (out.beam.minor_fwhm_rad, ob.minor_fwhm_rad)):
        assert abs(a - b2) <= 1e-4 * b2
    rest = OB.restore(ref["model"], ref["residual"], cell, ob)
    assert peak_norm_err(out.restored, rest) <= 1e-4


def test_wproj_loop_matches_oracle(ctx):
    nx = 256
    obs = _obs(12, nx, True)
    wt = np.ones(obs.rows, np.float32)
    wmax = float(np.max(np.abs(obs.w)))
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, obs.cell, obs.cell))
    gw = cc.WProjector(gg, wmax, planes=16, sampling=8, support_law=(4, 12))
    og = O.StdGridder(O.Geometry(nx, nx, obs.cell, obs.cell))
    ow = O.WProjector(og.geom, og, wmax, planes=16, sampling=8, support_min=4, support_max=12)
    p, d, acc = ow.grid_dirty(obs.u, obs.v, obs.w, wt, obs.vis, threads=8)
    psf_o, res_o, peak_o = ow.dirty_products(p, d, acc)

    def refresh(model):
        rg, _ = ow.residual(ow.model_grid(model.astype(np.float64)), obs.u, obs.v, obs.w, wt,
                            obs.vis, threads=8)
        return 2.0 * ow.corrected_image(O.centered_ifft2(rg)) / acc.normalization_sumwt / peak_o

    kw = dict(niter=200, gain=0.1, minor_cycle_length=50)
    ref = O.cotton_schwab(res_o, psf_o, refresh, sidelobe=0.2, **kw)
    b = cc.VisibilityBatch(obs.u, obs.v, obs.vis, wt, obs.w)
    out = cc.run_cotton_schwab(gg, b, cc.CleanConfig(**kw), wproj=gw, max_psf_sidelobe=0.2)
    assert ref["major_cycles"] >= 3
    _compare(out, ref)
