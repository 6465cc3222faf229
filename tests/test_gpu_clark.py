"""The Clark minor cycle and controller on the device against the oracle.

* the reference's 5 x 5 case (3 x 3 patch given by ncent = 0 is not
  possible, so the same PSF with ncent 1 builds a 4 x 4 patch; the oracle
  builds the same patch): components, model and residual agree;
* on a 128 x 128 dirty image with its fitted beam's patch, one minor cycle
  gives the oracle's components (positions exactly, fluxes within 1e-5
  relative), stop reason and residual (1e-5 of the peak);
* run_clark_cotton_schwab agrees with the oracle's controller driven by the
  FP64 residual refresh.
"""
import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import clark as OC
from oracle import oracle as O

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def _compare(out, ref):
    assert out.actual_updates == ref["actual"]
    assert out.stop_reason == ref["stop_reason"]
    pos = [tuple(p) for p in out.positions.tolist()]
    assert pos == [c[0] for c in ref["components"]]
    if pos:
        fo = np.array([c[1] for c in ref["components"]])
        assert float(np.max(np.abs(out.fluxes - fo) / np.abs(fo))) <= 1e-5


@pytest.mark.parametrize("device", [False, True])
def test_small_case(ctx, device):
    residual = np.zeros((6, 6), np.float32)
    residual[1:4, 1:4] = [[0.2, 0.4, 0.1], [0.3, 1.0, 0.3], [0.1, 0.4, 0.2]]
    psf = np.zeros((6, 6), np.float32)
    psf[3, 3] = 1.0
    psf[2, 3] = psf[4, 3] = psf[3, 2] = psf[3, 4] = 0.1
    psf[0, 0] = 0.2
    patch = OC.psf_patch(psf, 1)
    ref = OC.clark_minor_cycle(np.zeros_like(residual), residual, psf, patch, 0.2, 3)
    arr = residual
    if device:
        import torch
        arr = torch.from_numpy(residual).cuda()
        psf_in = torch.from_numpy(psf).cuda()
    else:
        psf_in = psf
    out = cc.run_clark_minor_cycle(ctx, np.zeros_like(residual) if not device else
                                   arr * 0, arr, psf_in, 1, 0.2, 3)
    assert ref["actual"] == 3
    _compare(out, ref)
    assert out.max_exterior_abs == pytest.approx(float(patch["max_exterior_abs"]))
    get = (lambda a: a.cpu().numpy()) if device else np.asarray
    np.testing.assert_allclose(get(out.residual), ref["residual"], atol=1e-6)
    np.testing.assert_allclose(get(out.model), ref["model"], atol=1e-7)


def _dirty(nx=128):
    obs = S.observation(1000.0, 1.0, 30.0, 1.4e9, nx, 8, 0.1, 1.0, 11, "loop")
    rng = np.random.default_rng(11)
    obs.vis = S.visibilities(obs.u, obs.v, np.zeros_like(obs.w), obs.sky, nx, nx, obs.cell,
                             0.0, rng, w_term=False)
    wt = np.ones(obs.rows, np.float32)
    og = O.StdGridder(O.Geometry(nx, nx, obs.cell, obs.cell), 128)
    p, d, acc = og.grid_dirty(obs.u, obs.v, wt, obs.vis, threads=8)
    psf_o, res_o, peak_o = og.dirty_products(p, d, acc)

    def refresh(model):
        rg, _, _ = og.residual(og.model_grid(model.astype(np.float64)), obs.u, obs.v, wt,
                               obs.vis, threads=8)
        return og.corrected_image(O.centered_ifft2(rg)) / acc.normalization_sumwt / peak_o
    return obs, wt, psf_o.astype(np.float32), res_o.astype(np.float32), refresh


def test_minor_cycle_on_a_dirty_image(ctx):
    obs, wt, psf, res, _ = _dirty()
    ncent = 6
    patch = OC.psf_patch(psf, ncent)
    ref = OC.clark_minor_cycle(np.zeros_like(res), res, psf, patch, 0.1, 200, 0.0, 0.02)
    out = cc.run_clark_minor_cycle(ctx, np.zeros_like(res), res, psf, ncent, 0.1, 200,
                                   cycle_threshold=0.02)
    assert out.actual_updates > 20
    _compare(out, ref)
    assert peak_norm_err(out.residual, ref["residual"]) <= 1e-5
    assert peak_norm_err(out.model, ref["model"]) <= 1e-5


def test_clark_cotton_schwab_matches_oracle(ctx):
    obs, wt, psf, res, refresh = _dirty()
    nx = obs.nx
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, obs.cell, obs.cell), 128)
    cfg = cc.CleanConfig(niter=300, gain=0.1, minor_cycle_length=60)
    out = cc.run_clark_cotton_schwab(gg, cc.VisibilityBatch(obs.u, obs.v, obs.vis, wt), cfg,
                                     max_psf_sidelobe=0.2)
    ncent = cc.clark_ncent(out.beam, (obs.cell, obs.cell))
    ref = OC.clark_cotton_schwab(res, psf, refresh, OC.psf_patch(psf, ncent), 300, gain=0.1,
                                 minor_cycle_length=60, sidelobe=0.2)
    assert ref["major_cycles"] >= 2 and len(ref["components"]) > 50
    assert out.stop_reason == ref["stop_reason"]
    assert out.major_cycles == ref["major_cycles"]
    assert out.minor_iterations == ref["actual"]
    np.testing.assert_allclose(out.cycle_thresholds, ref["thresholds"], rtol=1e-5)
    assert [c[0] for c in out.components] == [c[0] for c in ref["components"]]
    fl = np.array([c[1] for c in out.components])
    fo = np.array([c[1] for c in ref["components"]])
    assert float(np.max(np.abs(fl - fo) / np.abs(fo))) <= 1e-5
    assert peak_norm_err(out.residual, ref["residual"]) <= 1e-5
