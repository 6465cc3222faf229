"""Row runs on the device against the oracle's restatement.

Rows of a small observation with 4 correlations (XX, XY, YX, YY) over 6
channels, with seeded flags, zero / negative / non-finite weights, non-finite
visibilities, a weight spectrum or row weights, and non-gridable rows:

* cr_row_runs_prepare keeps the same samples as the oracle, in the same
  order, with bit-identical u, v, w, weights, sumwt factors, gridable flags,
  visibilities and density coordinates, for every plane (explicit
  correlations and all four pair transforms), from host and device inputs;
* cr_apply_weighting_rows (density built at the row path's VisImagingWeight
  coordinates, looked up at u, v) gives the oracle's weights: bit-exactly
  with unit row weights (every density sum exact), within 1e-5 relative with
  random weights (float32 density sums in another order);
* the dirty image of the prepared, weighted batch agrees with the oracle's
  within 1e-5 of the peak.
"""
import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import oracle as O
from oracle import rows as OR

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu

CORR = [9, 10, 11, 12]


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def runs():
    obs = S.cube_observation(channels=6, nx=128, hours=1.0, dump_s=90.0, n_sources=4, seed=13)
    R, C, K = obs.rows, obs.channels, 4
    rng = np.random.default_rng(17)
    vis = S.cube_visibilities(obs).T            # [R][C] Stokes-I-like sky
    data = np.empty((R, C, K), np.complex64)
    data[:, :, 0] = vis * (1 + 0.05j)
    data[:, :, 3] = vis * (1 - 0.03j)
    data[:, :, 1] = 0.01 * (rng.normal(size=(R, C)) + 1j * rng.normal(size=(R, C)))
    data[:, :, 2] = 0.01 * (rng.normal(size=(R, C)) + 1j * rng.normal(size=(R, C)))
    data[5, 2, 0] = np.nan
    data[7, 1, 3] = np.inf
    flag = (rng.random((R, C, K)) < 0.1).astype(np.uint8)
    weight = rng.uniform(0.5, 2.0, (R, K)).astype(np.float32)
    weight[3, 0] = 0.0
    weight[4, 3] = -1.0
    weight[6, 1] = np.nan
    spectrum = rng.uniform(0.5, 2.0, (R, C, K)).astype(np.float32)
    spectrum[8, 0, 0] = 0.0
    gridable = (rng.random(R) > 0.05).astype(np.uint8)
    uvw = np.stack([obs.u_m, obs.v_m, rng.normal(0.0, 50.0, R)], 1)
    return obs, uvw, data, flag, weight, spectrum, gridable


def _cases():
    out = []
    for plane in ("I", "Q", "U", "V", "XX", "YY"):
        for spec in (False, True):
            out.append((plane, spec))
    return out


@pytest.mark.parametrize("plane,spec", _cases())
def test_prepare_matches_oracle(ctx, runs, plane, spec):
    obs, uvw, data, flag, weight, spectrum, gridable = runs
    corr0, corr1, transform, factor = OR.plane_polarization(plane, CORR)
    ref = OR.prepare(uvw, obs.lambda_scale, data, flag, weight, spectrum if spec else None,
                     gridable, corr0, corr1, transform, factor)
    pol = cc.Polarization.for_plane(plane, CORR)
    rr = cc.RowRuns(uvw, obs.lambda_scale, data, flag, weight, spectrum if spec else None,
                    gridable)
    for device in (False, True):
        if device:
            import torch
            t = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()
            rr_d = cc.RowRuns(t(uvw), obs.lambda_scale, t(data), t(flag), t(weight),
                              t(spectrum) if spec else None, t(gridable))
            b, du, dv = cc.prepare_row_runs(ctx, rr_d, pol)
            get = lambda a: a.cpu().numpy()
        else:
            b, du, dv = cc.prepare_row_runs(ctx, rr, pol)
            get = np.asarray
        assert len(b) == len(ref["u"]) > 0
        for got, key in ((b.u_lambda, "u"), (b.v_lambda, "v"), (b.w_lambda, "w"),
                         (b.weight, "weight"), (b.sumwt_factor, "sumwt_factor"),
                         (b.gridable, "gridable"), (b.visibility, "vis"), (du, "du"),
                         (dv, "dv")):
            np.testing.assert_array_equal(get(got), ref[key], err_msg=key)


@pytest.mark.parametrize("mode,robust,unit", [("uniform", 0.0, True), ("briggs", 0.5, True),
                                              ("uniform", 0.0, False), ("briggs", 0.5, False)])
def test_row_weighting_and_dirty_image_match_oracle(ctx, runs, mode, robust, unit):
    obs, uvw, data, flag, weight, spectrum, gridable = runs
    if unit:
        weight = np.ones_like(weight)
    corr0, corr1, transform, factor = OR.plane_polarization("I", CORR)
    ref = OR.prepare(uvw, obs.lambda_scale, data, flag, weight, None, gridable, corr0, corr1,
                     transform, factor)
    geom = O.Geometry(obs.nx, obs.nx, obs.cell, obs.cell)
    wo, _, f2o = O.apply_weighting(geom, ref["u"], ref["v"], ref["weight"], mode, robust,
                                   build_u=ref["du"], build_v=ref["dv"])
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), 128)
    b, du, dv = cc.prepare_row_runs(ctx, cc.RowRuns(uvw, obs.lambda_scale, data, flag, weight,
                                                    None, gridable),
                                    cc.Polarization.for_plane("I", CORR))
    w, f2 = cc.apply_weighting_rows(gg, b, du, dv, mode, robust)
    if unit:
        np.testing.assert_array_equal(w, wo)
        assert f2 == f2o
    else:
        np.testing.assert_allclose(w, wo, rtol=1e-5)
        assert f2 == pytest.approx(f2o, rel=1e-6)
    wb = cc.VisibilityBatch(b.u_lambda, b.v_lambda, b.visibility, w, None, b.sumwt_factor,
                            b.gridable)
    psf, res, state, sums = cc.dirty_image(gg, wb)
    og = O.StdGridder(geom, 128)
    p, d, acc = og.grid_dirty(ref["u"], ref["v"], wo, ref["vis"], ref["sumwt_factor"],
                              ref["gridable"], threads=8)
    psf_o, res_o, _ = og.dirty_products(p, d, acc)
    assert sums.gridded_samples == acc.gridded
    assert peak_norm_err(psf, psf_o) <= 1e-5
    assert peak_norm_err(res, res_o) <= 1e-5
