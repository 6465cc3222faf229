"""Restoring-beam fit (host code of the library) against the oracle and the
reference's own unit tests of beam.rs:
fitted_beam_tracks_elliptical_psf (1069-1082), fitted_beam_preserves_casa_
float_output_quantization (1084-1107), beam_fit_retries_lower_cutoffs
(1172-1184); the fit of a real dirty-image PSF agrees with the oracle's."""
import math

import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import beam as OB
from oracle import oracle as O

CELL = (1.0e-4, 1.0e-4)


def _same(b, o):
    assert o is not None and b is not None
    for a, c in ((b.major_fwhm_rad, o.major_fwhm_rad), (b.minor_fwhm_rad, o.minor_fwhm_rad),
                 (b.position_angle_rad, o.position_angle_rad)):
        assert abs(a - c) <= 1e-6 * max(abs(c), 1e-300)


def test_fitted_beam_tracks_elliptical_psf():
    exp = OB.Beam(5.0e-4, 3.0e-4, 0.35)
    psf = OB.synthetic_gaussian_psf((64, 64), CELL, exp)
    b, attempts, used = cc.fit_beam(psf, CELL, 0.35)
    assert abs(b.major_fwhm_rad - exp.major_fwhm_rad) < 7.5e-5
    assert abs(b.minor_fwhm_rad - exp.minor_fwhm_rad) < 7.5e-5
    assert abs(b.position_angle_rad - exp.position_angle_rad) < 0.15
    o, _, _ = OB.fit_beam(psf, CELL, 0.35)
    _same(b, o)


def test_fitted_beam_preserves_float_output_quantization():
    psf = OB.synthetic_gaussian_psf((64, 64), CELL, OB.Beam(5.0e-4, 3.0e-4, 0.35))
    b, _, _ = cc.fit_beam(psf, CELL, 0.35)
    r2d = 180.0 / math.pi
    r2as = 3600.0 * r2d
    for v, k in ((b.major_fwhm_rad, r2as), (b.minor_fwhm_rad, r2as), (b.position_angle_rad, r2d)):
        assert v == float(np.float32(v * k)) / k


def test_beam_fit_retries_lower_cutoffs():
    psf = OB.synthetic_gaussian_psf((64, 64), CELL, OB.Beam(4.0e-4, 2.5e-4, -0.2))
    b, attempts, used = cc.fit_beam(psf, CELL, 0.95)
    assert attempts > 1 and used < 0.95 and b is not None
    o, ao, uo = OB.fit_beam(psf, CELL, 0.95)
    assert (attempts, used) == (ao, uo)
    _same(b, o)


@pytest.mark.parametrize("beam", [OB.Beam(6e-4, 2e-4, 1.2), OB.Beam(3e-4, 2.9e-4, -1.0),
                                  OB.Beam(8e-4, 4e-4, 0.0)])
def test_fit_matches_oracle_across_shapes(beam):
    psf = OB.synthetic_gaussian_psf((96, 96), CELL, beam)
    b, a, u = cc.fit_beam(psf, CELL, 0.35)
    o, ao, uo = OB.fit_beam(psf, CELL, 0.35)
    assert (a, u) == (ao, uo)
    _same(b, o)


def test_dirty_psf_fit_matches_oracle():
    obs = S.observation(1000.0, 1.0, 60.0, 1.4e9, 128, 4, 0.1, 1.0, 21, "beam")
    og = O.StdGridder(O.Geometry(128, 128, obs.cell, obs.cell), 128)
    wt = np.ones(obs.rows, np.float32)
    p, d, acc = og.grid_dirty(obs.u, obs.v, wt, np.ones(obs.rows, np.complex64), threads=4)
    psf, _, _ = og.dirty_products(p, d, acc)
    psf = psf.astype(np.float32)
    cell = (obs.cell, obs.cell)
    b, a, u = cc.fit_beam(psf, cell, 0.35)
    o, ao, uo = OB.fit_beam(psf, cell, 0.35)
    assert (a, u) == (ao, uo)
    _same(b, o)


def test_empty_psf_is_not_fitted():
    b, a, u = cc.fit_beam(np.zeros((16, 16), np.float32), CELL, 0.35)
    assert b is None and a == 0
