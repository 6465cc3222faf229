"""Restoration and the PSF sidelobe level on the device against the oracle
(FP64 centred FFT convolution, make_casa_gaussian_psf_image), with the
reference's unit tests of beam.rs: restoration_spreads_delta_component
(1186-1202), restoration_uses_casa_style_circular_fft_boundary (1204-1222),
restoration_skips_fft_for_empty_model (1224-1237)."""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import beam as OB

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu
CELL = (1.0e-4, 1.0e-4)
BEAM = cc.BeamFit(4.0e-4, 3.0e-4, 0.0)


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def test_restoration_spreads_delta_component(ctx):
    m = np.zeros((16, 16), np.float32)
    m[8, 8] = 1.0
    r = cc.restore(ctx, m, None, CELL, BEAM)
    assert r[8, 8] > r[8, 9] and r[8, 8] <= 1.0 and r[8, 9] > 0.0


def test_restoration_uses_circular_boundary(ctx):
    m = np.zeros((16, 16), np.float32)
    m[0, 8] = 1.0
    r = cc.restore(ctx, m, None, CELL, BEAM)
    assert r[0, 8] > 0.0 and r[15, 8] > 0.0


def test_restoration_skips_empty_model(ctx):
    m = np.zeros((16, 16), np.float32)
    r = cc.restore(ctx, m, None, CELL, cc.BeamFit(10.0, 10.0, 0.0))
    np.testing.assert_array_equal(r, m)


@pytest.mark.parametrize("shape", [(256, 256), (192, 320)])
def test_restore_matches_oracle(ctx, shape):
    rng = np.random.default_rng(2)
    model = np.zeros(shape, np.float32)
    idx = rng.integers(0, shape[0], 40), rng.integers(0, shape[1], 40)
    model[idx] = rng.uniform(0.01, 1.0, 40).astype(np.float32)
    residual = rng.normal(0, 0.01, shape).astype(np.float32)
    beam = cc.BeamFit(5e-4, 2.5e-4, 0.7)
    ob = OB.Beam(beam.major_fwhm_rad, beam.minor_fwhm_rad, beam.position_angle_rad)
    got = cc.restore(ctx, model, residual, CELL, beam)
    ref = OB.restore(model, residual, CELL, ob)
    assert peak_norm_err(got, ref) <= 1e-5
    import torch
    gd = cc.restore(ctx, torch.as_tensor(model).cuda(), torch.as_tensor(residual).cuda(), CELL,
                    beam)
    np.testing.assert_array_equal(gd.cpu().numpy(), got)


def test_sidelobe_matches_oracle_and_fit_from_device(ctx):
    import torch
    psf = OB.synthetic_gaussian_psf((128, 128), CELL, OB.Beam(5e-4, 3e-4, 0.35))
    psf[10, 20] = -0.07                       # a negative sidelobe
    psf[100, 90] = 0.12                       # and a positive one
    b, _, _ = cc.fit_beam(psf, CELL, 0.35)
    bd, _, _ = cc.fit_beam(torch.as_tensor(psf).cuda(), CELL, 0.35, ctx=ctx)
    assert b == bd
    ob = OB.Beam(b.major_fwhm_rad, b.minor_fwhm_rad, b.position_angle_rad)
    lvl = cc.psf_sidelobe(ctx, psf, CELL, b)
    ref = OB.sidelobe(psf, CELL, ob)
    assert abs(lvl - ref) <= 1e-6 * max(ref, 1.0)
    assert ref >= 0.12 - 1e-3
