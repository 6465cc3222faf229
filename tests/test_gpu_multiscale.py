"""Multiscale CLEAN on the device against the oracle (oracle/multiscale.py).

The device state (scale images, PSF cross terms, residual convolved with
every scale) agrees with the oracle's within 1e-6 of each image's peak (both
convolve in FP64 and round to float32); the minor cycle picks the same
components -- positions and scale indices exactly, strengths and fluxes
within 1e-5 relative -- stops for the same reason, and leaves model and
convolved residual within 1e-5 of the peak.  The Cotton-Schwab controller
(run_multiscale_cotton_schwab) on a small observation with extended emission
matches the oracle's loop: cycles, thresholds, components, stop reason.
"""
import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import multiscale as M
from oracle import oracle as O

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def _scene(n, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(n)[:, None] - n // 2
    y = np.arange(n)[None, :] - n // 2
    r2 = (x * x + y * y).astype(np.float64)
    psf = (np.exp(-r2 / 6.0) + 0.05 * np.cos(0.9 * x) * np.exp(-r2 / 400.0)).astype(np.float32)
    psf[n // 2, n // 2] = 1.0
    sky = np.zeros((n, n), np.float32)
    sky += 40.0 * M.make_multiscale_kernel((n, n), 6.0)
    sky = np.roll(np.roll(sky, 9, 0), -7, 1)
    sky[n // 4, n // 3] += 0.8
    sky[3 * n // 5, n // 2 + 5] += 0.5
    res = M.fft_convolve_real(psf, sky) + (0.002 * rng.normal(size=(n, n))).astype(np.float32)
    return res.astype(np.float32), psf


def _compare_cycle(out, comps, model, ref_model, res_g, ref_res, stop):
    assert out.actual_updates == len(comps) > 0
    assert out.stop_reason == stop
    np.testing.assert_array_equal(out.positions, np.array([c[0] for c in comps]))
    np.testing.assert_array_equal(out.scales, [c[1] for c in comps])
    st = np.array([c[2] for c in comps])
    fl = np.array([c[3] for c in comps])
    assert float(np.max(np.abs(out.strengths - st) / np.abs(st))) <= 1e-5
    assert float(np.max(np.abs(out.fluxes - fl) / np.abs(fl))) <= 1e-5
    assert peak_norm_err(model, ref_model) <= 1e-5
    assert peak_norm_err(res_g, ref_res) <= 1e-5


@pytest.mark.parametrize("scales,bias,device", [([0.0, 3.0, 6.0], 0.2, False),
                                                ([0.0, 3.0, 6.0], 0.3, False),
                                                ([0.0, 2.0, 5.0, 9.0], 0.0, True),
                                                ([], 0.0, False)])
def test_minor_cycle_matches_oracle(ctx, scales, bias, device):
    n = 96
    res, psf = _scene(n, 1)
    ref = M.MultiscaleState(res, psf, scales, bias)
    if device:
        import torch
        T = lambda a: torch.as_tensor(a).cuda().contiguous()
        ms = cc.Multiscale(ctx, T(psf), scales, bias)
        ms.set_residual(T(res))
        model = torch.zeros((n, n), dtype=torch.float32, device="cuda")
    else:
        ms = cc.Multiscale(ctx, psf, scales, bias)
        ms.set_residual(res)
        model = np.zeros((n, n), np.float32)
    g0 = ms.residual()
    g0 = g0.cpu().numpy() if device else g0
    assert peak_norm_err(g0, ref.dirty[0]) <= 1e-6
    has, peak = ms.peak()
    assert has and abs(peak - float(np.max(np.abs(ref.dirty[0])))) <= 1e-6 * peak
    ref_model = np.zeros((n, n), np.float32)
    comps, stop = M.minor_cycle(ref, ref_model, 0.1, 150, threshold=0.0, cycle_threshold=0.02)
    out = ms.minor_cycle(model, 0.1, 150, threshold=0.0, cycle_threshold=0.02)
    m = model.cpu().numpy() if device else model
    r = ms.residual()
    r = r.cpu().numpy() if device else r
    _compare_cycle(out, comps, m, ref_model, r, ref.dirty[0], stop)
    if bias == 0.3:
        assert stop == "DivergenceDetected"          # this scene diverges after two updates
    elif len(scales) > 1:
        assert len(set(out.scales.tolist())) > 1     # more than one scale was used
    ms.close()


def test_clean_mask_and_divergence_rules(ctx):
    """A clean mask restricts every scale to its scale mask (the mask
    convolved with the scale, above 0.9, less a border of 1.5 scales)."""
    n = 80
    res, psf = _scene(n, 2)
    mask = np.zeros((n, n), bool)
    mask[10:70, 12:72] = True
    scales = [0.0, 4.0]
    ref = M.MultiscaleState(res, psf, scales, 0.3, mask)
    ms = cc.Multiscale(ctx, psf, scales, 0.3, mask.astype(np.uint8))
    ms.set_residual(res)
    model = np.zeros((n, n), np.float32)
    ref_model = np.zeros((n, n), np.float32)
    comps, stop = M.minor_cycle(ref, ref_model, 0.2, 80)
    out = ms.minor_cycle(model, 0.2, 80)
    _compare_cycle(out, comps, model, ref_model, ms.residual(), ref.dirty[0], stop)
    for (x, y), k in zip(out.positions, out.scales):
        assert ref.scale_masks[k][x, y]


def test_multiscale_cotton_schwab_matches_oracle(ctx):
    nx = 128
    obs = S.observation(1000.0, 1.0, 30.0, 1.4e9, nx, 6, 0.1, 1.0, 31, "ms")
    rng = np.random.default_rng(31)
    sky = S.gaussian_model(rng, 4, nx, nx, 2.0, 6.0, fwhm_min=4.0, fwhm_max=10.0)
    sky += S.model_image(obs.sky, nx, nx)
    og = O.StdGridder(O.Geometry(nx, nx, obs.cell, obs.cell), 128)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, obs.cell, obs.cell), 128)
    # visibilities of the extended sky: the oracle's FP64 degridding of its model grid
    wt = np.ones(obs.rows, np.float32)
    vis = og.degrid(og.model_grid(sky.astype(np.float64)), obs.u, obs.v).astype(np.complex64)
    p, d, acc = og.grid_dirty(obs.u, obs.v, wt, vis, threads=8)
    psf_o, res_o, peak_o = og.dirty_products(p, d, acc)

    def refresh(model):
        rg, _, _ = og.residual(og.model_grid(model.astype(np.float64)), obs.u, obs.v, wt, vis,
                               threads=8)
        return og.corrected_image(O.centered_ifft2(rg)) / acc.normalization_sumwt / peak_o

    kw = dict(niter=300, gain=0.2, minor_cycle_length=60)
    scales = [0.0, 3.0, 6.0]
    ref = M.cotton_schwab(res_o, psf_o, refresh, scales=scales, small_scale_bias=0.5,
                          sidelobe=0.2, **kw)
    out = cc.run_multiscale_cotton_schwab(gg, cc.VisibilityBatch(obs.u, obs.v, vis, wt),
                                          cc.CleanConfig(**kw), scales, 0.5,
                                          max_psf_sidelobe=0.2)
    assert ref["major_cycles"] >= 2
    assert out.stop_reason == ref["stop_reason"]
    assert out.major_cycles == ref["major_cycles"]
    assert out.minor_iterations == ref["actual"]
    np.testing.assert_allclose(out.cycle_thresholds, ref["thresholds"], rtol=1e-5)
    assert [c[0] for c in out.components] == [tuple(c[0]) for c in ref["components"]]
    assert out.component_scales == [c[1] for c in ref["components"]]
    assert len(set(out.component_scales)) > 1
    err = float(np.max(np.abs(out.residual - ref["residual"])))
    assert err <= 1e-5 * float(np.max(np.abs(res_o)))
    assert peak_norm_err(out.model, ref["model"]) <= 1e-5
