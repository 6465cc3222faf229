"""Cotton-Schwab controller logic on the CPU: the reference's own unit tests
of the threshold helpers (lib.rs:95191-95201, 95239-95256, 96558-96574), the
product's host-side restatement against the oracle's, and the oracle loop's
behaviour (cyclefactor raises the major-cycle count as in lib.rs:94884-94963;
the divergence guard of lib.rs:74690-74712)."""
import math

import numpy as np
import pytest

from casars_cuda import clean as PC
from casars_cuda import synthetic as S
from oracle import oracle as O


def test_clean_cycle_threshold_uses_psf_fraction_only():
    # lib.rs:96558-96574: peak 10, sidelobe 0.02, threshold 0.5 -> 0.5
    assert O.clean_cycle_threshold(10.0, 0.02, 1.0, 0.05, 0.8, 0.5) == 0.5
    cfg = PC.CleanConfig(niter=10, gain=0.1, threshold_jy_per_beam=0.5, minor_cycle_length=5)
    assert PC.clean_cycle_threshold(10.0, 0.02, cfg) == 0.5


@pytest.mark.parametrize("peak,sidelobe,cf,lo,hi,thr", [
    (3.0, 0.3, 1.0, 0.05, 0.8, 0.0), (1.7, 0.9, 2.0, 0.1, 0.8, 0.01),
    (0.2, 0.01, 1.0, 0.05, 0.8, 0.0), (5.5, 0.25, 1.5, 0.05, 0.3, 0.4)])
def test_cycle_threshold_product_matches_oracle(peak, sidelobe, cf, lo, hi, thr):
    cfg = PC.CleanConfig(niter=1, threshold_jy_per_beam=thr, cyclefactor=cf,
                         min_psf_fraction=lo, max_psf_fraction=hi)
    assert PC.clean_cycle_threshold(peak, sidelobe, cfg) == \
        O.clean_cycle_threshold(peak, sidelobe, cf, lo, hi, thr)


def test_tolerant_clean_stop_reason_prefers_absolute_threshold():
    # lib.rs:95191-95201
    for f in (PC.tolerant_clean_stop_reason, O.tolerant_clean_stop_reason):
        assert f(0.995, 1.0, 2.0) == "GlobalThresholdReached"
        assert f(1.5, 1.0, 2.0) == "NsigmaThresholdReached"
        assert f(2.5, 1.0, 2.0) is None
        assert f(0.0, 0.0, 0.0) == "GlobalThresholdReached"
        assert f(1e-3, 0.0, 0.0) is None


def _std_problem(seed=5, nx=128, dump_s=60.0, sources=6):
    obs = S.observation(1000.0, 1.0, dump_s, 1.4e9, nx, sources, 0.1, 1.0, seed, "t")
    rng = np.random.default_rng(seed)
    vis = S.visibilities(obs.u, obs.v, np.zeros_like(obs.w), obs.sky, nx, nx, obs.cell, 0.0,
                         rng, w_term=False)
    og = O.StdGridder(O.Geometry(nx, nx, obs.cell, obs.cell), 128)
    wt = np.ones(obs.rows, np.float32)
    p, d, acc = og.grid_dirty(obs.u, obs.v, wt, vis, threads=4)
    psf, res, peak = og.dirty_products(p, d, acc)
    sumwt = acc.normalization_sumwt

    def refresh(model):
        rg, _, _ = og.residual(og.model_grid(model.astype(np.float64)), obs.u, obs.v, wt, vis,
                               threads=4)
        return og.corrected_image(O.centered_ifft2(rg)) / sumwt / peak

    return psf.astype(np.float32), res.astype(np.float32), refresh


def test_oracle_loop_higher_cyclefactor_more_major_cycles():
    psf, res, refresh = _std_problem()
    sl = 0.3
    relaxed = O.cotton_schwab(res, psf, refresh, niter=12, gain=0.2, minor_cycle_length=12,
                              cyclefactor=0.5, min_psf_fraction=0.01, max_psf_fraction=0.4,
                              sidelobe=sl)
    strict = O.cotton_schwab(res, psf, refresh, niter=12, gain=0.2, minor_cycle_length=12,
                             cyclefactor=3.0, min_psf_fraction=0.4, max_psf_fraction=0.9,
                             sidelobe=sl)
    assert strict["major_cycles"] > relaxed["major_cycles"]
    assert strict["reported"] == relaxed["reported"] == 12


def test_oracle_loop_reduces_residual_and_stops_on_threshold():
    psf, res, refresh = _std_problem()
    peak0 = float(np.max(np.abs(res)))
    out = O.cotton_schwab(res, psf, refresh, niter=2000, gain=0.1, threshold=0.05 * peak0,
                          minor_cycle_length=60, sidelobe=0.2)
    assert out["stop_reason"] == "GlobalThresholdReached"
    assert float(np.max(np.abs(out["residual"]))) <= 0.05 * peak0 * 1.01 + 2e-8
    assert out["major_cycles"] >= 2


def test_oracle_loop_divergence_guard():
    psf, res, _ = _std_problem()
    # a refresh that returns a residual 20 % above the minor cycle's peak
    grow = lambda model: 1.5 * res
    out = O.cotton_schwab(res, psf, grow, niter=100, gain=0.1, minor_cycle_length=10,
                          sidelobe=0.2)
    assert out["stop_reason"] == "DivergenceDetected"
    assert out["major_cycles"] == 1


def test_oracle_loop_major_cycle_limit():
    psf, res, refresh = _std_problem()
    out = O.cotton_schwab(res, psf, refresh, niter=500, gain=0.1, minor_cycle_length=5,
                          sidelobe=0.2, major_cycle_limit=2)
    assert out["stop_reason"] == "MajorCycleLimitReached"
    assert out["major_cycles"] == 2
