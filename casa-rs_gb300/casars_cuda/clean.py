"""Cotton-Schwab major/minor cycle with every image and grid on the device.

Restates run_hogbom_cotton_schwab (lib.rs:59354-59636): per major cycle the
peak of the residual sets the cycle threshold (clean_cycle_threshold,
lib.rs:74120-74127), a Hogbom minor cycle runs on the device (cr_hogbom),
the divergence guard stops the loop when the residual peak grows by more
than 10 % over its minimum (update_divergence_state, lib.rs:74690-74712),
and the residual is refreshed from the model through one materialised plan:
apodise + forward FFT, degrid, residual gridding, inverse FFT, correction
and the PSF normalisation (the residual refresh of compute_residual,
lib.rs:68560-68620 / 70592-70644).  The robust-RMS n-sigma threshold of the
reference is not restated; thresholds are absolute (Jy/beam).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import imaging as im

try:
    import torch
except Exception:  # pragma: no cover
    torch = None


@dataclass
class CleanConfig:
    """The CleanConfig fields the loop uses (types.rs:2165-2210)."""
    niter: int
    gain: float = 0.1
    threshold_jy_per_beam: float = 0.0
    minor_cycle_length: int = 2000
    cyclefactor: float = 1.0
    min_psf_fraction: float = 0.05
    max_psf_fraction: float = 0.8
    major_cycle_limit: Optional[int] = None
    inclusive: bool = True
    psf_cutoff: float = 0.35


@dataclass
class CleanResult:
    model: object
    residual: object
    psf: object
    psf_state: im.PsfState
    major_cycles: int
    minor_iterations: int
    reported_iterations: int
    stop_reason: Optional[str]
    components: list = field(default_factory=list)
    cycle_thresholds: list = field(default_factory=list)
    beam: Optional[im.BeamFit] = None
    restored: object = None
    max_psf_sidelobe: float = 0.0


def clean_cycle_threshold(peak: float, max_psf_sidelobe: float, cfg: CleanConfig) -> float:
    """clean_cycle_threshold (lib.rs:74120-74127), float32 arithmetic."""
    f32 = np.float32
    frac = f32(max_psf_sidelobe) * f32(cfg.cyclefactor)
    frac = min(max(frac, f32(cfg.min_psf_fraction)), f32(cfg.max_psf_fraction))
    return float(max(f32(peak) * f32(frac), f32(cfg.threshold_jy_per_beam)))


def threshold_reached_with_tolerance(peak_abs: float, threshold: float) -> bool:
    """threshold_reached_with_tolerance (lib.rs:74628-74635), float32."""
    f32 = np.float32
    p, t = f32(peak_abs), f32(threshold)
    if t <= 0:
        return bool(p <= t)
    tol = max(f32(0.01) * t, f32(2.0e-8))
    return bool(p <= t or abs(p - t) <= tol)


def tolerant_clean_stop_reason(peak_abs: float, threshold: float,
                               nsigma_threshold: float = 0.0) -> Optional[str]:
    """tolerant_clean_stop_reason (lib.rs:74637-74651)."""
    if threshold_reached_with_tolerance(peak_abs, threshold):
        return "GlobalThresholdReached"
    if nsigma_threshold > threshold and threshold_reached_with_tolerance(peak_abs,
                                                                         nsigma_threshold):
        return "NsigmaThresholdReached"
    return None


_HANDOFF = ("CycleThresholdReached", "NsigmaThresholdReached")


def psf_beam_and_sidelobe(ctx, psf, cell_rad, cutoff: float = 0.35):
    """The fitted beam and estimate_psf_sidelobe_level (beam.rs:292-304):
    max(|min psf|, |max(psf - fitted Gaussian)|), 0 when no beam fits."""
    beam, _, _ = im.fit_beam(psf, cell_rad, cutoff, ctx=ctx)
    if beam is None:
        return None, 0.0
    return beam, im.psf_sidelobe(ctx, psf, cell_rad, beam)


def _absmax(a) -> float:
    if torch is not None and isinstance(a, torch.Tensor):
        return float(torch.max(torch.abs(a)))
    return float(np.max(np.abs(a)))


def _zeros_like(a):
    if torch is not None and isinstance(a, torch.Tensor):
        return torch.zeros_like(a)
    return np.zeros_like(a)


def run_cotton_schwab(gridder, batch, cfg: CleanConfig, wproj=None,
                      max_psf_sidelobe: Optional[float] = None) -> CleanResult:
    """run_hogbom_cotton_schwab (lib.rs:59354-59636) with the minor cycle on
    the device (cr_hogbom) and the residual refresh through one materialised
    plan (cr_plan_residual_image).  Images stay where the batch is: torch
    CUDA tensors for a device batch, numpy arrays for a host batch."""
    psf, residual, state, _ = im.dirty_image(gridder, batch, wproj)
    plan = im.Plan(gridder, batch, wproj)
    geom = gridder.geometry
    cell = (geom.cell_x_rad, geom.cell_y_rad)
    beam, fitted_sidelobe = psf_beam_and_sidelobe(gridder.ctx, psf, cell, cfg.psf_cutoff)
    sidelobe = fitted_sidelobe if max_psf_sidelobe is None else max_psf_sidelobe
    model = _zeros_like(residual)
    ctx = gridder.ctx
    actual = reported = major = 0
    stop = None
    min_peak = np.float32(_absmax(residual))
    needs_refresh = False
    comps, thresholds = [], []
    try:
        while reported < cfg.niter:
            if cfg.major_cycle_limit is not None and major >= cfg.major_cycle_limit:
                stop = "MajorCycleLimitReached"
                break
            peak = _absmax(residual)
            s = tolerant_clean_stop_reason(peak, cfg.threshold_jy_per_beam)
            if s is not None:
                stop = s
                break
            cycle_niter = min(cfg.niter - reported, cfg.minor_cycle_length)
            thr = clean_cycle_threshold(peak, sidelobe, cfg)
            thresholds.append(thr)
            out = im.run_hogbom_minor_cycle(ctx, model, residual, psf, cfg.gain, cycle_niter,
                                            threshold=cfg.threshold_jy_per_beam,
                                            cycle_threshold=thr, inclusive=cfg.inclusive)
            model, residual = out.model, out.residual
            comps.extend(zip(map(tuple, out.positions.tolist()), out.fluxes.tolist()))
            actual += out.actual_updates
            reported += out.reported_updates
            updated = out.actual_updates > 0
            stop_after = None
            if out.stop_reason is not None:
                if updated and out.stop_reason in _HANDOFF:
                    pass
                elif out.stop_reason in _HANDOFF:
                    stop = out.stop_reason
                else:
                    stop = stop_after = out.stop_reason
            if not updated:
                break
            needs_refresh = True
            minor_peak = np.float32(_absmax(residual))
            if minor_peak < min_peak:
                min_peak = minor_peak
            elif min_peak > 0 and (minor_peak - min_peak) / min_peak > np.float32(0.1):
                stop = "DivergenceDetected"
                break
            if reported >= cfg.niter:
                stop = "IterationLimitReached"
                break
            residual = plan.residual_image(model, state)
            major += 1
            needs_refresh = False
            if stop_after is not None:
                break
            s = tolerant_clean_stop_reason(_absmax(residual), cfg.threshold_jy_per_beam)
            if s is not None:
                stop = s
                break
        if cfg.niter > 0 and stop is None:
            stop = "IterationLimitReached"
        if needs_refresh:
            residual = plan.residual_image(model, state)
    finally:
        plan.close()
    restored = im.restore(gridder.ctx, model, residual, cell, beam) if beam is not None else None
    return CleanResult(model, residual, psf, state, major, actual, reported, stop, comps,
                       thresholds, beam, restored, sidelobe)
