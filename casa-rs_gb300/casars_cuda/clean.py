"""Cotton-Schwab major/minor cycle with every image and grid on the device.

Restates run_hogbom_cotton_schwab (lib.rs:59354-59636): per major cycle the
peak of the residual sets the cycle threshold (clean_cycle_threshold,
lib.rs:74120-74127), a Hogbom minor cycle runs on the device (cr_hogbom),
the divergence guard stops the loop when the residual peak grows by more
than 10 % over its minimum (update_divergence_state, lib.rs:74690-74712),
and the residual is refreshed from the model through one materialised plan:
apodise + forward FFT, degrid, residual gridding, inverse FFT, correction
and the PSF normalisation (the residual refresh of compute_residual,
lib.rs:68560-68620 / 70592-70644).  With CleanConfig.nsigma > 0 the n-sigma
threshold (nsigma times the robust RMS of the residual, computed on the
device by cr_robust_rms) joins the stop rules at each cycle start and after
each refresh, and the minor cycle stops at it, as in the reference
(lib.rs:59395-59396, 59563-59564).
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
    nsigma: float = 0.0
    minor_cycle_length: int = 2000
    cyclefactor: float = 1.0
    min_psf_fraction: float = 0.05
    max_psf_fraction: float = 0.8
    major_cycle_limit: Optional[int] = None
    inclusive: bool = True
    psf_cutoff: float = 0.35


@dataclass
class HogbomPlaneMinorCycleControl:
    """HogbomPlaneMinorCycleControl (lib.rs:64555-64580)."""
    clean: CleanConfig
    cycle_limit: int
    cycle_threshold_jy_per_beam: float
    peak_relative_tolerance: float


@dataclass
class HogbomPlaneComponent:
    """HogbomPlaneComponent: position (x, y), peak residual, flux added."""
    position: tuple
    peak_value_jy_per_beam: float
    component_jy: float


@dataclass
class HogbomPlaneMinorCycleOutcome:
    model: object
    residual: object
    actual_updates: int
    reported_updates: int
    components: list


def run_hogbom_plane_minor_cycle(ctx, model, residual, psf, clean_mask,
                                 control: HogbomPlaneMinorCycleControl
                                 ) -> HogbomPlaneMinorCycleOutcome:
    """run_hogbom_plane_minor_cycle (lib.rs:64630-64680) on one image plane:
    gain, threshold and the CasaInclusive budget from control.clean, peaks
    with control.peak_relative_tolerance.  Returns updated copies of model
    and residual."""
    c = control.clean
    out = im.hogbom_plane_minor_cycle(ctx, model, residual, psf, c.gain, control.cycle_limit,
                                      control.cycle_threshold_jy_per_beam,
                                      control.peak_relative_tolerance,
                                      threshold=c.threshold_jy_per_beam, mask=clean_mask,
                                      inclusive=c.inclusive)
    comps = [HogbomPlaneComponent((int(p[0]), int(p[1])), float(pk), float(fl))
             for p, pk, fl in zip(out.positions, out.peaks, out.fluxes)]
    return HogbomPlaneMinorCycleOutcome(out.model, out.residual, out.actual_updates,
                                        out.reported_updates, comps)


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
    nsigma_thresholds: list = field(default_factory=list)


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
    comps, thresholds, nsigs = [], [], []
    try:
        while reported < cfg.niter:
            if cfg.major_cycle_limit is not None and major >= cfg.major_cycle_limit:
                stop = "MajorCycleLimitReached"
                break
            peak = _absmax(residual)
            nsig = im.nsigma_threshold(ctx, residual, cfg.nsigma)
            nsigs.append(nsig)
            s = tolerant_clean_stop_reason(peak, cfg.threshold_jy_per_beam, nsig)
            if s is not None:
                stop = s
                break
            cycle_niter = min(cfg.niter - reported, cfg.minor_cycle_length)
            thr = clean_cycle_threshold(peak, sidelobe, cfg)
            thresholds.append(thr)
            out = im.run_hogbom_minor_cycle(ctx, model, residual, psf, cfg.gain, cycle_niter,
                                            threshold=cfg.threshold_jy_per_beam,
                                            cycle_threshold=thr, nsigma_threshold=nsig,
                                            inclusive=cfg.inclusive)
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
            nsig = im.nsigma_threshold(ctx, residual, cfg.nsigma)
            if stop_after is not None:
                break
            s = tolerant_clean_stop_reason(_absmax(residual), cfg.threshold_jy_per_beam, nsig)
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
                       thresholds, beam, restored, sidelobe, nsigs)


def run_multiscale_cotton_schwab(gridder, batch, cfg: CleanConfig, scales,
                                 small_scale_bias: float = 0.0, wproj=None,
                                 max_psf_sidelobe: Optional[float] = None,
                                 mask=None) -> CleanResult:
    """run_multiscale_cotton_schwab (lib.rs:63543-63963): the deconvolver
    state on the device (im.Multiscale: scale images, PSF cross terms,
    residual convolved with every scale), one multiscale minor cycle per
    major cycle on the device, the residual refreshed through one
    materialised plan and the convolved residuals rebuilt from it, with the
    reference's stop, n-sigma and divergence rules.  Components are
    ((x, y), flux) as for Hogbom, with result.component_scales the scale index
    of each."""
    psf, residual, state, _ = im.dirty_image(gridder, batch, wproj)
    plan = im.Plan(gridder, batch, wproj)
    geom = gridder.geometry
    cell = (geom.cell_x_rad, geom.cell_y_rad)
    beam, fitted_sidelobe = psf_beam_and_sidelobe(gridder.ctx, psf, cell, cfg.psf_cutoff)
    sidelobe = fitted_sidelobe if max_psf_sidelobe is None else max_psf_sidelobe
    ctx = gridder.ctx
    ms = im.Multiscale(ctx, psf, scales, small_scale_bias, mask)
    ms.set_residual(residual)
    model = _zeros_like(residual)
    actual = reported = major = 0
    stop = None
    min_peak = np.float32(_absmax(residual))
    needs_refresh = False
    comps, comp_scales, thresholds, nsigs = [], [], [], []
    try:
        while reported < cfg.niter:
            if cfg.major_cycle_limit is not None and major >= cfg.major_cycle_limit:
                stop = "MajorCycleLimitReached"
                break
            has, peak = ms.peak()
            if not has:
                stop = "NoCleanablePixels"
                break
            nsig = im.nsigma_threshold(ctx, residual, cfg.nsigma, mask)
            nsigs.append(nsig)
            s = tolerant_clean_stop_reason(peak, cfg.threshold_jy_per_beam, nsig)
            if s is not None:
                stop = s
                break
            cycle_niter = min(cfg.niter - reported, cfg.minor_cycle_length)
            thr = clean_cycle_threshold(peak, sidelobe, cfg)
            thresholds.append(thr)
            out = ms.minor_cycle(model, cfg.gain, cycle_niter, cfg.threshold_jy_per_beam, thr,
                                 nsig)
            comps.extend(zip(map(tuple, out.positions.tolist()), out.fluxes.tolist()))
            comp_scales.extend(out.scales.tolist())
            actual += out.actual_updates
            reported += out.reported_updates
            if out.actual_updates == 0:
                stop = out.stop_reason
                break
            residual = ms.residual()
            needs_refresh = True
            minor_peak = np.float32(_absmax(residual))
            if minor_peak < min_peak:
                min_peak = minor_peak
            elif min_peak > 0 and (minor_peak - min_peak) / min_peak > np.float32(0.1):
                stop = "DivergenceDetected"
                break
            if stop is None and reported >= cfg.niter:
                stop = "IterationLimitReached"
                break
            residual = plan.residual_image(model, state)
            ms.set_residual(residual)
            major += 1
            needs_refresh = False
            nsig = im.nsigma_threshold(ctx, residual, cfg.nsigma, mask)
            s = tolerant_clean_stop_reason(_absmax(residual), cfg.threshold_jy_per_beam, nsig)
            if s is not None:
                stop = s
                break
        if cfg.niter > 0 and stop is None:
            stop = "IterationLimitReached"
        if needs_refresh:
            residual = plan.residual_image(model, state)
            major += 1
    finally:
        plan.close()
        ms.close()
    restored = im.restore(ctx, model, residual, cell, beam) if beam is not None else None
    res = CleanResult(model, residual, psf, state, major, actual, reported, stop, comps,
                      thresholds, beam, restored, sidelobe, nsigs)
    res.component_scales = comp_scales
    return res


# ----------------------------------------------------------------------------
# cube CLEAN
# ----------------------------------------------------------------------------
@dataclass
class CubeCleanResult:
    """StandardMfsCubeCleanResult (lib.rs:2995-3013) plus the plane images."""
    models: object
    residuals: object
    psfs: object
    states: list
    beams: list
    restored: object
    sidelobes: list
    initial_peak: float
    max_psf_sidelobe: float
    final_cycle_threshold: float
    minor_iterations: int
    major_cycles: int
    planes_at_or_below_initial_threshold: int
    plane_iterations: list
    plane_stop_reasons: list
    components: list
    cycle_thresholds: list
    active_planes: list


def _f32max(values) -> np.float32:
    """The finite maximum of values, 0 when none (fold with f32::max)."""
    m = np.float32(0.0)
    for v in values:
        v = np.float32(v)
        if np.isfinite(v) and v > m:
            m = v
    return m


def cube_clean_loop(residuals, psfs, models, sidelobes, cfg: CleanConfig, hogbom, refresh,
                    hogbom_many=None, nsigma_fn=None):
    """The control of run_standard_mfs_cube_clean (lib.rs:3026-3210).

    Planes advance in ascending order; per synchronized pass every plane whose
    residual peak is above the cube-wide cycle threshold (clean_cycle_threshold
    of the cube's peak and largest PSF sidelobe) runs one major cycle of its
    own Cotton-Schwab controller with the remaining global budget, one major
    cycle allowed and the cube threshold as override
    (run_standard_mfs_prepared_clean_plane_one_major_cycle, lib.rs:46465-46520).
    The residual refreshes of a pass are batched: a plane's refresh depends on
    its own model only, so refreshing every updated plane after the pass's
    minor cycles gives the same residuals as refreshing each in turn.

    residuals / models / psfs are indexable by plane (arrays [C][nx][ny]);
    hogbom(model, residual, psf, niter, threshold, cycle_threshold,
    nsigma_threshold) returns a HogbomOutcome-like object; refresh(planes)
    recomputes residuals[c] for the listed planes from models[c] in place.
    hogbom_many(planes, niter, threshold, cycle_threshold, nsigma_thresholds),
    when given, runs the listed planes' minor cycles together (in place;
    outcomes in list order) -- the planes are independent, so this equals
    running them in turn.  With cfg.nsigma > 0, nsigma_fn(planes) gives the
    listed planes' n-sigma thresholds from their current residuals; each
    plane's controller applies its own at its cycle start, in its minor
    cycle, after its refresh (lib.rs:59395-59396, 59563-59564) and in its
    final stop reason (lib.rs:46395-46409).  Returns a dict of the loop's
    results."""
    f32 = np.float32
    n = len(sidelobes)

    def nsigmas(planes):
        planes = list(planes)
        if not cfg.nsigma > 0.0 or not planes:
            return {c: 0.0 for c in planes}
        if nsigma_fn is None:
            raise ValueError("CleanConfig.nsigma > 0 needs nsigma_fn")
        return dict(zip(planes, (float(x) for x in nsigma_fn(planes))))

    def plane_peaks():
        # every plane's |residual| peak at once (one reduction, one copy)
        if torch is not None and isinstance(residuals, torch.Tensor):
            return residuals.abs().amax(dim=(1, 2)).float().cpu().numpy()
        if isinstance(residuals, np.ndarray):
            return np.abs(residuals).max(axis=(1, 2)).astype(np.float32)
        return np.array([_absmax(residuals[c]) for c in range(n)], np.float32)

    pk = plane_peaks()
    absmax = lambda c: f32(pk[c])
    cyc = lambda peak, sl: clean_cycle_threshold(float(peak), float(sl), cfg)
    initial_peak = _f32max(absmax(c) for c in range(n))
    max_sidelobe = _f32max(sidelobes)
    at_or_below = sum(1 for c in range(n) if absmax(c) <= f32(cyc(initial_peak, max_sidelobe)))
    plane_iters, plane_stop = [0] * n, [None] * n
    comps = [[] for _ in range(n)]
    completed = major = 0
    thresholds, actives = [], []
    t = f32(cfg.threshold_jy_per_beam)
    while True:
        peak = _f32max(absmax(c) for c in range(n))
        thr = cyc(peak, max_sidelobe)
        if peak <= t or (t > 0 and abs(peak - t) / t < f32(0.01)) or completed >= cfg.niter:
            break
        if cfg.major_cycle_limit is not None and major >= cfg.major_cycle_limit:
            break
        active = [c for c in range(n) if absmax(c) > f32(thr)]
        if not active:
            break
        major += 1
        cycle_niter = cfg.niter - completed
        thresholds.append(thr)
        actives.append(active)
        pass_iters = 0
        pending = {}   # plane -> (stop set before the refresh, stop_after, refreshed in loop)
        # the planes' controllers (run_hogbom_cotton_schwab, niter =
        # cycle_niter, major_cycle_limit = 1) up to their residual refresh
        todo, start_peak = [], {}
        nstart = nsigmas(active)
        for c in active:
            p = absmax(c)
            s = tolerant_clean_stop_reason(p, cfg.threshold_jy_per_beam, nstart[c])
            if s is not None:
                plane_stop[c] = s
                continue
            todo.append(c)
            start_peak[c] = p
        budget = min(cycle_niter, cfg.minor_cycle_length)
        if hogbom_many is not None:
            outs = hogbom_many(todo, budget, cfg.threshold_jy_per_beam, thr,
                               [nstart[c] for c in todo])
        else:
            outs = [hogbom(models[c], residuals[c], psfs[c], budget, cfg.threshold_jy_per_beam,
                           thr, nstart[c]) for c in todo]
        for c, out in zip(todo, outs):
            if out.model is not None:
                models[c], residuals[c] = out.model, out.residual
        pk = plane_peaks()
        for c, out in zip(todo, outs):
            stop = None
            min_peak = start_peak[c]
            comps[c].extend(zip(map(tuple, np.asarray(out.positions).tolist()),
                                np.asarray(out.fluxes).tolist()))
            plane_iters[c] += out.reported_updates
            pass_iters += out.reported_updates
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
                plane_stop[c] = stop if stop is not None else "IterationLimitReached"
                continue
            minor_peak = absmax(c)
            if not minor_peak < min_peak and min_peak > 0 and \
                    (minor_peak - min_peak) / min_peak > f32(0.1):
                pending[c] = ("DivergenceDetected", None, False)
            elif out.reported_updates >= cycle_niter:
                pending[c] = ("IterationLimitReached", None, False)
            else:
                pending[c] = (stop, stop_after, True)
        nafter = {}
        if pending:
            refresh(sorted(pending))
            pk = plane_peaks()
            nafter = nsigmas(c for c in sorted(pending) if pending[c][2] and pending[c][1] is None)
        for c, (stop, stop_after, in_loop) in pending.items():
            if in_loop and stop_after is None:
                s = tolerant_clean_stop_reason(absmax(c), cfg.threshold_jy_per_beam, nafter[c])
                # otherwise the next turn of the plane's loop meets its
                # one-major-cycle limit
                stop = s if s is not None else "MajorCycleLimitReached"
            elif in_loop:
                stop = stop_after
            plane_stop[c] = stop
        completed += pass_iters
        if pass_iters == 0:
            break
    final_thr = cyc(_f32max(absmax(c) for c in range(n)), max_sidelobe)
    nfinal = nsigmas(c for c in range(n) if plane_iters[c] < cfg.niter)
    stops = []
    for c in range(n):
        if plane_iters[c] >= cfg.niter:
            stops.append("IterationLimitReached")
            continue
        s = tolerant_clean_stop_reason(absmax(c), cfg.threshold_jy_per_beam, nfinal[c])
        if s is None:
            s = plane_stop[c]
            if s in (None, "MajorCycleLimitReached"):
                s = "CycleThresholdReached"
        stops.append(s)
    return dict(plane_iterations=plane_iters, plane_stops=stops, components=comps,
                minor_iterations=completed, major_cycles=major, thresholds=thresholds,
                active=actives, initial_peak=float(initial_peak),
                max_sidelobe=float(max_sidelobe), final_cycle_threshold=final_thr,
                planes_at_or_below_initial_threshold=at_or_below)


def run_cube_clean(gridder, cube, cfg: CleanConfig, weighting: str = "natural",
                   robust: float = 0.0, max_psf_sidelobe: Optional[float] = None,
                   restore: bool = True, fft_bits: int = 32) -> CubeCleanResult:
    """run_standard_mfs_cube_clean (lib.rs:3026-3210) on the device: one
    persistent cube plan (im.CubePlan) gives every plane's PSF and residual
    and replays the records for each pass's residual refresh (all updated
    planes in one batched degrid + grid); the minor cycles are cr_hogbom per
    plane; each plane's beam is fitted to its PSF and its sidelobe level
    estimated (beam.rs:292-304) unless max_psf_sidelobe is given.  fft_bits
    picks the image-stage transforms (im.CubePlan.set_fft_precision)."""
    plan = im.CubePlan(gridder, cube, weighting, robust, fft_bits)
    ctx = gridder.ctx
    geom = gridder.geometry
    cell = (geom.cell_x_rad, geom.cell_y_rad)
    try:
        psfs, residuals, states = plan.dirty_images()
        n = plan.channels
        beams, sidelobes = [], []
        fit = restore or max_psf_sidelobe is None   # beams feed restoration and sidelobes
        for c in range(n):
            if fit and states[c].psf_peak > 0:
                b, sl = psf_beam_and_sidelobe(ctx, psfs[c], cell, cfg.psf_cutoff)
            else:
                b, sl = None, 0.0
            beams.append(b)
            sidelobes.append(sl if max_psf_sidelobe is None else max_psf_sidelobe)
        models = _zeros_like(residuals)

        def hogbom(model, residual, psf, niter, threshold, cycle_threshold, nsigma_threshold):
            return im.run_hogbom_minor_cycle(ctx, model, residual, psf, cfg.gain, niter,
                                             threshold=threshold,
                                             cycle_threshold=cycle_threshold,
                                             nsigma_threshold=nsigma_threshold,
                                             inclusive=cfg.inclusive)

        def nsigma_fn(planes):
            # the listed planes' robust RMS in one batched call
            rms, _, _ = im.robust_rms(ctx, residuals, None, planes)
            return [float(np.float32(cfg.nsigma) * np.float32(r)) for r in rms]

        def refresh(planes):
            mask = np.zeros(n, np.uint8)
            mask[planes] = 1
            plan.residual_images(models, states, planes=mask, out=residuals)

        hogbom_many = None
        if torch is not None and isinstance(residuals, torch.Tensor) and residuals.is_cuda:
            def hogbom_many(planes, niter, threshold, cycle_threshold, nsigma_thresholds):
                return im.run_hogbom_planes(ctx, models, residuals, psfs, planes, cfg.gain,
                                            niter, threshold=threshold,
                                            cycle_threshold=cycle_threshold,
                                            nsigma_threshold=nsigma_thresholds,
                                            inclusive=cfg.inclusive)

        out = cube_clean_loop(residuals, psfs, models, sidelobes, cfg, hogbom, refresh,
                              hogbom_many, nsigma_fn)
    finally:
        plan.close()
    restored = None
    if restore:
        restored = _zeros_like(residuals)
        for c in range(n):
            if beams[c] is not None and _absmax(models[c]) > 0:
                restored[c] = im.restore(ctx, models[c], residuals[c], cell, beams[c])
            else:
                restored[c] = residuals[c]
    return CubeCleanResult(models, residuals, psfs, states, beams, restored, sidelobes,
                           out["initial_peak"], out["max_sidelobe"],
                           out["final_cycle_threshold"], out["minor_iterations"],
                           out["major_cycles"], out["planes_at_or_below_initial_threshold"],
                           out["plane_iterations"], out["plane_stops"], out["components"],
                           out["thresholds"], out["active"])


# ----------------------------------------------------------------------------
# Clark
# ----------------------------------------------------------------------------
def clark_step_niter(cycle_reported_niter: int) -> int:
    """casa_clark_step_niter (lib.rs:63168-63174)."""
    return cycle_reported_niter if cycle_reported_niter < 5000 else 2000


def run_clark_cotton_schwab(gridder, batch, cfg: CleanConfig, wproj=None,
                            max_psf_sidelobe: Optional[float] = None) -> CleanResult:
    """run_clark_cotton_schwab (lib.rs:63314-63520): per major cycle a Clark
    minor cycle on the device (cr_clark; PSF patch from the fitted beam),
    the residual refreshed whenever the model changed, CASA's stop and
    hand-off rules and divergence guard.  Images stay where the batch is."""
    psf, residual, state, _ = im.dirty_image(gridder, batch, wproj)
    plan = im.Plan(gridder, batch, wproj)
    geom = gridder.geometry
    cell = (geom.cell_x_rad, geom.cell_y_rad)
    beam, fitted_sidelobe = psf_beam_and_sidelobe(gridder.ctx, psf, cell, cfg.psf_cutoff)
    sidelobe = fitted_sidelobe if max_psf_sidelobe is None else max_psf_sidelobe
    ncent = im.clark_ncent(beam, cell)
    model = _zeros_like(residual)
    ctx = gridder.ctx
    actual = reported = major = 0
    stop = None
    min_peak = np.float32(_absmax(residual))
    comps, thresholds, nsigs = [], [], []
    try:
        while reported < cfg.niter:
            if cfg.major_cycle_limit is not None and major >= cfg.major_cycle_limit:
                stop = "MajorCycleLimitReached"
                break
            peak = _absmax(residual)
            nsig = im.nsigma_threshold(ctx, residual, cfg.nsigma)
            nsigs.append(nsig)
            s = tolerant_clean_stop_reason(peak, cfg.threshold_jy_per_beam, nsig)
            if s is not None:
                stop = s
                break
            step = clark_step_niter(min(cfg.niter - reported, cfg.minor_cycle_length))
            thr = clean_cycle_threshold(peak, sidelobe, cfg)
            thresholds.append(thr)
            out = im.run_clark_minor_cycle(ctx, model, residual, psf, ncent, cfg.gain, step,
                                           threshold=cfg.threshold_jy_per_beam,
                                           cycle_threshold=thr, nsigma_threshold=nsig)
            model, residual = out.model, out.residual
            comps.extend(zip(map(tuple, out.positions.tolist()), out.fluxes.tolist()))
            updated = out.actual_updates > 0
            after = reported + out.reported_updates
            if updated:
                residual = plan.residual_image(model, state)
                if after < cfg.niter:
                    major += 1
            actual += out.actual_updates
            reported = after
            stop_after = False
            if out.stop_reason is not None:
                if updated and out.stop_reason in _HANDOFF:
                    pass
                elif out.stop_reason in _HANDOFF:
                    stop = out.stop_reason
                else:
                    stop = out.stop_reason
                    stop_after = True
            if not updated or stop_after:
                break
            minor_peak = np.float32(_absmax(residual))
            if minor_peak < min_peak:
                min_peak = minor_peak
            elif min_peak > 0 and (minor_peak - min_peak) / min_peak > np.float32(0.1):
                stop = "DivergenceDetected"
                break
            if stop is None and reported >= cfg.niter:
                stop = "IterationLimitReached"
                break
            nsig = im.nsigma_threshold(ctx, residual, cfg.nsigma)
            s = tolerant_clean_stop_reason(_absmax(residual), cfg.threshold_jy_per_beam, nsig)
            if s is not None:
                stop = s
                break
        if cfg.niter > 0 and stop is None:
            stop = "IterationLimitReached"
    finally:
        plan.close()
    restored = im.restore(gridder.ctx, model, residual, cell, beam) if beam is not None else None
    return CleanResult(model, residual, psf, state, major, actual, reported, stop, comps,
                       thresholds, beam, restored, sidelobe, nsigs)

