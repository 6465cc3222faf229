"""The Clark minor cycle and its Cotton-Schwab controller: CPU restatement
(test infrastructure).

Restates with float32 arithmetic:
  * build_clark_psf_patch (casa-imaging lib.rs:64422-64456) from ncent,
    with max_abs_outside_patch;
  * run_clark_minor_cycle_cpu (lib.rs:62129-62355): subcycles over the active
    pixels (collect_clark_active_pixels, lib.rs:64467-64487, row-major),
    peak_clark_active_pixel (lib.rs:64489-64501: first strictly largest
    |value|), subtract_clark_component_from_active (lib.rs:64503-64539), at
    most CASA_CLARK_MAX_MAJOR_CYCLES = 10 subcycles, and the residual update
    by fft_convolve_real (lib.rs:64415-64420) -- here an FP64 circular
    convolution (numpy FFT) rounded to float32, where the reference uses
    float32 FFTs;
  * run_clark_cotton_schwab (lib.rs:63314-63520) without mask and n-sigma,
    with casa_clark_step_niter (lib.rs:63168-63174).
"""
import numpy as np

from . import oracle as O

f32 = np.float32
MAX_SUBCYCLES = 10


def psf_patch(psf, ncent: int):
    psf = np.asarray(psf, np.float32)
    nx, ny = psf.shape
    size = 3 * ncent + 1
    rx = ry = size // 2
    x0, y0 = max(0, nx // 2 - rx), max(0, ny // 2 - ry)
    x1, y1 = min(x0 + size, nx), min(y0 + size, ny)
    patch = psf[x0:x1, y0:y1].copy()
    outside = np.ones_like(psf, bool)
    outside[x0:x1, y0:y1] = False
    vals = np.abs(psf[outside])
    vals = vals[~np.isnan(vals)]
    mea = f32(vals.max()) if vals.size and vals.max() > 0 else f32(0.0)
    return dict(patch=patch, rx=rx, ry=ry, max_exterior_abs=mea)


def fft_convolve_real(psf, delta):
    """conv[x] = sum_p delta[p] psf[(x - p + floor(n/2)) mod n] (the centred
    transforms' circular convolution), FP64, rounded to float32."""
    nx, ny = psf.shape
    shifted = np.roll(np.roll(np.asarray(psf, np.float64), -(nx // 2), 0), -(ny // 2), 1)
    conv = np.fft.ifft2(np.fft.fft2(np.asarray(delta, np.float64)) * np.fft.fft2(shifted)).real
    return conv.astype(np.float32)


def _stop(peak_abs, threshold, cycle_threshold, nsigma=0.0):
    return O._STOP_NAMES[O.stop_reason(float(peak_abs), float(threshold),
                                       float(cycle_threshold), float(nsigma))]


def clark_minor_cycle(model, residual, psf, patch, gain, cycle_niter, threshold=0.0,
                      cycle_threshold=0.0, nsigma=0.0):
    model = np.array(model, np.float32, copy=True)
    res = np.array(residual, np.float32, copy=True)
    psf = np.asarray(psf, np.float32)
    nx, ny = res.shape
    p, rx, ry, mea = patch["patch"], patch["rx"], patch["ry"], patch["max_exterior_abs"]
    gain, thr, cyc = f32(gain), f32(threshold), f32(cycle_threshold)
    updates, updated, stop = 0, False, None
    approx = f32(np.abs(res).max())
    prev = approx
    factor = f32(1.5) / f32(4.5)
    warn = False
    max_iter = cycle_niter
    if mea > f32(0.5):
        max_iter = min(max_iter, 5)
    elif mea > f32(0.35):
        max_iter = min(max_iter, 50)
    comps = []
    sub = 0
    while updates < cycle_niter and sub < MAX_SUBCYCLES:
        r = _stop(approx, thr, cyc, nsigma)
        if r is not None:
            stop = r
            break
        flux_limit = f32(f32(approx * mea) * factor)
        if factor > 1.0:
            flux_limit = min(flux_limit, f32(f32(0.95) * approx))
        sel = max(flux_limit, cyc)
        keep = ~(np.abs(res) < sel)
        xs, ys = np.nonzero(keep)                     # row-major order
        vals = res[xs, ys].astype(np.float32)
        index = -np.ones((nx, ny), np.int64)
        index[xs, ys] = np.arange(len(xs))
        if len(vals) == 0:
            if warn:
                stop = "NoCleanablePixels"
                break
            factor = f32(factor * f32(1.2))
            warn = True
            sub += 1
            continue
        limit = min(cycle_niter - updates, max_iter)
        delta = np.zeros_like(res)
        fmn = f32(0.0)
        iter_limit = sel
        init_peak = f32(np.abs(vals).max())
        fac = f32(init_peak / flux_limit) if flux_limit > 0 and init_peak > 0 else f32(1.0)
        added = 0
        while added < limit:
            k = int(np.argmax(np.abs(vals)))
            pv = vals[k]
            r = _stop(abs(pv), thr, iter_limit, nsigma)
            if r is not None:
                stop = r
                break
            comp = f32(gain * pv)
            x, y = int(xs[k]), int(ys[k])
            model[x, y] = f32(model[x, y] + comp)
            delta[x, y] = f32(delta[x, y] + comp)
            comps.append(((x, y), float(comp)))
            for qx in range(p.shape[0]):
                px = x + qx - rx
                if px < 0 or px >= nx:
                    continue
                for qy in range(p.shape[1]):
                    py = y + qy - ry
                    if py < 0 or py >= ny:
                        continue
                    s = index[px, py]
                    if s >= 0:
                        vals[s] = f32(vals[s] - f32(comp * p[qx, qy]))
            updates += 1
            added += 1
            updated = True
            fmn = f32(fmn + f32(fac / f32(updates)))
            iter_limit = max(f32(flux_limit * fmn), cyc)
        approx = f32(np.abs(vals).max())
        if added > 0:
            res = (res - fft_convolve_real(psf, delta)).astype(np.float32)
        if approx > prev:
            factor = f32(factor * f32(3.0))
            max_iter = min(max_iter, 10)
            warn = True
        prev = approx
        if added == 0:
            break
        if stop is not None and updates < cycle_niter:
            stop = None
        sub += 1
    if not updated and stop is None:
        stop = "NoCleanablePixels"
    return dict(model=model, residual=res, components=comps, actual=updates, stop_reason=stop,
                updated=updated)


def clark_step_niter(n: int) -> int:
    return n if n < 5000 else 2000


def clark_cotton_schwab(residual, psf, refresh, patch, niter, gain=0.1, threshold=0.0,
                        minor_cycle_length=2000, cyclefactor=1.0, min_psf_fraction=0.05,
                        max_psf_fraction=0.8, major_cycle_limit=None, sidelobe=0.0):
    res = np.array(residual, np.float32, copy=True)
    model = np.zeros_like(res)
    actual = reported = major = 0
    stop = None
    min_peak = f32(np.abs(res).max())
    comps, thresholds = [], []
    handoff = ("CycleThresholdReached", "NsigmaThresholdReached")
    while reported < niter:
        if major_cycle_limit is not None and major >= major_cycle_limit:
            stop = "MajorCycleLimitReached"
            break
        pk = O.peak_location(res)
        if pk is None:
            stop = "NoCleanablePixels"
            break
        peak = abs(pk[1])
        s = O.tolerant_clean_stop_reason(peak, threshold, 0.0)
        if s is not None:
            stop = s
            break
        step = clark_step_niter(min(niter - reported, minor_cycle_length))
        thr = O.clean_cycle_threshold(peak, sidelobe, cyclefactor, min_psf_fraction,
                                      max_psf_fraction, threshold)
        thresholds.append(thr)
        out = clark_minor_cycle(model, res, psf, patch, gain, step, threshold, thr)
        model, res = out["model"], out["residual"]
        comps.extend(out["components"])
        after = reported + out["actual"]
        if out["updated"]:
            res = np.asarray(refresh(model), np.float32)
            if after < niter:
                major += 1
        actual += out["actual"]
        reported = after
        stop_after = False
        reason = out["stop_reason"]
        if reason is not None:
            if reason in handoff and out["updated"]:
                pass
            elif reason in handoff:
                stop = reason
            else:
                stop = reason
                stop_after = True
        if not out["updated"] or stop_after:
            break
        minor_peak = f32(np.abs(res).max())
        if minor_peak < min_peak:
            min_peak = minor_peak
        elif min_peak > 0 and (minor_peak - min_peak) / min_peak > f32(0.1):
            stop = "DivergenceDetected"
            break
        if stop is None and reported >= niter:
            stop = "IterationLimitReached"
            break
        s = O.tolerant_clean_stop_reason(f32(np.abs(res).max()), threshold, 0.0)
        if s is not None:
            stop = s
            break
    if niter > 0 and stop is None:
        stop = "IterationLimitReached"
    return dict(model=model, residual=res, major_cycles=major, actual=actual, reported=reported,
                stop_reason=stop, thresholds=thresholds, components=comps)
