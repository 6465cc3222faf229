"""Multiscale CLEAN: CPU restatement (test infrastructure).

Restates with float32 arithmetic, following crates/casa-imaging/src/lib.rs:
  * make_multiscale_kernel / multiscale_spheroidal (lib.rs:64325-64405): the
    tapered-disc scale images (FP64 where the reference promotes, float32
    elsewhere, `powf` from the C library), normalised to unit volume;
  * kernel_nonzero_support (lib.rs:74940-74964), add_shifted_kernel_with_support
    and shifted_kernel_image_bounds (lib.rs:74966-75040);
  * build_multiscale_state (lib.rs:64172-64230): residual and PSF convolved with
    the scales by fft_convolve_real -- here FP64 circular convolutions
    (numpy FFT) rounded to float32, where the reference uses float32 FFTs --
    the PSF cross terms, their peaks (at least 1e-6) and the small-scale bias;
    the scale masks of a clean mask (lib.rs:64232-64261);
  * select_multiscale_candidate (lib.rs:64263-64305) over
    peak_location_masked_in_bounds_zero_tolerance (lib.rs:74064-74118: first
    scanned pixel, replaced by a larger |value| or an equal one with a smaller
    y * nx + x), the divergence rule (lib.rs:64011-64023), the component
    window (ImageWindow::from_casa_shifted_support, lib.rs:63221-63238) and
    subtract_multiscale_component (lib.rs:64307-64323);
  * the minor cycle and run_multiscale_cotton_schwab (lib.rs:63543-63963).
NaN pixels never win a peak search here (the reference keeps one only when
it is the first pixel scanned).
"""
import numpy as np

from . import oracle as O
from .clark import fft_convolve_real

f32 = np.float32


def multiscale_spheroidal(nu):
    nu = f32(nu)
    if nu <= 0:
        return f32(1.0)
    if nu >= 1:
        return f32(0.0)
    if nu < f32(0.75):
        p = [8.203343e-2, -3.644705e-1, 6.27866e-1, -5.335581e-1, 2.312756e-1]
        q = [1.0, 8.212018e-1, 2.078043e-1]
        nuend = f32(0.75)
    else:
        p = [4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2]
        q = [1.0, 9.599102e-1, 2.918724e-1]
        nuend = f32(1.0)
    p = [f32(c) for c in p]
    q = [f32(c) for c in q]
    delnusq = f32(np.power(nu, f32(2.0)) - np.power(nuend, f32(2.0)))
    num = p[0]
    for k in range(1, 5):
        num = f32(num + f32(p[k] * np.power(delnusq, f32(k))))
    den = q[0]
    for k in range(1, 3):
        den = f32(den + f32(q[k] * np.power(delnusq, f32(k))))
    return f32(0.0) if den == 0 else f32(num / den)


def make_multiscale_kernel(shape, scale):
    nx, ny = shape
    k = np.zeros((nx, ny), np.float32)
    refi, refj = float(nx // 2), float(ny // 2)
    if scale == 0.0:
        k[int(refi), int(refj)] = 1.0
        return k
    s = float(f32(scale))
    mini = max(int(refi - s), 0)        # `as isize` truncates toward zero
    maxi = min(int(refi + s), nx - 1)
    minj = max(int(refj - s), 0)
    maxj = min(int(refj + s), ny - 1)
    vol = f32(0.0)
    for j in range(minj, maxj + 1):
        t = (refj - j) / s
        ypart = f32(t * t)
        for i in range(mini, maxi + 1):
            ti = (refi - i) / s
            rad2 = f32(float(ypart) + ti * ti)
            if rad2 < 1.0:
                rad = f32(0.0) if rad2 <= 0 else f32(np.sqrt(rad2))
                val = f32((1.0 - float(rad2)) * float(multiscale_spheroidal(rad)))
                k[i, j] = val
                vol = f32(vol + val)
    if vol > 0:
        k = (k / vol).astype(np.float32)
    return k


def kernel_support(k):
    xs, ys = np.nonzero(k != 0.0)
    if len(xs) == 0:
        return None
    return int(xs.min()), int(ys.min()), int(xs.max()), int(ys.max())


def add_shifted_kernel(image, kernel, support, pos, factor):
    """add_shifted_kernel_with_support: image += factor * kernel shifted so
    that its centre (nx/2, ny/2) lands on pos, over the kernel's support."""
    if support is None:
        return
    nx, ny = image.shape
    cx, cy = kernel.shape[0] // 2, kernel.shape[1] // 2
    x0 = pos[0] + support[0] - cx
    x1 = pos[0] + support[2] - cx
    y0 = pos[1] + support[1] - cy
    y1 = pos[1] + support[3] - cy
    if x1 < 0 or y1 < 0 or x0 > nx - 1 or y0 > ny - 1:
        return
    x0, y0, x1, y1 = max(x0, 0), max(y0, 0), min(x1, nx - 1), min(y1, ny - 1)
    if x0 > x1 or y0 > y1:
        return
    sub = kernel[x0 - pos[0] + cx:x1 - pos[0] + cx + 1, y0 - pos[1] + cy:y1 - pos[1] + cy + 1]
    image[x0:x1 + 1, y0:y1 + 1] = (image[x0:x1 + 1, y0:y1 + 1]
                                   + (f32(factor) * sub).astype(np.float32)).astype(np.float32)


def component_window(shape, pos):
    nx, ny = shape
    hx, hy = nx // 2, ny // 2
    return (max(pos[0] - hx, 0), max(pos[1] - hy, 0),
            min(max(pos[0] + hx - 1, 0), nx - 1), min(max(pos[1] + hy - 1, 0), ny - 1))


def subtract_in_window(image, kernel, pos, factor, window):
    """subtract_shifted_kernel_in_window (lib.rs:74805-74870)."""
    nx, ny = image.shape
    cx, cy = kernel.shape[0] // 2, kernel.shape[1] // 2
    kx0, ky0 = pos[0] - cx, pos[1] - cy
    kx1, ky1 = kx0 + kernel.shape[0] - 1, ky0 + kernel.shape[1] - 1
    if kx1 < 0 or ky1 < 0 or kx0 > nx - 1 or ky0 > ny - 1:
        return
    x0, y0 = max(window[0], kx0, 0), max(window[1], ky0, 0)
    x1, y1 = min(window[2], kx1, nx - 1), min(window[3], ky1, ny - 1)
    if x0 > x1 or y0 > y1:
        return
    sub = kernel[x0 - kx0:x1 - kx0 + 1, y0 - ky0:y1 - ky0 + 1]
    image[x0:x1 + 1, y0:y1 + 1] = (image[x0:x1 + 1, y0:y1 + 1]
                                   - (f32(factor) * sub).astype(np.float32)).astype(np.float32)


def peak_in_window(image, mask, window):
    """peak_location_masked_in_bounds_zero_tolerance over the window: the
    largest |value|, ties to the smallest y * nx + x; None when no pixel."""
    nx, ny = image.shape
    x0, y0, x1, y1 = window
    sub = np.abs(image[x0:x1 + 1, y0:y1 + 1]).astype(np.float32)
    ok = np.isfinite(sub)
    if mask is not None:
        ok &= mask[x0:x1 + 1, y0:y1 + 1]
    if not ok.any():
        return None
    vals = np.where(ok, sub, f32(-1.0))
    best = vals.max()
    xs, ys = np.nonzero(vals == best)
    keys = (ys + y0) * nx + (xs + x0)
    i = int(np.argmin(keys))
    x, y = int(xs[i] + x0), int(ys[i] + y0)
    return (x, y), f32(image[x, y])


def scale_masks(mask, scales, kernels):
    vals = np.asarray(mask, bool).astype(np.float32)
    out = []
    for s, k in zip(scales, kernels):
        m = fft_convolve_real(k, vals) > f32(0.9)
        nx, ny = m.shape
        border = int(f32(s) * f32(1.5))
        xs = np.arange(nx)[:, None]
        ys = np.arange(ny)[None, :]
        edge = (xs <= border) | (ys <= border) | (xs >= nx - (border + 1)) | (ys >= ny - (border + 1))
        out.append(m & ~edge)
    return out


class MultiscaleState:
    """build_multiscale_state (lib.rs:64172-64230)."""

    def __init__(self, residual, psf, scales, small_scale_bias, mask=None):
        residual = np.asarray(residual, np.float32)
        psf = np.asarray(psf, np.float32)
        self.shape = residual.shape
        self.scale_sizes = [float(s) for s in scales] if len(scales) else [0.0]
        self.kernels = [make_multiscale_kernel(self.shape, s) for s in self.scale_sizes]
        self.supports = [kernel_support(k) for k in self.kernels]
        K = len(self.kernels)
        self.set_residual(residual)
        pk = [fft_convolve_real(k, psf) for k in self.kernels]
        self.psf_conv = [[fft_convolve_real(self.kernels[l], pk[k]) for l in range(K)]
                         for k in range(K)]
        self.peak_psf = [max(f32(np.max(np.abs(self.psf_conv[k][k]))), f32(1e-6))
                         for k in range(K)]
        mx = max([f32(0.0)] + [f32(s) for s in self.scale_sizes])
        if mx > 0 and K > 1:
            self.bias = [f32(f32(1.0) - f32(f32(small_scale_bias) * f32(f32(s) / mx)))
                         for s in self.scale_sizes]
        else:
            self.bias = [f32(1.0)] * K
        self.scale_masks = None if mask is None else scale_masks(mask, self.scale_sizes,
                                                                 self.kernels)
        self.mask = None if mask is None else np.asarray(mask, bool)

    def set_residual(self, residual):
        """refresh_multiscale_dirty_conv_scales (lib.rs:63261-63267)."""
        r = np.asarray(residual, np.float32)
        self.dirty = [fft_convolve_real(k, r) for k in self.kernels]

    def candidate(self, window):
        best = None
        for k in range(len(self.kernels)):
            m = self.scale_masks[k] if self.scale_masks is not None else self.mask
            pk = peak_in_window(self.dirty[k], m, window)
            if pk is None:
                continue
            pos, val = pk
            peak = self.peak_psf[k]
            if peak <= 0 or val == 0:
                continue
            strength = f32(val / peak)
            score = f32(f32(self.bias[k] * val) * strength)
            if best is None or abs(score) > abs(best[1]):
                best = (dict(scale=k, pos=pos, strength=strength, value=val), score)
        return None if best is None else best[0]

    def residual(self):
        return self.dirty[0].copy()


def full_window(shape):
    return (0, 0, shape[0] - 1, shape[1] - 1)


def minor_cycle(state, model, gain, cycle_niter, threshold=0.0, cycle_threshold=0.0,
                nsigma_threshold=0.0):
    """The minor cycle of run_multiscale_cotton_schwab (lib.rs:63700-63800):
    model is updated in place; returns the components and the stop reason."""
    shape = state.shape
    window = full_window(shape)
    comps = []
    stop = None
    initial = None
    while len(comps) < cycle_niter:
        c = state.candidate(window)
        if c is None:
            stop = "NoCleanablePixels"
            break
        a = abs(c["strength"])
        s = O._STOP_NAMES[O.stop_reason(float(a), float(threshold), float(cycle_threshold),
                                        float(nsigma_threshold))]
        if s is not None:
            stop = s
            break
        if initial is None:
            initial = a
        if len(comps) > 0 and a > f32(abs(initial) * f32(1.5)):
            stop = "DivergenceDetected"
            break
        comp = f32(f32(gain) * c["strength"])
        k = c["scale"]
        add_shifted_kernel(model, state.kernels[k], state.supports[k], c["pos"], comp)
        win = component_window(shape, c["pos"])
        for j in range(len(state.kernels)):
            subtract_in_window(state.dirty[j], state.psf_conv[j][k], c["pos"], comp, win)
        window = win
        comps.append((c["pos"], k, float(c["strength"]), float(comp)))
    return comps, stop


def cotton_schwab(residual, psf, refresh, niter, scales, small_scale_bias=0.0, gain=0.1,
                  threshold=0.0, minor_cycle_length=2000, cyclefactor=1.0,
                  min_psf_fraction=0.05, max_psf_fraction=0.8, major_cycle_limit=None,
                  sidelobe=0.0, nsigma=0.0, mask=None):
    """run_multiscale_cotton_schwab (lib.rs:63543-63963) with the oracle's
    FP64 refresh.  Returns model, residual, cycles, iterations, stop reason,
    thresholds and components (position, scale index, strength, flux)."""
    res = np.asarray(residual, np.float32).copy()
    st = MultiscaleState(res, psf, scales, small_scale_bias, mask)
    model = np.zeros_like(res)
    mk = None if mask is None else np.asarray(mask, np.uint8)
    actual = reported = major = 0
    stop = None
    min_peak = f32(np.max(np.abs(res)))
    needs_refresh = False
    comps, thresholds = [], []
    while reported < niter:
        if major_cycle_limit is not None and major >= major_cycle_limit:
            stop = "MajorCycleLimitReached"
            break
        if st.candidate(full_window(res.shape)) is None:
            stop = "NoCleanablePixels"
            break
        pk = O.peak_location(st.dirty[0], mk)
        peak = f32(abs(pk[1])) if pk is not None else f32(0.0)
        nsig = O.nsigma_threshold(res, nsigma, mk)
        s = O.tolerant_clean_stop_reason(peak, threshold, nsig)
        if s is not None:
            stop = s
            break
        cyc_niter = min(niter - reported, minor_cycle_length)
        thr = O.clean_cycle_threshold(peak, sidelobe, cyclefactor, min_psf_fraction,
                                      max_psf_fraction, threshold)
        thresholds.append(thr)
        cc, reason = minor_cycle(st, model, gain, cyc_niter, threshold, thr, nsig)
        comps.extend(cc)
        actual += len(cc)
        reported += min(len(cc), cyc_niter)
        if not cc:
            stop = reason
            break
        res = st.residual()
        needs_refresh = True
        mp = f32(np.max(np.abs(res)))
        if mp < min_peak:
            min_peak = mp
        elif min_peak > 0 and (mp - min_peak) / min_peak > f32(0.1):
            stop = "DivergenceDetected"
            break
        if stop is None and reported >= niter:
            stop = "IterationLimitReached"
            break
        res = np.asarray(refresh(model), np.float32)
        st.set_residual(res)
        major += 1
        needs_refresh = False
        pk = O.peak_location(res, mk)
        rp = f32(abs(pk[1])) if pk is not None else f32(0.0)
        s = O.tolerant_clean_stop_reason(rp, threshold, O.nsigma_threshold(res, nsigma, mk))
        if s is not None:
            stop = s
            break
    if niter > 0 and stop is None:
        stop = "IterationLimitReached"
    if needs_refresh:
        res = np.asarray(refresh(model), np.float32)
        major += 1
    return dict(model=model, residual=res, major_cycles=major, actual=actual,
                reported=reported, stop_reason=stop, thresholds=thresholds, components=comps)
