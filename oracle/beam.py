"""Restoring-beam oracle (test infrastructure only): the PSF beam fit,
restoration and sidelobe level restated in Python/numpy.

Follows crates/casa-imaging/src/beam.rs: fit_beam_from_psf (27-103),
extract_casa_fit_samples (374-409), find_points_in_lobe (411-480),
resample_psf (505-525), fit_gaussian_beam_casa_seeded (535-610),
casa_gaussian_value_and_jacobian (676-713), casa_params_to_beam (721-768),
casa_wrap_beam_position_angle (770-789), casa_interp_cubic /
casa_interp_linear / casa_bcucof (791-964), restore_model (105-120),
make_casa_gaussian_psf_image (330-372), estimate_psf_sidelobe_level_with_beam
(319-328); the LDL^T solve of least_squares.rs:10-51.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

import numpy as np

F32 = np.float32
FWHM_TO_INTERNAL = 0.6005612043932249
PATCH_RADIUS, REGION_PADDING, TARGET_POINTS, MAX_ATTEMPTS = 20, 5, 3001, 50
MIN_SIGMA = 1.0e-12


@dataclass
class Beam:
    major_fwhm_rad: float
    minor_fwhm_rad: float
    position_angle_rad: float


def _first_max(img):
    flat = img.reshape(-1)
    best, bi = flat[0], 0
    for k in range(1, flat.size):        # strict '>' keeps the first maximum
        if flat[k] > best:
            best, bi = flat[k], k
    return divmod(bi, img.shape[1]), F32(best)


def _first_max_fast(img):
    k = int(np.argmax(img))             # numpy returns the first maximum too
    return divmod(k, img.shape[1]), F32(img.reshape(-1)[k])


def _lobe(psf, px, py, nrow, amin, dx, dy):
    nx, ny = psf.shape
    samples = []
    blc = [nx - 1, ny - 1]
    trc = [0, 0]
    iflip = jflip = 1
    maxn = (2 * nrow + 1) ** 2
    amin = F32(amin)
    done = False
    for jlo in range(2):
        if done:
            break
        jflip = -jflip
        for j in range(jlo, nrow + 1):
            if done:
                break
            jrow = py + j * jflip
            for ilo in range(2):
                iflip = -iflip
                if jrow > ny - 1 or jrow < 0:
                    break
                inlobe = psf[px, jrow] > amin
                for i in range(ilo, nrow + 1):
                    if len(samples) >= maxn:
                        done = True
                        break
                    irow = px + i * iflip
                    if irow > nx - 1 or irow < 0:
                        break
                    v = psf[irow, jrow]
                    if inlobe and v < amin:
                        break
                    if v > amin:
                        inlobe = True
                        blc = [min(blc[0], irow), min(blc[1], jrow)]
                        trc = [max(trc[0], irow), max(trc[1], jrow)]
                        samples.append(((irow - px) * dx, (jrow - py) * dy, float(v)))
                if done:
                    break
    if not samples:
        return None
    if blc[0] > blc[1]:
        blc[0] = blc[1]
    else:
        blc[1] = blc[0]
    if trc[0] > trc[1]:
        trc[1] = trc[0]
    else:
        trc[0] = trc[1]
    return samples, blc, trc


_WT = np.array([
    [1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0],
    [-3, 0, 0, 3, 0, 0, 0, 0, -2, 0, 0, -1, 0, 0, 0, 0],
    [2, 0, 0, -2, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0],
    [0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0],
    [0, 0, 0, 0, -3, 0, 0, 3, 0, 0, 0, 0, -2, 0, 0, -1],
    [0, 0, 0, 0, 2, 0, 0, -2, 0, 0, 0, 0, 1, 0, 0, 1],
    [-3, 3, 0, 0, -2, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, -3, 3, 0, 0, -2, -1, 0, 0],
    [9, -9, 9, -9, 6, 3, -3, -6, 6, -6, -3, 3, 4, 2, 1, 2],
    [-6, 6, -6, 6, -4, -2, 2, 4, -3, 3, 3, -3, -2, -1, -1, -2],
    [2, -2, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 2, -2, 0, 0, 1, 1, 0, 0],
    [-6, 6, -6, 6, -3, -3, 3, 3, -4, 4, 2, -2, -2, -2, -1, -1],
    [4, -4, 4, -4, 2, 2, -2, -2, 2, -2, -2, 2, 1, 1, 1, 1]], np.float64)


def _interp_linear(d, x, y):
    nx, ny = d.shape
    i, j = int(x), int(y)
    if i == nx - 1:
        i -= 1
    if j == ny - 1:
        j -= 1
    tt, uu = x - i, y - j
    return ((1.0 - tt) * (1.0 - uu) * float(d[i, j]) + tt * (1.0 - uu) * float(d[i + 1, j])
            + tt * uu * float(d[i + 1, j + 1]) + (1.0 - tt) * uu * float(d[i, j + 1]))


def _interp_cubic(d, x, y):
    nx, ny = d.shape
    i, j = int(x), int(y)
    if i <= 0 or i >= nx - 2 or j <= 0 or j >= ny - 2:
        return _interp_linear(d, x, y)
    tt, uu = x - i, y - j
    f = lambda a, b: d[a, b]            # float32 values, float32 arithmetic below
    v = [float(f(i, j)), float(f(i + 1, j)), float(f(i + 1, j + 1)), float(f(i, j + 1))]
    gx = [float(f(i + 1, j) - f(i - 1, j)), float(f(i + 2, j) - f(i, j)),
          float(f(i + 2, j + 1) - f(i, j + 1)), float(f(i + 1, j + 1) - f(i - 1, j + 1))]
    gy = [float(f(i, j + 1) - f(i, j - 1)), float(f(i + 1, j + 1) - f(i + 1, j - 1)),
          float(f(i + 1, j + 2) - f(i + 1, j)), float(f(i, j + 2) - f(i, j))]
    gxy = [float(f(i + 1, j + 1) + f(i - 1, j - 1) - f(i - 1, j + 1) - f(i + 1, j - 1)),
           float(f(i + 2, j + 1) + f(i, j - 1) - f(i, j + 1) - f(i + 2, j - 1)),
           float(f(i + 2, j + 2) + f(i, j) - f(i, j + 2) - f(i + 2, j)),
           float(f(i + 1, j + 2) + f(i - 1, j) - f(i - 1, j + 2) - f(i + 1, j))]
    gx = [g / 2.0 for g in gx]
    gy = [g / 2.0 for g in gy]
    gxy = [g / 4.0 for g in gxy]
    packed = np.array(v + gx + gy + gxy)
    cl = [0.0] * 16
    for r in range(16):
        acc = 0.0
        for k in range(16):
            acc += _WT[r, k] * packed[k]
        cl[r] = acc
    c = [cl[4 * r:4 * r + 4] for r in range(4)]
    result = F32(0.0)
    for r in range(3, -1, -1):
        result = F32(tt * float(result) + ((c[r][3] * uu + c[r][2]) * uu + c[r][1]) * uu + c[r][0])
    return float(result)


def _samples(psf, peak_idx, peak, dx, dy, cutoff):
    first = _lobe(psf, peak_idx[0], peak_idx[1], PATCH_RADIUS, cutoff, dx, dy)
    if first is None:
        return None
    _, blc, trc = first
    nx0, ny0 = psf.shape
    bx, by = max(blc[0] - REGION_PADDING, 0), max(blc[1] - REGION_PADDING, 0)
    tx, ty = min(trc[0] + REGION_PADDING, nx0 - 1), min(trc[1] + REGION_PADDING, ny0 - 1)
    side = max(tx - bx + 1, ty - by + 1)
    if tx - bx + 1 < side:
        bx = max(bx - (side - (tx - bx + 1)) // 2, 0)
        tx = min(bx + side - 1, nx0 - 1)
        bx = tx + 1 - side
    if ty - by + 1 < side:
        by = max(by - (side - (ty - by + 1)) // 2, 0)
        ty = min(by + side - 1, ny0 - 1)
        by = ty + 1 - side
    nx, ny = tx - bx + 1, ty - by + 1
    win = (psf[bx:tx + 1, by:ty + 1] / F32(peak)).astype(F32)
    os_ = TARGET_POINTS // (nx * ny)
    os_ = int(math.sqrt(os_))
    if os_ == 0:
        os_ = 1
    rx, ry = nx * os_ - os_ + 1, ny * os_ - os_ + 1
    res = np.zeros((rx, ry), F32)
    for i in range(rx):
        for j in range(ry):
            x = float(F32(i) / F32(os_))
            y = float(F32(j) / F32(os_))
            res[i, j] = F32(_interp_cubic(win, x, y))
    mx = F32(np.nanmax(res)) if np.any(~np.isnan(res)) else F32(-np.inf)
    if not (np.isfinite(mx) and mx > 0):
        return None
    res = (res / mx).astype(F32)
    (qx, qy), _ = _first_max(res)
    nrow = max(os_ * min(nx, ny) - 1, 0) // 2
    second = _lobe(res, qx, qy, nrow, cutoff, dx / os_, dy / os_)
    return None if second is None else second[0]


def _model_jac(p, x, y):
    w, q, pa = p
    if not (np.isfinite(w) and abs(w) > MIN_SIGMA and np.isfinite(q) and abs(q) > 1e-6
            and np.isfinite(pa)):
        return None
    c, s = math.cos(pa), math.sin(pa)
    xn, yn = x * c + y * s, -x * s + y * c
    xw = w * q
    xw2 = xw * xw * FWHM_TO_INTERNAL * FWHM_TO_INTERNAL
    yw2 = w * w * FWHM_TO_INTERNAL * FWHM_TO_INTERNAL
    x2w, y2w = 2.0 * xn / xw2, 2.0 * yn / yw2
    x2w2, y2w2 = x2w * xn, y2w * yn
    m = np.exp(-(xn * xn / xw2 + yn * yn / yw2))
    j = np.stack([m * ((x2w2 + y2w2) / w), m * x2w2 * w / xw,
                  -m * (x2w * (-x * s + y * c) + y2w * (-x * c - y * s))])
    if not (np.all(np.isfinite(m)) and np.all(np.isfinite(j))):
        return None
    return m, j


def _cost(S, p):
    w, q, pa = p
    if not (np.isfinite(w) and abs(w) > MIN_SIGMA and np.isfinite(q) and np.isfinite(pa)):
        return None
    r = _model_jac(p, S[:, 0], S[:, 1])
    m = r[0] if r is not None else np.zeros(len(S))
    c = 0.0
    for v in (m - S[:, 2]):            # sample order, as the reference sums
        c += v * v
    return c if np.isfinite(c) else None


def _normal(S, p):
    r = _model_jac(p, S[:, 0], S[:, 1])
    if r is None:
        return None
    m, J = r
    res = m - S[:, 2]
    N = np.zeros((3, 3))
    g = np.zeros(3)
    for k in range(len(S)):            # per-sample accumulation order
        jk = J[:, k]
        for a in range(3):
            g[a] += jk[a] * res[k]
            for b in range(a, 3):
                N[a, b] += jk[a] * jk[b]
    for a in range(3):
        for b in range(a):
            N[a, b] = N[b, a]
    return N, g


def _ldlt(N, k):
    N = N.copy()
    for r in range(3):
        orig = N[r, r]
        d = orig
        for p in range(r):
            d -= N[p, r] * N[p, r] / N[p, p]
        if not np.isfinite(d) or d * d / orig <= 1.0e-12:
            return None
        N[r, r] = d
        for c in range(r + 1, 3):
            for p in range(r):
                N[r, c] -= N[p, r] * N[p, c] / N[p, p]
    x = np.zeros(3)
    for r in range(3):
        x[r] = k[r]
        for p in range(r):
            x[r] -= N[p, r] * x[p] / N[p, p]
    for r in range(2, -1, -1):
        for c in range(r + 1, 3):
            x[r] -= N[r, c] * x[c]
        x[r] /= N[r, r]
    return x


def _wrap(a):
    h = math.pi / 2
    while abs(a / h) > 1.0:
        if a > 3 * h:
            a -= 2 * math.pi
        elif a > h:
            a -= math.pi
        elif a < -3 * h:
            a += 2 * math.pi
        else:
            a += math.pi
    return a


def _to_beam(p):
    w, q, pa = p
    if not all(np.isfinite(v) for v in p):
        return None
    if abs(q) > 1.0:
        maj, mn, pa = abs(w * q), abs(w), pa - math.pi / 2
    else:
        maj, mn = abs(w), abs(w * q)
    pa = _wrap(pa)
    if mn > maj:
        maj, mn = mn, maj
        pa = _wrap(pa + math.pi / 2)
    r2d = 180.0 / math.pi
    r2as = 3600.0 * r2d
    return Beam(float(F32(maj * r2as)) / r2as, float(F32(mn * r2as)) / r2as,
                float(F32(pa * r2d)) / r2d)


def _fit(S, cell_x):
    acc = (2.5 * abs(cell_x), 0.5, 1.0)
    ne = _normal(S, acc)
    if ne is None:
        return None
    N, k = ne
    k = -k
    cost = _cost(S, acc)
    if cost is None:
        return None
    lam, step = 1.0e-3, 2.0
    cand, delta, first = acc, np.zeros(3), True
    for _ in range(1000):
        if not first:
            cc = _cost(S, cand)
            if cc is None:
                return None
            expected = 0.0
            for a in range(3):
                expected += delta[a] * (lam * delta[a] * N[a, a] + k[a])
            expected *= 0.5
            actual = (cost - cc) * 0.5
            if expected > 0.0 and actual > 0.0:
                acc, cost = cand, cc
                ne = _normal(S, acc)
                if ne is None:
                    return None
                N, k = ne
                k = -k
                lam *= 0.3
                step = 2.0
                if np.all(np.abs(k) <= 1.0e-8):
                    break
            else:
                lam *= step
                step *= 2.0
                if step > 1.0e10:
                    break
        D = N.copy()
        for a in range(3):
            D[a, a] *= 1.0 + lam
        delta = _ldlt(D, k)
        if delta is None:
            return None
        cand = (acc[0] + delta[0], acc[1] + delta[1], acc[2] + delta[2])
        first = False
        dn = math.sqrt(sum(v * v for v in delta))
        pn = math.sqrt(sum(v * v for v in acc))
        if dn <= 1.0e-8 * (pn + 1.0e-8):
            break
    ne = _normal(S, cand)
    if ne is None:
        return None
    F, fk = ne
    fd = _ldlt(F, -fk)
    if fd is None:
        return None
    fin = (cand[0] + fd[0], cand[1] + fd[1], cand[2] + fd[2])
    if _cost(S, fin) is None:
        return None
    return _to_beam(fin)


def fit_beam(psf, cell, cutoff=0.35):
    """fit_beam_from_psf: (Beam or None, attempts, cutoff used)."""
    psf = np.ascontiguousarray(psf, F32)
    (px, py), peak = _first_max_fast(psf)
    if not (np.isfinite(peak) and peak > 0):
        return None, 0, None
    active = F32(min(max(cutoff, 0.01), 0.99))
    dx, dy = abs(cell[0]), abs(cell[1])
    for attempt in range(1, MAX_ATTEMPTS + 1):
        S = _samples(psf, (px, py), peak, dx, dy, active)
        if S is not None and len(S) >= 12:
            b = _fit(np.array(S), cell[0])
            if b is not None:
                return b, attempt, float(active)
        active = F32(active / F32(1.5))
    return None, MAX_ATTEMPTS, None


def gaussian_image(shape, cell, beam: Beam, normalize=False):
    """make_casa_gaussian_psf_image (float32 values of an FP64 evaluation)."""
    nx, ny = shape
    pa = beam.position_angle_rad + math.pi / 2
    c, s = math.cos(pa), math.sin(pa)
    rx, ry = nx // 2, ny // 2
    dx, dy = abs(cell[0]), abs(cell[1])
    sbmaj = 4.0 * math.log(2.0) * (1.0 / beam.major_fwhm_rad) ** 2
    sbmin = 4.0 * math.log(2.0) * (1.0 / beam.minor_fwhm_rad) ** 2
    X = (np.arange(nx)[:, None] - rx).astype(np.float64)
    Y = (np.arange(ny)[None, :] - ry).astype(np.float64)
    major = c * X * dx + s * Y * dy
    minor = -s * X * dx + c * Y * dy
    r = sbmaj * major ** 2 + sbmin * minor ** 2
    v = np.where(r < 20.0, np.exp(-np.minimum(r, 20.0)), 0.0)
    if normalize and v.sum() > 0:
        v = v / v.sum()
    return v.astype(F32)


def _cfft(x):
    return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(x)))


def _cifft(x):
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(x)))


def restore(model, residual, cell, beam: Beam):
    """restore_model + residual, with the centred FFTs in FP64."""
    model = np.asarray(model, np.float64)
    if np.all(np.abs(model) <= 1.0e-12):
        out = model
    else:
        g = gaussian_image(model.shape, cell, beam).astype(np.float64)
        out = _cifft(_cfft(model) * _cfft(g)).real
    return out + (0.0 if residual is None else np.asarray(residual, np.float64))


def sidelobe(psf, cell, beam: Beam):
    """estimate_psf_sidelobe_level_with_beam."""
    psf = np.asarray(psf, F32)
    g = gaussian_image(psf.shape, cell, beam)
    lo = min(0.0, float(np.min(psf)))
    hi = max(0.0, float(np.max(psf - g)))
    return max(abs(lo), abs(hi))


def synthetic_gaussian_psf(shape, cell, beam: Beam):
    """The reference tests' elliptical Gaussian PSF (beam.rs:1011-1035)."""
    nx, ny = shape
    out = np.zeros(shape, F32)
    sma = beam.major_fwhm_rad / 2.3548200450309493
    smi = beam.minor_fwhm_rad / 2.3548200450309493
    c, s = math.cos(beam.position_angle_rad), math.sin(beam.position_angle_rad)
    for x in range(nx):
        for y in range(ny):
            dx = (x - nx / 2.0) * cell[0]
            dy = (y - ny / 2.0) * cell[1]
            major = -dx * s + dy * c
            minor = dx * c + dy * s
            out[x, y] = F32(math.exp(-0.5 * ((major / sma) ** 2 + (minor / smi) ** 2)))
    return out
