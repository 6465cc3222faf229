"""The cube planner's float32-pair fast path, emulated on the CPU.

The device tries every index decision of the cube (grid anchor and
oversampling offset per axis, density cell per axis) first in float32 pairs
(cr_fixed.cuh: df_product, df_nearest, df_tap_span) and takes it only when
the value lies more than 2^-12 from a boundary.  This test restates those
operations with exact IEEE float32 arithmetic (fused multiply-adds rounded
once, from exact rationals) and checks, on random cube samples and on
samples placed on and one ulp around every kind of boundary, that each
decision the fast path takes equals the oracle's FP64 decision
(sample_tap_span, gridder.rs:1976-1995; the rounded density cell,
weight_density_cell_anchor, gridder.rs:1888-1934), and that it leaves only
a small fraction undecided.
"""
from fractions import Fraction

import numpy as np

from casars_cuda import synthetic as S
from oracle import oracle as O

MARGIN = np.float32(1.0 / 4096.0)
LIMIT = np.float32(1048576.0)
f32 = np.float32


def rn32(q: Fraction) -> np.float32:
    """Round a rational to the nearest float32 (ties to even); normal range."""
    if q == 0:
        return f32(0.0)
    s = -1 if q < 0 else 1
    q = abs(q)
    e = q.numerator.bit_length() - q.denominator.bit_length()
    while Fraction(2) ** e > q:
        e -= 1
    while Fraction(2) ** (e + 1) <= q:
        e += 1
    scaled = q / Fraction(2) ** (e - 23)          # in [2^23, 2^24)
    m, r = divmod(scaled.numerator, scaled.denominator)
    if 2 * r > scaled.denominator or (2 * r == scaled.denominator and m % 2 == 1):
        m += 1
    return f32(s * m * 2.0 ** (e - 23))


def fma32(a, b, c):
    return rn32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def pair(x) -> tuple:
    """A value as a float32 pair (hi, lo)."""
    q = Fraction(x)
    hi = rn32(q)
    return hi, rn32(q - Fraction(float(hi)))


def product(ah, al, kh, kl):
    p = f32(ah * kh)
    e = fma32(ah, kh, -p)
    e = fma32(ah, kl, e)
    e = fma32(al, kh, e)
    return p, e


def nearest(p, e, h):
    if not abs(p) < LIMIT:
        return None
    q = f32(p + f32(h))
    r = f32(np.rint(q))
    d = f32(f32(q - r) + e)
    if not abs(abs(d) - f32(0.5)) > MARGIN:
        return None
    n = r + (1 if d > 0.5 else -1 if d < -0.5 else 0)
    return int(n), f32(q - f32(n))


def tap_span(p, e, size, os_, rows):
    """1 / 0 / None (undecided) and (start, row) -- df_tap_span."""
    t = nearest(p, e, 0.5 if size & 1 else 0.0)
    if t is None:
        return None, None
    a, dh = t
    anchor = size // 2 + a
    if anchor - 3 < 0 or anchor + 3 >= size:
        return 0, None
    osf = f32(os_)
    v = -fma32(dh, osf, f32(e * osf))
    o = f32(np.rint(v))
    if not f32(0.5) - abs(f32(v - o)) > MARGIN:
        return None, None
    idx = int(o) + os_ // 2
    if idx < 0 or idx >= rows:
        return 0, None
    return 1, (anchor - 3, idx)


def density_axis(p, e, n):
    t = nearest(p, e, 0.5 if n & 1 else 0.0)
    return None if t is None else n // 2 + t[0]


def _samples():
    obs = S.cube_observation(channels=4, nx=256, hours=2.0, dump_s=300.0, seed=3)
    rng = np.random.default_rng(5)
    ls = obs.lambda_scale
    um = np.concatenate([obs.u_m[:1500], rng.normal(0.0, 300.0, 500)])
    vm = np.concatenate([obs.v_m[:1500], rng.normal(0.0, 300.0, 500)])
    return obs, ls, um, vm


def _boundary_metres(centre, scale, targets):
    out = []
    for x in targets:
        base = (x - centre) / scale
        for _ in range(3):
            out.append(base)
            base = np.nextafter(base, np.inf)
        base = (x - centre) / scale
        for _ in range(2):
            base = np.nextafter(base, -np.inf)
            out.append(base)
    return np.array(out)


def test_fast_grid_decisions_equal_fp64():
    obs, ls, um, vm = _samples()
    os_ = 128
    geom = O.Geometry(obs.nx, obs.nx, obs.cell, obs.cell)
    og = O.StdGridder(geom, os_)
    rows = os_ + 1
    # boundary samples for the middle channel: anchors and offsets
    c0 = 2
    kx = ls[c0] / og.du
    xs = [b + k * 2.0 ** -20 for k in (-1, 0, 1) for b in (10.5, 100.5, og.gnx - 3.5, 3.5)]
    xs += [150.0 - (j + 0.5) / os_ for j in range(-66, 66)]
    ub = _boundary_metres(og.gnx / 2.0, kx, xs)
    um = np.concatenate([um, ub])
    vm = np.concatenate([vm, -ub[::-1]])
    decided = undecided = 0
    for c, s in enumerate(ls):
        ox, oy, orx, ory = og.plan_many(um * s, vm * s)
        fx = pair(Fraction(s) / Fraction(og.du))
        fy = pair(Fraction(s) / Fraction(og.dv))
        for i in range(len(um)):
            uh, ul = pair(um[i])
            vh, vl = pair(vm[i])
            px, ex = product(uh, ul, *fx)
            py, ey = product(-vh, -vl, *fy)
            sx, tx = tap_span(px, ex, og.gnx, os_, rows)
            sy, ty = (0, None) if sx == 0 else tap_span(py, ey, og.gny, os_, rows)
            if sx == 0 or sy == 0:
                assert ox[i] == -1, (c, i)
                decided += 1
            elif sx is None or sy is None:
                undecided += 1
            else:
                assert (ox[i], orx[i]) == tx and (oy[i], ory[i]) == ty, (c, i)
                decided += 1
    assert decided > 0.9 * (decided + undecided)
    assert undecided > 0   # the boundary samples reach the integer path


def test_fast_density_cells_equal_fp64():
    obs, ls, um, vm = _samples()
    nx = obs.nx + 1     # odd size: the centre is a half-integer
    geom = O.Geometry(nx, nx, obs.cell, obs.cell)
    dus = nx * obs.cell
    xs = [b + k * 2.0 ** -20 for k in (-1, 0, 1) for b in (5.5, 60.5, nx - 1.5)]
    ub = _boundary_metres(nx / 2.0, ls[1] * dus, xs)
    um = np.concatenate([um, ub])
    vm = np.concatenate([vm, ub[::-1]])
    decided = undecided = 0
    for s in ls:
        fd = pair(Fraction(s) * Fraction(dus))
        for i in range(len(um)):
            uh, ul = pair(um[i])
            vh, vl = pair(vm[i])
            px, ex = product(uh, ul, *fd)
            py, ey = product(-vh, -vl, *fd)
            for sign in (1, -1):
                cx = density_axis(f32(sign * px), f32(sign * ex), nx)
                cy = density_axis(f32(sign * py), f32(sign * ey), nx)
                ref = O.density_cell(geom, sign * um[i] * s, sign * vm[i] * s, convention=1)
                if cx is None or cy is None:
                    undecided += 1
                    continue
                decided += 1
                ok = not (cx <= 0 or cy <= 0 or cx >= nx or cy >= nx)
                assert (ref is not None) == ok, (i, sign)
                if ok:
                    assert tuple(ref) == (cx, cy), (i, sign)
    assert decided > 0.9 * (decided + undecided)
    assert undecided > 0
