"""The planners' float32-pair operations, emulated on the CPU.

The W-projection and standard plan kernels (csrc/cr_plan.cu) avoid FP64
instructions on their common path: a coordinate is split into a float32 pair
from its bits (df_split, csrc/cr_fixed.cuh), the w-plane round(sqrt(w_scale
|w|)) is decided on a pair product with a 2^-36 relative margin
(df_plane_of, falling back to exact FP64 products when undecided), and the
sums of weights are compensated pair sums of exact products (PairSum).
These tests restate those operations in exact IEEE float32 arithmetic and
check: the split's error bound; that every plane the pair path decides
equals the reference's FP64 plane (WProjector::plan_sample,
gridder.rs:3588-3624), for random w and for w placed on and a few ulps
around every plane boundary, with few undecided; and the pair sums'
accuracy against exact rational sums.
"""
import math
import struct
from fractions import Fraction

import numpy as np

from test_fastpath_cpu import f32, pair, product

TWO_M36 = f32(2.0 ** -36)


def df_split(x: float):
    """df_split: hi = x truncated to 24 significant bits, lo = RN32(x - hi)."""
    b = struct.unpack("<Q", struct.pack("<d", x))[0]
    sign = b >> 63
    if (b << 1) & ((1 << 64) - 1) == 0:
        return f32(-0.0 if sign else 0.0), f32(0.0)
    e = ((b >> 52) & 0x7FF) - 1023
    if e < -70 or e >= 100:
        return None
    hi_bits = (sign << 31) | ((e + 127) << 23) | ((b >> 29) & 0x7FFFFF)
    hi = np.frombuffer(struct.pack("<I", hi_bits), np.float32)[0]
    r = f32(b & 0x1FFFFFFF) * f32(2.0 ** (e - 52))
    return hi, (-r if sign else r)


def df_plane(wh, wl, kwh, kwl, planes):
    """df_plane_of: the plane, or None when undecided."""
    qh, ql = product(f32(abs(wh)), f32(abs(wl)), kwh, kwl)
    if not qh < f32(4.0e6):
        return None
    k = int(np.rint(np.sqrt(qh)))

    def diff(j):
        t = f32(j) - f32(0.5)
        return f32(f32(qh - f32(t * t)) + ql)

    if k > 0 and diff(k) < 0:
        k -= 1
    elif diff(k + 1) >= 0:
        k += 1
    tl, th = f32(k) - f32(0.5), f32(k) + f32(0.5)
    if (k > 0 and not diff(k) > f32(tl * tl) * TWO_M36) or not (-diff(k + 1) > f32(th * th) * TWO_M36):
        return None
    return min(k, planes - 1)


def fp64_plane(w, w_scale, planes):
    """The reference's plane: round half away from zero of sqrt(RN64(w_scale |w|))."""
    c = math.sqrt(max(w_scale * abs(w), 0.0))
    r = math.floor(c)
    if c - r >= 0.5:
        r += 1
    return int(min(max(r, 0), planes - 1))


def test_split_error_bound():
    rng = np.random.default_rng(3)
    xs = list(rng.uniform(0.5, 1.0, 2000) * rng.choice([-1, 1], 2000) * 2.0 ** rng.integers(-69, 99, 2000))
    xs += [0.0, -0.0, 1.0, -1.5, 2.0 ** -70, -(2.0 ** 99), 123456.789, 1e-3, 3e5]
    for x in xs:
        s = df_split(float(x))
        assert s is not None
        hi, lo = s
        assert abs(float(hi)) <= abs(x)                       # truncation toward zero
        err = abs(Fraction(float(x)) - Fraction(float(hi)) - Fraction(float(lo)))
        assert err <= Fraction(abs(float(x))) / 2 ** 47
    for x in (2.0 ** -71, 2.0 ** 100, float("inf"), float("nan"), 5e-324):
        assert df_split(x) is None


def test_planes_equal_fp64():
    rng = np.random.default_rng(11)
    decided = total = 0
    for planes, w_max in ((128, 3000.0), (64, 150.0), (16, 2.5e4), (1000, 1.0e5)):
        w_scale = (planes - 1) ** 2 / w_max
        kwh, kwl = pair(w_scale)
        ws = list(rng.uniform(-w_max * 1.1, w_max * 1.1, 3000))
        # on and around every boundary (k + 1/2)^2 = w_scale |w|
        for k in range(0, min(planes, 300)):
            wb = (k + 0.5) ** 2 / w_scale
            for sgn in (1.0, -1.0):
                x = sgn * wb
                ws.append(x)
                up = dn = x
                for _ in range(3):
                    up = np.nextafter(up, np.inf)
                    dn = np.nextafter(dn, -np.inf)
                    ws += [float(up), float(dn)]
        for w in ws:
            w = float(w)
            wh, wl = df_split(w)
            got = df_plane(wh, wl, kwh, kwl, planes)
            total += 1
            if got is None:
                continue
            decided += 1
            assert got == fp64_plane(w, w_scale, planes), (planes, w)
    # the boundary cases are mostly undecided; random ones almost never are
    assert decided >= 0.6 * total


def test_random_planes_mostly_decided():
    rng = np.random.default_rng(13)
    planes, w_max = 128, 3000.0
    w_scale = (planes - 1) ** 2 / w_max
    kwh, kwl = pair(w_scale)
    ws = rng.uniform(-w_max, w_max, 5000)
    undecided = sum(df_plane(*df_split(float(w)), kwh, kwl, planes) is None for w in ws)
    assert undecided <= 5


def pair_add(h, l, ph, pl):
    """PairSum.add."""
    s = f32(h + ph)
    bb = f32(s - h)
    err = f32(f32(h - f32(s - bb)) + f32(ph - bb))
    t = f32(err + f32(l + pl))
    nh = f32(s + t)
    return nh, f32(t - f32(nh - s))


def test_pair_sums_of_exact_products():
    rng = np.random.default_rng(17)
    wt = rng.uniform(0.1, 3.0, 4000).astype(np.float32)
    nrm = rng.uniform(0.5, 2.0, 4000).astype(np.float32)
    h = l = f32(0.0)
    exact = Fraction(0)
    for a, b in zip(wt, nrm):
        p = f32(a * b)
        e = f32(Fraction(float(a)) * Fraction(float(b)) - Fraction(float(p)))   # fma(a, b, -p)
        assert Fraction(float(p)) + Fraction(float(e)) == Fraction(float(a)) * Fraction(float(b))
        h, l = pair_add(h, l, f32(2) * p, f32(2) * e)
        exact += 2 * Fraction(float(a)) * Fraction(float(b))
    got = Fraction(float(h)) + Fraction(float(l))
    assert abs(got - exact) <= exact * Fraction(1, 2 ** 40)

