// cr_fixed.cuh -- exact index selection with integer arithmetic.
//
// The reference chooses cells and oversampling offsets from FP64 values
// such as x = RN(RN(RN(u_m * s) / du) + G/2) (grid_coordinate_x,
// gridder.rs:1877-1879, after the cube batch scaling u = u_m * f/c of
// casars-imager/src/lib.rs:49571-49573) and then rounds half away from zero
// (sample_tap_span, gridder.rs:1976-1995).  FP64 runs at a small fraction of
// the FP32/integer rate on this GPU, so the common path evaluates the exact
// real value x* = u_m * (s/du) + G/2 in 64-bit fixed point instead:
//
//   * a = +-Ma 2^(ex-1075) (Ma the 53-bit significand) times a constant
//     K = m 2^e (m a 64-bit significand computed on the host to at least 63
//     correct bits) is formed with one 64 x 64 -> high-64 multiply and a
//     shift to F = 40 fractional bits; its error is below 4 units of 2^-40;
//   * the reference's own value differs from x* by at most 2^-38 for
//     |x| < 2^14 (three roundings of relative size 2^-53);
//   * every decision (the anchor, the offset, the density cell) compares x
//     against boundaries -- half-integers, or anchor - (k + 1/2)/os -- and is
//     taken only when x lies more than 2^-30 from the nearest one.
//     Otherwise the caller redoes the sample with the reference's FP64
//     operations (about one sample in 2^20).
// Decisions taken on the fixed-point path therefore equal the FP64 ones.
#pragma once

#include <cmath>
#include <cstdint>

namespace cr {

// K ~= m * 2^e with m in [2^63, 2^64).
struct FixScale {
    unsigned long long m;
    int e;
    int pad;
};

constexpr int kFixF = 40;
constexpr long long kFixOne = 1ll << kFixF;
constexpr long long kFixHalf = kFixOne >> 1;
constexpr long long kFixMask = kFixOne - 1;
constexpr long long kFixMargin = 1ll << (kFixF - 30);

// K = num / den (or num * den when `multiply`), rounded to 64 significant
// bits in long double (at least 64-bit significand on both supported hosts).
inline FixScale fix_scale_of(double num, double den, bool multiply) {
    long double k = multiply ? (long double)num * (long double)den
                             : (long double)num / (long double)den;
    FixScale s{0ull, 0, 0};
    if (!(k > 0.0L) || !std::isfinite((double)k)) return s;
    int e = 0;
    long double f = std::frexp(k, &e);            // k = f 2^e, f in [0.5, 1)
    long double mf = std::ldexp(f, 64);           // [2^63, 2^64)
    unsigned long long m = (unsigned long long)mf;
    if (m < (1ull << 63)) m = 1ull << 63;
    s.m = m;
    s.e = e - 64;
    return s;
}

// t ~= a * K * 2^F (|error| < 4 units).  False when a is not finite, is
// subnormal, or |a * K| >= 2^21 (the caller then takes the FP64 path).
__device__ __forceinline__ bool fix_mul(double a, FixScale k, long long* t) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(a);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) {
        if ((b << 1) == 0ull) {
            *t = 0;
            return true;
        }
        return false;
    }
    if (ex == 0x7ff || k.m == 0ull) return false;
    const unsigned long long ma = ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11;
    const unsigned long long h = __umul64hi(ma, k.m);   // [2^62, 2^64)
    // a * K = h * 2^(ex - 1086 + e + 64) up to the dropped low product
    const int sh = ex - 1022 + k.e + kFixF;
    if (sh > -3) return false;
    const int r = -sh;
    const unsigned long long v = r >= 64 ? 0ull : (h >> r);
    *t = (b >> 63) ? -(long long)v : (long long)v;
    return true;
}

// round half away from zero of X * 2^-F.  Returns false when X lies within
// `margin` of a half-integer boundary.
__device__ __forceinline__ bool fix_round(long long X, long long margin, long long* out) {
    const long long ax = X < 0 ? -X : X;
    const long long z = ax + kFixHalf;
    const long long rem = z & kFixMask;
    if (rem < margin || rem > kFixOne - margin) return false;
    const long long q = z >> kFixF;
    *out = X < 0 ? -q : q;
    return true;
}

// sample_tap_span (gridder.rs:1976-1995) of the coordinate X * 2^-F:
// 1 = accepted (start cell, tap row), 0 = rejected, -1 = too close to a
// rounding boundary to decide.
__device__ __forceinline__ int fix_tap_span(long long X, int64_t size, int32_t os, int32_t rows,
                                            int64_t* start, int32_t* row) {
    long long anchor;
    if (!fix_round(X, kFixMargin, &anchor)) return -1;
    if (anchor - 3 < 0 || anchor + 3 >= size) return 0;
    const long long d = (anchor << kFixF) - X;   // (anchor - x) 2^F, |d| <= 1/2 + margin
    long long off;
    if (!fix_round(d * (long long)os, kFixMargin * (long long)os, &off)) return -1;
    const long long idx = off + os / 2;
    if (idx < 0 || idx >= rows) return 0;
    *start = anchor - 3;
    *row = (int32_t)idx;
    return 1;
}

// ---- float32-pair fast path ---------------------------------------------------
// Before the integer path, the same decisions are tried in float32 pairs:
// a = ah + al (ah = RN32(a), al = RN32(a - ah), or df_split's truncated ah)
// and K = kh + kl, both to about 2^-47 relative; the product a K is then p + e with p = RN(ah kh),
// e = fma(ah, kh, -p) + ah kl + al kh (three FMAs), about 2^-44 |a K| from
// the exact value.  A decision is taken only when the exact value lies more
// than kDfMargin (in the decision's own units: cells for the anchor,
// oversampled cells for the offset) from its boundaries.  With |x| < 2^20
// the pair's error (below 2^-14 after the offset's scaling by os <= 512)
// and the reference's own FP64 error (below 2^-38) are far inside the
// margin, so the decision equals the FP64 one.  Otherwise (about one
// decision in 2^11) the caller takes the integer path.
constexpr float kDfMargin = 1.0f / 4096.0f;
constexpr float kDfLimit = 1048576.0f;   // |p| < 2^20

struct DfScale {
    float hi, lo;
};

// K = num / den (or num * den), as a float32 pair.
inline DfScale df_scale_of(double num, double den, bool multiply) {
    long double k = multiply ? (long double)num * (long double)den
                             : (long double)num / (long double)den;
    DfScale s{0.0f, 0.0f};
    if (!std::isfinite((double)k)) return s;
    s.hi = (float)k;
    s.lo = (float)(k - (long double)s.hi);
    return s;
}

__device__ __forceinline__ void df_product(float ah, float al, DfScale k, float* p, float* e) {
    const float ph = __fmul_rn(ah, k.hi);
    float er = __fmaf_rn(ah, k.hi, -ph);
    er = __fmaf_rn(ah, k.lo, er);
    er = __fmaf_rn(al, k.hi, er);
    *p = ph;
    *e = er;
}

// The float32 pair of a double from its bits, without FP64 instructions
// (GB300 issues FP64 at a small fraction of its float32 rate): hi = x with
// its significand truncated to 24 bits, lo = RN32(x - hi) (x - hi is the
// low 29 significand bits, converted as an integer and scaled by an exact
// power of two), so |x - (hi + lo)| <= 2^-47 |x|.  False for non-finite x
// and for 0 < |x| < 2^-70 or |x| >= 2^100; zero splits into (+-0, 0).
__device__ __forceinline__ bool df_split(double x, float* hi, float* lo) {
    // on the 32-bit halves of the double (with the 64-bit form, the FP64
    // pipe was half busy in the plan kernel)
    const unsigned bh = (unsigned)__double2hiint(x), bl = (unsigned)__double2loint(x);
    const unsigned sign = bh & 0x80000000u;
    if (((bh & 0x7fffffffu) | bl) == 0u) {
        *hi = __uint_as_float(sign);
        *lo = 0.0f;
        return true;
    }
    const int e = (int)((bh >> 20) & 0x7ffu) - 1023;
    if (e < -70 || e >= 100) return false;
    *hi = __uint_as_float(sign | (unsigned)(e + 127) << 23 | (bh & 0xfffffu) << 3 | bl >> 29);
    // RN32 of the low 29 significand bits as an integer, scaled by an exact
    // power of two
    const float r = __fmul_rn(__int2float_rn((int)(bl & 0x1fffffffu)),
                              __uint_as_float((unsigned)(e - 52 + 127) << 23));
    *lo = sign ? -r : r;
    return true;
}

// A sum held as an unevaluated float32 pair h + l (Knuth's two-sum; about
// 2^-47 relative per addition): sums of weights without FP64 instructions.
struct PairSum {
    float h = 0.0f, l = 0.0f;
    __device__ __forceinline__ void add(float ph, float pl) {
        const float s = __fadd_rn(h, ph);
        const float bb = __fsub_rn(s, h);
        const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
        const float t = __fadd_rn(err, __fadd_rn(l, pl));
        h = __fadd_rn(s, t);
        l = __fsub_rn(t, __fsub_rn(h, s));
    }
};

// The integer a nearest to x = p + e + h (h = 0 or 1/2) and dh = RN(p + h) - a
// (exact), or false when x is within the margin of a half-integer, is
// large, or is not finite.
__device__ __forceinline__ bool df_nearest(float p, float e, float h, float* a, float* dh) {
    if (!(fabsf(p) < kDfLimit)) return false;
    const float q = __fadd_rn(p, h);
    const float r = rintf(q);
    const float d = __fadd_rn(__fsub_rn(q, r), e);
    if (!(fabsf(fabsf(d) - 0.5f) > kDfMargin)) return false;
    float n = r;
    if (d > 0.5f) n = r + 1.0f;
    if (d < -0.5f) n = r - 1.0f;
    *a = n;
    *dh = __fsub_rn(q, n);
    return true;
}

// sample_tap_span of x = p + e + size / 2 (the grid coordinate): 1 =
// accepted, 0 = rejected, -1 = undecided (take the integer path).
__device__ __forceinline__ int df_tap_span(float p, float e, int64_t size, int32_t os,
                                           int32_t rows, int64_t* start, int32_t* row) {
    float a, dh;
    if (!df_nearest(p, e, (size & 1) ? 0.5f : 0.0f, &a, &dh)) return -1;
    // |a| < 2^20
    const int64_t anchor = (size >> 1) + (int)a;
    if (anchor - 3 < 0 || anchor + 3 >= size) return 0;
    // offset round((anchor - x) os) = round(-(dh + e) os)
    const float osf = (float)os;
    const float v = -__fmaf_rn(dh, osf, __fmul_rn(e, osf));
    const float o = rintf(v);
    if (!(0.5f - fabsf(__fsub_rn(v, o)) > kDfMargin)) return -1;
    const int64_t idx = (int)o + os / 2;
    if (idx < 0 || idx >= rows) return 0;
    *start = anchor - 3;
    *row = (int32_t)idx;
    return 1;
}

// sample_tap_span in the reference's FP64 operations.
__device__ __forceinline__ bool f64_tap_span(double coord, int64_t size, int32_t os,
                                             int32_t rows, int64_t* start, int32_t* row) {
    if (!isfinite(coord) || !(fabs(coord) < 1.0e15)) return false;
    const int64_t anchor = (int64_t)round(coord);
    const int64_t off = (int64_t)round(__dmul_rn(__dsub_rn((double)anchor, coord), (double)os));
    const int64_t s = anchor - 3, e = anchor + 3;
    if (s < 0 || e >= size) return false;
    const int64_t idx = off + os / 2;
    if (idx < 0 || idx >= rows) return false;
    *start = s;
    *row = (int32_t)idx;
    return true;
}

}  // namespace cr
