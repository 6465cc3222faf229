// cr_plan.cu -- per-sample planning (FP64 index selection), key sort and
// deduplication into records.
//
// The plan restates WProjector::plan_sample (gridder.rs:3588-3624) and
// StandardGridder::plan_positive_taps / sample_tap_span (gridder.rs:540-566,
// 1877-1886, 1958-1995) with the reference's FP64 rounding (round half away
// from zero), so the chosen cell, oversampling offset and w-plane are
// bit-identical to the reference's.  The decisions are taken on float32
// pairs where they lie clear of a rounding boundary (cr_fixed.cuh) and by
// the reference's FP64 operations otherwise: GB300 issues FP64 at a small
// fraction of its float32 rate, and planning was FP64-bound.  Each valid
// sample gets a 64-bit key
//   home tile | (plane | conj | offset)  or  (x tap row | y tap row) | cell
// and the keys are radix-sorted.  Samples with equal keys have identical taps;
// their weighted visibilities and weights are summed into one record, so
// every distinct tap footprint is convolved once.  The sort is stable; the
// sums of weights and the record sums are compensated float32-pair sums of
// exact products, carried in FP64 across warps.
#include <cmath>

#include "cr_fixed.cuh"
#include "cr_internal.cuh"

namespace cr {

namespace {

__host__ __device__ inline int bits_for(uint64_t max_value) {
    int b = 0;
    while ((max_value >> b) != 0) ++b;
    return b;
}

struct WpPlanArgs {
    int64_t first, n;   // samples [first, n)
    const double *u, *v, *w;
    const float *weight, *sumwt;
    const uint8_t* gridable;
    const float2* vis;
    int64_t gnx, gny;
    double du, dv, w_scale;
    int32_t sampling, planes, radius, axis;
    const int32_t* support;
    const float* norm;
    int64_t nty;
    int plane_bits, off_bits;
    DfScale kx, ky;            // 1 / du, 1 / dv as float32 pairs
    DfScale kw;                // w_scale as a float32 pair
    uint64_t* keys;
    uint32_t* vals;
    double* sums;
    unsigned long long* counts;
};

__device__ __forceinline__ double warp_sum_d(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ unsigned long long warp_sum_u(unsigned long long x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Block-wide accumulation of two FP64 sums and two counters, from values
// already summed over each warp (held by lane 0).
__device__ void block_finish(double s0, double s1, unsigned long long c0, unsigned long long c1,
                             double* sums, unsigned long long* counts) {
    __shared__ double sh_s[2][32];
    __shared__ unsigned long long sh_c[2][32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        sh_s[0][warp] = s0;
        sh_s[1][warp] = s1;
        sh_c[0][warp] = c0;
        sh_c[1][warp] = c1;
    }
    __syncthreads();
    if (warp == 0) {
        s0 = lane < nw ? sh_s[0][lane] : 0.0;
        s1 = lane < nw ? sh_s[1][lane] : 0.0;
        c0 = lane < nw ? sh_c[0][lane] : 0ull;
        c1 = lane < nw ? sh_c[1][lane] : 0ull;
        s0 = warp_sum_d(s0);
        s1 = warp_sum_d(s1);
        c0 = warp_sum_u(c0);
        c1 = warp_sum_u(c1);
        if (lane == 0) {
            if (s0 != 0.0) atomicAdd(&sums[0], s0);
            if (s1 != 0.0) atomicAdd(&sums[1], s1);
            if (c0) atomicAdd(&counts[0], c0);
            if (c1) atomicAdd(&counts[1], c1);
        }
    }
    __syncthreads();
}

// The FP64 operations kept out of line, so that the compiler branches around
// them instead of predicating them on the common path.
__device__ __noinline__ double fp64_product(float a, float b, float m) {
    return (double)m * ((double)a * (double)b);
}
__device__ __noinline__ double fp64_of(float f) { return (double)f; }

// m a b (m a power of two) into s exactly, as the pair (p, fma(a, b, -p));
// a product outside the range where that pair is exact goes to the FP64
// sum fb instead (and sets used).
__device__ __forceinline__ void add_product(PairSum& s, double& fb, bool& used, float a, float b,
                                            float m) {
    const float p = __fmul_rn(a, b);
    const float ap = fabsf(p);
    if (ap < 0x1p100f && ap > 0x1p-90f) {
        s.add(__fmul_rn(p, m), __fmul_rn(__fmaf_rn(a, b, -p), m));
    } else if (a != 0.0f && b != 0.0f) {
        fb += fp64_product(a, b, m);
        used = true;
    }
}

// float -> double from the bits (exact, no FP64 instruction); zeros keep
// their sign, subnormal, infinite and NaN values take the conversion.
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    if (e == 0u || e == 0xffu) {
        if ((u << 1) == 0u) return __longlong_as_double((long long)sign);
        return fp64_of(f);
    }
    return __longlong_as_double((long long)(sign | (unsigned long long)(e + 896u) << 52 |
                                            (unsigned long long)(u & 0x7fffffu) << 29));
}

// *p += h + l, one FP64 atomic per nonzero part
__device__ __forceinline__ void atomic_add_pair(double* p, float h, float l) {
    if (h != 0.0f) atomicAdd(p, f2d(h));
    if (l != 0.0f) atomicAdd(p, f2d(l));
}

__device__ __forceinline__ PairSum warp_sum_pair(PairSum s) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        s.add(__shfl_xor_sync(0xffffffffu, s.h, o), __shfl_xor_sync(0xffffffffu, s.l, o));
    return s;
}

// Block accumulation of two pair sums (plus their rare FP64 parts) and two
// counters: pairs summed over the warps, then over the block's warps, and
// added to the FP64 totals by their parts.
__device__ void block_accumulate(PairSum s0, PairSum s1, double f0, double f1, bool fb_used,
                                 unsigned long long c0, unsigned long long c1, double* sums,
                                 unsigned long long* counts) {
    __shared__ float4 sh_s[32];
    __shared__ unsigned long long sh_c[2][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (__any_sync(0xffffffffu, fb_used)) {
        f0 = warp_sum_d(f0);
        f1 = warp_sum_d(f1);
        if (lane == 0) {
            if (f0 != 0.0) atomicAdd(&sums[0], f0);
            if (f1 != 0.0) atomicAdd(&sums[1], f1);
        }
    }
    s0 = warp_sum_pair(s0);
    s1 = warp_sum_pair(s1);
    c0 = warp_sum_u(c0);
    c1 = warp_sum_u(c1);
    if (lane == 0) {
        sh_s[warp] = make_float4(s0.h, s0.l, s1.h, s1.l);
        sh_c[0][warp] = c0;
        sh_c[1][warp] = c1;
    }
    __syncthreads();
    if (warp == 0) {
        const float4 v = lane < nw ? sh_s[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        s0.h = v.x;
        s0.l = v.y;
        s1.h = v.z;
        s1.l = v.w;
        c0 = lane < nw ? sh_c[0][lane] : 0ull;
        c1 = lane < nw ? sh_c[1][lane] : 0ull;
        s0 = warp_sum_pair(s0);
        s1 = warp_sum_pair(s1);
        c0 = warp_sum_u(c0);
        c1 = warp_sum_u(c1);
        if (lane == 0) {
            atomic_add_pair(&sums[0], s0.h, s0.l);
            atomic_add_pair(&sums[1], s1.h, s1.l);
            if (c0) atomicAdd(&counts[0], c0);
            if (c1) atomicAdd(&counts[1], c1);
        }
    }
    __syncthreads();
}

__device__ __forceinline__ bool finite_f(float x) { return isfinite(x); }
// finiteness of a double from the exponent bits of its high half (no FP64
// instruction, no 64-bit shift)
__device__ __forceinline__ bool finite_d(double x) {
    return (((unsigned)__double2hiint(x) >> 20) & 0x7ffu) != 0x7ffu;
}

// The anchor loc = round(x) and offset round((loc - x) s) of the grid
// coordinate x = u / du + G/2 in float32 pairs (x - G/2 = p + e from one
// pair product with 1/du): the decisions of cr_fixed.cuh's fast path, taken
// only more than kDfMargin from their rounding boundaries, where they equal
// the reference's FP64 ones.  False when undecided.
__device__ __forceinline__ bool df_wp_axis(float p, float e, int64_t size, int32_t s,
                                           int64_t* loc, int64_t* off) {
    float a, dh;
    if (!df_nearest(p, e, (size & 1) ? 0.5f : 0.0f, &a, &dh)) return false;
    const float sf = (float)s;
    const float v = -__fmaf_rn(dh, sf, __fmul_rn(e, sf));
    const float o = rintf(v);
    if (!(0.5f - fabsf(__fsub_rn(v, o)) > kDfMargin)) return false;
    *loc = (size >> 1) + (int)a;
    *off = (int)o;
    return true;
}

// The plane round(sqrt(q)) (half away from zero) of q = RN(w_scale |w|)
// without the FP64 square root: the candidate from a float32 root, moved to
// the k with (k - 1/2)^2 <= q < (k + 1/2)^2 by exact FP64 products, and
// undecided (false) when q lies within 2^-40 relative of either bound,
// where the reference's rounded root could land on the half-integer.
// Planes at or above `planes` - 1 need no decision (they clamp).
__device__ __forceinline__ bool wp_plane_of(double q, int32_t planes, int32_t* plane) {
    const double top = ((double)planes - 0.5) * ((double)planes - 0.5);
    if (q >= top) {
        *plane = planes - 1;
        return true;
    }
    int k = (int)rintf(sqrtf(__double2float_rn(q)));
    auto lo = [](int j) {
        const double t = (double)j - 0.5;
        return __dmul_rn(t, t);
    };
    if (k > 0 && q < lo(k)) --k;
    else if (q >= lo(k + 1)) ++k;
    const double bl = lo(k), bh = lo(k + 1);
    if ((k > 0 && __dsub_rn(q, bl) < bl * 0x1p-40) || __dsub_rn(bh, q) < bh * 0x1p-40)
        return false;
    *plane = min(k, planes - 1);
    return true;
}

// wp_plane_of on float32 pairs: q = w_scale |w| from |w| and w_scale as
// pairs (about 2^-44 relative), the candidate from a float32 root moved to
// the k with (k - 1/2)^2 <= q < (k + 1/2)^2 (bounds exact in float32 for
// k <= 2000), and decided only when q lies more than 2^-36 of a bound from
// both, where RN64(q) and the reference's rounded root give the same k.
// False when undecided (then wp_plane_of decides on exact FP64 products).
__device__ __forceinline__ bool df_plane_of(float wh, float wl, DfScale ws, int32_t planes,
                                            int32_t* plane) {
    float qh, ql;
    df_product(fabsf(wh), fabsf(wl), ws, &qh, &ql);
    if (!(qh < 4.0e6f)) return false;
    int k = (int)rintf(sqrtf(qh));
    // q - (j - 1/2)^2 as a float: qh - b is exact when b/2 <= qh <= 2b, and
    // its sign is plain otherwise
    auto diff = [&](int j) {
        const float t = (float)j - 0.5f;
        return __fadd_rn(__fsub_rn(qh, __fmul_rn(t, t)), ql);
    };
    if (k > 0 && diff(k) < 0.0f)
        --k;
    else if (diff(k + 1) >= 0.0f)
        ++k;
    const float tl = (float)k - 0.5f, th = (float)k + 0.5f;
    if ((k > 0 && !(diff(k) > __fmul_rn(tl, tl) * 0x1p-36f)) ||
        !(-diff(k + 1) > __fmul_rn(th, th) * 0x1p-36f))
        return false;
    *plane = min(k, planes - 1);
    return true;
}

// The FP64 decisions, out of line so that the common float32-pair path
// branches around them instead of issuing them predicated.
// wp_plane_of of RN64(w_scale |w|): the plane, or -1 when undecided.
__device__ __noinline__ int wp_plane_fp64(double w_scale, double w, int32_t planes) {
    int32_t plane = 0;
    return wp_plane_of(__dmul_rn(w_scale, fabs(w)), planes, &plane) ? plane : -1;
}

struct WpDecision {
    long long lx, ly, ox, oy;
    int plane, ok;
};

// Anchors, offsets and plane in the reference's FP64 operations.
__device__ __noinline__ WpDecision wp_decide_fp64(double u, double v, double w, double du,
                                                  double dv, int64_t gnx, int64_t gny,
                                                  int32_t sampling, int32_t planes,
                                                  double w_scale) {
    WpDecision d{0, 0, 0, 0, 0, 0};
    const double px = __dadd_rn(__ddiv_rn(u, du), (double)gnx / 2.0);
    const double py = __dadd_rn(__ddiv_rn(-v, dv), (double)gny / 2.0);
    if (!(isfinite(px) && isfinite(py) && fabs(px) < 1.0e15 && fabs(py) < 1.0e15)) return d;
    d.ok = 1;
    d.lx = (long long)round(px);
    d.ly = (long long)round(py);
    d.ox = (long long)round(__dmul_rn(__dsub_rn((double)d.lx, px), (double)sampling));
    d.oy = (long long)round(__dmul_rn(__dsub_rn((double)d.ly, py), (double)sampling));
    if (planes > 1) {
        const double c = sqrt(fmax(__dmul_rn(w_scale, fabs(w)), 0.0));
        double r = round(c);
        r = fmin(fmax(r, 0.0), (double)(planes - 1));
        d.plane = (int)r;
    }
    return d;
}

// WProjector::plan_sample (gridder.rs:3588-3624) + raw_w_project_sample_is_valid
// (lib.rs:73666-73676) + w_project_accumulation_for_sample (lib.rs:71463-71470).
// The anchors, offsets and plane come from the float32-pair path above when
// it decides them, else from the reference's FP64 operations.
__global__ void __launch_bounds__(256) wp_plan_kernel(WpPlanArgs a) {
    PairSum s_norm, s_rep;
    double f_norm = 0.0, f_rep = 0.0;
    bool fb_used = false;
    unsigned long long c_ok = 0, c_skip = 0;
    const uint64_t invalid = ~0ull;
    for (int64_t i = a.first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t key = invalid;
        float wt = a.weight[i];
        float f = a.sumwt ? a.sumwt[i] : 1.0f;
        float2 vis = a.vis[i];
        double u = a.u[i], v = a.v[i], w = a.w[i];
        bool ok = (!a.gridable || a.gridable[i]) && finite_f(wt) && wt > 0.0f && finite_f(f) &&
                  f > 0.0f && finite_f(vis.x) && finite_f(vis.y) && finite_d(u) &&
                  finite_d(v) && finite_d(w);
        if (ok) {
            int64_t lx = 0, ly = 0, ox = 0, oy = 0;
            int32_t plane = 0;
            // float32 pairs first: u = uh + ul, x - G/2 = u (1/du), y - G/2 = -v (1/dv)
            float uh, ul, vh, vl;
            bool fast = df_split(u, &uh, &ul) && df_split(v, &vh, &vl);
            if (fast) {
                float px32, ex, py32, ey;
                df_product(uh, ul, a.kx, &px32, &ex);
                df_product(-vh, -vl, a.ky, &py32, &ey);
                fast = df_wp_axis(px32, ex, a.gnx, a.sampling, &lx, &ox) &&
                       df_wp_axis(py32, ey, a.gny, a.sampling, &ly, &oy);
            }
            if (fast && a.planes > 1) {
                float wh, wl;
                if (!(df_split(w, &wh, &wl) && df_plane_of(wh, wl, a.kw, a.planes, &plane))) {
                    plane = wp_plane_fp64(a.w_scale, w, a.planes);
                    fast = plane >= 0;
                }
            }
            if (!fast) {
                const WpDecision d = wp_decide_fp64(u, v, w, a.du, a.dv, a.gnx, a.gny,
                                                    a.sampling, a.planes, a.w_scale);
                ok = d.ok;
                lx = d.lx;
                ly = d.ly;
                ox = d.ox;
                oy = d.oy;
                plane = d.plane;
            }
            if (ok) {
                int64_t s = a.support[plane];
                ok = s > 0 && lx - s >= 0 && ly - s >= 0 && lx + s < a.gnx && ly + s < a.gny &&
                     ox >= -a.radius && ox <= a.radius && oy >= -a.radius && oy <= a.radius;
                if (ok) {
                    int offidx = (int)(ox + a.radius) * a.axis + (int)(oy + a.radius);
                    float nrm = a.norm[((int64_t)plane * a.axis) * a.axis + offidx];
                    // 2 w nrm and w f, exact products of floats, summed in pairs
                    add_product(s_norm, f_norm, fb_used, wt, nrm, 2.0f);
                    add_product(s_rep, f_rep, fb_used, wt, f, 1.0f);
                    // w > 0 from the bits (w is finite here)
                    const int wh32 = __double2hiint(w);
                    const uint64_t wpos = (wh32 > 0 || (wh32 == 0 && __double2loint(w) != 0)) ? 1u : 0u;
                    uint64_t tile = (uint64_t)(lx >> 5) * (uint64_t)a.nty + (uint64_t)(ly >> 5);
                    uint64_t cell = (uint64_t)(((lx & 31) << 5) | (ly & 31));
                    key = tile;
                    key = (key << a.plane_bits) | (uint64_t)plane;
                    key = (key << 1) | wpos;
                    key = (key << a.off_bits) | (uint64_t)offidx;
                    key = (key << 10) | cell;
                }
            }
        }
        if (ok)
            c_ok++;
        else
            c_skip++;
        a.keys[i] = key;
        a.vals[i] = (uint32_t)i;
    }
    block_accumulate(s_norm, s_rep, f_norm, f_rep, fb_used, c_ok, c_skip, a.sums, a.counts);
}

struct StdPlanArgs {
    int64_t first, n;   // samples [first, n)
    const double *u, *v;
    const float *weight, *sumwt;
    const uint8_t* gridable;
    int64_t gnx, gny;
    double du, dv;
    int32_t os, tap_rows;
    int64_t nty;
    DfScale kx, ky;            // 1 / du, 1 / dv as float32 pairs
    uint64_t* keys;
    uint32_t* vals;
    double* sums;
    unsigned long long* counts;
};

// sample_tap_span (gridder.rs:1976-1995): start cell and tap row.
__device__ __forceinline__ bool tap_span(double coord, int64_t size, int32_t os, int32_t rows,
                                         int64_t* start, int32_t* row) {
    if (!isfinite(coord) || !(fabs(coord) < 1.0e15)) return false;
    int64_t anchor = (int64_t)round(coord);
    int64_t off = (int64_t)round(__dmul_rn(__dsub_rn((double)anchor, coord), (double)os));
    int64_t s = anchor - 3, e = anchor + 3;
    if (s < 0 || e >= size) return false;
    int64_t idx = off + os / 2;
    if (idx < 0 || idx >= rows) return false;
    *start = s;
    *row = (int32_t)idx;
    return true;
}

struct StdSpans {
    long long x0, y0;
    int rx, ry, ok;
};

// Both axes' tap spans in the reference's FP64 operations, out of line (the
// common path takes them on float32 pairs).
__device__ __noinline__ StdSpans std_spans_fp64(double u, double v, double du, double dv,
                                                int64_t gnx, int64_t gny, int32_t os,
                                                int32_t rows) {
    StdSpans d{0, 0, 0, 0, 0};
    int64_t x0 = 0, y0 = 0;
    int32_t rx = 0, ry = 0;
    const double x = __dadd_rn(__ddiv_rn(u, du), (double)gnx / 2.0);
    const double y = __dadd_rn(__ddiv_rn(-v, dv), (double)gny / 2.0);
    d.ok = tap_span(x, gnx, os, rows, &x0, &rx) && tap_span(y, gny, os, rows, &y0, &ry);
    d.x0 = x0;
    d.y0 = y0;
    d.rx = rx;
    d.ry = ry;
    return d;
}

// accumulate_dirty_psf_and_residual_standard_streaming_grid_serial
// (lib.rs:68433-68500): validity, taps, sum of weights grid_weight = w*f.
__global__ void __launch_bounds__(256) std_plan_kernel(StdPlanArgs a) {
    PairSum s_norm;
    double f_norm = 0.0;
    unsigned long long c_ok = 0, c_skip = 0;
    for (int64_t i = a.first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t key = ~0ull;
        float wt = a.weight[i];
        float f = a.sumwt ? a.sumwt[i] : 1.0f;
        bool ok = (!a.gridable || a.gridable[i]) && finite_f(wt) && wt > 0.0f && finite_f(f) &&
                  f > 0.0f;
        if (ok) {
            int64_t x0 = 0, y0 = 0;
            int32_t rx = 0, ry = 0;
            // float32 pairs first (cr_fixed.cuh's decisions, 1 / 0 / -1 =
            // accepted / rejected / undecided), the FP64 operations otherwise
            const double u = a.u[i], v = a.v[i];
            int dx = -1, dy = -1;
            float uh, ul, vh, vl;
            if (df_split(u, &uh, &ul) && df_split(v, &vh, &vl)) {
                float px, ex, py, ey;
                df_product(uh, ul, a.kx, &px, &ex);
                df_product(-vh, -vl, a.ky, &py, &ey);
                dx = df_tap_span(px, ex, a.gnx, a.os, a.tap_rows, &x0, &rx);
                if (dx == 1) dy = df_tap_span(py, ey, a.gny, a.os, a.tap_rows, &y0, &ry);
            }
            if (dx == 0 || dy == 0) {
                ok = false;
            } else if (dx != 1 || dy != 1) {
                const StdSpans d = std_spans_fp64(u, v, a.du, a.dv, a.gnx, a.gny, a.os,
                                                  a.tap_rows);
                ok = d.ok;
                x0 = d.x0;
                y0 = d.y0;
                rx = d.rx;
                ry = d.ry;
            }
            if (ok) {
                // the float32 product w f, as the reference sums it
                s_norm.add(__fmul_rn(wt, f), 0.0f);
                uint64_t tile = (uint64_t)(x0 >> 5) * (uint64_t)a.nty + (uint64_t)(y0 >> 5);
                uint64_t cell = (uint64_t)(((x0 & 31) << 5) | (y0 & 31));
                key = (((tile << 8 | (uint64_t)rx) << 8 | (uint64_t)ry) << 10) | cell;
            }
        }
        if (ok)
            c_ok++;
        else
            c_skip++;
        a.keys[i] = key;
        a.vals[i] = (uint32_t)i;
    }
    block_accumulate(s_norm, s_norm, f_norm, f_norm, false, c_ok, c_skip, a.sums, a.counts);
}

__global__ void head_flags(const uint64_t* keys, const unsigned long long* counts, int64_t n,
                           uint32_t* flags) {
    int64_t nv = (int64_t)counts[0];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        flags[i] = (i < nv && (i == 0 || keys[i] != keys[i - 1])) ? 1u : 0u;
}

struct RecArgs {
    const uint64_t* keys;
    const uint32_t* vals;
    const uint32_t* flags;
    const uint32_t* excl;
    const unsigned long long* counts;
    int64_t n;
    int mode;  // 0 wproj, 1 standard
    int plane_bits, off_bits;
    int64_t nty;
    int32_t *rx, *ry, *ra, *rb, *rconj;
    double2* vsum;
    double* wsum;
    int32_t* sample_rec;
    const float* weight;
    const float* sumwt;
    const float2* vis;
    uint32_t* tile_of;
    const int32_t* support;   // per plane (W-projection); null: 7 x 7 standard taps
};

// Record fields decoded from the head key of each run.
// Also counts the taps one grid pass applies (counts[3]).
__global__ void records_init(RecArgs a) {
    int64_t nv = (int64_t)a.counts[0];
    unsigned long long taps = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (!a.flags[i]) continue;
        uint32_t r = a.excl[i];
        uint64_t k = a.keys[i];
        int cx = (int)((k >> 5) & 31), cy = (int)(k & 31);
        k >>= 10;
        uint64_t tile;
        if (a.mode == 0) {
            a.rb[r] = (int32_t)(k & ((1ull << a.off_bits) - 1));
            k >>= a.off_bits;
            a.rconj[r] = (int32_t)(k & 1);
            k >>= 1;
            a.ra[r] = (int32_t)(k & ((1ull << a.plane_bits) - 1));
            k >>= a.plane_bits;
            tile = k;
        } else {
            a.rb[r] = (int32_t)(k & 255);
            a.ra[r] = (int32_t)((k >> 8) & 255);
            a.rconj[r] = 0;
            tile = k >> 16;
        }
        a.tile_of[r] = (uint32_t)tile;
        a.rx[r] = (int32_t)((tile / (uint64_t)a.nty) * 32 + cx);
        a.ry[r] = (int32_t)((tile % (uint64_t)a.nty) * 32 + cy);
        a.vsum[r] = make_double2(0.0, 0.0);
        a.wsum[r] = 0.0;
        const unsigned long long side =
            a.support ? 2ull * (unsigned long long)a.support[a.ra[r]] + 1ull : 7ull;
        taps += side * side;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) taps += __shfl_xor_sync(0xffffffffu, taps, o);
    if ((threadIdx.x & 31) == 0 && taps)
        atomicAdd(const_cast<unsigned long long*>(&a.counts[3]), taps);
}

// Sums of weight * vis per record: a warp-level segmented reduction over the
// sorted run in float32 pairs, then one FP64 atomic per segment piece.
__global__ void records_accumulate(RecArgs a) {
    int64_t nv = (int64_t)a.counts[0];
    const int lane = threadIdx.x & 31;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t limit = ((nv + 31) / 32) * 32;
    for (int64_t i = start; i < limit; i += stride) {
        bool valid = i < nv;
        int32_t r = -1;
        // w vis and w as float32 pairs: the products of two floats exact,
        // the segment sums compensated (FP64 only for the per-segment atomics)
        PairSum vr, vi, ww;
        if (valid) {
            r = (int32_t)(a.flags[i] ? a.excl[i] : a.excl[i] - 1);
            uint32_t s = a.vals[i];
            a.sample_rec[s] = r;
            float wt = a.weight[s];
            float f = a.sumwt ? a.sumwt[s] : 1.0f;
            float gw = a.mode == 0 ? wt : wt * f;
            float2 v = a.vis[s];
            ww.h = gw;
            if (isfinite(v.x) && isfinite(v.y)) {
                vr.h = __fmul_rn(v.x, gw);
                vr.l = __fmaf_rn(v.x, gw, -vr.h);
                vi.h = __fmul_rn(v.y, gw);
                vi.l = __fmaf_rn(v.y, gw, -vi.h);
            }
        }
        // segmented inclusive scan by record id
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float trh = __shfl_up_sync(0xffffffffu, vr.h, o);
            const float trl = __shfl_up_sync(0xffffffffu, vr.l, o);
            const float tih = __shfl_up_sync(0xffffffffu, vi.h, o);
            const float til = __shfl_up_sync(0xffffffffu, vi.l, o);
            const float twh = __shfl_up_sync(0xffffffffu, ww.h, o);
            const float twl = __shfl_up_sync(0xffffffffu, ww.l, o);
            int32_t rr = __shfl_up_sync(0xffffffffu, r, o);
            if (lane >= o && rr == r) {
                vr.add(trh, trl);
                vi.add(tih, til);
                ww.add(twh, twl);
            }
        }
        int32_t next = __shfl_down_sync(0xffffffffu, r, 1);
        bool last = (lane == 31) || (next != r);
        if (valid && last) {
            atomic_add_pair(&a.vsum[r].x, vr.h, vr.l);
            atomic_add_pair(&a.vsum[r].y, vi.h, vi.l);
            atomic_add_pair(&a.wsum[r], ww.h, ww.l);
        }
    }
}

__global__ void fill_u32(uint32_t* p, int64_t n, const unsigned long long* value) {
    uint32_t v = (uint32_t)*value;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// tile_start[t] = first record whose home tile is >= t.
__global__ void tile_starts(const uint32_t* tile_of, const unsigned long long* counts,
                            uint32_t* start) {
    int64_t nr = (int64_t)counts[2];
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nr;
         r += (int64_t)gridDim.x * blockDim.x) {
        int64_t prev = r == 0 ? -1 : (int64_t)tile_of[r - 1];
        int64_t cur = tile_of[r];
        for (int64_t t = prev + 1; t <= cur; ++t) start[t] = (uint32_t)r;
    }
}

// The plan kernels' grids: one resident wave (4 blocks of 256 per SM), each
// thread striding over many samples, so that the block reduction of the
// sums is paid once per thread rather than once per sample.
inline int64_t plan_wave(cr_ctx* ctx) { return (int64_t)ctx->sms * 4; }

// fn(lo, hi) over the batch's samples: once over all of them, or piece by
// piece for a staged upload, each after the main stream has waited for its
// copies (the last wait also orders every later use of the batch)
template <typename F>
void for_each_piece(cr_ctx* ctx, const DeviceBatch& b, F fn) {
    if (b.nchunks == 0) {
        fn(0, b.n);
        return;
    }
    int64_t lo = 0;
    for (int k = 0; k < b.nchunks; ++k) {
        CR_CUDA_CHECK(cudaStreamWaitEvent(ctx->stream, b.stage_ev[k], 0));
        if (b.chunk_end[k] > lo) fn(lo, b.chunk_end[k]);
        lo = b.chunk_end[k];
    }
}

Records allocate_records(cr_ctx* ctx, int64_t n, int64_t ntx, int64_t nty, Pool* pool) {
    Records r;
    size_t nn = (size_t)(n > 0 ? n : 1);
    r.n_samples = n;
    r.ntx = ntx;
    r.nty = nty;
    Pool& P = pool ? *pool : ctx->ws;
    auto A = [&](const char* name, size_t bytes) { return pool_alloc(ctx, P, name, bytes); };
    // keys and order are needed only while planning: always context workspaces
    r.keys = (uint64_t*)workspace(ctx, "rec_keys", nn * 8);
    r.order = (uint32_t*)workspace(ctx, "rec_order", nn * 4);
    r.sample_rec = (int32_t*)A("rec_sample", nn * 4);
    r.rec_x = (int32_t*)A("rec_x", nn * 4);
    r.rec_y = (int32_t*)A("rec_y", nn * 4);
    r.rec_a = (int32_t*)A("rec_a", nn * 4);
    r.rec_b = (int32_t*)A("rec_b", nn * 4);
    r.rec_conj = (int32_t*)A("rec_conj", nn * 4);
    r.rec_vsum = (double2*)A("rec_vsum", nn * 16);
    r.rec_wsum = (double*)A("rec_wsum", nn * 8);
    r.rec_pred = (float2*)A("rec_pred", nn * 8);
    r.tile_start = (uint32_t*)A("rec_tile_start", (size_t)(ntx * nty + 1) * 4);
    r.counts = (unsigned long long*)A("rec_counts", 4 * 8);
    r.sums = (double*)A("rec_sums", 2 * 8);
    CR_CUDA_CHECK(cudaMemsetAsync(r.counts, 0, 4 * 8, ctx->stream));
    CR_CUDA_CHECK(cudaMemsetAsync(r.sums, 0, 2 * 8, ctx->stream));
    CR_CUDA_CHECK(cudaMemsetAsync(r.sample_rec, 0xFF, nn * 4, ctx->stream));
    return r;
}

void finish_records(cr_ctx* ctx, Records& r, int mode, int key_bits, int plane_bits,
                    int off_bits, const DeviceBatch& b, const int32_t* support) {
    const int64_t n = r.n_samples;
    const unsigned T = 256;
    radix_sort_pairs(ctx, r.keys, r.order, n, key_bits);
    size_t nn = (size_t)(n > 0 ? n : 1);
    uint32_t* flags = (uint32_t*)workspace(ctx, "rec_flags", nn * 4);
    uint32_t* excl = (uint32_t*)workspace(ctx, "rec_excl", nn * 4);
    uint32_t* tile_of = (uint32_t*)workspace(ctx, "rec_tile_of", nn * 4);
    if (n > 0) {
        head_flags<<<grid_blocks(n, T), T, 0, ctx->stream>>>(r.keys, r.counts, n, flags);
        note_launch(ctx, "head_flags");
    }
    exclusive_scan_u32(ctx, flags, excl, n, r.counts + 2);
    RecArgs a{r.keys, r.order, flags, excl, r.counts, n, mode, plane_bits, off_bits, r.nty,
              r.rec_x, r.rec_y, r.rec_a, r.rec_b, r.rec_conj, r.rec_vsum, r.rec_wsum,
              r.sample_rec, b.weight, b.sumwt_factor, b.vis, tile_of, support};
    if (n > 0) {
        records_init<<<grid_blocks(n, T), T, 0, ctx->stream>>>(a);
        note_launch(ctx, "records_init");
        records_accumulate<<<grid_blocks(n, T), T, 0, ctx->stream>>>(a);
        note_launch(ctx, "records_accumulate");
    }
    int64_t ntiles = r.ntx * r.nty;
    fill_u32<<<grid_blocks(ntiles + 1, T), T, 0, ctx->stream>>>(r.tile_start, ntiles + 1,
                                                                 r.counts + 2);
    note_launch(ctx, "fill_u32");
    if (n > 0) {
        tile_starts<<<grid_blocks(n, T), T, 0, ctx->stream>>>(tile_of, r.counts, r.tile_start);
        note_launch(ctx, "tile_starts");
    }
}

}  // namespace

Records plan_wproj(cr_ctx* ctx, cr_wproj* wp, const DeviceBatch& b, Pool* pool) {
    const cr_grid_info& gi = wp->g->info;
    int64_t ntx = (gi.grid_nx + kTile - 1) / kTile, nty = (gi.grid_ny + kTile - 1) / kTile;
    Records r = allocate_records(ctx, b.n, ntx, nty, pool);
    int tile_bits = bits_for((uint64_t)(ntx * nty));
    int plane_bits = bits_for((uint64_t)(wp->info.planes > 1 ? wp->info.planes - 1 : 1));
    int off_bits = bits_for((uint64_t)(wp->axis * wp->axis - 1));
    int key_bits = tile_bits + plane_bits + 1 + off_bits + 10;
    if (key_bits > 64) fail(CR_INVALID, "grid too large for the 64-bit sample key");
    if (b.n > 0) {
        WpPlanArgs a{0, b.n, b.u, b.v, b.w, b.weight, b.sumwt_factor, b.gridable, b.vis,
                     gi.grid_nx, gi.grid_ny, gi.du, gi.dv, wp->info.w_scale,
                     wp->info.sampling, wp->info.planes, wp->radius, wp->axis,
                     wp->support_d, wp->norm_d, nty, plane_bits, off_bits,
                     df_scale_of(1.0, gi.du, false), df_scale_of(1.0, gi.dv, false),
                     df_scale_of(wp->info.w_scale, 1.0, true), r.keys,
                     r.order, r.sums, r.counts};
        for_each_piece(ctx, b, [&](int64_t lo, int64_t hi) {
            a.first = lo;
            a.n = hi;
            wp_plan_kernel<<<grid_blocks(hi - lo, 256, plan_wave(ctx)), 256, 0, ctx->stream>>>(a);
            note_launch(ctx, "wp_plan_kernel");
        });
    }
    finish_records(ctx, r, 0, key_bits, plane_bits, off_bits, b, wp->support_d);
    return r;
}

Records plan_standard(cr_ctx* ctx, cr_gridder* g, const DeviceBatch& b, Pool* pool) {
    const cr_grid_info& gi = g->info;
    int64_t ntx = (gi.grid_nx + kTile - 1) / kTile, nty = (gi.grid_ny + kTile - 1) / kTile;
    Records r = allocate_records(ctx, b.n, ntx, nty, pool);
    int tile_bits = bits_for((uint64_t)(ntx * nty));
    int key_bits = tile_bits + 16 + 10;
    if (key_bits > 64) fail(CR_INVALID, "grid too large for the 64-bit sample key");
    if (b.n > 0) {
        StdPlanArgs a{0, b.n, b.u, b.v, b.weight, b.sumwt_factor, b.gridable, gi.grid_nx,
                      gi.grid_ny, gi.du, gi.dv, gi.oversampling, g->tap_rows, nty,
                      df_scale_of(1.0, gi.du, false), df_scale_of(1.0, gi.dv, false), r.keys,
                      r.order, r.sums, r.counts};
        for_each_piece(ctx, b, [&](int64_t lo, int64_t hi) {
            a.first = lo;
            a.n = hi;
            std_plan_kernel<<<grid_blocks(hi - lo, 256, plan_wave(ctx)), 256, 0, ctx->stream>>>(a);
            note_launch(ctx, "std_plan_kernel");
        });
    }
    finish_records(ctx, r, 1, key_bits, 0, 0, b, nullptr);
    return r;
}

void read_sums(cr_ctx* ctx, const Records& r, cr_sums* out) {
    if (!out) return;
    struct {
        unsigned long long c[4];
        double s[2];
    }* host = (decltype(host))ctx->pinned;
    CR_CUDA_CHECK(cudaMemcpyAsync(host->c, r.counts, 32, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaMemcpyAsync(host->s, r.sums, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    out->gridded = (int64_t)host->c[0];
    out->skipped = (int64_t)host->c[1];
    out->unique_records = (int64_t)host->c[2];
    out->taps = (int64_t)host->c[3];
    out->normalization_sumwt = host->s[0];
    out->reported_sumwt = host->s[1];
}

}  // namespace cr
