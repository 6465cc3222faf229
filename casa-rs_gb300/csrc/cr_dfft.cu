// cr_dfft.cu -- the image stage's centred transforms in float-pair arithmetic.
//
// The dirty-product stage of the reference runs its centred FFTs in FP64
// (fft.rs:600-630 on Complex64 grids; DirtyProductFftPolicy's default,
// lib.rs:2435-2445): the grid correction 1/grdsf amplifies transform rounding
// near the image edge, so float32 transforms miss the 1e-5 image bar there.
// GB300 runs FP64 at a small fraction of its float32 rate, which made the
// two 5000^2 FP64 transforms of a W-projection dirty image a third of the
// end-to-end call.  These kernels compute the same transforms with every
// value held as an unevaluated sum of two floats (hi + lo, about 48
// significant bits): Knuth's two-sum and Dekker's product with a fused
// multiply-add give each addition and multiplication with an error of about
// 2^-44 of its operands, far below what the final float32 image keeps.
//
// One 2-D transform is two passes of 1-D transforms, one line per block, the
// line held in shared memory: an in-place mixed-radix decimation-in-time
// transform (radices 4, 2, 3, 5: the grids are even and 5-smooth, the
// composite padding of gridder.rs:4152-4173) over an input loaded in
// digit-reversed order, twiddles from a per-length table of
// exp(2 pi i k / N) split into float pairs on the host.
//   grid -> image: columns first (half of the grid's columns, only the
//     image's rows kept), then the image's rows, two to a line, whose output
//     goes straight through the crop and correction of crop_correct_body;
//   image -> grid: the image's rows first, two to a line (the apodised
//     image is zero outside them), then half of the grid's columns, written
//     with their mirror images as the float32 grid.
// The centring is the checkerboard modulation of cr_fft.cu.
#include <cmath>
#include <memory>
#include <vector>

#include "cr_internal.cuh"

namespace cr {

struct DfPlan {
    int32_t n = 0, ns = 0;
    int32_t radix[16] = {};
    int32_t* src = nullptr;   // [n] input index loaded at each position
    float4* tw = nullptr;     // [n] exp(+2 pi i k / n) as (cos hi, cos lo, sin hi, sin lo)
    ~DfPlan() {
        cudaFree(src);
        cudaFree(tw);
    }
};

namespace {

constexpr int kDfThreads = 512;
constexpr int kDfMaxStages = 16;
// lines up to this length fit one block's shared memory (16 bytes a point)
constexpr int64_t kDfMaxN = 13824;

struct DfStages {
    int32_t n, ns;
    int32_t radix[kDfMaxStages];
};

struct DfConsts {
    float c1h, c1l, c2h, c2l;   // cos(2 pi / 5), cos(4 pi / 5)
    float s1h, s1l, s2h, s2l;   // sin(2 pi / 5), sin(4 pi / 5)
    float s3h, s3l;             // sin(2 pi / 3)
};

struct dd {
    float h, l;
};
struct cdd {
    dd re, im;
};

// s + e = a + b exactly (Knuth); quick form when |a| >= |b| (Dekker)
__device__ __forceinline__ dd two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ dd quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dd dadd(dd a, dd b) {
    const dd s = two_sum(a.h, b.h);
    return quick_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dd dneg(dd a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dd dsub(dd a, dd b) { return dadd(a, dneg(b)); }
// the product's rounding error from one fused multiply-add (Dekker's product)
__device__ __forceinline__ dd dmul(dd a, dd b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return quick_two_sum(p, e);
}

__device__ __forceinline__ cdd cadd(cdd a, cdd b) { return {dadd(a.re, b.re), dadd(a.im, b.im)}; }
__device__ __forceinline__ cdd csub(cdd a, cdd b) { return {dsub(a.re, b.re), dsub(a.im, b.im)}; }
// a b + sgn c d as one float pair: the two products' high parts are summed
// exactly, their rounding errors and cross terms gathered by fused
// multiply-adds into one correction
__device__ __forceinline__ dd dot2(dd a, dd b, dd c, dd d, float sgn) {
    const float p = __fmul_rn(a.h, b.h), q = sgn * __fmul_rn(c.h, d.h);
    float t = __fmaf_rn(a.h, b.h, -p);
    t = __fmaf_rn(a.h, b.l, t);
    t = __fmaf_rn(a.l, b.h, t);
    t = __fmaf_rn(sgn, __fmaf_rn(c.h, d.h, -sgn * q), t);
    t = __fmaf_rn(sgn * c.h, d.l, t);
    t = __fmaf_rn(sgn * c.l, d.h, t);
    const dd s = two_sum(p, q);
    return quick_two_sum(s.h, __fadd_rn(s.l, t));
}
__device__ __forceinline__ cdd cmul(cdd a, cdd b) {
    return {dot2(a.re, b.re, a.im, b.im, -1.0f), dot2(a.re, b.im, a.im, b.re, 1.0f)};
}
__device__ __forceinline__ cdd cscale(cdd a, dd c) { return {dmul(a.re, c), dmul(a.im, c)}; }
// times +i for the inverse transform, -i for the forward one
template <bool INV>
__device__ __forceinline__ cdd mul_i(cdd a) {
    return INV ? cdd{dneg(a.im), a.re} : cdd{a.im, dneg(a.re)};
}

__device__ __forceinline__ cdd ld(const float4* sm, int i) {
    const float4 v = sm[i];
    return {{v.x, v.y}, {v.z, v.w}};
}
__device__ __forceinline__ void st(float4* sm, int i, cdd a) {
    sm[i] = make_float4(a.re.h, a.re.l, a.im.h, a.im.l);
}
template <bool INV>
__device__ __forceinline__ cdd twiddle(const float4* tw, int k) {
    const float4 v = __ldg(tw + k);
    return INV ? cdd{{v.x, v.y}, {v.z, v.w}} : cdd{{v.x, v.y}, {-v.z, -v.w}};
}

// Butterflies of stage span m at base: inputs base + q m, the q-th times
// W^(q k) (k = j N / L), then a DFT of the radix with the transform's sign.
template <bool INV>
__device__ __forceinline__ void bfly2(float4* sm, int base, int m, int k, const float4* tw) {
    const cdd x0 = ld(sm, base);
    cdd x1 = ld(sm, base + m);
    if (k) x1 = cmul(x1, twiddle<INV>(tw, k));
    st(sm, base, cadd(x0, x1));
    st(sm, base + m, csub(x0, x1));
}

template <bool INV>
__device__ __forceinline__ void bfly3(float4* sm, int base, int m, int k, const float4* tw,
                                      const DfConsts& c) {
    const cdd x0 = ld(sm, base);
    cdd x1 = ld(sm, base + m), x2 = ld(sm, base + 2 * m);
    if (k) {
        x1 = cmul(x1, twiddle<INV>(tw, k));
        x2 = cmul(x2, twiddle<INV>(tw, 2 * k));
    }
    const cdd t1 = cadd(x1, x2), t2 = csub(x1, x2);
    const cdd half{{0.5f * t1.re.h, 0.5f * t1.re.l}, {0.5f * t1.im.h, 0.5f * t1.im.l}};
    const cdd a = csub(x0, half);
    const cdd b = mul_i<INV>(cscale(t2, dd{c.s3h, c.s3l}));
    st(sm, base, cadd(x0, t1));
    st(sm, base + m, cadd(a, b));
    st(sm, base + 2 * m, csub(a, b));
}

template <bool INV>
__device__ __forceinline__ void bfly4(float4* sm, int base, int m, int k, const float4* tw) {
    cdd x0 = ld(sm, base), x1 = ld(sm, base + m), x2 = ld(sm, base + 2 * m),
        x3 = ld(sm, base + 3 * m);
    if (k) {
        x1 = cmul(x1, twiddle<INV>(tw, k));
        x2 = cmul(x2, twiddle<INV>(tw, 2 * k));
        x3 = cmul(x3, twiddle<INV>(tw, 3 * k));
    }
    const cdd t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3);
    const cdd t3 = mul_i<INV>(csub(x1, x3));
    st(sm, base, cadd(t0, t2));
    st(sm, base + m, cadd(t1, t3));
    st(sm, base + 2 * m, csub(t0, t2));
    st(sm, base + 3 * m, csub(t1, t3));
}

template <bool INV>
__device__ __forceinline__ void bfly5(float4* sm, int base, int m, int k, const float4* tw,
                                      const DfConsts& c) {
    const cdd x0 = ld(sm, base);
    cdd x1 = ld(sm, base + m), x2 = ld(sm, base + 2 * m), x3 = ld(sm, base + 3 * m),
        x4 = ld(sm, base + 4 * m);
    if (k) {
        x1 = cmul(x1, twiddle<INV>(tw, k));
        x2 = cmul(x2, twiddle<INV>(tw, 2 * k));
        x3 = cmul(x3, twiddle<INV>(tw, 3 * k));
        x4 = cmul(x4, twiddle<INV>(tw, 4 * k));
    }
    const dd c1{c.c1h, c.c1l}, c2{c.c2h, c.c2l}, s1{c.s1h, c.s1l}, s2{c.s2h, c.s2l};
    const cdd t1 = cadd(x1, x4), t2 = cadd(x2, x3), t3 = csub(x1, x4), t4 = csub(x2, x3);
    const cdd a1 = cadd(x0, cadd(cscale(t1, c1), cscale(t2, c2)));
    const cdd a2 = cadd(x0, cadd(cscale(t1, c2), cscale(t2, c1)));
    const cdd b1 = mul_i<INV>(cadd(cscale(t3, s1), cscale(t4, s2)));
    const cdd b2 = mul_i<INV>(csub(cscale(t3, s2), cscale(t4, s1)));
    st(sm, base, cadd(x0, cadd(t1, t2)));
    st(sm, base + m, cadd(a1, b1));
    st(sm, base + 2 * m, cadd(a2, b2));
    st(sm, base + 3 * m, csub(a2, b2));
    st(sm, base + 4 * m, csub(a1, b1));
}

// The line in sm (loaded in digit-reversed order) to its transform, in place.
template <bool INV>
__device__ void line_transform(float4* sm, const DfStages& s, const float4* tw,
                               const DfConsts& c) {
    const int n = s.n;
    int m = 1;
    for (int k = 0; k < s.ns; ++k) {
        const int r = s.radix[k], L = m * r, tstep = n / L, nb = n / r;
        for (int beta = threadIdx.x; beta < nb; beta += blockDim.x) {
            const int j = beta % m, base = (beta / m) * L + j, kk = j * tstep;
            if (r == 4)
                bfly4<INV>(sm, base, m, kk, tw);
            else if (r == 5)
                bfly5<INV>(sm, base, m, kk, tw, c);
            else if (r == 2)
                bfly2<INV>(sm, base, m, kk, tw);
            else
                bfly3<INV>(sm, base, m, kk, tw, c);
        }
        __syncthreads();
        m = L;
    }
}

// Only real images leave and enter these transforms, so each works on half
// of the spectrum.  With gnx and gny even, negating both indices keeps the
// checkerboard's sign, and with g' the modulated grid:
//   grid -> image: the real part of the inverse transform of g' is the
//     inverse transform of its Hermitian part h(x, y) = (g'(x, y) +
//     conj(g'(-x, -y))) / 2.  After the pass along x, column -y of h is the
//     conjugate of column y, so only columns 0..gny/2 are transformed, and
//     each image row is the real transform of a Hermitian line: two image
//     rows r1, r2 go through one complex line as r1 + i r2.
//   image -> grid: two real image rows go through one complex line as
//     m1 + i m2 and are separated by the same symmetry (columns 0..gny/2
//     kept); then columns 0..gny/2 are transformed along x and column -y
//     written as the conjugate of column y.
// The halves h, (Z + conj(Z')) / 2 are float-pair operations; h itself is
// exact (a two-sum halved).

// grid -> image, pass 1: column y (0 <= y <= gny/2) of h transformed along
// x; the image's rows [bx0, bx0 + nx) kept in t[(x - bx0) gnyh + y].
__global__ void __launch_bounds__(kDfThreads, 2) dfft_inv_cols(
    const float2* grid, const float* real_grid, int64_t gnx, int64_t gny, int64_t gnyh,
    int64_t bx0, int32_t nx, const int32_t* src, const float4* tw, DfStages s, DfConsts c,
    float4* t) {
    extern __shared__ float4 sm[];
    const int64_t y = blockIdx.x, ym = y ? gny - y : 0;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) {
        const int64_t x = src[i], xm = x ? gnx - x : 0;
        float ar, ai = 0.0f, br, bi = 0.0f;
        if (real_grid) {
            ar = real_grid[x * gny + y];
            br = real_grid[xm * gny + ym];
        } else {
            const float2 a = grid[x * gny + y], b = grid[xm * gny + ym];
            ar = a.x;
            ai = a.y;
            br = b.x;
            bi = b.y;
        }
        const dd re = two_sum(ar, br), im = two_sum(ai, -bi);
        const float h = ((x + y) & 1) ? -0.5f : 0.5f;
        sm[i] = make_float4(h * re.h, h * re.l, h * im.h, h * im.l);
    }
    __syncthreads();
    line_transform<true>(sm, s, tw, c);
    for (int xr = threadIdx.x; xr < nx; xr += blockDim.x) t[xr * gnyh + y] = sm[bx0 + xr];
}

// grid -> image, pass 2: image rows 2b and 2b + 1 as one Hermitian-extended
// line r1 + i r2 transformed along y (the real part is row 2b, the imaginary
// part row 2b + 1), then the crop and correction of crop_correct_body (the
// same operations on the FP64 value).
__global__ void __launch_bounds__(kDfThreads, 2) dfft_inv_rows(
    const float4* t, int64_t gny, int64_t gnyh, int32_t nx, int32_t ny, int64_t bx0,
    int64_t by0, int parity, double scale, const float* corr_x, const float* corr_y,
    const float* sx, const float* sy, int sinc_mode, const int32_t* src, const float4* tw,
    DfStages s, DfConsts c, float* image) {
    extern __shared__ float4 sm[];
    const int64_t xr0 = 2 * (int64_t)blockIdx.x;
    const bool two = xr0 + 1 < nx;
    const float4* row1 = t + xr0 * gnyh;
    const float4* row2 = row1 + gnyh;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) {
        const int64_t y = src[i];
        const bool lower = y < gnyh;
        const int64_t yy = lower ? y : gny - y;
        const float4 a = row1[yy];
        const float4 b = two ? row2[yy] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        // r1 + i r2 with r(-y) = conj(r(y)) for the upper half
        const dd ar{a.x, a.y}, ai{a.z, a.w}, br{b.x, b.y}, bi{b.z, b.w};
        const dd zr = lower ? dsub(ar, bi) : dadd(ar, bi);
        const dd zi = lower ? dadd(ai, br) : dsub(br, ai);
        sm[i] = make_float4(zr.h, zr.l, zi.h, zi.l);
    }
    __syncthreads();
    line_transform<true>(sm, s, tw, c);
    // the scale as a float pair: the product's high part is the float32
    // value (float)(r * scale) of the FP64 path, but for ties at half an ulp
    const float sh = (float)scale;
    const dd sc{sh, (float)(scale - (double)sh)};
    for (int k = threadIdx.x; k < (two ? 2 * ny : ny); k += blockDim.x) {
        const int q = k >= ny;
        const int64_t yr = k - q * ny, gy = by0 + yr, xr = xr0 + q, gx = bx0 + xr;
        const float4 w = sm[gy];
        dd r = q ? dd{w.z, w.w} : dd{w.x, w.y};
        if ((gx + gy + parity) & 1) r = dneg(r);
        float v = dmul(r, sc).h;
        const float factor = __fmul_rn(corr_x[gx], corr_y[gy]);
        if (sinc_mode == 1) {
            const float sf = __fmul_rn(sx[gx], sy[gy]);
            v = fabsf(sf) > 1.0e-6f ? v * (factor / sf) : 0.0f;
        } else if (sinc_mode == 2) {
            v = v * __fmul_rn(__fmul_rn(factor, sx[gx]), sy[gy]);
        } else {
            v = v * factor;
        }
        image[xr * ny + yr] = v;
    }
}

// image -> grid, pass 1: rows 2b and 2b + 1 of the apodised, modulated model
// (zero outside the image's columns) as one line m1 + i m2 transformed along
// y, separated into each row's half spectrum t[xr gnyh + y], y <= gny/2.
__global__ void __launch_bounds__(kDfThreads, 2) dfft_fwd_rows(
    const float* model, int32_t nx, int32_t ny, int64_t gny, int64_t gnyh, int64_t bx0,
    int64_t by0, const float* corr_x, const float* corr_y, const float* sinc_x,
    const float* sinc_y, const int32_t* src, const float4* tw, DfStages s, DfConsts c,
    float4* t) {
    extern __shared__ float4 sm[];
    const int64_t xr0 = 2 * (int64_t)blockIdx.x, gx0 = bx0 + xr0;
    const bool two = xr0 + 1 < nx;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) {
        const int64_t gy = src[i];
        float v[2] = {0.0f, 0.0f};
        if (gy >= by0 && gy < by0 + ny) {
            for (int q = 0; q < (two ? 2 : 1); ++q) {
                const int64_t gx = gx0 + q;
                // apodize_body's operations
                float f = __fmul_rn(corr_x[gx], corr_y[gy]);
                if (sinc_x) f = __fmul_rn(__fmul_rn(f, sinc_x[gx]), sinc_y[gy]);
                float u = model[(xr0 + q) * ny + (gy - by0)] * f;
                if ((gx + gy) & 1) u = -u;
                v[q] = u;
            }
        }
        sm[i] = make_float4(v[0], 0.0f, v[1], 0.0f);
    }
    __syncthreads();
    line_transform<false>(sm, s, tw, c);
    float4* row1 = t + xr0 * gnyh;
    for (int k = threadIdx.x; k < (two ? 2 * gnyh : gnyh); k += blockDim.x) {
        const int q = k >= gnyh;
        const int64_t y = k - q * gnyh;
        const float4 a = sm[y], b = sm[y ? gny - y : 0];
        const dd ar{a.x, a.y}, ai{a.z, a.w}, br{b.x, b.y}, bi{b.z, b.w};
        // row 1: (Z(y) + conj(Z(-y))) / 2; row 2: (Z(y) - conj(Z(-y))) / 2i
        const dd re = q ? dadd(ai, bi) : dadd(ar, br);
        const dd im = q ? dsub(br, ar) : dsub(ai, bi);
        row1[q * gnyh + y] = make_float4(0.5f * re.h, 0.5f * re.l, 0.5f * im.h, 0.5f * im.l);
    }
}

// image -> grid, pass 2: column y (0 <= y <= gny/2) transformed along x
// (rows outside [bx0, bx0 + nx) are zero), the output checkerboard, float32
// grid; column -y written as the conjugate of column y at -x.
__global__ void __launch_bounds__(kDfThreads, 2) dfft_fwd_cols(
    const float4* t, int64_t gny, int64_t gnyh, int32_t nx, int64_t bx0, int parity,
    const int32_t* src, const float4* tw, DfStages s, DfConsts c, float2* grid) {
    extern __shared__ float4 sm[];
    const int64_t y = blockIdx.x;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) {
        const int64_t x = src[i];
        sm[i] = (x >= bx0 && x < bx0 + nx) ? t[(x - bx0) * gnyh + y]
                                           : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncthreads();
    line_transform<false>(sm, s, tw, c);
    const bool mirror = y != 0 && y != gnyh - 1;
    for (int x = threadIdx.x; x < s.n; x += blockDim.x) {
        const float4 w = sm[x];
        // the pairs are normalised: the high part is the float32 value
        float re = w.x, im = w.z;
        if ((x + y + parity) & 1) {
            re = -re;
            im = -im;
        }
        grid[(int64_t)x * gny + y] = make_float2(re, im);
        if (mirror) grid[(int64_t)(x ? s.n - x : 0) * gny + (gny - y)] = make_float2(re, -im);
    }
}

void split(double v, float* h, float* l) {
    *h = (float)v;
    *l = (float)(v - (double)*h);
}

DfConsts consts() {
    const double pi = 3.14159265358979323846;
    DfConsts c;
    split(std::cos(2.0 * pi / 5.0), &c.c1h, &c.c1l);
    split(std::cos(4.0 * pi / 5.0), &c.c2h, &c.c2l);
    split(std::sin(2.0 * pi / 5.0), &c.s1h, &c.s1l);
    split(std::sin(4.0 * pi / 5.0), &c.s2h, &c.s2l);
    split(std::sqrt(3.0) / 2.0, &c.s3h, &c.s3l);
    return c;
}

// Radices for n (4s first, then 2, 3, 5); empty when n has another factor.
std::vector<int32_t> radices(int64_t n) {
    std::vector<int32_t> r;
    while (n % 4 == 0) {
        r.push_back(4);
        n /= 4;
    }
    for (int32_t f : {2, 3, 5})
        while (n % f == 0) {
            r.push_back(f);
            n /= f;
        }
    if (n != 1) r.clear();
    return r;
}

const DfPlan& plan_for(cr_ctx* ctx, int64_t n) {
    auto it = ctx->df_plans.find(n);
    if (it != ctx->df_plans.end()) return *it->second;
    const std::vector<int32_t> r = radices(n);
    if (r.empty() || (int)r.size() > kDfMaxStages) fail(CR_INVALID, "no float-pair plan");
    auto p = std::make_shared<DfPlan>();
    p->n = (int32_t)n;
    p->ns = (int32_t)r.size();
    for (size_t k = 0; k < r.size(); ++k) p->radix[k] = r[k];
    // position i = q0 + r0 (q1 + r1 (q2 + ...)) holds input sum_s q_s n / L_s
    std::vector<int32_t> src((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        int64_t rem = i, L = 1, v = 0;
        for (int32_t rs : r) {
            const int64_t q = rem % rs;
            rem /= rs;
            L *= rs;
            v += q * (n / L);
        }
        src[(size_t)i] = (int32_t)v;
    }
    std::vector<float4> tw((size_t)n);
    const double pi = 3.14159265358979323846;
    for (int64_t k = 0; k < n; ++k) {
        const double a = 2.0 * pi * (double)k / (double)n;
        float4 w;
        split(std::cos(a), &w.x, &w.y);
        split(std::sin(a), &w.z, &w.w);
        tw[(size_t)k] = w;
    }
    CR_CUDA_CHECK(cudaMalloc((void**)&p->src, (size_t)n * 4));
    CR_CUDA_CHECK(cudaMalloc((void**)&p->tw, (size_t)n * 16));
    CR_CUDA_CHECK(cudaMemcpy(p->src, src.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
    CR_CUDA_CHECK(cudaMemcpy(p->tw, tw.data(), (size_t)n * 16, cudaMemcpyHostToDevice));
    ctx->df_plans[n] = p;
    return *p;
}

DfStages stages(const DfPlan& p) {
    DfStages s{};
    s.n = p.n;
    s.ns = p.ns;
    for (int k = 0; k < p.ns; ++k) s.radix[k] = p.radix[k];
    return s;
}

template <typename K>
void allow_smem(K kernel, size_t bytes) {
    CR_CUDA_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bytes));
}

}  // namespace

bool dfft_supported(int64_t gnx, int64_t gny) {
    for (int64_t n : {gnx, gny})
        if (n < 2 || n > kDfMaxN || (n & 1) || radices(n).empty()) return false;
    return true;
}

void dfft_grid_to_image(cr_ctx* ctx, cr_gridder* g, const float2* grid, const float* real_grid,
                        double scale, const float* sx, const float* sy, int sinc_mode,
                        float* image) {
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny, gnyh = gny / 2 + 1;
    const int32_t nx = g->geom.nx, ny = g->geom.ny;
    const DfPlan& px = plan_for(ctx, gnx);
    const DfPlan& py = plan_for(ctx, gny);
    const DfConsts c = consts();
    float4* t = (float4*)workspace(ctx, "dfft_t", (size_t)nx * gnyh * 16);
    const size_t smx = (size_t)gnx * 16, smy = (size_t)gny * 16;
    allow_smem(dfft_inv_cols, smx);
    allow_smem(dfft_inv_rows, smy);
    dfft_inv_cols<<<(unsigned)gnyh, kDfThreads, smx, ctx->stream>>>(
        grid, real_grid, gnx, gny, gnyh, g->info.blc_x, nx, px.src, px.tw, stages(px), c, t);
    note_launch(ctx, "dfft_inv_cols");
    const int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    dfft_inv_rows<<<(unsigned)((nx + 1) / 2), kDfThreads, smy, ctx->stream>>>(
        t, gny, gnyh, nx, ny, g->info.blc_x, g->info.blc_y, parity, scale, g->corr_x_d,
        g->corr_y_d, sx, sy, sinc_mode, py.src, py.tw, stages(py), c, image);
    note_launch(ctx, "dfft_inv_rows");
}

void dfft_image_to_grid(cr_ctx* ctx, cr_gridder* g, const float* model, const float* sinc_x,
                        const float* sinc_y, float2* grid) {
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny, gnyh = gny / 2 + 1;
    const int32_t nx = g->geom.nx, ny = g->geom.ny;
    const DfPlan& px = plan_for(ctx, gnx);
    const DfPlan& py = plan_for(ctx, gny);
    const DfConsts c = consts();
    float4* t = (float4*)workspace(ctx, "dfft_t", (size_t)nx * gnyh * 16);
    const size_t smx = (size_t)gnx * 16, smy = (size_t)gny * 16;
    allow_smem(dfft_fwd_rows, smy);
    allow_smem(dfft_fwd_cols, smx);
    dfft_fwd_rows<<<(unsigned)((nx + 1) / 2), kDfThreads, smy, ctx->stream>>>(
        model, nx, ny, gny, gnyh, g->info.blc_x, g->info.blc_y, g->corr_x_d, g->corr_y_d,
        sinc_x, sinc_y, py.src, py.tw, stages(py), c, t);
    note_launch(ctx, "dfft_fwd_rows");
    const int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    dfft_fwd_cols<<<(unsigned)gnyh, kDfThreads, smx, ctx->stream>>>(
        t, gny, gnyh, nx, g->info.blc_x, parity, px.src, px.tw, stages(px), c, grid);
    note_launch(ctx, "dfft_fwd_cols");
}

}  // namespace cr
