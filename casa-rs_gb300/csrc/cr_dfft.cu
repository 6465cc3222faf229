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
//   grid -> image: columns first (every grid column, only the image's rows
//     kept), then the image's rows, whose output goes straight through the
//     crop and correction of crop_correct_body;
//   image -> grid: the image's rows first (the apodised image is zero
//     outside them), then every grid column, written as the float32 grid.
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

// grid -> image, pass 1: column y of the modulated grid transformed along x;
// the image's rows [bx0, bx0 + nx) kept in t[(x - bx0) gny + y].
__global__ void __launch_bounds__(kDfThreads, 2) dfft_inv_cols(
    const float2* grid, const float* real_grid, int64_t gny, int64_t bx0, int32_t nx,
    const int32_t* src, const float4* tw, DfStages s, DfConsts c, float4* t) {
    extern __shared__ float4 sm[];
    const int64_t y = blockIdx.x;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) {
        const int64_t x = src[i];
        float re, im = 0.0f;
        if (real_grid) {
            re = real_grid[x * gny + y];
        } else {
            const float2 v = grid[x * gny + y];
            re = v.x;
            im = v.y;
        }
        if ((x + y) & 1) {
            re = -re;
            im = -im;
        }
        sm[i] = make_float4(re, 0.0f, im, 0.0f);
    }
    __syncthreads();
    line_transform<true>(sm, s, tw, c);
    for (int xr = threadIdx.x; xr < nx; xr += blockDim.x) t[xr * gny + y] = sm[bx0 + xr];
}

// grid -> image, pass 2: image row xr transformed along y, then the crop and
// correction of crop_correct_body (the same operations on the FP64 value).
__global__ void __launch_bounds__(kDfThreads, 2) dfft_inv_rows(
    const float4* t, int64_t gny, int32_t ny, int64_t bx0, int64_t by0, int parity,
    double scale, const float* corr_x, const float* corr_y, const float* sx, const float* sy,
    int sinc_mode, const int32_t* src, const float4* tw, DfStages s, DfConsts c,
    float* image) {
    extern __shared__ float4 sm[];
    const int64_t xr = blockIdx.x, gx = bx0 + xr;
    const float4* row = t + xr * gny;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) sm[i] = row[src[i]];
    __syncthreads();
    line_transform<true>(sm, s, tw, c);
    // the scale as a float pair: the product's high part is the float32
    // value (float)(r * scale) of the FP64 path, but for ties at half an ulp
    const float sh = (float)scale;
    const dd sc{sh, (float)(scale - (double)sh)};
    for (int yr = threadIdx.x; yr < ny; yr += blockDim.x) {
        const int64_t gy = by0 + yr;
        const float4 w = sm[gy];
        const dd r = ((gx + gy + parity) & 1) ? dd{-w.x, -w.y} : dd{w.x, w.y};
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

// image -> grid, pass 1: row xr of the apodised, modulated model (zero
// outside the image's columns) transformed along y into t[xr gny + y].
__global__ void __launch_bounds__(kDfThreads, 2) dfft_fwd_rows(
    const float* model, int32_t ny, int64_t gny, int64_t bx0, int64_t by0, const float* corr_x,
    const float* corr_y, const float* sinc_x, const float* sinc_y, const int32_t* src,
    const float4* tw, DfStages s, DfConsts c, float4* t) {
    extern __shared__ float4 sm[];
    const int64_t xr = blockIdx.x, gx = bx0 + xr;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) {
        const int64_t gy = src[i];
        float v = 0.0f;
        if (gy >= by0 && gy < by0 + ny) {
            // apodize_body's operations
            float f = __fmul_rn(corr_x[gx], corr_y[gy]);
            if (sinc_x) f = __fmul_rn(__fmul_rn(f, sinc_x[gx]), sinc_y[gy]);
            v = model[xr * ny + (gy - by0)] * f;
            if ((gx + gy) & 1) v = -v;
        }
        sm[i] = make_float4(v, 0.0f, 0.0f, 0.0f);
    }
    __syncthreads();
    line_transform<false>(sm, s, tw, c);
    float4* row = t + xr * gny;
    for (int y = threadIdx.x; y < s.n; y += blockDim.x) row[y] = sm[y];
}

// image -> grid, pass 2: column y transformed along x (rows outside
// [bx0, bx0 + nx) are zero), the output checkerboard, float32 grid.
__global__ void __launch_bounds__(kDfThreads, 2) dfft_fwd_cols(
    const float4* t, int64_t gny, int32_t nx, int64_t bx0, int parity, const int32_t* src,
    const float4* tw, DfStages s, DfConsts c, float2* grid) {
    extern __shared__ float4 sm[];
    const int64_t y = blockIdx.x;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) {
        const int64_t x = src[i];
        sm[i] = (x >= bx0 && x < bx0 + nx) ? t[(x - bx0) * gny + y]
                                           : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncthreads();
    line_transform<false>(sm, s, tw, c);
    for (int x = threadIdx.x; x < s.n; x += blockDim.x) {
        const float4 w = sm[x];
        // the pairs are normalised: the high part is the float32 value
        float re = w.x, im = w.z;
        if ((x + y + parity) & 1) {
            re = -re;
            im = -im;
        }
        grid[(int64_t)x * gny + y] = make_float2(re, im);
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
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    const int32_t nx = g->geom.nx, ny = g->geom.ny;
    const DfPlan& px = plan_for(ctx, gnx);
    const DfPlan& py = plan_for(ctx, gny);
    const DfConsts c = consts();
    float4* t = (float4*)workspace(ctx, "dfft_t", (size_t)nx * gny * 16);
    const size_t smx = (size_t)gnx * 16, smy = (size_t)gny * 16;
    allow_smem(dfft_inv_cols, smx);
    allow_smem(dfft_inv_rows, smy);
    dfft_inv_cols<<<(unsigned)gny, kDfThreads, smx, ctx->stream>>>(
        grid, real_grid, gny, g->info.blc_x, nx, px.src, px.tw, stages(px), c, t);
    note_launch(ctx, "dfft_inv_cols");
    const int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    dfft_inv_rows<<<(unsigned)nx, kDfThreads, smy, ctx->stream>>>(
        t, gny, ny, g->info.blc_x, g->info.blc_y, parity, scale, g->corr_x_d, g->corr_y_d, sx,
        sy, sinc_mode, py.src, py.tw, stages(py), c, image);
    note_launch(ctx, "dfft_inv_rows");
}

void dfft_image_to_grid(cr_ctx* ctx, cr_gridder* g, const float* model, const float* sinc_x,
                        const float* sinc_y, float2* grid) {
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    const int32_t nx = g->geom.nx, ny = g->geom.ny;
    const DfPlan& px = plan_for(ctx, gnx);
    const DfPlan& py = plan_for(ctx, gny);
    const DfConsts c = consts();
    float4* t = (float4*)workspace(ctx, "dfft_t", (size_t)nx * gny * 16);
    const size_t smx = (size_t)gnx * 16, smy = (size_t)gny * 16;
    allow_smem(dfft_fwd_rows, smy);
    allow_smem(dfft_fwd_cols, smx);
    dfft_fwd_rows<<<(unsigned)nx, kDfThreads, smy, ctx->stream>>>(
        model, ny, gny, g->info.blc_x, g->info.blc_y, g->corr_x_d, g->corr_y_d, sinc_x, sinc_y,
        py.src, py.tw, stages(py), c, t);
    note_launch(ctx, "dfft_fwd_rows");
    const int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    dfft_fwd_cols<<<(unsigned)gny, kDfThreads, smx, ctx->stream>>>(
        t, gny, nx, g->info.blc_x, parity, px.src, px.tw, stages(px), c, grid);
    note_launch(ctx, "dfft_fwd_cols");
}

}  // namespace cr
