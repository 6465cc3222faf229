// cr_msclean.cu -- multiscale CLEAN on the device.
//
// Restates run_multiscale_cotton_schwab's state and minor cycle
// (crates/casa-imaging/src/lib.rs:63543-64405):
//   * scale images make_multiscale_kernel / multiscale_spheroidal
//     (lib.rs:64325-64405) built on the host in the reference's mixed
//     float32 / FP64 arithmetic, with their nonzero supports;
//   * build_multiscale_state (lib.rs:64172-64230): the residual convolved
//     with every scale, the PSF convolved with scale k then scale l (the
//     K x K cross terms), their diagonal peaks (at least 1e-6), the
//     small-scale bias, and the scale masks of a clean mask
//     (lib.rs:64232-64261).  fft_convolve_real's centred transforms reduce to
//     the circular convolution conv[x] = sum_p a[p] b[(x - p + n/2) mod n],
//     computed with cuFFT in FP64 and rounded to float32 (the reference uses
//     float32 transforms);
//   * the minor cycle (lib.rs:63700-63800) as one cooperative launch: each
//     iteration every block reduces the per-scale peak candidates of the
//     search window (peak_location_masked_in_bounds_zero_tolerance), all
//     blocks pick the same scale by the biased score of
//     select_multiscale_candidate (lib.rs:64263-64305), apply the stop and
//     divergence rules (lib.rs:64011-64023), add the scaled component to the
//     model over the scale image's support, and subtract component * the
//     cross term (k, chosen scale) from every convolved residual k inside
//     the component window (from_casa_shifted_support, lib.rs:63221-63238),
//     finding the next candidates in the same pass.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cr_clean.cuh"
#include "cr_internal.cuh"

struct cr_multiscale {
    cr_ctx* ctx = nullptr;
    int nx = 0, ny = 0, K = 0;
    std::vector<float> scales;
    std::vector<int> support;          // [K][4]: x0, y0, x1, y1 (x1 < 0: no support)
    std::vector<float> peak_psf, bias;
    cr::Pool pool;
    float* kernels = nullptr;          // [K][npix] scale images
    double2* fkernels = nullptr;       // [K][npix] their transforms
    float* dirty = nullptr;            // [K][npix] residual convolved with each scale
    float* psfc = nullptr;             // [K][K][npix] PSF convolved with scale k then l
    uint8_t* mask = nullptr;           // clean mask (nonzero: cleanable) or null
    uint8_t* smask = nullptr;          // [K][npix] scale masks or null
    float* params = nullptr;           // device: peak_psf [K], bias [K]
    int* supp_d = nullptr;             // device copy of support
};

namespace cr {
namespace {

constexpr int kMsThreads = 512;
constexpr int kMaxScales = 16;

// multiscale_spheroidal (lib.rs:64364-64405): float32, with powf.
float ms_spheroidal(float nu) {
    if (nu <= 0.0f) return 1.0f;
    if (nu >= 1.0f) return 0.0f;
    static const float pa[5] = {8.203343e-2f, -3.644705e-1f, 6.27866e-1f, -5.335581e-1f,
                                2.312756e-1f};
    static const float qa[3] = {1.0f, 8.212018e-1f, 2.078043e-1f};
    static const float pb[5] = {4.028559e-3f, -3.697768e-2f, 1.021332e-1f, -1.201436e-1f,
                                6.412774e-2f};
    static const float qb[3] = {1.0f, 9.599102e-1f, 2.918724e-1f};
    const bool lo = nu < 0.75f;
    const float* p = lo ? pa : pb;
    const float* q = lo ? qa : qb;
    const float nuend = lo ? 0.75f : 1.0f;
    const float delnusq = std::pow(nu, 2.0f) - std::pow(nuend, 2.0f);
    float num = p[0];
    for (int k = 1; k < 5; ++k) num += p[k] * std::pow(delnusq, (float)k);
    float den = q[0];
    for (int k = 1; k < 3; ++k) den += q[k] * std::pow(delnusq, (float)k);
    return den == 0.0f ? 0.0f : num / den;
}

// make_multiscale_kernel (lib.rs:64325-64362), x-major [nx][ny].
std::vector<float> ms_kernel(int nx, int ny, float scale) {
    std::vector<float> k((size_t)nx * ny, 0.0f);
    const double refi = (double)(nx / 2), refj = (double)(ny / 2);
    if (scale == 0.0f) {
        k[(size_t)(nx / 2) * ny + ny / 2] = 1.0f;
        return k;
    }
    const double s = (double)scale;
    const int64_t mini = std::max<int64_t>((int64_t)(refi - s), 0);
    const int64_t maxi = std::min<int64_t>((int64_t)(refi + s), nx - 1);
    const int64_t minj = std::max<int64_t>((int64_t)(refj - s), 0);
    const int64_t maxj = std::min<int64_t>((int64_t)(refj + s), ny - 1);
    float volume = 0.0f;
    for (int64_t j = minj; j <= maxj; ++j) {
        const double t = (refj - (double)j) / s;
        const float ypart = (float)(t * t);
        for (int64_t i = mini; i <= maxi; ++i) {
            const double ti = (refi - (double)i) / s;
            const float rad2 = (float)((double)ypart + ti * ti);
            if (rad2 < 1.0f) {
                const float rad = rad2 <= 0.0f ? 0.0f : std::sqrt(rad2);
                const float value = (float)((1.0 - (double)rad2) * (double)ms_spheroidal(rad));
                k[(size_t)i * ny + j] = value;
                volume += value;
            }
        }
    }
    if (volume > 0.0f)
        for (float& v : k) v = v / volume;
    return k;
}

__global__ void ms_pack_kernel(const float* src, const uint8_t* bsrc, int nx, int ny,
                               int shift, double2* out) {
    const int64_t n = (int64_t)nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(t / ny), y = (int)(t - (int64_t)x * ny);
        // out[k] = src[(k + n/2) mod n] when shift, else src[k]
        const int sx = shift ? (x + nx / 2) % nx : x, sy = shift ? (y + ny / 2) % ny : y;
        const int64_t i = (int64_t)sx * ny + sy;
        out[t] = make_double2(src ? (double)src[i] : (bsrc[i] ? 1.0 : 0.0), 0.0);
    }
}

__global__ void ms_mul_kernel(double2* out, const double2* a, const double2* b, int64_t n,
                              double scale) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const double2 x = a[t], y = b[t];
        out[t] = make_double2((x.x * y.x - x.y * y.y) * scale, (x.x * y.y + x.y * y.x) * scale);
    }
}

__global__ void ms_real_kernel(const double2* src, int64_t n, float* out) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        out[t] = (float)src[t].x;
}

// scale mask: conv > 0.9 and outside the border of (scale * 1.5) pixels
__global__ void ms_mask_kernel(const double2* conv, int nx, int ny, int border, uint8_t* out) {
    const int64_t n = (int64_t)nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(t / ny), y = (int)(t - (int64_t)x * ny);
        const bool edge = x <= border || y <= border || x >= nx - (border + 1) ||
                          y >= ny - (border + 1);
        out[t] = (!edge && (float)conv[t].x > 0.9f) ? 1 : 0;
    }
}

// largest finite |value| (masked), as float bits
__global__ void ms_absmax_kernel(const float* img, const uint8_t* mask, int64_t n,
                                 unsigned int* out) {
    unsigned int best = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (mask && !mask[t]) continue;
        const float a = fabsf(img[t]);
        if (isfinite(a)) best = max(best, __float_as_uint(a));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best) atomicMax(out, best);
}

struct MsArgs {
    float* dirty;            // [K][npix]
    const float* psfc;       // [K][K][npix]
    const float* kernels;    // [K][npix]
    const uint8_t* smask;    // [K][npix] or null
    float* model;
    int nx, ny, K;
    const float* params;     // peak_psf [K], bias [K]
    const int* supp;         // [K][4]
    float gain, threshold, cycle_threshold, nsigma_threshold;
    long long budget;
    Cand* cands;             // [2][K][nblocks]
    unsigned int* bar;
    long long barrier_polls;
    int* comp_x;
    int* comp_y;
    int* comp_scale;
    float* comp_strength;
    float* comp_flux;
    long long* out_actual;
    int* out_stop;
    int* out_status;
};

__device__ __forceinline__ bool in_window(int x, int y, const int* w) {
    return x >= w[0] && x <= w[2] && y >= w[1] && y <= w[3];
}

// the block's candidate of scale k over its pixels inside the window
__device__ Cand ms_block_candidate(const MsArgs& a, int k, int64_t p0, int64_t p1,
                                   const int* win) {
    const int64_t npix = (int64_t)a.nx * a.ny;
    const float* d = a.dirty + (int64_t)k * npix;
    const uint8_t* m = a.smask ? a.smask + (int64_t)k * npix : nullptr;
    float ba = -1.0f, bv = 0.0f;
    int bk = 0x7fffffff;
    for (int64_t t = p0 + threadIdx.x; t < p1; t += blockDim.x) {
        const int x = (int)(t / a.ny), y = (int)(t - (int64_t)x * a.ny);
        if (!in_window(x, y, win) || (m && !m[t])) continue;
        const float v = d[t], av = fabsf(v);
        if (!isfinite(av)) continue;
        const int key = y * a.nx + x;
        if (better(av, key, ba, bk)) {
            ba = av;
            bk = key;
            bv = v;
        }
    }
    return block_argmax(ba, bk, bv);
}

__global__ void __launch_bounds__(kMsThreads) msclean_kernel(MsArgs a) {
    const int nblocks = (int)gridDim.x, bidx = (int)blockIdx.x;
    const int64_t npix = (int64_t)a.nx * a.ny;
    const int64_t chunk = (npix + nblocks - 1) / nblocks;
    const int64_t p0 = (int64_t)bidx * chunk, p1 = min(npix, p0 + chunk);
    const float* peak_psf = a.params;
    const float* bias = a.params + a.K;
    __shared__ int s_win[4];
    __shared__ int s_sel, s_x, s_y, s_stop;
    __shared__ float s_strength;
    if (threadIdx.x == 0) {
        s_win[0] = 0;
        s_win[1] = 0;
        s_win[2] = a.nx - 1;
        s_win[3] = a.ny - 1;
    }
    __syncthreads();
    for (int k = 0; k < a.K; ++k) {
        const Cand c = ms_block_candidate(a, k, p0, p1, s_win);
        if (threadIdx.x == 0) a.cands[(int64_t)k * nblocks + bidx] = c;
    }
    if (!grid_barrier(a.bar, (unsigned)nblocks, a.barrier_polls)) {
        if (threadIdx.x == 0) atomicExch(a.out_status, CR_TIMEOUT);
        return;
    }
    long long it = 0;
    int stop = CR_STOP_NONE;
    float initial = 0.0f;
    for (; it < a.budget; ++it) {
        const Cand* cur = a.cands + (it & 1) * (int64_t)a.K * nblocks;
        Cand* nxt = a.cands + ((it + 1) & 1) * (int64_t)a.K * nblocks;
        // every block reduces every scale's candidates, then picks the scale
        // of largest |bias * value * strength| (the first on ties)
        int sel = -1;
        float sel_strength = 0.0f, sel_score = 0.0f;
        int sel_key = 0;
        for (int k = 0; k < a.K; ++k) {
            float ba = -1.0f, bv = 0.0f;
            int bk = 0x7fffffff;
            for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
                const int4 raw =
                    __ldcg(reinterpret_cast<const int4*>(cur + (int64_t)k * nblocks) + i);
                const Cand c{__int_as_float(raw.x), raw.y, __int_as_float(raw.z), 0};
                if (better(c.absval, c.key, ba, bk)) {
                    ba = c.absval;
                    bk = c.key;
                    bv = c.value;
                }
            }
            const Cand c = block_argmax(ba, bk, bv);
            if (threadIdx.x == 0 && c.absval >= 0.0f) {
                const float peak = peak_psf[k];
                if (peak > 0.0f && c.value != 0.0f) {
                    const float strength = __fdiv_rn(c.value, peak);
                    const float score = __fmul_rn(__fmul_rn(bias[k], c.value), strength);
                    if (sel < 0 || fabsf(score) > fabsf(sel_score)) {
                        sel = k;
                        sel_strength = strength;
                        sel_score = score;
                        sel_key = c.key;
                    }
                }
            }
        }
        if (threadIdx.x == 0) {
            int r = 0;
            if (sel < 0) {
                r = CR_STOP_NO_CLEANABLE_PIXELS;
            } else {
                const float av = fabsf(sel_strength);
                r = stop_reason(av, a.threshold, a.cycle_threshold, a.nsigma_threshold);
                if (!r) {
                    if (it == 0) initial = av;
                    else if (av > __fmul_rn(fabsf(initial), 1.5f)) r = -1;   // divergence
                }
            }
            s_stop = r;
            s_sel = sel;
            s_x = sel_key % a.nx;
            s_y = sel_key / a.nx;
            s_strength = sel_strength;
        }
        __syncthreads();
        if (s_stop) {
            stop = s_stop;
            break;
        }
        const int k_sel = s_sel, px = s_x, py = s_y;
        const float comp = __fmul_rn(a.gain, s_strength);
        if (bidx == 0 && threadIdx.x == 0 && a.comp_x) {
            a.comp_x[it] = px;
            a.comp_y[it] = py;
            a.comp_scale[it] = k_sel;
            a.comp_strength[it] = s_strength;
            a.comp_flux[it] = comp;
        }
        // the model over the scale image's support (add_shifted_kernel_with_support)
        {
            const int* sp = a.supp + 4 * k_sel;
            const int cx = a.nx / 2, cy = a.ny / 2;
            if (sp[2] >= 0) {
                const int x0 = max(px + sp[0] - cx, 0), x1 = min(px + sp[2] - cx, a.nx - 1);
                const int y0 = max(py + sp[1] - cy, 0), y1 = min(py + sp[3] - cy, a.ny - 1);
                const float* ker = a.kernels + (int64_t)k_sel * npix;
                for (int64_t t = p0 + threadIdx.x; t < p1; t += blockDim.x) {
                    const int x = (int)(t / a.ny), y = (int)(t - (int64_t)x * a.ny);
                    if (x < x0 || x > x1 || y < y0 || y > y1) continue;
                    const float kv = ker[(int64_t)(x - px + cx) * a.ny + (y - py + cy)];
                    a.model[t] = __fadd_rn(a.model[t], __fmul_rn(comp, kv));
                }
            }
        }
        // the component window, then per scale: subtract the cross term and
        // find the next candidate inside the window
        if (threadIdx.x == 0) {
            const int hx = a.nx / 2, hy = a.ny / 2;
            s_win[0] = max(px - hx, 0);
            s_win[1] = max(py - hy, 0);
            s_win[2] = min(max(px + hx - 1, 0), a.nx - 1);
            s_win[3] = min(max(py + hy - 1, 0), a.ny - 1);
        }
        __syncthreads();
        const int cx = a.nx / 2, cy = a.ny / 2;
        for (int k = 0; k < a.K; ++k) {
            float* d = a.dirty + (int64_t)k * npix;
            const float* ker = a.psfc + ((int64_t)k * a.K + k_sel) * npix;
            const uint8_t* m = a.smask ? a.smask + (int64_t)k * npix : nullptr;
            float ba = -1.0f, bv = 0.0f;
            int bk = 0x7fffffff;
            for (int64_t t = p0 + threadIdx.x; t < p1; t += blockDim.x) {
                const int x = (int)(t / a.ny), y = (int)(t - (int64_t)x * a.ny);
                if (!in_window(x, y, s_win)) continue;
                float v = d[t];
                const int kx = x - px + cx, ky = y - py + cy;
                if (kx >= 0 && kx < a.nx && ky >= 0 && ky < a.ny) {
                    v = __fsub_rn(v, __fmul_rn(comp, ker[(int64_t)kx * a.ny + ky]));
                    d[t] = v;
                }
                if (m && !m[t]) continue;
                const float av = fabsf(v);
                if (!isfinite(av)) continue;
                const int key = y * a.nx + x;
                if (better(av, key, ba, bk)) {
                    ba = av;
                    bk = key;
                    bv = v;
                }
            }
            const Cand c = block_argmax(ba, bk, bv);
            if (threadIdx.x == 0) nxt[(int64_t)k * nblocks + bidx] = c;
        }
        if (!grid_barrier(a.bar, (unsigned)nblocks, a.barrier_polls)) {
            if (threadIdx.x == 0) atomicExch(a.out_status, CR_TIMEOUT);
            return;
        }
    }
    if (bidx == 0 && threadIdx.x == 0) {
        *a.out_actual = it;
        *a.out_stop = stop;
    }
}

// out = float32 of the circular convolution of image (as given) with the
// transform `fk` of a kernel centred at (nx/2, ny/2); `fimg` receives the
// image's transform when not null
void conv_with(cr_ctx* ctx, cr_multiscale* ms, const double2* fimg, const double2* fk,
               float* out) {
    const int64_t n = (int64_t)ms->nx * ms->ny;
    double2* work = (double2*)workspace(ctx, "ms_work", (size_t)n * 16);
    ms_mul_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(work, fimg, fk, n,
                                                                   1.0 / (double)n);
    note_launch(ctx, "ms_mul_kernel");
    check_cufft(cufftExecZ2Z(fft_plan(ctx, ms->nx, ms->ny), (cufftDoubleComplex*)work,
                             (cufftDoubleComplex*)work, CUFFT_INVERSE),
                "cufftExecZ2Z");
    ms_real_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(work, n, out);
    note_launch(ctx, "ms_real_kernel");
}

// the transform of a float image (shift: centred kernel) into dst
void transform(cr_ctx* ctx, cr_multiscale* ms, const float* src, const uint8_t* bsrc,
               int shift, double2* dst) {
    const int64_t n = (int64_t)ms->nx * ms->ny;
    ms_pack_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(src, bsrc, ms->nx, ms->ny,
                                                                    shift, dst);
    note_launch(ctx, "ms_pack_kernel");
    check_cufft(cufftExecZ2Z(fft_plan(ctx, ms->nx, ms->ny), (cufftDoubleComplex*)dst,
                             (cufftDoubleComplex*)dst, CUFFT_FORWARD),
                "cufftExecZ2Z");
}

float absmax(cr_ctx* ctx, const float* img, const uint8_t* mask, int64_t n) {
    unsigned int* o = (unsigned int*)workspace(ctx, "ms_absmax", 16);
    CR_CUDA_CHECK(cudaMemsetAsync(o, 0, 4, ctx->stream));
    ms_absmax_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(img, mask, n, o);
    note_launch(ctx, "ms_absmax_kernel");
    unsigned int h = 0;
    CR_CUDA_CHECK(cudaMemcpyAsync(&h, o, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    float f;
    std::memcpy(&f, &h, 4);
    return f;
}

}  // namespace

void multiscale_set_residual(cr_multiscale* ms, const float* residual) {
    cr_ctx* ctx = ms->ctx;
    const int64_t n = (int64_t)ms->nx * ms->ny;
    double2* fr = (double2*)workspace(ctx, "ms_fimg", (size_t)n * 16);
    transform(ctx, ms, residual, nullptr, 0, fr);
    for (int k = 0; k < ms->K; ++k)
        conv_with(ctx, ms, fr, ms->fkernels + (int64_t)k * n, ms->dirty + (int64_t)k * n);
}

void multiscale_create(cr_multiscale* ms, const float* psf, const uint8_t* mask,
                       float small_scale_bias) {
    cr_ctx* ctx = ms->ctx;
    const int nx = ms->nx, ny = ms->ny, K = ms->K;
    const int64_t n = (int64_t)nx * ny;
    auto A = [&](const char* name, size_t bytes) { return pool_alloc(ctx, ms->pool, name, bytes); };
    ms->kernels = (float*)A("kernels", (size_t)K * n * 4);
    ms->fkernels = (double2*)A("fkernels", (size_t)K * n * 16);
    ms->dirty = (float*)A("dirty", (size_t)K * n * 4);
    ms->psfc = (float*)A("psfc", (size_t)K * K * n * 4);
    ms->params = (float*)A("params", (size_t)2 * K * 4);
    ms->supp_d = (int*)A("supp", (size_t)4 * K * 4);
    ms->support.assign((size_t)4 * K, -1);
    for (int k = 0; k < K; ++k) {
        const std::vector<float> h = ms_kernel(nx, ny, ms->scales[k]);
        int x0 = nx, y0 = ny, x1 = -1, y1 = -1;   // kernel_nonzero_support
        for (int x = 0; x < nx; ++x)
            for (int y = 0; y < ny; ++y)
                if (h[(size_t)x * ny + y] != 0.0f) {
                    x0 = std::min(x0, x);
                    y0 = std::min(y0, y);
                    x1 = std::max(x1, x);
                    y1 = std::max(y1, y);
                }
        if (x1 >= 0) {
            ms->support[4 * k] = x0;
            ms->support[4 * k + 1] = y0;
            ms->support[4 * k + 2] = x1;
            ms->support[4 * k + 3] = y1;
        }
        CR_CUDA_CHECK(cudaMemcpyAsync(ms->kernels + (int64_t)k * n, h.data(), (size_t)n * 4,
                                      cudaMemcpyHostToDevice, ctx->stream));
        transform(ctx, ms, ms->kernels + (int64_t)k * n, nullptr, 1, ms->fkernels + (int64_t)k * n);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));   // h leaves scope
    }
    // cross terms: (psf conv scale k, rounded to float32) conv scale l
    double2* fimg = (double2*)workspace(ctx, "ms_fimg", (size_t)n * 16);
    float* pk = (float*)workspace(ctx, "ms_pk", (size_t)n * 4);
    transform(ctx, ms, psf, nullptr, 0, fimg);
    double2* fpk = (double2*)workspace(ctx, "ms_fpk", (size_t)n * 16);
    for (int k = 0; k < K; ++k) {
        conv_with(ctx, ms, fimg, ms->fkernels + (int64_t)k * n, pk);
        transform(ctx, ms, pk, nullptr, 0, fpk);
        for (int l = 0; l < K; ++l)
            conv_with(ctx, ms, fpk, ms->fkernels + (int64_t)l * n,
                      ms->psfc + ((int64_t)k * K + l) * n);
    }
    ms->peak_psf.assign(K, 0.0f);
    ms->bias.assign(K, 1.0f);
    for (int k = 0; k < K; ++k)
        ms->peak_psf[k] = std::max(absmax(ctx, ms->psfc + ((int64_t)k * K + k) * n, nullptr, n),
                                   1.0e-6f);
    float mx = 0.0f;
    for (float s : ms->scales) mx = std::max(mx, s);
    if (mx > 0.0f && K > 1)
        for (int k = 0; k < K; ++k) ms->bias[k] = 1.0f - small_scale_bias * (ms->scales[k] / mx);
    std::vector<float> prm(ms->peak_psf);
    prm.insert(prm.end(), ms->bias.begin(), ms->bias.end());
    CR_CUDA_CHECK(cudaMemcpyAsync(ms->params, prm.data(), prm.size() * 4, cudaMemcpyHostToDevice,
                                  ctx->stream));
    CR_CUDA_CHECK(cudaMemcpyAsync(ms->supp_d, ms->support.data(), ms->support.size() * 4,
                                  cudaMemcpyHostToDevice, ctx->stream));
    if (mask) {
        ms->mask = (uint8_t*)A("mask", (size_t)n);
        CR_CUDA_CHECK(cudaMemcpyAsync(ms->mask, mask, (size_t)n, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        ms->smask = (uint8_t*)A("smask", (size_t)K * n);
        transform(ctx, ms, nullptr, mask, 0, fimg);
        double2* work = (double2*)workspace(ctx, "ms_work", (size_t)n * 16);
        for (int k = 0; k < K; ++k) {
            ms_mul_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(
                work, fimg, ms->fkernels + (int64_t)k * n, n, 1.0 / (double)n);
            note_launch(ctx, "ms_mul_kernel");
            check_cufft(cufftExecZ2Z(fft_plan(ctx, nx, ny), (cufftDoubleComplex*)work,
                                     (cufftDoubleComplex*)work, CUFFT_INVERSE),
                        "cufftExecZ2Z");
            const int border = (int)(ms->scales[k] * 1.5f);
            ms_mask_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(
                work, nx, ny, border, ms->smask + (int64_t)k * n);
            note_launch(ctx, "ms_mask_kernel");
        }
    }
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
}

// (has a candidate in the full window, peak |residual conv scale 0| under
// the clean mask)
void multiscale_peak(cr_multiscale* ms, int32_t* has_candidate, float* peak0) {
    cr_ctx* ctx = ms->ctx;
    const int64_t n = (int64_t)ms->nx * ms->ny;
    bool any = false;
    for (int k = 0; k < ms->K && !any; ++k) {
        const uint8_t* m = ms->smask ? ms->smask + (int64_t)k * n : nullptr;
        any = ms->peak_psf[k] > 0.0f && absmax(ctx, ms->dirty + (int64_t)k * n, m, n) > 0.0f;
    }
    if (has_candidate) *has_candidate = any ? 1 : 0;
    if (peak0) *peak0 = absmax(ctx, ms->dirty, ms->mask, n);
}

void multiscale_minor_cycle(cr_multiscale* ms, float* model, float gain, float threshold,
                            float cycle_threshold, float nsigma_threshold, int64_t cycle_niter,
                            int32_t* comp_x, int32_t* comp_y, int32_t* comp_scale,
                            float* comp_strength, float* comp_flux, int64_t* actual,
                            int64_t* reported, int32_t* stop_out) {
    cr_ctx* ctx = ms->ctx;
    if (cycle_niter < 0) fail(CR_INVALID, "cycle_niter is negative");
    const int64_t n = (int64_t)ms->nx * ms->ny;
    int sms = ctx->sms, per_sm = 0;
    CR_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msclean_kernel,
                                                                kMsThreads, 0));
    if (per_sm < 1) fail(CR_CUDA, "multiscale kernel cannot be resident");
    const int blocks = (int)std::min<int64_t>((int64_t)sms * std::min(per_sm, 2),
                                              std::max<int64_t>(1, (n + kMsThreads - 1) /
                                                                       kMsThreads));
    const size_t cap = (size_t)std::max<int64_t>(cycle_niter, 1);
    const size_t head = 256, cands = (size_t)2 * ms->K * blocks * sizeof(Cand);
    char* wsp = (char*)workspace(ctx, "ms_ws", head + cands + cap * 20);
    unsigned int* bar = (unsigned int*)wsp;
    long long* out_actual = (long long*)(wsp + 16);
    int* out_stop = (int*)(wsp + 24);
    int* out_status = (int*)(wsp + 28);
    Cand* cd = (Cand*)(wsp + head);
    int* cx = (int*)(wsp + head + cands);
    int* cy = cx + cap;
    int* cs = cy + cap;
    float* cst = (float*)(cs + cap);
    float* cf = cst + cap;
    CR_CUDA_CHECK(cudaMemsetAsync(wsp, 0, head, ctx->stream));
    MsArgs a{ms->dirty, ms->psfc, ms->kernels, ms->smask, model, ms->nx, ms->ny, ms->K,
             ms->params, ms->supp_d, gain, threshold, cycle_threshold, nsigma_threshold,
             (long long)cycle_niter, cd, bar, ctx->barrier_polls, cx, cy, cs, cst, cf,
             out_actual, out_stop, out_status};
    void* args[] = {&a};
    CR_CUDA_CHECK(cudaLaunchCooperativeKernel((void*)msclean_kernel, dim3(blocks),
                                              dim3(kMsThreads), args, 0, ctx->stream));
    note_launch(ctx, "msclean_kernel");
    struct {
        long long actual;
        int stop, status;
    } h;
    CR_CUDA_CHECK(cudaMemcpyAsync(&h, out_actual, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    if (h.status) fail(CR_TIMEOUT, "multiscale grid barrier timed out");
    if (comp_x && h.actual > 0) {
        const size_t nb = (size_t)h.actual * 4;
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_x, cx, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_y, cy, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_scale, cs, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_strength, cst, nb, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_flux, cf, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    }
    if (actual) *actual = h.actual;
    if (reported) *reported = std::min<int64_t>(h.actual, cycle_niter);
    // -1 marks the divergence rule (CleanStopReason::DivergenceDetected)
    if (stop_out) *stop_out = h.stop;
}

}  // namespace cr

// ---- C ABI -------------------------------------------------------------------------
extern "C" int cr_multiscale_create(cr_ctx* ctx, const float* psf, const uint8_t* mask,
                                    int32_t nx, int32_t ny, int32_t location,
                                    const float* scales, int32_t nscales,
                                    float small_scale_bias, cr_multiscale** out, char** err) {
    return cr::guarded(err, [&] {
        if (!ctx || !psf || !out) cr::fail(CR_INVALID, "null argument");
        *out = nullptr;
        if (nx <= 1 || ny <= 1) cr::fail(CR_INVALID, "image shape must be at least 2 x 2");
        if ((int64_t)nx * ny >= (1ll << 31)) cr::fail(CR_INVALID, "image larger than 2^31 pixels");
        if (nscales < 0 || nscales > cr::kMaxScales || (nscales > 0 && !scales))
            cr::fail(CR_INVALID, "between 0 and 16 scales");
        for (int k = 0; k < nscales; ++k)
            if (!(scales[k] >= 0.0f) || !std::isfinite(scales[k]))
                cr::fail(CR_INVALID, "scales must be finite and non-negative");
        if (location != CR_HOST && location != CR_DEVICE) cr::fail(CR_INVALID, "bad location");
        CR_CUDA_CHECK(cudaSetDevice(ctx->device));
        const size_t n = (size_t)nx * ny;
        const float* p = (const float*)cr::device_input(ctx, psf, n * 4, location, "ms_psf");
        const uint8_t* m = (const uint8_t*)cr::device_input(ctx, mask, n, location, "ms_mask");
        cr_multiscale* ms = new cr_multiscale();
        ms->ctx = ctx;
        ms->nx = nx;
        ms->ny = ny;
        if (nscales == 0)
            ms->scales = {0.0f};   // effective_multiscale_scales (lib.rs:64164-64170)
        else
            ms->scales.assign(scales, scales + nscales);
        ms->K = (int)ms->scales.size();
        try {
            cr::multiscale_create(ms, p, m, small_scale_bias);
        } catch (...) {
            cr::pool_free(ctx, ms->pool);
            delete ms;
            throw;
        }
        *out = ms;
    });
}

extern "C" void cr_multiscale_destroy(cr_multiscale* ms) {
    if (!ms) return;
    cudaSetDevice(ms->ctx->device);
    cudaStreamSynchronize(ms->ctx->stream);
    cr::pool_free(ms->ctx, ms->pool);
    cudaStreamSynchronize(ms->ctx->stream);
    delete ms;
}

extern "C" int cr_multiscale_set_residual(cr_multiscale* ms, const float* residual,
                                          int32_t location, char** err) {
    return cr::guarded(err, [&] {
        if (!ms || !residual) cr::fail(CR_INVALID, "null argument");
        CR_CUDA_CHECK(cudaSetDevice(ms->ctx->device));
        const float* r = (const float*)cr::device_input(
            ms->ctx, residual, (size_t)ms->nx * ms->ny * 4, location, "ms_residual");
        cr::multiscale_set_residual(ms, r);
        CR_CUDA_CHECK(cudaStreamSynchronize(ms->ctx->stream));
    });
}

extern "C" int cr_multiscale_residual(cr_multiscale* ms, float* out, int32_t location,
                                      char** err) {
    return cr::guarded(err, [&] {
        if (!ms || !out) cr::fail(CR_INVALID, "null argument");
        CR_CUDA_CHECK(cudaSetDevice(ms->ctx->device));
        cr::copy_out(ms->ctx, out, ms->dirty, (size_t)ms->nx * ms->ny * 4, location);
        CR_CUDA_CHECK(cudaStreamSynchronize(ms->ctx->stream));
    });
}

extern "C" int cr_multiscale_peak(cr_multiscale* ms, int32_t* has_candidate, float* peak0,
                                  char** err) {
    return cr::guarded(err, [&] {
        if (!ms) cr::fail(CR_INVALID, "null argument");
        CR_CUDA_CHECK(cudaSetDevice(ms->ctx->device));
        cr::multiscale_peak(ms, has_candidate, peak0);
    });
}

extern "C" int cr_multiscale_minor_cycle(cr_multiscale* ms, float* model, int32_t location,
                                         float gain, float threshold, float cycle_threshold,
                                         float nsigma_threshold, int64_t cycle_niter,
                                         int32_t* comp_x, int32_t* comp_y, int32_t* comp_scale,
                                         float* comp_strength, float* comp_flux,
                                         int64_t* actual, int64_t* reported,
                                         int32_t* stop_reason, char** err) {
    return cr::guarded(err, [&] {
        if (!ms || !model) cr::fail(CR_INVALID, "null argument");
        if (!comp_x != !comp_y || !comp_x != !comp_scale || !comp_x != !comp_strength ||
            !comp_x != !comp_flux)
            cr::fail(CR_INVALID, "component arrays must be all given or all null");
        if (location != CR_HOST && location != CR_DEVICE) cr::fail(CR_INVALID, "bad location");
        cr_ctx* ctx = ms->ctx;
        CR_CUDA_CHECK(cudaSetDevice(ctx->device));
        const size_t nb = (size_t)ms->nx * ms->ny * 4;
        float* m = location == CR_DEVICE ? model : (float*)cr::workspace(ctx, "ms_model", nb);
        if (location == CR_HOST)
            CR_CUDA_CHECK(cudaMemcpyAsync(m, model, nb, cudaMemcpyHostToDevice, ctx->stream));
        cr::multiscale_minor_cycle(ms, m, gain, threshold, cycle_threshold, nsigma_threshold,
                                   cycle_niter, comp_x, comp_y, comp_scale, comp_strength,
                                   comp_flux, actual, reported, stop_reason);
        if (location == CR_HOST)
            CR_CUDA_CHECK(cudaMemcpyAsync(model, m, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}
