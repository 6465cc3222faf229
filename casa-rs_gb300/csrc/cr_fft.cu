// cr_fft.cu -- the centred-FFT, grid-correction and normalisation stage.
//
// For even grid sizes the reference's centred transforms (ifftshift, DFT,
// fftshift; fft.rs:600-630, 969-1070) equal a checkerboard-modulated plain
// DFT: centred(g)[m] = (-1)^(mx+my+hx+hy) DFT((-1)^(kx+ky) g)[m], hx = Nx/2.
// The input modulation is fused with the widening of the FP32 grid to FP64,
// cuFFT does the bare transform, and the output modulation is folded into
// the crop and correction kernel (gridder.rs:1646-1657, 1685-1715) or into
// the narrowing of the model grid to FP32.
// Only real parts leave the stage: the image is Re(IDFT(g)), which equals the
// real inverse transform (C2R) of g's Hermitian part h(k) = (g(k) +
// conj(g(-k))) / 2, and the model grid is the DFT of a real image, whose
// upper half follows from the lower by the same symmetry.  So the bare
// transforms are C2R and R2C over half spectra: half the arithmetic of the
// complex transforms, which matters for FP64 on this part.
// The transform runs in FP64 like the reference's standard-gridder FFT
// (fft.rs:600-630 on Complex64 grids): the grid correction amplifies FFT
// rounding near the image edge by up to 1/grdsf, which an FP32 transform
// would carry into the image at the 1e-6 level.
#include <algorithm>

#include "cr_internal.cuh"

namespace cr {

namespace {

// The FP64 transforms work on double2, the float32 ones (cube images) on
// float2; sign flips are exact in either.
__device__ __forceinline__ double2 make_work(double re, double im, double2*) {
    return make_double2(re, im);
}
__device__ __forceinline__ float2 make_work(float re, float im, float2*) {
    return make_float2(re, im);
}

// h[kx][ky] = (-1)^(kx+ky) (g[k] + conj(g[-k])) / 2 for ky in [0, gny/2]
// (indices mod the grid size; both points of a pair carry the same sign on
// even grids): the input of the real inverse transform.  real_g: a PSF grid
// kept as its float32 real part.
template <typename W>
__device__ __forceinline__ void hermitian_half_body(const float2* g, const float* real_g,
                                                    int64_t gnx,
                                      int64_t gny, W* h) {
    using S = decltype(h->x);
    const int64_t hy = gny / 2 + 1, n = gnx * hy;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kx = t / hy, ky = t - kx * hy;
        const int64_t mx = kx == 0 ? 0 : gnx - kx, my = ky == 0 ? 0 : gny - ky;
        S re, im = S(0);
        if (real_g) {
            re = ((S)real_g[kx * gny + ky] + (S)real_g[mx * gny + my]) * S(0.5);
        } else {
            const float2 a = g[kx * gny + ky], b = g[mx * gny + my];
            re = ((S)a.x + (S)b.x) * S(0.5);
            im = ((S)a.y - (S)b.y) * S(0.5);
        }
        if ((kx + ky) & 1) {
            re = -re;
            im = -im;
        }
        h[t] = make_work(re, im, h);
    }
}

template <typename W>
__global__ void hermitian_half_kernel(const float2* g, const float* real_g, int64_t gnx,
                                      int64_t gny, W* h) {
    hermitian_half_body(g, real_g, gnx, gny, h);
}

// image(x, y) = Re(raw[blc + (x, y)]) * sign * scale * corr_x * corr_y.
// sinc_mode 1 (W-projection image correction) further divides by
// sinc_x * sinc_y with the reference's 1e-6 guard; sinc_mode 2 multiplies by
// it, which is the transpose of the W-projection model apodisation.
template <typename S>
__device__ __forceinline__ void crop_correct_body(const S* raw, int64_t gny, int32_t nx, int32_t ny,
                                    int64_t blc_x, int64_t blc_y, int parity, double scale,
                                    const float* corr_x, const float* corr_y, const float* sx,
                                    const float* sy, int sinc_mode, float* image) {
    const int64_t n = (int64_t)nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = t / ny, y = t - x * ny;
        int64_t gx = blc_x + x, gy = blc_y + y;
        double r = (double)raw[gx * gny + gy];
        if ((gx + gy + parity) & 1) r = -r;
        float v = (float)(r * scale);
        float factor = __fmul_rn(corr_x[gx], corr_y[gy]);
        if (sinc_mode == 1) {
            float sf = __fmul_rn(sx[gx], sy[gy]);
            v = fabsf(sf) > 1.0e-6f ? v * (factor / sf) : 0.0f;
        } else if (sinc_mode == 2) {
            v = v * __fmul_rn(__fmul_rn(factor, sx[gx]), sy[gy]);
        } else {
            v = v * factor;
        }
        image[t] = v;
    }
}

template <typename S>
__global__ void crop_correct_kernel(const S* raw, int64_t gny, int32_t nx, int32_t ny,
                                    int64_t blc_x, int64_t blc_y, int parity, double scale,
                                    const float* corr_x, const float* corr_y, const float* sx,
                                    const float* sy, int sinc_mode, float* image) {
    crop_correct_body(raw, gny, nx, ny, blc_x, blc_y, parity, scale, corr_x, corr_y, sx, sy,
                      sinc_mode, image);
}

// apodize_model / apodize_w_project_model (gridder.rs:1554-1592) into a
// zeroed grid, with the input checkerboard of the centred forward FFT.
template <typename S>
__device__ __forceinline__ void apodize_body(const float* model, int32_t nx, int32_t ny,
                                             int64_t gny,
                               int64_t blc_x, int64_t blc_y, const float* corr_x,
                               const float* corr_y, const float* sinc_x, const float* sinc_y,
                               S* grid) {
    const int64_t n = (int64_t)nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = t / ny, y = t - x * ny;
        int64_t gx = blc_x + x, gy = blc_y + y;
        float f = __fmul_rn(corr_x[gx], corr_y[gy]);
        if (sinc_x) f = __fmul_rn(__fmul_rn(f, sinc_x[gx]), sinc_y[gy]);
        float v = model[t] * f;
        if ((gx + gy) & 1) v = -v;
        grid[gx * gny + gy] = (S)v;
    }
}

template <typename S>
__global__ void apodize_kernel(const float* model, int32_t nx, int32_t ny, int64_t gny,
                               int64_t blc_x, int64_t blc_y, const float* corr_x,
                               const float* corr_y, const float* sinc_x, const float* sinc_y,
                               S* grid) {
    apodize_body(model, nx, ny, gny, blc_x, blc_y, corr_x, corr_y, sinc_x, sinc_y, grid);
}

// The full model grid from the half spectrum of the real forward transform:
// G[x][y] = half[x][y] for y <= gny/2, conj(half[-x][-y]) above; then the
// output checkerboard and the narrowing to float32.
template <typename W>
__device__ __forceinline__ void narrow_sign_body(const W* half, int64_t gnx, int64_t gny,
                                                 int parity,
                                   float2* out) {
    const int64_t n = gnx * gny, hy = gny / 2 + 1;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = t / gny, y = t - x * gny;
        float re, im;
        if (y < hy) {
            const W v = half[x * hy + y];
            re = (float)v.x;
            im = (float)v.y;
        } else {
            const W v = half[(x == 0 ? 0 : gnx - x) * hy + (gny - y)];
            re = (float)v.x;
            im = -(float)v.y;
        }
        if ((x + y + parity) & 1) {
            re = -re;
            im = -im;
        }
        out[t] = make_float2(re, im);
    }
}

template <typename W>
__global__ void narrow_sign_kernel(const W* half, int64_t gnx, int64_t gny, int parity,
                                   float2* out) {
    narrow_sign_body(half, gnx, gny, parity, out);
}

__global__ void abs_peak_kernel(const float* img, int64_t n, unsigned int* peak) {
    float m = 0.0f;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        float v = fabsf(img[t]);
        if (v > m) m = v;  // NaN never raises the peak, as f32::max
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(peak, __float_as_uint(m));
}

__global__ void scale_image_kernel(float* img, int64_t n, float scale, const unsigned int* peak) {
    float p = peak ? __uint_as_float(*peak) : 1.0f;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        float v = img[t] * scale;
        if (peak) v = v / p;
        img[t] = v;
    }
}

}  // namespace

// The bare transforms, out of place: C2R for images (Z2D in FP64, C2R in
// float32), R2C for model grids.  A C2R transform may overwrite its input,
// which is scratch here.
static void exec_c2r(cr_ctx* ctx, int64_t gnx, int64_t gny, double2* in, double* out) {
    check_cufft(cufftExecZ2D(fft_plan_type(ctx, gnx, gny, CUFFT_Z2D), (cufftDoubleComplex*)in,
                             (cufftDoubleReal*)out),
                "cufftExecZ2D");
}
static void exec_c2r(cr_ctx* ctx, int64_t gnx, int64_t gny, float2* in, float* out) {
    check_cufft(cufftExecC2R(fft_plan_type(ctx, gnx, gny, CUFFT_C2R), (cufftComplex*)in,
                             (cufftReal*)out),
                "cufftExecC2R");
}
static void exec_r2c(cr_ctx* ctx, int64_t gnx, int64_t gny, double* in, double2* out) {
    check_cufft(cufftExecD2Z(fft_plan_type(ctx, gnx, gny, CUFFT_D2Z), (cufftDoubleReal*)in,
                             (cufftDoubleComplex*)out),
                "cufftExecD2Z");
}
static void exec_r2c(cr_ctx* ctx, int64_t gnx, int64_t gny, float* in, float2* out) {
    check_cufft(cufftExecR2C(fft_plan_type(ctx, gnx, gny, CUFFT_R2C), (cufftReal*)in,
                             (cufftComplex*)out),
                "cufftExecR2C");
}

template <typename W>
static void grid_to_image_impl(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float2* grid,
                               float scale, float* image, bool adjoint, const float* real_grid) {
    using S = decltype(W::x);
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    if ((gnx & 1) || (gny & 1)) fail(CR_INVALID, "grid sizes must be even");
    const bool f64 = sizeof(S) == 8;
    int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    double inv = 1.0 / ((double)gnx * (double)gny);
    const int64_t n = (int64_t)g->geom.nx * g->geom.ny;
    const float* sx = nullptr;
    const float* sy = nullptr;
    int mode = 0;
    if (wp) {
        mode = adjoint ? 2 : 1;
        sx = adjoint ? wp->sinc_gx_d : wp->sinc_x_d;
        sy = adjoint ? wp->sinc_gy_d : wp->sinc_x_d;
    }
    if (f64 && ctx->image_fft_engine == 0 && dfft_supported(gnx, gny)) {
        dfft_grid_to_image(ctx, g, grid, real_grid, inv * (double)scale, sx, sy, mode, image);
        return;
    }
    const int64_t nh = gnx * (gny / 2 + 1);
    W* half = (W*)workspace(ctx, f64 ? "fft_h64" : "fft_h32", (size_t)nh * sizeof(W));
    S* raw = (S*)workspace(ctx, f64 ? "fft_r64" : "fft_r32", (size_t)gnx * gny * sizeof(S));
    hermitian_half_kernel<W><<<grid_blocks(nh, 256), 256, 0, ctx->stream>>>(
        grid, real_grid, gnx, gny, half);
    note_launch(ctx, "hermitian_half_kernel");
    exec_c2r(ctx, gnx, gny, half, raw);
    crop_correct_kernel<S><<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(
        raw, gny, g->geom.nx, g->geom.ny, g->info.blc_x, g->info.blc_y, parity,
        inv * (double)scale, g->corr_x_d, g->corr_y_d, sx, sy, mode, image);
    note_launch(ctx, "crop_correct_kernel");
}

template <typename W>
static void image_to_grid_impl(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float* model,
                               float2* grid) {
    using S = decltype(W::x);
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    if ((gnx & 1) || (gny & 1)) fail(CR_INVALID, "grid sizes must be even");
    const bool f64 = sizeof(S) == 8;
    if (f64 && ctx->image_fft_engine == 0 && dfft_supported(gnx, gny)) {
        dfft_image_to_grid(ctx, g, model, wp ? wp->sinc_gx_d : nullptr,
                           wp ? wp->sinc_gy_d : nullptr, grid);
        return;
    }
    const int64_t nh = gnx * (gny / 2 + 1);
    W* half = (W*)workspace(ctx, f64 ? "fft_h64" : "fft_h32", (size_t)nh * sizeof(W));
    S* raw = (S*)workspace(ctx, f64 ? "fft_r64" : "fft_r32", (size_t)gnx * gny * sizeof(S));
    CR_CUDA_CHECK(cudaMemsetAsync(raw, 0, (size_t)gnx * gny * sizeof(S), ctx->stream));
    const int64_t n = (int64_t)g->geom.nx * g->geom.ny;
    apodize_kernel<S><<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(
        model, g->geom.nx, g->geom.ny, gny, g->info.blc_x, g->info.blc_y, g->corr_x_d,
        g->corr_y_d, wp ? wp->sinc_gx_d : nullptr, wp ? wp->sinc_gy_d : nullptr, raw);
    note_launch(ctx, "apodize_kernel");
    exec_r2c(ctx, gnx, gny, raw, half);
    int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    narrow_sign_kernel<W><<<grid_blocks(gnx * gny, 256), 256, 0, ctx->stream>>>(half, gnx, gny,
                                                                               parity, grid);
    note_launch(ctx, "narrow_sign_kernel");
}

// ---- the same stage over planes of a cube, kPlaneBatch planes per cuFFT call ----
namespace {

constexpr int kPlaneBatch = 16;

struct PlaneChunk {
    int plane[kPlaneBatch];   // cube plane of batch entry b
    float scale[kPlaneBatch]; // its image scale (grid_to_image's `scale`)
};

template <typename W>
__global__ void hermitian_half_planes(const float2* grids, const float* real_grids,
                                      int64_t gnx, int64_t gny, PlaneChunk pc, W* half) {
    const int64_t cells = gnx * gny, nh = gnx * (gny / 2 + 1);
    const int b = blockIdx.y;
    const int64_t p = pc.plane[b];
    hermitian_half_body(grids ? grids + p * cells : nullptr,
                        real_grids ? real_grids + p * cells : nullptr, gnx, gny, half + b * nh);
}

template <typename S>
__global__ void crop_correct_planes(const S* raw, int64_t gnx, int64_t gny, int32_t nx,
                                    int32_t ny, int64_t blc_x, int64_t blc_y, int parity,
                                    double inv, PlaneChunk pc, const float* corr_x,
                                    const float* corr_y, float* images) {
    const int b = blockIdx.y;
    crop_correct_body(raw + b * gnx * gny, gny, nx, ny, blc_x, blc_y, parity,
                      inv * (double)pc.scale[b], corr_x, corr_y, nullptr, nullptr, 0,
                      images + (int64_t)pc.plane[b] * nx * ny);
}

template <typename S>
__global__ void apodize_planes(const float* models, int32_t nx, int32_t ny, int64_t gnx,
                               int64_t gny, int64_t blc_x, int64_t blc_y, const float* corr_x,
                               const float* corr_y, PlaneChunk pc, S* raw) {
    const int b = blockIdx.y;
    apodize_body(models + (int64_t)pc.plane[b] * nx * ny, nx, ny, gny, blc_x, blc_y, corr_x,
                 corr_y, nullptr, nullptr, raw + b * gnx * gny);
}

template <typename W>
__global__ void narrow_sign_planes(const W* half, int64_t gnx, int64_t gny, int parity,
                                   PlaneChunk pc, float2* grids) {
    const int b = blockIdx.y;
    narrow_sign_body(half + b * gnx * (gny / 2 + 1), gnx, gny, parity,
                     grids + (int64_t)pc.plane[b] * gnx * gny);
}

// abs_peak_kernel / scale_image_kernel over the planes of a chunk
__global__ void abs_peak_planes_kernel(const float* images, int64_t n, PlaneChunk pc,
                                       unsigned int* peaks) {
    const int64_t p = pc.plane[blockIdx.y];
    const float* img = images + p * n;
    float m = 0.0f;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        float v = fabsf(img[t]);
        if (v > m) m = v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(peaks + p, __float_as_uint(m));
}

__global__ void scale_planes(float* images, int64_t n, PlaneChunk pc, const unsigned int* peaks) {
    const int64_t p = pc.plane[blockIdx.y];
    float* img = images + p * n;
    const float scale = pc.scale[blockIdx.y];
    const float pk = peaks ? __uint_as_float(peaks[p]) : 1.0f;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        float v = img[t] * scale;
        if (peaks) v = v / pk;
        img[t] = v;
    }
}

void exec_c2r_many(cr_ctx* ctx, int64_t gnx, int64_t gny, int n, double2* in, double* out) {
    check_cufft(cufftExecZ2D(fft_plan_many(ctx, gnx, gny, CUFFT_Z2D, n),
                             (cufftDoubleComplex*)in, (cufftDoubleReal*)out),
                "cufftExecZ2D");
}
void exec_c2r_many(cr_ctx* ctx, int64_t gnx, int64_t gny, int n, float2* in, float* out) {
    check_cufft(cufftExecC2R(fft_plan_many(ctx, gnx, gny, CUFFT_C2R, n), (cufftComplex*)in,
                             (cufftReal*)out),
                "cufftExecC2R");
}
void exec_r2c_many(cr_ctx* ctx, int64_t gnx, int64_t gny, int n, double* in, double2* out) {
    check_cufft(cufftExecD2Z(fft_plan_many(ctx, gnx, gny, CUFFT_D2Z, n), (cufftDoubleReal*)in,
                             (cufftDoubleComplex*)out),
                "cufftExecD2Z");
}
void exec_r2c_many(cr_ctx* ctx, int64_t gnx, int64_t gny, int n, float* in, float2* out) {
    check_cufft(cufftExecR2C(fft_plan_many(ctx, gnx, gny, CUFFT_R2C, n), (cufftReal*)in,
                             (cufftComplex*)out),
                "cufftExecR2C");
}

template <typename W>
void grid_to_image_planes_impl(cr_ctx* ctx, cr_gridder* g, const float2* grids,
                               const float* real_grids, const std::vector<int>& planes,
                               const std::vector<float>& scales, float* images) {
    using S = decltype(W::x);
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    if ((gnx & 1) || (gny & 1)) fail(CR_INVALID, "grid sizes must be even");
    const bool f64 = sizeof(S) == 8;
    const int64_t nh = gnx * (gny / 2 + 1);
    W* half = (W*)workspace(ctx, f64 ? "fftp_h64" : "fftp_h32",
                            (size_t)nh * kPlaneBatch * sizeof(W));
    S* raw = (S*)workspace(ctx, f64 ? "fftp_r64" : "fftp_r32",
                           (size_t)gnx * gny * kPlaneBatch * sizeof(S));
    const int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    const double inv = 1.0 / ((double)gnx * (double)gny);
    const int64_t n = (int64_t)g->geom.nx * g->geom.ny;
    for (size_t k0 = 0; k0 < planes.size(); k0 += kPlaneBatch) {
        const int nb = (int)std::min<size_t>(kPlaneBatch, planes.size() - k0);
        PlaneChunk pc{};
        for (int b = 0; b < nb; ++b) {
            pc.plane[b] = planes[k0 + b];
            pc.scale[b] = scales[k0 + b];
        }
        hermitian_half_planes<W><<<dim3(grid_blocks(nh, 256, ctx->sms * 4), nb), 256, 0,
                                   ctx->stream>>>(grids, real_grids, gnx, gny, pc, half);
        note_launch(ctx, "hermitian_half_planes");
        exec_c2r_many(ctx, gnx, gny, nb, half, raw);
        crop_correct_planes<S><<<dim3(grid_blocks(n, 256, ctx->sms * 4), nb), 256, 0, ctx->stream>>>(
            raw, gnx, gny, g->geom.nx, g->geom.ny, g->info.blc_x, g->info.blc_y, parity, inv,
            pc, g->corr_x_d, g->corr_y_d, images);
        note_launch(ctx, "crop_correct_planes");
    }
}

template <typename W>
void image_to_grid_planes_impl(cr_ctx* ctx, cr_gridder* g, const float* models,
                               const std::vector<int>& planes, float2* grids) {
    using S = decltype(W::x);
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    if ((gnx & 1) || (gny & 1)) fail(CR_INVALID, "grid sizes must be even");
    const bool f64 = sizeof(S) == 8;
    const int64_t nh = gnx * (gny / 2 + 1);
    W* half = (W*)workspace(ctx, f64 ? "fftp_h64" : "fftp_h32",
                            (size_t)nh * kPlaneBatch * sizeof(W));
    S* raw = (S*)workspace(ctx, f64 ? "fftp_r64" : "fftp_r32",
                           (size_t)gnx * gny * kPlaneBatch * sizeof(S));
    const int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    const int64_t n = (int64_t)g->geom.nx * g->geom.ny;
    for (size_t k0 = 0; k0 < planes.size(); k0 += kPlaneBatch) {
        const int nb = (int)std::min<size_t>(kPlaneBatch, planes.size() - k0);
        PlaneChunk pc{};
        for (int b = 0; b < nb; ++b) pc.plane[b] = planes[k0 + b];
        CR_CUDA_CHECK(cudaMemsetAsync(raw, 0, (size_t)gnx * gny * nb * sizeof(S), ctx->stream));
        apodize_planes<S><<<dim3(grid_blocks(n, 256, ctx->sms * 4), nb), 256, 0, ctx->stream>>>(
            models, g->geom.nx, g->geom.ny, gnx, gny, g->info.blc_x, g->info.blc_y, g->corr_x_d,
            g->corr_y_d, pc, raw);
        note_launch(ctx, "apodize_planes");
        exec_r2c_many(ctx, gnx, gny, nb, raw, half);
        narrow_sign_planes<W><<<dim3(grid_blocks(gnx * gny, 256, ctx->sms * 4), nb), 256, 0,
                                ctx->stream>>>(half, gnx, gny, parity, pc, grids);
        note_launch(ctx, "narrow_sign_planes");
    }
}

}  // namespace

void abs_peak_planes(cr_ctx* ctx, const float* images, int64_t n,
                     const std::vector<int>& planes, unsigned int* peaks) {
    for (size_t k0 = 0; k0 < planes.size(); k0 += kPlaneBatch) {
        const int nb = (int)std::min<size_t>(kPlaneBatch, planes.size() - k0);
        PlaneChunk pc{};
        for (int b = 0; b < nb; ++b) pc.plane[b] = planes[k0 + b];
        abs_peak_planes_kernel<<<dim3(grid_blocks(n, 256, ctx->sms * 4), nb), 256, 0,
                                 ctx->stream>>>(images, n, pc, peaks);
        note_launch(ctx, "abs_peak_planes_kernel");
    }
}

void scale_image_planes(cr_ctx* ctx, float* images, int64_t n, const std::vector<int>& planes,
                        const std::vector<float>& scales, const unsigned int* peaks) {
    for (size_t k0 = 0; k0 < planes.size(); k0 += kPlaneBatch) {
        const int nb = (int)std::min<size_t>(kPlaneBatch, planes.size() - k0);
        PlaneChunk pc{};
        for (int b = 0; b < nb; ++b) {
            pc.plane[b] = planes[k0 + b];
            pc.scale[b] = scales[k0 + b];
        }
        scale_planes<<<dim3(grid_blocks(n, 256, ctx->sms * 4), nb), 256, 0, ctx->stream>>>(
            images, n, pc, peaks);
        note_launch(ctx, "scale_planes");
    }
}

void grid_to_image_planes(cr_ctx* ctx, cr_gridder* g, const float2* grids,
                          const float* real_grids, const std::vector<int>& planes,
                          const std::vector<float>& scales, float* images, bool single) {
    if (single)
        grid_to_image_planes_impl<float2>(ctx, g, grids, real_grids, planes, scales, images);
    else
        grid_to_image_planes_impl<double2>(ctx, g, grids, real_grids, planes, scales, images);
}

void image_to_grid_planes(cr_ctx* ctx, cr_gridder* g, const float* models,
                          const std::vector<int>& planes, float2* grids, bool single) {
    if (single)
        image_to_grid_planes_impl<float2>(ctx, g, models, planes, grids);
    else
        image_to_grid_planes_impl<double2>(ctx, g, models, planes, grids);
}

void grid_to_image(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, float2* grid, float scale,
                   float* image, bool single) {
    if (single)
        grid_to_image_impl<float2>(ctx, g, wp, grid, scale, image, false, nullptr);
    else
        grid_to_image_impl<double2>(ctx, g, wp, grid, scale, image, false, nullptr);
}

void grid_to_image_real(cr_ctx* ctx, cr_gridder* g, const float* grid, float scale,
                        float* image, bool single) {
    if (single)
        grid_to_image_impl<float2>(ctx, g, nullptr, nullptr, scale, image, false, grid);
    else
        grid_to_image_impl<double2>(ctx, g, nullptr, nullptr, scale, image, false, grid);
}

void grid_to_image_adjoint(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, float2* grid, float scale,
                           float* image, bool single) {
    if (single)
        grid_to_image_impl<float2>(ctx, g, wp, grid, scale, image, true, nullptr);
    else
        grid_to_image_impl<double2>(ctx, g, wp, grid, scale, image, true, nullptr);
}

void image_to_grid(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float* model, float2* grid,
                   bool single) {
    if (single)
        image_to_grid_impl<float2>(ctx, g, wp, model, grid);
    else
        image_to_grid_impl<double2>(ctx, g, wp, model, grid);
}

void abs_peak(cr_ctx* ctx, const float* image, int64_t n, unsigned int* peak_dev) {
    CR_CUDA_CHECK(cudaMemsetAsync(peak_dev, 0, 4, ctx->stream));
    abs_peak_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(image, n, peak_dev);
    note_launch(ctx, "abs_peak_kernel");
}

void scale_image(cr_ctx* ctx, float* image, int64_t n, float scale, const unsigned int* peak_dev) {
    scale_image_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(image, n, scale, peak_dev);
    note_launch(ctx, "scale_image_kernel");
}

}  // namespace cr
