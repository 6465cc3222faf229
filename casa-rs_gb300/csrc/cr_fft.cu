// cr_fft.cu -- the centred-FFT, grid-correction and normalisation stage.
//
// For even grid sizes the reference's centred transforms (ifftshift, DFT,
// fftshift; fft.rs:600-630, 969-1070) equal a checkerboard-modulated plain
// DFT: centred(g)[m] = (-1)^(mx+my+hx+hy) DFT((-1)^(kx+ky) g)[m], hx = Nx/2.
// The input modulation is fused with the widening of the FP32 grid to FP64,
// cuFFT does the bare transform (double precision, in place), and the output
// modulation is folded into the crop and correction kernel (gridder.rs:
// 1646-1657, 1685-1715) or into the narrowing of the model grid to FP32.
// The transform runs in FP64 like the reference's standard-gridder FFT
// (fft.rs:600-630 on Complex64 grids): the grid correction amplifies FFT
// rounding near the image edge by up to 1/grdsf, which an FP32 transform
// would carry into the image at the 1e-6 level.
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

template <typename W>
__global__ void widen_checker_kernel(const float2* g, int64_t gnx, int64_t gny, W* out) {
    using S = decltype(out->x);
    const int64_t n = gnx * gny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = t / gny, y = t - x * gny;
        float2 v = g[t];
        S s = ((x + y) & 1) ? S(-1) : S(1);
        out[t] = make_work(s * (S)v.x, s * (S)v.y, out);
    }
}

// The real part alone (a PSF grid kept as float32).
template <typename W>
__global__ void widen_checker_real_kernel(const float* g, int64_t gnx, int64_t gny, W* out) {
    using S = decltype(out->x);
    const int64_t n = gnx * gny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = t / gny, y = t - x * gny;
        S s = ((x + y) & 1) ? S(-1) : S(1);
        out[t] = make_work(s * (S)g[t], S(0), out);
    }
}

// image(x, y) = Re(raw[blc + (x, y)]) * sign * scale * corr_x * corr_y.
// sinc_mode 1 (W-projection image correction) further divides by
// sinc_x * sinc_y with the reference's 1e-6 guard; sinc_mode 2 multiplies by
// it, which is the transpose of the W-projection model apodisation.
template <typename W>
__global__ void crop_correct_kernel(const W* raw, int64_t gny, int32_t nx, int32_t ny,
                                    int64_t blc_x, int64_t blc_y, int parity, double scale,
                                    const float* corr_x, const float* corr_y, const float* sx,
                                    const float* sy, int sinc_mode, float* image) {
    const int64_t n = (int64_t)nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = t / ny, y = t - x * ny;
        int64_t gx = blc_x + x, gy = blc_y + y;
        double r = (double)raw[gx * gny + gy].x;
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

// apodize_model / apodize_w_project_model (gridder.rs:1554-1592) into a
// zeroed grid, with the input checkerboard of the centred forward FFT.
template <typename W>
__global__ void apodize_kernel(const float* model, int32_t nx, int32_t ny, int64_t gny,
                               int64_t blc_x, int64_t blc_y, const float* corr_x,
                               const float* corr_y, const float* sinc_x, const float* sinc_y,
                               W* grid) {
    using S = decltype(grid->x);
    const int64_t n = (int64_t)nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = t / ny, y = t - x * ny;
        int64_t gx = blc_x + x, gy = blc_y + y;
        float f = __fmul_rn(corr_x[gx], corr_y[gy]);
        if (sinc_x) f = __fmul_rn(__fmul_rn(f, sinc_x[gx]), sinc_y[gy]);
        float v = model[t] * f;
        if ((gx + gy) & 1) v = -v;
        grid[gx * gny + gy] = make_work((S)v, S(0), grid);
    }
}

template <typename W>
__global__ void narrow_sign_kernel(const W* g, int64_t gnx, int64_t gny, int parity,
                                   float2* out) {
    const int64_t n = gnx * gny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = t / gny, y = t - x * gny;
        W v = g[t];
        float re = (float)v.x, im = (float)v.y;
        if ((x + y + parity) & 1) {
            re = -re;
            im = -im;
        }
        out[t] = make_float2(re, im);
    }
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

// The bare transform in place: cuFFT Z2Z (FP64) or C2C (float32).
static void exec_fft(cr_ctx* ctx, int64_t gnx, int64_t gny, double2* work, int dir) {
    check_cufft(cufftExecZ2Z(fft_plan(ctx, gnx, gny), (cufftDoubleComplex*)work,
                             (cufftDoubleComplex*)work, dir),
                "cufftExecZ2Z");
}
static void exec_fft(cr_ctx* ctx, int64_t gnx, int64_t gny, float2* work, int dir) {
    check_cufft(cufftExecC2C(fft_plan_c2c(ctx, gnx, gny), (cufftComplex*)work,
                             (cufftComplex*)work, dir),
                "cufftExecC2C");
}

template <typename W>
static void grid_to_image_impl(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float2* grid,
                               float scale, float* image, bool adjoint, const float* real_grid) {
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    if ((gnx & 1) || (gny & 1)) fail(CR_INVALID, "grid sizes must be even");
    W* work = (W*)workspace(ctx, sizeof(W) == 16 ? "fft_z" : "fft_c",
                            (size_t)gnx * gny * sizeof(W));
    if (real_grid) {
        widen_checker_real_kernel<W><<<grid_blocks(gnx * gny, 256), 256, 0, ctx->stream>>>(
            real_grid, gnx, gny, work);
        note_launch(ctx, "widen_checker_real_kernel");
    } else {
        widen_checker_kernel<W><<<grid_blocks(gnx * gny, 256), 256, 0, ctx->stream>>>(
            grid, gnx, gny, work);
        note_launch(ctx, "widen_checker_kernel");
    }
    exec_fft(ctx, gnx, gny, work, CUFFT_INVERSE);
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
    crop_correct_kernel<W><<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(
        work, gny, g->geom.nx, g->geom.ny, g->info.blc_x, g->info.blc_y, parity,
        inv * (double)scale, g->corr_x_d, g->corr_y_d, sx, sy, mode, image);
    note_launch(ctx, "crop_correct_kernel");
}

template <typename W>
static void image_to_grid_impl(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float* model,
                               float2* grid) {
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    if ((gnx & 1) || (gny & 1)) fail(CR_INVALID, "grid sizes must be even");
    W* work = (W*)workspace(ctx, sizeof(W) == 16 ? "fft_z" : "fft_c",
                            (size_t)gnx * gny * sizeof(W));
    CR_CUDA_CHECK(cudaMemsetAsync(work, 0, (size_t)gnx * gny * sizeof(W), ctx->stream));
    const int64_t n = (int64_t)g->geom.nx * g->geom.ny;
    apodize_kernel<W><<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(
        model, g->geom.nx, g->geom.ny, gny, g->info.blc_x, g->info.blc_y, g->corr_x_d,
        g->corr_y_d, wp ? wp->sinc_gx_d : nullptr, wp ? wp->sinc_gy_d : nullptr, work);
    note_launch(ctx, "apodize_kernel");
    exec_fft(ctx, gnx, gny, work, CUFFT_FORWARD);
    int parity = (int)(((gnx / 2) + (gny / 2)) & 1);
    narrow_sign_kernel<W><<<grid_blocks(gnx * gny, 256), 256, 0, ctx->stream>>>(work, gnx, gny,
                                                                               parity, grid);
    note_launch(ctx, "narrow_sign_kernel");
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
