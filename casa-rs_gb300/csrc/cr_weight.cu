// cr_weight.cu -- natural, uniform and Briggs weighting.
//
// Restates apply_weighting_with_density_source (weighting.rs:1055-1180) in the
// Combined density mode, or with the cube PerPlane cells (rounded FP64
// u*scale + centre, weighting.rs:1455-1483): the density grid is image-sized, every sample
// with a finite positive weight adds its weight at its VisImagingWeight cell
// and at the cell of its Hermitian mirror (accumulate_density_sample_serial,
// weighting.rs:1831-1854; weight_density_cell_anchor, gridder.rs:1888-1934,
// whose float32 multiply-then-add order is kept with __fmul_rn/__fadd_rn);
// Briggs f2 = (5 * 10^-robust)^2 / (sum d^2 / sum d) with FP64 sums; the
// reweight divides by d (uniform) or by the CASA denominator d*f2 + 1 computed
// as a separate float multiply and add (casa_briggs_denominator,
// weighting.rs:2440-2443).
#include <cmath>

#include "cr_internal.cuh"

namespace cr {

namespace {

struct DensityCellParams {
    int32_t nx, ny;
    float u_scale, v_scale, cx, cy;
    int32_t convention;          // 0 VisImagingWeight, 1 cube PerPlane (rounded, FP64)
    double du_scale, dv_scale, dcx, dcy;
};

__device__ __forceinline__ bool density_cell(const DensityCellParams& p, double u, double v,
                                             int* ox, int* oy) {
    if (p.convention == 1) {
        // CubeBriggsWeightor{Density,Lookup}: u*scale + centre in FP64, rounded
        const double x = __dadd_rn(__dmul_rn(u, p.du_scale), p.dcx);
        const double y = __dadd_rn(__dmul_rn(-v, p.dv_scale), p.dcy);
        if (!isfinite(x) || !isfinite(y)) return false;
        const double rx = round(x), ry = round(y);
        if (!(rx >= 1.0 && ry >= 1.0 && rx < (double)p.nx && ry < (double)p.ny)) return false;
        *ox = (int)rx;
        *oy = (int)ry;
        return true;
    }
    float uf = __double2float_rn(u), vf = __double2float_rn(v);
    float x = __fadd_rn(__fmul_rn(-uf, p.u_scale), p.cx);
    float y = __fadd_rn(__fmul_rn(vf, p.v_scale), p.cy);
    if (!(isfinite(x) && isfinite(y))) return false;
    // trunc(x) in (0, nx) <=> 1 <= x < nx
    if (!(x >= 1.0f && x < (float)p.nx && y >= 1.0f && y < (float)p.ny)) return false;
    *ox = (int)x;
    *oy = (int)y;
    return true;
}

__global__ void density_kernel(const double* u, const double* v, const float* weight, int64_t n,
                               DensityCellParams p, float* density) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float w = weight[i];
        if (!(isfinite(w) && w > 0.0f)) continue;
        int x, y;
        if (density_cell(p, u[i], v[i], &x, &y)) atomicAdd(&density[(int64_t)x * p.ny + y], w);
        if (density_cell(p, -u[i], -v[i], &x, &y)) atomicAdd(&density[(int64_t)x * p.ny + y], w);
    }
}

__global__ void density_sums_kernel(const float* d, int64_t n, double* sums) {
    double s = 0.0, s2 = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double v = (double)d[i];
        s += v;
        if (v > 0.0) s2 += v * v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums[0], s);
        atomicAdd(&sums[1], s2);
    }
}

__global__ void reweight_kernel(const double* u, const double* v, const float* weight, int64_t n,
                                DensityCellParams p, const float* density, int mode, float f2,
                                float* out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float w = weight[i];
        if (mode == CR_WEIGHT_NATURAL) {
            out[i] = w;
            continue;
        }
        int x, y;
        float r = 0.0f;
        if (density_cell(p, u[i], v[i], &x, &y)) {
            float d = density[(int64_t)x * p.ny + y];
            if (isfinite(w) && w > 0.0f && isfinite(d) && d > 0.0f) {
                if (mode == CR_WEIGHT_UNIFORM)
                    r = __fdiv_rn(w, d);
                else
                    r = __fdiv_rn(w, __fadd_rn(__fmul_rn(d, f2), 1.0f));
            }
        }
        out[i] = r;
    }
}

}  // namespace

void apply_weighting(cr_ctx* ctx, cr_gridder* g, const DeviceBatch& b, int32_t mode,
                     float robust, float* out_weight, float* f2_out, int32_t convention,
                     const double* build_u, const double* build_v) {
    if (mode != CR_WEIGHT_NATURAL && mode != CR_WEIGHT_UNIFORM && mode != CR_WEIGHT_BRIGGS)
        fail(CR_INVALID, "unknown weighting mode");
    const int32_t nx = g->geom.nx, ny = g->geom.ny;
    DensityCellParams p;
    p.nx = nx;
    p.ny = ny;
    p.u_scale = (float)((double)nx * g->geom.cell_x_rad);
    p.v_scale = (float)((double)ny * g->geom.cell_y_rad);
    p.cx = (float)((double)nx / 2.0);
    p.cy = (float)((double)ny / 2.0);
    p.convention = convention;
    p.du_scale = (double)nx * g->geom.cell_x_rad;
    p.dv_scale = (double)ny * g->geom.cell_y_rad;
    p.dcx = (double)nx / 2.0;
    p.dcy = (double)ny / 2.0;
    float f2 = 0.0f;
    float* density = nullptr;
    if (mode != CR_WEIGHT_NATURAL) {
        density = (float*)workspace(ctx, "wt_density", (size_t)nx * ny * 4);
        CR_CUDA_CHECK(cudaMemsetAsync(density, 0, (size_t)nx * ny * 4, ctx->stream));
        if (b.n > 0) {
            // the density is built at build_u, build_v when given (the row
            // path's VisImagingWeight coordinates), looked up at u, v
            density_kernel<<<grid_blocks(b.n, 256), 256, 0, ctx->stream>>>(
                build_u ? build_u : b.u, build_v ? build_v : b.v, b.weight, b.n, p, density);
            note_launch(ctx, "density_kernel");
        }
        if (mode == CR_WEIGHT_BRIGGS) {
            double* sums = (double*)workspace(ctx, "wt_sums", 16);
            CR_CUDA_CHECK(cudaMemsetAsync(sums, 0, 16, ctx->stream));
            density_sums_kernel<<<grid_blocks((int64_t)nx * ny, 256), 256, 0, ctx->stream>>>(
                density, (int64_t)nx * ny, sums);
            note_launch(ctx, "density_sums_kernel");
            double h[2];
            CR_CUDA_CHECK(cudaMemcpyAsync(h, sums, 16, cudaMemcpyDeviceToHost, ctx->stream));
            CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
            if (h[1] > 0.0 && h[0] > 0.0) {
                double a = 5.0 * std::pow(10.0, -(double)robust);
                f2 = (float)(a * a / (h[1] / h[0]));
            }
        }
    }
    if (b.n > 0) {
        reweight_kernel<<<grid_blocks(b.n, 256), 256, 0, ctx->stream>>>(b.u, b.v, b.weight, b.n, p,
                                                                        density, mode, f2, out_weight);
        note_launch(ctx, "reweight_kernel");
    }
    if (f2_out) *f2_out = f2;
}

}  // namespace cr
