// cr_rows.cu -- row-runs to visibility samples on the device.
//
// Restates how casa-imaging turns MeasurementSet-shaped rows into weighted
// scalar samples (routed_weighted_grid_sample_from_run, lib.rs:880-1062, with
// the pair collapse of collapse_standard_mfs_pair_visibility,
// execution.rs:2323-2340, and ParallelHandBatch::collapse_with_transform,
// types.rs:2090-2160): per (row, channel) either one explicit correlation or
// a collapsed pair of parallel hands.  A sample is dropped when a used
// correlation is flagged, its visibility is not finite, a hand's weight is
// not finite and positive, the natural weight (the explicit weight, or the
// float32 mean 0.5 (w1 + w2) of a pair) is not finite and positive, or the
// plane's sumwt factor is not.  Weights come from WEIGHT_SPECTRUM when given,
// else from the row's WEIGHT.  u, v, w in wavelengths are the FP64 products
// uvw_m * lambda_scale; the density coordinates are the VisImagingWeight
// ones of casa_vis_imaging_weight_uv_lambda (weighting.rs:748-756): the
// float32 scale f/c, the FP64 product, rounded to float32.
//
// Two launches and a scan: the first marks the kept samples, an exclusive
// scan gives each its slot, the second writes the compacted batch in
// (row, channel) order.
#include "cr_internal.cuh"

namespace cr {

namespace {

struct RowArgs {
    int64_t R;
    int32_t C, ncorr;
    const double* uvw;
    const double* ls;          // [C] f / c, device copy
    const float2* data;        // [R][C][ncorr]
    const uint8_t* flag;       // [R][C][ncorr]
    const float* weight;       // [R][ncorr]
    const float* spectrum;     // [R][C][ncorr] or null
    const uint8_t* gridable;   // [R] or null
    int32_t mode, corr0, corr1, transform;
    float sumwt_factor;
};

// StandardMfsPairCollapseTransform::collapse in num-complex's operations
// (Complex32 * f32 scales both parts; a complex product is
// (a c - b d, a d + b c) without fused operations).
__device__ __forceinline__ float2 collapse(float2 a, float2 b, int transform) {
    if (transform == 0)
        return make_float2(__fmul_rn(__fadd_rn(a.x, b.x), 0.5f), __fmul_rn(__fadd_rn(a.y, b.y), 0.5f));
    const float dr = __fsub_rn(a.x, b.x), di = __fsub_rn(a.y, b.y);
    if (transform == 1) return make_float2(__fmul_rn(dr, 0.5f), __fmul_rn(di, 0.5f));
    const float s = transform == 2 ? 0.5f : -0.5f;   // multiply by (0, s)
    return make_float2(__fsub_rn(__fmul_rn(dr, 0.0f), __fmul_rn(di, s)),
                       __fadd_rn(__fmul_rn(dr, s), __fmul_rn(di, 0.0f)));
}

__device__ __forceinline__ bool pos_finite(float w) { return isfinite(w) && w > 0.0f; }

// The sample of (row r, channel c): false when it is dropped.
__device__ __forceinline__ bool row_sample(const RowArgs& a, int64_t r, int c, float2* vis,
                                           float* natural) {
    if (!pos_finite(a.sumwt_factor)) return false;
    const int64_t base = (r * a.C + c) * a.ncorr;
    if (a.mode == 0) {
        if (a.flag && a.flag[base + a.corr0]) return false;
        const float2 v = a.data[base + a.corr0];
        if (!(isfinite(v.x) && isfinite(v.y))) return false;
        const float w = a.spectrum ? a.spectrum[base + a.corr0] : a.weight[r * a.ncorr + a.corr0];
        if (!pos_finite(w)) return false;
        *vis = v;
        *natural = w;
        return true;
    }
    if (a.flag && (a.flag[base + a.corr0] || a.flag[base + a.corr1])) return false;
    const float2 v = collapse(a.data[base + a.corr0], a.data[base + a.corr1], a.transform);
    if (!(isfinite(v.x) && isfinite(v.y))) return false;
    const float w0 = a.spectrum ? a.spectrum[base + a.corr0] : a.weight[r * a.ncorr + a.corr0];
    const float w1 = a.spectrum ? a.spectrum[base + a.corr1] : a.weight[r * a.ncorr + a.corr1];
    if (!(pos_finite(w0) && pos_finite(w1))) return false;
    const float w = __fmul_rn(0.5f, __fadd_rn(w0, w1));
    if (!pos_finite(w)) return false;
    *vis = v;
    *natural = w;
    return true;
}

__global__ void rows_mark_kernel(RowArgs a, uint32_t* keep) {
    const int64_t n = a.R * a.C;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float2 v;
        float w;
        keep[i] = row_sample(a, i / a.C, (int)(i % a.C), &v, &w) ? 1u : 0u;
    }
}

struct RowOut {
    double *u, *v, *w, *du, *dv;
    float* weight;
    float* sumwt_factor;
    uint8_t* gridable;
    float2* vis;
};

__global__ void rows_write_kernel(RowArgs a, const uint32_t* keep, const uint32_t* slot,
                                  RowOut o) {
    const int64_t n = a.R * a.C;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        const int64_t r = i / a.C;
        const int c = (int)(i % a.C);
        float2 vis;
        float w;
        row_sample(a, r, c, &vis, &w);
        const uint32_t k = slot[i];
        const double ls = a.ls[c];
        const double um = a.uvw[3 * r], vm = a.uvw[3 * r + 1], wm = a.uvw[3 * r + 2];
        o.u[k] = __dmul_rn(um, ls);
        o.v[k] = __dmul_rn(vm, ls);
        o.w[k] = __dmul_rn(wm, ls);
        const double ls32 = (double)__double2float_rn(ls);
        o.du[k] = (double)__double2float_rn(__dmul_rn(um, ls32));
        o.dv[k] = (double)__double2float_rn(__dmul_rn(vm, ls32));
        o.weight[k] = w;
        o.sumwt_factor[k] = a.sumwt_factor;
        o.gridable[k] = a.gridable ? (a.gridable[r] ? 1 : 0) : 1;
        o.vis[k] = vis;
    }
}

}  // namespace

int64_t prepare_rows(cr_ctx* ctx, const cr_row_runs* rr, const cr_polarization* pol,
                     const RowsOut& out) {
    if (!rr || !pol) fail(CR_INVALID, "null argument");
    if (rr->rows < 0 || rr->channels <= 0 || rr->correlations <= 0)
        fail(CR_INVALID, "row runs need rows >= 0, channels > 0 and correlations > 0");
    if ((uint64_t)rr->rows * (uint64_t)rr->channels >= (1ull << 31))
        fail(CR_INVALID, "row runs larger than 2^31 samples");
    if (pol->mode != 0 && pol->mode != 1) fail(CR_INVALID, "polarization mode must be 0 or 1");
    if (pol->corr0 < 0 || pol->corr0 >= rr->correlations ||
        (pol->mode == 1 && (pol->corr1 < 0 || pol->corr1 >= rr->correlations)))
        fail(CR_INVALID, "polarization correlations exceed the correlation count");
    if (pol->mode == 1 && (pol->transform < 0 || pol->transform > 3))
        fail(CR_INVALID, "pair transform must be 0..3");
    if (!rr->lambda_scale) fail(CR_INVALID, "lambda_scale is null");
    const int64_t R = rr->rows, C = rr->channels, K = rr->correlations, n = R * C;
    if (R > 0 && (!rr->uvw_m || !rr->data || (!rr->weight && !rr->weight_spectrum)))
        fail(CR_INVALID, "row runs lack uvw, data or weights");
    RowArgs a{};
    a.R = R;
    a.C = (int32_t)C;
    a.ncorr = (int32_t)K;
    a.uvw = (const double*)device_input(ctx, rr->uvw_m, (size_t)R * 24, rr->location, "rr_uvw");
    a.data = (const float2*)device_input(ctx, rr->data, (size_t)n * K * 8, rr->location, "rr_data");
    a.flag = (const uint8_t*)device_input(ctx, rr->flag, (size_t)n * K, rr->location, "rr_flag");
    a.weight = (const float*)device_input(ctx, rr->weight, (size_t)R * K * 4, rr->location,
                                          "rr_weight");
    a.spectrum = (const float*)device_input(ctx, rr->weight_spectrum, (size_t)n * K * 4,
                                            rr->location, "rr_spectrum");
    a.gridable = (const uint8_t*)device_input(ctx, rr->gridable, (size_t)R, rr->location,
                                              "rr_gridable");
    double* ls = (double*)workspace(ctx, "rr_ls", (size_t)C * 8);
    CR_CUDA_CHECK(cudaMemcpyAsync(ls, rr->lambda_scale, (size_t)C * 8, cudaMemcpyHostToDevice,
                                  ctx->stream));
    a.ls = ls;
    a.mode = pol->mode;
    a.corr0 = pol->corr0;
    a.corr1 = pol->corr1;
    a.transform = pol->transform;
    a.sumwt_factor = pol->sumwt_factor;
    const size_t nn = (size_t)std::max<int64_t>(n, 1);
    uint32_t* keep = (uint32_t*)workspace(ctx, "rr_keep", nn * 4);
    uint32_t* slot = (uint32_t*)workspace(ctx, "rr_slot", nn * 4);
    unsigned long long* total = (unsigned long long*)workspace(ctx, "rr_total", 8);
    if (n > 0) {
        rows_mark_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(a, keep);
        note_launch(ctx, "rows_mark_kernel");
    }
    exclusive_scan_u32(ctx, keep, slot, n, total);
    if (n > 0) {
        RowOut o{out.u, out.v, out.w, out.du, out.dv, out.weight, out.sumwt_factor, out.gridable,
                 out.vis};
        rows_write_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(a, keep, slot, o);
        note_launch(ctx, "rows_write_kernel");
    }
    unsigned long long h = 0;
    CR_CUDA_CHECK(cudaMemcpyAsync(&h, total, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    return (int64_t)h;
}

}  // namespace cr
