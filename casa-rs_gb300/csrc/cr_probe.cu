// cr_probe.cu -- the tap-rate ceiling of the W-projection gridding loop.
//
// A W-projection tap is one complex kernel value read from the L2-resident
// residue cube plus three paired FP32 FMAs into the lane's accumulators
// (wp_grid_kernel).  This probe runs exactly that and nothing else: each
// warp reads 8 rows of 32 consecutive float2 values at scattered row
// addresses of a buffer the size of a benchmark cube (rows 65 elements
// apart, as the cube's rows are at support 64), and accumulates them into 8
// rows of (X, Y, P) register pairs with __ffma2_rn.  No candidate
// examination, addressing, bounds test or flush: its tap rate is a ceiling
// for any kernel that must read each tap's value and do its arithmetic.
#include <cmath>
#include <cstring>

#include "cr_internal.cuh"

namespace cr {
namespace {

constexpr int kProbeRows = 8;
constexpr int kProbeRowStride = 65;

__global__ void __launch_bounds__(256, 3) tap_probe_kernel(const float2* __restrict__ buf,
                                                           uint32_t mask, int iters,
                                                           float2* out) {
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    float2 X[kProbeRows], Y[kProbeRows], P[kProbeRows];
#pragma unroll
    for (int k = 0; k < kProbeRows; ++k) X[k] = Y[k] = P[k] = make_float2(0.f, 0.f);
    uint32_t h = gw * 2654435761u + 12345u;
    const float2 v1 = make_float2(1.0f + 1e-7f * lane, -0.5f), v2 = make_float2(0.25f, 0.75f);
    const float2 pw = make_float2(1.0f, -1.0f);
    for (int it = 0; it < iters; ++it) {
        h = h * 1664525u + 1013904223u;
        const uint32_t base = (h >> 4) & mask;
        float2 kv[kProbeRows];
#pragma unroll
        for (int k = 0; k < kProbeRows; ++k)
            kv[k] = __ldg(buf + ((base + (uint32_t)(k * kProbeRowStride)) & mask) + lane);
#pragma unroll
        for (int k = 0; k < kProbeRows; ++k) {
            X[k] = __ffma2_rn(kv[k], v1, X[k]);
            Y[k] = __ffma2_rn(kv[k], v2, Y[k]);
            P[k] = __ffma2_rn(kv[k], pw, P[k]);
        }
    }
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < kProbeRows; ++k) {
        s.x += X[k].x + Y[k].x + P[k].x;
        s.y += X[k].y + Y[k].y + P[k].y;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace cr

extern "C" int cr_probe_tap_rate(cr_ctx* ctx, int64_t buffer_bytes, int32_t iters,
                                 double* taps_per_second, double* taps, char** err) {
    if (err) *err = nullptr;
    try {
        if (!ctx || !taps_per_second) cr::fail(CR_INVALID, "null argument");
        if (iters <= 0) cr::fail(CR_INVALID, "iters must be positive");
        CR_CUDA_CHECK(cudaSetDevice(ctx->device));
        // a power-of-two element count of at least buffer_bytes (plus one
        // row of 32 past the mask for the lane offsets)
        uint64_t n = 1;
        while (n * 8 < (uint64_t)buffer_bytes) n <<= 1;
        if (n > (1ull << 31)) cr::fail(CR_INVALID, "probe buffer too large");
        float2* buf = (float2*)cr::workspace(ctx, "probe_buf", (size_t)(n + 64) * 8);
        CR_CUDA_CHECK(cudaMemsetAsync(buf, 0x3c, (size_t)(n + 64) * 8, ctx->stream));
        const int threads = 256;
        int per_sm = 0;
        CR_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, cr::tap_probe_kernel, threads, 0));
        const int blocks = ctx->sms * (per_sm > 0 ? per_sm : 1);
        float2* out = (float2*)cr::workspace(ctx, "probe_out", (size_t)blocks * threads * 8);
        const uint32_t mask = (uint32_t)(n - 1) & ~31u;
        // warm the buffer into L2 once, then time one launch
        cr::tap_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(buf, mask, iters, out);
        cr::note_launch(ctx, "tap_probe_kernel");
        cudaEvent_t e0 = ctx->ev[0], e1 = ctx->ev[1];
        CR_CUDA_CHECK(cudaEventRecord(e0, ctx->stream));
        cr::tap_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(buf, mask, iters, out);
        cr::note_launch(ctx, "tap_probe_kernel");
        CR_CUDA_CHECK(cudaEventRecord(e1, ctx->stream));
        CR_CUDA_CHECK(cudaEventSynchronize(e1));
        float ms = 0.0f;
        CR_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        const double t = (double)blocks * threads * iters * cr::kProbeRows;
        if (taps) *taps = t;
        *taps_per_second = t / (ms * 1e-3);
        return CR_OK;
    } catch (const cr::Error& e) {
        if (err) *err = strdup(e.what());
        return e.code;
    } catch (const std::exception& e) {
        if (err) *err = strdup(e.what());
        return CR_INVALID;
    }
}
