// cr_std.cu -- standard (prolate-spheroidal, 7 x 7 taps) gridding and
// degridding over deduplicated records.
//
// Gridding restates grid_sample_taps_real_complex_pair_planned_f64
// (gridder.rs:1021-1071): PSF += gw * wx*wy and dirty += vis*gw * wx*wy, the
// tap product wx*wy rounded in float32.  A block owns one home tile of
// 32 x 32 start cells, privatises its 38 x 38 footprint in shared memory,
// lets each warp scatter one record's 49 taps with shared-memory float
// atomics, and flushes the footprint to the grid with FP32 atomics.
// Degridding restates degrid_sample_taps_planned_normalized
// (gridder.rs:1278-1312) with a warp per record.
#include "cr_internal.cuh"

namespace cr {

namespace {

constexpr int kStdThreads = 256;
constexpr int kFoot = kTile + 6;   // 38
// footprint rows 39 floats apart (= 7 mod 32): the 49 taps of a record hit
// distinct banks within each warp-wide atomic
constexpr int kFootRow = 39;
constexpr int kStdChunk = 2048;    // records per work item

struct StdGridArgs {
    const int32_t *rx, *ry, *ra, *rb;
    const double2* vsum;
    const double* wsum;
    const float2* pred;
    const uint32_t* tile_start;
    int64_t ntx, nty;
    const float* taps;
    const uint32_t* item_tile;
    const uint32_t* item_begin;
    const unsigned long long* n_items;
    unsigned int* item_counter;
    float2* psf;
    float2* dirty;
    int64_t gnx, gny;
};

template <bool RESIDUAL>
__global__ void __launch_bounds__(kStdThreads) std_grid_kernel(StdGridArgs a) {
    __shared__ float s_psf[kFoot * kFootRow];
    __shared__ float s_dr[kFoot * kFootRow];
    __shared__ float s_di[kFoot * kFootRow];
    __shared__ int s_item;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned long long n_items = *a.n_items;
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(a.item_counter, 1u);
        for (int c = tid; c < kFoot * kFootRow; c += kStdThreads) {
            s_psf[c] = 0.0f;
            s_dr[c] = 0.0f;
            s_di[c] = 0.0f;
        }
        __syncthreads();
        const int item = s_item;
        if ((unsigned long long)item >= n_items) break;
        const uint32_t T = a.item_tile[item];
        const uint32_t r0 = a.tile_start[T] + a.item_begin[item];
        const uint32_t r1 = min(a.tile_start[T + 1], r0 + (uint32_t)kStdChunk);
        const int x0 = (int)((T / a.nty) * kTile), y0 = (int)((T % a.nty) * kTile);
        // lanes load 32 records at once; the warp then scatters them in turn
        for (uint32_t rb0 = r0 + warp * 32; rb0 < r1; rb0 += kStdThreads) {
            const uint32_t r = rb0 + lane;
            int lx = 0, ly = 0, ia = 0, ib = 0;
            float vr = 0.0f, vi = 0.0f, pw = 0.0f;
            if (r < r1) {
                lx = a.rx[r] - x0;
                ly = a.ry[r] - y0;
                ia = a.ra[r] * 7;
                ib = a.rb[r] * 7;
                const double2 vs = a.vsum[r];
                const double ws = a.wsum[r];
                if (RESIDUAL) {
                    const float2 p = a.pred[r];
                    vr = (float)(vs.x - (double)p.x * ws);
                    vi = (float)(vs.y - (double)p.y * ws);
                } else {
                    vr = (float)vs.x;
                    vi = (float)vs.y;
                }
                pw = (float)ws;
            }
            const int nrec = (int)min(32u, r1 - rb0);
            for (int k = 0; k < nrec; ++k) {
                const int klx = __shfl_sync(0xffffffffu, lx, k);
                const int kly = __shfl_sync(0xffffffffu, ly, k);
                const float* wx = a.taps + __shfl_sync(0xffffffffu, ia, k);
                const float* wy = a.taps + __shfl_sync(0xffffffffu, ib, k);
                const float kvr = __shfl_sync(0xffffffffu, vr, k);
                const float kvi = __shfl_sync(0xffffffffu, vi, k);
                const float kpw = __shfl_sync(0xffffffffu, pw, k);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    int t = lane + 32 * h;
                    if (t < 49) {
                        int tx = t / 7, ty = t - 7 * (t / 7);
                        float wgt = __fmul_rn(__ldg(&wx[tx]), __ldg(&wy[ty]));
                        int c = (klx + tx) * kFootRow + (kly + ty);
                        if (!RESIDUAL) atomicAdd(&s_psf[c], kpw * wgt);
                        atomicAdd(&s_dr[c], kvr * wgt);
                        atomicAdd(&s_di[c], kvi * wgt);
                    }
                }
            }
        }
        __syncthreads();
        for (int k = tid; k < kFoot * kFoot; k += kStdThreads) {
            const int fx = k / kFoot, fy = k % kFoot, c = fx * kFootRow + fy;
            int64_t x = x0 + fx, y = y0 + fy;
            if (x < a.gnx && y < a.gny) {
                int64_t cell = x * a.gny + y;
                if (!RESIDUAL && s_psf[c] != 0.0f) atomicAdd(&a.psf[cell].x, s_psf[c]);
                if (s_dr[c] != 0.0f || s_di[c] != 0.0f)
                    atomicAdd(&a.dirty[cell], make_float2(s_dr[c], s_di[c]));
            }
        }
        __syncthreads();
    }
}

__global__ void std_work_count(const uint32_t* tile_start, int64_t ntiles, uint32_t* nchunks) {
    for (int64_t T = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; T < ntiles;
         T += (int64_t)gridDim.x * blockDim.x) {
        uint32_t n = tile_start[T + 1] - tile_start[T];
        nchunks[T] = (n + kStdChunk - 1) / kStdChunk;
    }
}

__global__ void std_work_fill(const uint32_t* nchunks, const uint32_t* first, int64_t ntiles,
                              uint32_t* item_tile, uint32_t* item_begin) {
    for (int64_t T = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; T < ntiles;
         T += (int64_t)gridDim.x * blockDim.x) {
        uint32_t c = nchunks[T], f = first[T];
        for (uint32_t k = 0; k < c; ++k) {
            item_tile[f + k] = (uint32_t)T;
            item_begin[f + k] = k * kStdChunk;
        }
    }
}

struct StdDegridArgs {
    const int32_t *rx, *ry, *ra, *rb;
    const unsigned long long* counts;
    const float* taps;
    const float2* grid;
    int64_t gny;
    float2* pred;
};

__global__ void __launch_bounds__(256) std_degrid_kernel(StdDegridArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t nrec = (int64_t)a.counts[2];
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrec;
         r += nwarps) {
        const float* wx = a.taps + a.ra[r] * 7;
        const float* wy = a.taps + a.rb[r] * 7;
        const float2* g = a.grid + (int64_t)a.rx[r] * a.gny + a.ry[r];
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            int t = lane + 32 * h;
            if (t < 49) {
                int tx = t / 7, ty = t - 7 * (t / 7);
                float wgt = __fmul_rn(__ldg(&wx[tx]), __ldg(&wy[ty]));
                float2 gv = g[(int64_t)tx * a.gny + ty];
                re = fmaf(gv.x, wgt, re);
                im = fmaf(gv.y, wgt, im);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o);
            im += __shfl_xor_sync(0xffffffffu, im, o);
        }
        if (lane == 0) a.pred[r] = make_float2(re, im);
    }
}

}  // namespace

void std_grid(cr_ctx* ctx, cr_gridder* g, const Records& r, float2* psf, float2* dirty,
              int mode) {
    const int64_t ntiles = r.ntx * r.nty;
    uint32_t* nchunks = (uint32_t*)workspace(ctx, "sg_nchunks", (size_t)ntiles * 4);
    uint32_t* first = (uint32_t*)workspace(ctx, "sg_first", (size_t)ntiles * 4);
    unsigned long long* nitems = (unsigned long long*)workspace(ctx, "sg_nitems", 16);
    std_work_count<<<grid_blocks(ntiles, 256), 256, 0, ctx->stream>>>(r.tile_start, ntiles,
                                                                       nchunks);
    note_launch(ctx, "std_work_count");
    exclusive_scan_u32(ctx, nchunks, first, ntiles, nitems);
    size_t max_items = (size_t)ntiles + (size_t)(r.n_samples / kStdChunk + 1);
    uint32_t* item_tile = (uint32_t*)workspace(ctx, "sg_item_tile", max_items * 4);
    uint32_t* item_begin = (uint32_t*)workspace(ctx, "sg_item_begin", max_items * 4);
    std_work_fill<<<grid_blocks(ntiles, 256), 256, 0, ctx->stream>>>(nchunks, first, ntiles,
                                                                      item_tile, item_begin);
    note_launch(ctx, "std_work_fill");
    unsigned int* counter = (unsigned int*)(nitems + 1);
    CR_CUDA_CHECK(cudaMemsetAsync(counter, 0, 4, ctx->stream));
    StdGridArgs a{r.rec_x, r.rec_y, r.rec_a, r.rec_b, r.rec_vsum, r.rec_wsum, r.rec_pred,
                  r.tile_start, r.ntx, r.nty, g->taps_d, item_tile, item_begin, nitems,
                  counter, psf, dirty, g->info.grid_nx, g->info.grid_ny};
    int sms = 0;
    CR_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    kernel_mark(ctx, 0, false);
    if (mode == 0) {
        std_grid_kernel<false><<<sms * 4, kStdThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "std_grid_kernel");
    } else {
        std_grid_kernel<true><<<sms * 4, kStdThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "std_grid_kernel_residual");
    }
    kernel_mark(ctx, 0, true);
}

void std_degrid(cr_ctx* ctx, cr_gridder* g, const Records& r, const float2* grid) {
    StdDegridArgs a{r.rec_x, r.rec_y, r.rec_a, r.rec_b, r.counts, g->taps_d, grid,
                    g->info.grid_ny, r.rec_pred};
    int sms = 0;
    CR_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    kernel_mark(ctx, 1, false);
    std_degrid_kernel<<<sms * 8, 256, 0, ctx->stream>>>(a);
    note_launch(ctx, "std_degrid_kernel");
    kernel_mark(ctx, 1, true);
}

}  // namespace cr
