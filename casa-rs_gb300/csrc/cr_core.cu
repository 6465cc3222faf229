// cr_core.cu -- context, workspaces, host tables, scan and radix sort.
#include <cmath>
#include <cstring>

#include <cudaTypedefs.h>

#include "cr_internal.cuh"
#include "cr_tma.cuh"

namespace cr {

void fail(int code, const std::string& msg) { throw Error(code, msg); }

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        fail(CR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void check_cufft(cufftResult r, const char* what) {
    if (r != CUFFT_SUCCESS) fail(CR_CUDA, std::string(what) + ": cuFFT error " + std::to_string((int)r));
}

// Grow-only, stream-ordered buffers: a request larger than the current
// buffer frees it on the stream and allocates a larger one.
void* pool_alloc(cr_ctx* ctx, Pool& pool, const std::string& name, size_t bytes) {
    if (bytes == 0) bytes = 16;
    DevBuf& b = pool[name];
    if (b.bytes >= bytes) return b.ptr;
    if (ctx->capturing) fail(CR_CUDA, "workspace '" + name + "' grew during graph capture");
    if (ctx->alloc_limit > 0 && &pool == &ctx->ws) {
        size_t held = 0;
        for (const auto& kv : pool) held += kv.second.bytes;
        if (held - b.bytes + bytes > (size_t)ctx->alloc_limit)
            fail(CR_CUDA, "workspace '" + name + "' of " + std::to_string(bytes) +
                              " bytes exceeds the context's allocation limit (out of memory)");
    }
    ctx->ws_epoch++;
    if (b.ptr) CR_CUDA_CHECK(cudaFreeAsync(b.ptr, ctx->stream));
    size_t want = bytes + bytes / 8;
    want = (want + 255) & ~size_t(255);
    CR_CUDA_CHECK(cudaMallocAsync(&b.ptr, want, ctx->stream));
    b.bytes = want;
    return b.ptr;
}

void pool_free(cr_ctx* ctx, Pool& pool) {
    for (auto& kv : pool)
        if (kv.second.ptr) cudaFreeAsync(kv.second.ptr, ctx->stream);
    pool.clear();
}

void* workspace(cr_ctx* ctx, const std::string& name, size_t bytes) {
    return pool_alloc(ctx, ctx->ws, name, bytes);
}

void note_launch(cr_ctx* ctx, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) fail(CR_CUDA, std::string("launch of ") + what + ": " + cudaGetErrorString(e));
    ctx->launches++;
}

void check_device_status(cr_ctx* ctx) {
    volatile int* st = ctx->status_h;
    if (!st) return;
    const int s = *st;
    if (s == 0) return;
    *st = 0;
    fail(s, "a kernel's bounded wait for a bulk copy gave up");
}

void kernel_mark(cr_ctx* ctx, int which, bool end) {
    // a captured graph is timed as a whole; with timings off nothing is recorded
    if (ctx->capturing || !ctx->timings_enabled) return;
    CR_CUDA_CHECK(cudaEventRecord(ctx->kev[which * 2 + (end ? 1 : 0)], ctx->stream));
    if (end) ctx->kev_used |= 1 << which;
}

static cufftHandle cached_plan(cr_ctx* ctx,
                               std::map<std::pair<int64_t, int64_t>, cufftHandle>& plans,
                               int64_t nx, int64_t ny, cufftType type) {
    auto key = std::make_pair(nx, ny);
    auto it = plans.find(key);
    if (it != plans.end()) {
        check_cufft(cufftSetStream(it->second, ctx->stream), "cufftSetStream");
        return it->second;
    }
    cufftHandle h;
    check_cufft(cufftPlan2d(&h, (int)nx, (int)ny, type), "cufftPlan2d");
    check_cufft(cufftSetStream(h, ctx->stream), "cufftSetStream");
    plans[key] = h;
    return h;
}

cufftHandle fft_plan(cr_ctx* ctx, int64_t nx, int64_t ny) {
    return cached_plan(ctx, ctx->fft_plans, nx, ny, CUFFT_Z2Z);
}

cufftHandle fft_plan_c2c(cr_ctx* ctx, int64_t nx, int64_t ny) {
    return cached_plan(ctx, ctx->fft_plans_c2c, nx, ny, CUFFT_C2C);
}

cufftHandle fft_plan_type(cr_ctx* ctx, int64_t nx, int64_t ny, cufftType type) {
    return cached_plan(ctx, ctx->fft_plans_real[(int)type], nx, ny, type);
}

cufftHandle fft_plan_many(cr_ctx* ctx, int64_t nx, int64_t ny, cufftType type, int batch) {
    auto& plans = ctx->fft_plans_many[std::make_pair((int)type, batch)];
    auto key = std::make_pair(nx, ny);
    auto it = plans.find(key);
    if (it == plans.end()) {
        cufftHandle h;
        int n[2] = {(int)nx, (int)ny};
        check_cufft(cufftPlanMany(&h, 2, n, nullptr, 1, 0, nullptr, 1, 0, type, batch),
                    "cufftPlanMany");
        it = plans.emplace(key, h).first;
    }
    check_cufft(cufftSetStream(it->second, ctx->stream), "cufftSetStream");
    return it->second;
}

// ---- host tables --------------------------------------------------------------
// casa_composite_padded_len (gridder.rs:4152-4173).
int64_t casa_composite_padded_len(int64_t image_len, double padding) {
    int64_t padded = (int64_t)std::floor(padding * (double)image_len - 0.5);
    if (padded < image_len) padded = image_len;
    if (padded % 2) padded += 1;
    for (;;) {
        int64_t v = padded;
        for (int64_t f : {2, 3, 5})
            while (v > 1 && v % f == 0) v /= f;
        if (v == 1) return padded;
        padded += 2;
    }
}

int64_t image_blc(int64_t grid_len, int64_t image_len) {
    return (grid_len - image_len + (grid_len % 2 == 0 ? 1 : 0)) / 2;
}

// grdsf (gridder.rs:4230-4265), powers by repeated squaring.
double grdsf(double nu) {
    static const double P0[5] = {8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1};
    static const double P1[5] = {4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2};
    static const double Q0[3] = {1.0, 8.212018e-1, 2.078043e-1};
    static const double Q1[3] = {1.0, 9.599102e-1, 2.918724e-1};
    if (!(nu >= 0.0 && nu <= 1.0)) return 0.0;
    const bool lo = nu < 0.75;
    const double* p = lo ? P0 : P1;
    const double* q = lo ? Q0 : Q1;
    double e = lo ? 0.75 : 1.0;
    double d = nu * nu - e * e;
    double d2 = d * d;
    double pw[5] = {1.0, d, d2, d2 * d, d2 * d2};
    double num = 0.0, den = 0.0;
    for (int k = 0; k < 5; ++k) num = num + p[k] * pw[k];
    for (int k = 0; k < 3; ++k) den = den + q[k] * pw[k];
    return den == 0.0 ? 0.0 : num / den;
}

static float spheroidal_kernel(double distance, double support) {
    if (!(std::isfinite(distance) && distance <= support)) return 0.0f;
    double nu = distance / support;
    if (nu > 1.0) return 0.0f;
    return (float)((1.0 - nu * nu) * grdsf(nu));
}

// Kernel table (gridder.rs:407-416) and build_normalized_tap_weights
// (gridder.rs:2026-2051): rows for offsets -os/2..os/2, float32 sums.
std::vector<float> std_normalized_taps(int32_t os, int32_t support) {
    int64_t tlen = (int64_t)os * (support + 1);
    std::vector<float> table(tlen, 0.0f);
    for (int64_t i = 0; i < (int64_t)os * support; ++i) {
        double distance = (double)i / ((double)support * (double)os);
        table[i] = spheroidal_kernel(distance * (double)support, (double)support);
    }
    int32_t half = os / 2, taps = 2 * support + 1;
    std::vector<float> rows((size_t)(2 * half + 1) * taps);
    for (int32_t off = -half; off <= half; ++off) {
        float* row = &rows[(size_t)(off + half) * taps];
        float norm = 0.0f;
        for (int32_t t = 0; t < taps; ++t) {
            int64_t lookup = (int64_t)(t - support) * os + off;
            if (lookup < 0) lookup = -lookup;
            float w = lookup < tlen ? table[lookup] : 0.0f;
            row[t] = w;
            norm = norm + w;
        }
        if (norm > 0.0f)
            for (int32_t t = 0; t < taps; ++t) row[t] = row[t] / norm;
    }
    return rows;
}

// build_correction_axis (gridder.rs:4175-4188).
std::vector<float> correction_axis(int64_t size) {
    std::vector<float> out(size);
    double c = (double)size / 2.0;
    for (int64_t i = 0; i < size; ++i) {
        double nu = std::fabs((double)i - c) / c;
        nu = nu < 0.0 ? 0.0 : (nu > 1.0 ? 1.0 : nu);
        double v = grdsf(nu);
        out[i] = v > 1.0e-6 ? (float)(1.0 / v) : 0.0f;
    }
    return out;
}

// build_gridder_correction_axis (gridder.rs:4190-4198).
std::vector<float> gridder_correction_axis(int64_t size) {
    std::vector<float> out(size);
    double c = (double)size / 2.0;
    for (int64_t i = 0; i < size; ++i) {
        double nu = std::fabs((double)i - c) / c;
        nu = nu < 0.0 ? 0.0 : (nu > 1.0 ? 1.0 : nu);
        out[i] = (float)grdsf(nu);
    }
    return out;
}

// build_sinc_axis (gridder.rs:4211-4228).
std::vector<float> sinc_axis(int64_t size, int64_t conv_sampling) {
    std::vector<float> out(size);
    for (int64_t i = 0; i < size; ++i) {
        float offset = (float)(i - size / 2);
        float denom = (float)size * (float)conv_sampling;
        float arg = (float)(3.14159265358979323846 * (double)offset / (double)denom);
        out[i] = (i == size / 2) ? 1.0f : std::sin(arg) / arg;
    }
    return out;
}

// ---- exclusive scan (uint32) ------------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        uint32_t s = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    uint32_t warp_prefix = warp ? warp_sums[warp - 1] : 0;
    uint32_t res = warp_prefix + x - v;
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return res;
}

__global__ void scan_block_sums(const uint32_t* in, int64_t n, uint32_t* sums) {
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) s += in[i];
    }
    uint32_t total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_apply(const uint32_t* in, uint32_t* out, int64_t n, const uint32_t* offs,
                           unsigned long long* total_dev, int64_t nblocks) {
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(s, &total) + (offs ? offs[blockIdx.x] : 0);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (total_dev && blockIdx.x == nblocks - 1 && threadIdx.x == 0)
        *total_dev = (unsigned long long)(offs ? offs[blockIdx.x] : 0) + total;
}

void exclusive_scan_u32(cr_ctx* ctx, const uint32_t* in, uint32_t* out, int64_t n,
                        unsigned long long* total_dev) {
    if (n <= 0) {
        if (total_dev) CR_CUDA_CHECK(cudaMemsetAsync(total_dev, 0, 8, ctx->stream));
        return;
    }
    int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        scan_apply<<<1, kScanThreads, 0, ctx->stream>>>(in, out, n, nullptr, total_dev, 1);
        note_launch(ctx, "scan_apply");
        return;
    }
    // the block sums get their own (recursive) scan; each recursion level
    // uses a distinct workspace
    static thread_local int depth = 0;
    std::string tag = "scan_sums_" + std::to_string(depth);
    uint32_t* sums = (uint32_t*)workspace(ctx, tag, (size_t)nb * 4);
    scan_block_sums<<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(in, n, sums);
    note_launch(ctx, "scan_block_sums");
    depth++;
    exclusive_scan_u32(ctx, sums, sums, nb, nullptr);
    depth--;
    scan_apply<<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(in, out, n, sums, total_dev, nb);
    note_launch(ctx, "scan_apply");
}

// ---- stable LSD radix sort, 8-bit digits ------------------------------------------
// Items are striped over the block (item j of thread t sits at j*256 + t), so
// processing rounds j in order with in-round ranks by thread index keeps the
// sort stable.
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

__global__ void __launch_bounds__(kSortThreads) radix_hist(const uint64_t* keys, int64_t n,
                                                           int shift, uint32_t* hist,
                                                           int64_t nblocks) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        int64_t i = base + j * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads)
    radix_scatter(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                  uint32_t* vals_out, int64_t n, int shift, const uint32_t* offsets,
                  int64_t nblocks) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t goff[256];
    __shared__ uint32_t cnt[kSortThreads / 32][256];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    goff[t] = offsets[(int64_t)t * nblocks + blockIdx.x];
    base[t] = 0;
    const uint32_t lt_mask = (1u << lane) - 1u;
    int64_t blk = (int64_t)blockIdx.x * kSortTile;
    for (int j = 0; j < kSortItems; ++j) {
        int64_t i = blk + j * kSortThreads + t;
        bool valid = i < n;
        uint64_t k = valid ? keys_in[i] : 0;
        uint32_t v = valid ? vals_in[i] : 0;
        uint32_t d = (uint32_t)(k >> shift) & 255u;
#pragma unroll
        for (int w = 0; w < kSortThreads / 32; ++w) cnt[w][t] = 0;
        __syncthreads();
        uint32_t tag = valid ? d : (256u + lane);
        uint32_t peers = __match_any_sync(0xffffffffu, tag);
        uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) cnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = base[t];
#pragma unroll
            for (int w = 0; w < kSortThreads / 32; ++w) {
                uint32_t c = cnt[w][t];
                cnt[w][t] = run;
                run += c;
            }
            base[t] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = goff[d] + cnt[warp][d] + rank;
            keys_out[pos] = k;
            vals_out[pos] = v;
        }
        __syncthreads();
    }
}

void radix_sort_pairs(cr_ctx* ctx, uint64_t* keys, uint32_t* vals, int64_t n, int bits) {
    if (n <= 1 || bits <= 0) return;
    int64_t nb = (n + kSortTile - 1) / kSortTile;
    uint64_t* kalt = (uint64_t*)workspace(ctx, "sort_keys_alt", (size_t)n * 8);
    uint32_t* valt = (uint32_t*)workspace(ctx, "sort_vals_alt", (size_t)n * 4);
    uint32_t* hist = (uint32_t*)workspace(ctx, "sort_hist", (size_t)nb * 256 * 4);
    uint64_t* ksrc = keys;
    uint32_t* vsrc = vals;
    uint64_t* kdst = kalt;
    uint32_t* vdst = valt;
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        radix_hist<<<(unsigned)nb, kSortThreads, 0, ctx->stream>>>(ksrc, n, shift, hist, nb);
        note_launch(ctx, "radix_hist");
        exclusive_scan_u32(ctx, hist, hist, nb * 256, nullptr);
        radix_scatter<<<(unsigned)nb, kSortThreads, 0, ctx->stream>>>(ksrc, vsrc, kdst, vdst, n,
                                                                       shift, hist, nb);
        note_launch(ctx, "radix_scatter");
        std::swap(ksrc, kdst);
        std::swap(vsrc, vdst);
    }
    if (ksrc != keys) {
        CR_CUDA_CHECK(cudaMemcpyAsync(keys, ksrc, (size_t)n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(vals, vsrc, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    }
}

// ---- inputs and outputs ----------------------------------------------------------
const void* device_input(cr_ctx* ctx, const void* p, size_t bytes, int32_t location,
                         const char* name) {
    if (!p) return nullptr;
    if (location == CR_DEVICE) return p;
    if (location != CR_HOST) fail(CR_INVALID, "location must be CR_HOST or CR_DEVICE");
    void* d = workspace(ctx, std::string("in_") + name, bytes);
    CR_CUDA_CHECK(cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return d;
}

void copy_out(cr_ctx* ctx, void* dst, const void* src_dev, size_t bytes, int32_t location) {
    if (!dst || bytes == 0) return;
    if (location == CR_DEVICE) {
        if (dst != src_dev)
            CR_CUDA_CHECK(cudaMemcpyAsync(dst, src_dev, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else if (location == CR_HOST) {
        CR_CUDA_CHECK(cudaMemcpyAsync(dst, src_dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    } else {
        fail(CR_INVALID, "location must be CR_HOST or CR_DEVICE");
    }
}

DeviceBatch device_batch(cr_ctx* ctx, const cr_vis_batch* b, bool need_w) {
    if (!b) fail(CR_INVALID, "batch is null");
    if (b->n < 0) fail(CR_INVALID, "batch size is negative");
    if (b->n >= (int64_t)1 << 31) fail(CR_INVALID, "batch larger than 2^31 samples");
    if (b->n > 0 && (!b->u || !b->v || !b->weight || !b->vis))
        fail(CR_INVALID, "batch lacks u, v, weight or vis");
    if (need_w && b->n > 0 && !b->w) fail(CR_INVALID, "W-projection needs w coordinates");
    DeviceBatch d;
    d.n = b->n;
    size_t n = (size_t)b->n;
    d.u = (const double*)device_input(ctx, b->u, n * 8, b->location, "u");
    d.v = (const double*)device_input(ctx, b->v, n * 8, b->location, "v");
    d.w = need_w ? (const double*)device_input(ctx, b->w, n * 8, b->location, "w") : nullptr;
    d.weight = (const float*)device_input(ctx, b->weight, n * 4, b->location, "weight");
    d.sumwt_factor = (const float*)device_input(ctx, b->sumwt_factor, n * 4, b->location, "sumwt");
    d.gridable = (const uint8_t*)device_input(ctx, b->gridable, n, b->location, "gridable");
    d.vis = (const float2*)device_input(ctx, b->vis, n * 8, b->location, "vis");
    return d;
}

// Host batches below this many samples are uploaded in one go.
constexpr int64_t kStageMinSamples = (int64_t)1 << 20;

StagedBatch::StagedBatch(cr_ctx* c, const cr_vis_batch* b, bool need_w) : ctx(c) {
    if (!b || b->location != CR_HOST || b->n < kStageMinSamples) {
        static_cast<DeviceBatch&>(*this) = device_batch(c, b, need_w);
        return;
    }
    // device_batch's checks
    if (b->n >= (int64_t)1 << 31) fail(CR_INVALID, "batch larger than 2^31 samples");
    if (!b->u || !b->v || !b->weight || !b->vis) fail(CR_INVALID, "batch lacks u, v, weight or vis");
    if (need_w && !b->w) fail(CR_INVALID, "W-projection needs w coordinates");
    const size_t n_s = (size_t)b->n;
    struct Col {
        const void* host;
        size_t elem;
        const char* name;
        void* dev;
    } cols[7] = {{b->u, 8, "u", nullptr},
                 {b->v, 8, "v", nullptr},
                 {need_w ? b->w : nullptr, 8, "w", nullptr},
                 {b->weight, 4, "weight", nullptr},
                 {b->sumwt_factor, 4, "sumwt", nullptr},
                 {b->gridable, 1, "gridable", nullptr},
                 {b->vis, 8, "vis", nullptr}};
    // the same workspaces as device_input's, allocated on the main stream
    // before the auxiliary stream is forked from it
    for (Col& col : cols)
        if (col.host) col.dev = workspace(c, std::string("in_") + col.name, n_s * col.elem);
    n = b->n;
    u = (const double*)cols[0].dev;
    v = (const double*)cols[1].dev;
    w = (const double*)cols[2].dev;
    weight = (const float*)cols[3].dev;
    sumwt_factor = (const float*)cols[4].dev;
    gridable = (const uint8_t*)cols[5].dev;
    vis = (const float2*)cols[6].dev;
    CR_CUDA_CHECK(cudaEventRecord(c->fork_ev, c->stream));
    CR_CUDA_CHECK(cudaStreamWaitEvent(c->aux_stream, c->fork_ev, 0));
    // from here on the destructor joins whatever was queued
    nchunks = kStageChunks;
    stage_ev = c->stage_ev;
    int64_t lo = 0;
    try {
        for (int k = 0; k < kStageChunks; ++k) {
            const int64_t hi = b->n * (k + 1) / kStageChunks;
            chunk_end[k] = hi;
            for (const Col& col : cols)
                if (col.host)
                    CR_CUDA_CHECK(cudaMemcpyAsync((char*)col.dev + lo * col.elem,
                                                  (const char*)col.host + lo * col.elem,
                                                  (size_t)(hi - lo) * col.elem,
                                                  cudaMemcpyHostToDevice, c->aux_stream));
            CR_CUDA_CHECK(cudaEventRecord(c->stage_ev[k], c->aux_stream));
            lo = hi;
        }
    } catch (...) {
        // no destructor runs for a half-built batch: join the copies here
        cudaEventRecord(c->join_ev, c->aux_stream);
        cudaStreamWaitEvent(c->stream, c->join_ev, 0);
        throw;
    }
}

StagedBatch::~StagedBatch() {
    if (nchunks > 0) cudaStreamWaitEvent(ctx->stream, ctx->stage_ev[nchunks - 1], 0);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
bool encode_tensor_map_3d(CUtensorMap* map, const void* base, uint64_t d0, uint64_t d1,
                          uint64_t d2, uint64_t stride1, uint64_t stride2, uint32_t b0,
                          uint32_t b1) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
        cudaGetLastError();
        return (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }();
    if (!encode) return false;
    if (((uintptr_t)base & 15) || (stride1 & 15) || (stride2 & 15) || ((b0 * 4) & 15) ||
        b0 == 0 || b1 == 0 || b0 > 256 || b1 > 256 || d0 == 0 || d1 == 0 || d2 == 0)
        return false;
    const cuuint64_t dims[3] = {d0, d1, d2};
    const cuuint64_t strides[2] = {stride1, stride2};
    const cuuint32_t box[3] = {b0, b1, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}


}  // namespace cr
