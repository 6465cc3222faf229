// cr_hogbom.cu -- the Hogbom minor cycle as one persistent device loop.
//
// Restates run_hogbom_minor_cycle_cpu_with_progress (lib.rs:59748-59883):
// repeat up to the component budget (hogbom_component_budget, lib.rs:64541-
// 64552): find the unmasked pixel of largest |residual| with ties going to
// the smallest y*nx + x (peak_location_masked_in_bounds_zero_tolerance,
// lib.rs:74064-74118), stop on the threshold rules (minor_cycle_stop_reason,
// lib.rs:74653-74676), add gain*peak to the model and subtract the shifted
// PSF over the overlap (subtract_shifted_kernel_in_window, lib.rs:74805-
// 74870) as a float32 multiply then subtract.
//
// Each block owns a contiguous range of pixels.  One pass per iteration
// subtracts the previous component and finds the block's next candidate with
// a warp-shuffle argmax; one grid barrier publishes the candidates, and every
// block reduces all candidates to the same global peak.  The kernel is
// launched cooperatively (all blocks resident); the barrier's wait is bounded
// and reports CR_TIMEOUT instead of spinning forever.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "cr_clean.cuh"
#include "cr_internal.cuh"

namespace cr {

namespace {

constexpr int kHogThreads = 512;

struct HogArgs {
    float* model;
    float* residual;
    const float* psf;
    const uint8_t* mask;
    int nx, ny;
    float gain, threshold, cycle_threshold, nsigma_threshold;
    long long budget;
    Cand* cands;  // [2][gridDim]
    unsigned int* bar;  // [0] arrivals, [1] generation
    int* comp_x;
    int* comp_y;
    float* comp_peak;
    float* comp_flux;
    long long* out_actual;
    int* out_stop;
    int* out_status;
    // run_hogbom_plane_minor_cycle's rules (lib.rs:64630-64680): peaks over
    // finite values only, stop when |peak| <= threshold or <= the cycle
    // threshold, no nsigma rule
    int plane_rules;
    // polls of a grid-barrier wait before it gives up (each poll sleeps
    // ~64 ns); set from the context by every launch
    long long barrier_polls;
};

// The minor cycle of one image by `nblocks` co-resident blocks, this one
// being block `bidx` of them.
__device__ void hogbom_body(const HogArgs& a, int nblocks, int bidx) {
    const int64_t npix = (int64_t)a.nx * a.ny;
    const int64_t chunk = (npix + nblocks - 1) / nblocks;
    const int64_t p0 = (int64_t)bidx * chunk;
    const int64_t p1 = min(npix, p0 + chunk);
    const int kcx = a.nx / 2, kcy = a.ny / 2;
    __shared__ Cand s_best;
    __shared__ int s_stop;

    // initial candidates
    {
        float ba = -1.0f, bv = 0.0f;
        int bk = 0x7fffffff;
        for (int64_t t = p0 + threadIdx.x; t < p1; t += blockDim.x) {
            if (a.mask && !a.mask[t]) continue;
            int x = (int)(t / a.ny), y = (int)(t - (int64_t)x * a.ny);
            float v = a.residual[t];
            if (a.plane_rules && !isfinite(v)) continue;
            float av = fabsf(v);
            int key = y * a.nx + x;
            if (better(av, key, ba, bk)) {
                ba = av;
                bk = key;
                bv = v;
            }
        }
        Cand c = block_argmax(ba, bk, bv);
        if (threadIdx.x == 0) a.cands[bidx] = c;
    }
    if (!grid_barrier(a.bar, (unsigned)nblocks, a.barrier_polls)) {
        if (threadIdx.x == 0) atomicExch(a.out_status, CR_TIMEOUT);
        return;
    }
    long long it = 0;
    int stop = CR_STOP_NONE;
    for (; it < a.budget; ++it) {
        const Cand* cur = a.cands + (it & 1) * nblocks;
        Cand* nxt = a.cands + ((it + 1) & 1) * nblocks;
        // every block reduces all candidates to the same global peak
        {
            float ba = -1.0f, bv = 0.0f;
            int bk = 0x7fffffff;
            for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
                // other blocks wrote these: read through L2, not a stale L1 line
                int4 raw = __ldcg(reinterpret_cast<const int4*>(cur) + i);
                Cand c{__int_as_float(raw.x), raw.y, __int_as_float(raw.z), 0};
                if (better(c.absval, c.key, ba, bk)) {
                    ba = c.absval;
                    bk = c.key;
                    bv = c.value;
                }
            }
            Cand c = block_argmax(ba, bk, bv);
            if (threadIdx.x == 0) {
                s_best = c;
                int r = 0;
                if (c.absval < 0.0f)
                    r = CR_STOP_NO_CLEANABLE_PIXELS;
                else if (a.plane_rules)
                    r = c.absval <= a.threshold         ? CR_STOP_GLOBAL_THRESHOLD
                        : c.absval <= a.cycle_threshold ? CR_STOP_CYCLE_THRESHOLD
                                                        : 0;
                else
                    r = stop_reason(c.absval, a.threshold, a.cycle_threshold, a.nsigma_threshold);
                s_stop = r;
            }
            __syncthreads();
        }
        if (s_stop) {
            stop = s_stop;
            break;
        }
        const Cand best = s_best;
        const int px = best.key % a.nx, py = best.key / a.nx;
        const float comp = __fmul_rn(a.gain, best.value);
        if (bidx == 0 && threadIdx.x == 0) {
            int64_t m = (int64_t)px * a.ny + py;
            a.model[m] = __fadd_rn(a.model[m], comp);
            if (a.comp_x) {
                a.comp_x[it] = px;
                a.comp_y[it] = py;
                a.comp_peak[it] = best.value;
                a.comp_flux[it] = comp;
            }
        }
        // subtract the shifted PSF over the block's pixels and find the next
        // candidate in the same pass
        float ba = -1.0f, bv = 0.0f;
        int bk = 0x7fffffff;
        // (x, y) stepped along with t, without a division per pixel; PSF
        // offsets in 32 bits (npix < 2^31)
        const int step = (int)blockDim.x, sx = step / a.ny, sy = step - sx * a.ny;
        int64_t t = p0 + threadIdx.x;
        int x = (int)(t / a.ny), y = (int)(t - (int64_t)x * a.ny);
#pragma unroll 4
        for (; t < p1; t += step) {
            const int kx = x - px + kcx, ky = y - py + kcy;
            float v = a.residual[t];
            if (kx >= 0 && kx < a.nx && ky >= 0 && ky < a.ny) {
                v = __fsub_rn(v, __fmul_rn(comp, a.psf[kx * a.ny + ky]));
                a.residual[t] = v;
            }
            if ((!a.mask || a.mask[t]) && (!a.plane_rules || isfinite(v))) {
                const float av = fabsf(v);
                const int key = y * a.nx + x;
                if (better(av, key, ba, bk)) {
                    ba = av;
                    bk = key;
                    bv = v;
                }
            }
            x += sx;
            y += sy;
            if (y >= a.ny) {
                y -= a.ny;
                ++x;
            }
        }
        Cand c = block_argmax(ba, bk, bv);
        if (threadIdx.x == 0) nxt[bidx] = c;
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

__global__ void __launch_bounds__(kHogThreads) hogbom_kernel(HogArgs a) {
    hogbom_body(a, (int)gridDim.x, (int)blockIdx.x);
}

// Several images [P][nx][ny] at once: `per_plane` blocks for each listed
// plane, each group with its own barrier words, candidates, component list
// and results (slot s = the plane's position in the list).
struct HogPlanesArgs {
    HogArgs base;           // pointers to plane 0; cands / bar / comp / out of slot 0
    const int* planes;      // [n] plane indices
    const float* nsigma;    // [n] n-sigma threshold of each slot, or null (base's)
    int per_plane;
    int64_t comp_cap;       // components per slot
};

__global__ void __launch_bounds__(kHogThreads) hogbom_planes_kernel(HogPlanesArgs pa) {
    const int slot = (int)blockIdx.x / pa.per_plane;
    const int bidx = (int)blockIdx.x % pa.per_plane;
    const int64_t npix = (int64_t)pa.base.nx * pa.base.ny;
    const int64_t off = (int64_t)pa.planes[slot] * npix;
    HogArgs a = pa.base;
    a.model += off;
    a.residual += off;
    a.psf += off;
    if (a.mask) a.mask += off;
    a.cands += (int64_t)slot * 2 * pa.per_plane;
    a.bar += 4 * slot;
    if (a.comp_x) {
        a.comp_x += slot * pa.comp_cap;
        a.comp_y += slot * pa.comp_cap;
        a.comp_peak += slot * pa.comp_cap;
        a.comp_flux += slot * pa.comp_cap;
    }
    a.out_actual += slot;
    a.out_stop += slot;
    if (pa.nsigma) a.nsigma_threshold = pa.nsigma[slot];
    hogbom_body(a, pa.per_plane, bidx);
}

// run_hogbom_plane_minor_cycle with a relative peak tolerance > 0
// (finite_peak_location_masked_with_relative_tolerance, lib.rs:73998-74026):
// the scan runs y-major (x fastest) and a value replaces the current peak
// only if |v| > |peak| * (1 + tol) in float32, so the result depends on the
// scan order and is not a plain argmax.  One block replays it exactly: all
// threads form each scan row's largest finite unmasked |r|; one warp then
// walks the rows, skipping a row whose largest value cannot replace the
// current peak and, inside a row that can, jumping with ballots to the next
// value that does.  Subtraction and the model update follow as in the fast
// loop.  No inter-block waits.
constexpr int kTolThreads = 1024;

struct HogTolArgs {
    float* model;
    float* residual;
    const float* psf;
    const uint8_t* mask;
    int nx, ny;
    float gain, threshold, cycle_threshold, tol;
    long long budget;
    float* rowmax;  // [ny]
    int* comp_x;
    int* comp_y;
    float* comp_peak;
    float* comp_flux;
    long long* out_actual;
};

__global__ void __launch_bounds__(kTolThreads) hogbom_tol_kernel(HogTolArgs a) {
    __shared__ int s_have, s_x, s_y;
    __shared__ float s_v;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float k1 = __fadd_rn(1.0f, a.tol);
    const int kcx = a.nx / 2, kcy = a.ny / 2;
    const int64_t npix = (int64_t)a.nx * a.ny;
    long long it = 0;
    for (; it < a.budget; ++it) {
        for (int y = tid; y < a.ny; y += kTolThreads) {
            float m = -1.0f;
            for (int x = 0; x < a.nx; ++x) {
                const int64_t t = (int64_t)x * a.ny + y;
                const float v = a.residual[t];
                if ((!a.mask || a.mask[t]) && isfinite(v)) m = fmaxf(m, fabsf(v));
            }
            a.rowmax[y] = m;
        }
        __syncthreads();
        if (warp == 0) {
            bool have = false;
            int bx = 0, by = 0;
            float bv = 0.0f, thr = 0.0f;
            for (int y0 = 0; y0 < a.ny;) {
                const int yy = y0 + lane;
                const float rm = yy < a.ny ? a.rowmax[yy] : -1.0f;
                const unsigned rows = __ballot_sync(0xffffffffu, have ? rm > thr : rm >= 0.0f);
                if (!rows) {
                    y0 += 32;
                    continue;
                }
                const int y = y0 + __ffs(rows) - 1;
                for (int x0 = 0; x0 < a.nx;) {
                    const int xx = x0 + lane;
                    float v = 0.0f;
                    bool ok = false;
                    if (xx < a.nx) {
                        const int64_t t = (int64_t)xx * a.ny + y;
                        v = a.residual[t];
                        ok = (!a.mask || a.mask[t]) && isfinite(v) && (!have || fabsf(v) > thr);
                    }
                    const unsigned hit = __ballot_sync(0xffffffffu, ok);
                    if (!hit) {
                        x0 += 32;
                        continue;
                    }
                    const int src = __ffs(hit) - 1;
                    bv = __shfl_sync(0xffffffffu, v, src);
                    bx = x0 + src;
                    by = y;
                    have = true;
                    thr = __fmul_rn(fabsf(bv), k1);
                    x0 = bx + 1;
                }
                y0 = y + 1;
            }
            if (lane == 0) {
                s_have = have;
                s_x = bx;
                s_y = by;
                s_v = bv;
            }
        }
        __syncthreads();
        if (!s_have) break;
        const float peak = s_v, pabs = fabsf(peak);
        if (pabs <= a.threshold || pabs <= a.cycle_threshold) break;
        const int px = s_x, py = s_y;
        const float comp = __fmul_rn(a.gain, peak);
        if (tid == 0) {
            const int64_t m = (int64_t)px * a.ny + py;
            a.model[m] = __fadd_rn(a.model[m], comp);
            a.comp_x[it] = px;
            a.comp_y[it] = py;
            a.comp_peak[it] = peak;
            a.comp_flux[it] = comp;
        }
        for (int64_t t = tid; t < npix; t += kTolThreads) {
            const int x = (int)(t / a.ny), y = (int)(t - (int64_t)x * a.ny);
            const int kx = x - px + kcx, ky = y - py + kcy;
            if (kx >= 0 && kx < a.nx && ky >= 0 && ky < a.ny)
                a.residual[t] = __fsub_rn(a.residual[t], __fmul_rn(comp, a.psf[kx * a.ny + ky]));
        }
        __syncthreads();
    }
    if (tid == 0) *a.out_actual = it;
}

}  // namespace

void hogbom(cr_ctx* ctx, float* model, float* residual, const float* psf, const uint8_t* mask,
            int32_t nx, int32_t ny, float gain, float threshold, float cycle_threshold,
            float nsigma_threshold, int64_t cycle_niter, int32_t inclusive, int32_t* comp_x,
            int32_t* comp_y, float* comp_peak, float* comp_flux, int64_t* actual,
            int64_t* reported, int32_t* stop_reason_out, int plane_rules) {
    if (nx <= 0 || ny <= 0) fail(CR_INVALID, "image shape must be positive");
    if ((int64_t)nx * ny >= (1ll << 31)) fail(CR_INVALID, "image larger than 2^31 pixels");
    if (cycle_niter < 0) fail(CR_INVALID, "cycle_niter is negative");
    long long budget = inclusive ? cycle_niter + 1 : cycle_niter;
    int sms = 0, per_sm = 0;
    CR_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    CR_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hogbom_kernel,
                                                                kHogThreads, 0));
    if (per_sm < 1) fail(CR_CUDA, "Hogbom kernel cannot be resident");
    int64_t npix = (int64_t)nx * ny;
    int blocks = (int)std::min<int64_t>((int64_t)sms * std::min(per_sm, 2),
                                        std::max<int64_t>(1, (npix + kHogThreads - 1) / kHogThreads));
    size_t cap = (size_t)(budget > 0 ? budget : 1);
    char* wsp = (char*)workspace(ctx, "hog_ws", 256 + (size_t)blocks * 2 * sizeof(Cand) + cap * 16);
    unsigned int* bar = (unsigned int*)wsp;
    long long* out_actual = (long long*)(wsp + 16);
    int* out_stop = (int*)(wsp + 24);
    int* out_status = (int*)(wsp + 28);
    Cand* cands = (Cand*)(wsp + 256);
    int* cx = (int*)(wsp + 256 + (size_t)blocks * 2 * sizeof(Cand));
    int* cy = cx + cap;
    float* cp = (float*)(cy + cap);
    float* cf = cp + cap;
    CR_CUDA_CHECK(cudaMemsetAsync(wsp, 0, 256, ctx->stream));
    HogArgs a{model, residual, psf, mask, nx, ny, gain, threshold, cycle_threshold,
              nsigma_threshold, budget, cands, bar, cx, cy, cp, cf, out_actual, out_stop,
              out_status, plane_rules, ctx->barrier_polls};
    void* args[] = {&a};
    CR_CUDA_CHECK(cudaLaunchCooperativeKernel((void*)hogbom_kernel, dim3(blocks), dim3(kHogThreads),
                                              args, 0, ctx->stream));
    note_launch(ctx, "hogbom_kernel");
    struct {
        long long actual;
        int stop, status;
    } h;
    CR_CUDA_CHECK(cudaMemcpyAsync(&h, out_actual, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    if (h.status) fail(CR_TIMEOUT, "Hogbom grid barrier timed out");
    if (comp_x && h.actual > 0) {
        const size_t nb = (size_t)h.actual * 4;
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_x, cx, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_y, cy, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_peak, cp, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_flux, cf, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    }
    if (actual) *actual = h.actual;
    if (reported) *reported = std::min<int64_t>(h.actual, cycle_niter);
    if (stop_reason_out) *stop_reason_out = h.stop;
}

void hogbom_plane(cr_ctx* ctx, float* model, float* residual, const float* psf,
                  const uint8_t* mask, int32_t nx, int32_t ny, float gain, float threshold,
                  float cycle_threshold, float peak_relative_tolerance, int64_t cycle_limit,
                  int32_t inclusive, int32_t* comp_x, int32_t* comp_y, float* comp_peak,
                  float* comp_flux, int64_t* actual, int64_t* reported) {
    if (!(peak_relative_tolerance >= 0.0f) || !std::isfinite(peak_relative_tolerance))
        fail(CR_INVALID, "peak_relative_tolerance must be finite and non-negative");
    if (peak_relative_tolerance == 0.0f) {
        int32_t stop = 0;
        hogbom(ctx, model, residual, psf, mask, nx, ny, gain, threshold, cycle_threshold, 0.0f,
               cycle_limit, inclusive, comp_x, comp_y, comp_peak, comp_flux, actual, reported,
               &stop, 1);
        return;
    }
    if (nx <= 0 || ny <= 0) fail(CR_INVALID, "image shape must be positive");
    if ((int64_t)nx * ny >= (1ll << 31)) fail(CR_INVALID, "image larger than 2^31 pixels");
    if (cycle_limit < 0) fail(CR_INVALID, "cycle_limit is negative");
    const long long budget = inclusive ? cycle_limit + 1 : cycle_limit;
    const size_t cap = (size_t)(budget > 0 ? budget : 1);
    char* wsp = (char*)workspace(ctx, "hogtol_ws", 256 + (size_t)ny * 4 + cap * 16);
    long long* out_actual = (long long*)wsp;
    float* rowmax = (float*)(wsp + 256);
    int* cx = (int*)(rowmax + ny);
    int* cy = cx + cap;
    float* cp = (float*)(cy + cap);
    float* cf = cp + cap;
    CR_CUDA_CHECK(cudaMemsetAsync(wsp, 0, 256, ctx->stream));
    HogTolArgs a{model, residual, psf, mask, nx, ny, gain, threshold, cycle_threshold,
                 peak_relative_tolerance, budget, rowmax, cx, cy, cp, cf, out_actual};
    hogbom_tol_kernel<<<1, kTolThreads, 0, ctx->stream>>>(a);
    note_launch(ctx, "hogbom_tol_kernel");
    long long n = 0;
    CR_CUDA_CHECK(cudaMemcpyAsync(&n, out_actual, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    if (comp_x && n > 0) {
        // one synchronisation for the four lists, on the context's stream
        const size_t b = (size_t)n * 4;
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_x, cx, b, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_y, cy, b, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_peak, cp, b, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_flux, cf, b, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    }
    if (actual) *actual = n;
    // CasaInclusive reports at most the cycle limit when the budget ran out
    if (reported) *reported = std::min<int64_t>(n, cycle_limit);
}

void hogbom_planes(cr_ctx* ctx, float* model, float* residual, const float* psf,
                   const uint8_t* mask, int32_t nx, int32_t ny, int32_t nplanes,
                   const int32_t* planes, int32_t n, float gain, float threshold,
                   float cycle_threshold, float nsigma_threshold,
                   const float* nsigma_per_plane, int64_t cycle_niter, int32_t inclusive,
                   int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
                   int64_t* actual, int64_t* reported, int32_t* stop_reason_out) {
    if (nx <= 0 || ny <= 0) fail(CR_INVALID, "image shape must be positive");
    if ((int64_t)nx * ny >= (1ll << 31)) fail(CR_INVALID, "image larger than 2^31 pixels");
    if (cycle_niter < 0) fail(CR_INVALID, "cycle_niter is negative");
    if (n < 0 || (n > 0 && !planes)) fail(CR_INVALID, "plane list is null");
    for (int32_t s = 0; s < n; ++s)
        if (planes[s] < 0 || planes[s] >= nplanes) fail(CR_INVALID, "plane index out of range");
    if (n == 0) return;
    const long long budget = inclusive ? cycle_niter + 1 : cycle_niter;
    const int64_t cap = budget > 0 ? budget : 1;
    int sms = 0, per_sm = 0;
    CR_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    CR_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hogbom_planes_kernel,
                                                                kHogThreads, 0));
    if (per_sm < 1) fail(CR_CUDA, "Hogbom kernel cannot be resident");
    const int resident = sms * per_sm;
    // blocks per plane: as many as keep every listed plane's group resident,
    // at most 8; planes beyond one launch's room go in further launches
    const int batch = std::min<int>(n, resident);
    const int per_plane = std::max(1, std::min(8, resident / batch));
    const size_t head = 16 * (size_t)batch + 8 * (size_t)batch + 4 * (size_t)batch + 16;
    const size_t head_al = (head + 255) & ~(size_t)255;
    const size_t cand_b = (size_t)batch * 2 * per_plane * sizeof(Cand);
    char* wsp = (char*)workspace(ctx, "hogp_ws", head_al + cand_b + (size_t)batch * cap * 16);
    unsigned int* bar = (unsigned int*)wsp;
    long long* out_actual = (long long*)(wsp + 16 * (size_t)batch);
    int* out_stop = (int*)(wsp + 24 * (size_t)batch);
    int* out_status = (int*)(wsp + 28 * (size_t)batch);
    Cand* cands = (Cand*)(wsp + head_al);
    int* cx = (int*)(wsp + head_al + cand_b);
    int* cy = cx + (size_t)batch * cap;
    float* cp = (float*)(cy + (size_t)batch * cap);
    float* cf = cp + (size_t)batch * cap;
    int* plist = (int*)workspace(ctx, "hogp_planes", (size_t)batch * 4);
    float* nslist = nsigma_per_plane
                        ? (float*)workspace(ctx, "hogp_nsigma", (size_t)batch * 4)
                        : nullptr;
    std::vector<long long> h_actual((size_t)batch);
    std::vector<int> h_stop((size_t)batch);
    for (int32_t s0 = 0; s0 < n; s0 += batch) {
        const int m = std::min<int>(batch, n - s0);
        CR_CUDA_CHECK(cudaMemsetAsync(wsp, 0, head_al, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(plist, planes + s0, (size_t)m * 4, cudaMemcpyHostToDevice,
                                      ctx->stream));
        if (nslist)
            CR_CUDA_CHECK(cudaMemcpyAsync(nslist, nsigma_per_plane + s0, (size_t)m * 4,
                                          cudaMemcpyHostToDevice, ctx->stream));
        HogPlanesArgs pa;
        pa.base = HogArgs{model, residual, psf, mask, nx, ny, gain, threshold, cycle_threshold,
                          nsigma_threshold, budget, cands, bar, cx, cy, cp, cf, out_actual,
                          out_stop, out_status, 0, ctx->barrier_polls};
        pa.planes = plist;
        pa.nsigma = nslist;
        pa.per_plane = per_plane;
        pa.comp_cap = cap;
        void* args[] = {&pa};
        CR_CUDA_CHECK(cudaLaunchCooperativeKernel((void*)hogbom_planes_kernel,
                                                  dim3((unsigned)(m * per_plane)),
                                                  dim3(kHogThreads), args, 0, ctx->stream));
        note_launch(ctx, "hogbom_planes_kernel");
        int status = 0;
        CR_CUDA_CHECK(cudaMemcpyAsync(h_actual.data(), out_actual, (size_t)m * 8,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(h_stop.data(), out_stop, (size_t)m * 4,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(&status, out_status, 4, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        if (status) fail(CR_TIMEOUT, "Hogbom grid barrier timed out");
        long long most = 0;
        for (int s = 0; s < m; ++s) {
            const int64_t k = s0 + s;
            const long long got = h_actual[(size_t)s];
            most = std::max(most, got);
            if (actual) actual[k] = got;
            if (reported) reported[k] = std::min<int64_t>(got, cycle_niter);
            if (stop_reason_out) stop_reason_out[k] = h_stop[(size_t)s];
        }
        if (comp_x && most > 0) {
            // the batch's component lists in one copy per array (the slots
            // past each plane's count are not read)
            const size_t ho = (size_t)s0 * cap, len = (size_t)m * cap * 4;
            CR_CUDA_CHECK(cudaMemcpyAsync(comp_x + ho, cx, len, cudaMemcpyDeviceToHost,
                                          ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(comp_y + ho, cy, len, cudaMemcpyDeviceToHost,
                                          ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(comp_peak + ho, cp, len, cudaMemcpyDeviceToHost,
                                          ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(comp_flux + ho, cf, len, cudaMemcpyDeviceToHost,
                                          ctx->stream));
            CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        }
    }
}

}  // namespace cr

// ---- allocation-free variant ------------------------------------------------------
//
// For callers that must not allocate device memory once they are running:
// a host that reserved its device memory up front (a fixed arena or budget
// handed to it by a resource manager) and forbids allocations afterwards,
// or a process in which another allocator already holds nearly all device
// memory, so that a new cudaMalloc could fail or stall the device in the
// middle of a minor cycle.  This entry point runs the same Hogbom kernel
// with its scratch (grid-barrier words, per-block peak candidates and the
// component list) in a fixed array in this library's device memory, which
// every GPU that loads the library holds until the process exits.
// Inputs and outputs stay the caller's device buffers.

namespace cr {
namespace {

constexpr int kNoAllocMaxBlocks = 1024;
constexpr long long kNoAllocMaxComponents = 16384;
constexpr size_t kNoAllocHeader = 256;  // barrier words and result scalars
constexpr size_t kNoAllocCands = (size_t)2 * kNoAllocMaxBlocks * sizeof(Cand);
constexpr size_t kNoAllocBytes = kNoAllocHeader + kNoAllocCands + (size_t)kNoAllocMaxComponents * 16;

// 295,168 bytes per device: header, candidates, then x, y, peak and flux of
// up to kNoAllocMaxComponents components.
static __device__ __align__(256) unsigned char g_hogbom_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 256;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array for the current device, looked up once
// per device (the caller has made `device` current).  cr_ctx_create does the
// lookup, so the module holding the array (and the array's memory) is
// loaded when a context is created, not during a later call.
void* scratch_address(int device) {
    if (device < 0 || device >= kMaxDevices) fail(CR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        check_cuda(cudaGetSymbolAddress(&p, g_hogbom_scratch), "cudaGetSymbolAddress");
        g_scratch_addr[device] = p;
    }
    return g_scratch_addr[device];
}

void hogbom_noalloc(cr_ctx* ctx, float* model, float* residual, const float* psf,
                    const uint8_t* mask, int32_t nx, int32_t ny, float gain, float threshold,
                    float cycle_threshold, float nsigma_threshold, int64_t cycle_niter,
                    int32_t inclusive, int32_t* comp_x, int32_t* comp_y, float* comp_peak,
                    float* comp_flux, int64_t* actual, int64_t* reported,
                    int32_t* stop_reason_out) {
    if (nx <= 0 || ny <= 0) fail(CR_INVALID, "image shape must be positive");
    if ((int64_t)nx * ny >= (1ll << 31)) fail(CR_INVALID, "image larger than 2^31 pixels");
    if (cycle_niter < 0) fail(CR_INVALID, "cycle_niter is negative");
    long long budget = inclusive ? cycle_niter + 1 : cycle_niter;
    if (budget > kNoAllocMaxComponents)
        fail(CR_INVALID, "cr_hogbom_noalloc: the component budget (cycle_niter, plus one when "
                         "inclusive) exceeds its fixed scratch of 16384 components");
    CR_CUDA_CHECK(cudaSetDevice(ctx->device));
    char* base = (char*)scratch_address(ctx->device);
    int sms = 0, per_sm = 0;
    CR_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    CR_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hogbom_kernel,
                                                                kHogThreads, 0));
    if (per_sm < 1) fail(CR_CUDA, "Hogbom kernel cannot be resident");
    int64_t npix = (int64_t)nx * ny;
    int blocks = (int)std::min<int64_t>((int64_t)sms * std::min(per_sm, 2),
                                        std::max<int64_t>(1, (npix + kHogThreads - 1) / kHogThreads));
    blocks = std::min(blocks, kNoAllocMaxBlocks);
    unsigned int* bar = (unsigned int*)base;
    long long* out_actual = (long long*)(base + 16);
    int* out_stop = (int*)(base + 24);
    int* out_status = (int*)(base + 28);
    Cand* cands = (Cand*)(base + kNoAllocHeader);
    int* cx = (int*)(base + kNoAllocHeader + kNoAllocCands);
    int* cy = cx + kNoAllocMaxComponents;
    float* cp = (float*)(cy + kNoAllocMaxComponents);
    float* cf = cp + kNoAllocMaxComponents;
    // the array keeps the previous call's contents: the barrier and the
    // result words must start at zero
    CR_CUDA_CHECK(cudaMemsetAsync(base, 0, kNoAllocHeader, ctx->stream));
    HogArgs a{model, residual, psf, mask, nx, ny, gain, threshold, cycle_threshold,
              nsigma_threshold, budget, cands, bar, cx, cy, cp, cf, out_actual, out_stop,
              out_status, 0, ctx->barrier_polls};
    void* args[] = {&a};
    CR_CUDA_CHECK(cudaLaunchCooperativeKernel((void*)hogbom_kernel, dim3(blocks), dim3(kHogThreads),
                                              args, 0, ctx->stream));
    note_launch(ctx, "hogbom_kernel");
    struct {
        long long actual;
        int stop, status;
    } h;
    CR_CUDA_CHECK(cudaMemcpyAsync(&h, out_actual, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    if (h.status) fail(CR_TIMEOUT, "Hogbom grid barrier timed out");
    if (comp_x && h.actual > 0) {
        const size_t nb = (size_t)h.actual * 4;
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_x, cx, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_y, cy, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_peak, cp, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_flux, cf, nb, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    }
    if (actual) *actual = h.actual;
    if (reported) *reported = std::min<int64_t>(h.actual, cycle_niter);
    if (stop_reason_out) *stop_reason_out = h.stop;
}

}  // namespace

void noalloc_prepare(int device) { scratch_address(device); }

}  // namespace cr

extern "C" int cr_hogbom_noalloc(cr_ctx* ctx, float* model, float* residual, const float* psf,
                                 const uint8_t* mask, int32_t nx, int32_t ny, float gain,
                                 float threshold, float cycle_threshold, float nsigma_threshold,
                                 int64_t cycle_niter, int32_t inclusive, int32_t* comp_x,
                                 int32_t* comp_y, float* comp_peak, float* comp_flux,
                                 int64_t* actual, int64_t* reported, int32_t* stop_reason,
                                 char** err) {
    if (err) *err = nullptr;
    try {
        if (!ctx || !model || !residual || !psf) cr::fail(CR_INVALID, "null argument");
        if (!comp_x != !comp_y || !comp_x != !comp_peak || !comp_x != !comp_flux)
            cr::fail(CR_INVALID, "component arrays must be all given or all null");
        cr::hogbom_noalloc(ctx, model, residual, psf, mask, nx, ny, gain, threshold,
                           cycle_threshold, nsigma_threshold, cycle_niter, inclusive, comp_x,
                           comp_y, comp_peak, comp_flux, actual, reported, stop_reason);
        return CR_OK;
    } catch (const cr::Error& e) {
        if (err) *err = strdup(e.what());
        return e.code;
    } catch (const std::exception& e) {
        if (err) *err = strdup(e.what());
        return CR_INVALID;
    }
}
