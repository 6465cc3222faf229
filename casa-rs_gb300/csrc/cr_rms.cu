// cr_rms.cu -- robust RMS of residual images, for the n-sigma threshold.
//
// Restates robust_rms_jy_per_beam (lib.rs:74130-74183) on the device, for
// one plane or many at once:
//   * the values are the finite residuals; with a clean mask that is not
//     all true, only those outside the mask (residual_noise_values,
//     lib.rs:74486-74510);
//   * without such a mask they are clipped by Chauvenet's criterion with
//     the automatic z and at most 5 iterations (apply_chauvenet_clipping,
//     lib.rs:74512-74558): each iteration takes the mean and the sample
//     standard deviation in FP64 and keeps mean - z sd <= v <= mean + z sd;
//   * MADFM = median |v - median(v)| with casacore's even-count mean of the
//     two middle values (casa-lattices statistics.rs:1346-1379), all in
//     FP64, and rms = f32(MADFM) * 1.4826f.
//
// No value is moved or compacted.  A clipped set is the values inside the
// intersection of the iterations' windows, so each iteration is two passes
// over the image (count and sum, then the squared deviations from the
// mean), reduced in a fixed order: per-block partials, then one block per
// plane.  The FP64 sums run in another order than the reference's
// sequential sums; the windows then differ in the last bits, which changes
// the clipped set only for a value within that distance of a window edge.
// The host applies the iteration rules and the Chauvenet z (erfc from the C
// library, as the reference takes it from libm).
//
// The medians are order statistics found by radix selection on keys built
// on the fly: the f32 total-order key of a value (4 passes of 8-bit
// digits), then the FP64 bits of |v - median| (8 passes; non-negative
// doubles order like their bits).  Each pass histograms the next digit of
// the keys that match the digits chosen so far; a one-block kernel per
// plane picks the digit holding the wanted rank.  Selection is exact, so the
// MADFM equals the sorted one bit for bit on the same clipped set.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "cr_internal.cuh"

namespace cr {
namespace {

constexpr int kRmsThreads = 256;

struct RmsState {
    double lo, hi;               // clip window, inclusive
    unsigned long long n;        // values in the window
    double sum, sumsq;           // their sum, and of squared deviations from the mean
    unsigned long long zeros;    // mask entries that are zero (not cleanable)
    int full;                    // 1: all finite values count (no restricting mask)
    int pad;
    // radix selection
    unsigned long long prefix;   // the key digits chosen so far
    unsigned long long rank;     // wanted rank among keys with that prefix
    unsigned long long eq;       // keys equal to the selected key (after the last digit)
    unsigned long long next;     // smallest key above the selected key
    double med;                  // median of the values
    double madfm;                // median absolute deviation from it
};

struct RmsArgs {
    const float* images;    // [P][npix]
    const uint8_t* masks;   // [P][npix] or null
    const int* planes;      // [slots] image plane of each slot
    int64_t npix;
    RmsState* st;           // [slots]
    double* part;           // [slots][bx][2] per-block partials
    unsigned int* hist;     // [slots][256]
    int bx;                 // blocks per slot
};

__device__ __forceinline__ bool take(const RmsArgs& a, const RmsState& s, int64_t base,
                                     int64_t i, float& v) {
    v = a.images[base + i];
    if (!isfinite(v)) return false;
    if (!s.full && a.masks[base + i]) return false;   // inside the clean mask
    const double x = (double)v;
    return x >= s.lo && x <= s.hi;
}

__device__ __forceinline__ unsigned int f32_key(float v) {
    const unsigned int b = __float_as_uint(v);
    return (b & 0x80000000u) ? ~b : (b ^ 0x80000000u);
}

__device__ __forceinline__ float f32_from_key(unsigned int k) {
    return __uint_as_float((k & 0x80000000u) ? (k ^ 0x80000000u) : ~k);
}

// KEY 0: f32 total-order key of v; KEY 1: FP64 bits of |v - med|
template <int KEY>
__device__ __forceinline__ unsigned long long key_of(float v, double med) {
    if (KEY == 0) return f32_key(v);
    return (unsigned long long)__double_as_longlong(fabs(__dsub_rn((double)v, med)));
}

// Block sum of two doubles in a fixed order; result in thread 0.
__device__ void block_sum2(double& x, double& y) {
    __shared__ double sx[kRmsThreads / 32], sy[kRmsThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x = __dadd_rn(x, __shfl_down_sync(0xffffffffu, x, o));
        y = __dadd_rn(y, __shfl_down_sync(0xffffffffu, y, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sx[warp] = x;
        sy[warp] = y;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tx = 0.0, ty = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            tx = __dadd_rn(tx, sx[w]);
            ty = __dadd_rn(ty, sy[w]);
        }
        x = tx;
        y = ty;
    }
    __syncthreads();
}

// MODE 0: (count, sum) of the values in the window; MODE 1: (0, sum of
// (v - mean)^2) with mean = sum / n; MODE 2: (zero mask entries, 0).
template <int MODE>
__global__ void __launch_bounds__(kRmsThreads) rms_partials(RmsArgs a) {
    const int slot = blockIdx.y;
    const RmsState s = a.st[slot];
    const int64_t base = (int64_t)a.planes[slot] * a.npix;
    const double mean = MODE == 1 && s.n > 0 ? __ddiv_rn(s.sum, (double)s.n) : 0.0;
    double c = 0.0, acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.npix;
         i += (int64_t)a.bx * blockDim.x) {
        if (MODE == 2) {
            c += a.masks[base + i] ? 0.0 : 1.0;
            continue;
        }
        float v;
        if (!take(a, s, base, i, v)) continue;
        if (MODE == 0) {
            c += 1.0;
            acc = __dadd_rn(acc, (double)v);
        } else {
            const double d = __dsub_rn((double)v, mean);
            acc = __dadd_rn(acc, __dmul_rn(d, d));
        }
    }
    block_sum2(c, acc);
    if (threadIdx.x == 0) {
        double* p = a.part + ((int64_t)slot * a.bx + blockIdx.x) * 2;
        p[0] = c;
        p[1] = acc;
    }
}

template <int MODE>
__global__ void __launch_bounds__(kRmsThreads) rms_reduce(RmsArgs a) {
    const int slot = blockIdx.x;
    const double* p = a.part + (int64_t)slot * a.bx * 2;
    double c = 0.0, acc = 0.0;
    for (int b = threadIdx.x; b < a.bx; b += blockDim.x) {
        c = __dadd_rn(c, p[2 * b]);
        acc = __dadd_rn(acc, p[2 * b + 1]);
    }
    block_sum2(c, acc);
    if (threadIdx.x == 0) {
        RmsState& s = a.st[slot];
        if (MODE == 0) {
            s.n = (unsigned long long)c;
            s.sum = acc;
        } else if (MODE == 1) {
            s.sumsq = acc;
        } else {
            s.zeros = (unsigned long long)c;
        }
    }
}

// Start a selection of the lower middle rank (n - 1) / 2.
__global__ void rms_select_init(RmsArgs a) {
    RmsState& s = a.st[blockIdx.x];
    if (threadIdx.x == 0) {
        s.prefix = 0ull;
        s.rank = s.n > 0 ? (s.n - 1) / 2 : 0ull;
        s.eq = 0ull;
        s.next = ~0ull;
    }
}

// Histogram of the digit at `shift` of the keys whose bits above it equal
// the prefix.
template <int KEY>
__global__ void __launch_bounds__(kRmsThreads) rms_hist(RmsArgs a, int shift) {
    __shared__ unsigned int h[256];
    for (int t = threadIdx.x; t < 256; t += blockDim.x) h[t] = 0u;
    __syncthreads();
    const int slot = blockIdx.y;
    const RmsState s = a.st[slot];
    const int64_t base = (int64_t)a.planes[slot] * a.npix;
    const int hib = shift + 8;
    const int bits = KEY == 0 ? 32 : 64;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.npix;
         i += (int64_t)a.bx * blockDim.x) {
        float v;
        if (!take(a, s, base, i, v)) continue;
        const unsigned long long k = key_of<KEY>(v, s.med);
        if (hib < bits && (k >> hib) != s.prefix) continue;
        atomicAdd(&h[(unsigned)(k >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 256; t += blockDim.x)
        if (h[t]) atomicAdd(&a.hist[slot * 256 + t], h[t]);
}

// One block of 256 threads per slot: the digit whose bin holds the rank.
__global__ void __launch_bounds__(256) rms_pick(RmsArgs a) {
    __shared__ unsigned int scan[256];
    const int slot = blockIdx.x, t = threadIdx.x;
    RmsState& s = a.st[slot];
    const unsigned int c = a.hist[slot * 256 + t];
    scan[t] = c;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {   // inclusive scan
        const unsigned int add = t >= o ? scan[t - o] : 0u;
        __syncthreads();
        scan[t] += add;
        __syncthreads();
    }
    const unsigned long long rank = s.rank;
    const unsigned long long before = scan[t] - c;
    __syncthreads();
    if (c > 0 && before <= rank && rank < before + c) {
        s.prefix = (s.prefix << 8) | (unsigned long long)t;
        s.rank = rank - before;
        s.eq = c;
    }
    a.hist[slot * 256 + t] = 0u;
}

// The smallest key above the selected one (the upper middle value of an
// even count when the selected key is the last of its equals).
template <int KEY>
__global__ void __launch_bounds__(kRmsThreads) rms_next(RmsArgs a) {
    const int slot = blockIdx.y;
    const RmsState s = a.st[slot];
    if (s.n == 0 || (s.n & 1ull) || s.rank + 1 < s.eq) return;
    const int64_t base = (int64_t)a.planes[slot] * a.npix;
    unsigned long long best = ~0ull;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.npix;
         i += (int64_t)a.bx * blockDim.x) {
        float v;
        if (!take(a, s, base, i, v)) continue;
        const unsigned long long k = key_of<KEY>(v, s.med);
        if (k > s.prefix && k < best) best = k;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long b2 = __shfl_down_sync(0xffffffffu, best, o);
        best = b2 < best ? b2 : best;
    }
    if ((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(&a.st[slot].next, best);
}

// The median from the selected key(s): KEY 0 sets med, KEY 1 sets madfm.
template <int KEY>
__global__ void rms_median(RmsArgs a) {
    if (threadIdx.x != 0) return;
    RmsState& s = a.st[blockIdx.x];
    double lower = 0.0, upper = 0.0;
    if (s.n > 0) {
        const bool same = (s.n & 1ull) || s.rank + 1 < s.eq;
        const unsigned long long up = same ? s.prefix : s.next;
        if (KEY == 0) {
            lower = (double)f32_from_key((unsigned int)s.prefix);
            upper = (double)f32_from_key((unsigned int)up);
        } else {
            lower = __longlong_as_double((long long)s.prefix);
            upper = __longlong_as_double((long long)up);
        }
    }
    const double m = (s.n & 1ull) ? lower : __ddiv_rn(__dadd_rn(lower, upper), 2.0);
    if (KEY == 0)
        s.med = s.n > 0 ? m : 0.0;
    else
        s.madfm = s.n > 0 ? m : 0.0;
}

// `(0.5 / erfc(z / sqrt 2)) as u64` with Rust's saturating cast
// (chauvenet_zscore_to_npts, lib.rs:74624-74626).
uint64_t chauvenet_npts(double z) {
    const double x = 0.5 / std::erfc(z / 1.4142135623730951);
    if (!(x >= 0.0)) return 0;
    if (x >= 18446744073709551615.0) return std::numeric_limits<uint64_t>::max();
    return (uint64_t)x;
}

}  // namespace

// chauvenet_max_zscore (lib.rs:74578-74622).
double chauvenet_max_zscore(uint64_t npts) {
    static const uint64_t cnt[14] = {0,       1,        3,         10,          40,
                                     185,     1074,     7893,      73579,       872138,
                                     13165126ull, 253398672ull, 6225098696ull,
                                     195341107722ull};
    static const double zs[14] = {0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 3.5,
                                  4.0, 4.5, 5.0, 5.5, 6.0, 6.5, 7.0};
    const int L = 14;
    for (int i = 0; i < L; ++i)
        if (cnt[i] == npts) return zs[i];
    int lo = 0, hi = 1;
    if (npts > cnt[L - 1]) {
        double z = zs[L - 1] + 0.5;
        for (;;) {
            if (chauvenet_npts(z) >= npts) {
                lo = L - 2;
                hi = L - 1;
                break;
            }
            z += 0.5;
        }
    } else {
        while (hi < L && cnt[hi] < npts) {
            ++lo;
            ++hi;
        }
    }
    double low_z = zs[lo], high_z = zs[hi];
    double z = (low_z + high_z) / 2.0;
    for (;;) {
        const uint64_t m = chauvenet_npts(z);
        if (m == npts || std::fabs(high_z - low_z) <= 1e-12) return z;
        if (m > npts)
            high_z = z;
        else
            low_z = z;
        z = (low_z + high_z) / 2.0;
    }
}

void robust_rms(cr_ctx* ctx, const float* images, const uint8_t* masks, int64_t npix,
                const std::vector<int>& planes, float* rms, double* madfm, int64_t* counts) {
    const int np = (int)planes.size();
    if (np == 0) return;
    if (npix <= 0) fail(CR_INVALID, "image shape must be positive");
    if (np > 65535) fail(CR_INVALID, "at most 65535 planes per call");
    // blocks per plane: about four waves of the device over all planes
    const int bx = (int)std::max<int64_t>(
        1, std::min<int64_t>((npix + kRmsThreads - 1) / kRmsThreads,
                             std::max<int64_t>(1, (int64_t)ctx->sms * 8 / np)));
    int* planes_d = (int*)workspace(ctx, "rms_planes", (size_t)np * 4);
    RmsState* st = (RmsState*)workspace(ctx, "rms_state", (size_t)np * sizeof(RmsState));
    double* part = (double*)workspace(ctx, "rms_part", (size_t)np * bx * 16);
    unsigned int* hist = (unsigned int*)workspace(ctx, "rms_hist", (size_t)np * 256 * 4);
    CR_CUDA_CHECK(cudaMemcpyAsync(planes_d, planes.data(), (size_t)np * 4,
                                  cudaMemcpyHostToDevice, ctx->stream));
    CR_CUDA_CHECK(cudaMemsetAsync(hist, 0, (size_t)np * 256 * 4, ctx->stream));
    std::vector<RmsState> h((size_t)np);
    for (auto& s : h) {
        std::memset(&s, 0, sizeof(s));
        s.lo = -std::numeric_limits<double>::infinity();
        s.hi = std::numeric_limits<double>::infinity();
        s.full = 1;
    }
    RmsArgs a{images, masks, planes_d, npix, st, part, hist, bx};
    const dim3 grid(bx, np);
    auto upload = [&] {
        CR_CUDA_CHECK(cudaMemcpyAsync(st, h.data(), (size_t)np * sizeof(RmsState),
                                      cudaMemcpyHostToDevice, ctx->stream));
    };
    auto download = [&] {
        CR_CUDA_CHECK(cudaMemcpyAsync(h.data(), st, (size_t)np * sizeof(RmsState),
                                      cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    };
    upload();
    if (masks) {
        // a mask that is all true does not restrict the values (full_mask)
        rms_partials<2><<<grid, kRmsThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "rms_partials");
        rms_reduce<2><<<np, kRmsThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "rms_reduce");
        download();
        for (auto& s : h) s.full = s.zeros == 0 ? 1 : 0;
        upload();
    }
    // Chauvenet clipping of the full-mask planes: apply_chauvenet_clipping
    // (values, -1.0, 5): while iteration <= 5 and values remain, stop when
    // the count did not change, or the mean or deviation is not finite or
    // the deviation is not positive.
    std::vector<int> active((size_t)np), iter((size_t)np, 0);
    std::vector<unsigned long long> prev((size_t)np, 0);
    for (int k = 0; k < np; ++k) active[k] = h[k].full;
    for (;;) {
        rms_partials<0><<<grid, kRmsThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "rms_partials");
        rms_reduce<0><<<np, kRmsThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "rms_reduce");
        rms_partials<1><<<grid, kRmsThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "rms_partials");
        rms_reduce<1><<<np, kRmsThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "rms_reduce");
        download();
        bool any = false;
        for (int k = 0; k < np; ++k) {
            if (!active[k]) continue;
            RmsState& s = h[k];
            const unsigned long long n = s.n;
            if (n == 0 || iter[k] > 5 || (iter[k] > 0 && n == prev[k])) {
                active[k] = 0;
                continue;
            }
            const double nn = (double)n;
            const double mean = s.sum / nn;
            const double var = n > 1 ? s.sumsq / (nn - 1.0) : 0.0;
            const double sd = std::sqrt(var);
            if (!std::isfinite(mean) || !std::isfinite(sd) || sd <= 0.0) {
                active[k] = 0;
                continue;
            }
            const double z = chauvenet_max_zscore(n);
            const double low = mean - z * sd, high = mean + z * sd;
            s.lo = std::max(s.lo, low);
            s.hi = std::min(s.hi, high);
            prev[k] = n;
            ++iter[k];
            any = true;
        }
        if (!any) break;
        upload();
    }
    // the two medians
    rms_select_init<<<np, 32, 0, ctx->stream>>>(a);
    note_launch(ctx, "rms_select_init");
    for (int shift = 24; shift >= 0; shift -= 8) {
        rms_hist<0><<<grid, kRmsThreads, 0, ctx->stream>>>(a, shift);
        note_launch(ctx, "rms_hist");
        rms_pick<<<np, 256, 0, ctx->stream>>>(a);
        note_launch(ctx, "rms_pick");
    }
    rms_next<0><<<grid, kRmsThreads, 0, ctx->stream>>>(a);
    note_launch(ctx, "rms_next");
    rms_median<0><<<np, 32, 0, ctx->stream>>>(a);
    note_launch(ctx, "rms_median");
    rms_select_init<<<np, 32, 0, ctx->stream>>>(a);
    note_launch(ctx, "rms_select_init");
    for (int shift = 56; shift >= 0; shift -= 8) {
        rms_hist<1><<<grid, kRmsThreads, 0, ctx->stream>>>(a, shift);
        note_launch(ctx, "rms_hist");
        rms_pick<<<np, 256, 0, ctx->stream>>>(a);
        note_launch(ctx, "rms_pick");
    }
    rms_next<1><<<grid, kRmsThreads, 0, ctx->stream>>>(a);
    note_launch(ctx, "rms_next");
    rms_median<1><<<np, 32, 0, ctx->stream>>>(a);
    note_launch(ctx, "rms_median");
    download();
    for (int k = 0; k < np; ++k) {
        const RmsState& s = h[k];
        if (rms) rms[k] = s.n > 0 ? (float)s.madfm * 1.4826f : 0.0f;
        if (madfm) madfm[k] = s.n > 0 ? s.madfm : 0.0;
        if (counts) counts[k] = (int64_t)s.n;
    }
}

}  // namespace cr
