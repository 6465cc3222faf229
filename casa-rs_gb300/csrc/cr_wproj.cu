// cr_wproj.cu -- W-projection kernels: construction, gridding, degridding.
//
// Construction restates WProjector::new (gridder.rs:3403-3586): per w-plane a
// phase screen corr(l)corr(m) exp(2 pi i w_k (sqrt(1-l^2-m^2) - 1)) with the
// phase in FP64, a forward 2-D FFT (cuFFT, the bare transform), a crop to
// the plane's support, division by the plane-zero integral, and the
// per-(plane, offset) normalisation table.
//
// The cropped kernel K_p[kx, ky] (kx = |i s + off_x| for tap i of a sample
// with oversampling offset off_x) is stored once per plane as a residue cube
//   C_p[rx][ry][qx][qy] = K_p[qx s + rx, qy s + ry],
// so the address of tap (i, j) separates into A(i) + B(j) with
//   A = rx s Q^2 + qx Q and B = ry Q^2 + qy  (Q = qx extent of the plane),
// and consecutive taps of one row are consecutive in memory on each side of
// the sample.  The cube holds each kernel value once (about 0.1 GB for 128
// planes with supports up to 64 at oversampling 8), small enough to stay in
// L2, where per-offset copies of the taps would not.
//
// Gridding is output-stationary: a warp owns an 8-row band of a 32 x 32
// tile of the grid in registers (each lane one column), streams the
// deduplicated records whose windows can reach the tile, and adds
// value * kernel for every owned cell inside a record's window.  The band is
// flushed once per work item with FP32 atomics.  Degridding is a gather: a
// warp per record takes the window's rows in pairs, 16 lanes per row, with
// the cube column addresses held in registers, and reduces with warp
// shuffles.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "cr_internal.cuh"

namespace cr {

namespace {

constexpr int kMaxSegRadius = 4;   // neighbourhood radius in tiles (supports up to 127)

// ---- construction ----------------------------------------------------------------
__global__ void screen_kernel(float2* buf, int64_t conv, int64_t inner, int planes_in_batch,
                              int plane0, int32_t nplanes, double w_scale, double s0, double s1,
                              const float* corr) {
    const int64_t half = inner / 2;
    const int64_t total = inner * inner * planes_in_batch;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int b = (int)(t / (inner * inner));
        int64_t rem = t - (int64_t)b * inner * inner;
        int64_t ixi = rem / inner, iyi = rem - ixi * inner;
        int64_t ix = ixi - half, iy = iyi - half;
        int plane = plane0 + b;
        double w = nplanes > 1 ? (double)((int64_t)plane * plane) / w_scale : 0.0;
        double l = s0 * (double)ix, m = s1 * (double)iy;
        double rsq = __dadd_rn(__dmul_rn(l, l), __dmul_rn(m, m));
        if (rsq >= 1.0) continue;
        double phase = __dmul_rn(__dmul_rn(6.283185307179586476925, w), sqrt(1.0 - rsq) - 1.0);
        double sn, cs;
        sincos(phase, &sn, &cs);
        float c = __fmul_rn(corr[ixi], corr[iyi]);
        int64_t x = ix >= 0 ? ix : ix + conv;
        int64_t y = iy >= 0 ? iy : iy + conv;
        buf[(int64_t)b * conv * conv + x * conv + y] =
            make_float2(__fmul_rn(c, (float)cs), __fmul_rn(c, (float)sn));
    }
}

__global__ void crop_kernel(const float2* buf, int64_t conv, int planes_in_batch, int plane0,
                            const int32_t* crop, int32_t width, float2* kernels) {
    const int64_t total = (int64_t)planes_in_batch * width * width;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int b = (int)(t / ((int64_t)width * width));
        int64_t rem = t - (int64_t)b * width * width;
        int x = (int)(rem / width), y = (int)(rem - (int64_t)x * width);
        int plane = plane0 + b;
        int cw = crop[plane];
        float2 v = make_float2(0.0f, 0.0f);
        if (x < cw && y < cw) v = buf[(int64_t)b * conv * conv + (int64_t)x * conv + y];
        kernels[(int64_t)plane * width * width + (int64_t)x * width + y] = v;
    }
}

__global__ void axis_kernel(const float2* buf, int64_t conv, int planes_in_batch,
                            int64_t axis_len, double* axes) {
    const int64_t total = (int64_t)planes_in_batch * axis_len;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int b = (int)(t / axis_len);
        int64_t c = t - (int64_t)b * axis_len;
        const float2* p = buf + (int64_t)b * conv * conv;
        float2 ax = p[c * conv];  // T(c, 0)
        float2 ay = p[c];         // T(0, c)
        axes[((int64_t)b * 2) * axis_len + c] = hypot((double)ax.x, (double)ax.y);
        axes[((int64_t)b * 2 + 1) * axis_len + c] = hypot((double)ay.x, (double)ay.y);
    }
}

// FP64 sum of Re K over the integer taps of one plane (w_project_plane_sum,
// gridder.rs:3991-4002), or over one offset (compute_w_project_sample_
// normalization, gridder.rs:3782-3799).  One block per (plane, offset).
__global__ void tap_sum_kernel(const float2* kernels, int32_t width, const int32_t* support,
                               int32_t sampling, int32_t radius, int32_t axis, int plane0,
                               double* out_double, float* out_float) {
    int plane = plane0 + blockIdx.y;
    int offidx = blockIdx.x;
    int ox = offidx / axis - radius, oy = offidx % axis - radius;
    int s = support[plane];
    int w = 2 * s + 1;
    const float2* k = kernels + (int64_t)plane * width * width;
    double acc = 0.0;
    bool ok = true;
    for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
        int ix = t / w - s, iy = t % w - s;
        int kx = abs(ix * sampling + ox), ky = abs(iy * sampling + oy);
        if (kx >= width || ky >= width) {
            ok = false;
            continue;
        }
        acc += (double)k[(int64_t)kx * width + ky].x;
    }
    __shared__ double sh[32];
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    if (!ok) bad = 1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
        if (bad) t = 0.0;
        int64_t idx = ((int64_t)plane * axis) * axis + offidx;
        if (out_double) out_double[idx] = t;
        if (out_float) out_float[idx] = (float)t;
    }
}

__global__ void scale_kernels(float2* k, int64_t n, float scale) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        float2 v = k[t];
        k[t] = make_float2(v.x * scale, v.y * scale);
    }
}

__global__ void cube_kernel(const float2* kernels, int32_t width, int plane, int32_t s,
                            int32_t q, float2* cube) {
    const int64_t qq = (int64_t)q * q;
    const int64_t total = (int64_t)s * s * qq;
    const float2* k = kernels + (int64_t)plane * width * width;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t res = t / qq;
        int64_t rem = t - res * qq;
        int rx = (int)(res / s), ry = (int)(res % s);
        int qx = (int)(rem / q), qy = (int)(rem % q);
        int kx = qx * s + rx, ky = qy * s + ry;
        cube[t] = (kx < width && ky < width) ? k[(int64_t)kx * width + ky] : make_float2(0.f, 0.f);
    }
}

// floor(k / s) for 0 <= k < 2^26 and 1 <= s <= 64 by a multiply-high with
// magic = floor(2^32 / s) + 1 (exact in that range).
__device__ __forceinline__ int qdiv(int k, unsigned long long magic) {
    return (int)(((unsigned long long)(unsigned)k * magic) >> 32);
}

struct CubeGeom {
    int s;                     // sampling
    unsigned long long magic;  // for qdiv by s
};

// Address parts of kernel tap t (t in [-S, S]) for offset off:
// x-side A = rx s Q^2 + qx Q, y-side B = ry Q^2 + qy.
__device__ __forceinline__ int cube_a(int t, int off, int q, const CubeGeom& c) {
    int k = abs(t * c.s + off);
    int qk = qdiv(k, c.magic);
    return (k - qk * c.s) * c.s * q * q + qk * q;
}

__device__ __forceinline__ int cube_b(int t, int off, int q, const CubeGeom& c) {
    int k = abs(t * c.s + off);
    int qk = qdiv(k, c.magic);
    return (k - qk * c.s) * q * q + qk;
}

// ---- gridding ---------------------------------------------------------------------
// One warp per work item (output tile, band of kBandRows rows, chunk of
// candidate records); no block-level barriers.  Lane l owns column l of the
// tile and keeps per band row three float2 accumulators,
//   X = sum k (.) (vr, -t vi),  Y = sum k (.) (vi, t vr),  P = sum k (.) (w, t w)
// (k = (kr, ki) the kernel value, t = -1 for a conjugated record, (.) the
// element-wise product), one paired FMA each per tap; the flush forms
// dirty = (X.x + X.y, Y.x + Y.y) and psf = P.  The warp examines its
// candidates 32 at a time, one per lane, from records packed once per pass
// (16 bytes each, prefetched a batch ahead with cp.async), and compacts those
// whose window reaches its band into warp-private shared memory with their
// row addresses.
constexpr int kBandRows = 8;
constexpr int kBands = kTile / kBandRows;   // 4 bands per tile
constexpr int kBandWarps = 8;               // warps per block
constexpr int kBandChunk = 256;             // candidate records per work item
constexpr int kNbr = (2 * kMaxSegRadius + 1) * (2 * kMaxSegRadius + 1);

struct __align__(16) BandEntry {
    float4 vx;        // (vr, -t vi, vi, t vr)
    float2 pw;        // (w, t w)
    int cb, w;        // window column of tile column 0; window width 2S+1
    long long base;   // element offset of the plane's residue cube
    int s, oy, q, pad;
};

// Each record packed once per pass: x = (lx << 16) | ly, y = plane |
// (ox + radius) << 12 | (oy + radius) << 18 | conj << 24 | support << 25,
// z, w = the float32 value (vr, vi) (w vis - w pred with RESIDUAL); the
// weight separately.
inline bool band_pack_fits(int64_t gn, int planes, int radius, int smax) {
    return gn <= 65536 && planes <= 4096 && 2 * radius + 1 <= 64 && smax <= 127;
}

template <bool RESIDUAL>
__global__ void band_pack_kernel(const int32_t* rx, const int32_t* ry, const int32_t* rplane,
                                 const int32_t* roff, const int32_t* rconj, const double2* vsum,
                                 const double* wsum, const float2* pred, const int32_t* support,
                                 int32_t axis, const unsigned long long* counts, uint4* packed,
                                 float* weight) {
    const int64_t n = (int64_t)counts[2];
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int plane = rplane[r];
        const int off = roff[r];
        const unsigned meta = (unsigned)plane | (unsigned)(off / axis) << 12 |
                              (unsigned)(off % axis) << 18 | (unsigned)(rconj[r] ? 1 : 0) << 24 |
                              (unsigned)support[plane] << 25;
        const double2 vs = vsum[r];
        const double ws = wsum[r];
        float vr, vi;
        if (RESIDUAL) {
            const float2 p = pred[r];
            vr = (float)(vs.x - (double)p.x * ws);
            vi = (float)(vs.y - (double)p.y * ws);
        } else {
            vr = (float)vs.x;
            vi = (float)vs.y;
        }
        packed[r] = make_uint4((unsigned)rx[r] << 16 | (unsigned)ry[r], meta, __float_as_uint(vr),
                               __float_as_uint(vi));
        weight[r] = (float)ws;
    }
}

struct BandArgs {
    const uint4* packed;
    const float* weight;
    const int64_t* cube_off;
    const int32_t* cube_q;
    const float2* cube;
    CubeGeom cg;
    int32_t radius;
    int64_t nty;
    const uint32_t* seg_lo;    // [ntiles][kNbr] first candidate record of each segment
    const uint32_t* seg_pre;   // [ntiles][kNbr + 1] exclusive prefix of segment lengths
    const uint8_t* nseg;       // [ntiles]
    const uint2* items;        // (tile * kBands + band, first candidate)
    const unsigned long long* n_items;
    unsigned int* item_counter;
    float2* psf;
    float2* dirty;
    int64_t gnx, gny;
};

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <bool RESIDUAL>
__global__ void __launch_bounds__(kBandWarps * 32, 3) wp_grid_kernel(BandArgs a) {
    __shared__ BandEntry s_ent[kBandWarps][32];
    __shared__ __align__(16) int s_rows[kBandWarps][32][kBandRows];
    __shared__ uint32_t s_lo[kBandWarps][kNbr];
    __shared__ uint32_t s_pre[kBandWarps][kNbr + 1];
    // the packed candidates of the current and the next batch
    __shared__ uint4 s_pk[kBandWarps][2][32];
    __shared__ float s_wt[kBandWarps][2][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long n_items = *a.n_items;
    BandEntry* ent = s_ent[warp];
    uint32_t* lo_s = s_lo[warp];
    uint32_t* pre_s = s_pre[warp];
    for (;;) {
        unsigned int item = 0;
        if (lane == 0) item = atomicAdd(a.item_counter, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if ((unsigned long long)item >= n_items) break;
        const uint2 it = a.items[item];
        const int64_t T = it.x / kBands;
        const int band = (int)(it.x % kBands);
        const int x0 = (int)((T / a.nty) * kTile) + band * kBandRows;
        const int y0 = (int)((T % a.nty) * kTile);
        const int ns = a.nseg[T];
        for (int k = lane; k < ns; k += 32) lo_s[k] = a.seg_lo[T * kNbr + k];
        for (int k = lane; k <= ns; k += 32) pre_s[k] = a.seg_pre[T * (kNbr + 1) + k];
        __syncwarp();
        const uint32_t cbeg = it.y, cend = min(pre_s[ns], cbeg + (uint32_t)kBandChunk);
        // lane l's candidate c (segment k with pre[k] <= c < pre[k+1]) into
        // candidate buffer b
        auto fetch = [&](uint32_t c, int b) {
            if (c < cend) {
                int lo = 0, hi = ns - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (pre_s[mid] <= c) lo = mid; else hi = mid - 1;
                }
                const uint32_t r = lo_s[lo] + (c - pre_s[lo]);
                cp_async16(&s_pk[warp][b][lane], a.packed + r);
                cp_async4(&s_wt[warp][b][lane], a.weight + r);
            }
            cp_async_commit();
        };
        fetch(cbeg + lane, 0);
        int buf = 0;

        float2 X[kBandRows], Y[kBandRows], P[kBandRows];
#pragma unroll
        for (int k = 0; k < kBandRows; ++k) X[k] = Y[k] = P[k] = make_float2(0.f, 0.f);

        for (uint32_t c0 = cbeg; c0 < cend; c0 += 32) {
            // 1. one candidate per lane: does its window reach the band?  The
            // taken ones write their entry and row addresses straight into
            // their compacted slot.  The next batch's candidates are copied
            // in while this batch is worked on.
            if (c0 + 32 < cend) {
                fetch(c0 + 32 + lane, buf ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            const bool valid = c0 + lane < cend;
            const uint4 pk = valid ? s_pk[warp][buf][lane] : make_uint4(0u, 0u, 0u, 0u);
            const float wt = valid ? s_wt[warp][buf][lane] : 0.0f;
            buf ^= 1;
            const int lx = (int)(pk.x >> 16), ly = (int)(pk.x & 0xffffu);
            const int sup = (int)(pk.y >> 25);
            const bool take = valid && lx - sup <= x0 + kBandRows - 1 && lx + sup >= x0 &&
                              ly - sup <= y0 + kTile - 1 && ly + sup >= y0;
            const unsigned bal = __ballot_sync(0xffffffffu, take);
            if (take) {
                const int slot = __popc(bal & ((1u << lane) - 1u));
                BandEntry& e = ent[slot];
                const int plane = (int)(pk.y & 0xfffu);
                const int ox = (int)((pk.y >> 12) & 63u) - a.radius;
                const int q = a.cube_q[plane];
                const int w = 2 * sup + 1;
                e.oy = (int)((pk.y >> 18) & 63u) - a.radius;
                e.s = sup;
                e.w = w;
                e.q = q;
                e.base = a.cube_off[plane];
                e.cb = y0 - ly + sup;
                const float vr = __uint_as_float(pk.z), vi = __uint_as_float(pk.w);
                const float t = ((pk.y >> 24) & 1u) ? -1.0f : 1.0f;
                e.vx = make_float4(vr, -t * vi, vi, t * vr);
                e.pw = make_float2(wt, t * wt);
                int* rows = s_rows[warp][slot];
#pragma unroll
                for (int k = 0; k < kBandRows; ++k) {
                    const int i = x0 + k - lx + sup;   // window row
                    rows[k] = (i >= 0 && i < w) ? cube_a(i - sup, ox, q, a.cg) : -1;
                }
            }
            __syncwarp();
            // 2. accumulate the taken entries into the band: all the rows'
            // kernel values are loaded (zero outside the window) before the
            // paired FMAs
            const int nt = __popc(bal);
            for (int q = 0; q < nt; ++q) {
                const BandEntry& E = ent[q];
                const int col = E.cb + lane;
                const bool colok = (unsigned)col < (unsigned)E.w;
                const int bcol = colok ? cube_b(col - E.s, E.oy, E.q, a.cg) : 0;
                const float2* kp = a.cube + E.base + bcol;
                const int4 ra = *reinterpret_cast<const int4*>(&s_rows[warp][q][0]);
                const int4 rb = *reinterpret_cast<const int4*>(&s_rows[warp][q][4]);
                const int av[kBandRows] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w};
                float2 kv[kBandRows];
#pragma unroll
                for (int k = 0; k < kBandRows; ++k)
                    kv[k] = (colok && av[k] >= 0) ? __ldg(kp + av[k]) : make_float2(0.f, 0.f);
                const float4 vx = E.vx;
                const float2 v1 = make_float2(vx.x, vx.y), v2 = make_float2(vx.z, vx.w);
                const float2 pw = E.pw;
#pragma unroll
                for (int k = 0; k < kBandRows; ++k) {
                    X[k] = __ffma2_rn(kv[k], v1, X[k]);
                    Y[k] = __ffma2_rn(kv[k], v2, Y[k]);
                    if (!RESIDUAL) P[k] = __ffma2_rn(kv[k], pw, P[k]);
                }
            }
            __syncwarp();
        }
        // 3. flush the band
#pragma unroll
        for (int k = 0; k < kBandRows; ++k) {
            const int64_t x = x0 + k, y = y0 + lane;
            if (x < a.gnx && y < a.gny) {
                const int64_t cell = x * a.gny + y;
                const float2 d = make_float2(X[k].x + X[k].y, Y[k].x + Y[k].y);
                if (!RESIDUAL && (P[k].x != 0.0f || P[k].y != 0.0f)) atomicAdd(&a.psf[cell], P[k]);
                if (d.x != 0.0f || d.y != 0.0f) atomicAdd(&a.dirty[cell], d);
            }
        }
        __syncwarp();
    }
}

// Per output tile: the segments of candidate records of its neighbourhood
// (home tiles within R tiles), each trimmed to the records whose support can
// reach the tile when supports grow with the plane index (records of a home
// tile are sorted by plane); the work items are the tile's bands times the
// chunks of kBandChunk candidates.
__global__ void band_work_count(const uint32_t* tile_start, const int32_t* rplane,
                                const int32_t* first_plane, int32_t max_support, int monotone,
                                int64_t ntx, int64_t nty, int R, int64_t gnx,
                                uint32_t* seg_lo, uint32_t* seg_pre, uint8_t* nseg,
                                uint32_t* nitems) {
    const int64_t ntiles = ntx * nty;
    for (int64_t T = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; T < ntiles;
         T += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tx = T / nty, ty = T % nty;
        uint32_t total = 0;
        int n = 0;
        for (int dx = -R; dx <= R; ++dx) {
            const int64_t hx = tx + dx;
            if (hx < 0 || hx >= ntx) continue;
            for (int dy = -R; dy <= R; ++dy) {
                const int64_t hy = ty + dy;
                if (hy < 0 || hy >= nty) continue;
                const int64_t h = hx * nty + hy;
                uint32_t lo = tile_start[h];
                const uint32_t hi = tile_start[h + 1];
                if (lo >= hi) continue;
                if (monotone) {
                    const int ax = dx == 0 ? 0 : kTile * (abs(dx) - 1) + 1;
                    const int ay = dy == 0 ? 0 : kTile * (abs(dy) - 1) + 1;
                    const int need = max(ax, ay);
                    if (need > max_support) continue;
                    const int p = first_plane[need];
                    uint32_t l = lo, u = hi;   // first record with plane >= p
                    while (l < u) {
                        const uint32_t m = l + ((u - l) >> 1);
                        if (rplane[m] < p) l = m + 1; else u = m;
                    }
                    lo = l;
                    if (lo >= hi) continue;
                }
                seg_lo[T * kNbr + n] = lo;
                seg_pre[T * (kNbr + 1) + n] = total;
                total += hi - lo;
                ++n;
            }
        }
        seg_pre[T * (kNbr + 1) + n] = total;
        nseg[T] = (uint8_t)n;
        const int64_t rows_left = gnx - tx * kTile;
        const int64_t nb = (rows_left + kBandRows - 1) / kBandRows;
        const int bands = (int)(nb < kBands ? nb : kBands);
        nitems[T] = total ? (uint32_t)bands * ((total + kBandChunk - 1) / kBandChunk) : 0u;
    }
}

__global__ void band_work_fill(const uint32_t* nitems, const uint32_t* first, int64_t ntx,
                               int64_t nty, int64_t gnx, uint2* items) {
    const int64_t ntiles = ntx * nty;
    for (int64_t T = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; T < ntiles;
         T += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t n = nitems[T];
        if (!n) continue;
        const int64_t rows_left = gnx - (T / nty) * kTile;
        const int64_t nb = (rows_left + kBandRows - 1) / kBandRows;
        const uint32_t bands = (uint32_t)(nb < kBands ? nb : kBands);
        const uint32_t chunks = n / bands, f = first[T];
        // chunk-major, band-minor: the bands of one chunk are consecutive items
        for (uint32_t ch = 0; ch < chunks; ++ch)
            for (uint32_t b = 0; b < bands; ++b)
                items[f + ch * bands + b] =
                    make_uint2((uint32_t)T * kBands + b, ch * (uint32_t)kBandChunk);
    }
}

// ---- degridding --------------------------------------------------------------------
struct DegridArgs {
    const int32_t *rx, *ry, *rplane, *roff, *rconj;
    const unsigned long long* counts;
    const int32_t* support;
    const int64_t* cube_off;
    const int32_t* cube_q;
    const float2* cube;
    CubeGeom cg;
    int32_t radius, axis;
    const float2* grid;
    int64_t gny;
    float2* pred;
};

// Rows of one record's window in pairs (lanes 0-15 row i, lanes 16-31 row
// i+1), 16-lane column chunks whose cube column addresses stay in registers
// for the whole record; NCH chunks cover windows up to 16*NCH wide.
template <int NCH>
__device__ __forceinline__ void degrid_rows(const float2* g, const float2* cube, int gny, int s,
                                            int w, int ox, int oy, int q, const CubeGeom& cg,
                                            int half, int hl, float2& AC, float2& DB) {
    int bcol[NCH];
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
        const int j = hl + 16 * c;
        bcol[c] = j < w ? cube_b(j - s, oy, q, cg) : -1;
    }
    for (int i = half; i < w; i += 2) {
        const float2* grow = g + (int64_t)i * gny + hl;
        const float2* krow = cube + cube_a(i - s, ox, q, cg);
        float2 gv[NCH], kv[NCH];
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            const bool ok = bcol[c] >= 0;
            gv[c] = ok ? grow[16 * c] : make_float2(0.f, 0.f);
            kv[c] = ok ? __ldg(krow + bcol[c]) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            AC = __ffma2_rn(make_float2(kv[c].x, kv[c].x), gv[c], AC);
            DB = __ffma2_rn(make_float2(kv[c].y, kv[c].y), gv[c], DB);
        }
    }
}

// Any window: lane l takes taps l, l+32, ... of the flattened (2S+1)^2
// window, tracking its (row, column) incrementally.
__device__ void degrid_flat(const float2* g, const float2* cube, int gny, int s, int w, int ox,
                            int oy, int q, const CubeGeom& cg, int lane, float2& AC,
                            float2& DB) {
    const int nt = w * w;
    int i = lane / w, j = lane - (lane / w) * w;
    int goff = i * gny + j;
    int arow = cube_a(i - s, ox, q, cg);
    for (int t = lane; t < nt; t += 32) {
        const float2 gv = g[goff];
        const float2 kv = __ldg(cube + arow + cube_b(j - s, oy, q, cg));
        AC = __ffma2_rn(make_float2(kv.x, kv.x), gv, AC);
        DB = __ffma2_rn(make_float2(kv.y, kv.y), gv, DB);
        j += 32;
        goff += 32;
        bool wrapped = false;
        while (j >= w) {
            j -= w;
            ++i;
            goff += gny - w;
            wrapped = true;
        }
        if (wrapped && i < w) arow = cube_a(i - s, ox, q, cg);
    }
}

// One warp per record: sum conj(cwt) * grid over the window
// (degrid_sample_planned, gridder.rs:3726-3747), then warp shuffles.
__global__ void __launch_bounds__(256, 4) wp_degrid_kernel(DegridArgs a) {
    const int lane = threadIdx.x & 31;
    const int half = lane >> 4, hl = lane & 15;
    const int64_t nrec = (int64_t)a.counts[2];
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int gny = (int)a.gny;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrec;
         r += nwarps) {
        const int plane = a.rplane[r];
        const int s = a.support[plane];
        const int w = 2 * s + 1;
        const int q = a.cube_q[plane];
        const int off = a.roff[r];
        const int ox = off / a.axis - a.radius, oy = off % a.axis - a.radius;
        const float2* cube = a.cube + a.cube_off[plane];
        const float2* g = a.grid + (int64_t)(a.rx[r] - s) * a.gny + (a.ry[r] - s);
        // (A, C) = sum kx (gx, gy), (D, B) = sum ky (gx, gy)
        float2 AC = make_float2(0.f, 0.f), DB = make_float2(0.f, 0.f);
        switch ((w + 15) >> 4) {
#define CR_DEGRID_CASE(N) \
    case N:               \
        degrid_rows<N>(g, cube, gny, s, w, ox, oy, q, a.cg, half, hl, AC, DB); \
        break;
            CR_DEGRID_CASE(1)
            CR_DEGRID_CASE(2)
            CR_DEGRID_CASE(3)
            CR_DEGRID_CASE(4)
            CR_DEGRID_CASE(5)
            CR_DEGRID_CASE(6)
            CR_DEGRID_CASE(7)
            CR_DEGRID_CASE(8)
            CR_DEGRID_CASE(9)
#undef CR_DEGRID_CASE
            default:
                degrid_flat(g, cube, gny, s, w, ox, oy, q, a.cg, lane, AC, DB);
        }
        float A = AC.x, C = AC.y, D = DB.x, B = DB.y;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            A += __shfl_xor_sync(0xffffffffu, A, o);
            B += __shfl_xor_sync(0xffffffffu, B, o);
            C += __shfl_xor_sync(0xffffffffu, C, o);
            D += __shfl_xor_sync(0xffffffffu, D, o);
        }
        if (lane == 0)
            a.pred[r] = a.rconj[r] ? make_float2(A - B, C + D) : make_float2(A + B, C - D);
    }
}

__global__ void broadcast_kernel(const int32_t* sample_rec, const float2* rec_pred, int64_t n,
                                 float2* pred) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int32_t r = sample_rec[i];
        pred[i] = r >= 0 ? rec_pred[r] : make_float2(0.0f, 0.0f);
    }
}

CubeGeom cube_geom(const cr_wproj* wp) {
    CubeGeom c;
    c.s = wp->info.sampling;
    c.magic = (1ull << 32) / (unsigned long long)c.s + 1ull;
    return c;
}

int sm_count(cr_ctx* ctx) {
    int v = 0;
    CR_CUDA_CHECK(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, ctx->device));
    return v;
}

}  // namespace

// ---- construction driver ------------------------------------------------------------
void build_wproj(cr_ctx* ctx, cr_wproj* wp, double max_abs_w, int32_t planes,
                 int32_t sampling, int32_t support_min, int32_t support_max) {
    cr_gridder* g = wp->g;
    const cr_geometry& geom = g->geom;
    const int64_t gnx = g->info.grid_nx, gny = g->info.grid_ny;
    bool explicit_planes = planes > 0;
    if (!explicit_planes) {
        // choose_w_project_plane_count (gridder.rs:3801-3830)
        int64_t p = 1;
        if (std::isfinite(max_abs_w) && max_abs_w > 0.0) {
            double half = std::max((double)geom.nx * std::fabs(geom.cell_x_rad),
                                   (double)geom.ny * std::fabs(geom.cell_y_rad)) / 2.0;
            p = (int64_t)(1.05 * max_abs_w * std::fabs(std::sin(half)));
        }
        planes = (int32_t)std::max<int64_t>(p, 1);
    }
    if (planes > 4096) fail(CR_INVALID, "more than 4096 w-planes");
    if (sampling <= 0) sampling = planes > 1 ? 4 : 1;
    const int64_t conv = std::max(gnx, gny);
    const int64_t inner = std::max<int64_t>(conv / sampling, 2);
    const int64_t quarter = conv / 2 - 1;
    const int32_t radius = (sampling + 1) / 2;
    const int32_t axis = 2 * radius + 1;
    double s0 = std::fabs(geom.cell_x_rad) * sampling * (double)gnx / (double)conv;
    double s1 = std::fabs(geom.cell_y_rad) * sampling * (double)gny / (double)conv;
    double eff = explicit_planes ? 0.25 / std::fabs(geom.cell_x_rad) : 1.05 * max_abs_w;
    double w_scale = (planes > 1 && std::isfinite(eff) && eff > 0.0)
                         ? (double)((int64_t)(planes - 1) * (planes - 1)) / eff
                         : 1.0;
    const bool law = support_min > 0;
    std::vector<int32_t> support(planes, 0), crop(planes, 0);
    if (law) {
        if (support_max < support_min) fail(CR_INVALID, "support_max < support_min");
        for (int32_t p = 0; p < planes; ++p) {
            double frac = planes > 1 ? (double)p / (double)(planes - 1) : 0.0;
            support[p] = support_min + (int32_t)std::llround((double)(support_max - support_min) * frac);
            int64_t cw = (int64_t)support[p] * sampling + radius + 1;
            if (cw > quarter) fail(CR_INVALID, "W-projection support too large for the grid");
            crop[p] = (int32_t)cw;
        }
    } else {
        int64_t ms = std::max<int64_t>(quarter / sampling - 1, 1);
        int64_t cw = std::min<int64_t>(ms * sampling + radius + 1, quarter);
        for (int32_t p = 0; p < planes; ++p) crop[p] = (int32_t)std::max<int64_t>(cw, 1);
    }
    int32_t stride = *std::max_element(crop.begin(), crop.end());

    std::vector<float> corr = gridder_correction_axis(inner);
    float* corr_d = (float*)workspace(ctx, "wk_corr", (size_t)inner * 4);
    CR_CUDA_CHECK(cudaMemcpyAsync(corr_d, corr.data(), (size_t)inner * 4, cudaMemcpyHostToDevice, ctx->stream));
    int32_t* crop_d = (int32_t*)workspace(ctx, "wk_crop", (size_t)planes * 4);
    CR_CUDA_CHECK(cudaMemcpyAsync(crop_d, crop.data(), (size_t)planes * 4, cudaMemcpyHostToDevice, ctx->stream));

    // raw (unnormalised) crops at the largest crop width
    float2* raw = nullptr;
    CR_CUDA_CHECK(cudaMallocAsync(&raw, (size_t)planes * stride * stride * 8, ctx->stream));
    const size_t plane_bytes = (size_t)conv * conv * 8;
    int batch = (int)std::max<int64_t>(1, std::min<int64_t>(planes, (int64_t)(2ull << 30) / (int64_t)plane_bytes));
    float2* buf = nullptr;
    CR_CUDA_CHECK(cudaMallocAsync(&buf, plane_bytes * batch, ctx->stream));
    cufftHandle plan;
    {
        int n[2] = {(int)conv, (int)conv};
        check_cufft(cufftPlanMany(&plan, 2, n, nullptr, 1, 0, nullptr, 1, 0, CUFFT_C2C, batch),
                    "cufftPlanMany");
        check_cufft(cufftSetStream(plan, ctx->stream), "cufftSetStream");
    }
    const int64_t axis_len = law ? 0 : std::max<int64_t>(quarter, 1);
    std::vector<double> axes_h;
    double* axes_d = nullptr;
    if (!law) {
        axes_d = (double*)workspace(ctx, "wk_axes", (size_t)batch * 2 * axis_len * 8);
        axes_h.resize((size_t)batch * 2 * axis_len);
    }
    double peak = 0.0;
    for (int32_t p0 = 0; p0 < planes; p0 += batch) {
        int nb = std::min<int32_t>(batch, planes - p0);
        CR_CUDA_CHECK(cudaMemsetAsync(buf, 0, plane_bytes * nb, ctx->stream));
        screen_kernel<<<grid_blocks(inner * inner * nb, 256, (int64_t)ctx->sms * 64), 256, 0, ctx->stream>>>(
            buf, conv, inner, nb, p0, planes, w_scale, s0, s1, corr_d);
        note_launch(ctx, "screen_kernel");
        // cufftExecC2C on a plan of `batch` transforms; a short final batch
        // transforms zero-filled spare planes, which are ignored
        if (nb < batch)
            CR_CUDA_CHECK(cudaMemsetAsync((char*)buf + plane_bytes * nb, 0,
                                          plane_bytes * (batch - nb), ctx->stream));
        check_cufft(cufftExecC2C(plan, (cufftComplex*)buf, (cufftComplex*)buf, CUFFT_FORWARD),
                    "cufftExecC2C");
        if (p0 == 0) {
            float2 t00;
            CR_CUDA_CHECK(cudaMemcpyAsync(&t00, buf, 8, cudaMemcpyDeviceToHost, ctx->stream));
            CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
            peak = std::hypot((double)t00.x, (double)t00.y);
            if (!(peak > 0.0)) fail(CR_NORMALIZATION, "wproject plane-zero kernel peak is zero");
        }
        if (!law) {
            axis_kernel<<<grid_blocks(nb * axis_len, 256), 256, 0, ctx->stream>>>(buf, conv, nb,
                                                                                axis_len, axes_d);
            note_launch(ctx, "axis_kernel");
            CR_CUDA_CHECK(cudaMemcpyAsync(axes_h.data(), axes_d, (size_t)nb * 2 * axis_len * 8,
                                          cudaMemcpyDeviceToHost, ctx->stream));
            CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
            for (int b = 0; b < nb; ++b) {
                // find_w_project_support_from_transformed (gridder.rs:3832-3855)
                const double* ax = &axes_h[(size_t)(2 * b) * axis_len];
                const double* ay = &axes_h[(size_t)(2 * b + 1) * axis_len];
                int64_t trial = 0;
                bool found = false;
                for (int64_t c = quarter - 1; c >= 1; --c) {
                    if (ax[c] / peak > 1.0e-3 || ay[c] / peak > 1.0e-3) {
                        trial = c;
                        found = true;
                        break;
                    }
                }
                int64_t ms = std::max<int64_t>(quarter / sampling - 1, 1);
                int64_t s = found ? std::min<int64_t>(
                                        (int64_t)std::floor((float)trial / (float)sampling + 0.5f) + 1, ms)
                                  : ms;
                support[p0 + b] = (int32_t)s;
                int64_t cw = std::min<int64_t>(s * sampling + radius + 1, quarter);
                crop[p0 + b] = (int32_t)std::max<int64_t>(cw, 1);
            }
            CR_CUDA_CHECK(cudaMemcpyAsync(crop_d + p0, crop.data() + p0, (size_t)nb * 4,
                                          cudaMemcpyHostToDevice, ctx->stream));
        }
        crop_kernel<<<grid_blocks((int64_t)nb * stride * stride, 256), 256, 0, ctx->stream>>>(
            buf, conv, nb, p0, crop_d, stride, raw);
        note_launch(ctx, "crop_kernel");
    }
    cufftDestroy(plan);
    CR_CUDA_CHECK(cudaFreeAsync(buf, ctx->stream));

    const int32_t width = *std::max_element(crop.begin(), crop.end());
    // compact to the common width
    float2* kernels = nullptr;
    CR_CUDA_CHECK(cudaMalloc(&kernels, (size_t)planes * width * width * 8));
    // rows of a plane are `stride` apart in raw and `width` apart in kernels
    for (int32_t p = 0; p < planes; ++p)
        CR_CUDA_CHECK(cudaMemcpy2DAsync(kernels + (size_t)p * width * width, (size_t)width * 8,
                                        raw + (size_t)p * stride * stride, (size_t)stride * 8,
                                        (size_t)width * 8, (size_t)width, cudaMemcpyDeviceToDevice,
                                        ctx->stream));
    CR_CUDA_CHECK(cudaFreeAsync(raw, ctx->stream));

    wp->radius = radius;
    wp->axis = axis;
    wp->support_h = support;
    CR_CUDA_CHECK(cudaMalloc(&wp->support_d, (size_t)planes * 4));
    CR_CUDA_CHECK(cudaMemcpyAsync(wp->support_d, support.data(), (size_t)planes * 4,
                                  cudaMemcpyHostToDevice, ctx->stream));
    // plane-zero integral over the integer taps: K = T / sum Re T0(|i s|, |j s|)
    double* pb_d = (double*)workspace(ctx, "wk_pb", (size_t)axis * axis * 8);
    {
        dim3 grid_pb(axis * axis, 1);
        tap_sum_kernel<<<grid_pb, 256, 0, ctx->stream>>>(kernels, width, wp->support_d, sampling,
                                                          radius, axis, 0, pb_d, nullptr);
        note_launch(ctx, "tap_sum_kernel");
    }
    double pb_raw = 0.0;
    {
        int centre = radius * axis + radius;  // offset (0, 0)
        CR_CUDA_CHECK(cudaMemcpyAsync(&pb_raw, pb_d + centre, 8, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    }
    if (!(std::isfinite(pb_raw) && pb_raw / peak > 0.0))
        fail(CR_NORMALIZATION, "wproject plane-zero kernel integral is non-positive");
    scale_kernels<<<grid_blocks((int64_t)planes * width * width, 256), 256, 0, ctx->stream>>>(
        kernels, (int64_t)planes * width * width, (float)(1.0 / pb_raw));
    note_launch(ctx, "scale_kernels");
    wp->kernels_d = kernels;
    CR_CUDA_CHECK(cudaMalloc(&wp->norm_d, (size_t)planes * axis * axis * 4));
    {
        dim3 grid_n(axis * axis, planes);
        tap_sum_kernel<<<grid_n, 256, 0, ctx->stream>>>(kernels, width, wp->support_d, sampling,
                                                         radius, axis, 0, nullptr, wp->norm_d);
        note_launch(ctx, "tap_sum_kernel");
    }
    // residue cubes, one per plane: Q = (S s + radius) / s + 1 residue rows
    wp->cube_off_h.resize(planes);
    wp->cube_q_h.resize(planes);
    int64_t total = 0;
    for (int32_t p = 0; p < planes; ++p) {
        int32_t q = (support[p] * sampling + radius) / sampling + 1;
        wp->cube_q_h[p] = q;
        wp->cube_off_h[p] = total;
        total += (int64_t)sampling * sampling * q * q;
    }
    if ((int64_t)(support.back() + 1) * sampling * sampling * 4 >= (1ll << 26))
        fail(CR_INVALID, "W-projection support too large for the kernel cube addressing");
    if (total >= (1ll << 31)) fail(CR_INVALID, "W-projection kernel cube above 2^31 elements");
    CR_CUDA_CHECK(cudaMalloc(&wp->cube_d, (size_t)total * 8));
    CR_CUDA_CHECK(cudaMalloc(&wp->cube_off_d, (size_t)planes * 8));
    CR_CUDA_CHECK(cudaMalloc(&wp->cube_q_d, (size_t)planes * 4));
    CR_CUDA_CHECK(cudaMemcpyAsync(wp->cube_off_d, wp->cube_off_h.data(), (size_t)planes * 8,
                                  cudaMemcpyHostToDevice, ctx->stream));
    CR_CUDA_CHECK(cudaMemcpyAsync(wp->cube_q_d, wp->cube_q_h.data(), (size_t)planes * 4,
                                  cudaMemcpyHostToDevice, ctx->stream));
    for (int32_t p = 0; p < planes; ++p) {
        int64_t n = (int64_t)sampling * sampling * wp->cube_q_h[p] * wp->cube_q_h[p];
        cube_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(
            kernels, width, p, sampling, wp->cube_q_h[p], wp->cube_d + wp->cube_off_h[p]);
        note_launch(ctx, "cube_kernel");
    }
    // sinc axes for the image correction and the model apodisation
    {
        int64_t m = std::max(gnx, gny);
        std::vector<float> s = sinc_axis(m, sampling);
        std::vector<float> sx = sinc_axis(gnx, sampling), sy = sinc_axis(gny, sampling);
        CR_CUDA_CHECK(cudaMalloc(&wp->sinc_x_d, (size_t)m * 4));
        CR_CUDA_CHECK(cudaMalloc(&wp->sinc_gx_d, (size_t)gnx * 4));
        CR_CUDA_CHECK(cudaMalloc(&wp->sinc_gy_d, (size_t)gny * 4));
        CR_CUDA_CHECK(cudaMemcpy(wp->sinc_x_d, s.data(), (size_t)m * 4, cudaMemcpyHostToDevice));
        CR_CUDA_CHECK(cudaMemcpy(wp->sinc_gx_d, sx.data(), (size_t)gnx * 4, cudaMemcpyHostToDevice));
        CR_CUDA_CHECK(cudaMemcpy(wp->sinc_gy_d, sy.data(), (size_t)gny * 4, cudaMemcpyHostToDevice));
    }
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    wp->info.planes = planes;
    wp->info.sampling = sampling;
    wp->info.w_scale = w_scale;
    wp->info.max_support = *std::max_element(support.begin(), support.end());
    // first plane whose support reaches S, for S = 0 .. max support (the
    // gridder trims candidates that cannot reach a tile when supports grow
    // with the plane index)
    {
        wp->support_monotone = std::is_sorted(support.begin(), support.end());
        const int32_t ms = wp->info.max_support;
        std::vector<int32_t> fp((size_t)ms + 1, planes);
        for (int32_t S = 0; S <= ms; ++S)
            for (int32_t p = 0; p < planes; ++p)
                if (support[p] >= S) {
                    fp[S] = p;
                    break;
                }
        CR_CUDA_CHECK(cudaMalloc(&wp->first_plane_d, fp.size() * 4));
        CR_CUDA_CHECK(cudaMemcpy(wp->first_plane_d, fp.data(), fp.size() * 4,
                                 cudaMemcpyHostToDevice));
    }
    wp->info.kernel_width = width;
    wp->info.cube_elements = total;
}

// ---- gridding / degridding drivers ------------------------------------------------------
static void wproj_grid_band(cr_ctx* ctx, cr_wproj* wp, const Records& r, float2* psf,
                            float2* dirty, int mode) {
    const int64_t ntiles = r.ntx * r.nty;
    const int R = (31 + wp->info.max_support) / kTile;
    if (R > kMaxSegRadius) fail(CR_INVALID, "W-projection support above 127 is not supported");
    const int64_t gnx = wp->g->info.grid_nx;
    uint32_t* seg_lo = (uint32_t*)workspace(ctx, "wb_seg_lo", (size_t)ntiles * kNbr * 4);
    uint32_t* seg_pre = (uint32_t*)workspace(ctx, "wb_seg_pre", (size_t)ntiles * (kNbr + 1) * 4);
    uint8_t* nseg = (uint8_t*)workspace(ctx, "wb_nseg", (size_t)ntiles);
    uint32_t* nitems = (uint32_t*)workspace(ctx, "wb_nitems", (size_t)ntiles * 4);
    uint32_t* first = (uint32_t*)workspace(ctx, "wb_first", (size_t)ntiles * 4);
    unsigned long long* total = (unsigned long long*)workspace(ctx, "wb_total", 16);
    band_work_count<<<grid_blocks(ntiles, 256), 256, 0, ctx->stream>>>(
        r.tile_start, r.rec_a, wp->first_plane_d, wp->info.max_support,
        wp->support_monotone ? 1 : 0, r.ntx, r.nty, R, gnx, seg_lo, seg_pre, nseg, nitems);
    note_launch(ctx, "band_work_count");
    exclusive_scan_u32(ctx, nitems, first, ntiles, total);
    // every record is a candidate of at most (2R+1)^2 tiles; each tile has
    // at most kBands items per started chunk
    const size_t max_items = (size_t)kBands * ((size_t)ntiles +
                             (size_t)((2 * R + 1) * (2 * R + 1)) *
                                 (size_t)(r.n_samples / kBandChunk + 1));
    uint2* items = (uint2*)workspace(ctx, "wb_items", max_items * 8);
    band_work_fill<<<grid_blocks(ntiles, 256), 256, 0, ctx->stream>>>(nitems, first, r.ntx,
                                                                       r.nty, gnx, items);
    note_launch(ctx, "band_work_fill");
    unsigned int* counter = (unsigned int*)(total + 1);
    CR_CUDA_CHECK(cudaMemsetAsync(counter, 0, 4, ctx->stream));
    const size_t nrec = (size_t)std::max<int64_t>(r.n_samples, 1);
    uint4* packed = (uint4*)workspace(ctx, "wb_packed", nrec * 16);
    float* weight = (float*)workspace(ctx, "wb_weight", nrec * 4);
    if (mode == 0)
        band_pack_kernel<false><<<grid_blocks(r.n_samples, 256), 256, 0, ctx->stream>>>(
            r.rec_x, r.rec_y, r.rec_a, r.rec_b, r.rec_conj, r.rec_vsum, r.rec_wsum, r.rec_pred,
            wp->support_d, wp->axis, r.counts, packed, weight);
    else
        band_pack_kernel<true><<<grid_blocks(r.n_samples, 256), 256, 0, ctx->stream>>>(
            r.rec_x, r.rec_y, r.rec_a, r.rec_b, r.rec_conj, r.rec_vsum, r.rec_wsum, r.rec_pred,
            wp->support_d, wp->axis, r.counts, packed, weight);
    note_launch(ctx, "band_pack_kernel");
    BandArgs a{packed, weight, wp->cube_off_d, wp->cube_q_d, wp->cube_d, cube_geom(wp),
               wp->radius, r.nty, seg_lo, seg_pre, nseg, items, total, counter, psf, dirty, gnx,
               wp->g->info.grid_ny};
    auto kern = mode == 0 ? wp_grid_kernel<false> : wp_grid_kernel<true>;
    CR_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
    int per_sm = 0;
    CR_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBandWarps * 32, 0));
    const int blocks = sm_count(ctx) * std::max(per_sm, 1);
    kernel_mark(ctx, 0, false);
    kern<<<blocks, kBandWarps * 32, 0, ctx->stream>>>(a);
    note_launch(ctx, mode == 0 ? "wp_grid_kernel" : "wp_grid_kernel_residual");
    kernel_mark(ctx, 0, true);
}

void wproj_grid(cr_ctx* ctx, cr_wproj* wp, const Records& r, float2* psf, float2* dirty,
                int mode) {
    if (!band_pack_fits(std::max(wp->g->info.grid_nx, wp->g->info.grid_ny), wp->info.planes,
                        wp->radius, wp->info.max_support))
        fail(CR_INVALID, "W-projection gridding needs grid sides of at most 65536 cells, at "
                         "most 4096 planes, oversampling below 63 and supports up to 127");
    wproj_grid_band(ctx, wp, r, psf, dirty, mode);
}

void wproj_degrid(cr_ctx* ctx, cr_wproj* wp, const Records& r, const float2* grid) {
    DegridArgs a{r.rec_x, r.rec_y, r.rec_a, r.rec_b, r.rec_conj, r.counts, wp->support_d,
                 wp->cube_off_d, wp->cube_q_d, wp->cube_d, cube_geom(wp), wp->radius, wp->axis,
                 grid, wp->g->info.grid_ny, r.rec_pred};
    int blocks = sm_count(ctx) * 8;
    kernel_mark(ctx, 1, false);
    wp_degrid_kernel<<<blocks, 256, 0, ctx->stream>>>(a);
    note_launch(ctx, "wp_degrid_kernel");
    kernel_mark(ctx, 1, true);
}

void broadcast_pred(cr_ctx* ctx, const Records& r, float2* pred) {
    if (r.n_samples <= 0) return;
    broadcast_kernel<<<grid_blocks(r.n_samples, 256), 256, 0, ctx->stream>>>(
        r.sample_rec, r.rec_pred, r.n_samples, pred);
    note_launch(ctx, "broadcast_kernel");
}

}  // namespace cr
