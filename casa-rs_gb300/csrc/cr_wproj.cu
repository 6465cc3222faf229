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
// Gridding is output-stationary: a block owns a 32 x 32 tile of the grid in
// registers (each of 8 warps owns a band of 4 rows, each lane one column),
// streams the
// deduplicated records whose windows can reach the tile, and adds
// value * kernel for every owned cell inside a record's window.  The tile is
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

constexpr int kGridThreads = 256;
constexpr int kRowsPerWarp = kTile / (kGridThreads / 32);  // 4
constexpr int kMaxSegRadius = 4;
constexpr int kMaxSeg = (2 * kMaxSegRadius + 1) * (2 * kMaxSegRadius + 1);
constexpr int kChunk = 512;  // candidate records per work item

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

// ---- gridding ----------------------------------------------------------------------
struct GridArgs {
    const int32_t *rx, *ry, *rplane, *roff, *rconj;
    const double2* vsum;
    const double* wsum;
    const float2* pred;
    const uint32_t* tile_start;
    int64_t ntx, nty;
    const int32_t* support;
    const int64_t* cube_off;
    const int32_t* cube_q;
    const float2* cube;
    CubeGeom cg;
    int32_t radius, axis;
    int32_t seg_radius;
    const uint32_t* item_tile;
    const uint32_t* item_begin;
    const unsigned long long* n_items;
    unsigned int* item_counter;
    float2* psf;
    float2* dirty;
    int64_t gnx, gny;
};

struct __align__(16) Entry {
    int64_t base;    // element offset of the record's plane cube
    int32_t cb;      // window column of tile column 0
    int32_t ra;      // window row of tile row 0
    int32_t w;       // window width 2S+1
    int32_t s;       // support S
    int32_t ox, oy;  // oversampling offsets
    int32_t q;       // cube extent Q of the plane
    int32_t pad;
    float vr, vi, tvi, tvr, pw, tpw, pad2, pad3;
};

constexpr int kCand = 128;  // candidate records examined per batch

template <bool RESIDUAL>
__global__ void __launch_bounds__(kGridThreads, 6) wp_grid_kernel(GridArgs a) {
    __shared__ int s_item;
    __shared__ uint32_t s_seg_start[kMaxSeg];
    __shared__ uint32_t s_seg_pref[kMaxSeg + 1];
    __shared__ int s_nseg;
    __shared__ Entry s_list[kCand];
    // x-side cube address of each tile row per entry, -1 outside the window
    __shared__ int s_rowa[kCand][kTile + 1];
    __shared__ int s_nlist;
    __shared__ int s_warp_cnt[kCand / 32];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned long long n_items = *a.n_items;
    const int R = a.seg_radius;

    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(a.item_counter, 1u);
        __syncthreads();
        const int item = s_item;
        if ((unsigned long long)item >= n_items) break;
        const uint32_t T = a.item_tile[item];
        const uint32_t begin = a.item_begin[item];
        const int64_t tx = T / a.nty, ty = T % a.nty;
        const int x0 = (int)(tx * kTile), y0 = (int)(ty * kTile);
        if (tid == 0) {
            int ns = 0;
            uint32_t run = 0;
            for (int dx = -R; dx <= R; ++dx) {
                int64_t hx = tx + dx;
                if (hx < 0 || hx >= a.ntx) continue;
                int64_t h0 = hx * a.nty + (ty - R < 0 ? 0 : ty - R);
                int64_t h1 = hx * a.nty + (ty + R >= a.nty ? a.nty - 1 : ty + R);
                // the home tiles of one column dx are consecutive: one segment
                uint32_t st = a.tile_start[h0], en = a.tile_start[h1 + 1];
                s_seg_start[ns] = st;
                s_seg_pref[ns] = run;
                run += en - st;
                ns++;
            }
            s_seg_pref[ns] = run;
            s_nseg = ns;
        }
        __syncthreads();
        const int nseg = s_nseg;
        const uint32_t total = s_seg_pref[nseg];
        const uint32_t end = min(total, begin + (uint32_t)kChunk);

        float pr[kRowsPerWarp], pi[kRowsPerWarp], dr[kRowsPerWarp], di[kRowsPerWarp];
#pragma unroll
        for (int k = 0; k < kRowsPerWarp; ++k) pr[k] = pi[k] = dr[k] = di[k] = 0.0f;

        for (uint32_t base = begin; base < end; base += kCand) {
            // 1. candidates -> overlapping entries (the first kCand threads)
            uint32_t vidx = base + tid;
            bool take = false;
            Entry e;
            if (tid < kCand && vidx < end) {
                int k = 0;
                while (k + 1 < nseg && s_seg_pref[k + 1] <= vidx) ++k;
                uint32_t r = s_seg_start[k] + (vidx - s_seg_pref[k]);
                int lx = a.rx[r], ly = a.ry[r];
                int plane = a.rplane[r];
                int sup = a.support[plane];
                if (lx - sup <= x0 + kTile - 1 && lx + sup >= x0 && ly - sup <= y0 + kTile - 1 &&
                    ly + sup >= y0) {
                    take = true;
                    int off = a.roff[r];
                    e.ox = off / a.axis - a.radius;
                    e.oy = off % a.axis - a.radius;
                    e.s = sup;
                    e.w = 2 * sup + 1;
                    e.q = a.cube_q[plane];
                    e.base = a.cube_off[plane];
                    e.ra = x0 - lx + sup;
                    e.cb = y0 - ly + sup;
                    double2 vs = a.vsum[r];
                    double ws = a.wsum[r];
                    float vr, vi;
                    if (RESIDUAL) {
                        float2 p = a.pred[r];
                        vr = (float)(vs.x - (double)p.x * ws);
                        vi = (float)(vs.y - (double)p.y * ws);
                    } else {
                        vr = (float)vs.x;
                        vi = (float)vs.y;
                    }
                    float t = a.rconj[r] ? -1.0f : 1.0f;
                    e.vr = vr;
                    e.vi = vi;
                    e.tvi = t * vi;
                    e.tvr = t * vr;
                    e.pw = (float)ws;
                    e.tpw = t * (float)ws;
                    e.pad = 0;
                    e.pad2 = e.pad3 = 0.0f;
                }
            }
            unsigned bal = 0;
            if (tid < kCand) {  // whole warps: kCand is a multiple of 32
                bal = __ballot_sync(0xffffffffu, take);
                if (lane == 0) s_warp_cnt[warp] = __popc(bal);
            }
            __syncthreads();
            if (take) {
                int slot = 0;
                for (int w2 = 0; w2 < warp; ++w2) slot += s_warp_cnt[w2];
                slot += __popc(bal & ((1u << lane) - 1u));
                s_list[slot] = e;
            }
            if (tid == 0) {
                int t = 0;
                for (int w2 = 0; w2 < kCand / 32; ++w2) t += s_warp_cnt[w2];
                s_nlist = t;
            }
            __syncthreads();
            // x-side cube address of every (entry, tile row), all threads
            const int nlist = s_nlist;
            for (int idx = tid; idx < nlist * kTile; idx += kGridThreads) {
                const int qn = idx / kTile, rr = idx - (idx / kTile) * kTile;
                const Entry& en = s_list[qn];
                const int i = en.ra + rr;  // window row index
                s_rowa[qn][rr] = (i >= 0 && i < en.w) ? cube_a(i - en.s, en.ox, en.q, a.cg) : -1;
            }
            __syncthreads();
            // 2. accumulate the entries into the register tile; warp w owns
            // rows 4w .. 4w+3 and skips entries whose window misses them
            const int band0 = warp * kRowsPerWarp;
            for (int qn = 0; qn < nlist; ++qn) {
                const Entry& en = s_list[qn];
                if (band0 > en.w - 1 - en.ra || band0 + kRowsPerWarp - 1 < -en.ra) continue;
                const int col = en.cb + lane;
                const bool colok = (unsigned)col < (unsigned)en.w;
                const int bcol = colok ? cube_b(col - en.s, en.oy, en.q, a.cg) : 0;
                const float2* cube = a.cube + en.base + bcol;
                float2 kv[kRowsPerWarp];
                bool ok[kRowsPerWarp];
#pragma unroll
                for (int k = 0; k < kRowsPerWarp; ++k) {
                    const int av = s_rowa[qn][band0 + k];
                    ok[k] = av >= 0 && colok;
                    kv[k] = ok[k] ? __ldg(cube + av) : make_float2(0.f, 0.f);
                }
                // (paired float32 FMAs here measured 9.40 -> 9.53 ms: the
                // operand swaps and extra spills cost more than they saved)
#pragma unroll
                for (int k = 0; k < kRowsPerWarp; ++k) {
                    if (ok[k]) {
                        if (!RESIDUAL) {
                            pr[k] = fmaf(en.pw, kv[k].x, pr[k]);
                            pi[k] = fmaf(en.tpw, kv[k].y, pi[k]);
                        }
                        dr[k] = fmaf(-en.tvi, kv[k].y, fmaf(en.vr, kv[k].x, dr[k]));
                        di[k] = fmaf(en.vi, kv[k].x, fmaf(en.tvr, kv[k].y, di[k]));
                    }
                }
            }
            __syncthreads();
        }
        // 3. flush the tile
#pragma unroll
        for (int k = 0; k < kRowsPerWarp; ++k) {
            int64_t x = x0 + warp * kRowsPerWarp + k;
            int64_t y = y0 + lane;
            if (x < a.gnx && y < a.gny) {
                int64_t cell = x * a.gny + y;
                if (!RESIDUAL && (pr[k] != 0.0f || pi[k] != 0.0f))
                    atomicAdd(&a.psf[cell], make_float2(pr[k], pi[k]));
                if (dr[k] != 0.0f || di[k] != 0.0f)
                    atomicAdd(&a.dirty[cell], make_float2(dr[k], di[k]));
            }
        }
    }
}

// Work items: per output tile, the candidate records of its neighbourhood,
// cut into chunks of kChunk.
__global__ void tile_work_count(const uint32_t* tile_start, int64_t ntx, int64_t nty, int R,
                                uint32_t* nchunks) {
    int64_t ntiles = ntx * nty;
    for (int64_t T = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; T < ntiles;
         T += (int64_t)gridDim.x * blockDim.x) {
        int64_t tx = T / nty, ty = T % nty;
        uint64_t total = 0;
        for (int dx = -R; dx <= R; ++dx) {
            int64_t hx = tx + dx;
            if (hx < 0 || hx >= ntx) continue;
            int64_t h0 = hx * nty + (ty - R < 0 ? 0 : ty - R);
            int64_t h1 = hx * nty + (ty + R >= nty ? nty - 1 : ty + R);
            total += tile_start[h1 + 1] - tile_start[h0];
        }
        nchunks[T] = (uint32_t)((total + kChunk - 1) / kChunk);
    }
}

__global__ void tile_work_fill(const uint32_t* nchunks, const uint32_t* first, int64_t ntiles,
                               uint32_t* item_tile, uint32_t* item_begin) {
    for (int64_t T = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; T < ntiles;
         T += (int64_t)gridDim.x * blockDim.x) {
        uint32_t c = nchunks[T], f = first[T];
        for (uint32_t k = 0; k < c; ++k) {
            item_tile[f + k] = (uint32_t)T;
            item_begin[f + k] = k * kChunk;
        }
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
    wp->info.kernel_width = width;
    wp->info.cube_elements = total;
}

// ---- gridding / degridding drivers ------------------------------------------------------
void wproj_grid(cr_ctx* ctx, cr_wproj* wp, const Records& r, float2* psf, float2* dirty,
                int mode) {
    const int64_t ntiles = r.ntx * r.nty;
    int R = (31 + wp->info.max_support) / kTile;
    if (R > kMaxSegRadius) fail(CR_INVALID, "W-projection support above 127 is not supported");
    uint32_t* nchunks = (uint32_t*)workspace(ctx, "wg_nchunks", (size_t)ntiles * 4);
    uint32_t* first = (uint32_t*)workspace(ctx, "wg_first", (size_t)ntiles * 4);
    unsigned long long* nitems = (unsigned long long*)workspace(ctx, "wg_nitems", 16);
    tile_work_count<<<grid_blocks(ntiles, 256), 256, 0, ctx->stream>>>(r.tile_start, r.ntx, r.nty,
                                                                        R, nchunks);
    note_launch(ctx, "tile_work_count");
    exclusive_scan_u32(ctx, nchunks, first, ntiles, nitems);
    // upper bound on the items: every candidate list chunked
    size_t max_items = (size_t)ntiles + (size_t)((2 * R + 1) * (2 * R + 1)) *
                                            (size_t)(r.n_samples / kChunk + 1);
    uint32_t* item_tile = (uint32_t*)workspace(ctx, "wg_item_tile", max_items * 4);
    uint32_t* item_begin = (uint32_t*)workspace(ctx, "wg_item_begin", max_items * 4);
    tile_work_fill<<<grid_blocks(ntiles, 256), 256, 0, ctx->stream>>>(nchunks, first, ntiles,
                                                                       item_tile, item_begin);
    note_launch(ctx, "tile_work_fill");
    unsigned int* counter = (unsigned int*)(nitems + 1);
    CR_CUDA_CHECK(cudaMemsetAsync(counter, 0, 4, ctx->stream));
    GridArgs a{r.rec_x, r.rec_y, r.rec_a, r.rec_b, r.rec_conj, r.rec_vsum, r.rec_wsum,
               r.rec_pred, r.tile_start, r.ntx, r.nty, wp->support_d, wp->cube_off_d,
               wp->cube_q_d, wp->cube_d, cube_geom(wp), wp->radius, wp->axis, R, item_tile,
               item_begin, nitems, counter, psf, dirty, wp->g->info.grid_nx, wp->g->info.grid_ny};
    int blocks = sm_count(ctx) * 8;
    kernel_mark(ctx, 0, false);
    if (mode == 0) {
        wp_grid_kernel<false><<<blocks, kGridThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "wp_grid_kernel");
    } else {
        wp_grid_kernel<true><<<blocks, kGridThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "wp_grid_kernel_residual");
    }
    kernel_mark(ctx, 0, true);
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
