// cr_cube.cu -- the batched spectral cube: every channel weighted, planned
// and gridded (or degridded) by one sequence of launches whose number does
// not depend on the number of channels.
//
// Channel c's visibility batch is the unflagged samples of rows r = 0..R-1
// with u_lambda = u_m[r] * s_c, v_lambda = v_m[r] * s_c, s_c = f_c / c (the
// cube batch assembly of casars-imager/src/lib.rs:49571-49576, which leaves
// flagged samples out of the channel batch).  Per channel the path restates
//   * PerPlane density weighting (apply_weighting_with_density_source,
//     weighting.rs:1055-1180 with density_build_cell_convention /
//     density_cell_convention = CubeBriggsWeightor{Density,Lookup},
//     weighting.rs:1455-1483): the density is image-sized, a sample adds its
//     weight at the rounded cell of (u, v) and of (-u, -v)
//     (weight_density_cell_anchor, gridder.rs:1888-1934), f2 uses FP64 sums
//     of d and d^2 (weighting.rs:1108-1121) and the reweight is w / d or
//     w / (d f2 + 1) (casa_briggs_denominator, weighting.rs:2440-2443);
//   * the standard PSWF plan (sample_tap_span, gridder.rs:1976-1995) and
//     gridding (grid_sample_taps_real_complex_pair_planned_f64,
//     gridder.rs:1021-1071) with sumwt = sum of f64 weights (lib.rs:68433-68500);
//   * degridding (degrid_sample_taps_planned_normalized, gridder.rs:1278-1312).
//
// Layout: rows' u, v (f64 metres) are shared by all channels; vis, weight
// and flags are channel-major [C][R].  Planning makes one pass that builds
// the weight density and histograms the samples by (channel, 32 x 32 home
// tile, start cell), a scan, and a second pass that forms each imaging weight
// and scatters 16-byte records {cell | tap rows, sample, w vis} plus the
// weight into bin order.  The index selection runs on the integer fixed-point path of
// cr_fixed.cuh with the FP64 operations as the fallback.  Gridding gives
// every (channel, output tile) to one block, which gathers the records of
// the four home tiles whose 7 x 7 footprints reach it, accumulates the tile
// in shared memory and writes it once with coalesced stores -- no memset and
// no global atomics on the output grids.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cr_fixed.cuh"
#include "cr_internal.cuh"
#include "cr_tma.cuh"

namespace cr {

namespace {

constexpr int kCubeThreads = 256;
constexpr int kRowsPerBlock = 4096;   // rows of one channel per planning block
// Shared-memory tile rows are 39 floats apart (39 = 7 mod 32): the 49 taps
// t = 7 ix + iy of one record then fall in 49 consecutive banks mod 32, so
// each warp-wide atomic touches 32 distinct banks.
constexpr int kRow = 39;
constexpr int kMaxTapRows = 513;      // oversampling up to 512
// the tap table in floats, rounded up to whole 16-byte bulk-copy units
constexpr int kTapFloats = (kMaxTapRows * 7 + 3) / 4 * 4;

struct CubeChan {
    double lscale;       // f / c
    FixScale kx, ky;     // lscale / du, lscale / dv
    FixScale kdx, kdy;   // lscale * nx cell_x, lscale * ny cell_y
    DfScale fx, fy, fdx, fdy;   // the same four as float32 pairs
};

struct CubeArgs {
    int64_t R;
    int32_t C;
    const double* u;
    const double* v;
    const float4* uvdf;        // per row (u_hi, u_lo, v_hi, v_lo); NaN u_hi: exact path only
    const CubeChan* ch;
    const float2* vis;
    const float* weight;
    const uint8_t* flags;
    // gridder
    double du, dv;
    int64_t gnx, gny;
    int32_t os, tap_rows;
    int64_t ntx, nty;
    long long cx_fix, cy_fix;
    // density
    int32_t nx, ny;
    double dus, dvs, dcx, dcy;
    long long dcx_fix, dcy_fix;
    int32_t mode;
    float* density;            // [C][nx][ny]
    const float* f2;           // [C]
    // planning
    uint32_t* hist;            // [C * ntiles]
    uint32_t* cursor;          // [C * ntiles]
    double* sumwt;             // [C]
    unsigned long long* counts;// [C][2]: gridded, skipped
    uint4* rec;                // {meta, c R + r, w vis.re, w vis.im}
    float* rec_w;
    // per-sample results kept between the passes ([C][R])
    uint32_t* dcell;           // density cell x ny + y of (u, v), ~0 when none
    uint32_t* ev_tile;         // home tile, or kFlaggedSample / kUngriddedSample
    uint32_t* ev_meta;         // cell in tile | tap rows
};

// Rows' u, v as float32 pairs for the fast path.  Rows whose coordinates are
// not finite, exceed 2^60 or are below 2^-60 (but not zero) get a NaN u_hi
// and always take the integer path.
__global__ void cube_rows_df_kernel(const double* u, const double* v, int64_t R, float4* out) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < R;
         r += (int64_t)gridDim.x * blockDim.x) {
        const double um = u[r], vm = v[r];
        const bool ok = isfinite(um) && isfinite(vm) && fabs(um) < 0x1p60 &&
                        fabs(vm) < 0x1p60 && (um == 0.0 || fabs(um) > 0x1p-60) &&
                        (vm == 0.0 || fabs(vm) > 0x1p-60);
        const float uh = __double2float_rn(um), vh = __double2float_rn(vm);
        const float ul = __double2float_rn(__dsub_rn(um, (double)uh));
        const float vl = __double2float_rn(__dsub_rn(vm, (double)vh));
        out[r] = ok ? make_float4(uh, ul, vh, vl) : make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
    }
}

// The density cell (x, y) of x = s_x p_x + e_x + nx/2 (valid when 1 <= x <
// nx, likewise y) on the float32-pair path; false when undecided.
__device__ __forceinline__ bool df_density_cell(float px, float ex, float py, float ey,
                                                int32_t nx, int32_t ny, int* x, int* y,
                                                bool* ok) {
    float ax, ay, dh;
    if (!df_nearest(px, ex, (nx & 1) ? 0.5f : 0.0f, &ax, &dh) ||
        !df_nearest(py, ey, (ny & 1) ? 0.5f : 0.0f, &ay, &dh))
        return false;
    const int cx = (nx >> 1) + (int)ax, cy = (ny >> 1) + (int)ay;
    *ok = !(cx <= 0 || cy <= 0 || cx >= nx || cy >= ny);
    *x = cx;
    *y = cy;
    return true;
}

// Both density cells of a sample, of (u, v) and of the mirror (-u, -v),
// from one pair of fixed-point products (FP64 fallback per cell).
__device__ __forceinline__ void density_cells(const CubeArgs& a, const CubeChan& ch, double um,
                                              double vm, int* x, int* y, bool* ok, int* xm,
                                              int* ym, bool* okm);

// weight_density_cell_anchor with the cube (rounded) conventions.
__device__ __forceinline__ bool density_cell(const CubeArgs& a, const CubeChan& ch, double um,
                                             double vm, bool mirror, int* ox, int* oy) {
    long long tx, ty;
    if (fix_mul(um, ch.kdx, &tx) && fix_mul(vm, ch.kdy, &ty)) {
        const long long X = (mirror ? -tx : tx) + a.dcx_fix;
        const long long Y = (mirror ? ty : -ty) + a.dcy_fix;
        long long ax, ay;
        if (fix_round(X, kFixMargin, &ax) && fix_round(Y, kFixMargin, &ay)) {
            if (ax <= 0 || ay <= 0 || ax >= a.nx || ay >= a.ny) return false;
            *ox = (int)ax;
            *oy = (int)ay;
            return true;
        }
    }
    double u = __dmul_rn(um, ch.lscale), v = __dmul_rn(vm, ch.lscale);
    if (mirror) {
        u = -u;
        v = -v;
    }
    const double x = __dadd_rn(__dmul_rn(u, a.dus), a.dcx);
    const double y = __dadd_rn(__dmul_rn(-v, a.dvs), a.dcy);
    if (!isfinite(x) || !isfinite(y)) return false;
    const double rx = round(x), ry = round(y);
    if (!(rx >= 1.0 && ry >= 1.0 && rx < (double)a.nx && ry < (double)a.ny)) return false;
    *ox = (int)rx;
    *oy = (int)ry;
    return true;
}

__device__ __forceinline__ void density_cells(const CubeArgs& a, const CubeChan& ch, double um,
                                              double vm, int* x, int* y, bool* ok, int* xm,
                                              int* ym, bool* okm) {
    long long tx, ty;
    if (fix_mul(um, ch.kdx, &tx) && fix_mul(vm, ch.kdy, &ty)) {
        long long ax, ay;
        // (u, v): x = u s + c, y = -v s + c; mirror: x = -u s + c, y = v s + c
        if (fix_round(tx + a.dcx_fix, kFixMargin, &ax) &&
            fix_round(a.dcy_fix - ty, kFixMargin, &ay)) {
            *ok = !(ax <= 0 || ay <= 0 || ax >= a.nx || ay >= a.ny);
            *x = (int)ax;
            *y = (int)ay;
        } else {
            *ok = density_cell(a, ch, um, vm, false, x, y);
        }
        if (fix_round(a.dcx_fix - tx, kFixMargin, &ax) &&
            fix_round(a.dcy_fix + ty, kFixMargin, &ay)) {
            *okm = !(ax <= 0 || ay <= 0 || ax >= a.nx || ay >= a.ny);
            *xm = (int)ax;
            *ym = (int)ay;
        } else {
            *okm = density_cell(a, ch, um, vm, true, xm, ym);
        }
        return;
    }
    *ok = density_cell(a, ch, um, vm, false, x, y);
    *okm = density_cell(a, ch, um, vm, true, xm, ym);
}

__device__ __forceinline__ bool finite_f(float x) { return isfinite(x); }

struct Eval {
    bool ok;
    uint32_t tile;
    uint32_t meta;
    float w;
};

// sample_tap_span of row r at channel ch: the home tile and meta = start cell
// in the tile | tap rows; float32 pairs first, then the integer path, then
// the reference's FP64 operations.  False when the sample does not grid.
__device__ __forceinline__ bool plan_sample(const CubeArgs& a, const CubeChan& ch, float4 uv,
                                            int64_t r, uint32_t* tile, uint32_t* meta) {
    int64_t x0 = 0, y0 = 0;
    int32_t rx = 0, ry = 0;
    // x = u K_x + G/2, y = -v K_y + G/2
    float px, ex, py, ey;
    df_product(uv.x, uv.y, ch.fx, &px, &ex);
    df_product(-uv.z, -uv.w, ch.fy, &py, &ey);
    int sx = df_tap_span(px, ex, a.gnx, a.os, a.tap_rows, &x0, &rx);
    int sy = sx == 0 ? 0 : df_tap_span(py, ey, a.gny, a.os, a.tap_rows, &y0, &ry);
    if (sx == 0 || sy == 0) return false;
    long long tx, ty;
    if ((sx < 0 || sy < 0) && fix_mul(a.u[r], ch.kx, &tx) && fix_mul(a.v[r], ch.ky, &ty)) {
        sx = fix_tap_span(tx + a.cx_fix, a.gnx, a.os, a.tap_rows, &x0, &rx);
        if (sx != 0) sy = fix_tap_span(a.cy_fix - ty, a.gny, a.os, a.tap_rows, &y0, &ry);
        if (sx == 0 || sy == 0) return false;
    }
    if (sx < 0 || sy < 0) {
        const double u = __dmul_rn(a.u[r], ch.lscale), v = __dmul_rn(a.v[r], ch.lscale);
        const double x = __dadd_rn(__ddiv_rn(u, a.du), (double)a.gnx / 2.0);
        const double y = __dadd_rn(__ddiv_rn(-v, a.dv), (double)a.gny / 2.0);
        if (!f64_tap_span(x, a.gnx, a.os, a.tap_rows, &x0, &rx) ||
            !f64_tap_span(y, a.gny, a.os, a.tap_rows, &y0, &ry))
            return false;
    }
    *tile = (uint32_t)((x0 >> 5) * a.nty + (y0 >> 5));
    *meta = ((uint32_t)(x0 & 31) << 27) | ((uint32_t)(y0 & 31) << 22) | ((uint32_t)rx << 11) |
            (uint32_t)ry;
    return true;
}

// ev_tile values of samples without a home tile
constexpr uint32_t kFlaggedSample = ~0u;        // flagged: left out of the channel batch
constexpr uint32_t kUngriddedSample = ~0u - 1;  // unflagged, but no grid plan or weight

// Samples are evaluated kVec at a time per thread (rows row0 + 32 j): their
// loads are issued together, so each thread keeps kVec gathers in flight.
constexpr int kVec = 4;
constexpr int kWarpRows = 32 * kVec;

// kVec samples of channel c: flags, reweighting, validity and taps.
__device__ __forceinline__ void eval_samples(const CubeArgs& a, const CubeChan& ch, float f2,
                                             int c, int64_t row0, int64_t r1,
                                             Eval (&e)[kVec]) {
    float w[kVec];
    float4 uv[kVec];
    bool live[kVec];
#pragma unroll
    for (int j = 0; j < kVec; ++j) {
        const int64_t r = row0 + 32 * j;
        e[j] = Eval{false, 0u, 0u, 0.0f};
        live[j] = r < r1;
        const int64_t i = (int64_t)c * a.R + (live[j] ? r : 0);
        if (live[j] && a.flags) live[j] = a.flags[i] == 0;
        w[j] = a.weight ? a.weight[i] : 1.0f;
        uv[j] = a.uvdf[live[j] ? r : 0];
    }
    if (a.mode != CR_WEIGHT_NATURAL) {
        float d[kVec];
        const float* dens = a.density + (int64_t)c * a.nx * a.ny;
        if (a.dcell) {
            uint32_t cell[kVec];
#pragma unroll
            for (int j = 0; j < kVec; ++j)
                cell[j] = live[j] ? a.dcell[(int64_t)c * a.R + row0 + 32 * j] : ~0u;
#pragma unroll
            for (int j = 0; j < kVec; ++j) d[j] = cell[j] != ~0u ? dens[cell[j]] : 0.0f;
        } else {
#pragma unroll
            for (int j = 0; j < kVec; ++j) {
                int x, y;
                d[j] = 0.0f;
                const int64_t r = row0 + 32 * j;
                if (live[j] && density_cell(a, ch, a.u[r], a.v[r], false, &x, &y))
                    d[j] = dens[(int64_t)x * a.ny + y];
            }
        }
#pragma unroll
        for (int j = 0; j < kVec; ++j) {
            float nw = 0.0f;
            if (finite_f(w[j]) && w[j] > 0.0f && finite_f(d[j]) && d[j] > 0.0f)
                nw = a.mode == CR_WEIGHT_UNIFORM
                         ? __fdiv_rn(w[j], d[j])
                         : __fdiv_rn(w[j], __fadd_rn(__fmul_rn(d[j], f2), 1.0f));
            w[j] = nw;
        }
    }
#pragma unroll
    for (int j = 0; j < kVec; ++j) {
        if (!live[j] || !(finite_f(w[j]) && w[j] > 0.0f)) continue;
        if (!plan_sample(a, ch, uv[j], row0 + 32 * j, &e[j].tile, &e[j].meta)) continue;
        e[j].ok = true;
        e[j].w = w[j];
    }
}

// Records are binned by (channel, home tile, start cell in the tile), so that
// within a home tile they follow the cell order and records with one start
// cell are adjacent.
__device__ __forceinline__ int64_t cell_bin(int c, int64_t ntiles, uint32_t tile,
                                            uint32_t meta) {
    return (((int64_t)c * ntiles + tile) << 10) | (int64_t)(meta >> 22);
}

// Pass 1 over every sample: with DENSITY the weight density of both cells
// (u, v) and (-u, -v) and the sample's own density cell; then its grid plan
// and the histogram of (channel, home tile, cell) over the samples that can
// grid -- unflagged, a positive natural weight, an own density cell
// (DENSITY) and a plan.  This counts a superset of the gridded samples: the
// imaging weight w / d or w / (d f2 + 1), known only once every density is
// complete, must also come out positive; the scatter gives a sample for
// which it does not a null record, so the counts stay exact.
template <bool DENSITY>
__global__ void __launch_bounds__(kCubeThreads, 4) cube_density_kernel(CubeArgs a) {
    const int c = blockIdx.y;
    const CubeChan ch = a.ch[c];
    const int64_t ntiles = a.ntx * a.nty;
    const int64_t r0 = (int64_t)blockIdx.x * kRowsPerBlock;
    const int64_t r1 = min(a.R, r0 + kRowsPerBlock);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* dens = DENSITY ? a.density + (int64_t)c * a.nx * a.ny : nullptr;
    for (int64_t base = r0 + warp * kWarpRows; base < r1; base += kCubeThreads * kVec) {
        float w[kVec];
        float4 uv[kVec];
        bool live[kVec];
#pragma unroll
        for (int j = 0; j < kVec; ++j) {
            const int64_t r = base + lane + 32 * j;
            live[j] = r < r1;
            const int64_t i = (int64_t)c * a.R + (live[j] ? r : 0);
            if (live[j] && a.flags) live[j] = a.flags[i] == 0;
            w[j] = a.weight ? a.weight[i] : 1.0f;
            uv[j] = a.uvdf[live[j] ? r : 0];
        }
#pragma unroll
        for (int j = 0; j < kVec; ++j) {
            const int64_t r = base + lane + 32 * j;
            if (r >= r1) continue;
            const int64_t i = (int64_t)c * a.R + r;
            const bool pos = finite_f(w[j]) && w[j] > 0.0f;
            bool own = true;
            if (DENSITY) {
                uint32_t cell = ~0u;
                if (live[j]) {
                    int x = 0, y = 0, xm = 0, ym = 0;
                    bool ok = false, okm = false;
                    // float32 pairs first: (u, v) -> x = u s_x + nx/2,
                    // y = -v s_y + ny/2; the mirror negates both products
                    float px, ex, py, ey;
                    df_product(uv[j].x, uv[j].y, ch.fdx, &px, &ex);
                    df_product(-uv[j].z, -uv[j].w, ch.fdy, &py, &ey);
                    if (!df_density_cell(px, ex, py, ey, a.nx, a.ny, &x, &y, &ok) ||
                        !df_density_cell(-px, -ex, -py, -ey, a.nx, a.ny, &xm, &ym, &okm))
                        density_cells(a, ch, a.u[r], a.v[r], &x, &y, &ok, &xm, &ym, &okm);
                    if (ok) {
                        cell = (uint32_t)x * (uint32_t)a.ny + (uint32_t)y;
                        if (pos) atomicAdd(&dens[cell], w[j]);
                    }
                    if (okm && pos) atomicAdd(&dens[(int64_t)xm * a.ny + ym], w[j]);
                }
                a.dcell[i] = cell;
                own = cell != ~0u;
            }
            uint32_t tile = kUngriddedSample, meta = 0u;
            if (!live[j]) {
                tile = kFlaggedSample;
            } else if (pos && own && plan_sample(a, ch, uv[j], r, &tile, &meta)) {
                atomicAdd(&a.hist[cell_bin(c, ntiles, tile, meta)], 1u);
            } else {
                tile = kUngriddedSample;
            }
            a.ev_tile[i] = tile;
            a.ev_meta[i] = meta;
        }
    }
}

// hi + lo += x without rounding error (Knuth's two-sum; lo collects errors)
__device__ __forceinline__ void two_sum(float& hi, float& lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, err);
}

// Per channel: sum d and sum d^2 (d > 0) in FP64, then f2 (weighting.rs:1108-1121).
__global__ void __launch_bounds__(kCubeThreads) cube_density_sums(const float* density,
                                                                  int64_t cells, double* sums) {
    const int c = blockIdx.y;
    const float* d = density + (int64_t)c * cells;
    // per thread in float32 pairs (error-free sums and products: exact for
    // sums below 2^48 of integer-valued densities), FP64 only to combine
    float s_hi = 0.f, s_lo = 0.f, q_hi = 0.f, q_lo = 0.f;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cells;
         k += (int64_t)gridDim.x * blockDim.x) {
        const float v = d[k];
        two_sum(s_hi, s_lo, v);
        if (v > 0.0f) {
            const float p = __fmul_rn(v, v);
            two_sum(q_hi, q_lo, p);
            q_lo = __fadd_rn(q_lo, fmaf(v, v, -p));
        }
    }
    double s = (double)s_hi + (double)s_lo, s2 = (double)q_hi + (double)q_lo;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    __shared__ double sh[2][kCubeThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][warp] = s;
        sh[1][warp] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, t2 = 0.0;
        for (int k = 0; k < kCubeThreads / 32; ++k) {
            t += sh[0][k];
            t2 += sh[1][k];
        }
        atomicAdd(&sums[2 * c], t);
        atomicAdd(&sums[2 * c + 1], t2);
    }
}

__global__ void cube_f2_kernel(const double* sums, int32_t C, double a2, float* f2) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const double s = sums[2 * c], s2 = sums[2 * c + 1];
    f2[c] = (s2 > 0.0 && s > 0.0) ? (float)__ddiv_rn(a2, __ddiv_rn(s2, s)) : 0.0f;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Tile-level starts from the cell-level exclusive scan.
__global__ void tile_starts_from_cells(const uint32_t* cell_start, int64_t nbins,
                                       uint32_t* bin_start) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b <= nbins;
         b += (int64_t)gridDim.x * blockDim.x)
        bin_start[b] = cell_start[b << 10];
}

// Pass 2: records scattered into (channel, home tile, cell) bins from pass
// 1's plans, kScatterVec samples per thread and iteration so that more
// cursor atomics are in flight.  The imaging weight is formed here, from the
// complete density: w itself, w / d (uniform) or w / (d f2 + 1) (Briggs,
// casa_briggs_denominator, weighting.rs:2440-2443).  A counted sample whose
// weight does not come out positive and finite gets a null record (zero
// weight and value, no sample index), which grids and degrids nothing.  The
// channel's sum of weights and its gridded and unflagged-but-not-gridded
// counts are summed here.
constexpr int kScatterVec = 6;
constexpr uint32_t kNullSample = ~0u;   // sample index of a null record
__global__ void __launch_bounds__(kCubeThreads, 4) cube_scatter_kernel(CubeArgs a) {
    __shared__ double s_sum[kCubeThreads / 32];
    __shared__ unsigned long long s_ok[kCubeThreads / 32], s_skip[kCubeThreads / 32];
    const int c = blockIdx.y;
    const int64_t ntiles = a.ntx * a.nty;
    const int lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * kRowsPerBlock;
    const int64_t r1 = min(a.R, r0 + kRowsPerBlock);
    const int wp = threadIdx.x >> 5;
    const float f2 = a.mode == CR_WEIGHT_BRIGGS ? a.f2[c] : 0.0f;
    const float* dens = a.mode != CR_WEIGHT_NATURAL ? a.density + (int64_t)c * a.nx * a.ny
                                                    : nullptr;
    // the channel's sum of weights as a float pair (no FP64 instruction per
    // sample), in FP64 from the warp sums on
    PairSum swp;
    unsigned long long n_ok = 0, n_skip = 0;
    for (int64_t base = r0 + wp * 32 * kScatterVec; base < r1;
         base += kCubeThreads * kScatterVec) {
        // loads first, then every cursor atomic, then the stores: the kScatterVec
        // atomics of a thread are in flight together.  (The samples of a
        // warp -- consecutive rows of one channel, different baselines --
        // almost never share a cell bin, so the atomics are not aggregated:
        // a warp match cost more than it saved.)
        uint32_t tile[kScatterVec], meta[kScatterVec], pos[kScatterVec];
        float w[kScatterVec];
        float2 vv[kScatterVec];
#pragma unroll
        for (int j = 0; j < kScatterVec; ++j) {
            const int64_t r = base + lane + 32 * j;
            const int64_t i = (int64_t)c * a.R + (r < r1 ? r : r0);
            tile[j] = r < r1 ? a.ev_tile[i] : kFlaggedSample;
            meta[j] = a.ev_meta[i];
            w[j] = a.weight ? a.weight[i] : 1.0f;
            vv[j] = a.vis[i];
        }
        if (dens) {
            float d[kScatterVec];
#pragma unroll
            for (int j = 0; j < kScatterVec; ++j) {
                const int64_t i = (int64_t)c * a.R + base + lane + 32 * j;
                d[j] = tile[j] < kUngriddedSample ? dens[a.dcell[i]] : 0.0f;
            }
#pragma unroll
            for (int j = 0; j < kScatterVec; ++j) {
                float nw = 0.0f;
                if (finite_f(w[j]) && w[j] > 0.0f && finite_f(d[j]) && d[j] > 0.0f)
                    nw = a.mode == CR_WEIGHT_UNIFORM
                             ? __fdiv_rn(w[j], d[j])
                             : __fdiv_rn(w[j], __fadd_rn(__fmul_rn(d[j], f2), 1.0f));
                w[j] = nw;
            }
        }
#pragma unroll
        for (int j = 0; j < kScatterVec; ++j) {
            pos[j] = 0u;
            if (tile[j] < kUngriddedSample)
                pos[j] = atomicAdd(&a.cursor[cell_bin(c, ntiles, tile[j], meta[j])], 1u);
        }
#pragma unroll
        for (int j = 0; j < kScatterVec; ++j) {
            if (tile[j] == kFlaggedSample) continue;
            const bool ok = tile[j] != kUngriddedSample && finite_f(w[j]) && w[j] > 0.0f;
            if (!ok) ++n_skip;
            if (tile[j] == kUngriddedSample) continue;
            const int64_t i = (int64_t)c * a.R + base + lane + 32 * j;
            float vr = 0.0f, vi = 0.0f, wr = 0.0f;
            uint32_t sample = kNullSample;
            if (ok) {
                if (finite_f(vv[j].x) && finite_f(vv[j].y)) {
                    vr = __fmul_rn(vv[j].x, w[j]);
                    vi = __fmul_rn(vv[j].y, w[j]);
                }
                wr = w[j];
                sample = (uint32_t)i;
                ++n_ok;
                swp.add(wr, 0.0f);
            }
            a.rec[pos[j]] = make_uint4(meta[j], sample, __float_as_uint(vr),
                                       __float_as_uint(vi));
            a.rec_w[pos[j]] = wr;
        }
    }
    double sw = (double)swp.h + (double)swp.l;
    sw = warp_sum(sw);
    n_ok = warp_sum(n_ok);
    n_skip = warp_sum(n_skip);
    const int warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_sum[warp] = sw;
        s_ok[warp] = n_ok;
        s_skip[warp] = n_skip;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long o = 0, k = 0;
        for (int q = 0; q < kCubeThreads / 32; ++q) {
            t += s_sum[q];
            o += s_ok[q];
            k += s_skip[q];
        }
        if (t != 0.0) atomicAdd(&a.sumwt[c], t);
        if (o) atomicAdd(&a.counts[2 * c], o);
        if (k) atomicAdd(&a.counts[2 * c + 1], k);
    }
}

// Source records per gridding work item: chosen per cube shape by a
// first-use tuning pass over these candidates (the default before tuning).
constexpr uint32_t kGridChunkCandidates[3] = {1024, 2048, 4096};
constexpr uint32_t kGridChunkDefault = 2048;
constexpr uint32_t kGridChunkMin = 1024;
constexpr uint32_t kDegridChunk = 4096; // records per degridding work item

// Work lists.  Gridding: an output tile (channel, tx, ty) gathers the bins
// (tx, ty), (tx-1, ty), (tx, ty-1), (tx-1, ty-1); their records, taken in
// that order, are cut into chunks (of the tuned size).  A tile with one chunk is
// written with plain stores; the chunks of a heavier tile add into the grid
// with atomics after cube_work_fill zeroed it.  Degridding: each bin's
// records in chunks of kDegridChunk.
__device__ __forceinline__ uint32_t bin_count(const uint32_t* bin_start, int64_t bin) {
    return bin_start[bin + 1] - bin_start[bin];
}

// Start of cell bin cb: cell_end holds each cell bin's end (= the next
// bin's start) once the scatter has advanced the cursors.
__device__ __forceinline__ uint32_t cell_start(const uint32_t* cell_end, int64_t cb) {
    return cb == 0 ? 0u : cell_end[cb - 1];
}

// The records of output tile (c, tx, ty)'s four sources that can reach it:
// all of the home tile; of (tx-1, ty) and (tx-1, ty-1) only start cells with
// x >= 26 (a contiguous suffix, records being in cell order); all of
// (tx, ty-1) (its reaching cells, y >= 26, are not contiguous).
__device__ __forceinline__ void source_ranges(const uint32_t* bin_start,
                                              const uint32_t* cell_end, int64_t c,
                                              int64_t ntiles, int64_t nty, int64_t tx,
                                              int64_t ty, uint32_t (&lo)[4],
                                              uint32_t (&hi)[4]) {
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int64_t sx = tx - (s & 1), sy = ty - (s >> 1);
        lo[s] = hi[s] = 0u;
        if (sx < 0 || sy < 0) continue;
        const int64_t sb = c * ntiles + sx * nty + sy;
        hi[s] = bin_start[sb + 1];
        lo[s] = (s & 1) ? cell_start(cell_end, (sb << 10) + (kTile - 6) * kTile)
                        : bin_start[sb];
    }
}

// Channels whose plane_mask entry is 0 get no work items.
__global__ void cube_work_count(const uint32_t* bin_start, const uint32_t* cell_end,
                                int64_t nbins, int64_t ntiles, int64_t nty, uint32_t grid_chunk,
                                const uint8_t* plane_mask, uint32_t* grid_chunks,
                                uint32_t* degrid_chunks) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nbins;
         b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = b / ntiles, T = b % ntiles;
        if (plane_mask && !plane_mask[c]) {
            grid_chunks[b] = degrid_chunks[b] = 0u;
            continue;
        }
        uint32_t lo[4], hi[4];
        source_ranges(bin_start, cell_end, c, ntiles, nty, T / nty, T % nty, lo, hi);
        const uint32_t n = (hi[0] - lo[0]) + (hi[1] - lo[1]) + (hi[2] - lo[2]) + (hi[3] - lo[3]);
        grid_chunks[b] = n == 0 ? 1u : (n + grid_chunk - 1) / grid_chunk;
        degrid_chunks[b] = (bin_count(bin_start, b) + kDegridChunk - 1) / kDegridChunk;
    }
}

__global__ void cube_work_fill(const uint32_t* grid_chunks, const uint32_t* grid_first,
                               const uint32_t* degrid_chunks, const uint32_t* degrid_first,
                               int64_t nbins, int64_t ntiles, int64_t nty, int64_t gnx,
                               int64_t gny, uint2* grid_items, uint2* degrid_items, float* psf,
                               float2* dirty) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nbins;
         b += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t n = grid_chunks[b], f = grid_first[b];
        for (uint32_t k = 0; k < n; ++k) grid_items[f + k] = make_uint2((uint32_t)b, k);
        const uint32_t nd = degrid_chunks[b], fd = degrid_first[b];
        for (uint32_t k = 0; k < nd; ++k) degrid_items[fd + k] = make_uint2((uint32_t)b, k);
        if (n > 1 && dirty) {
            const int64_t c = b / ntiles, T = b % ntiles;
            const int64_t x0 = (T / nty) * kTile, y0 = (T % nty) * kTile;
            float* pc = psf ? psf + c * gnx * gny : nullptr;
            float2* dc = dirty + c * gnx * gny;
            for (int64_t x = x0; x < min(x0 + kTile, gnx); ++x)
                for (int64_t y = y0; y < min(y0 + kTile, gny); ++y) {
                    if (pc) pc[x * gny + y] = 0.0f;
                    dc[x * gny + y] = make_float2(0.0f, 0.0f);
                }
        }
    }
}

struct CubeGridArgs {
    const uint4* rec;
    const float* rec_w;
    const uint32_t* bin_start;   // [C * ntiles + 1]
    const uint32_t* cell_end;    // [C * ntiles * 1024] end of each cell bin
    const float* taps;           // [tap_rows][7], zero-padded to taps_bytes
    int32_t tap_rows;
    uint32_t taps_bytes;
    int* status;                 // set to CR_TIMEOUT when a bounded wait gives up
    int64_t ntx, nty, gnx, gny;
    const uint2* items;          // (output tile bin, chunk)
    uint32_t grid_chunk;         // records per chunk
    const uint32_t* grid_chunks; // chunks of each output tile
    const unsigned long long* n_items;
    unsigned int* item_counter;
    float* psf;                  // [C][gnx][gny] real part of the PSF grid
    float2* dirty;               // [C][gnx][gny] (the residual grid with RESIDUAL)
    const float2* res;           // RESIDUAL: w (vis - pred) per record
    long long wait_polls;        // bound of the tap-table wait (the drain keeps the default)
};

// A block per work item: the chunk's records (from the four source bins)
// accumulate into a shared-memory copy of the output tile, which is then
// stored (single-chunk tile) or added (heavier tile) to the grid.  A warp
// loads 32 records, keeps those whose footprint reaches the tile and runs
// them in turn, one lane per tap; tile rows are kRow floats apart so that a
// record's 49 taps hit distinct banks.  (A variant with a private tile per
// warp and plain read-modify-writes ran 1.5x slower: 8 warps per SM could
// not hide the dependent shared-memory chain of consecutive records.)
constexpr int kGridThreads = kCubeThreads;

// With RESIDUAL the records carry w (vis - pred) from `res` and no PSF is
// formed.
template <bool RESIDUAL>
__global__ void __launch_bounds__(kGridThreads, 6) cube_grid_kernel(CubeGridArgs a) {
    __shared__ float s_psf[kTile * kRow];
    __shared__ float s_re[kTile * kRow];
    __shared__ float s_im[kTile * kRow];
    __shared__ __align__(16) float s_taps[kTapFloats];
    __shared__ __align__(8) uint64_t s_bar;
    // per warp, the decoded records of its current batch of 32:
    // {run key, x tap row * 7, y tap row * 7, weight} and {w vis}
    __shared__ int4 s_ra[kGridThreads];
    __shared__ float2 s_rb[kGridThreads];
    __shared__ int s_item;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t ntiles = a.ntx * a.nty;
    const unsigned long long n_items = *a.n_items;
    // the tap table by one bulk copy
    if (tid == 0) {
        mbar_init(&s_bar, 1);
        mbar_fence_init();
        mbar_expect_tx(&s_bar, a.taps_bytes);
        bulk_load(s_taps, a.taps, a.taps_bytes, &s_bar);
    }
    __syncthreads();
    if (!__syncthreads_and(mbar_wait(&s_bar, 0, a.wait_polls))) {
        if (tid == 0) {
            atomicExch(a.status, CR_TIMEOUT);
            mbar_wait(&s_bar, 0);   // let the copy land before the block exits
        }
        return;
    }
    int4* w_ra = s_ra + warp * 32;
    float2* w_rb = s_rb + warp * 32;
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(a.item_counter, 1u);
        __syncthreads();
        const int64_t item = s_item;
        if ((unsigned long long)item >= n_items) break;
        const uint2 it = a.items[item];
        const int64_t bin = it.x;
        const int64_t c = bin / ntiles, T = bin % ntiles;
        const int64_t tx = T / a.nty, ty = T % a.nty;
        const bool shared_tile = a.grid_chunks[bin] > 1;
        const uint32_t clo = it.y * a.grid_chunk, chi = clo + a.grid_chunk;
        // source s = home tile (tx - (s & 1), ty - (s >> 1)); [b0, b1) its records
        // inside this chunk (empty when none)
        uint32_t b0[4], b1[4];
        source_ranges(a.bin_start, a.cell_end, c, ntiles, a.nty, tx, ty, b0, b1);
        int nsrc = 0;
        uint32_t off = 0;   // position of this source in the concatenated order
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint32_t lo = b0[s], n = b1[s] - b0[s];
            const uint32_t a0 = max(off, clo), a1 = min(off + n, chi);
            b0[s] = b1[s] = 0;
            if (a0 < a1) {
                b0[s] = lo + (a0 - off);
                b1[s] = lo + (a1 - off);
                ++nsrc;
            }
            off += n;
        }
        const int64_t gx0 = tx * kTile, gy0 = ty * kTile;
        float* psf_c = RESIDUAL ? nullptr : a.psf + c * a.gnx * a.gny;
        float2* dirty_c = a.dirty + c * a.gnx * a.gny;
        if (nsrc == 0) {
            if (!shared_tile)
                for (int k = tid; k < kTile * kTile; k += kGridThreads) {
                    const int64_t x = gx0 + k / kTile, y = gy0 + k % kTile;
                    if (x < a.gnx && y < a.gny) {
                        if (!RESIDUAL) psf_c[x * a.gny + y] = 0.0f;
                        dirty_c[x * a.gny + y] = make_float2(0.0f, 0.0f);
                    }
                }
            __syncthreads();
            continue;
        }
        for (int k = tid; k < kTile * kRow; k += kGridThreads) {
            s_psf[k] = 0.0f;
            s_re[k] = 0.0f;
            s_im[k] = 0.0f;
        }
        __syncthreads();
        // Records of a home tile arrive in start-cell order, so a warp's
        // consecutive records often share a start cell: lane t sums tap t of
        // such a run in registers and adds it to the tile once per run.
        // Lane t holds taps t (slot 0) and t + 32 (slot 1, lanes 0-16; the
        // other lanes form a dummy product that is never added).  A run is
        // keyed by (source, start cell); a run whose footprint lies inside
        // the tile adds at run base + a per-lane offset without bounds tests.
        const int ix0 = lane / 7, iy0 = lane % 7;
        const int ix1 = (lane + 32) / 7, iy1 = (lane + 32) % 7;
        const bool has1 = lane + 32 < 49;
        const int jx1 = has1 ? ix1 : 0, jy1 = has1 ? iy1 : 0;
        const int off0 = ix0 * kRow + iy0, off1 = ix1 * kRow + iy1;
        uint32_t cur_key = ~0u;
        int cur_lx = 0, cur_ly = 0, cur_base = 0;
        bool cur_inside = false;
        // (psf slot 0, psf slot 1), (re, im) slot 0, (re, im) slot 1: paired
        // float32 FMAs (FFMA2) update two sums per instruction
        float2 pp = make_float2(0.f, 0.f), ri0 = pp, ri1 = pp;
        auto flush = [&]() {
            if (cur_inside) {
                const int c0 = cur_base + off0;
                if (!RESIDUAL) atomicAdd(&s_psf[c0], pp.x);
                atomicAdd(&s_re[c0], ri0.x);
                atomicAdd(&s_im[c0], ri0.y);
                if (has1) {
                    const int c1 = cur_base + off1;
                    if (!RESIDUAL) atomicAdd(&s_psf[c1], pp.y);
                    atomicAdd(&s_re[c1], ri1.x);
                    atomicAdd(&s_im[c1], ri1.y);
                }
                return;
            }
            int cx = cur_lx + ix0, cy = cur_ly + iy0;
            if (cx >= 0 && cx < kTile && cy >= 0 && cy < kTile) {
                const int cell = cx * kRow + cy;
                if (!RESIDUAL) atomicAdd(&s_psf[cell], pp.x);
                atomicAdd(&s_re[cell], ri0.x);
                atomicAdd(&s_im[cell], ri0.y);
            }
            cx = cur_lx + ix1;
            cy = cur_ly + iy1;
            if (has1 && cx >= 0 && cx < kTile && cy >= 0 && cy < kTile) {
                const int cell = cx * kRow + cy;
                if (!RESIDUAL) atomicAdd(&s_psf[cell], pp.y);
                atomicAdd(&s_re[cell], ri1.x);
                atomicAdd(&s_im[cell], ri1.y);
            }
        };
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const int sox = -(s & 1) * kTile, soy = -(s >> 1) * kTile;
            for (uint32_t base = b0[s] + warp * 32; base < b1[s]; base += kGridThreads) {
                // lanes load and decode 32 records; those that reach the
                // tile are packed into the warp's staging slots
                const uint32_t rr = base + lane;
                bool rel = false;
                int4 ra = make_int4(0, 0, 0, 0);
                float2 rb = make_float2(0.0f, 0.0f);
                if (rr < b1[s]) {
                    const uint4 q = a.rec[rr];
                    float qw = 0.0f;
                    if (RESIDUAL) {
                        rb = a.res[rr];
                    } else {
                        qw = a.rec_w[rr];
                        rb = make_float2(__uint_as_float(q.z), __uint_as_float(q.w));
                    }
                    const int lx = sox + (int)(q.x >> 27), ly = soy + (int)((q.x >> 22) & 31);
                    rel = lx + 6 >= 0 && ly + 6 >= 0;
                    ra = make_int4((int)((q.x >> 22) | ((uint32_t)s << 10)),
                                   (int)((q.x >> 11) & 2047u) * 7, (int)(q.x & 2047u) * 7,
                                   __float_as_int(qw));
                }
                const unsigned m = __ballot_sync(0xffffffffu, rel);
                if (rel) {
                    const int pos = __popc(m & ((1u << lane) - 1u));
                    w_ra[pos] = ra;
                    w_rb[pos] = rb;
                }
                __syncwarp();
                const int nrel = __popc(m);
                for (int k = 0; k < nrel; ++k) {
                    const int4 A = w_ra[k];
                    const float2 B = w_rb[k];
                    const float pw = __int_as_float(A.w);
                    const uint32_t key = (uint32_t)A.x;
                    if (key != cur_key) {
                        if (cur_key != ~0u) flush();
                        cur_key = key;
                        cur_lx = sox + (int)((key >> 5) & 31);
                        cur_ly = soy + (int)(key & 31);
                        cur_base = cur_lx * kRow + cur_ly;
                        cur_inside = cur_lx >= 0 && cur_ly >= 0 && cur_lx <= kTile - 7 &&
                                     cur_ly <= kTile - 7;
                        pp = ri0 = ri1 = make_float2(0.f, 0.f);
                    }
                    const float* wx = s_taps + A.y;
                    const float* wy = s_taps + A.z;
                    // w0 = wx[ix0] wy[iy0], w1 = wx[jx1] wy[jy1] (float32
                    // products), then one fused multiply-add per sum as before
                    const float2 w = __fmul2_rn(make_float2(wx[ix0], wx[jx1]),
                                                make_float2(wy[iy0], wy[jy1]));
                    if (!RESIDUAL) pp = __ffma2_rn(make_float2(pw, pw), w, pp);
                    ri0 = __ffma2_rn(B, make_float2(w.x, w.x), ri0);
                    ri1 = __ffma2_rn(B, make_float2(w.y, w.y), ri1);
                }
                __syncwarp();   // the slots are refilled by the next batch
            }
        }
        if (cur_key != ~0u) flush();
        __syncthreads();
        for (int k = tid; k < kTile * kTile; k += kGridThreads) {
            const int cx = k / kTile, cy = k % kTile;
            const int64_t x = gx0 + cx, y = gy0 + cy;
            if (x < a.gnx && y < a.gny) {
                const int cell = cx * kRow + cy;
                if (!shared_tile) {
                    if (!RESIDUAL) psf_c[x * a.gny + y] = s_psf[cell];
                    dirty_c[x * a.gny + y] = make_float2(s_re[cell], s_im[cell]);
                } else {
                    if (!RESIDUAL && s_psf[cell] != 0.0f)
                        atomicAdd(&psf_c[x * a.gny + y], s_psf[cell]);
                    if (s_re[cell] != 0.0f || s_im[cell] != 0.0f)
                        atomicAdd(&dirty_c[x * a.gny + y], make_float2(s_re[cell], s_im[cell]));
                }
            }
        }
        __syncthreads();
    }
}

struct CubeDegridArgs {
    const uint4* rec;
    const uint32_t* bin_start;   // [C * ntiles + 1]
    int32_t tap_rows;
    int64_t ntiles, nty, gnx, gny, R;
    const uint2* items;          // (bin, chunk)
    const unsigned long long* n_items;
    unsigned int* item_counter;
    const float* taps8;          // [tap_rows][8], rows padded to 32 bytes
    uint32_t taps8_bytes;
    const float2* grid;          // [C][gnx][gny]
    float2* pred;                // [C][R]
    const float* rec_w;          // RESIDUAL: imaging weight per record
    float2* res;                 // RESIDUAL: w vis - w pred per record
    int* status;                 // set to CR_TIMEOUT when a bounded wait gives up
    long long wait_polls;        // bound of the first waits (the drains keep the default)
};

// Bins in turn.  The block stages the 38 x 38 model footprint of its home
// tile in shared memory; a warp takes 4 records at a time, 7 lanes per
// record, lane ix forming wx[ix] * sum_iy wy[iy] g[x0 + ix][y0 + iy]
// (float32), and the 7 lanes' sums are reduced with shuffles.
// With RESIDUAL each record's w vis - w pred goes to res (record order)
// instead of pred (sample order).
// With TMA the footprints come as tensor-map boxes (float32 view
// [C][gnx][2 gny], box 76 x 38, zero-filled past the grid edge) into two
// buffers: while the block works on one item, the next item's footprint is
// already in flight.  Without TMA (a grid whose rows are not a multiple of
// 16 bytes, or an unaligned base) the block loads each footprint itself.
// The tap table arrives by one bulk copy in either case, its rows padded to
// 8 floats so that a record's 7 y taps come in two 16-byte loads (the
// kernel is bound by shared-memory instructions).
template <bool RESIDUAL, bool TMA>
__global__ void __launch_bounds__(kCubeThreads) cube_degrid_kernel(
    const __grid_constant__ CUtensorMap gmap, CubeDegridArgs a) {
    constexpr int kFoot = kTile + 6;
    constexpr int kPitch = TMA ? kFoot : kRow;   // float2 per footprint row
    constexpr int kBufs = TMA ? 2 : 1;
    constexpr uint32_t kBoxBytes = kFoot * kFoot * 8;
    // each buffer starts on a 128-byte boundary (tensor copy destinations)
    constexpr int kBufElems = (kFoot * kPitch * 8 + 127) / 128 * 16;
    __shared__ __align__(128) float2 s_g[kBufs][kBufElems];
    __shared__ __align__(8) uint64_t s_bar[3];   // footprint buffers 0, 1; taps
    __shared__ int s_item[2];
    extern __shared__ __align__(16) float s_taps[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int sub = lane >> 3, ix = lane & 7;   // record slot, tap column (7 = idle)
    const unsigned long long n_items = *a.n_items;
    // thread 0: the footprint of `item` into buffer `buf`
    auto issue = [&](int item, int buf) {
        const int64_t bin = a.items[item].x;
        const int64_t c = bin / a.ntiles, T = bin % a.ntiles;
        const int gx0 = (int)((T / a.nty) * kTile), gy0 = (int)((T % a.nty) * kTile);
        mbar_expect_tx(&s_bar[buf], kBoxBytes);
        tensor_load_3d(&s_g[buf][0], &gmap, 2 * gy0, gx0, (int)c, &s_bar[buf]);
    };
    if (tid == 0) {
        for (int k = 0; k < 3; ++k) mbar_init(&s_bar[k], 1);
        mbar_fence_init();
        mbar_expect_tx(&s_bar[2], a.taps8_bytes);
        bulk_load(s_taps, a.taps8, a.taps8_bytes, &s_bar[2]);
        const int first = (int)atomicAdd(a.item_counter, 1u);
        s_item[0] = first;
        if (TMA) {
            tensormap_prefetch(&gmap);
            if ((unsigned long long)first < n_items) issue(first, 0);
        }
    }
    __syncthreads();
    if (!__syncthreads_and(mbar_wait(&s_bar[2], 0, a.wait_polls))) {
        if (tid == 0) {
            atomicExch(a.status, CR_TIMEOUT);
            // let this block's copies in flight land before it exits
            mbar_wait(&s_bar[2], 0);
            if (TMA && (unsigned long long)s_item[0] < n_items) mbar_wait(&s_bar[0], 0);
        }
        return;
    }
    uint32_t phase = 0u;   // bit k: parity of buffer k's next phase
    int b = 0;
    for (;;) {
        const int64_t item = s_item[b];
        if ((unsigned long long)item >= n_items) break;
        if (TMA) {
            if (tid == 0) {
                const int next = (int)atomicAdd(a.item_counter, 1u);
                s_item[b ^ 1] = next;
                if ((unsigned long long)next < n_items) issue(next, b ^ 1);
            }
        } else if (tid == 0) {
            s_item[b ^ 1] = (int)atomicAdd(a.item_counter, 1u);
        }
        const uint2 it = a.items[item];
        const int64_t bin = it.x;
        const uint32_t lo = a.bin_start[bin] + it.y * kDegridChunk;
        const uint32_t hi = min(a.bin_start[bin + 1], lo + kDegridChunk);
        const float2* sg = &s_g[TMA ? b : 0][0];
        if (TMA) {
            if (!__syncthreads_and(mbar_wait(&s_bar[b], (phase >> b) & 1u, a.wait_polls))) {
                if (tid == 0) {
                    atomicExch(a.status, CR_TIMEOUT);
                    // let this block's copies in flight land before it exits
                    mbar_wait(&s_bar[b], (phase >> b) & 1u);
                    if ((unsigned long long)s_item[b ^ 1] < n_items)
                        mbar_wait(&s_bar[b ^ 1], (phase >> (b ^ 1)) & 1u);
                }
                return;
            }
            phase ^= 1u << b;
        } else {
            const int64_t c = bin / a.ntiles, T = bin % a.ntiles;
            const int64_t gx0 = (T / a.nty) * kTile, gy0 = (T % a.nty) * kTile;
            const float2* g = a.grid + c * a.gnx * a.gny;
            for (int k = tid; k < kFoot * kFoot; k += kCubeThreads) {
                const int fx = k / kFoot, fy = k % kFoot;
                const int64_t x = gx0 + fx, y = gy0 + fy;
                float2 v = make_float2(0.0f, 0.0f);
                if (x < a.gnx && y < a.gny) v = __ldg(&g[x * a.gny + y]);
                s_g[0][fx * kPitch + fy] = v;
            }
            __syncthreads();
        }
        // each record is loaded one iteration ahead of its use, so a warp
        // keeps the next batch's loads in flight while it computes
        uint4 qn = make_uint4(0u, 0u, 0u, 0u);
        float wn = 0.0f;
        if (lo + warp * 4 + sub < hi) {
            qn = a.rec[lo + warp * 4 + sub];
            if (RESIDUAL) wn = a.rec_w[lo + warp * 4 + sub];
        }
        for (uint32_t base = lo + warp * 4; base < hi; base += kCubeThreads / 8) {
            const uint32_t k = base + sub;
            const uint4 q = qn;
            const float w = wn;
            if (k + kCubeThreads / 8 < hi) {
                qn = a.rec[k + kCubeThreads / 8];
                if (RESIDUAL) wn = a.rec_w[k + kCubeThreads / 8];
            }
            float2 acc = make_float2(0.0f, 0.0f);   // (re, im), paired FMAs
            uint32_t sample = 0;
            if (k < hi) {
                sample = q.y;
                if (ix < 7) {
                    const uint32_t meta = q.x;
                    const float wxi = s_taps[((meta >> 11) & 2047u) * 8 + ix];
                    const float4* wy4 = reinterpret_cast<const float4*>(s_taps) +
                                        (meta & 2047u) * 2;
                    const float4 ya = wy4[0], yb = wy4[1];
                    const float wy[7] = {ya.x, ya.y, ya.z, ya.w, yb.x, yb.y, yb.z};
                    const int row =
                        ((int)(meta >> 27) + ix) * kPitch + (int)((meta >> 22) & 31);
#pragma unroll
                    for (int iy = 0; iy < 7; ++iy) {
                        const float wgt = __fmul_rn(wxi, wy[iy]);
                        acc = __ffma2_rn(sg[row + iy], make_float2(wgt, wgt), acc);
                    }
                }
            }
            float re = acc.x, im = acc.y;
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) {
                re += __shfl_xor_sync(0xffffffffu, re, o);
                im += __shfl_xor_sync(0xffffffffu, im, o);
            }
            if (ix == 0 && k < hi) {
                if (RESIDUAL) {
                    a.res[k] = make_float2(__fsub_rn(__uint_as_float(q.z), __fmul_rn(w, re)),
                                           __fsub_rn(__uint_as_float(q.w), __fmul_rn(w, im)));
                } else if (sample != kNullSample) {
                    a.pred[sample] = make_float2(re, im);
                }
            }
        }
        __syncthreads();
        b ^= 1;
    }
}

// Per-sample plan of every channel (start cells, tap rows, imaging weight).
__global__ void __launch_bounds__(kCubeThreads) cube_taps_kernel(CubeArgs a, CubeTaps t) {
    const int c = blockIdx.y;
    const CubeChan ch = a.ch[c];
    const float f2 = a.mode == CR_WEIGHT_BRIGGS ? a.f2[c] : 0.0f;
    const int64_t r0 = (int64_t)blockIdx.x * kRowsPerBlock;
    const int64_t r1 = min(a.R, r0 + kRowsPerBlock);
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int64_t base = r0 + wp * kWarpRows; base < r1; base += kCubeThreads * kVec) {
        Eval ev[kVec];
        eval_samples(a, ch, f2, c, base + lane, r1, ev);
#pragma unroll
        for (int j = 0; j < kVec; ++j) {
            const int64_t r = base + lane + 32 * j;
            if (r >= r1) continue;
            const int64_t i = (int64_t)c * a.R + r;
            const Eval e = ev[j];
            if (e.ok) {
                const int64_t tx = e.tile / a.nty, ty = e.tile % a.nty;
                t.start_x[i] = (int32_t)(tx * kTile + (e.meta >> 27));
                t.start_y[i] = (int32_t)(ty * kTile + ((e.meta >> 22) & 31));
                t.row_x[i] = (int32_t)((e.meta >> 11) & 2047u);
                t.row_y[i] = (int32_t)(e.meta & 2047u);
                t.weight[i] = e.w;
            } else {
                t.start_x[i] = t.start_y[i] = t.row_x[i] = t.row_y[i] = -1;
                t.weight[i] = 0.0f;
            }
        }
    }
}

}  // namespace

void cube_upload_channels(cr_ctx* ctx, cr_gridder* g, const CubeInput& in) {
    const cr_grid_info& gi = g->info;
    const double dus = (double)g->geom.nx * g->geom.cell_x_rad;
    const double dvs = (double)g->geom.ny * g->geom.cell_y_rad;
    std::vector<CubeChan> chh((size_t)in.C);
    for (int c = 0; c < in.C; ++c) {
        const double s = in.lambda_scale[c];
        if (!(std::isfinite(s) && s > 0.0)) fail(CR_INVALID, "lambda_scale must be finite and > 0");
        chh[c].lscale = s;
        chh[c].kx = fix_scale_of(s, gi.du, false);
        chh[c].ky = fix_scale_of(s, gi.dv, false);
        chh[c].kdx = fix_scale_of(s, dus, true);
        chh[c].kdy = fix_scale_of(s, dvs, true);
        chh[c].fx = df_scale_of(s, gi.du, false);
        chh[c].fy = df_scale_of(s, gi.dv, false);
        chh[c].fdx = df_scale_of(s, dus, true);
        chh[c].fdy = df_scale_of(s, dvs, true);
    }
    CubeChan* chd = (CubeChan*)workspace(ctx, "cube_chan", chh.size() * sizeof(CubeChan));
    CR_CUDA_CHECK(cudaMemcpyAsync(chd, chh.data(), chh.size() * sizeof(CubeChan),
                                  cudaMemcpyHostToDevice, ctx->stream));
    // the pageable source must outlive the copy
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
}

CubeRecords cube_plan(cr_ctx* ctx, cr_gridder* g, const CubeInput& in, int32_t mode,
                      float robust, const CubeTaps* taps, Pool* keep) {
    // buffers the records and work lists live in: the plan's own pool when
    // given (a persistent plan), else the context's workspaces
    auto kept = [&](const char* name, size_t bytes) {
        return keep ? pool_alloc(ctx, *keep, name, bytes) : workspace(ctx, name, bytes);
    };
    if (mode != CR_WEIGHT_NATURAL && mode != CR_WEIGHT_UNIFORM && mode != CR_WEIGHT_BRIGGS)
        fail(CR_INVALID, "unknown weighting mode");
    if (in.C <= 0 || in.C > 65535) fail(CR_INVALID, "channels must lie in [1, 65535]");
    if (in.R < 0) fail(CR_INVALID, "negative row count");
    if ((uint64_t)in.C * (uint64_t)in.R >= (1ull << 32))
        fail(CR_INVALID, "cube larger than 2^32 samples");
    const cr_grid_info& gi = g->info;
    if (gi.oversampling > kMaxTapRows - 1) fail(CR_INVALID, "cube oversampling above 512");
    CubeRecords cr{};
    cr.R = in.R;
    cr.C = in.C;
    cr.ntx = (gi.grid_nx + kTile - 1) / kTile;
    cr.nty = (gi.grid_ny + kTile - 1) / kTile;
    cr.ntiles = cr.ntx * cr.nty;
    const int64_t nbins = (int64_t)in.C * cr.ntiles;
    const size_t ns = (size_t)std::max<int64_t>((int64_t)in.C * in.R, 1);
    // per-channel constants (uploaded before a capture by the caller)
    const double dus = (double)g->geom.nx * g->geom.cell_x_rad;
    const double dvs = (double)g->geom.ny * g->geom.cell_y_rad;
    if (!ctx->capturing) cube_upload_channels(ctx, g, in);
    CubeChan* chd = (CubeChan*)workspace(ctx, "cube_chan", (size_t)in.C * sizeof(CubeChan));
    cr.rec = (uint4*)kept("cube_rec", ns * 16);
    cr.rec_w = (float*)kept("cube_rec_w", ns * 4);
    cr.bin_start = (uint32_t*)kept("cube_bin_start", (size_t)(nbins + 1) * 4);
    const int64_t ncells = (nbins << 10) + 1;   // (channel, tile, cell) bins + total
    if (ncells >= (1ll << 32)) fail(CR_INVALID, "cube has too many (channel, tile, cell) bins");
    uint32_t* hist = (uint32_t*)kept("cube_hist", (size_t)ncells * 4);
    cr.sumwt = (double*)kept("cube_sumwt", (size_t)in.C * 8);
    cr.counts = (unsigned long long*)kept("cube_counts", (size_t)in.C * 16 + 8);
    cr.n_rec = cr.counts + 2 * in.C;
    CR_CUDA_CHECK(cudaMemsetAsync(hist, 0, (size_t)ncells * 4, ctx->stream));
    CR_CUDA_CHECK(cudaMemsetAsync(cr.sumwt, 0, (size_t)in.C * 8, ctx->stream));
    CR_CUDA_CHECK(cudaMemsetAsync(cr.counts, 0, (size_t)in.C * 16 + 8, ctx->stream));

    CubeArgs a{};
    a.R = in.R;
    a.C = in.C;
    a.u = in.u;
    a.v = in.v;
    a.ch = chd;
    a.vis = in.vis;
    a.weight = in.weight;
    a.flags = in.flags;
    a.du = gi.du;
    a.dv = gi.dv;
    a.gnx = gi.grid_nx;
    a.gny = gi.grid_ny;
    a.os = gi.oversampling;
    a.tap_rows = g->tap_rows;
    a.ntx = cr.ntx;
    a.nty = cr.nty;
    a.cx_fix = (long long)gi.grid_nx << (kFixF - 1);
    a.cy_fix = (long long)gi.grid_ny << (kFixF - 1);
    a.nx = g->geom.nx;
    a.ny = g->geom.ny;
    a.dus = dus;
    a.dvs = dvs;
    a.dcx = (double)g->geom.nx / 2.0;
    a.dcy = (double)g->geom.ny / 2.0;
    a.dcx_fix = (long long)g->geom.nx << (kFixF - 1);
    a.dcy_fix = (long long)g->geom.ny << (kFixF - 1);
    a.mode = mode;
    a.hist = hist;
    a.cursor = hist;
    a.sumwt = cr.sumwt;
    a.counts = cr.counts;
    a.rec = cr.rec;
    a.rec_w = cr.rec_w;
    const dim3 grid((unsigned)std::max<int64_t>((in.R + kRowsPerBlock - 1) / kRowsPerBlock, 1),
                    (unsigned)in.C);
    float4* uvdf = (float4*)workspace(ctx, "cube_uvdf", (size_t)std::max<int64_t>(in.R, 1) * 16);
    if (in.R > 0) {
        cube_rows_df_kernel<<<grid_blocks(in.R, 256), 256, 0, ctx->stream>>>(in.u, in.v, in.R,
                                                                             uvdf);
        note_launch(ctx, "cube_rows_df_kernel");
    }
    a.uvdf = uvdf;
    a.ev_tile = (uint32_t*)workspace(ctx, "cube_ev_tile", ns * 4);
    a.ev_meta = (uint32_t*)workspace(ctx, "cube_ev_meta", ns * 4);
    if (mode == CR_WEIGHT_NATURAL && in.R > 0) {
        cube_density_kernel<false><<<grid, kCubeThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "cube_plan_kernel");
    }
    if (mode != CR_WEIGHT_NATURAL) {
        const int64_t cells = (int64_t)g->geom.nx * g->geom.ny;
        a.density = (float*)workspace(ctx, "cube_density", (size_t)(in.C * cells) * 4);
        a.dcell = (uint32_t*)workspace(ctx, "cube_dcell", ns * 4);
        CR_CUDA_CHECK(cudaMemsetAsync(a.density, 0, (size_t)(in.C * cells) * 4, ctx->stream));
        if (in.R > 0) {
            cube_density_kernel<true><<<grid, kCubeThreads, 0, ctx->stream>>>(a);
            note_launch(ctx, "cube_density_kernel");
        }
        float* f2 = (float*)workspace(ctx, "cube_f2", (size_t)in.C * 4);
        if (mode == CR_WEIGHT_BRIGGS) {
            double* sums = (double*)workspace(ctx, "cube_dsums", (size_t)in.C * 16);
            CR_CUDA_CHECK(cudaMemsetAsync(sums, 0, (size_t)in.C * 16, ctx->stream));
            const dim3 sg((unsigned)std::min<int64_t>((cells + 255) / 256, 64), (unsigned)in.C);
            cube_density_sums<<<sg, 256, 0, ctx->stream>>>(a.density, cells, sums);
            note_launch(ctx, "cube_density_sums");
            const double am = 5.0 * std::pow(10.0, -(double)robust);
            cube_f2_kernel<<<(in.C + 127) / 128, 128, 0, ctx->stream>>>(sums, in.C, am * am, f2);
            note_launch(ctx, "cube_f2_kernel");
        }
        a.f2 = f2;
    }
    if (taps) {
        if (in.R > 0) {
            cube_taps_kernel<<<grid, kCubeThreads, 0, ctx->stream>>>(a, *taps);
            note_launch(ctx, "cube_taps_kernel");
        }
        return cr;
    }
    // in place: hist becomes each cell bin's first slot, the scatter's cursor
    exclusive_scan_u32(ctx, hist, hist, ncells, nullptr);
    tile_starts_from_cells<<<grid_blocks(nbins + 1, 256), 256, 0, ctx->stream>>>(hist, nbins,
                                                                                 cr.bin_start);
    note_launch(ctx, "tile_starts_from_cells");
    if (in.R > 0) {
        cube_scatter_kernel<<<grid, kCubeThreads, 0, ctx->stream>>>(a);
        note_launch(ctx, "cube_scatter_kernel");
    }
    // work-list buffers (the lists are made by cube_grid / cube_degrid)
    cr.grid_chunks = (uint32_t*)kept("cube_gchunks", (size_t)nbins * 4);
    cr.degrid_chunks = (uint32_t*)kept("cube_dchunks", (size_t)nbins * 4);
    cr.cell_end = hist;
    cr.grid_first = (uint32_t*)kept("cube_gfirst", (size_t)nbins * 4);
    cr.degrid_first = (uint32_t*)kept("cube_dfirst", (size_t)nbins * 4);
    cr.n_items = (unsigned long long*)kept("cube_nitems", 16);
    // sum over tiles of ceil(n / K) <= tiles + (sum n) / K, and each record is a
    // source of at most four output tiles
    const size_t max_grid_items = (size_t)nbins + 4 * ns / kGridChunkMin + 1;
    const size_t max_degrid_items = (size_t)nbins + ns / kDegridChunk + 1;
    cr.grid_items = (uint2*)kept("cube_gitems", max_grid_items * 8);
    cr.degrid_items = (uint2*)kept("cube_ditems", max_degrid_items * 8);
    return cr;
}

// Work lists for one gridding chunk size; with psf/dirty, heavy output tiles
// are zeroed for their atomic chunks.
static void make_work_lists(cr_ctx* ctx, cr_gridder* g, CubeRecords& cr, uint32_t chunk,
                            float* psf, float2* dirty, const uint8_t* plane_mask = nullptr) {
    const cr_grid_info& gi = g->info;
    const int64_t nbins = (int64_t)cr.C * cr.ntiles;
    cube_work_count<<<grid_blocks(nbins, 256), 256, 0, ctx->stream>>>(
        cr.bin_start, cr.cell_end, nbins, cr.ntiles, cr.nty, chunk, plane_mask, cr.grid_chunks,
        cr.degrid_chunks);
    note_launch(ctx, "cube_work_count");
    exclusive_scan_u32(ctx, cr.grid_chunks, cr.grid_first, nbins, cr.n_items);
    exclusive_scan_u32(ctx, cr.degrid_chunks, cr.degrid_first, nbins, cr.n_items + 1);
    cube_work_fill<<<grid_blocks(nbins, 256), 256, 0, ctx->stream>>>(
        cr.grid_chunks, cr.grid_first, cr.degrid_chunks, cr.degrid_first, nbins, cr.ntiles,
        cr.nty, gi.grid_nx, gi.grid_ny, cr.grid_items, cr.degrid_items, psf, dirty);
    note_launch(ctx, "cube_work_fill");
    cr.grid_chunk = chunk;
    cr.fill_done = true;
    cr.lists_masked = plane_mask != nullptr;
}

template <bool RESIDUAL>
static void launch_cube_grid(cr_ctx* ctx, cr_gridder* g, const CubeRecords& cr, float* psf,
                             float2* dirty, const float2* res = nullptr) {
    const cr_grid_info& gi = g->info;
    unsigned int* counter = (unsigned int*)workspace(ctx, "cube_counter", 8);
    CR_CUDA_CHECK(cudaMemsetAsync(counter, 0, 8, ctx->stream));
    CubeGridArgs a{cr.rec, cr.rec_w, cr.bin_start, cr.cell_end, g->taps_d, g->tap_rows,
                   g->taps_bytes, ctx->status_d, cr.ntx, cr.nty, gi.grid_nx, gi.grid_ny,
                   cr.grid_items, cr.grid_chunk, cr.grid_chunks, cr.n_items, counter, psf,
                   dirty, res, ctx->mbar_polls};
    int sms = 0;
    CR_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    int per_sm = 0;
    CR_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, cube_grid_kernel<RESIDUAL>, kGridThreads, 0));
    cube_grid_kernel<RESIDUAL><<<sms * std::max(per_sm, 1), kGridThreads, 0, ctx->stream>>>(a);
    note_launch(ctx, RESIDUAL ? "cube_grid_kernel_residual" : "cube_grid_kernel");
}

static std::string cube_shape_key(const cr_gridder* g, const CubeRecords& cr) {
    return std::to_string(cr.C) + "x" + std::to_string(cr.ntx) + "x" + std::to_string(cr.nty) +
           "/" + std::to_string(g->info.oversampling);
}

bool cube_grid_chunk_valid(uint32_t chunk) {
    for (uint32_t c : kGridChunkCandidates)
        if (c == chunk) return true;
    return false;
}

void cube_grid(cr_ctx* ctx, cr_gridder* g, CubeRecords& cr, float* psf, float2* dirty) {
    const std::string key = cube_shape_key(g, cr);
    auto tuned = ctx->cube_chunk.find(key);
    if (tuned == ctx->cube_chunk.end() && !ctx->capturing && !ctx->cube_chunk_forced) {
        // first use of this cube shape: time the gridding pass (work lists
        // and kernel) for every candidate chunk size and keep the fastest
        cudaEvent_t e0 = ctx->kev[0], e1 = ctx->kev[1];
        float best_ms = 0.0f;
        uint32_t best = kGridChunkDefault;
        for (uint32_t chunk : kGridChunkCandidates) {
            CR_CUDA_CHECK(cudaEventRecord(e0, ctx->stream));
            make_work_lists(ctx, g, cr, chunk, psf, dirty);
            launch_cube_grid<false>(ctx, g, cr, psf, dirty);
            CR_CUDA_CHECK(cudaEventRecord(e1, ctx->stream));
            CR_CUDA_CHECK(cudaEventSynchronize(e1));
            float ms = 0.0f;
            CR_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
            if (chunk == kGridChunkCandidates[0] || ms < best_ms) {
                best_ms = ms;
                best = chunk;
            }
        }
        ctx->cube_chunk[key] = best;
        tuned = ctx->cube_chunk.find(key);
    }
    uint32_t chunk = tuned != ctx->cube_chunk.end() ? tuned->second : kGridChunkDefault;
    if (ctx->cube_chunk_forced) chunk = ctx->cube_chunk_forced;
    make_work_lists(ctx, g, cr, chunk, psf, dirty);
    kernel_mark(ctx, 0, false);
    launch_cube_grid<false>(ctx, g, cr, psf, dirty);
    kernel_mark(ctx, 0, true);
}

template <bool RESIDUAL>
static void launch_cube_degrid(cr_ctx* ctx, cr_gridder* g, const CubeRecords& cr,
                               const float2* grid, float2* pred, float2* res) {
    const cr_grid_info& gi = g->info;
    unsigned int* counter = (unsigned int*)workspace(ctx, "cube_counter", 8);
    CR_CUDA_CHECK(cudaMemsetAsync(counter, 0, 8, ctx->stream));
    const uint32_t taps8_bytes = (uint32_t)g->tap_rows * 32u;
    CubeDegridArgs a{cr.rec, cr.bin_start, g->tap_rows, cr.ntiles, cr.nty, gi.grid_nx,
                     gi.grid_ny, cr.R, cr.degrid_items, cr.n_items + 1, counter, g->taps8_d,
                     taps8_bytes, grid, pred, cr.rec_w, res, ctx->status_d, ctx->mbar_polls};
    int sms = 0;
    CR_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    // the grids as float32 [C][gnx][2 gny] for footprint boxes of 76 x 38
    CUtensorMap map;
    std::memset(&map, 0, sizeof(map));
    const uint64_t row = (uint64_t)gi.grid_ny * 8;
    const bool tma = encode_tensor_map_3d(&map, grid, 2 * (uint64_t)gi.grid_ny,
                                          (uint64_t)gi.grid_nx, (uint64_t)cr.C, row,
                                          row * (uint64_t)gi.grid_nx, 2 * (kTile + 6), kTile + 6);
    if (tma)
        cube_degrid_kernel<RESIDUAL, true>
            <<<sms * 8, kCubeThreads, taps8_bytes, ctx->stream>>>(map, a);
    else
        cube_degrid_kernel<RESIDUAL, false>
            <<<sms * 8, kCubeThreads, taps8_bytes, ctx->stream>>>(map, a);
    note_launch(ctx, RESIDUAL ? "cube_degrid_kernel_residual" : "cube_degrid_kernel");
}

void cube_grid_residual(cr_ctx* ctx, cr_gridder* g, CubeRecords& cr, const float2* model,
                        float2* residual, const uint8_t* plane_mask) {
    auto tuned = ctx->cube_chunk.find(cube_shape_key(g, cr));
    uint32_t chunk = tuned != ctx->cube_chunk.end() ? tuned->second : kGridChunkDefault;
    if (ctx->cube_chunk_forced) chunk = ctx->cube_chunk_forced;
    // the lists skip masked planes and zero the heavy tiles of the others
    make_work_lists(ctx, g, cr, chunk, nullptr, residual, plane_mask);
    const size_t nrec = cr.n_records >= 0 ? (size_t)std::max<int64_t>(cr.n_records, 1)
                                          : (size_t)std::max<int64_t>((int64_t)cr.C * cr.R, 1);
    float2* res = (float2*)workspace(ctx, "cube_res", nrec * 8);
    kernel_mark(ctx, 1, false);
    launch_cube_degrid<true>(ctx, g, cr, model, nullptr, res);
    kernel_mark(ctx, 1, true);
    kernel_mark(ctx, 0, false);
    launch_cube_grid<true>(ctx, g, cr, nullptr, residual, res);
    kernel_mark(ctx, 0, true);
}

void cube_degrid(cr_ctx* ctx, cr_gridder* g, CubeRecords& cr, const float2* grid,
                 float2* pred) {
    CR_CUDA_CHECK(cudaMemsetAsync(pred, 0, (size_t)cr.C * cr.R * 8, ctx->stream));
    // the degridding work list without a gridding pass before it
    if (!cr.fill_done || cr.lists_masked)
        make_work_lists(ctx, g, cr, cr.fill_done ? cr.grid_chunk : kGridChunkDefault, nullptr,
                        nullptr);
    kernel_mark(ctx, 1, false);
    launch_cube_degrid<false>(ctx, g, cr, grid, pred, nullptr);
    kernel_mark(ctx, 1, true);
}

void cube_read_sums(cr_ctx* ctx, const CubeRecords& cr, cr_sums* out) {
    if (!out) return;
    std::vector<double> sw((size_t)cr.C);
    std::vector<unsigned long long> cnt((size_t)cr.C * 2);
    CR_CUDA_CHECK(cudaMemcpyAsync(sw.data(), cr.sumwt, sw.size() * 8, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    CR_CUDA_CHECK(cudaMemcpyAsync(cnt.data(), cr.counts, cnt.size() * 8, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < cr.C; ++c) {
        out[c].normalization_sumwt = sw[c];
        out[c].reported_sumwt = sw[c];
        out[c].gridded = (int64_t)cnt[2 * c];
        out[c].skipped = (int64_t)cnt[2 * c + 1];
        out[c].unique_records = (int64_t)cnt[2 * c];
        out[c].taps = 49 * (int64_t)cnt[2 * c];
    }
}

}  // namespace cr
