// cr_clean.cuh -- device pieces shared by the minor cycles (Hogbom,
// multiscale): the peak candidate of a block and its reductions (largest
// |value|, ties to the smallest y * nx + x, as
// peak_location_masked_in_bounds_zero_tolerance, lib.rs:74064-74118), the
// bounded grid barrier of the cooperative launches, and the stop rules
// (threshold_reached_with_tolerance and minor_cycle_stop_reason,
// lib.rs:74628-74676).
#pragma once

#include <cstdint>

#include "casars_cuda.h"

namespace cr {

struct Cand {
    float absval;  // -1 when the block has no cleanable pixel
    int key;       // y * nx + x
    float value;
    int pad;
};

__device__ __forceinline__ bool better(float a_abs, int a_key, float b_abs, int b_key) {
    return a_abs > b_abs || (a_abs == b_abs && a_key < b_key);
}

__device__ __forceinline__ void warp_argmax(float& a, int& k, float& v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float a2 = __shfl_xor_sync(0xffffffffu, a, o);
        int k2 = __shfl_xor_sync(0xffffffffu, k, o);
        float v2 = __shfl_xor_sync(0xffffffffu, v, o);
        if (better(a2, k2, a, k)) {
            a = a2;
            k = k2;
            v = v2;
        }
    }
}

// Block argmax of (abs, key, value); result valid in thread 0.
static __device__ Cand block_argmax(float a, int k, float v) {
    __shared__ Cand sh[32];
    warp_argmax(a, k, v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = Cand{a, k, v, 0};
    __syncthreads();
    Cand c{-1.0f, 0x7fffffff, 0.0f, 0};
    if (warp == 0) {
        Cand m = lane < (int)(blockDim.x >> 5) ? sh[lane] : Cand{-1.0f, 0x7fffffff, 0.0f, 0};
        a = m.absval;
        k = m.key;
        v = m.value;
        warp_argmax(a, k, v);
        c = Cand{a, k, v, 0};
    }
    __syncthreads();
    return c;
}

// Bounded grid barrier (all blocks are co-resident under the cooperative
// launch).  A waiting block polls the generation word at most `polls` times
// after its first look.  Returns false on every thread of a block whose
// wait timed out.
static __device__ bool grid_barrier(unsigned int* bar, unsigned int nblocks, long long polls) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int* gen = bar + 1;
        unsigned int g = *gen;
        __threadfence();
        unsigned int arrived = atomicAdd(&bar[0], 1u);
        if (arrived == nblocks - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicAdd(&bar[1], 1u);
        } else {
            long long spins = 0;
            while (*gen == g) {
                if (++spins > polls) {
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ bool threshold_reached(float peak, float thr) {
    if (thr <= 0.0f) return peak <= thr;
    float tol = fmaxf(__fmul_rn(0.01f, thr), 2.0e-8f);
    return peak <= thr || fabsf(__fsub_rn(peak, thr)) <= tol;
}

static __device__ int stop_reason(float peak_abs, float thr, float cyc, float nsig) {
    bool floor_active = thr > 0.0f && __fmul_rn(0.01f, thr) < 2.0e-8f && cyc <= thr;
    if (peak_abs < thr || (floor_active && threshold_reached(peak_abs, thr)))
        return CR_STOP_GLOBAL_THRESHOLD;
    if (cyc >= nsig) return peak_abs < cyc ? CR_STOP_CYCLE_THRESHOLD : 0;
    if (nsig > thr) return peak_abs < nsig ? CR_STOP_NSIGMA_THRESHOLD : 0;
    return 0;
}

}  // namespace cr
