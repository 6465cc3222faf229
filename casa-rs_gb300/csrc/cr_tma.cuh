// Bulk asynchronous copies (TMA) into shared memory, completed on mbarriers.
//
// Two forms are used: the one-dimensional cp.async.bulk (both addresses
// 16-byte aligned, a size that is a multiple of 16 bytes) for tables, and
// the tiled cp.async.bulk.tensor with a tensor map for 2-D grid footprints
// (innermost coordinate x element size a multiple of 16 bytes; elements
// outside the tensor are filled with zeros and still count toward the
// transaction bytes).  Every wait is bounded: after kMbarSpinLimit polls the
// caller gets false and reports CR_TIMEOUT through the context's status
// word instead of spinning on.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace cr {

constexpr long long kMbarSpinLimit = 1ll << 22;   // equals kMbarPollsDefault

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

// makes the initialised barriers visible to the async proxy
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// true once the phase with this parity has completed; false after `limit`
// unsuccessful polls (0: give up without polling)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
    for (long long i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    return mbar_wait(bar, parity, kMbarSpinLimit);
}

// bytes from global src to shared dst (both 16-byte aligned, bytes % 16 == 0)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// the box of a 3-D tensor map at (x, y, z) (x innermost) into shared dst
// (128-byte aligned)
__device__ __forceinline__ void tensor_load_3d(void* dst, const CUtensorMap* map, int x, int y,
                                               int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z),
        "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tensormap_prefetch(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Host: a 3-D tiled tensor map over float32 data [d2][d1][d0] (d0 innermost,
// strides in bytes for d1 and d2) with box {b0, b1, 1}.  Returns false when
// the shape breaks the tensor-map rules (16-byte aligned base, strides that
// are multiples of 16 bytes, an inner box of a multiple of 16 bytes) or the
// driver entry point is missing; callers then take their plain-load path.
bool encode_tensor_map_3d(CUtensorMap* map, const void* base, uint64_t d0, uint64_t d1,
                          uint64_t d2, uint64_t stride1, uint64_t stride2, uint32_t b0,
                          uint32_t b1);

}  // namespace cr
