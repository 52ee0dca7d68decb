// Tensor-memory-accelerator (TMA) helpers: 3D tiled tensor maps on the host,
// mbarrier + cp.async.bulk.tensor on the device (inline PTX, sm_90 and later
// syntax; the kernels here are built for sm_103a).
//
// Rules the callers keep (checked where the maps are made):
//  * global base 16-byte aligned, row and plane pitches multiples of 16 bytes;
//  * the innermost box extent x elem a multiple of 16 bytes;
//  * every copy starts at an x coordinate whose byte offset is a multiple of
//    16 (the hardware does not check this before the copy runs);
//  * shared-memory destinations 128-byte aligned.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstdint>

#include "common.cuh"

namespace mlau {

// --- host -----------------------------------------------------------------------
// 3D map of an (nz, ny, nx) array with row pitch px elements (px >= nx); the
// box is bx x by x bz elements.  Returns MLAU_OK or an error with a message.
int tma_map_3d(CUtensorMap *map, const void *base, int elem_bytes, int nx, int ny, int nz,
               long long px, int bx, int by, int bz);

// --- device ---------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

// Make mbarrier initialisation and earlier generic-proxy shared-memory
// accesses visible to the async proxy (TMA).
__device__ __forceinline__ void fence_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for phase `parity` of an mbarrier; false when it gave up.
constexpr long long kMbarSpinLimit = 1LL << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    for (long long it = 0; it < kMbarSpinLimit; it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 3D tiled load of one box at element coordinates (x, y, z) into shared
// memory; completion is signalled on `bar` as transaction bytes.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace mlau
