// Tensor-memory-accelerator (TMA) loads and mbarrier waits for the volume
// walks.  A CTA stages boxes of z planes of the volume into shared memory with
// cp.async.bulk.tensor; completion is tracked by an mbarrier whose expected
// transaction count is the box size.  Every wait is bounded: after
// TMA_SPIN_LIMIT polls the caller gets false and reports ERR_TMA_TIMEOUT
// instead of hanging.
#pragma once
#include <cuda.h>

#include "mesh_internal.cuh"

namespace mesh {

constexpr unsigned ERR_TMA_TIMEOUT = 8u;
constexpr int TMA_SPIN_LIMIT = 1 << 20;  // polls of ~1 us each at most

// Box of one volume stage: BX samples in x (a multiple of 16 bytes, starting on
// a 16-byte boundary at or below the tile's first sample: the 32 samples of a
// warp tile plus the rounding, at most ALIGN - 1), BY sample rows, BZ planes.
template <class T> struct TmaBox;
template <> struct TmaBox<float> { static constexpr int BX = 36, ALIGN = 4; };
template <> struct TmaBox<uint16_t> { static constexpr int BX = 40, ALIGN = 8; };
template <> struct TmaBox<double> { static constexpr int BX = 34, ALIGN = 2; };
constexpr int TMA_BY = 8 * WY + 1;  // the CTA's 32 cell rows + 1
constexpr int TMA_BZ = 4;           // planes per stage
constexpr int TMA_STAGES = 3;       // stages in the shared-memory ring
// Bytes between consecutive stages: one box rounded up to 128 bytes.
template <class T> __host__ __device__ constexpr size_t tma_stage_bytes() {
    return ((size_t)TMA_BZ * TMA_BY * TmaBox<T>::BX * sizeof(T) + 127) / 128 * 128;
}

#ifdef __CUDACC__
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(1000)
        : "memory");
    return ok != 0;
}

// Wait for phase `parity` of `bar`; false if it did not complete within the limit.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    for (int i = 0; i < TMA_SPIN_LIMIT; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
#endif

}  // namespace mesh
