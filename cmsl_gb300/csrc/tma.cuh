// tma.cuh -- Blackwell tensor-memory-access staging: mbarrier-completed
// cp.async.bulk.tensor copies of 2.5D stencil tiles into shared memory.
//
// The first lanes of the block's warps issue a plane's copies (a few boxes
// each), each copy counts its bytes on the stage's mbarrier, and every
// thread waits on that barrier's phase before reading the stage.  Waits are bounded: after TMA_SPIN_LIMIT
// unsuccessful tries the wait records an error in the device error word and
// returns, so a kernel never spins forever.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cmsl {

// A wait gives up after TMA_SPIN_LIMIT tries of at most TMA_SUSPEND_NS each
// (about one second).
constexpr unsigned TMA_SPIN_LIMIT = 1u << 20;
constexpr unsigned TMA_SUSPEND_NS = 1000;
constexpr int TMA_ERR_WAIT = 1;          // bit in the device error word: a tensor-copy wait gave up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the barrier initialisations visible to the async proxy (the tensor
// copies that complete on them).
__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Orders this thread's (and, after a block barrier, the block's) generic
// shared-memory accesses before later async-proxy writes to the same memory.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "n"(TMA_SUSPEND_NS)
        : "memory");
    return ok != 0;
}

// Waits for the phase of `bar` with the given parity; gives up after
// TMA_SPIN_LIMIT tries, setting TMA_ERR_WAIT in *err (false returned).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err)
{
    for (unsigned i = 0; i < TMA_SPIN_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicOr(err, TMA_ERR_WAIT);
    return false;
}

// Tiled tensor copies global -> shared, completing on `bar` (byte count).
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];\n" ::"l"((uint64_t)map) : "memory");
}

// One tensor copy of a plane: which map (4D maps take the field index as
// their fourth coordinate), where in the stage (bytes), and the x / y box
// origin; the plane index (z) is given at issue time.
struct TmaOp {
    const CUtensorMap *map;
    int dst;        // byte offset in the stage
    int x, y, q;    // q < 0: a 3D map
    int pad;
};

// Issues the `n` copies of plane z into the stage at byte address `stage`,
// spread over the first lane of every warp of the block (warp w: copies w,
// w + nw, ...), so no warp carries the whole plane's issue work.  Thread 0
// arms the stage's barrier with the stage's byte count (copies that complete
// before the arming only take the barrier's byte count below zero; the phase
// cannot complete before the arrival).  Every issuing lane first orders the
// block's earlier generic reads of the stage before its async-proxy writes.
__device__ __forceinline__ void tma_issue_plane(const TmaOp *ops, int n, uint32_t stage, int z, uint64_t *bar,
                                                uint32_t bytes)
{
    if ((threadIdx.x & 31) != 0) return;
    const int w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    if (w == 0) mbar_arrive_expect_tx(bar, bytes);
    if (w < n) fence_proxy_async_smem();
    for (int i = w; i < n; i += nw) {
        const TmaOp o = ops[i];
        if (o.q < 0) tma_load_3d(stage + o.dst, o.map, o.x, o.y, z, bar);
        else tma_load_4d(stage + o.dst, o.map, o.x, o.y, z, o.q, bar);
    }
}

}  // namespace cmsl
