// ifx_tma.cuh -- Tensor Memory Accelerator helpers for sm_103a: tiled bulk
// copies of 2-D boxes out of 3-D stacks of planes, global -> shared, completing
// on an mbarrier, with bounded waits.
//
// A tiled copy's innermost coordinate times the element size must be a
// multiple of 16 bytes; callers start every box on that boundary.  Only loads
// are issued (never a store or reduce), and a load box may reach past the
// image on any side: those elements arrive as zeros, and the kernels give the
// ones their windows use the border's values before reading them.
#pragma once
#include <cuda.h>
#include <cstdint>

namespace ifx {

// Encodes a 3-D tensor map over a stack of nz planes of ny rows of nx
// elements of `elt_bytes` (1 or 4), row pitch `pitch_bytes`, plane pitch
// `plane_bytes`, box box_w x box_h x 1.  Returns false when the image does not
// meet the copy engine's rules (16-byte base and pitches, box limits) or the
// driver refuses.
bool tma_encode_3d(CUtensorMap *map, const void *base, int elt_bytes, long long nx, long long ny, long long nz,
                   long long pitch_bytes, long long plane_bytes, int box_w, int box_h);

// Per-device error word for kernels whose bounded waits ran out (0 = none);
// allocated on first use.  tma_error_take reads and clears it.
int *tma_error_word(int device);
int tma_error_take(int device);

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// Waits for phase `parity` of *bar, giving up after `tries` polls.
// Default poll budgets of the kernels' first wait for a tile's copies.
constexpr unsigned kFirstWaitBatch = 1u << 22, kFirstWaitTma = 4096u;
// Testing: every first wait gives up at once (true) or takes its default budget.
cudaError_t set_first_wait_tma(bool force_timeout);
cudaError_t set_first_wait_batch(bool force_timeout);

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t tries = 1u << 22)
{
    for (uint32_t i = 0; i < tries; ++i)
        if (mbar_test(bar, parity)) return true;
    return false;
}

// Waits for phase `parity` of *bar with the suspend-time hint of try_wait
// (the thread sleeps until the phase completes or about `ns` nanoseconds
// pass) instead of polling: waiting warps issue almost nothing.  Gives up
// after `tries` waits (a few seconds at most).
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t *bar, uint32_t parity, uint32_t tries = 4096u,
                                                uint32_t ns = 1000000u)
{
    for (uint32_t i = 0; i < tries; ++i) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity), "r"(ns) : "memory");
        if (ok) return true;
    }
    return false;
}

// Box (x, y, z) of a 3-D `map` (box depth 1) -> shared memory at `dst`
// (128-byte aligned), completing the box's bytes of transaction count on
// *bar.  x * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
                 "[%0], [%1, {%2, %3, %4}], [%5];"
                 :: "r"(smem_addr(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];" :: "l"((uint64_t)map) : "memory");
}

// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA, tensor core) accesses of the same memory.
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

} // namespace ifx
