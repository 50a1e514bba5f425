// Asynchronous bulk-tensor copies (TMA) and shared-memory mbarriers, through
// inline PTX (sm_90 and later; sm_103a here).
//
// A tiled copy moves a box of a tensor described by a CUtensorMap between
// global and shared memory without the issuing thread holding the data:
//   load:  cp.async.bulk.tensor ... mbarrier::complete_tx::bytes: the copy
//          counts its bytes against an mbarrier whose expected transaction
//          count the issuer raised first (mbarrier.arrive.expect_tx); waiters
//          on that barrier phase then see the data;
//   store: cp.async.bulk.tensor ... bulk_group: writers of the shared source
//          fence it into the async proxy (fence.proxy.async.shared::cta)
//          before the issuer starts the copy; cp.async.bulk.wait_group.read N
//          returns once all but the last N committed groups have finished
//          reading shared memory.
// Rules the callers keep: the innermost box coordinate x times the element
// size is a multiple of 16 bytes (coordinates of 64-byte column groups here),
// global strides are multiples of 16 bytes, and stores never start at a
// negative coordinate. A load box reaching past the tensor is filled with
// zeros; a store box is clipped to the tensor.
//
// Every wait on an mbarrier is bounded (WAIT_LIMIT_NS of the global timer):
// it returns false instead of spinning on a phase that never completes, and
// the kernel then records the failure and winds down.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ps {
namespace async {

constexpr unsigned long long WAIT_LIMIT_NS = 1000000000ull;  // 1 s

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Makes the initialisation visible to the async proxy (the copies that
// complete transactions on the barrier); a CTA barrier follows.
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Arrive and raise the phase's expected transaction bytes.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// Wait for the completion of the barrier phase of the given parity; false
// once WAIT_LIMIT_NS have passed (or 2^26 polls) without it.
static __device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    for (uint32_t i = 0; i < (1u << 26); ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 63) == 63 && globaltimer() - t0 > WAIT_LIMIT_NS) return false;
    }
    return false;
}

// Tiled 3D load of one box into shared memory (dst aligned to the swizzle
// span), completing its bytes on bar.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const void *map, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// Contiguous load of `bytes` (a multiple of 16; both addresses 16-byte
// aligned) into shared memory, completing its bytes on bar.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Tiled 3D store of one box from shared memory (x, y, z >= 0).
__device__ __forceinline__ void tma_store_3d(const void *map, int x, int y, int z, uint32_t src)
{
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(map),
                 "r"(x), "r"(y), "r"(z), "r"(src)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// All but the newest N committed store groups have finished reading shared memory.
template <int N> __device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

// Every committed store group has completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Orders this thread's shared-memory writes before later async-proxy reads.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Byte offset of (row, column c8 < 8) of 8-byte elements in a box of 64-byte
// rows written with CU_TENSOR_MAP_SWIZZLE_64B (the 16-byte unit index, bits
// 4-5, XOR address bits 7-8; the box starts on a 512-byte boundary).
__device__ __forceinline__ int swizzle64(int row, int c8)
{
    const int off = row * 64 + c8 * 8;
    return off ^ (((off >> 7) & 3) << 4);
}

// For rows congruent to t modulo 8 the swizzle term depends on t only:
// swizzle64(row, c8) = row * 64 + swizzle64_col(t, c8), a per-thread constant
// plus an offset the compiler folds into the access.
__device__ __forceinline__ int swizzle64_col(int t, int c8) { return (c8 * 8) ^ (((t >> 1) & 3) << 4); }

}  // namespace async
}  // namespace ps
