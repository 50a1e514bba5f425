// Tensor memory (TMEM) as per-thread storage, through tcgen05 inline PTX
// (sm_100a family: sm_103a here).
//
// Every SM has 128 lanes x 512 columns of 32-bit TMEM. A CTA allocates a
// power-of-two number of columns (32..512) with tcgen05.alloc, executed by one
// whole warp, which writes the base address to shared memory. Warp w of the
// CTA reaches lanes 32 (w mod 4) .. 32 (w mod 4) + 31 only; with the 32x32b
// shape thread i of the warp reads and writes lane 32 (w mod 4) + i, so each
// thread owns a private row of columns. Warps w and w + 4 share lanes and use
// disjoint column ranges.
//
// tcgen05.ld and tcgen05.st are asynchronous: tcgen05.wait::ld must come
// before the loaded registers are used (the wait below takes the registers as
// in-out operands, so the compiler cannot hoist a use above it), and
// tcgen05.wait::st before a later load of the same columns.
//
// An allocation blocks while the SM's free columns are fewer than requested;
// the launcher keeps (resident CTAs per SM) x (columns per CTA) <= 512 so
// that it never waits.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ps {
namespace tmem {

constexpr int COLUMNS_PER_SM = 512;

__device__ __forceinline__ void alloc(uint32_t *smem_slot, int ncols)
{
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(smem_slot);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void relinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void dealloc(uint32_t taddr, int ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Store 16 consecutive columns of this thread's lane.
__device__ __forceinline__ void st16(uint32_t taddr, const uint32_t (&v)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}

// Load 16 consecutive columns of this thread's lane (valid after wait_ld16).
__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t (&v)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}

// Wait for this thread's outstanding loads; the registers pass through the
// wait so that their uses stay behind it.
__device__ __forceinline__ void wait_ld16(uint32_t (&v)[16])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                   "+r"(v[15])
                 :
                 : "memory");
}

__device__ __forceinline__ void wait_ld16x2(uint32_t (&a)[16], uint32_t (&b)[16])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7]),
                   "+r"(a[8]), "+r"(a[9]), "+r"(a[10]), "+r"(a[11]), "+r"(a[12]), "+r"(a[13]), "+r"(a[14]),
                   "+r"(a[15]), "+r"(b[0]), "+r"(b[1]), "+r"(b[2]), "+r"(b[3]), "+r"(b[4]), "+r"(b[5]), "+r"(b[6]),
                   "+r"(b[7]), "+r"(b[8]), "+r"(b[9]), "+r"(b[10]), "+r"(b[11]), "+r"(b[12]), "+r"(b[13]),
                   "+r"(b[14]), "+r"(b[15])
                 :
                 : "memory");
}

// Lane field of this warp's TMEM addresses.
__device__ __forceinline__ uint32_t lane_base(int warp) { return (uint32_t)(32 * (warp & 3)) << 16; }

}  // namespace tmem
}  // namespace ps
