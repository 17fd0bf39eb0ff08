// Inline-PTX helpers for the sm_100-family tensor-core path (tcgen05) used
// by the reciprocal-space kernels: mbarriers, bulk copies, tensor-memory
// allocation, the bf16 MMA with FP32 accumulation in tensor memory, and
// tensor-memory loads.
//
// Operand layout.  Both operands are K-major and unswizzled: an operand of R
// rows and K columns (bf16) is stored as 8-row x 16-byte "core matrices"
// (row r of a core matrix at byte 16 r); core matrices of consecutive row
// groups are SBO bytes apart and those of consecutive 8-column groups LBO
// bytes apart.  The kernels use [column group][row group][8 rows][16 bytes]
// (SBO = 128, LBO = 128 R / 8), so a warp writing 32 consecutive rows of one
// column group touches 512 contiguous bytes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "f32x2.cuh"

namespace mdgpu {
namespace tc {

constexpr unsigned int WAIT_LIMIT = 1u << 22;   // try_wait rounds before a wait gives up

__device__ __forceinline__ unsigned int saddr(const void *p)
{
   return (unsigned int)__cvta_generic_to_shared(p);
}

// ------------------------------------------------------------ mbarriers
__device__ __forceinline__ void bar_init(uint64_t *bar, unsigned int count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" : : "r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_init_fence()
{
   asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t *bar)
{
   asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" : : "r"(saddr(bar)) : "memory");
}
__device__ __forceinline__ void bar_expect_tx(uint64_t *bar, unsigned int bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" : : "r"(saddr(bar)), "r"(bytes)
                : "memory");
}
// Bounded wait for the phase with the given parity; false if it did not
// complete within WAIT_LIMIT rounds.
__device__ __forceinline__ bool bar_wait(uint64_t *bar, unsigned int parity)
{
   const unsigned int a = saddr(bar);
   for (unsigned int it = 0; it < WAIT_LIMIT; it++) {
      unsigned int done;
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                   "selp.u32 %0, 1, 0, p;\n\t}"
                   : "=r"(done)
                   : "r"(a), "r"(parity)
                   : "memory");
      if (done) return true;
   }
   return false;
}

// Bulk copy global -> shared (TMA engine), completion counted in bytes on bar.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned int bytes, uint64_t *bar)
{
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                :
                : "r"(saddr(dst)), "l"(src), "r"(bytes), "r"(saddr(bar))
                : "memory");
}

// Makes this thread's generic-proxy shared-memory writes visible to the
// async proxy (the tensor cores' operand reads).
__device__ __forceinline__ void fence_async_smem()
{
   asm volatile("fence.proxy.async.shared::cta;" : : : "memory");
}

// ------------------------------------------------------- tensor memory
// Allocation by one full warp; the address lands in *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(unsigned int *dst, unsigned int ncols)
{
   asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" : : "r"(saddr(dst)), "r"(ncols)
                : "memory");
   asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" : : : "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned int taddr, unsigned int ncols)
{
   asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" : : "r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync()
{
   asm volatile("tcgen05.fence::before_thread_sync;" : : : "memory");
}
__device__ __forceinline__ void fence_after_sync()
{
   asm volatile("tcgen05.fence::after_thread_sync;" : : : "memory");
}

// Shared-memory matrix descriptor: K-major, no swizzle.
__device__ __forceinline__ uint64_t sdesc(unsigned int addr, unsigned int lbo, unsigned int sbo)
{
   return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
          ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16 with bf16 A and B, FP32 D, both
// operands K-major; negA negates A.
__host__ __device__ constexpr unsigned int idesc_bf16(int M, int N, bool negA)
{
   return (1u << 4) | (1u << 7) | (1u << 10) | ((negA ? 1u : 0u) << 13) | ((unsigned int)(N >> 3) << 17) |
          ((unsigned int)(M >> 4) << 24);
}

// The same with fp16 A and B.
__host__ __device__ constexpr unsigned int idesc_f16(int M, int N, bool negA)
{
   return (1u << 4) | ((negA ? 1u : 0u) << 13) | ((unsigned int)(N >> 3) << 17) | ((unsigned int)(M >> 4) << 24);
}

// D (tensor memory) = A B^T (+ D if acc), issued by one thread.
// (kind::f16 takes bf16 or fp16 operands, the same type for A and B)
__device__ __forceinline__ void mma_f16(unsigned int d, uint64_t a, uint64_t b, unsigned int idesc, bool acc)
{
   asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                :
                : "r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc ? 1u : 0u)
                : "memory");
}
// The mbarrier receives one arrival when every MMA this thread issued
// before has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" : : "r"(saddr(bar))
                : "memory");
}

// 16 consecutive FP32 columns of this thread's lane (warp w of a warpgroup
// reaches lanes 32 (w % 4) .. + 31).  The values are valid after tmem_wait,
// which takes them as operands so no use can move above it.
__device__ __forceinline__ void tmem_ld16(unsigned int taddr, float (&v)[16])
{
   asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]),
                  "=f"(v[7]), "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]),
                  "=f"(v[14]), "=f"(v[15])
                : "r"(taddr)
                : "memory");
}
__device__ __forceinline__ void tmem_wait(float (&v)[16])
{
   asm volatile("tcgen05.wait::ld.sync.aligned;"
                : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]),
                  "+f"(v[7]), "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]),
                  "+f"(v[14]), "+f"(v[15])
                :
                : "memory");
}
__device__ __forceinline__ void tmem_wait2(float (&v)[16], float (&u)[16])
{
   tmem_wait(v);
   asm volatile(""
                : "+f"(u[0]), "+f"(u[1]), "+f"(u[2]), "+f"(u[3]), "+f"(u[4]), "+f"(u[5]), "+f"(u[6]),
                  "+f"(u[7]), "+f"(u[8]), "+f"(u[9]), "+f"(u[10]), "+f"(u[11]), "+f"(u[12]), "+f"(u[13]),
                  "+f"(u[14]), "+f"(u[15])
                :
                : "memory");
}

// ----------------------------------------------------- bf16 splitting
// The tensor cores' FP32 accumulation rounds toward zero (measured: an
// addend of +1.5 ulp to 1.0 is dropped, -3.5 ulp gives -4), so a long
// accumulation of rounded sums drifts toward zero.  Operands are therefore
// split on fixed grids: for |v| <= 1,
//     hi  = v rounded to a multiple of 2^-7,
//     mid = (v - hi) to a multiple of 2^-15,
//     lo  = (v - hi - mid) to a multiple of 2^-23,
// each an integer of at most 8 bits times a power of two (exact in bf16),
// |v - hi - mid - lo| <= 2^-24.  Products hi*hi are multiples of 2^-14, so
// their sums are exact in FP32 while below 2^10 in magnitude: the large
// accumulator takes no rounding at all, whatever the rounding mode; the
// smaller products (hm, mh, hl, lh, mm) go to a second accumulator whose
// rounding is 2^-8 smaller.  Rounding to a grid is (v + C) - C with C =
// 1.5 2^(23 - bits) (round to nearest even, |v| < C / 2), two values at a
// time as paired FP32 additions.  Packed results: first value in the low half.
__device__ __forceinline__ unsigned int pack_bf16(float lo, float hi)
{
   unsigned int r;
   asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
   return r;
}
__device__ __forceinline__ unsigned int pack_bf16(f2x v)
{
   float a, b;
   upk2(v, a, b);
   return pack_bf16(a, b);
}
__device__ __forceinline__ f2x round_grid(f2x v, float c)
{
   return add2(add2(v, pk2(c, c)), pk2(-c, -c));
}
__device__ __forceinline__ void split3(f2x v, unsigned int &h, unsigned int &m, unsigned int &l)
{
   const f2x m1 = pk2(-1.f, -1.f);
   const f2x vh = round_grid(v, 98304.f);            // 1.5 2^16: grid 2^-7
   const f2x r = fma2(vh, m1, v);                     // v - hi, exact
   const f2x vm = round_grid(r, 384.f);               // 1.5 2^8: grid 2^-15
   const f2x r2 = fma2(vm, m1, r);
   const f2x vl = round_grid(r2, 1.5f);               // grid 2^-23
   h = pack_bf16(vh);
   m = pack_bf16(vm);
   l = pack_bf16(vl);
}
__device__ __forceinline__ void split3(float a, float b, unsigned int &h, unsigned int &m, unsigned int &l)
{
   split3(pk2(a, b), h, m, l);
}

}  // namespace tc
}  // namespace mdgpu
