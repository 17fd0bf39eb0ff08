// Packed FP32 pairs for the sm_100-family paired FP32 instructions
// (PTX fma/mul/add with the .f32x2 type): one instruction performs the same
// operation on two FP32 lanes held in a 64-bit register, halving the issue
// slots of the FMA-bound inner loops.  Each lane is rounded as the scalar
// instruction would round it.
#pragma once
#include <cuda_runtime.h>

namespace mdgpu {

typedef unsigned long long f2x;   // two FP32 values: .x in the low word

__device__ __forceinline__ f2x pk2(float lo, float hi)
{
   f2x r;
   asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
   return r;
}
__device__ __forceinline__ void upk2(f2x r, float &lo, float &hi)
{
   asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r));
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c)   // a * b + c
{
   f2x d;
   asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
   return d;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b)
{
   f2x d;
   asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
   return d;
}
__device__ __forceinline__ f2x add2(f2x a, f2x b)
{
   f2x d;
   asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
   return d;
}
__device__ __forceinline__ f2x neg2(f2x a)   // flips both sign bits
{
   return a ^ 0x8000000080000000ull;
}

}  // namespace mdgpu
