// FMA-throughput probe: the FP32 and FP64 roofline denominators of the force
// kernels (their bound is the FMA pipe, not HBM or the tensor cores).  Every
// thread runs 16 independent dependent-FMA chains; the result is stored only
// when an impossible condition holds, so the chains cannot be removed.
#include "f32x2.cuh"
#include "mdgpu_internal.h"

namespace mdgpu {

// The same with paired FP32 instructions (two FMAs per instruction).
__global__ void __launch_bounds__(256) k_fma2_probe(float a, float b, int iters, float *sink)
{
   f2x x[16];
   const f2x A = pk2(a, a), B = pk2(b, b);
#pragma unroll
   for (int k = 0; k < 16; k++) x[k] = pk2(a + (float)(threadIdx.x + k), a - (float)k);
   for (int i = 0; i < iters; i++) {
#pragma unroll
      for (int k = 0; k < 16; k++) x[k] = fma2(x[k], B, A);
   }
   float s = 0.f;
#pragma unroll
   for (int k = 0; k < 16; k++) {
      float lo, hi;
      upk2(x[k], lo, hi);
      s += lo + hi;
   }
   if (s == -1.2345e-30f) sink[threadIdx.x] = s;
}

template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(T a, T b, int iters, T *sink)
{
   T x[16];
#pragma unroll
   for (int k = 0; k < 16; k++) x[k] = a + (T)(threadIdx.x + k);
   for (int i = 0; i < iters; i++) {
#pragma unroll
      for (int k = 0; k < 16; k++) x[k] = x[k] * b + a;
   }
   T s = 0;
#pragma unroll
   for (int k = 0; k < 16; k++) s += x[k];
   if (s == (T)-1.2345e-30) sink[threadIdx.x] = s;
}

}  // namespace mdgpu

// fp64: 0 FP32 (FFMA), 1 FP64 (DFMA), 2 FP32 with paired instructions
extern "C" mdgpu_status mdgpu_fma_peak(int device, int fp64, double *tflops)
{
   using namespace mdgpu;
   if (!tflops) return MDGPU_E_ARG;
   if (cudaSetDevice(device) != cudaSuccess) return MDGPU_E_CUDA;
   int nsm = 0;
   cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
   const int blocks = nsm * 8, threads = 256, iters = fp64 ? 512 : 4096;
   void *sink = nullptr;
   cudaEvent_t e0, e1;
   if (cudaMalloc(&sink, 256 * sizeof(double)) != cudaSuccess) return MDGPU_E_NOMEM;
   cudaEventCreate(&e0);
   cudaEventCreate(&e1);
   float best = 1e30f;
   for (int rep = 0; rep < 4; rep++) {
      cudaEventRecord(e0);
      if (fp64 == 2)
         k_fma2_probe<<<blocks, threads>>>(1.0001f, 0.9999f, iters / 2, (float *)sink);
      else if (fp64)
         k_fma_probe<double><<<blocks, threads>>>(1.0000001, 0.9999999, iters, (double *)sink);
      else
         k_fma_probe<float><<<blocks, threads>>>(1.0001f, 0.9999f, iters, (float *)sink);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms < best) best = ms;
   }
   cudaError_t err = cudaGetLastError();
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   cudaFree(sink);
   if (err != cudaSuccess) return MDGPU_E_CUDA;
   const double flops = 2.0 * 16.0 * iters * (double)blocks * threads;   // (the paired probe: iters/2 x 2)
   *tflops = flops / (best * 1e-3) / 1e12;
   return MDGPU_OK;
}

// ------------------------------------------------------- tensor-core probe
// One CTA computes D = A0 B0^T and then (unless flags & 4) D += A1 B1^T,
// negating A1 if flags & 2, with M = 128, N = n, K = 16 (bf16 operands, or
// fp16 if flags & 8; FP32 accumulation in tensor memory), operands in the
// K-major unswizzled layout
// of tc.cuh.  flags & 1 exchanges the two offset fields of the operand
// descriptors (the operand regions are sized so that both readings stay
// inside them).  It checks the operand layout, the negation flag and the
// rounding of the accumulator against a host computation.
#include "tc.cuh"

namespace mdgpu {

constexpr int TCP_REGION = 32768;   // bytes per operand region

__global__ void __launch_bounds__(128)
k_tc_probe(const uint4 *__restrict__ a0, const uint4 *__restrict__ b0, const uint4 *__restrict__ a1,
           const uint4 *__restrict__ b1, int n, int flags, float *__restrict__ d, int *__restrict__ err)
{
   using namespace tc;
   extern __shared__ __align__(1024) unsigned char sm[];
   __shared__ __align__(8) uint64_t bar;
   __shared__ unsigned int taddr_s;
   const int m = threadIdx.x, w = m >> 5;
   unsigned char *A0 = sm, *A1 = sm + TCP_REGION, *B0 = sm + 2 * TCP_REGION, *B1 = sm + 3 * TCP_REGION;
   for (int i = m; i < 4 * TCP_REGION / 16; i += 128) reinterpret_cast<uint4 *>(sm)[i] = make_uint4(0, 0, 0, 0);
   __syncthreads();
   for (int g = 0; g < 2; g++) {
      const int off = g * 2048 + (m >> 3) * 128 + (m & 7) * 16;
      *reinterpret_cast<uint4 *>(A0 + off) = a0[m * 2 + g];
      *reinterpret_cast<uint4 *>(A1 + off) = a1[m * 2 + g];
      for (int r = m; r < n; r += 128) {
         const int offb = g * (n / 8) * 128 + (r >> 3) * 128 + (r & 7) * 16;
         *reinterpret_cast<uint4 *>(B0 + offb) = b0[r * 2 + g];
         *reinterpret_cast<uint4 *>(B1 + offb) = b1[r * 2 + g];
      }
   }
   fence_async_smem();
   if (m == 0) {
      bar_init(&bar, 1);
      bar_init_fence();
   }
   __syncwarp();
   if (w == 0) tmem_alloc(&taddr_s, 256);
   fence_before_sync();
   __syncthreads();
   fence_after_sync();
   const unsigned int tb = taddr_s;
   if (m == 0) {
      const bool swap = flags & 1;
      auto desc = [&](const unsigned char *p, unsigned int lbo) {
         return swap ? sdesc(saddr(p), 128u, lbo) : sdesc(saddr(p), lbo, 128u);
      };
      const bool h = (flags & 8) != 0;   // fp16 operands instead of bf16
      mma_f16(tb, desc(A0, 2048u), desc(B0, 16u * n), h ? idesc_f16(128, n, false) : idesc_bf16(128, n, false),
              false);
      if (!(flags & 4))
         mma_f16(tb, desc(A1, 2048u), desc(B1, 16u * n),
                 h ? idesc_f16(128, n, (flags & 2) != 0) : idesc_bf16(128, n, (flags & 2) != 0), true);
      mma_commit(&bar);
   }
   __syncwarp();
   const bool ok = __all_sync(0xffffffffu, bar_wait(&bar, 0));
   if (!ok && (m & 31) == 0) atomicOr(err, 1);
   fence_after_sync();
   if (ok)
      for (int c = 0; c < n; c += 16) {
         float v[16];
         tmem_ld16(tb + ((unsigned int)(32 * w) << 16) + (unsigned int)c, v);
         tmem_wait(v);
         for (int j = 0; j < 16; j++) d[m * n + c + j] = v[j];
      }
   fence_before_sync();
   __syncthreads();
   if (w == 0) tmem_dealloc(tb, 256);
}

}  // namespace mdgpu

// a0, a1: 128 x 16 bf16 (row-major); b0, b1: n x 16; d: 128 x n FP32.
// n a multiple of 16 in 16..128.
extern "C" mdgpu_status mdgpu_tc_probe(int device, const unsigned short *a0, const unsigned short *b0,
                                       const unsigned short *a1, const unsigned short *b1, int n, int flags,
                                       float *d)
{
   using namespace mdgpu;
   if (!a0 || !b0 || !a1 || !b1 || !d || n < 16 || n > 128 || n % 16) return MDGPU_E_ARG;
   if (cudaSetDevice(device) != cudaSuccess) return MDGPU_E_CUDA;
   const size_t sa = 128 * 16 * 2, sb = (size_t)n * 16 * 2, sd = 128 * (size_t)n * 4;
   unsigned char *buf = nullptr;
   if (cudaMalloc(&buf, 2 * sa + 2 * sb + sd + 16) != cudaSuccess) return MDGPU_E_NOMEM;
   unsigned char *pa0 = buf, *pa1 = buf + sa, *pb0 = buf + 2 * sa, *pb1 = pb0 + sb, *pd = pb1 + sb;
   int *perr = reinterpret_cast<int *>(pd + sd);
   cudaMemcpy(pa0, a0, sa, cudaMemcpyHostToDevice);
   cudaMemcpy(pa1, a1, sa, cudaMemcpyHostToDevice);
   cudaMemcpy(pb0, b0, sb, cudaMemcpyHostToDevice);
   cudaMemcpy(pb1, b1, sb, cudaMemcpyHostToDevice);
   cudaMemset(perr, 0, sizeof(int));
   cudaFuncSetAttribute(k_tc_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * TCP_REGION);
   k_tc_probe<<<1, 128, 4 * TCP_REGION>>>(reinterpret_cast<const uint4 *>(pa0), reinterpret_cast<const uint4 *>(pb0),
                                          reinterpret_cast<const uint4 *>(pa1), reinterpret_cast<const uint4 *>(pb1),
                                          n, flags, reinterpret_cast<float *>(pd), perr);
   cudaError_t e = cudaDeviceSynchronize();
   int herr = 0;
   if (e == cudaSuccess) e = cudaMemcpy(d, pd, sd, cudaMemcpyDeviceToHost);
   if (e == cudaSuccess) e = cudaMemcpy(&herr, perr, sizeof(int), cudaMemcpyDeviceToHost);
   cudaFree(buf);
   if (e != cudaSuccess) return MDGPU_E_CUDA;
   return herr ? MDGPU_E_CUDA : MDGPU_OK;
}

// ------------------------------------------------ tensor-core issue rate
// One CTA per SM (the shared-memory request keeps it alone); its elected
// thread issues reps MMAs of 128 x n x 16 (bf16, FP32 accumulation) from
// zeroed operands, rotating over nacc accumulators of n columns, then waits
// for their completion: the sustained MMA rate of one issuing thread at
// this shape.
namespace mdgpu {

// issuers > 1: that many warps' lane 0 each issue reps / issuers MMAs into
// their own accumulators (nacc per issuer); small selects 100 KB of shared
// memory (two CTAs per SM, 256 tensor-memory columns each) instead of 200 KB.
__global__ void __launch_bounds__(128, 1) k_tc_rate(int n, int reps, int nacc, int issuers, int ncols, int *__restrict__ err)
{
   using namespace tc;
   extern __shared__ __align__(1024) unsigned char sm[];
   __shared__ __align__(8) uint64_t bar[4];
   __shared__ unsigned int taddr_s;
   const int m = threadIdx.x, w = m >> 5;
   for (int i = m; i < 32768 / 16; i += 128) reinterpret_cast<uint4 *>(sm)[i] = make_uint4(0, 0, 0, 0);
   fence_async_smem();
   if (m == 0) {
      for (int k = 0; k < 4; k++) bar_init(&bar[k], 1);
      bar_init_fence();
   }
   __syncwarp();
   if (w == 0) tmem_alloc(&taddr_s, (unsigned int)ncols);
   fence_before_sync();
   __syncthreads();
   fence_after_sync();
   const unsigned int tb = taddr_s;
   if ((m & 31) == 0 && w < issuers) {
      const unsigned int id = idesc_bf16(128, n, false);
      const uint64_t ad = sdesc(saddr(sm), 2048u, 128u), bd = sdesc(saddr(sm + 8192), 16u * n, 128u);
      const unsigned int base = tb + (unsigned int)(w * nacc * n);
      for (int r = 0; r < reps / issuers; r++) mma_f16(base + (unsigned int)((r % nacc) * n), ad, bd, id, r >= nacc);
      mma_commit(&bar[w]);
   }
   __syncwarp();
   bool ok = true;
   for (int k = 0; k < issuers; k++) ok = ok && bar_wait(&bar[k], 0);
   ok = __all_sync(0xffffffffu, ok);
   if (!ok && (m & 31) == 0) atomicOr(err, 1);
   fence_before_sync();
   __syncthreads();
   if (w == 0) tmem_dealloc(tb, (unsigned int)ncols);
}

}  // namespace mdgpu

// n a multiple of 16 in 16..256, 1 <= issuers <= 4, issuers * nacc * n <=
// 512 (256 with two CTAs per SM), reps >= issuers: bf16 MMA TFLOP/s over
// all SMs (2 * 128 * n * 16 per MMA).
extern "C" mdgpu_status mdgpu_tc_rate(int device, int n, int reps, int nacc, int issuers, int two_per_sm,
                                      double *tflops)
{
   using namespace mdgpu;
   const int ncols = two_per_sm ? 256 : 512;
   if (!tflops || n < 16 || n > 256 || n % 16 || nacc < 1 || issuers < 1 || issuers > 4 ||
       issuers * nacc * n > ncols || reps < issuers)
      return MDGPU_E_ARG;
   if (cudaSetDevice(device) != cudaSuccess) return MDGPU_E_CUDA;
   int nsm = 0;
   cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
   int *perr = nullptr;
   if (cudaMalloc(&perr, sizeof(int)) != cudaSuccess) return MDGPU_E_NOMEM;
   cudaMemset(perr, 0, sizeof(int));
   const int smem = two_per_sm ? 100 * 1024 : 200 * 1024;
   cudaFuncSetAttribute(k_tc_rate, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   const int blocks = two_per_sm ? 2 * nsm : nsm;
   cudaEvent_t e0, e1;
   cudaEventCreate(&e0);
   cudaEventCreate(&e1);
   float best = 1e30f;
   for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0);
      k_tc_rate<<<blocks, 128, smem>>>(n, reps, nacc, issuers, ncols, perr);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms < best) best = ms;
   }
   int herr = 0;
   cudaError_t e = cudaGetLastError();
   if (e == cudaSuccess) e = cudaMemcpy(&herr, perr, sizeof(int), cudaMemcpyDeviceToHost);
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   cudaFree(perr);
   if (e != cudaSuccess || herr) return MDGPU_E_CUDA;
   *tflops = 2.0 * 128.0 * n * 16.0 * (double)(reps / issuers * issuers) * (double)blocks / (best * 1e-3) / 1e12;
   return MDGPU_OK;
}
