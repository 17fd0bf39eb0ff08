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
