// Device helpers shared by the reciprocal-space kernels (kspace.cu) and
// their adjoint (adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include "f32x2.cuh"

namespace mdgpu {

// exp(2 pi i p / 2^32) by quadrant reduction of the integer phase and
// polynomials in the reduced phase x in [-1/8, 1/8) revolution:
// sin(2 pi x) = x P(x^2) (degree 9), cos(2 pi x) = Q(x^2) (degree 8), with
// coefficients fitted by (weighted) least squares on Chebyshev nodes and
// rounded to FP32; max abs error about 1e-7 over the interval.
__device__ __forceinline__ void sincos_poly(unsigned int p, float *s, float *c)
{
   const unsigned int qd = (p + 0x20000000u) >> 30;
   const int r = (int)(p - (qd << 30));
   const float x = (float)r * 2.3283064365386963e-10f;   // 2^-32
   const float x2 = x * x;
   float ps = fmaf(fmaf(fmaf(fmaf(41.46983337402344f, x2, -76.69776916503906f), x2, 81.6052017211914f),
                        x2, -41.34170150756836f), x2, 6.2831854820251465f);
   float sn = ps * x;
   float cs = fmaf(fmaf(fmaf(fmaf(59.22028732299805f, x2, -85.4428482055664f), x2, 64.93931579589844f),
                        x2, -19.739208221435547f), x2, 1.0f);
   if (qd & 1u) {
      const float t = sn;
      sn = cs;
      cs = -t;
   }
   if (qd & 2u) {
      sn = -sn;
      cs = -cs;
   }
   *s = sn;
   *c = cs;
}

// sincos_poly for two phases at once: the polynomials run as the two lanes
// of paired FP32 instructions (each lane rounds as the scalar form does, so
// the results are those of two sincos_poly calls), the quadrant reduction
// and its fix-up per lane.  s and c hold (first, second) as f2x pairs.
__device__ __forceinline__ void sincos_poly2(unsigned int pa, unsigned int pb, f2x &s, f2x &c)
{
   const unsigned int qa = (pa + 0x20000000u) >> 30, qb = (pb + 0x20000000u) >> 30;
   const int ra = (int)(pa - (qa << 30)), rb = (int)(pb - (qb << 30));
   const f2x x = pk2((float)ra * 2.3283064365386963e-10f, (float)rb * 2.3283064365386963e-10f);
   const f2x x2 = mul2(x, x);
   const f2x ps = fma2(fma2(fma2(fma2(pk2(41.46983337402344f, 41.46983337402344f), x2,
                                      pk2(-76.69776916503906f, -76.69776916503906f)),
                                 x2, pk2(81.6052017211914f, 81.6052017211914f)),
                            x2, pk2(-41.34170150756836f, -41.34170150756836f)),
                       x2, pk2(6.2831854820251465f, 6.2831854820251465f));
   const f2x sn2 = mul2(ps, x);
   const f2x cs2 = fma2(fma2(fma2(fma2(pk2(59.22028732299805f, 59.22028732299805f), x2,
                                       pk2(-85.4428482055664f, -85.4428482055664f)),
                                  x2, pk2(64.93931579589844f, 64.93931579589844f)),
                             x2, pk2(-19.739208221435547f, -19.739208221435547f)),
                        x2, pk2(1.0f, 1.0f));
   float sa, sb, ca, cb;
   upk2(sn2, sa, sb);
   upk2(cs2, ca, cb);
   if (qa & 1u) {
      const float t = sa;
      sa = ca;
      ca = -t;
   }
   if (qa & 2u) {
      sa = -sa;
      ca = -ca;
   }
   if (qb & 1u) {
      const float t = sb;
      sb = cb;
      cb = -t;
   }
   if (qb & 2u) {
      sb = -sb;
      cb = -cb;
   }
   s = pk2(sa, sb);
   c = pk2(ca, cb);
}

// exp(2 pi i p / 2^32) for a 32-bit phase p, to about 1 FP32 ulp: the top 24
// bits go exactly into sincospif, the low 8 bits (< 2^-23 revolution) are
// added to first order.
__device__ __forceinline__ void sincos_rev32(unsigned int p, float *s, float *c)
{
   float s0, c0;
   sincospif((float)(int)(p & 0xFFFFFF00u) * 4.656612873077393e-10f, &s0, &c0);   // 2^-31
   const float d = (float)(p & 0xFFu) * 1.4629180792671596e-09f;                  // 2 pi / 2^32
   *c = fmaf(-s0, d, c0);
   *s = fmaf(c0, d, s0);
}

}  // namespace mdgpu
