// Reciprocal-space Ewald sum on the GPU (the work of ewald(),
// src/ewald.c:280-589).
//
// Phases.  With s = h^-1 r the fractional co-ordinate of a site, the phase of
// k-vector (h,k,l) is k.r = 2 pi (h s_x + k s_y + l s_z) (the reference's
// trig tables, src/ewald.c:148-193, are cos/sin of 2 pi s per axis).  Each
// site's s is converted once to 64-bit fixed point u = frac(s) 2^64, so the
// phase of any k-vector, in revolutions, is the exact integer
// h u_x + k u_y + l u_z mod 2^64.  Work items are runs of up to KI
// consecutive l values of one (h,k) column of the reference's k-list: each
// item seeds exp(i k.r) from the exact integer phase and walks l by complex
// multiplication with exp(2 pi i s_z) -- the reference's addition-formula
// recurrence, re-seeded exactly every KI k-vectors so its drift stays
// bounded.  FP64 form: 64-bit phases, sincospi seeds, FP64 recurrence.
// Mixed form: phases rounded to 32 bits, FP32 seeds and recurrence, FP32
// partial sums folded into FP64.
//
// Passes:
//   k_prep     per site: fixed-point phases, q, exp(2 pi i s_z);
//   k_sfac     S(k) = sum_i q_i exp(i k.r_i): one thread per item, the sites
//              of one chunk streamed through shared memory; partial sums per
//              (chunk, k) written out (no atomics);
//   k_kreduce  per k: S(k) over chunks (FP64, fixed order), energy
//              1/2 coeff |S|^2, stress, and A = coeff Re S, B = coeff Im S
//              (src/ewald.c:525-553);
//   k_force    per site: F_i = q_i sum_k k (sin_i A_k - cos_i B_k)
//              (src/ewald.c:557-566), the k-list split over blockIdx.y,
//              per-split FP64 partials;
//   k_fsum     partial forces summed in fixed order into the output.
#include <cstring>

#include "mdgpu_internal.h"
#include "f32x2.cuh"
#include "phase.cuh"

namespace mdgpu {

__device__ __forceinline__ unsigned long long to_fixed64(double s)
{
   // frac(s) * 2^64 for |s| < 2: s * 2^62 is exact in range, rounded to an
   // integer, then scaled by 4 with wrap-around.
   long long t = __double2ll_rn(s * 4611686018427387904.0);
   return (unsigned long long)t << 2;
}

// Per-site records are written in link-cell order (slot i holds site
// sorted[i]; ns is the stride of the site array): the structure-factor
// chunks are then compact regions of the cell, close to neutral, so their
// FP32 partial sums stay small even where the full sum cancels (an ionic
// crystal listed species by species would otherwise give chunks of a
// single charge sign).  mixed: 0 the FP64 records, 1 the FP32 records and
// z tables, 2 the FP32 phases only (the tensor-core passes build their own
// tables).
__global__ void k_prep(int N, int ns, const int *__restrict__ sorted, const double *__restrict__ site,
                       const double *__restrict__ chg, double hi0, double hi1, double hi2,
                       double hi3, double hi4, double hi5, double hi6, double hi7, double hi8,
                       int mixed, int4 *__restrict__ ph32, float2 *__restrict__ z32,
                       float2 *__restrict__ zp32, ulonglong2 *__restrict__ ph64a,
                       ulonglong2 *__restrict__ ph64b, double2 *__restrict__ z64)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;   // slot
   if (i >= N) return;
   const int si = sorted[i];                                // site
   double x = site[si], y = site[ns + si], z = site[2 * (size_t)ns + si];
   double s0 = hi0 * x + hi1 * y + hi2 * z;
   double s1 = hi3 * x + hi4 * y + hi5 * z;
   double s2 = hi6 * x + hi7 * y + hi8 * z;
   unsigned long long ux = to_fixed64(s0), uy = to_fixed64(s1), uz = to_fixed64(s2);
   double q = chg[si];
   if (mixed) {
      // round the 64-bit phases to 32 bits
      unsigned int ux32 = (unsigned int)((ux + 0x80000000ull) >> 32);
      unsigned int uy32 = (unsigned int)((uy + 0x80000000ull) >> 32);
      unsigned int uz32 = (unsigned int)((uz + 0x80000000ull) >> 32);
      ph32[i] = make_int4((int)ux32, (int)uy32, (int)uz32, __float_as_int((float)q));
      if (mixed == 2) return;   // the tensor-core passes build their own z tables
      double sz, cz;
      sincospi(2.0 * ((double)(long long)uz * 5.421010862427522e-20), &sz, &cz);   // 2^-64
      z32[i] = make_float2((float)cz, (float)sz);
      // exp(2 pi i t s_z), t = 0..KI-1, each from its exact integer phase;
      // the site's KI cosines, then its KI sines
      float *zf = reinterpret_cast<float *>(zp32) + (size_t)i * 2 * KI;
      for (int t = 0; t < KI; t++) {
         float st, ct;
         sincos_rev32((unsigned int)t * uz32, &st, &ct);
         zf[t] = ct;
         zf[KI + t] = st;
      }
   } else {
      double sz, cz;
      sincospi(2.0 * ((double)(long long)uz * 5.421010862427522e-20), &sz, &cz);   // 2^-64
      ph64a[i] = make_ulonglong2(ux, uy);
      ph64b[i] = make_ulonglong2(uz, (unsigned long long)__double_as_longlong(q));
      z64[i] = make_double2(cz, sz);
   }
}



// ---------------------------------------------------------------- S(k)
constexpr int SF_TILE = 128;     // sites per shared-memory tile (FP64 pass: half)

// Each site's k-vectors of one item are seed * zp[t] with zp[t] =
// exp(2 pi i t s_z) from the per-site table (k_prep): every term is at most
// two roundings from its exact phase, so no error accumulates along l.  The
// structure factor of a crystal is a near-cancelling sum, and its force
// error grows with the per-site phase error.
//
// The accumulators of neighbouring k (t, t+1) run as the two lanes of paired
// FP32 instructions: the table holds a site's KI cosines and then its KI
// sines, so one 128-bit shared load gives the (t, t+1) and (t+2, t+3) pairs
// with no repacking, and each lane rounds exactly as the scalar form
// fmaf(c, zc, fmaf(-s, zs, acc)) does.
static_assert(KI % 4 == 0, "the structure-factor pass takes k in fours");

// Tiles of a chunk's sites reach shared memory by bulk asynchronous copies
// (the TMA engine's cp.async.bulk, completion counted on an mbarrier) into
// two buffers: tile j+1 is in flight while tile j is summed.  A tile is
// contiguous in global memory (per-slot records and tables), 16-byte
// aligned, and a multiple of 16 bytes long, as the bulk copy requires.
constexpr int SF_TILE32 = 128;              // sites per buffer
constexpr unsigned int SF_WAIT_LIMIT = 1u << 22;   // try_wait rounds before giving up

__device__ __forceinline__ unsigned int smem_addr(const void *p)
{
   return (unsigned int)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned int bytes, unsigned long long *bar)
{
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                :
                : "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
                : "memory");
}

// Bounded wait for the given phase of an mbarrier; false if it did not
// complete (the caller records the error and skips the tile).
__device__ __forceinline__ bool bar_wait(unsigned long long *bar, unsigned int parity)
{
   const unsigned int a = smem_addr(bar);
   for (unsigned int it = 0; it < SF_WAIT_LIMIT; it++) {
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

__global__ void __launch_bounds__(128)
k_sfac32(const int4 *__restrict__ item, const int *__restrict__ item_k0, int nitems,
         const int4 *__restrict__ ph, const float2 *__restrict__ zp, int N, int chunk, int nk,
         float2 *__restrict__ part, int *__restrict__ err)
{
   __shared__ __align__(128) float szp[2][SF_TILE32 * 2 * KI];
   __shared__ __align__(16) int4 sph[2][SF_TILE32];
   __shared__ __align__(8) unsigned long long bar[2];
   const int it = blockIdx.x * blockDim.x + threadIdx.x;
   const int4 hd = it < nitems ? item[it] : make_int4(0, 0, 0, 0);
   const int s0 = blockIdx.y * chunk, s1 = min(N, s0 + chunk);
   const int ntiles = s1 > s0 ? (s1 - s0 + SF_TILE32 - 1) / SF_TILE32 : 0;
   f2x ac[KI / 2], as[KI / 2];   // (t, t+1) pairs of Re and Im S(k)
#pragma unroll
   for (int j = 0; j < KI / 2; j++) ac[j] = as[j] = 0ull;
   const unsigned int H = (unsigned int)hd.x, K = (unsigned int)hd.y, L = (unsigned int)hd.z;
   // one thread issues the copies: a tile's records and its z tables
   auto issue = [&](int j) {
      const int b = j & 1, tb = s0 + j * SF_TILE32, nt = min(SF_TILE32, s1 - tb);
      const unsigned int bytes = (unsigned int)nt * (16u + 8u * KI);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                   :
                   : "r"(smem_addr(&bar[b])), "r"(bytes)
                   : "memory");
      bulk_load(sph[b], ph + tb, (unsigned int)nt * 16u, &bar[b]);
      bulk_load(szp[b], zp + (size_t)tb * KI, (unsigned int)nt * 8u * KI, &bar[b]);
   };
   if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" : : "r"(smem_addr(&bar[0])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" : : "r"(smem_addr(&bar[1])) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
   }
   __syncthreads();
   if (threadIdx.x == 0) {
      if (ntiles > 0) issue(0);
      if (ntiles > 1) issue(1);
   }
   const int nq4 = (hd.w + 3) >> 2;   // k quads of this item (uniform over a warp but at group edges)
   for (int j = 0; j < ntiles; j++) {
      const int b = j & 1, tb = s0 + j * SF_TILE32, nt = min(SF_TILE32, s1 - tb);
      if (bar_wait(&bar[b], (unsigned int)(j >> 1) & 1u)) {
         const float *zb = szp[b];
#pragma unroll 2
         for (int q = 0; q < nt; q++) {
            const int4 v = sph[b][q];
            const unsigned int p = H * (unsigned int)v.x + K * (unsigned int)v.y + L * (unsigned int)v.z;
            float sn, cs;
            sincos_poly(p, &sn, &cs);
            const float qv = __int_as_float(v.w);
            cs *= qv;
            sn *= qv;
            const f2x c2 = pk2(cs, cs), s2 = pk2(sn, sn), ns2 = neg2(s2);
            const ulonglong2 *zc = reinterpret_cast<const ulonglong2 *>(zb + q * 2 * KI);
            const ulonglong2 *zs = zc + KI / 4;
#pragma unroll
            for (int jj = 0; jj < KI / 4; jj++) {
               if (jj < nq4) {
                  const ulonglong2 c = zc[jj], sv = zs[jj];
                  ac[2 * jj] = fma2(c2, c.x, fma2(ns2, sv.x, ac[2 * jj]));
                  as[2 * jj] = fma2(s2, c.x, fma2(c2, sv.x, as[2 * jj]));
                  ac[2 * jj + 1] = fma2(c2, c.y, fma2(ns2, sv.y, ac[2 * jj + 1]));
                  as[2 * jj + 1] = fma2(s2, c.y, fma2(c2, sv.y, as[2 * jj + 1]));
               }
            }
         }
      } else if (threadIdx.x == 0) {
         atomicOr(err, 4);
      }
      __syncthreads();   // every thread is done with buffer b
      if (threadIdx.x == 0 && j + 2 < ntiles) issue(j + 2);
   }
   if (it < nitems) {
      const int k0 = item_k0[it];
      float2 *dst = part + (size_t)blockIdx.y * nk + k0;
#pragma unroll
      for (int j = 0; j < KI / 2; j++) {
         float c0, c1, v0, v1;
         upk2(ac[j], c0, c1);
         upk2(as[j], v0, v1);
         if (2 * j < hd.w) dst[2 * j] = make_float2(c0, v0);
         if (2 * j + 1 < hd.w) dst[2 * j + 1] = make_float2(c1, v1);
      }
   }
}

__global__ void __launch_bounds__(128)
k_sfac64(const int4 *__restrict__ item, const int *__restrict__ item_k0, int nitems,
         const ulonglong2 *__restrict__ pha, const ulonglong2 *__restrict__ phb,
         const double2 *__restrict__ zz, int N, int chunk, int nk, double2 *__restrict__ part)
{
   __shared__ ulonglong2 sa[SF_TILE / 2], sb[SF_TILE / 2];
   __shared__ double2 sz[SF_TILE / 2];
   const int it = blockIdx.x * blockDim.x + threadIdx.x;
   const int4 hd = it < nitems ? item[it] : make_int4(0, 0, 0, 0);
   const int s0 = blockIdx.y * chunk, s1 = min(N, s0 + chunk);
   double ac[KI], as[KI];
#pragma unroll
   for (int t = 0; t < KI; t++) ac[t] = as[t] = 0.0;
   const unsigned long long H = (unsigned long long)(long long)hd.x,
                            K = (unsigned long long)(long long)hd.y,
                            L = (unsigned long long)(long long)hd.z;
   for (int tb = s0; tb < s1; tb += SF_TILE / 2) {
      const int nt = min(SF_TILE / 2, s1 - tb);
      for (int q = threadIdx.x; q < nt; q += blockDim.x) {
         sa[q] = pha[tb + q];
         sb[q] = phb[tb + q];
         sz[q] = zz[tb + q];
      }
      __syncthreads();
      for (int q = 0; q < nt; q++) {
         const ulonglong2 a = sa[q], b = sb[q];
         const double2 z = sz[q];
         const unsigned long long p = H * a.x + K * a.y + L * b.x;
         double sn, cs;
         sincospi(2.0 * ((double)(long long)p * 5.421010862427522e-20), &sn, &cs);
         const double qv = __longlong_as_double((long long)b.y);
         cs *= qv;
         sn *= qv;
#pragma unroll
         for (int t = 0; t < KI; t++) {
            if (t < hd.w) {
               ac[t] += cs;
               as[t] += sn;
            }
            const double nc = cs * z.x - sn * z.y;
            sn = sn * z.x + cs * z.y;
            cs = nc;
         }
      }
      __syncthreads();
   }
   if (it < nitems) {
      const int k0 = item_k0[it];
      double2 *dst = part + (size_t)blockIdx.y * nk + k0;
#pragma unroll
      for (int t = 0; t < KI; t++)
         if (t < hd.w) dst[t] = make_double2(ac[t], as[t]);
   }
}

// ------------------------------------------------- per-k energy and stress
__device__ __forceinline__ double bsum(double v, double *sh)
{
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
   __syncthreads();
   if (lane == 0) sh[w] = v;
   __syncthreads();
   double s = 0.0;
   if (threadIdx.x == 0)
      for (int i = 0; i < nw; i++) s += sh[i];
   return s;
}

// s += x with the rounding error carried in c (Kahan's compensated sum;
// s - c is the running total).
__device__ __forceinline__ void kahan_add(float &s, float &c, float x)
{
   const float y = x - c;
   const float t = s + y;
   c = (t - s) - y;
   s = t;
}

// Per k: S(k) over the structure-factor chunks, then the energy, stress and
// force coefficients.  A block takes KR_K consecutive k (one per lane) and
// spreads the chunks over its KR_W warps (chunks w, w + KR_W, ... in warp w:
// coalesced rows), whose sums warp 0 adds in warp order.
constexpr int KR_K = 32, KR_W = 8;

template <bool MIXED>
__global__ void __launch_bounds__(KR_K * KR_W)
k_kreduce(int nk, int nchunks, const float2 *__restrict__ p32, const double2 *__restrict__ p64,
          const double *__restrict__ kvec /*[3][nk]*/, const double *__restrict__ coeff,
          const double *__restrict__ coeff2, float4 *__restrict__ kd32, double4 *__restrict__ kd64,
          double *__restrict__ blk)
{
   __shared__ double sC[KR_W][KR_K], sS[KR_W][KR_K];
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   const int k = blockIdx.x * KR_K + lane;
   {
      double C = 0.0, S = 0.0;
      if (k < nk) {
         if (MIXED) {
            // FP32 partials: two interleaved Kahan-compensated FP32 sums per
            // lane (the FP64 pipe retires two lanes per clock per SM, a
            // conversion and add per partial was the pass's bound), then FP64
            float c0 = 0.f, e0 = 0.f, s0 = 0.f, f0 = 0.f, c1 = 0.f, e1 = 0.f, s1 = 0.f, f1 = 0.f;
            int c = w;
            for (; c + KR_W < nchunks; c += 2 * KR_W) {
               const float2 v = p32[(size_t)c * nk + k], u = p32[(size_t)(c + KR_W) * nk + k];
               kahan_add(c0, e0, v.x);
               kahan_add(s0, f0, v.y);
               kahan_add(c1, e1, u.x);
               kahan_add(s1, f1, u.y);
            }
            if (c < nchunks) {
               const float2 v = p32[(size_t)c * nk + k];
               kahan_add(c0, e0, v.x);
               kahan_add(s0, f0, v.y);
            }
            C = ((double)c0 - (double)e0) + ((double)c1 - (double)e1);
            S = ((double)s0 - (double)f0) + ((double)s1 - (double)f1);
         } else {
            for (int c = w; c < nchunks; c += KR_W) {
               const double2 v = p64[(size_t)c * nk + k];
               C += v.x;
               S += v.y;
            }
         }
      }
      sC[w][lane] = C;
      sS[w][lane] = S;
   }
   __syncthreads();
   if (w != 0) return;
   double pek = 0, st[6] = {0, 0, 0, 0, 0, 0};
   if (k < nk) {
      double C = 0.0, S = 0.0;
      for (int i = 0; i < KR_W; i++) {
         C += sC[i][lane];
         S += sS[i][lane];
      }
      const double kx = kvec[k], ky = kvec[nk + k], kz = kvec[2 * nk + k];
      const double cf = coeff[k], cf2 = coeff2[k];
      pek = 0.5 * cf * (C * C + S * S);
      st[0] = pek - pek * cf2 * kx * kx;
      st[1] = -(pek * cf2 * kx * ky);
      st[2] = -(pek * cf2 * kx * kz);
      st[3] = pek - pek * cf2 * ky * ky;
      st[4] = -(pek * cf2 * ky * kz);
      st[5] = pek - pek * cf2 * kz * kz;
      const double A = cf * C, B = cf * S;
      if (MIXED)
         kd32[k] = make_float4((float)A, (float)B, (float)kz, 0.f);
      else
         kd64[k] = make_double4(A, B, kz, 0.0);
   }
   // the block's energy and stress: warp 0 holds them all
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) {
      pek += __shfl_down_sync(0xffffffffu, pek, o);
#pragma unroll
      for (int i = 0; i < 6; i++) st[i] += __shfl_down_sync(0xffffffffu, st[i], o);
   }
   if (lane == 0) {
      blk[blockIdx.x * 8] = pek;
      for (int i = 0; i < 6; i++) blk[blockIdx.x * 8 + 1 + i] = st[i];
   }
}

// The k-space energy/stress sum when there are many per-k blocks: block b
// sums the contiguous slice b of the block records (fixed order), and the
// block that finishes last (a counter, reset by it for the next evaluation)
// sums the gridDim.x slice records in a fixed order into out (one SM's FP64
// adds were the cost of a one-level sum).
constexpr int KF_PARTS = 64;   // first-level blocks of the k-space energy/stress sum

__global__ void __launch_bounds__(128) k_kfinal_part(const double *__restrict__ blk, int nblocks,
                                                     double *__restrict__ blk2, unsigned int *__restrict__ count,
                                                     DevOut *__restrict__ out)
{
   __shared__ double sh[4][8];
   __shared__ bool last;
   const int t = threadIdx.x, lane = t & 31, w = t >> 5;
   const int per = (nblocks + gridDim.x - 1) / gridDim.x;
   const int b0 = blockIdx.x * per, b1 = min(nblocks, b0 + per);
   double v[7] = {0, 0, 0, 0, 0, 0, 0};
   for (int b = b0 + t; b < b1; b += blockDim.x)
      for (int k = 0; k < 7; k++) v[k] += blk[b * 8 + k];
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
      for (int k = 0; k < 7; k++) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
   if (lane == 0)
      for (int k = 0; k < 7; k++) sh[w][k] = v[k];
   __syncthreads();
   if (t < 7) {
      blk2[blockIdx.x * 8 + t] = ((sh[0][t] + sh[1][t]) + sh[2][t]) + sh[3][t];
      __threadfence();
   }
   __syncthreads();
   if (t == 0) last = atomicAdd(count, 1u) == gridDim.x - 1;
   __syncthreads();
   if (!last) return;
   __threadfence();
   if (t < 7) {
      double s = 0.0;
      for (int b = 0; b < (int)gridDim.x; b++) s += __ldcg(&blk2[b * 8 + t]);
      if (t == 0)
         out->pe_k = s;
      else
         out->st_k[t - 1] = s;
   }
   if (t == 0) *count = 0u;
}

// Per-block energy/stress partials summed in a fixed order by one block
// (any multiple of 32 threads up to 1024): thread t takes blocks t, t + T,
// ..., then fixed-shape warp and cross-warp trees.
__global__ void __launch_bounds__(1024) k_kfinal(const double *__restrict__ blk, int nblocks, DevOut *out)
{
   __shared__ double sh[32][8];
   const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
   double v[7] = {0, 0, 0, 0, 0, 0, 0};
   for (int b = t; b < nblocks; b += blockDim.x)
      for (int k = 0; k < 7; k++) v[k] += blk[b * 8 + k];
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
      for (int k = 0; k < 7; k++) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
   if (lane == 0)
      for (int k = 0; k < 7; k++) sh[w][k] = v[k];
   __syncthreads();
   if (w != 0) return;
   for (int k = 0; k < 7; k++) v[k] = lane < nw ? sh[lane][k] : 0.0;
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
      for (int k = 0; k < 7; k++) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
   if (lane == 0) {
      out->pe_k = v[0];
      for (int k = 1; k < 7; k++) out->st_k[k - 1] = v[k];
   }
}

// ---------------------------------------------------------------- forces
constexpr int FT_ITEMS = 64;


static_assert(KI == 16, "k_force32 unrolls item counts 1..16");

// One item's k-vectors for two sites (the two lanes): sum over t of
// f = sin(k.r) A - cos(k.r) B and of t f, with exp(i k.r) = seed * zp[t].
template <int W>
__device__ __forceinline__ void item_force(const f2x *zc, const f2x *zs, f2x c0, f2x s0, f2x ns0,
                                           const ulonglong2 *abq, f2x &sf, f2x &st)
{
#pragma unroll
   for (int t = 0; t < W; t++) {
      const ulonglong2 ab = abq[t];
      const f2x cs = fma2(c0, zc[t], mul2(ns0, zs[t]));   // cos of k.r, both sites
      const f2x sn = fma2(s0, zc[t], mul2(c0, zs[t]));    // sin of k.r
      const f2x f = fma2(sn, ab.x, mul2(cs, ab.y));       // sin A - cos B
      sf = add2(sf, f);
      if (t > 0) st = fma2(pk2((float)t, (float)t), f, st);
   }
}

__global__ void __launch_bounds__(FT_THREADS)
k_force32(const int4 *__restrict__ item, const int *__restrict__ item_k0,
          const float2 *__restrict__ item_kxy, int nitems, int nk, int per_split,
          const float4 *__restrict__ kd, const int4 *__restrict__ ph, const float2 *__restrict__ zz,
          const double *__restrict__ chg, const int *__restrict__ sorted, int N, int obase, float dkz,
          double *__restrict__ fpart)
{
   __shared__ int4 s_it[FT_ITEMS];
   __shared__ float2 s_kxy[FT_ITEMS];
   __shared__ int s_k0[FT_ITEMS];
   __shared__ float s_kz0[FT_ITEMS];
   // per k, duplicated for the paired instructions: (A, A, -B, -B).  Along
   // an item kz is linear in t (kz = kz0 + t dkz, the k-list's l step), so
   // the z force needs only sum f and sum t f per item: no kz per k.
   __shared__ ulonglong2 s_ab[FT_ITEMS * KI];
   // two sites per thread, FT_THREADS apart: they share every load of the
   // per-k coefficients and the item bookkeeping, and run as the two lanes
   // of paired FP32 instructions (f32x2)
   const int i0 = blockIdx.x * (2 * FT_THREADS) + threadIdx.x, i1 = i0 + FT_THREADS;
   const bool live0 = i0 < N, live1 = i1 < N;
   const int4 va = live0 ? ph[i0] : make_int4(0, 0, 0, 0);
   const int4 vb = live1 ? ph[i1] : make_int4(0, 0, 0, 0);
   // exp(2 pi i t s_z), t = 0..KI-1, each from its exact integer phase: the
   // k-vectors of an item are seed * zp[t], so per-site phase errors do not
   // accumulate along l (the force multiplies them by |S(k)|, which is of
   // order N q at the Bragg peaks of a crystal).
   f2x zc[KI], zs[KI];
#pragma unroll
   for (int t = 0; t < KI; t++) {
      // the table holds a site's KI cosines, then its KI sines
      const float *za = reinterpret_cast<const float *>(zz) + (size_t)i0 * 2 * KI;
      const float *zb = reinterpret_cast<const float *>(zz) + (size_t)i1 * 2 * KI;
      zc[t] = pk2(live0 ? za[t] : 1.f, live1 ? zb[t] : 1.f);
      zs[t] = pk2(live0 ? za[KI + t] : 0.f, live1 ? zb[KI + t] : 0.f);
   }
   const f2x dkz2 = pk2(dkz, dkz);
   const int a = blockIdx.y * per_split, b = min(nitems, a + per_split);
   // compensated (Kahan) FP32 sums, taken every 8 items of plain FP32
   // partials: no FP64 instruction in the loop (on this part the FP64 pipe
   // retires two lanes per clock per SM; a periodic FP64 fold halved the rate)
   float fxa = 0.f, fya = 0.f, fza = 0.f, exa = 0.f, eya = 0.f, eza = 0.f;
   float fxb = 0.f, fyb = 0.f, fzb = 0.f, exb = 0.f, eyb = 0.f, ezb = 0.f;
   f2x px = 0ull, py = 0ull, pz = 0ull;
   int npart = 0;
   for (int tb = a; tb < b; tb += FT_ITEMS) {
      const int nt = min(FT_ITEMS, b - tb);
      const int kb = item_k0[tb];
      const int ke = (tb + nt < nitems) ? item_k0[tb + nt] : nk;
      __syncthreads();
      for (int q = threadIdx.x; q < nt; q += blockDim.x) {
         s_it[q] = item[tb + q];
         s_kxy[q] = item_kxy[tb + q];
         s_k0[q] = item_k0[tb + q] - kb;
         s_kz0[q] = kd[item_k0[tb + q]].z;
      }
      for (int q = threadIdx.x; q < ke - kb; q += blockDim.x) {
         const float4 k4 = kd[kb + q];
         s_ab[q] = make_ulonglong2(pk2(k4.x, k4.x), pk2(-k4.y, -k4.y));
      }
      __syncthreads();
      for (int q = 0; q < nt; q++) {
         const int4 hd = s_it[q];
         const unsigned int pa = (unsigned int)hd.x * (unsigned int)va.x +
                                 (unsigned int)hd.y * (unsigned int)va.y +
                                 (unsigned int)hd.z * (unsigned int)va.z;
         const unsigned int pb = (unsigned int)hd.x * (unsigned int)vb.x +
                                 (unsigned int)hd.y * (unsigned int)vb.y +
                                 (unsigned int)hd.z * (unsigned int)vb.z;
         float sa0, ca0, sb0, cb0;
         sincos_poly(pa, &sa0, &ca0);
         sincos_poly(pb, &sb0, &cb0);
         const f2x c0 = pk2(ca0, cb0), s0 = pk2(sa0, sb0), ns0 = pk2(-sa0, -sb0);
         f2x sf = 0ull, st = 0ull;   // sum f, sum t f
         const ulonglong2 *abq = s_ab + s_k0[q];
         // the item's count is block-uniform: a loop unrolled for each
         // count, no per-k predicate
         switch (hd.w) {
#define MDGPU_ITEM(W) \
         case W: item_force<W>(zc, zs, c0, s0, ns0, abq, sf, st); break;
            MDGPU_ITEM(16) MDGPU_ITEM(15) MDGPU_ITEM(14) MDGPU_ITEM(13) MDGPU_ITEM(12) MDGPU_ITEM(11)
            MDGPU_ITEM(10) MDGPU_ITEM(9) MDGPU_ITEM(8) MDGPU_ITEM(7) MDGPU_ITEM(6) MDGPU_ITEM(5)
            MDGPU_ITEM(4) MDGPU_ITEM(3) MDGPU_ITEM(2) MDGPU_ITEM(1)
#undef MDGPU_ITEM
         default: break;
         }
         const float2 kxy = s_kxy[q];
         const float kz0 = s_kz0[q];
         px = fma2(pk2(kxy.x, kxy.x), sf, px);
         py = fma2(pk2(kxy.y, kxy.y), sf, py);
         pz = fma2(pk2(kz0, kz0), sf, fma2(dkz2, st, pz));   // sum (kz0 + t dkz) f
         if (++npart == 8) {
            float xa, xb, ya, yb, za, zb;
            upk2(px, xa, xb);
            upk2(py, ya, yb);
            upk2(pz, za, zb);
            kahan_add(fxa, exa, xa);
            kahan_add(fya, eya, ya);
            kahan_add(fza, eza, za);
            kahan_add(fxb, exb, xb);
            kahan_add(fyb, eyb, yb);
            kahan_add(fzb, ezb, zb);
            px = py = pz = 0ull;
            npart = 0;
         }
      }
   }
   {
      float xa, xb, ya, yb, za, zb;
      upk2(px, xa, xb);
      upk2(py, ya, yb);
      upk2(pz, za, zb);
      kahan_add(fxa, exa, xa);
      kahan_add(fya, eya, ya);
      kahan_add(fza, eza, za);
      kahan_add(fxb, exb, xb);
      kahan_add(fyb, eyb, yb);
      kahan_add(fzb, ezb, zb);
   }
   // site oi's partial goes to row oi - obase of [3][N] (obase = 0 except
   // for a subset of sites held compactly)
   // rows by slot (obase < 0) or by site - obase
   double *dst = fpart + (size_t)blockIdx.y * 3 * N;
   if (live0) {
      const int oi = sorted[i0];   // slot i0 holds site oi
      const double q = chg[oi];
      const int r = obase < 0 ? i0 : oi - obase;
      dst[r] = q * ((double)fxa - (double)exa);
      dst[N + r] = q * ((double)fya - (double)eya);
      dst[2 * N + r] = q * ((double)fza - (double)eza);
   }
   if (live1) {
      const int oi = sorted[i1];
      const double q = chg[oi];
      const int r = obase < 0 ? i1 : oi - obase;
      dst[r] = q * ((double)fxb - (double)exb);
      dst[N + r] = q * ((double)fyb - (double)eyb);
      dst[2 * N + r] = q * ((double)fzb - (double)ezb);
   }
}

__global__ void __launch_bounds__(256)
k_force64(const int4 *__restrict__ item, const int *__restrict__ item_k0,
          const double2 *__restrict__ item_kxy, int nitems, int nk, int per_split,
          const double4 *__restrict__ kd, const ulonglong2 *__restrict__ pha,
          const ulonglong2 *__restrict__ phb, const double2 *__restrict__ zz,
          const double *__restrict__ chg, const int *__restrict__ sorted, int N, int obase,
          double *__restrict__ fpart)
{
   __shared__ int4 s_it[FT_ITEMS];
   __shared__ double2 s_kxy[FT_ITEMS];
   __shared__ int s_k0[FT_ITEMS];
   __shared__ double4 s_kd[FT_ITEMS * KI];
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const bool live = i < N;
   const ulonglong2 ua = live ? pha[i] : make_ulonglong2(0, 0);
   const ulonglong2 ub = live ? phb[i] : make_ulonglong2(0, 0);
   const double2 z = live ? zz[i] : make_double2(1.0, 0.0);
   const int a = blockIdx.y * per_split, b = min(nitems, a + per_split);
   double Fx = 0.0, Fy = 0.0, Fz = 0.0;
   for (int tb = a; tb < b; tb += FT_ITEMS) {
      const int nt = min(FT_ITEMS, b - tb);
      const int kb = item_k0[tb];
      const int ke = (tb + nt < nitems) ? item_k0[tb + nt] : nk;
      __syncthreads();
      for (int q = threadIdx.x; q < nt; q += blockDim.x) {
         s_it[q] = item[tb + q];
         s_kxy[q] = item_kxy[tb + q];
         s_k0[q] = item_k0[tb + q] - kb;
      }
      for (int q = threadIdx.x; q < ke - kb; q += blockDim.x) s_kd[q] = kd[kb + q];
      __syncthreads();
      for (int q = 0; q < nt; q++) {
         const int4 hd = s_it[q];
         const unsigned long long p = (unsigned long long)(long long)hd.x * ua.x +
                                      (unsigned long long)(long long)hd.y * ua.y +
                                      (unsigned long long)(long long)hd.z * ub.x;
         double sn, cs;
         sincospi(2.0 * ((double)(long long)p * 5.421010862427522e-20), &sn, &cs);
         double sf = 0.0, skz = 0.0;
         const double4 *kq = s_kd + s_k0[q];
         for (int t = 0; t < hd.w; t++) {
            const double4 k4 = kq[t];
            const double f = sn * k4.x - cs * k4.y;
            sf += f;
            skz += k4.z * f;
            const double nc = cs * z.x - sn * z.y;
            sn = sn * z.x + cs * z.y;
            cs = nc;
         }
         const double2 kxy = s_kxy[q];
         Fx += kxy.x * sf;
         Fy += kxy.y * sf;
         Fz += skz;
      }
   }
   if (live) {
      const int oi = sorted[i];   // slot i holds site oi
      const double q = chg[oi];
      double *dst = fpart + (size_t)blockIdx.y * 3 * N;
      const int r = obase < 0 ? i : oi - obase;   // rows by slot (obase < 0) or by site - obase
      dst[r] = q * Fx;
      dst[N + r] = q * Fy;
      dst[2 * N + r] = q * Fz;
   }
}

// ----------------------------------------------------------- frameworks
// With a framework molecule, ewald() leaves out framework-framework terms
// (src/ewald.c:528-579): the energy is 1/2 coeff (Cn (Cn + 2 Cf) + Sn (Sn +
// 2 Sf)) from the non-framework (n) and framework (f) structure factors;
// non-framework sites feel the whole S(k), framework sites only Sn.  The
// charges are split into the two channels in the per-slot records (the
// framework sites are the last ones, site index >= fw0), each channel gets
// its own structure-factor pass, and the framework sites' forces are
// corrected by a force pass over them alone with the framework
// coefficients negated.
__global__ void k_fw_split(int N, int fw0, const int *__restrict__ sorted, int mixed, int4 *__restrict__ ph32,
                           int4 *__restrict__ phf32, ulonglong2 *__restrict__ ph64b,
                           ulonglong2 *__restrict__ phf64b, int *__restrict__ fslot)
{
   const int p = blockIdx.x * blockDim.x + threadIdx.x;
   if (p >= N) return;
   const int s = sorted[p];
   const bool f = s >= fw0;
   if (f) fslot[s - fw0] = p;
   if (mixed) {
      int4 v = ph32[p], w = v;
      if (f) v.w = __float_as_int(0.f); else w.w = __float_as_int(0.f);
      ph32[p] = v;
      phf32[p] = w;
   } else {
      ulonglong2 v = ph64b[p], w = v;
      if (f) v.y = (unsigned long long)__double_as_longlong(0.0); else w.y = (unsigned long long)__double_as_longlong(0.0);
      ph64b[p] = v;
      phf64b[p] = w;
   }
}

// The framework sites' per-slot records, compacted (site fw0 + i at row i).
__global__ void k_fw_gather(int nf, int fw0, const int *__restrict__ fslot, int mixed, const int4 *__restrict__ ph32,
                            const float2 *__restrict__ zp32, const ulonglong2 *__restrict__ ph64a,
                            const ulonglong2 *__restrict__ ph64b, const double2 *__restrict__ z64,
                            int4 *__restrict__ phc, float2 *__restrict__ zpc, ulonglong2 *__restrict__ pac,
                            ulonglong2 *__restrict__ pbc, double2 *__restrict__ zc, int *__restrict__ sortedc)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= nf) return;
   const int p = fslot[i];
   sortedc[i] = fw0 + i;
   if (mixed) {
      phc[i] = ph32[p];
      for (int t = 0; t < KI; t++) zpc[(size_t)i * KI + t] = zp32[(size_t)p * KI + t];
   } else {
      pac[i] = ph64a[p];
      pbc[i] = ph64b[p];
      zc[i] = z64[p];
   }
}

template <bool MIXED>
__global__ void __launch_bounds__(256)
k_kreduce_fw(int nk, int nchunks, const float2 *__restrict__ pn32, const float2 *__restrict__ pf32,
             const double2 *__restrict__ pn64, const double2 *__restrict__ pf64,
             const double *__restrict__ kvec, const double *__restrict__ coeff,
             const double *__restrict__ coeff2, float4 *__restrict__ kd32, float4 *__restrict__ kdf32,
             double4 *__restrict__ kd64, double4 *__restrict__ kdf64, double *__restrict__ blk)
{
   __shared__ double red[32];
   const int k = blockIdx.x * blockDim.x + threadIdx.x;
   double pek = 0, st[6] = {0, 0, 0, 0, 0, 0};
   if (k < nk) {
      double Cn = 0.0, Sn = 0.0, Cf = 0.0, Sf = 0.0;
      for (int c = 0; c < nchunks; c++) {
         const size_t o = (size_t)c * nk + k;
         if (MIXED) {
            Cn += (double)pn32[o].x;
            Sn += (double)pn32[o].y;
            Cf += (double)pf32[o].x;
            Sf += (double)pf32[o].y;
         } else {
            Cn += pn64[o].x;
            Sn += pn64[o].y;
            Cf += pf64[o].x;
            Sf += pf64[o].y;
         }
      }
      const double kx = kvec[k], ky = kvec[nk + k], kz = kvec[2 * nk + k];
      const double cf = coeff[k], cf2 = coeff2[k];
      pek = 0.5 * cf * (Cn * (Cn + Cf + Cf) + Sn * (Sn + Sf + Sf));
      st[0] = pek - pek * cf2 * kx * kx;
      st[1] = -(pek * cf2 * kx * ky);
      st[2] = -(pek * cf2 * kx * kz);
      st[3] = pek - pek * cf2 * ky * ky;
      st[4] = -(pek * cf2 * ky * kz);
      st[5] = pek - pek * cf2 * kz * kz;
      const double A = cf * (Cn + Cf), B = cf * (Sn + Sf);
      if (MIXED) {
         kd32[k] = make_float4((float)A, (float)B, (float)kz, 0.f);
         kdf32[k] = make_float4((float)(-cf * Cf), (float)(-cf * Sf), (float)kz, 0.f);
      } else {
         kd64[k] = make_double4(A, B, kz, 0.0);
         kdf64[k] = make_double4(-cf * Cf, -cf * Sf, kz, 0.0);
      }
   }
   double s = bsum(pek, red);
   if (threadIdx.x == 0) blk[blockIdx.x * 8] = s;
   for (int i = 0; i < 6; i++) {
      s = bsum(st[i], red);
      if (threadIdx.x == 0) blk[blockIdx.x * 8 + 1 + i] = s;
   }
}

// force[comp][fw0 + i] += sum over splits of fpart[split][comp][i], i < nf
__global__ void k_fsum_fw(int nf, int N, int fw0, int nsplit, const double *__restrict__ fpart,
                          double *__restrict__ force)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= 3 * nf) return;
   double s = 0.0;
   for (int k = 0; k < nsplit; k++) s += fpart[(size_t)k * 3 * nf + i];
   const int comp = i / nf, r = i - comp * nf;
   force[(size_t)comp * N + fw0 + r] += s;
}

__global__ void k_fsum(int n3, int nsplit, const double *__restrict__ fpart, double *__restrict__ force,
                       int accumulate)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n3) return;
   double s = 0.0;
   for (int k = 0; k < nsplit; k++) s += fpart[(size_t)k * n3 + i];
   force[i] = accumulate ? force[i] + s : s;
}

// force[comp][slots[j]] += sum over splits of fpart[split][comp][j], j < n
// (partials by slot of the charged-site list; the other sites get nothing)
__global__ void k_fsum_slots(int n, int N, int nsplit, const double *__restrict__ fpart,
                             const int *__restrict__ slots, double *__restrict__ force)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= 3 * n) return;
   const int comp = i / n, j = i - comp * n;
   double s = 0.0;
   for (int k = 0; k < nsplit; k++) s += fpart[(size_t)k * 3 * n + i];
   force[(size_t)comp * N + slots[j]] += s;
}

// Compaction of the link-cell order to the charged sites: per block of
// 1024 slots an exclusive scan of the flags (charge != 0), the block totals
// scanned by one block, then each charged slot's site written to its place.
__device__ __forceinline__ int block_scan_1024(int v, int *sh)   // exclusive, blockDim 1024
{
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   int x = v;
#pragma unroll
   for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
   }
   if (lane == 31) sh[w] = x;
   __syncthreads();
   if (w == 0) {
      int t = sh[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
         const int y = __shfl_up_sync(0xffffffffu, t, o);
         if (lane >= o) t += y;
      }
      sh[lane] = t;   // inclusive over warps
   }
   __syncthreads();
   return x - v + (w > 0 ? sh[w - 1] : 0);
}

__global__ void __launch_bounds__(1024) k_kflag_scan(int N, const int *__restrict__ sorted,
                                                     const double *__restrict__ chg, int *__restrict__ ex,
                                                     int *__restrict__ bsum)
{
   __shared__ int sh[32];
   const int i = blockIdx.x * 1024 + threadIdx.x;
   const int f = (i < N && chg[sorted[i]] != 0.0) ? 1 : 0;
   const int e = block_scan_1024(f, sh);
   if (i < N) ex[i] = e;
   if (threadIdx.x == 1023) bsum[blockIdx.x] = e + f;
}

__global__ void __launch_bounds__(1024) k_kbsum_scan(int nb, int *__restrict__ bsum)
{
   __shared__ int sh[32];
   __shared__ int carry;
   if (threadIdx.x == 0) carry = 0;
   __syncthreads();
   for (int b0 = 0; b0 < nb; b0 += 1024) {
      const int i = b0 + threadIdx.x;
      const int v = i < nb ? bsum[i] : 0;
      const int e = block_scan_1024(v, sh);
      const int c0 = carry;
      __syncthreads();
      if (i < nb) bsum[i] = c0 + e;
      if (threadIdx.x == 1023) carry = c0 + e + v;
      __syncthreads();
   }
}

__global__ void k_kcompact(int N, const int *__restrict__ sorted, const double *__restrict__ chg,
                           const int *__restrict__ ex, const int *__restrict__ bsum, int *__restrict__ slots)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= N) return;
   const int si = sorted[i];
   if (chg[si] != 0.0) slots[bsum[i >> 10] + ex[i]] = si;
}

// -------------------------------------------------------------- host side
#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_check(c, e_, #x); } while (0)

mdgpu_status ks_prepare(mdgpu_ctx *c)
{
   KsDev &d = c->kd;
   const KList &kl = c->kl;
   cudaStream_t st = c->stream;
   const int N = c->nsites;
   if (!c->kl_uploaded) {
      const int nk = kl.nk, ni = kl.nitems;
      CK(d.item.ensure(ni));
      CK(d.item_k0.ensure(ni + 1));
      CK(d.item_kxy64.ensure(ni));
      CK(d.item_kxy32.ensure(ni));
      CK(d.kz64.ensure(3 * (size_t)nk));
      CK(d.coeff.ensure(nk));
      CK(d.coeff2.ensure(nk));
      CK(d.kdat32.ensure(nk));
      CK(d.kdat64.ensure(nk));
      std::vector<float2> kxy32(ni);
      for (int i = 0; i < ni; i++) kxy32[i] = make_float2((float)kl.item_kxy[i].x, (float)kl.item_kxy[i].y);
      std::vector<double> kv(3 * (size_t)nk);
      for (int i = 0; i < ni; i++)
         for (int t = 0; t < kl.item[i].w; t++) {
            int k = kl.item_k0[i] + t;
            kv[k] = kl.item_kxy[i].x;
            kv[nk + k] = kl.item_kxy[i].y;
            kv[2 * (size_t)nk + k] = kl.kz[k];
         }
      CK(cudaMemcpyAsync(d.item.p, kl.item.data(), ni * sizeof(int4), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.item_k0.p, kl.item_k0.data(), ni * sizeof(int), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.item_kxy64.p, kl.item_kxy.data(), ni * sizeof(double2), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.item_kxy32.p, kxy32.data(), ni * sizeof(float2), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.kz64.p, kv.data(), kv.size() * sizeof(double), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.coeff.p, kl.coeff.data(), nk * sizeof(double), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.coeff2.p, kl.coeff2.data(), nk * sizeof(double), cudaMemcpyHostToDevice, st));
      const size_t nt = kl.tc_item.size();
      CK(d.tc_item.ensure(nt));
      CK(d.tc_k0.ensure(nt));
      CK(d.tc_kxy.ensure(nt));
      CK(d.tc_coef.ensure(nt));
      CK(cudaMemcpyAsync(d.tc_kxy.p, kl.tc_kxy.data(), nt * sizeof(float2), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.tc_item.p, kl.tc_item.data(), nt * sizeof(int4), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.tc_k0.p, kl.tc_k0.data(), nt * sizeof(int4), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
      d.tc_ver++;
      c->kl_uploaded = true;
   }
   if (c->prec == MDGPU_MIXED && c->tc_sfac) {
      CK(ks_tc_init(c->device));
      CK(d.ztab.ensure(ks_tc_ztab_len(N)));
      CK(d.zsite.ensure(ks_tc_zsite_len(N)));
      CK(d.utab.ensure(ks_tc_utab_len((int)kl.tc_item.size())));
   }
   CK(d.ph32.ensure(N + 128));
   if (!d.kcount.p) {   // k_kfinal_part's finished-block counter, zero between evaluations
      CK(d.kcount.ensure(1));
      CK(cudaMemsetAsync(d.kcount.p, 0, sizeof(unsigned int), st));
   }
   CK(d.z32.ensure(N));
   CK(d.zp32.ensure((size_t)N * KI));
   CK(d.ph64a.ensure(N));
   CK(d.ph64b.ensure(N));
   CK(d.z64.ensure(N));
   return MDGPU_OK;
}

// Chunks of the structure-factor pass and k-splits of the force pass, sized
// for about two waves of resident threads; ipt items per thread in the
// former, spt sites per thread in the latter.  Chunks hold 64 sites or more
// (their FP32 partial sums stay short: a crystal's near-cancelling
// structure factor lost accuracy with 256-site chunks), splits 32 items or
// more (below that the per-block set-up, tables and staging, outweighs the
// extra parallelism).
KsShape ks_shape(int N, int nitems, int ipt, int spt)
{
   KsShape s;
   const long long target = 152LL * 2048;          // resident threads on a full GB300
   const long long sf_threads = (nitems + ipt - 1) / ipt, f_threads = (N + spt - 1) / spt;
   long long ch = target / (sf_threads > 0 ? sf_threads : 1);
   long long max_ch = (N + 63) / 64;                // chunks of at least 64 sites
   if (ch < 1) ch = 1;
   if (ch > max_ch) ch = max_ch;
   s.chunk = (int)(((N + ch - 1) / ch + 31) / 32 * 32);
   s.chunks = (N + s.chunk - 1) / s.chunk;
   long long sp = (2 * target) / (f_threads > 0 ? f_threads : 1);
   long long max_sp = (nitems + 31) / 32;           // at least 32 items per block
   if (sp < 1) sp = 1;
   if (sp > max_sp) sp = max_sp;
   if (sp < 1) sp = 1;
   s.per_split = (int)((nitems + sp - 1) / sp);
   s.splits = (nitems + s.per_split - 1) / s.per_split;
   if (s.splits < 1) s.splits = 1;
   return s;
}

mdgpu_status ks_launch(mdgpu_ctx *c, const double *d_site, double *d_force, bool accumulate, cudaEvent_t join)
{
   KsDev &d = c->kd;
   const KList &kl = c->kl;
   cudaStream_t st = c->stream;
   const int N = c->nsites, nk = kl.nk, ni = kl.nitems;
   const bool mixed = c->prec == MDGPU_MIXED;
   DevOut *out = c->out.p;
   if (nk == 0) {
      if (join) CK(cudaStreamWaitEvent(st, join, 0));
      if (!accumulate) CK(cudaMemsetAsync(d_force, 0, 3 * (size_t)N * sizeof(double), st));
      return MDGPU_OK;
   }
   double hinv[9];
   memcpy(hinv, kl.hinv, sizeof hinv);
   const int fw0 = c->fw_site0, nf = N - fw0;   // framework sites, if any
   phase_mark(c, MDGPU_PH_KPREP);
   // The passes run over the charged sites only (a site without charge adds
   // nothing to S(k) and has no k-space force; rigid water's O sites are a
   // quarter of the work), kept in link-cell order -- except with a
   // framework molecule and under the adjoint, which read every site.
   const bool compact = nf <= 0 && !c->ks_all_sites;
   int Nk = N;
   const int *slots = c->rd.sorted.p;
   if (compact) {
      if (c->ncharged_gen != c->gen) {
         int n = 0;
         double qm = 0;
         for (double q : c->chg) {
            n += q != 0.0;
            qm = std::max(qm, std::fabs(q));
         }
         c->ncharged = n;
         c->qmax = qm;
         c->ncharged_gen = c->gen;
      }
      Nk = c->ncharged;
      if (Nk == 0) {
         if (join) CK(cudaStreamWaitEvent(st, join, 0));
         if (!accumulate) CK(cudaMemsetAsync(d_force, 0, 3 * (size_t)N * sizeof(double), st));
         return MDGPU_OK;
      }
      const int nb = (N + 1023) / 1024;
      CK(d.kslots.ensure(N));   // room for every site whatever the device-side count
      CK(d.kscan.ensure(N));
      CK(d.kbsum.ensure(nb));
      k_kflag_scan<<<nb, 1024, 0, st>>>(N, c->rd.sorted.p, c->rd.chg.p, d.kscan.p, d.kbsum.p);
      k_kbsum_scan<<<1, 1024, 0, st>>>(nb, d.kbsum.p);
      k_kcompact<<<(N + 255) / 256, 256, 0, st>>>(N, c->rd.sorted.p, c->rd.chg.p, d.kscan.p, d.kbsum.p,
                                                  d.kslots.p);
      CK(cudaGetLastError());
      c->launches += 3;
      slots = d.kslots.p;
   }
   // mixed form over the charged sites: both passes on the tensor cores
   const bool tc = mixed && compact && c->tc_sfac;
   k_prep<<<(Nk + 255) / 256, 256, 0, st>>>(Nk, N, slots, d_site, c->rd.chg.p, hinv[0], hinv[1], hinv[2],
                                            hinv[3], hinv[4], hinv[5], hinv[6], hinv[7], hinv[8],
                                            tc ? 2 : mixed ? 1 : 0, d.ph32.p, d.z32.p, d.zp32.p, d.ph64a.p,
                                            d.ph64b.p, d.z64.p);
   CK(cudaGetLastError());
   if (tc) {
      CK(d.ztab.ensure(ks_tc_ztab_len(Nk)));
      CK(d.zsite.ensure(ks_tc_zsite_len(Nk)));
      CK(d.utab.ensure(ks_tc_utab_len((int)kl.tc_item.size())));
      ks_tables_tc(st, Nk, d);
      c->launches += 1;
   }
   KsShape sh = mixed ? ks_shape(Nk, ni, 1, 2) : ks_shape(Nk, ni, 1, 1);
   if (nf > 0) {
      CK(d.fslot.ensure(nf));
      if (mixed) CK(d.phf32.ensure(N)); else CK(d.phf64b.ensure(N));
      k_fw_split<<<(N + 255) / 256, 256, 0, st>>>(N, fw0, c->rd.sorted.p, mixed ? 1 : 0, d.ph32.p, d.phf32.p,
                                                  d.ph64b.p, d.phf64b.p, d.fslot.p);
      c->launches += 1;
   }
   phase_mark(c, MDGPU_PH_SFAC);
   const dim3 gs((ni + 127) / 128, sh.chunks);
   if (tc) {
      CK(d.part32.ensure((size_t)ks_tc_chunks(Nk) * nk));
      sh.chunks = ks_sfac_tc(st, Nk, nk, d, (int)(kl.tc_item.size() / 128), c->qmax, &out->err);
   } else if (mixed) {
      CK(d.part32.ensure((size_t)sh.chunks * nk));
      k_sfac32<<<gs, 128, 0, st>>>(d.item.p, d.item_k0.p, ni, d.ph32.p, d.zp32.p, Nk, sh.chunk, nk, d.part32.p,
                                   &out->err);
      if (nf > 0) {
         CK(d.partf32.ensure((size_t)sh.chunks * nk));
         k_sfac32<<<gs, 128, 0, st>>>(d.item.p, d.item_k0.p, ni, d.phf32.p, d.zp32.p, N, sh.chunk, nk,
                                      d.partf32.p, &out->err);
      }
   } else {
      CK(d.part64.ensure((size_t)sh.chunks * nk));
      k_sfac64<<<gs, 128, 0, st>>>(d.item.p, d.item_k0.p, ni, d.ph64a.p, d.ph64b.p, d.z64.p, Nk, sh.chunk,
                                   nk, d.part64.p);
      if (nf > 0) {
         CK(d.partf64.ensure((size_t)sh.chunks * nk));
         k_sfac64<<<gs, 128, 0, st>>>(d.item.p, d.item_k0.p, ni, d.ph64a.p, d.phf64b.p, d.z64.p, N, sh.chunk,
                                      nk, d.partf64.p);
      }
   }
   CK(cudaGetLastError());
   // blocks of the per-k reduction: KR_K k each (the framework form: 256)
   const int nbk = nf > 0 ? (nk + 255) / 256 : (nk + KR_K - 1) / KR_K;
   CK(d.blk.ensure((size_t)nbk * 8));
   phase_mark(c, MDGPU_PH_KREDUCE);
   if (nf > 0) {
      if (mixed) {
         CK(d.kdatf32.ensure(nk));
         k_kreduce_fw<true><<<nbk, 256, 0, st>>>(nk, sh.chunks, d.part32.p, d.partf32.p, nullptr, nullptr,
                                                 d.kz64.p, d.coeff.p, d.coeff2.p, d.kdat32.p, d.kdatf32.p,
                                                 nullptr, nullptr, d.blk.p);
      } else {
         CK(d.kdatf64.ensure(nk));
         k_kreduce_fw<false><<<nbk, 256, 0, st>>>(nk, sh.chunks, nullptr, nullptr, d.part64.p, d.partf64.p,
                                                  d.kz64.p, d.coeff.p, d.coeff2.p, nullptr, nullptr, d.kdat64.p,
                                                  d.kdatf64.p, d.blk.p);
      }
      c->launches += 2;
   } else if (mixed) {
      k_kreduce<true><<<nbk, KR_K * KR_W, 0, st>>>(nk, sh.chunks, d.part32.p, nullptr, d.kz64.p, d.coeff.p,
                                           d.coeff2.p, d.kdat32.p, nullptr, d.blk.p);
   } else {
      k_kreduce<false><<<nbk, KR_K * KR_W, 0, st>>>(nk, sh.chunks, nullptr, d.part64.p, d.kz64.p, d.coeff.p,
                                            d.coeff2.p, nullptr, d.kdat64.p, d.blk.p);
   }
   if (nbk > 4 * KF_PARTS) {
      CK(d.blk2.ensure(8 * (size_t)KF_PARTS));
      k_kfinal_part<<<KF_PARTS, 128, 0, st>>>(d.blk.p, nbk, d.blk2.p, d.kcount.p, out);
   } else {
      k_kfinal<<<1, 512, 0, st>>>(d.blk.p, nbk, out);
   }
   CK(cudaGetLastError());
   if (tc) {
      sh.splits = ks_force_tc_splits(Nk);
      ks_coef_tc(st, d, (int)kl.tc_item.size(), (float)kl.dkz);
      c->launches += 1;
   }
   CK(d.fpart.ensure((size_t)sh.splits * 3 * Nk));
   phase_mark(c, MDGPU_PH_KFORCE);
   dim3 gf((Nk + 255) / 256, sh.splits);
   const int obase = compact ? -1 : 0;   // partial rows by slot of the charged list, or by site
   if (tc) {
      if (c->nsm <= 0) CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device));
      const int nl = ks_force_tc(st, Nk, d, (int)kl.tc_item.size(), c->nsm, c->rd.chg.p, slots, d.fpart.p,
                                 &out->err);
      if (nl < 0) return fail(c, MDGPU_E_NOMEM, "device allocation failed (force-pass work ranges)");
      c->launches += nl - 1;
   } else if (mixed)
      k_force32<<<gf, FT_THREADS, 0, st>>>(d.item.p, d.item_k0.p, d.item_kxy32.p, ni, nk, sh.per_split,
                                           d.kdat32.p, d.ph32.p, d.zp32.p, c->rd.chg.p, slots, Nk, obase,
                                           (float)kl.dkz, d.fpart.p);
   else
      k_force64<<<gf, 256, 0, st>>>(d.item.p, d.item_k0.p, d.item_kxy64.p, ni, nk, sh.per_split,
                                    d.kdat64.p, d.ph64a.p, d.ph64b.p, d.z64.p, c->rd.chg.p, slots, Nk, obase,
                                    d.fpart.p);
   CK(cudaGetLastError());
   phase_mark(c, MDGPU_PH_FINAL);
   if (join) CK(cudaStreamWaitEvent(st, join, 0));
   if (compact) {
      if (!accumulate) CK(cudaMemsetAsync(d_force, 0, 3 * (size_t)N * sizeof(double), st));
      k_fsum_slots<<<(3 * Nk + 255) / 256, 256, 0, st>>>(Nk, N, sh.splits, d.fpart.p, slots, d_force);
   } else {
      k_fsum<<<(3 * N + 255) / 256, 256, 0, st>>>(3 * N, sh.splits, d.fpart.p, d_force, accumulate ? 1 : 0);
   }
   CK(cudaGetLastError());
   if (nf > 0) {
      // the framework sites' framework-framework k-space forces, taken off
      const KsShape shf = ks_shape(nf, ni, 1, mixed ? 2 : 1);
      CK(d.sortedc.ensure(nf));
      CK(d.fpartf.ensure((size_t)shf.splits * 3 * nf));
      if (mixed) {
         CK(d.phc32.ensure(nf));
         CK(d.zpc32.ensure((size_t)nf * KI));
      } else {
         CK(d.pac64.ensure(nf));
         CK(d.pbc64.ensure(nf));
         CK(d.zc64.ensure(nf));
      }
      k_fw_gather<<<(nf + 255) / 256, 256, 0, st>>>(nf, fw0, d.fslot.p, mixed ? 1 : 0, d.ph32.p, d.zp32.p,
                                                    d.ph64a.p, d.ph64b.p, d.z64.p, d.phc32.p, d.zpc32.p,
                                                    d.pac64.p, d.pbc64.p, d.zc64.p, d.sortedc.p);
      const dim3 gff((nf + 255) / 256, shf.splits);
      if (mixed)
         k_force32<<<gff, FT_THREADS, 0, st>>>(d.item.p, d.item_k0.p, d.item_kxy32.p, ni, nk, shf.per_split,
                                               d.kdatf32.p, d.phc32.p, d.zpc32.p, c->rd.chg.p, d.sortedc.p, nf,
                                               fw0, (float)kl.dkz, d.fpartf.p);
      else
         k_force64<<<gff, 256, 0, st>>>(d.item.p, d.item_k0.p, d.item_kxy64.p, ni, nk, shf.per_split,
                                        d.kdatf64.p, d.pac64.p, d.pbc64.p, d.zc64.p, c->rd.chg.p, d.sortedc.p, nf,
                                        fw0, d.fpartf.p);
      k_fsum_fw<<<(3 * nf + 255) / 256, 256, 0, st>>>(nf, N, fw0, shf.splits, d.fpartf.p, d_force);
      CK(cudaGetLastError());
      c->launches += 3;
   }
   c->launches += 6;
   return MDGPU_OK;
}

}  // namespace mdgpu
