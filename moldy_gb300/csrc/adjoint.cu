// Adjoint of the force path: gradients of the potential energy and of a
// force-matching loss with respect to the potential table, the site charges
// and the Ewald alpha.  No counterpart in the reference.
//
// With F_i the site forces the forward path computes (force_calc + ewald,
// src/force.c:1108-1320, src/ewald.c:280-589), F_ref given reference forces
// and w a weight, the loss is L = w sum_i |F_i - F_ref_i|^2.  Its gradient
// is dL/dtheta = sum_i v_i . dF_i/dtheta with v_i = 2 w (F_i - F_ref_i): the
// parameter derivative of G = sum_i v_i . F_i at fixed v, a Hessian-vector
// product of the energy (F = -dE/dx) along v.
//
// Real space (realspace.cu, k_pairs_adj): the stencil walk of the forward
// kernel is run again (no pair list is stored) and each pair's derivatives
// are accumulated per site and per table entry.
//
// Reciprocal space, with the forward's notation (k-sum over the half
// sphere, C + iS = sum_i q_i exp(i k.r_i), coeff_k = c_k, A = c C, B = c S):
//   E_k   = sum_k c_k (C^2 + S^2)/2,          F_i = q_i sum_k k (A s_i - B c_i)
//   dE/dq_i     = sum_k A cos_i + B sin_i
//   dE/dalpha   = sum_k dc/dalpha (C^2 + S^2)/2,  dc/dalpha = c k^2/(2 alpha^3)
//   G           = sum_k c (C Ts - S Tc),   Tc + i Ts = sum_i q_i (k.v_i) e^{ik.r_i}
//   dG/dq_i     = sum_k cos_i Q - sin_i P + (k.v_i)(A sin_i - B cos_i),
//                 P = c Tc, Q = c Ts
//   dG/dalpha   = sum_k dc/dalpha (C Ts - S Tc)
// T is formed from three weighted structure factors V_a = sum_i q_i v_ai
// e^{ik.r_i} (a = x, y, z), T = kx V_x + ky V_y + kz V_z, computed by the
// forward's structure-factor kernel with the weights in place of the
// charges.  The self and sheet terms are added on the host
// (ewald_self_sheet_grad).
//
// With a framework molecule (sites fw0.. N-1) the forward leaves out the
// framework-framework part: E_k = sum_k c (|S|^2 - |S_f|^2)/2 and
// G = sum_k c ((C Ts - S Tc) - (C_f Ts_f - S_f Tc_f)), S = S_n + S_f and
// T = T_n + T_f split into the non-framework (n) and framework (f) sites.
// A non-framework site's dE/dq and dG/dq keep the forms above with the
// whole S and T; a framework site's take S_n and T_n in their place.  Both
// are linear in (A, B, P, Q), so every site is first given the whole-sum
// form and the framework sites then a second pass with the framework's
// coefficients negated, as the forward corrects the framework forces.
#include <cstring>

#include "mdgpu_internal.h"
#include "phase.cuh"

namespace mdgpu {

// kernels of kspace.cu
__global__ void k_sfac32(const int4 *item, const int *item_k0, int nitems, const int4 *ph, const float2 *zp,
                         int N, int chunk, int nk, float2 *part, int *err);
__global__ void k_sfac64(const int4 *item, const int *item_k0, int nitems, const ulonglong2 *pha,
                         const ulonglong2 *phb, const double2 *zz, int N, int chunk, int nk, double2 *part);
__global__ void k_fsum(int n3, int nsplit, const double *fpart, double *force, int accumulate);

__device__ __forceinline__ void kahan(float &s, float &c, float x)
{
   const float y = x - c;
   const float t = s + y;
   c = (t - s) - y;
   s = t;
}

__device__ __forceinline__ double block_sum256(double v, double *sh)
{
   // fixed-shape reduction of a 256-thread block (valid in thread 0)
   sh[threadIdx.x] = v;
   __syncthreads();
   for (int w = 128; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
      __syncthreads();
   }
   const double s = sh[0];
   __syncthreads();
   return s;
}

// Residual weights v = 2 w (F - F_ref) in slot order and the loss partial
// sums w |F - F_ref|^2 per block.
__global__ void __launch_bounds__(256)
k_residual(int N, const int *__restrict__ sorted, const double *__restrict__ force,
           const double *__restrict__ fref, double weight, int mixed, double4 *__restrict__ res64,
           float4 *__restrict__ res32, double *__restrict__ lpart)
{
   __shared__ double sh[256];
   const int p = blockIdx.x * blockDim.x + threadIdx.x;
   double l = 0.0;
   if (p < N) {
      const int i = sorted[p];
      const double dx = force[i] - fref[i], dy = force[N + i] - fref[N + i], dz = force[2 * N + i] - fref[2 * N + i];
      l = weight * (dx * dx + dy * dy + dz * dz);
      const double s = 2.0 * weight;
      if (mixed)
         res32[p] = make_float4((float)(s * dx), (float)(s * dy), (float)(s * dz), 0.f);
      else
         res64[p] = make_double4(s * dx, s * dy, s * dz, 0.0);
   }
   l = block_sum256(l, sh);
   if (threadIdx.x == 0) lpart[blockIdx.x] = l;
}

__global__ void k_sum_to(const double *__restrict__ part, int n, double *__restrict__ dst)
{
   if (threadIdx.x != 0 || blockIdx.x != 0) return;
   double s = 0.0;
   for (int b = 0; b < n; b++) s += part[b];
   *dst = s;
}

// Per-slot phase records with the charge replaced by the weights q v_a.
__global__ void k_adj_channels(int N, int mixed, const int4 *__restrict__ ph32, const float4 *__restrict__ res32,
                               const ulonglong2 *__restrict__ ph64b, const double4 *__restrict__ res64,
                               int4 *__restrict__ phv32, ulonglong2 *__restrict__ phv64)
{
   const int p = blockIdx.x * blockDim.x + threadIdx.x;
   if (p >= N) return;
   if (mixed) {
      const int4 v = ph32[p];
      const float q = __int_as_float(v.w);
      const float4 r = res32[p];
      phv32[p] = make_int4(v.x, v.y, v.z, __float_as_int(q * r.x));
      phv32[N + p] = make_int4(v.x, v.y, v.z, __float_as_int(q * r.y));
      phv32[2 * N + p] = make_int4(v.x, v.y, v.z, __float_as_int(q * r.z));
   } else {
      const ulonglong2 v = ph64b[p];
      const double q = __longlong_as_double((long long)v.y);
      const double4 r = res64[p];
      phv64[p] = make_ulonglong2(v.x, (unsigned long long)__double_as_longlong(q * r.x));
      phv64[N + p] = make_ulonglong2(v.x, (unsigned long long)__double_as_longlong(q * r.y));
      phv64[2 * N + p] = make_ulonglong2(v.x, (unsigned long long)__double_as_longlong(q * r.z));
   }
}

// The framework sites' residual weights in the compacted order of the
// forward's framework records (site fw0 + i at row i; fslot[i] its slot).
__global__ void k_adj_fw_res(int nf, const int *__restrict__ fslot, int mixed, const float4 *__restrict__ res32,
                             const double4 *__restrict__ res64, float4 *__restrict__ resc32,
                             double4 *__restrict__ resc64)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= nf) return;
   const int p = fslot[i];
   if (mixed)
      resc32[i] = res32[p];
   else
      resc64[i] = res64[p];
}

// gq[comp][fw0 + r] += sum over splits of part[split][comp][r], r < nf
__global__ void k_adj_gsum_fw(int nf, int N, int fw0, int nsplit, const double *__restrict__ part,
                              double *__restrict__ gq)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= 2 * nf) return;
   double s = 0.0;
   for (int k = 0; k < nsplit; k++) s += part[(size_t)k * 2 * nf + i];
   const int comp = i / nf, r = i - comp * nf;
   gq[(size_t)comp * N + fw0 + r] += s;
}

// Per k: structure factors summed over chunks in FP64 (fixed order), the
// alpha derivatives, and the per-k coefficients of the per-site pass.  The
// weighted partials pv hold the x, y, z planes; with a framework (fw) p and
// pv hold the non-framework sites' sums, pf and pv's planes 3..5 the
// framework's, and kdf receives the framework coefficients negated.
template <bool MIXED>
__global__ void __launch_bounds__(256)
k_adj_kreduce(int nk, int nchunks, int loss, int fw, const float2 *__restrict__ p32,
              const float2 *__restrict__ pf32, const float2 *__restrict__ pv32, const double2 *__restrict__ p64,
              const double2 *__restrict__ pf64, const double2 *__restrict__ pv64,
              const double *__restrict__ kvec /*[3][nk]*/, const double *__restrict__ coeff, double alpha,
              float4 *__restrict__ kd32, float4 *__restrict__ kdf32, float *__restrict__ kz32,
              double4 *__restrict__ kd64, double4 *__restrict__ kdf64, double *__restrict__ blk)
{
   __shared__ double sh[256];
   const int k = blockIdx.x * blockDim.x + threadIdx.x;
   double ea = 0.0, la = 0.0;
   if (k < nk) {
      // channel 0: S; 1..3: the weighted x, y, z sums; 4..7 the same over
      // the framework sites
      double S[8][2] = {};
      const size_t plane = (size_t)nchunks * nk;
      const int nch = loss ? 4 : 1;
      for (int g = 0; g < (fw ? 2 : 1); g++)
         for (int ch = 0; ch < nch; ch++)
            for (int c = 0; c < nchunks; c++) {
               const size_t o = (size_t)c * nk + k;
               const size_t ov = ch > 0 ? (size_t)(3 * g + ch - 1) * plane + o : 0;
               double x, y;
               if (MIXED) {
                  const float2 v = ch > 0 ? pv32[ov] : g ? pf32[o] : p32[o];
                  x = v.x;
                  y = v.y;
               } else {
                  const double2 v = ch > 0 ? pv64[ov] : g ? pf64[o] : p64[o];
                  x = v.x;
                  y = v.y;
               }
               S[4 * g + ch][0] += x;
               S[4 * g + ch][1] += y;
            }
      const double kx = kvec[k], ky = kvec[nk + k], kz = kvec[2 * nk + k];
      const double cf = coeff[k];
      const double dcf = cf * (kx * kx + ky * ky + kz * kz) / (2.0 * alpha * alpha * alpha);
      const double Cn = S[0][0], Sn = S[0][1], Cf = S[4][0], Sf = S[4][1];
      const double C = Cn + Cf, Sv = Sn + Sf;
      // |S|^2 - |S_f|^2 without the cancellation
      ea = 0.5 * dcf * (Cn * (Cn + Cf + Cf) + Sn * (Sn + Sf + Sf));
      double P = 0.0, Q = 0.0, Pf = 0.0, Qf = 0.0;
      if (loss) {
         const double Tcn = kx * S[1][0] + ky * S[2][0] + kz * S[3][0];
         const double Tsn = kx * S[1][1] + ky * S[2][1] + kz * S[3][1];
         const double Tcf = kx * S[5][0] + ky * S[6][0] + kz * S[7][0];
         const double Tsf = kx * S[5][1] + ky * S[6][1] + kz * S[7][1];
         const double Tc = Tcn + Tcf, Ts = Tsn + Tsf;
         // (C Ts - S Tc) - (C_f Ts_f - S_f Tc_f)
         la = dcf * (Cn * Ts + Cf * Tsn - Sn * Tc - Sf * Tcn);
         P = cf * Tc;
         Q = cf * Ts;
         Pf = -cf * Tcf;
         Qf = -cf * Tsf;
      }
      if (MIXED) {
         kd32[k] = make_float4((float)(cf * C), (float)(cf * Sv), (float)P, (float)Q);
         if (fw) kdf32[k] = make_float4((float)(-cf * Cf), (float)(-cf * Sf), (float)Pf, (float)Qf);
         kz32[k] = (float)kz;
      } else {
         kd64[k] = make_double4(cf * C, cf * Sv, P, Q);
         if (fw) kdf64[k] = make_double4(-cf * Cf, -cf * Sf, Pf, Qf);
      }
   }
   ea = block_sum256(ea, sh);
   la = block_sum256(la, sh);
   if (threadIdx.x == 0) {
      blk[2 * blockIdx.x] = ea;
      blk[2 * blockIdx.x + 1] = la;
   }
}

__global__ void k_adj_kfinal(const double *__restrict__ blk, int nblocks, double *__restrict__ scal)
{
   const int t = threadIdx.x;
   if (t >= 2 || blockIdx.x != 0) return;
   double s = 0.0;
   for (int b = 0; b < nblocks; b++) s += blk[2 * b + t];
   scal[1 + t] = s;
}

constexpr int AD_ITEMS = 64;     // k-vector items per shared-memory tile
constexpr int AD_THREADS = 128;

// Per site (slot), over the items of one split: dE/dq and dG/dq partials,
// written to row sorted[i] of the split's [2][N] block (row i when sorted
// is null: the framework sites' compacted records).
// Mixed form: the forward's phases (32-bit fixed point, polynomial seeds,
// exact per-site tables exp(2 pi i t s_z)), FP32 terms summed in short
// plain runs and Kahan-compensated across runs.
__global__ void __launch_bounds__(AD_THREADS)
k_adj_site32(const int4 *__restrict__ item, const int *__restrict__ item_k0, const float2 *__restrict__ item_kxy,
             int nitems, int nk, int per_split, const float4 *__restrict__ kd, const float *__restrict__ kzv,
             const int4 *__restrict__ ph, const float2 *__restrict__ zz, const float4 *__restrict__ res,
             const int *__restrict__ sorted, int N, int loss, double *__restrict__ gpart)
{
   __shared__ int4 s_it[AD_ITEMS];
   __shared__ float2 s_kxy[AD_ITEMS];
   __shared__ int s_k0[AD_ITEMS];
   __shared__ float4 s_kd[AD_ITEMS * KI];
   __shared__ float s_kz[AD_ITEMS * KI];
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const bool live = i < N;
   const int4 va = live ? ph[i] : make_int4(0, 0, 0, 0);
   float zc[KI], zs[KI];
#pragma unroll
   for (int t = 0; t < KI; t++) {
      // the table holds a site's KI cosines, then its KI sines
      const float *zf = reinterpret_cast<const float *>(zz) + (size_t)i * 2 * KI;
      zc[t] = live ? zf[t] : 1.f;
      zs[t] = live ? zf[KI + t] : 0.f;
   }
   float vx = 0.f, vy = 0.f, vz = 0.f;
   if (live && loss) {
      const float4 v = res[i];
      vx = v.x;
      vy = v.y;
      vz = v.z;
   }
   const int a = blockIdx.y * per_split, b = min(nitems, a + per_split);
   float se = 0.f, ce = 0.f, sl = 0.f, cl = 0.f, pe = 0.f, pl = 0.f;
   int npart = 0;
   for (int tb = a; tb < b; tb += AD_ITEMS) {
      const int nt = min(AD_ITEMS, b - tb);
      const int kb = item_k0[tb];
      const int ke = (tb + nt < nitems) ? item_k0[tb + nt] : nk;
      __syncthreads();
      for (int q = threadIdx.x; q < nt; q += blockDim.x) {
         s_it[q] = item[tb + q];
         s_kxy[q] = item_kxy[tb + q];
         s_k0[q] = item_k0[tb + q] - kb;
      }
      for (int q = threadIdx.x; q < ke - kb; q += blockDim.x) {
         s_kd[q] = kd[kb + q];
         s_kz[q] = kzv[kb + q];
      }
      __syncthreads();
      for (int q = 0; q < nt; q++) {
         const int4 hd = s_it[q];
         const unsigned int p = (unsigned int)hd.x * (unsigned int)va.x + (unsigned int)hd.y * (unsigned int)va.y +
                                (unsigned int)hd.z * (unsigned int)va.z;
         float s0, c0;
         sincos_poly(p, &s0, &c0);
         const float2 kxy = s_kxy[q];
         const float kxv = fmaf(kxy.x, vx, kxy.y * vy);
         const float4 *kq = s_kd + s_k0[q];
         const float *kzq = s_kz + s_k0[q];
#pragma unroll
         for (int t = 0; t < KI; t++) {
            if (t < hd.w) {
               const float4 k4 = kq[t];
               const float cs = c0 * zc[t] - s0 * zs[t];
               const float sn = fmaf(s0, zc[t], c0 * zs[t]);
               pe = fmaf(k4.x, cs, fmaf(k4.y, sn, pe));
               if (loss) {
                  const float kv = fmaf(kzq[t], vz, kxv);
                  const float f = fmaf(k4.x, sn, -k4.y * cs);
                  pl = fmaf(cs, k4.w, fmaf(-sn, k4.z, fmaf(kv, f, pl)));
               }
            }
         }
         if (++npart == 4) {
            kahan(se, ce, pe);
            kahan(sl, cl, pl);
            pe = pl = 0.f;
            npart = 0;
         }
      }
   }
   kahan(se, ce, pe);
   kahan(sl, cl, pl);
   if (live) {
      const int oi = sorted ? sorted[i] : i;
      double *dst = gpart + (size_t)blockIdx.y * 2 * N;
      dst[oi] = (double)se - (double)ce;
      dst[N + oi] = (double)sl - (double)cl;
   }
}

// FP64 form: the forward's 64-bit phases, sincospi seeds and recurrence.
__global__ void __launch_bounds__(AD_THREADS)
k_adj_site64(const int4 *__restrict__ item, const int *__restrict__ item_k0, const double2 *__restrict__ item_kxy,
             int nitems, int nk, int per_split, const double4 *__restrict__ kd, const double *__restrict__ kvec,
             const ulonglong2 *__restrict__ pha, const ulonglong2 *__restrict__ phb,
             const double2 *__restrict__ zz, const double4 *__restrict__ res, const int *__restrict__ sorted,
             int N, int loss, double *__restrict__ gpart)
{
   __shared__ int4 s_it[AD_ITEMS];
   __shared__ double2 s_kxy[AD_ITEMS];
   __shared__ int s_k0[AD_ITEMS];
   __shared__ double4 s_kd[AD_ITEMS * KI];
   __shared__ double s_kz[AD_ITEMS * KI];
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const bool live = i < N;
   const ulonglong2 ua = live ? pha[i] : make_ulonglong2(0, 0);
   const ulonglong2 ub = live ? phb[i] : make_ulonglong2(0, 0);
   const double2 z = live ? zz[i] : make_double2(1.0, 0.0);
   double vx = 0, vy = 0, vz = 0;
   if (live && loss) {
      const double4 v = res[i];
      vx = v.x;
      vy = v.y;
      vz = v.z;
   }
   const int a = blockIdx.y * per_split, b = min(nitems, a + per_split);
   double ge = 0.0, gl = 0.0;
   for (int tb = a; tb < b; tb += AD_ITEMS) {
      const int nt = min(AD_ITEMS, b - tb);
      const int kb = item_k0[tb];
      const int ke = (tb + nt < nitems) ? item_k0[tb + nt] : nk;
      __syncthreads();
      for (int q = threadIdx.x; q < nt; q += blockDim.x) {
         s_it[q] = item[tb + q];
         s_kxy[q] = item_kxy[tb + q];
         s_k0[q] = item_k0[tb + q] - kb;
      }
      for (int q = threadIdx.x; q < ke - kb; q += blockDim.x) {
         s_kd[q] = kd[kb + q];
         s_kz[q] = kvec[2 * (size_t)nk + kb + q];
      }
      __syncthreads();
      for (int q = 0; q < nt; q++) {
         const int4 hd = s_it[q];
         const unsigned long long p = (unsigned long long)(long long)hd.x * ua.x +
                                      (unsigned long long)(long long)hd.y * ua.y +
                                      (unsigned long long)(long long)hd.z * ub.x;
         double sn, cs;
         sincospi(2.0 * ((double)(long long)p * 5.421010862427522e-20), &sn, &cs);
         const double2 kxy = s_kxy[q];
         const double kxv = kxy.x * vx + kxy.y * vy;
         const double4 *kq = s_kd + s_k0[q];
         const double *kzq = s_kz + s_k0[q];
         for (int t = 0; t < hd.w; t++) {
            const double4 k4 = kq[t];
            ge += k4.x * cs + k4.y * sn;
            if (loss) {
               const double kv = kxv + kzq[t] * vz;
               gl += cs * k4.w - sn * k4.z + kv * (k4.x * sn - k4.y * cs);
            }
            const double nc = cs * z.x - sn * z.y;
            sn = sn * z.x + cs * z.y;
            cs = nc;
         }
      }
   }
   if (live) {
      const int oi = sorted ? sorted[i] : i;
      double *dst = gpart + (size_t)blockIdx.y * 2 * N;
      dst[oi] = ge;
      dst[N + oi] = gl;
   }
}

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_check(c, e_, #x); } while (0)

// Reciprocal-space adjoint after a forward ks_launch on the same sites: adds
// the k-space dE/dq, dG/dq into c->ad.gq and writes dE/dalpha, dG/dalpha to
// c->ad.scal[1..2].
static mdgpu_status ks_adjoint(mdgpu_ctx *c, bool loss)
{
   KsDev &d = c->kd;
   AdjDev &a = c->ad;
   const KList &kl = c->kl;
   cudaStream_t st = c->stream;
   const int N = c->nsites, nk = kl.nk, ni = kl.nitems;
   const bool mixed = c->prec == MDGPU_MIXED;
   // framework sites fw0..N-1: the forward has split the charges of the
   // per-slot records into the non-framework (ph) and framework (phf)
   // channels and left the framework sites' records compacted
   const int fw0 = c->fw_site0, nf = N - fw0;
   const bool fw = nf > 0;
   if (nk == 0) {
      CK(cudaMemsetAsync(a.scal.p + 1, 0, 2 * sizeof(double), st));
      return MDGPU_OK;
   }
   // the forward's structure-factor chunks (its partial sums are reused)
   const KsShape sh = ks_shape(N, ni, 1, 1);
   const size_t plane = (size_t)sh.chunks * nk;
   if (loss) {
      const int ngroups = fw ? 2 : 1;   // weighted channels of n (or all) sites, then f sites
      if (mixed) {
         CK(a.phv32.ensure(3 * (size_t)ngroups * N));
         CK(a.partv32.ensure(3 * (size_t)ngroups * plane));
      } else {
         CK(a.phv64.ensure(3 * (size_t)ngroups * N));
         CK(a.partv64.ensure(3 * (size_t)ngroups * plane));
      }
      const dim3 g((ni + 127) / 128, sh.chunks);
      for (int grp = 0; grp < ngroups; grp++) {
         const size_t vo = (size_t)3 * grp * N;
         k_adj_channels<<<(N + 255) / 256, 256, 0, st>>>(N, mixed ? 1 : 0, grp ? d.phf32.p : d.ph32.p, a.res32.p,
                                                         grp ? d.phf64b.p : d.ph64b.p, a.res64.p,
                                                         a.phv32.p + (mixed ? vo : 0),
                                                         a.phv64.p + (mixed ? 0 : vo));
         for (int ch = 0; ch < 3; ch++) {
            const size_t po = (size_t)(3 * grp + ch) * plane;
            if (mixed)
               k_sfac32<<<g, 128, 0, st>>>(d.item.p, d.item_k0.p, ni, a.phv32.p + vo + (size_t)ch * N, d.zp32.p,
                                           N, sh.chunk, nk, a.partv32.p + po, &c->out.p->err);
            else
               k_sfac64<<<g, 128, 0, st>>>(d.item.p, d.item_k0.p, ni, d.ph64a.p, a.phv64.p + vo + (size_t)ch * N,
                                           d.z64.p, N, sh.chunk, nk, a.partv64.p + po);
         }
      }
      CK(cudaGetLastError());
      c->launches += 4 * ngroups;
   }
   const int nbk = (nk + 255) / 256;
   CK(a.blk.ensure(2 * (size_t)nbk));
   if (mixed) {
      CK(a.kadj32.ensure(nk));
      CK(a.kz32.ensure(nk));
      if (fw) CK(a.kadjf32.ensure(nk));
      k_adj_kreduce<true><<<nbk, 256, 0, st>>>(nk, sh.chunks, loss ? 1 : 0, fw ? 1 : 0, d.part32.p,
                                               fw ? d.partf32.p : nullptr, a.partv32.p, nullptr, nullptr,
                                               nullptr, d.kz64.p, d.coeff.p, c->ctl.alpha, a.kadj32.p,
                                               a.kadjf32.p, a.kz32.p, nullptr, nullptr, a.blk.p);
   } else {
      CK(a.kadj64.ensure(nk));
      if (fw) CK(a.kadjf64.ensure(nk));
      k_adj_kreduce<false><<<nbk, 256, 0, st>>>(nk, sh.chunks, loss ? 1 : 0, fw ? 1 : 0, nullptr, nullptr,
                                                nullptr, d.part64.p, fw ? d.partf64.p : nullptr, a.partv64.p,
                                                d.kz64.p, d.coeff.p, c->ctl.alpha, nullptr, nullptr, nullptr,
                                                a.kadj64.p, a.kadjf64.p, a.blk.p);
   }
   k_adj_kfinal<<<1, 32, 0, st>>>(a.blk.p, nbk, a.scal.p);
   CK(a.gkpart.ensure((size_t)sh.splits * 2 * N));
   const dim3 gs((N + AD_THREADS - 1) / AD_THREADS, sh.splits);
   if (mixed)
      k_adj_site32<<<gs, AD_THREADS, 0, st>>>(d.item.p, d.item_k0.p, d.item_kxy32.p, ni, nk, sh.per_split,
                                              a.kadj32.p, a.kz32.p, d.ph32.p, d.zp32.p, a.res32.p, c->rd.sorted.p,
                                              N, loss ? 1 : 0, a.gkpart.p);
   else
      k_adj_site64<<<gs, AD_THREADS, 0, st>>>(d.item.p, d.item_k0.p, d.item_kxy64.p, ni, nk, sh.per_split,
                                              a.kadj64.p, d.kz64.p, d.ph64a.p, d.ph64b.p, d.z64.p, a.res64.p,
                                              c->rd.sorted.p, N, loss ? 1 : 0, a.gkpart.p);
   k_fsum<<<(2 * N + 255) / 256, 256, 0, st>>>(2 * N, sh.splits, a.gkpart.p, a.gq.p, 1);
   CK(cudaGetLastError());
   c->launches += 4;
   if (fw) {
      // the framework sites again, with the framework's coefficients negated
      const KsShape shf = ks_shape(nf, ni, 1, 1);
      CK(a.gkpartf.ensure((size_t)shf.splits * 2 * nf));
      if (loss) {
         if (mixed) CK(a.resc32.ensure(nf)); else CK(a.resc64.ensure(nf));
         k_adj_fw_res<<<(nf + 255) / 256, 256, 0, st>>>(nf, d.fslot.p, mixed ? 1 : 0, a.res32.p, a.res64.p,
                                                        a.resc32.p, a.resc64.p);
         c->launches += 1;
      }
      const dim3 gf((nf + AD_THREADS - 1) / AD_THREADS, shf.splits);
      if (mixed)
         k_adj_site32<<<gf, AD_THREADS, 0, st>>>(d.item.p, d.item_k0.p, d.item_kxy32.p, ni, nk, shf.per_split,
                                                 a.kadjf32.p, a.kz32.p, d.phc32.p, d.zpc32.p, a.resc32.p,
                                                 nullptr, nf, loss ? 1 : 0, a.gkpartf.p);
      else
         k_adj_site64<<<gf, AD_THREADS, 0, st>>>(d.item.p, d.item_k0.p, d.item_kxy64.p, ni, nk, shf.per_split,
                                                 a.kadjf64.p, d.kz64.p, d.pac64.p, d.pbc64.p, d.zc64.p,
                                                 a.resc64.p, nullptr, nf, loss ? 1 : 0, a.gkpartf.p);
      k_adj_gsum_fw<<<(2 * nf + 255) / 256, 256, 0, st>>>(nf, N, fw0, shf.splits, a.gkpartf.p, a.gq.p);
      CK(cudaGetLastError());
      c->launches += 2;
   }
   return MDGPU_OK;
}

// Checks the adjoint's limits for the current system and control record.
static mdgpu_status adjoint_supported(mdgpu_ctx *c)
{
   if (c->max_id > MDGPU_ADJ_MAX_ID)
      return fail(c, MDGPU_E_UNSUPPORTED, "adjoint: more than MDGPU_ADJ_MAX_ID site identifiers");
   if (pot_nparams(c->ptype) == 0)
      return fail(c, MDGPU_E_PTYPE, "KERNEL called with unknown potential type " + std::to_string(c->ptype));
   if (c->ctl.strict_cutoff && !c->ctl.molpbc) {
      // an intramolecular pair beyond the cutoff is clamped in strict mode;
      // the adjoint leaves intramolecular pairs out of the energy terms,
      // which is exact only when none is clamped
      size_t so = 0;
      const double cut2 = c->ctl.cutoff * c->ctl.cutoff;
      for (const auto &sp : c->spec) {
         const double *pf = c->spec_pf.data() + 3 * so;
         for (int i = 0; i < sp.nsites; i++)
            for (int j = i + 1; j < sp.nsites; j++) {
               double d2 = 0.0;
               for (int k = 0; k < 3; k++) d2 += (pf[3 * i + k] - pf[3 * j + k]) * (pf[3 * i + k] - pf[3 * j + k]);
               if (d2 > cut2)
                  return fail(c, MDGPU_E_UNSUPPORTED,
                              "adjoint: a molecule is larger than the strict cutoff");
            }
         so += sp.nsites;
      }
   }
   return MDGPU_OK;
}

static mdgpu_status run_adjoint(mdgpu_ctx *c, const mdgpu_params *prm, const double *h, const double *site_soa,
                                const double *c_of_m, const double *fref, double weight, bool loss,
                                double *value, mdgpu_grad *grad)
{
   mdgpu_status s;
   if (prm && (s = mdgpu_set_params(c, prm)) != MDGPU_OK) return s;
   if ((s = ensure_ready(c, h, true, true)) != MDGPU_OK) return s;
   if ((s = adjoint_supported(c)) != MDGPU_OK) return s;
   cudaStream_t st = c->stream;
   AdjDev &a = c->ad;
   const int N = c->nsites;
   CK(cudaMemcpyAsync(c->site.p, site_soa, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, st));
   if (c->ctl.molpbc) {
      if (!c_of_m) return fail(c, MDGPU_E_ARG, "molecular cutoff needs the centres of mass");
      CK(cudaMemcpyAsync(c->cofm_in.p, c_of_m, 3 * (size_t)c->nmols * sizeof(double), cudaMemcpyHostToDevice, st));
   }
   CK(c->small.ensure(16));
   CK(a.scal.ensure(4));
   CK(cudaMemsetAsync(a.scal.p, 0, 4 * sizeof(double), st));
   // forward: forces and energies, leaving the binned sites, the phases and
   // the structure-factor partials in place for the backward passes
   c->ks_all_sites = true;   // the backward passes read every site's phases
   s = mdgpu_forces_device(c, h, c->site.p, c->cofm_in.p, c->force.p, c->small.p, c->small.p + 2);
   c->ks_all_sites = false;
   if (s) return s;
   const bool mixed = c->prec == MDGPU_MIXED;
   if (mixed) CK(a.res32.ensure(N)); else CK(a.res64.ensure(N));
   if (loss) {
      CK(a.fref.ensure(3 * (size_t)N));
      CK(cudaMemcpyAsync(a.fref.p, fref, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, st));
      const int nb = (N + 255) / 256;
      CK(a.lpart.ensure(nb));
      k_residual<<<nb, 256, 0, st>>>(N, c->rd.sorted.p, c->force.p, a.fref.p, weight, mixed ? 1 : 0, a.res64.p,
                                     a.res32.p, a.lpart.p);
      k_sum_to<<<1, 32, 0, st>>>(a.lpart.p, nb, a.scal.p);
      CK(cudaGetLastError());
      c->launches += 2;
   }
   if ((s = rs_adjoint(c, loss)) != MDGPU_OK) return s;
   const bool ew = c->ctl.alpha > ALPHAMIN;
   if (ew && (s = ks_adjoint(c, loss)) != MDGPU_OK) return s;

   const int np = pot_nparams(c->ptype), M = c->max_id;
   const size_t T = (size_t)M * M * np, nslot = 2 * T + 2;
   std::vector<double> gq(2 * (size_t)N), slots(nslot), small(2), scal(3);
   CK(cudaMemcpyAsync(gq.data(), a.gq.p, gq.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
   CK(cudaMemcpyAsync(slots.data(), a.slots.p, nslot * sizeof(double), cudaMemcpyDeviceToHost, st));
   CK(cudaMemcpyAsync(small.data(), c->small.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
   CK(cudaMemcpyAsync(scal.data(), a.scal.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
   if ((s = sync_out(c)) != MDGPU_OK) return s;

   const size_t off = loss ? T : 0;
   *value = loss ? scal[0] : small[0] + small[1];
   if (!grad) return MDGPU_OK;
   if (grad->potpar) {
      std::memset(grad->potpar, 0, (size_t)M * M * NPOTP * sizeof(double));
      for (size_t t = 0; t < (size_t)M * M; t++)
         for (int k = 0; k < np; k++) grad->potpar[t * NPOTP + k] = slots[off + t * np + k];
   }
   double ga = slots[2 * T + (loss ? 1 : 0)] + (ew ? scal[loss ? 2 : 1] : 0.0);
   if (grad->chg) std::memcpy(grad->chg, gq.data() + (loss ? N : 0), N * sizeof(double));
   if (ew && !loss) {
      std::vector<double> gs(N, 0.0);
      ewald_self_sheet_grad(c->spec, c->spec_pf, c->chg, c->ctl.alpha, c->kl.vol, gs.data(), &ga);
      if (grad->chg)
         for (int i = 0; i < N; i++) grad->chg[i] += gs[i];
   }
   grad->alpha = ga;
   return MDGPU_OK;
}

}  // namespace mdgpu

using namespace mdgpu;

extern "C" mdgpu_status mdgpu_set_params(mdgpu_ctx *c, const mdgpu_params *p)
{
   if (!c || !p) return MDGPU_E_ARG;
   if (!c->have_system) return fail(c, MDGPU_E_ARG, "mdgpu_set_system has not been called");
   if (p->potpar) {
      const size_t n = (size_t)c->max_id * c->max_id * NPOTP;
      if (std::memcmp(p->potpar, c->potpar.data(), n * sizeof(double)) != 0) {
         c->potpar.assign(p->potpar, p->potpar + n);
         c->sys_dirty = true;
         c->have_eintra = false;
         c->gen++;
      }
   }
   if (p->chg && std::memcmp(p->chg, c->chg.data(), c->chg.size() * sizeof(double)) != 0) {
      c->chg.assign(p->chg, p->chg + c->nsites);
      c->sys_dirty = true;
      c->gen++;
      c->have_eintra = false;
      c->have_self = false;
   }
   if (p->alpha > 0.0 && p->alpha != c->ctl.alpha) {
      if (!c->have_control) return fail(c, MDGPU_E_ARG, "mdgpu_set_control has not been called");
      c->ctl.alpha = p->alpha;
      c->gen++;
      c->have_eintra = false;
      c->have_self = false;
   }
   return MDGPU_OK;
}

extern "C" mdgpu_status mdgpu_energy_grad(mdgpu_ctx *c, const mdgpu_params *params, const double *h,
                                          const double *site_soa, const double *c_of_m, double *energy,
                                          mdgpu_grad *grad)
{
   if (!c || !site_soa || !energy) return fail(c, MDGPU_E_ARG, "NULL argument");
   return run_adjoint(c, params, h, site_soa, c_of_m, nullptr, 0.0, false, energy, grad);
}

extern "C" mdgpu_status mdgpu_fm_loss_grad(mdgpu_ctx *c, const mdgpu_params *params, const double *h,
                                           const double *site_soa, const double *c_of_m,
                                           const double *f_ref_soa, double weight, double *loss,
                                           mdgpu_grad *grad)
{
   if (!c || !site_soa || !f_ref_soa || !loss) return fail(c, MDGPU_E_ARG, "NULL argument");
   return run_adjoint(c, params, h, site_soa, c_of_m, f_ref_soa, weight, true, loss, grad);
}
