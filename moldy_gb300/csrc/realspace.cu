// Real-space link-cell forces on the GPU (the work of force_calc,
// src/force.c:1108-1320, and kernel(), src/kernel.c:157-463).
//
// Pipeline, all on one stream:
//   1. k_bin        FP64 binning of every site (or molecule centre of mass in
//                   molecular-cutoff mode) with the reference's arithmetic and
//                   edge fix-ups (cellbin, src/force.c:119-137);
//   2. scan         cell counts -> cell starts (3-kernel block scan);
//   3. k_scatter +  sites placed cell by cell, then each cell's members put
//      k_cellsort   in ascending site order (deterministic layout);
//   4. k_gather     per-slot records: FP64 (x,y,z,q), or FP32 co-ordinates
//                   relative to the cell origin plus q, and (site id, molecule);
//   5. k_pairs      one warp per site walks the full neighbour-cell stencil
//                   (the reference's half-space list and its mirror) and
//                   evaluates every candidate pair the reference evaluates,
//                   accumulating the force on its own site only; energy and
//                   virial take half of each evaluation.  No atomics on forces.
//   6. k_reduce_rs  per-block energy/virial partials summed in fixed order.
//
// The pair set is the reference's exactly: every site pair of a cell and of
// each stencil cell, with no per-pair cutoff in lazy mode and r^2 clamped to
// 1e4 rc^2 in strict mode (src/force.c:951-954).  In FP64 form r and r^2 are
// formed with the reference's operation order and no fused multiply-adds, so
// the clamp and the too-close test decide exactly as the reference does.  In
// mixed form r is formed in FP32 from cell-relative co-ordinates and an
// (hi, lo) pair of the exact cell-offset vector; decisions within a narrow
// band of the threshold are re-made in FP64 from the original co-ordinates.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "mdgpu_internal.h"

namespace mdgpu {

struct RsParams {
   int nsites, nent, nx, ny, nz, ncells, nfull, max_id, molpbc, strict, ptype, pot_in_smem;
   // the framework molecule (-1: none), its first site, and the number of
   // molecule entities binned by centre of mass in molecular-cutoff mode
   // (the framework's sites are binned one by one, src/force.c:458-470)
   int fw_mol, fw_site0, nmol_ent;
   int ncols;             // stencil columns (k_pairs_col)
   double hinv[9];
   double h[9];
   double rn[3];          // 1/nx, 1/ny, 1/nz
   double reloc[27][3];
   double cut2, cut100, alpha, norm;
   float cut2f, bandf, alphaf, normf;
};

// Launch parameters of the real-space adjoint.
struct AdjParams {
   int loss;              // nonzero: residual weights given, loss terms wanted
   unsigned type_mask;    // bit b set: some site has identifier b
   int nslot;             // 2 max_id^2 NP + 2 gradient slots
};

// ---------------------------------------------------------------- binning
__device__ __forceinline__ int cellbin_dev(double s, int n, double fn, int *bad)
{
   const double eps = 8.0 * 2.220446049250313e-16;   // 8 * precision(), force.c:437
   if (s < -0.5 + eps || s >= 0.5 - eps) {
      if (s < -0.5 + eps && s >= -0.5 - eps)
         s = -0.5;
      else if (s >= 0.5 - eps && s <= 0.5 + eps)
         s = 0.5 - eps;
      else
         *bad = 1;
   }
   int ib = (int)floor(__dmul_rn(__dadd_rn(s, 0.5), fn));
   if (ib >= n || ib < 0) {
      *bad = 1;
      ib = ib < 0 ? 0 : n - 1;
   }
   return ib;
}

// s = hinv . x with mat_vec_mul's order (src/matrix.c:54-56), no FMA.
__device__ __forceinline__ double hrow(const double *m, double a0, double a1, double a2)
{
   return __dadd_rn(__dadd_rn(__dmul_rn(m[0], a0), __dmul_rn(m[1], a1)), __dmul_rn(m[2], a2));
}

__global__ void k_bin(RsParams P, const double *__restrict__ site, const double *__restrict__ cofm,
                      const int *__restrict__ mol_first, const int *__restrict__ mol_n,
                      int *__restrict__ cell_of, int *__restrict__ cell_count, DevOut *out)
{
   int e = blockIdx.x * blockDim.x + threadIdx.x;
   if (e >= P.nent) return;
   int bad = 0;
   double s0, s1, s2;
   const bool by_site = !P.molpbc || e >= P.nmol_ent;
   const int si = !P.molpbc ? e : P.fw_site0 + (e - P.nmol_ent);   // site of a site entity
   if (by_site) {
      const int N = P.nsites;
      double x = site[si], y = site[N + si], z = site[2 * N + si];
      s0 = hrow(P.hinv, x, y, z);
      s1 = hrow(P.hinv + 3, x, y, z);
      s2 = hrow(P.hinv + 6, x, y, z);
   } else {
      s0 = cofm[3 * e];
      s1 = cofm[3 * e + 1];
      s2 = cofm[3 * e + 2];
   }
   int cx = cellbin_dev(s0, P.nx, (double)P.nx, &bad);
   int cy = cellbin_dev(s1, P.ny, (double)P.ny, &bad);
   int cz = cellbin_dev(s2, P.nz, (double)P.nz, &bad);
   int c = cz + P.nz * (cy + P.ny * cx);
   if (bad) atomicOr(&out->err, 1);
   if (by_site) {
      cell_of[si] = c;
      atomicAdd(&cell_count[c], 1);
   } else {
      int f = mol_first[e], n = mol_n[e];
      for (int s = 0; s < n; s++) cell_of[f + s] = c;
      atomicAdd(&cell_count[c], n);
   }
}

// ---------------------------------------------------------- exclusive scan
__device__ __forceinline__ int warp_incl_scan(int v)
{
   const int lane = threadIdx.x & 31;
#pragma unroll
   for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
   }
   return v;
}

// Block-wide exclusive scan of 1024 values.
__device__ void block_excl_scan(int v, int *out_excl)
{
   __shared__ int wsum[32];
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   int inc = warp_incl_scan(v);
   if (lane == 31) wsum[w] = inc;
   __syncthreads();
   if (w == 0) {
      int s = wsum[lane];
      int si = warp_incl_scan(s);
      wsum[lane] = si - s;
   }
   __syncthreads();
   *out_excl = inc - v + wsum[w];
   __syncthreads();
}

__global__ void __launch_bounds__(1024) k_scan_blocks(const int *__restrict__ in, int *__restrict__ out,
                                                      int *__restrict__ bsum, int n)
{
   int i = blockIdx.x * 1024 + threadIdx.x;
   int v = i < n ? in[i] : 0, ex;
   __shared__ int last;
   block_excl_scan(v, &ex);
   if (threadIdx.x == 1023) last = ex + v;
   __syncthreads();
   if (i < n) out[i] = ex;
   if (threadIdx.x == 0) bsum[blockIdx.x] = last;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int *__restrict__ bsum, int nb, int *__restrict__ total)
{
   __shared__ int carry_s;
   if (threadIdx.x == 0) carry_s = 0;
   __syncthreads();
   for (int b0 = 0; b0 < nb; b0 += 1024) {
      int i = b0 + threadIdx.x;
      int v = i < nb ? bsum[i] : 0, ex;
      __shared__ int last;
      block_excl_scan(v, &ex);
      if (threadIdx.x == 1023) last = ex + v;
      __syncthreads();
      int carry = carry_s;
      if (i < nb) bsum[i] = ex + carry;
      __syncthreads();
      if (threadIdx.x == 0) carry_s = carry + last;
      __syncthreads();
   }
   if (threadIdx.x == 0) *total = carry_s;
}

__global__ void k_scan_add(int *__restrict__ out, const int *__restrict__ bsum, int n)
{
   int i = blockIdx.x * 1024 + threadIdx.x;
   if (i < n) out[i] += bsum[blockIdx.x];
}

// ------------------------------------------------------ placement by cell
__global__ void k_scatter(int n, const int *__restrict__ cell_of, const int *__restrict__ cell_start,
                          int *__restrict__ cursor, int *__restrict__ sorted)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) return;
   int c = cell_of[i];
   sorted[cell_start[c] + atomicAdd(&cursor[c], 1)] = i;
}

__global__ void k_cellsort(int ncells, const int *__restrict__ cell_start, int *__restrict__ sorted)
{
   int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= ncells) return;
   int a = cell_start[c], b = cell_start[c + 1];
   for (int i = a + 1; i < b; i++) {
      int v = sorted[i], j = i - 1;
      while (j >= a && sorted[j] > v) {
         sorted[j + 1] = sorted[j];
         j--;
      }
      sorted[j + 1] = v;
   }
}

__global__ void k_gather(RsParams P, const double *__restrict__ site, const double *__restrict__ chg,
                         const int *__restrict__ siteid, const int *__restrict__ molmap,
                         const int *__restrict__ sorted, const int *__restrict__ cell_of,
                         double4 *__restrict__ pos64, float4 *__restrict__ pos32,
                         int2 *__restrict__ tag, int *__restrict__ slot_cell)
{
   int p = blockIdx.x * blockDim.x + threadIdx.x;
   const int N = P.nsites;
   if (p >= N) return;
   int i = sorted[p], c = cell_of[i];
   double x = site[i], y = site[N + i], z = site[2 * N + i], q = chg[i];
   tag[p] = make_int2(siteid[i], molmap[i]);
   slot_cell[p] = c;
   if (pos64) pos64[p] = make_double4(x, y, z, q);
   if (pos32) {
      int cx = c / (P.ny * P.nz), cy = (c / P.nz) % P.ny, cz = c % P.nz;
      // the cell's corner in fractional co-ordinates (reciprocals: the FP64
      // pipe is the cost of this kernel; FP32 cell-relative co-ordinates
      // need the corner only to FP64 rounding)
      double s0 = (double)cx * P.rn[0] - 0.5, s1 = (double)cy * P.rn[1] - 0.5, s2 = (double)cz * P.rn[2] - 0.5;
      double ox = P.h[0] * s0 + P.h[1] * s1 + P.h[2] * s2;
      double oy = P.h[3] * s0 + P.h[4] * s1 + P.h[5] * s2;
      double oz = P.h[6] * s0 + P.h[7] * s1 + P.h[8] * s2;
      pos32[p] = make_float4((float)(x - ox), (float)(y - oy), (float)(z - oz), (float)q);
   }
}

// ---------------------------------------------------------- pair potential
#define AS1 0.254829592
#define AS2 -0.284496736
#define AS3 1.421413741
#define AS4 -1.453152027
#define AS5 1.061405429
#define ASP 0.3275911

template <typename R> __device__ __forceinline__ R dsqrt(R x);
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <typename R> __device__ __forceinline__ R dexp(R x);
template <> __device__ __forceinline__ double dexp<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float dexp<float>(float x) { return expf(x); }

template <int PT> struct NPar { static constexpr int v = 8; };
template <> struct NPar<0> { static constexpr int v = 2; };
template <> struct NPar<1> { static constexpr int v = 3; };
template <> struct NPar<2> { static constexpr int v = 4; };
template <> struct NPar<3> { static constexpr int v = 6; };
template <> struct NPar<4> { static constexpr int v = 3; };
template <> struct NPar<6> { static constexpr int v = 7; };

// Reciprocal square root, reciprocal and exponential: correctly rounded
// (FAST false), or the FP32 hardware approximations (FAST true: rsqrt and
// reciprocal within 2 ulp, exp within a few ulp over the arguments of the
// potentials here), which the column-walk pair kernel of the mixed form
// uses.
template <typename R, bool FAST> struct PairMath {
   static __device__ __forceinline__ R rsqrt(R x) { return R(1) / dsqrt<R>(x); }
   static __device__ __forceinline__ R rcp(R x) { return R(1) / x; }
   static __device__ __forceinline__ R ex(R x) { return dexp<R>(x); }
};
template <> struct PairMath<float, true> {
   static __device__ __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
   static __device__ __forceinline__ float rcp(float x) { return __fdividef(1.0f, x); }
   static __device__ __forceinline__ float ex(float x) { return __expf(x); }
};

// One pair of kernel(): f = -U'(r)/r and U, with the erfc real-space Ewald
// term by the A&S polynomial when EW (src/kernel.c:182-353 / 355-460).
template <int PT, bool EW, typename R, bool FAST = false>
__device__ __forceinline__ void pair_fu(R r2, R qq, const R *p, R alpha, R norm, R &f, R &u)
{
   typedef PairMath<R, FAST> M;
   R t = R(0), ef = R(0), r = R(0), r_r = R(0), rs_r;
   if (EW || PT != 0) {
      if (FAST) {
         r_r = M::rsqrt(r2);
         r = r2 * r_r;
      } else {
         r = dsqrt<R>(r2);
         r_r = R(1) / r;
      }
      rs_r = r_r * r_r;
   } else {
      rs_r = M::rcp(r2);
   }
   if (EW) {
      R ar = alpha * r;
      t = M::rcp(R(1) + R(ASP) * ar);
      ef = qq * M::ex(-(ar * ar));
      t = (t * (R(AS1) + t * (R(AS2) + t * (R(AS3) + t * (R(AS4) + t * R(AS5)))))) * ef * r_r;
      ef = t + norm * ef;
   }
   if (PT == 0) {
      R r6 = (p[1] * p[1]) * rs_r;
      r6 = r6 * r6 * r6;
      R r12 = r6 * r6;
      u = t + p[0] * (r12 - r6);
      f = rs_r * (R(6) * p[0] * (R(2) * r12 - r6) + ef);
   } else if (PT == 1) {
      R e1 = p[1] * M::ex(-p[2] * r);
      R r6 = p[0] * (rs_r * rs_r * rs_r);
      u = t - r6 + e1;
      f = rs_r * (R(-6) * r6 + ef) + p[2] * e1 * r_r;
   } else if (PT == 2) {
      R e1 = p[0] * M::ex(-p[1] * r);
      R e2 = -p[2] * M::ex(-p[3] * r);
      u = t + e1 + e2;
      f = (p[1] * e1 + p[3] * e2) * r_r + ef * rs_r;
   } else if (PT == 3) {
      R e1 = p[0] * M::ex(-p[1] * r);
      R r4 = rs_r * rs_r;
      R r6 = rs_r * r4;
      R r8 = p[5] * (r4 * r4);
      R r12 = p[2] * (r6 * r6);
      r4 *= p[3];
      r6 *= p[4];
      u = t + e1 + r12 - r4 - r6 - r8;
      f = rs_r * (R(12) * r12 - R(4) * r4 - R(6) * r6 - R(8) * r8 + ef) + p[1] * e1 * r_r;
   } else if (PT == 4) {
      R r4 = rs_r * rs_r;
      R r6 = rs_r * r4;
      R r12 = p[2] * (r6 * r6);
      r6 *= p[1];
      r4 *= p[0];
      u = t + r4 + r6 + r12;
      f = rs_r * (R(4) * r4 + R(6) * r6 + R(12) * r12 + ef);
   } else {  // Morse (PT == 6)
      R e1 = p[0] * M::ex((p[1] - r) * p[2]);
      R r6 = p[3] * (rs_r * rs_r * rs_r);
      R e2 = p[4] * M::ex(R(-2) * p[5] * (r - p[6]));
      R e3 = -p[4] * R(2) * M::ex(-p[5] * (r - p[6]));
      u = t + e1 - r6 + e2 + e3;
      f = rs_r * (R(-6) * r6 + ef) + r_r * (p[2] * e1 + (R(2) * p[5]) * e2 + p[5] * e3);
   }
}

// --------------------------------------------------------------- pair loop
// s += x: plain in FP64, Kahan-compensated in FP32 (s - c is the total).
__device__ __forceinline__ void accum(double &s, double &c, double x)
{
   (void)c;
   s += x;
}
__device__ __forceinline__ void accum(float &s, float &c, float x)
{
   const float y = x - c;
   const float t = s + y;
   c = (t - s) - y;
   s = t;
}
__device__ __forceinline__ void note_too_close(DevOut *out, int a, int b)
{
   int k = atomicAdd(&out->n_too_close, 1);
   if (k < MAX_TOO_CLOSE_REC) {
      out->too_close[k][0] = a;
      out->too_close[k][1] = b;
   }
}

__device__ __forceinline__ double block_sum_d(double v, double *sh)
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
   return s;   // valid in thread 0
}

constexpr int PAIR_WARPS = 4;   // warps per block

// Per-warp shared rows of the stencil walk (32 WALK_E entries), and the
// stencil's cell-offset vectors (global, read by entry).
constexpr int WALK_E = 4;   // stencil entries per lane in one pass of the walk

struct WalkRows {
   int *inc, *jb, *info;
   const float4 *oh, *ol;
};

// Walks the full stencil of home slot p (in cell c) with one warp and calls
// visit(j, e, kimg) for every candidate slot j, the home site itself
// excluded: e is the stencil entry j belongs to (its cell-offset vectors are
// rows.oh[e], rows.ol[e]) and kimg the periodic image code.  A pass takes
// 32 WALK_E stencil entries (WALK_E consecutive ones per lane), lays their
// cells' slot ranges end to end by a warp prefix sum, and deals the
// candidates out 32 at a time; each lane finds its candidate's entry by
// binary search over the scanned counts.  With a few sites per cell, wider
// passes keep the lanes busier (fewer, fuller rounds).
template <bool MIXED, class Visit>
__device__ __forceinline__ void walk_stencil(const RsParams &P, int p, int c, int lane,
                                             const int *__restrict__ cell_start,
                                             const int4 *__restrict__ full,
                                             const float4 *__restrict__ off_hi,
                                             const float4 *__restrict__ off_lo, const WalkRows &rows,
                                             Visit &&visit)
{
   (void)off_hi;
   (void)off_lo;
   const int cx = c / (P.ny * P.nz), cy = (c / P.nz) % P.ny, cz = c % P.nz;
   for (int base = 0; base < P.nfull; base += 32 * WALK_E) {
      int cnt[WALK_E], jb[WALK_E], info[WALK_E], tot = 0;
#pragma unroll
      for (int u = 0; u < WALK_E; u++) {
         const int e = base + lane * WALK_E + u;
         cnt[u] = jb[u] = info[u] = 0;
         if (e < P.nfull) {
            const int4 d = __ldg(&full[e]);
            int bx = cx + d.x, by = cy + d.y, bz = cz + d.z;
            const int ix = bx < 0 ? -1 : (bx >= P.nx ? 1 : 0);
            const int iy = by < 0 ? -1 : (by >= P.ny ? 1 : 0);
            const int iz = bz < 0 ? -1 : (bz >= P.nz ? 1 : 0);
            bx -= ix * P.nx;
            by -= iy * P.ny;
            bz -= iz * P.nz;
            const int cb = bz + P.nz * (by + P.ny * bx);
            const int j0 = __ldg(&cell_start[cb]);
            cnt[u] = __ldg(&cell_start[cb + 1]) - j0;
            jb[u] = j0;
            info[u] = (9 * (ix + 1) + 3 * (iy + 1) + (iz + 1)) | (d.w << 8);
         }
         tot += cnt[u];
      }
      const int linc = warp_incl_scan(tot);
      const int T = __shfl_sync(0xffffffffu, linc, 31);
      int run = linc - tot;   // candidates before this lane's entries
#pragma unroll
      for (int u = 0; u < WALK_E; u++) {
         const int q = lane * WALK_E + u;
         rows.jb[q] = jb[u] - run;    // slot = jb[q] + candidate index
         run += cnt[u];
         rows.inc[q] = run;
         rows.info[q] = info[u];
      }
      __syncwarp();
      for (int r = 0; r < T; r += 32) {
         const int idx = r + lane;
         if (idx < T) {
            int k = 0;
#pragma unroll
            for (int s = 16 * WALK_E; s >= 1; s >>= 1)
               if (rows.inc[k + s - 1] <= idx) k += s;
            const int j = rows.jb[k] + idx;
            const int inf = rows.info[k];
            if (!((inf >> 8) && j == p)) visit(j, base + k, inf & 255);
         }
      }
      __syncwarp();
   }
}

// Separation r = x_j - x_i (+ image) from the home site to slot j, r^2 and
// q_j.  FP64 form: the reference's operation order, no fused multiply-adds.
// Mixed form: cell-relative FP32 co-ordinates plus the exact cell offset as
// an FP32 (hi, lo) pair.
template <bool MIXED, typename R>
__device__ __forceinline__ void pair_sep(const RsParams &P, int j, int k, int kimg, const WalkRows &rows,
                                         const float4 &xi32, const double4 &xi64,
                                         const double4 *__restrict__ pos64,
                                         const float4 *__restrict__ pos32, R &rx, R &ry, R &rz, R &r2,
                                         R &qj)
{
   if (MIXED) {
      const float4 xj = __ldg(&pos32[j]);
      const float4 h4 = __ldg(&rows.oh[k]), l4 = __ldg(&rows.ol[k]);
      rx = (h4.x + (xj.x - xi32.x)) + l4.x;
      ry = (h4.y + (xj.y - xi32.y)) + l4.y;
      rz = (h4.z + (xj.z - xi32.z)) + l4.z;
      r2 = rx * rx + ry * ry + rz * rz;
      qj = xj.w;
   } else {
      const double4 xj = pos64[j];
      const double *rl = P.reloc[kimg];
      rx = __dadd_rn(__dsub_rn(xj.x, xi64.x), rl[0]);
      ry = __dadd_rn(__dsub_rn(xj.y, xi64.y), rl[1]);
      rz = __dadd_rn(__dsub_rn(xj.z, xi64.z), rl[2]);
      r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
      qj = xj.w;
   }
}

// Threshold decisions (too-close warning, strict-cutoff clamp).  FP64 form:
// exact, on the reference's r^2.  Mixed form: on the FP32 r^2, except
// within a narrow band of either threshold, where r^2 is re-formed in FP64
// from the original co-ordinates (rare).
template <bool MIXED, typename R>
__device__ __forceinline__ void pair_flags(const RsParams &P, R r2, int oi, int j, int kimg,
                                           const int *__restrict__ sorted, const double *__restrict__ site,
                                           bool &too_close, bool &clip)
{
   if (MIXED) {
      const int N = P.nsites;
      const float r2f = (float)r2;
      const bool near_clip = P.strict && !P.molpbc && fabsf(r2f - P.cut2f) < P.bandf * P.cut2f;
      const bool near_close = fabsf(r2f - (float)TOO_CLOSE) < 1e-3f;
      too_close = r2f < (float)TOO_CLOSE;
      clip = P.strict && !P.molpbc && r2f > P.cut2f;
      if (near_clip || near_close) {
         const int oj = sorted[j];
         const double *rl = P.reloc[kimg];
         double ax = __dadd_rn(__dsub_rn(site[oj], site[oi]), rl[0]);
         double ay = __dadd_rn(__dsub_rn(site[N + oj], site[N + oi]), rl[1]);
         double az = __dadd_rn(__dsub_rn(site[2 * N + oj], site[2 * N + oi]), rl[2]);
         const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)), __dmul_rn(az, az));
         too_close = d2 < TOO_CLOSE;
         clip = P.strict && !P.molpbc && d2 > P.cut2;
      }
   } else {
      too_close = (double)r2 < TOO_CLOSE;
      clip = P.strict && !P.molpbc && (double)r2 > P.cut2;
   }
}

// MODE 0: forces/energy/virial; MODE 1: emit canonical pair keys only.
//
// One warp per home site.  The warp walks the full stencil 32 entries at a
// time: lane e finds the slot range of stencil cell e (a contiguous run of
// the cell-sorted arrays), a warp prefix sum lays the ranges end to end, and
// the candidates are then dealt out 32 at a time, each lane locating its
// candidate's stencil entry by binary search over the scanned counts.  Every
// lane runs the same pair arithmetic on a different candidate, so the warp
// stays converged however unevenly the sites are spread over the cells.
template <int PT, bool EW, bool MIXED, int MODE>
__global__ void __launch_bounds__(PAIR_WARPS * 32)
k_pairs(RsParams P, const int *__restrict__ cell_start, const int *__restrict__ slot_cell,
        const int4 *__restrict__ full, const float4 *__restrict__ off_hi,
        const float4 *__restrict__ off_lo, const double4 *__restrict__ pos64,
        const float4 *__restrict__ pos32, const int2 *__restrict__ tag,
        const int *__restrict__ sorted, const double *__restrict__ site,
        const double *__restrict__ potg64, const float *__restrict__ potg32,
        const double *__restrict__ chg64,
        double *__restrict__ force, double *__restrict__ part, DevOut *out,
        unsigned long long *__restrict__ keys, long long key_cap)
{
   typedef typename std::conditional<MIXED, float, double>::type R;
   constexpr int NP = NPar<PT>::v;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ int s_inc[PAIR_WARPS][32 * WALK_E], s_jb[PAIR_WARPS][32 * WALK_E], s_info[PAIR_WARPS][32 * WALK_E];
   R *pot_s = reinterpret_cast<R *>(smem_raw);
   const int npot = P.max_id * P.max_id;
   const R *potg = MIXED ? (const R *)(const void *)potg32 : (const R *)(const void *)potg64;
   if (P.pot_in_smem)
      for (int q = threadIdx.x; q < npot * NPOTP; q += blockDim.x) pot_s[q] = potg[q];
   __syncthreads();
   const R *pot = P.pot_in_smem ? pot_s : potg;

   const int N = P.nsites;
   const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int p = blockIdx.x * PAIR_WARPS + w;   // home slot of this warp
   const WalkRows rows{s_inc[w], s_jb[w], s_info[w], off_hi, off_lo};
   // per-lane partial sums: few terms each, then a warp tree reduction
   R fx = 0, fy = 0, fz = 0, pe = 0, v0 = 0, v1 = 0, v2 = 0, v3 = 0, v4 = 0, v5 = 0;
   int nev = 0;                                  // evaluations by this lane
   const R cut100 = (R)P.cut100;
   if (p < N) {
      const int c = slot_cell[p];
      const int2 ti = tag[p];
      const R *prow = pot + (size_t)ti.x * P.max_id * NPOTP;
      double4 xi64 = make_double4(0, 0, 0, 0);
      float4 xi32 = make_float4(0, 0, 0, 0);
      if (MIXED) xi32 = pos32[p]; else xi64 = pos64[p];
      const R qi = MIXED ? (R)xi32.w : (R)xi64.w;
      const R alpha = MIXED ? (R)P.alphaf : (R)P.alpha, norm = MIXED ? (R)P.normf : (R)P.norm;
      const int oi = sorted[p];
      walk_stencil<MIXED>(P, p, c, lane, cell_start, full, off_hi, off_lo, rows, [&](int j, int k, int kimg) {
         R rx, ry, rz, r2, qj;
         const int2 tj = __ldg(&tag[j]);
         if (ti.y == P.fw_mol && tj.y == P.fw_mol) return;   // no framework-framework pairs
         pair_sep<MIXED>(P, j, k, kimg, rows, xi32, xi64, pos64, pos32, rx, ry, rz, r2, qj);
         if (MODE == 1) {
            const long long a = oi, bb = sorted[j];
            if (a < bb || (a == bb && kimg < 13)) {
               unsigned long long key = ((unsigned long long)a << 37) |
                                        ((unsigned long long)bb << 5) | (unsigned long long)kimg;
               unsigned long long slot = atomicAdd((unsigned long long *)&out->npairs2, 1ull);
               if ((long long)slot < key_cap) keys[slot] = key;
            }
            return;
         }
         const bool intra = ti.y == tj.y;
         bool too_close, clip;
         pair_flags<MIXED>(P, r2, oi, j, kimg, sorted, site, too_close, clip);
         if (too_close && !intra) {
            const int oj = sorted[j];
            if (oi < oj) note_too_close(out, oi, oj);
         }
         const R r2a = r2;
         if (clip) r2 = cut100;
         R pp[NP];
         const R *pj = prow + (size_t)tj.x * NPOTP;
#pragma unroll
         for (int q = 0; q < NP; q++) pp[q] = pj[q];
         R f, u;
         pair_fu<PT, EW, R>(r2, qj * qi, pp, alpha, norm, f, u);
         if (MIXED && intra) {
            // Mixed form: an intramolecular pair's energy is exactly what
            // the intramolecular correction subtracts again, so it is left
            // out of both (FP32 roundings of identical molecules would add
            // up coherently instead of cancelling); a clamped pair keeps the
            // difference between its clamped and true energies.
            R fa, ua = R(0);
            if (clip) pair_fu<PT, EW, R>(r2a, qj * qi, pp, alpha, norm, fa, ua);
            u = clip ? u - ua : R(0);
         }
         const R hf = R(0.5) * f;
         fx -= f * rx;
         fy -= f * ry;
         fz -= f * rz;
         pe += R(0.5) * u;
         v0 += hf * rx * rx;
         v1 += hf * rx * ry;
         v2 += hf * rx * rz;
         v3 += hf * ry * ry;
         v4 += hf * ry * rz;
         v5 += hf * rz * rz;
         nev++;
      });
      if (MODE == 0) {
         // warp tree reduction of the home site's force, in the working
         // precision (each lane holds a sum of a few pairs)
         R Fx = fx, Fy = fy, Fz = fz;
#pragma unroll
         for (int o = 16; o > 0; o >>= 1) {
            Fx += __shfl_down_sync(0xffffffffu, Fx, o);
            Fy += __shfl_down_sync(0xffffffffu, Fy, o);
            Fz += __shfl_down_sync(0xffffffffu, Fz, o);
         }
         if (lane == 0) {
            force[oi] = (double)Fx;
            force[N + oi] = (double)Fy;
            force[2 * N + oi] = (double)Fz;
         }
      }
   }
   if (MODE == 1) return;
   // energy and virial: warp trees in the working precision, then the
   // block's warps summed in FP64 (FP64 is slow on this part: keep it to a
   // handful of operations per block)
   __shared__ R wred[7][PAIR_WARPS];
   R vv[7] = {pe, v0, v1, v2, v3, v4, v5};
#pragma unroll
   for (int k = 0; k < 7; k++) {
      R s = vv[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) wred[k][w] = s;
   }
   __syncthreads();
   if (threadIdx.x < 7) {
      double s = 0.0;
      for (int q = 0; q < PAIR_WARPS; q++) s += (double)wred[threadIdx.x][q];
      part[blockIdx.x * 8 + threadIdx.x] = s;
   }
   unsigned long long cnt = (unsigned long long)nev;
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
   if (lane == 0 && cnt) atomicAdd((unsigned long long *)&out->npairs2, cnt);
}

// Per-block energy/virial partials of the pair kernel summed in a fixed
// order, in two levels: RS_RED blocks of 256 threads each reduce a fixed
// slice of the partials into one record (k_reduce_rs), then one block sums
// those (k_reduce_rs2).  The result does not depend on timing.
constexpr int RS_RED = 64;

__device__ __forceinline__ void tree7(double (*sh)[256], int t)
{
   __syncthreads();
   for (int w = 128; w > 0; w >>= 1) {
      if (t < w)
         for (int k = 0; k < 7; k++) sh[k][t] += sh[k][t + w];
      __syncthreads();
   }
}

__global__ void __launch_bounds__(256) k_reduce_rs(const double *__restrict__ part, int nblocks,
                                                   double *__restrict__ part2)
{
   __shared__ double sh[7][256];
   const int t = threadIdx.x;
   const int per = (nblocks + gridDim.x - 1) / gridDim.x;
   const int b0 = blockIdx.x * per, b1 = min(nblocks, b0 + per);
   double s[7] = {0, 0, 0, 0, 0, 0, 0};
   for (int b = b0 + t; b < b1; b += 256)
      for (int k = 0; k < 7; k++) s[k] += part[b * 8 + k];
   for (int k = 0; k < 7; k++) sh[k][t] = s[k];
   tree7(sh, t);
   if (t < 7) part2[blockIdx.x * 8 + t] = sh[t][0];
}

// One block over all the partials (few blocks: the column walk's grid of a
// few blocks per SM): thread t takes blocks t, t + 256, ..., then the tree.
__global__ void __launch_bounds__(256) k_reduce_rs1(const double *__restrict__ part, int nblocks, DevOut *out)
{
   __shared__ double sh[7][256];
   const int t = threadIdx.x;
   double s[7] = {0, 0, 0, 0, 0, 0, 0};
   for (int b = t; b < nblocks; b += 256)
      for (int k = 0; k < 7; k++) s[k] += part[b * 8 + k];
   for (int k = 0; k < 7; k++) sh[k][t] = s[k];
   tree7(sh, t);
   if (t == 0) {
      out->pe_rs = sh[0][0];
      for (int k = 0; k < 6; k++) out->vir_rs[k] = sh[k + 1][0];
   }
}

__global__ void __launch_bounds__(256) k_reduce_rs2(const double *__restrict__ part2, int n, DevOut *out)
{
   __shared__ double sh[7][256];
   const int t = threadIdx.x;
   for (int k = 0; k < 7; k++) sh[k][t] = t < n ? part2[t * 8 + k] : 0.0;
   tree7(sh, t);
   if (t == 0) {
      out->pe_rs = sh[0][0];
      for (int k = 0; k < 6; k++) out->vir_rs[k] = sh[k + 1][0];
   }
}

// ------------------------------------------------- column walk (mixed form)
// The pair kernel of the mixed form, k_pairs_col, walks the stencil by
// columns and over one interaction class at a time.
//
// Columns: for a home cell (cx, cy, cz) and a stencil column (dx, dy, dz0,
// len) the partner cells (cx+dx, cy+dy, cz+dz0 .. cz+dz0+len-1) are
// consecutive cells of the link-cell order (at most two runs where the
// column wraps the periodic cell in z), so their sites are one or two
// contiguous slot ranges: a home site needs about 75 column lookups on the
// benchmark workload instead of about 485 cell lookups.
//
// Classes: identifiers are split into class 0 (those that interact with a
// charged site, directly or through a potential with nonzero parameters)
// and class 1 (the rest).  A pair across the classes has no charge product
// and a potential with all parameters zero, so it adds exactly nothing to
// forces, energy and virial: each home site walks the sites of its own class
// only (rigid water: O meets only O, H and M only H and M -- 37.5% of the
// ordered pairs skipped).  The slots are re-laid class by class, each class
// in link-cell order, with per-class cell starts.  The reference's evaluated
// pair count (every class) is counted on demand by k_count_col, and pairs
// across the classes closer than the too-close distance are reported by
// k_tooclose_x.
constexpr int COL_E = 3;                    // stencil columns per lane in one pass
constexpr int COL_ROWS = 32 * COL_E * 2;    // slot runs per pass (two per column at most)
constexpr int COL_WIN = 256;                // candidates decoded per window
constexpr int COL_CHUNK = 16;               // consecutive home slots a block takes at a time

// per slot (link-cell order): 1 when its identifier is in class 0; the
// entry after the last is 0 (so the exclusive scan ends with the class-0
// count)
__global__ void k_cls_flag(int N, const int2 *__restrict__ tag, const int *__restrict__ cls_of_id,
                           int *__restrict__ flag)
{
   const int p = blockIdx.x * blockDim.x + threadIdx.x;
   if (p < N) flag[p] = cls_of_id[tag[p].x] == 0 ? 1 : 0;
   else if (p == N) flag[p] = 0;
}

// Slots re-laid class by class (stable): class 0 first, then class 1, each
// in link-cell order; per-class cell starts cs[K][c].  pre[p] is the number
// of class-0 slots before p (pre[N] their total).  The per-slot tag carries
// the identifier in its low 16 bits and the cell's z index above them.
__global__ void k_cls_split(RsParams P, const int *__restrict__ pre, const int *__restrict__ cls_of_id,
                            const int *__restrict__ cell_start, const float4 *__restrict__ pos32,
                            const int2 *__restrict__ tag, const int *__restrict__ sorted,
                            const int *__restrict__ slot_cell, int *__restrict__ cs, float4 *__restrict__ posc,
                            int2 *__restrict__ tagc, int *__restrict__ sortc, int *__restrict__ cellc)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const int N = P.nsites, n0 = pre[N];
   if (i < N) {
      const int2 t = tag[i];
      const int q = cls_of_id[t.x] == 0 ? pre[i] : n0 + (i - pre[i]);
      const int c = slot_cell[i];
      posc[q] = pos32[i];
      tagc[q] = make_int2(t.x | ((c % P.nz) << 16), t.y);
      sortc[q] = sorted[i];
      cellc[q] = c;
   }
   if (i <= P.ncells) {
      const int a = cell_start[i], b = pre[a];
      cs[i] = b;
      cs[P.ncells + 1 + i] = n0 + (a - b);
   }
}

// A column offset's hi and lo parts (32 bytes, 32-byte aligned) in one load.
__device__ __forceinline__ void ld_coff(const float4 *p, float4 &h, float4 &l)
{
   asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
       : "=f"(h.x), "=f"(h.y), "=f"(h.z), "=f"(h.w), "=f"(l.x), "=f"(l.y), "=f"(l.z), "=f"(l.w)
       : "l"(p));
}

// The partner cells of a home cell (cx, cy, cz) in stencil column cd =
// (dx, dy, dz0, len): cc, the link-cell index of the partner column's first
// cell; ns (1 or 2) runs of consecutive cells za[s] .. zb[s] in that column,
// with their periodic images ix, iy (-1, 0, 1) and iz[s].
struct ColRuns {
   int cc, ns, ix, iy;
   int za[2], zb[2], iz[2];
};
__device__ __forceinline__ ColRuns col_runs(const RsParams &P, int cx, int cy, int cz, int4 cd)
{
   ColRuns r;
   int bx = cx + cd.x, by = cy + cd.y;
   r.ix = bx < 0 ? -1 : (bx >= P.nx ? 1 : 0);
   r.iy = by < 0 ? -1 : (by >= P.ny ? 1 : 0);
   bx -= r.ix * P.nx;
   by -= r.iy * P.ny;
   r.cc = P.nz * (by + P.ny * bx);
   const int z0 = cz + cd.z, z1 = z0 + cd.w - 1;
   r.ns = 1;
   if (z1 < 0) { r.za[0] = z0 + P.nz; r.zb[0] = z1 + P.nz; r.iz[0] = -1; }
   else if (z0 >= P.nz) { r.za[0] = z0 - P.nz; r.zb[0] = z1 - P.nz; r.iz[0] = 1; }
   else if (z0 < 0) { r.za[0] = z0 + P.nz; r.zb[0] = P.nz - 1; r.iz[0] = -1; r.za[1] = 0; r.zb[1] = z1; r.iz[1] = 0; r.ns = 2; }
   else if (z1 >= P.nz) { r.za[0] = z0; r.zb[0] = P.nz - 1; r.iz[0] = 0; r.za[1] = 0; r.zb[1] = z1 - P.nz; r.iz[1] = 1; r.ns = 2; }
   else { r.za[0] = z0; r.zb[0] = z1; r.iz[0] = 0; }
   return r;
}

// Each warp takes home slots of the class-major layout in turn (eight
// blocks per SM, the grid's warps striding over the slots, so that the
// block's set-up and energy reduction are paid once per block).  Per home
// slot, a pass gives each lane
// COL_E columns (up to two slot runs each, of the home site's class); a warp
// prefix sum lays the runs end to end; windows of COL_WIN candidates are
// decoded into shared memory (slot | run << 24) and dealt out 32 at a time.
// The pair arithmetic is k_pairs's mixed form: FP32 from cell-relative
// co-ordinates and the exact cell offset as an (hi, lo) pair, decisions near
// a threshold re-made in FP64, Kahan-free per-lane sums reduced by warp
// trees.
template <int PT, bool EW>
__global__ void __launch_bounds__(PAIR_WARPS * 32, 8)
k_pairs_col(RsParams P, const int *__restrict__ cell_start, const int *__restrict__ cs,
            const int *__restrict__ pre, const int4 *__restrict__ cols, const int *__restrict__ col_base,
            const float4 *__restrict__ coff, const float4 *__restrict__ posc, const int2 *__restrict__ tagc,
            const int *__restrict__ cellc,
            const int *__restrict__ sortc, const double *__restrict__ site, const float *__restrict__ potg,
            double *__restrict__ force, double *__restrict__ part, DevOut *out)
{
   typedef float R;
   constexpr int NP = NPar<PT>::v;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ int s_inc[PAIR_WARPS][COL_ROWS], s_jb[PAIR_WARPS][COL_ROWS], s_inf[PAIR_WARPS][COL_ROWS];
   __shared__ int s_cand[PAIR_WARPS][COL_WIN];
   R *pot_s = reinterpret_cast<R *>(smem_raw);
   const int npot = P.max_id * P.max_id;
   if (P.pot_in_smem)
      for (int q = threadIdx.x; q < npot * NPOTP; q += blockDim.x) pot_s[q] = potg[q];
   __syncthreads();
   const R *pot = P.pot_in_smem ? pot_s : potg;

   const int N = P.nsites, n0 = pre[N];
   const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
   int *inc = s_inc[w], *jbr = s_jb[w], *infr = s_inf[w], *cand = s_cand[w];
   // the lane's energy and virial over all its home sites (per-site sums
   // added in: two levels of FP32), kept in shared memory, which the
   // candidate loop's registers leave no room for
   __shared__ R s_tot[7][PAIR_WARPS * 32];
#pragma unroll
   for (int k = 0; k < 7; k++) s_tot[k][threadIdx.x] = R(0);
   // home slots (class-major) in chunks of COL_CHUNK consecutive slots, the
   // grid's blocks taking the chunks in turn and the block's warps the
   // chunk's slots in turn: a few resident blocks per SM take every site,
   // neighbouring sites (shared candidates and column starts in L1) at
   // about the same time
   for (int it = 0, p = blockIdx.x * COL_CHUNK + w; p < N;
        it++, p = ((it / (COL_CHUNK / PAIR_WARPS)) * gridDim.x + blockIdx.x) * COL_CHUNK +
                  (it % (COL_CHUNK / PAIR_WARPS)) * PAIR_WARPS + w) {
      R fx = 0, fy = 0, fz = 0, pe = 0, v0 = 0, v1 = 0, v2 = 0, v3 = 0, v4 = 0, v5 = 0;
      const int *csk = cs + (p < n0 ? 0 : P.ncells + 1);
      const int c = cellc[p];
      const int cx = c / (P.ny * P.nz), cy = (c / P.nz) % P.ny, cz = c % P.nz;
      const int2 ti = tagc[p];
      const R *prow = pot + (size_t)(ti.x & 0xffff) * P.max_id * NPOTP;
      const float4 xi = posc[p];
      const R qi = xi.w;
      const R alpha = P.alphaf, norm = P.normf;
      const int oi = sortc[p];
      const R cut100 = (R)P.cut100;
      for (int base = 0; base < P.ncols; base += 32 * COL_E) {
         // this lane's runs go straight to its rows (counts in inc for now)
         int tot = 0;
#pragma unroll
         for (int u = 0; u < COL_E; u++) {
            const int q0 = lane * 2 * COL_E + 2 * u;
            inc[q0] = inc[q0 + 1] = 0;
            jbr[q0] = jbr[q0 + 1] = 0;
            infr[q0] = infr[q0 + 1] = 0;
            const int col = base + lane * COL_E + u;
            if (col < P.ncols) {
               const int4 cd = __ldg(&cols[col]);
               const int ob = __ldg(&col_base[col]);
               const ColRuns cr = col_runs(P, cx, cy, cz, cd);
#pragma unroll
               for (int s = 0; s < 2; s++) {
                  if (s < cr.ns) {
                     const int a = __ldg(&csk[cr.cc + cr.za[s]]), b = __ldg(&csk[cr.cc + cr.zb[s] + 1]);
                     inc[q0 + s] = b - a;
                     jbr[q0 + s] = a;
                     tot += b - a;
                     // offset-table index of a candidate in cell z: z + eb
                     const int eb = ob - cd.z - cz + cr.iz[s] * P.nz;
                     infr[q0 + s] = (eb * 32) | (9 * (cr.ix + 1) + 3 * (cr.iy + 1) + (cr.iz[s] + 1));
                  }
               }
            }
         }
         const int linc = warp_incl_scan(tot);
         const int T = __shfl_sync(0xffffffffu, linc, 31);
         int run = linc - tot;
#pragma unroll
         for (int r = 0; r < 2 * COL_E; r++) {
            const int q = lane * 2 * COL_E + r;
            jbr[q] -= run;               // slot = jbr[q] + candidate index
            run += inc[q];
            inc[q] = run;                // the row's inclusive end
         }
         __syncwarp();
         for (int w0 = 0; w0 < T; w0 += COL_WIN) {
            const int w1 = min(T, w0 + COL_WIN);
            // decode this lane's runs that fall in [w0, w1)
#pragma unroll
            for (int r = 0; r < 2 * COL_E; r++) {
               const int q = lane * 2 * COL_E + r;
               const int e1 = inc[q], e0 = q > 0 ? inc[q - 1] : 0;
               const int a = max(e0, w0), b = min(e1, w1);
               const int jq = jbr[q];
               for (int t = a; t < b; t++) cand[t - w0] = (jq + t) | (q << 24);
            }
            __syncwarp();
            for (int r0 = w0; r0 < w1; r0 += 32) {
               const int idx = r0 + lane;
               if (idx < w1) {
                  const int v = cand[idx - w0];
                  const int j = v & 0xffffff, q = (unsigned)v >> 24;
                  const int inf_q = infr[q];
                  const int kimg = inf_q & 31;
                  if (j != p || kimg != 13) {
                     const int2 tj = __ldg(&tagc[j]);
                     const int e = (tj.x >> 16) + (inf_q >> 5);
                     const float4 xj = __ldg(&posc[j]);
                     float4 h4, l4;
                     ld_coff(coff + 2 * e, h4, l4);
                     const R rx = (h4.x + (xj.x - xi.x)) + l4.x;
                     const R ry = (h4.y + (xj.y - xi.y)) + l4.y;
                     const R rz = (h4.z + (xj.z - xi.z)) + l4.z;
                     R r2 = rx * rx + ry * ry + rz * rz;
                     const bool intra = ti.y == tj.y;
                     bool too_close, clip;
                     pair_flags<true>(P, r2, oi, j, kimg, sortc, site, too_close, clip);
                     if (too_close && !intra) {
                        const int oj = sortc[j];
                        if (oi < oj) note_too_close(out, oi, oj);
                     }
                     const R r2a = r2;
                     if (clip) r2 = cut100;
                     R pp[NP];
                     const R *pj = prow + (size_t)(tj.x & 0xffff) * NPOTP;
#pragma unroll
                     for (int k = 0; k < NP; k++) pp[k] = pj[k];
                     R f, u;
                     pair_fu<PT, EW, R, true>(r2, xj.w * qi, pp, alpha, norm, f, u);
                     if (intra) {
                        // as in k_pairs: an intramolecular pair's energy is
                        // what the intramolecular correction subtracts again
                        R fa, ua = R(0);
                        if (clip) pair_fu<PT, EW, R, true>(r2a, xj.w * qi, pp, alpha, norm, fa, ua);
                        u = clip ? u - ua : R(0);
                     }
                     const R hf = R(0.5) * f;
                     fx -= f * rx;
                     fy -= f * ry;
                     fz -= f * rz;
                     pe += R(0.5) * u;
                     v0 += hf * rx * rx;
                     v1 += hf * rx * ry;
                     v2 += hf * rx * rz;
                     v3 += hf * ry * ry;
                     v4 += hf * ry * rz;
                     v5 += hf * rz * rz;
                  }
               }
            }
            __syncwarp();
         }
      }
      R Fx = fx, Fy = fy, Fz = fz;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
         Fx += __shfl_down_sync(0xffffffffu, Fx, o);
         Fy += __shfl_down_sync(0xffffffffu, Fy, o);
         Fz += __shfl_down_sync(0xffffffffu, Fz, o);
      }
      if (lane == 0) {
         force[oi] = (double)Fx;
         force[N + oi] = (double)Fy;
         force[2 * N + oi] = (double)Fz;
      }
      s_tot[0][threadIdx.x] += pe;
      s_tot[1][threadIdx.x] += v0;
      s_tot[2][threadIdx.x] += v1;
      s_tot[3][threadIdx.x] += v2;
      s_tot[4][threadIdx.x] += v3;
      s_tot[5][threadIdx.x] += v4;
      s_tot[6][threadIdx.x] += v5;
   }
   __shared__ R wred[7][PAIR_WARPS];
   R vv[7];
#pragma unroll
   for (int k = 0; k < 7; k++) vv[k] = s_tot[k][threadIdx.x];
#pragma unroll
   for (int k = 0; k < 7; k++) {
      R s = vv[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) wred[k][w] = s;
   }
   __syncthreads();
   if (threadIdx.x < 7) {
      double s = 0.0;
      for (int q = 0; q < PAIR_WARPS; q++) s += (double)wred[threadIdx.x][q];
      part[blockIdx.x * 8 + threadIdx.x] = s;
   }
}

// The reference's evaluated pair count after a column-walk pass (which
// leaves it out of the hot loop): per home slot the sites of every class in
// the stencil's column runs, less the site itself, summed into
// out->npairs2.  One thread per slot; run on demand (mdgpu_get_info).
__global__ void __launch_bounds__(256)
k_count_col(RsParams P, const int *__restrict__ cell_start, const int4 *__restrict__ cols,
            const int *__restrict__ cellc, DevOut *out)
{
   __shared__ unsigned long long sh[8];
   const int p = blockIdx.x * blockDim.x + threadIdx.x;
   unsigned long long n = 0;
   if (p < P.nsites) {
      const int c = cellc[p];
      const int cx = c / (P.ny * P.nz), cy = (c / P.nz) % P.ny, cz = c % P.nz;
      for (int col = 0; col < P.ncols; col++) {
         const ColRuns cr = col_runs(P, cx, cy, cz, __ldg(&cols[col]));
         for (int s = 0; s < cr.ns; s++)
            n += (unsigned long long)(__ldg(&cell_start[cr.cc + cr.zb[s] + 1]) - __ldg(&cell_start[cr.cc + cr.za[s]]));
      }
      n -= 1;   // the home site itself
   }
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xffffffffu, n, o);
   if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = n;
   __syncthreads();
   if (threadIdx.x == 0) {
      unsigned long long t = 0;
      for (int w = 0; w < 8; w++) t += sh[w];
      if (t) atomicAdd((unsigned long long *)&out->npairs2, t);
   }
}

// Pairs across the interaction classes that come closer than the too-close
// distance (the reference warns of every evaluated pair with r^2 < 0.25,
// src/force.c:943-948, whatever its potential): such a pair lies in the
// 27-cell neighbourhood (cells at least 0.5 A thick).  For each class-0
// slot (class-major layout) nine threads take the class-1 sites of the
// neighbourhood, one column run of 3 cells each, and form r^2 in FP32 from the
// cell-relative co-ordinates and the exact cell offset (hi + lo), re-made
// in FP64 from the original co-ordinates with the reference's operation
// order within 1e-3 A^2 of the threshold, as k_pairs decides.  Reported
// once per pair, as (lower site index, higher), intramolecular pairs
// excepted.  nbcol[9]: the stencil column of each (dx, dy) in [-1, 1]^2.
struct NbCols {
   int col[9];
};

__global__ void __launch_bounds__(256)
k_tooclose_x(RsParams P, NbCols nb, const int *__restrict__ cs, const int *__restrict__ pre,
             const int4 *__restrict__ cols, const int *__restrict__ col_base,
             const float4 *__restrict__ coff, const float4 *__restrict__ posc, const int2 *__restrict__ tagc,
             const int *__restrict__ cellc,
             const int *__restrict__ sortc, const double *__restrict__ site, DevOut *out)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   const int p = t / 9, d = t - 9 * p;   // one column of the neighbourhood per thread
   const int N = P.nsites, n0 = pre[N];
   if (p >= n0) return;
   const int *cs1 = cs + P.ncells + 1;
   const int c = cellc[p];
   const int cx = c / (P.ny * P.nz), cy = (c / P.nz) % P.ny, cz = c % P.nz;
   const float4 xi = posc[p];
   const int moli = tagc[p].y, oi = sortc[p];
   {
      const int dx = d / 3 - 1, dy = d % 3 - 1;
      int bx = cx + dx, by = cy + dy;
      const int ix = bx < 0 ? -1 : (bx >= P.nx ? 1 : 0);
      const int iy = by < 0 ? -1 : (by >= P.ny ? 1 : 0);
      bx -= ix * P.nx;
      by -= iy * P.ny;
      const int cc = P.nz * (by + P.ny * bx);
      const int ci = nb.col[d];
      const int eb = __ldg(&col_base[ci]) - __ldg(&cols[ci]).z - cz;   // offset index of cell z: z + eb
      // cells cz-1 .. cz+1 of the column, split where they wrap in z (the
      // scan runs only with nz >= 3, so one side at most)
      const int z0 = cz - 1, z1 = cz + 1;
      int za[2], zb[2], iz[2], ns = 1;
      if (z0 < 0) { za[0] = z0 + P.nz; zb[0] = P.nz - 1; iz[0] = -1; za[1] = 0; zb[1] = z1; iz[1] = 0; ns = 2; }
      else if (z1 >= P.nz) { za[0] = z0; zb[0] = P.nz - 1; iz[0] = 0; za[1] = 0; zb[1] = z1 - P.nz; iz[1] = 1; ns = 2; }
      else { za[0] = z0; zb[0] = z1; iz[0] = 0; }
      for (int s = 0; s < ns; s++) {
         const int kimg = 9 * (ix + 1) + 3 * (iy + 1) + (iz[s] + 1);
         for (int j = cs1[cc + za[s]]; j < cs1[cc + zb[s] + 1]; j++) {
            const int2 tj = tagc[j];
            if (tj.y == moli) continue;
            const int e = (tj.x >> 16) + iz[s] * P.nz + eb;
            const float4 xj = posc[j];
            float4 h4, l4;
            ld_coff(coff + 2 * e, h4, l4);
            const float rx = (h4.x + (xj.x - xi.x)) + l4.x;
            const float ry = (h4.y + (xj.y - xi.y)) + l4.y;
            const float rz = (h4.z + (xj.z - xi.z)) + l4.z;
            const float r2 = rx * rx + ry * ry + rz * rz;
            if (r2 >= (float)TOO_CLOSE + 1e-3f) continue;
            bool close = r2 < (float)TOO_CLOSE;
            const int oj = sortc[j];
            if (fabsf(r2 - (float)TOO_CLOSE) < 1e-3f) {
               const double *rl = P.reloc[kimg];
               const double ax = __dadd_rn(__dsub_rn(site[oj], site[oi]), rl[0]);
               const double ay = __dadd_rn(__dsub_rn(site[N + oj], site[N + oi]), rl[1]);
               const double az = __dadd_rn(__dsub_rn(site[2 * (size_t)N + oj], site[2 * (size_t)N + oi]), rl[2]);
               close = __dadd_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)), __dmul_rn(az, az)) < TOO_CLOSE;
            }
            if (close) note_too_close(out, min(oi, oj), max(oi, oj));
         }
      }
   }
}

// ----------------------------------------------------------------- adjoint
// Derivatives of one pair evaluation of pair_fu (f = -U'(r)/r, U) with
// respect to the potential parameters and the Ewald terms:
//   du[k] = dU/dp_k, df[k] = df/dp_k               (short-range part)
//   uc = erfc(alpha r)/r, fc = (uc + norm exp(-alpha^2 r^2))/r^2
//                                                   (per unit q_i q_j)
//   duc = d uc/d alpha, dfc = d fc/d alpha          (per unit q_i q_j)
// erfc is pair_fu's A&S polynomial t P(t) exp(-x^2), t = 1/(1 + p x), and
// is differentiated as such: these are the derivatives of the energy and
// force the forward kernel computes.
template <int NP, typename R>
struct PairGrad {
   R du[NP], df[NP];
   R uc, fc, duc, dfc;
};

template <int PT, bool EW, typename R>
__device__ __forceinline__ void pair_grad(R r2, const R *p, R alpha, R norm, PairGrad<NPar<PT>::v, R> &g)
{
   const R r = dsqrt<R>(r2), r_r = R(1) / r, rs_r = r_r * r_r;
   g.uc = g.fc = g.duc = g.dfc = R(0);
   if (EW) {
      const R x = alpha * r;
      const R t = R(1) / (R(1) + R(ASP) * x);
      const R pt = R(AS1) + t * (R(AS2) + t * (R(AS3) + t * (R(AS4) + t * R(AS5))));
      const R dpt = R(AS2) + t * (R(2.0 * AS3) + t * (R(3.0 * AS4) + t * R(4.0 * AS5)));
      const R ex = dexp<R>(-(x * x));
      // d/dx [t P(t) e^{-x^2}] with dt/dx = -p t^2
      const R derfc = ex * (-R(ASP) * t * t * (pt + t * dpt) - R(2) * x * t * pt);
      g.uc = t * pt * ex * r_r;
      g.fc = rs_r * (g.uc + norm * ex);
      g.duc = derfc;
      g.dfc = rs_r * (derfc + R(1.1283791670955126) * ex * (R(1) - R(2) * x * x));   // 2/sqrt(pi)
   }
   if (PT == 0) {   // p0 ((p1/r)^12 - (p1/r)^6)
      const R p1s = p[1] * p[1];
      R s6 = p1s * rs_r;
      s6 = s6 * s6 * s6;
      const R s12 = s6 * s6;
      const R t5 = p1s * p1s * p[1] * (rs_r * rs_r * rs_r);   // d s6 / d p1 / 6
      g.du[0] = s12 - s6;
      g.du[1] = R(6) * p[0] * t5 * (R(2) * s6 - R(1));
      g.df[0] = rs_r * R(6) * (R(2) * s12 - s6);
      g.df[1] = rs_r * R(36) * p[0] * t5 * (R(4) * s6 - R(1));
   } else if (PT == 1) {   // -p0/r^6 + p1 exp(-p2 r)
      const R E = dexp<R>(-p[2] * r);
      const R r6 = rs_r * rs_r * rs_r;
      g.du[0] = -r6;
      g.du[1] = E;
      g.du[2] = -r * p[1] * E;
      g.df[0] = R(-6) * rs_r * r6;
      g.df[1] = p[2] * E * r_r;
      g.df[2] = p[1] * E * (r_r - p[2]);
   } else if (PT == 2) {   // p0 exp(-p1 r) - p2 exp(-p3 r)
      const R E1 = dexp<R>(-p[1] * r), E3 = dexp<R>(-p[3] * r);
      const R e1 = p[0] * E1, e2 = -p[2] * E3;
      g.du[0] = E1;
      g.du[1] = -r * e1;
      g.du[2] = -E3;
      g.du[3] = -r * e2;
      g.df[0] = p[1] * E1 * r_r;
      g.df[1] = e1 * (r_r - p[1]);
      g.df[2] = -p[3] * E3 * r_r;
      g.df[3] = e2 * (r_r - p[3]);
   } else if (PT == 3) {   // p0 exp(-p1 r) + p2/r^12 - p3/r^4 - p4/r^6 - p5/r^8
      const R E1 = dexp<R>(-p[1] * r), e1 = p[0] * E1;
      const R r4 = rs_r * rs_r, r6 = r4 * rs_r, r8 = r4 * r4, r12 = r6 * r6;
      g.du[0] = E1;
      g.du[1] = -r * e1;
      g.du[2] = r12;
      g.du[3] = -r4;
      g.du[4] = -r6;
      g.du[5] = -r8;
      g.df[0] = p[1] * E1 * r_r;
      g.df[1] = e1 * (r_r - p[1]);
      g.df[2] = R(12) * rs_r * r12;
      g.df[3] = R(-4) * rs_r * r4;
      g.df[4] = R(-6) * rs_r * r6;
      g.df[5] = R(-8) * rs_r * r8;
   } else if (PT == 4) {   // p0/r^4 + p1/r^6 + p2/r^12
      const R r4 = rs_r * rs_r, r6 = r4 * rs_r, r12 = r6 * r6;
      g.du[0] = r4;
      g.du[1] = r6;
      g.du[2] = r12;
      g.df[0] = R(4) * rs_r * r4;
      g.df[1] = R(6) * rs_r * r6;
      g.df[2] = R(12) * rs_r * r12;
   } else {   // Morse: p0 e^{(p1-r)p2} - p3/r^6 + p4 (e^{-2 p5 (r-p6)} - 2 e^{-p5 (r-p6)})
      const R E1 = dexp<R>((p[1] - r) * p[2]), e1 = p[0] * E1;
      const R r6 = rs_r * rs_r * rs_r;
      const R d6 = r - p[6];
      const R E2 = dexp<R>(R(-2) * p[5] * d6), E3 = dexp<R>(-p[5] * d6);
      const R e2 = p[4] * E2, e3 = R(-2) * p[4] * E3;
      g.du[0] = E1;
      g.du[1] = p[2] * e1;
      g.du[2] = (p[1] - r) * e1;
      g.du[3] = -r6;
      g.du[4] = E2 - R(2) * E3;
      g.du[5] = -d6 * (R(2) * e2 + e3);
      g.du[6] = p[5] * (R(2) * e2 + e3);
      g.df[0] = r_r * p[2] * E1;
      g.df[1] = r_r * p[2] * p[2] * e1;
      g.df[2] = r_r * e1 * (R(1) + p[2] * (p[1] - r));
      g.df[3] = R(-6) * rs_r * r6;
      g.df[4] = R(2) * p[5] * r_r * (E2 - E3);
      g.df[5] = r_r * (R(2) * e2 + e3 - d6 * p[5] * (R(4) * e2 + e3));
      g.df[6] = r_r * p[5] * p[5] * (R(4) * e2 + e3);
   }
}

template <typename R>
__device__ __forceinline__ R warp_sum(R v)
{
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
   return v;   // valid in lane 0
}

// Gradients of the real-space energy and of G = sum_i v_i . F_i (the
// force-matching loss for residual weights v, the Hessian-vector product of
// the loss) with respect to the potential table, the site charges and
// alpha.  The same stencil walk as k_pairs, recomputed (no stored pair
// list), with the walk repeated once per partner site identifier b so that
// every lane accumulates the table entries (id_i, b, k) in registers.
//   slots [0, T)      dE/dp(a,b,k) at (a*max_id + b)*NP + k, T = max_id^2 NP
//   slots [T, 2T)     dG/dp(a,b,k)
//   slots 2T, 2T+1    dE/dalpha, dG/dalpha
//   gq[oi], gq[N+oi]  dE/dq, dG/dq of the home site (written, not added)
// The table entry (a, b) is the one the force on a site of id a from a site
// of id b reads; each ordered evaluation carries half the pair energy.
// Intramolecular pairs are left out of the energy terms (the
// intramolecular correction removes them again); the forces keep them.
// Persistent blocks: each warp takes home slots blockIdx.x*PAIR_WARPS + w,
// stepping by the grid; per-block slot sums are written to gpart.
template <int PT, bool EW, bool MIXED>
__global__ void __launch_bounds__(PAIR_WARPS * 32)
k_pairs_adj(RsParams P, AdjParams A, const int *__restrict__ cell_start,
            const int *__restrict__ slot_cell, const int4 *__restrict__ full,
            const float4 *__restrict__ off_hi, const float4 *__restrict__ off_lo,
            const double4 *__restrict__ pos64, const float4 *__restrict__ pos32,
            const int2 *__restrict__ tag, const int *__restrict__ sorted,
            const double *__restrict__ site, const double *__restrict__ potg64,
            const float *__restrict__ potg32, const double4 *__restrict__ res64,
            const float4 *__restrict__ res32, double *__restrict__ gq, double *__restrict__ gpart)
{
   typedef typename std::conditional<MIXED, float, double>::type R;
   constexpr int NP = NPar<PT>::v;
   extern __shared__ double s_acc[];
   __shared__ int s_inc[PAIR_WARPS][32 * WALK_E], s_jb[PAIR_WARPS][32 * WALK_E], s_info[PAIR_WARPS][32 * WALK_E];
   for (int q = threadIdx.x; q < A.nslot; q += blockDim.x) s_acc[q] = 0.0;
   __syncthreads();
   const R *pot = MIXED ? (const R *)(const void *)potg32 : (const R *)(const void *)potg64;
   const int N = P.nsites, T = P.max_id * P.max_id * NP;
   const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const WalkRows rows{s_inc[w], s_jb[w], s_info[w], off_hi, off_lo};
   const R alpha = MIXED ? (R)P.alphaf : (R)P.alpha, norm = MIXED ? (R)P.normf : (R)P.norm;
   const R cut100 = (R)P.cut100;
   for (int p0 = blockIdx.x * PAIR_WARPS; p0 < N; p0 += gridDim.x * PAIR_WARPS) {
      const int p = p0 + w;
      if (p >= N) break;
      const int c = slot_cell[p];
      const int2 ti = tag[p];
      double4 xi64 = make_double4(0, 0, 0, 0);
      float4 xi32 = make_float4(0, 0, 0, 0);
      if (MIXED) xi32 = pos32[p]; else xi64 = pos64[p];
      const R qi = MIXED ? (R)xi32.w : (R)xi64.w;
      R vix = 0, viy = 0, viz = 0;
      if (A.loss) {
         if (MIXED) {
            const float4 v = res32[p];
            vix = v.x; viy = v.y; viz = v.z;
         } else {
            const double4 v = res64[p];
            vix = v.x; viy = v.y; viz = v.z;
         }
      }
      const int oi = sorted[p];
      R gqe = 0, gql = 0, gae = 0, gal = 0;
      for (int b = 0; b < P.max_id; b++) {
         if (!((A.type_mask >> b) & 1u)) continue;
         R pp[NP], ge[NP], gl[NP];
         const R *pj = pot + ((size_t)ti.x * P.max_id + b) * NPOTP;
#pragma unroll
         for (int q = 0; q < NP; q++) {
            pp[q] = pj[q];
            ge[q] = gl[q] = R(0);
         }
         walk_stencil<MIXED>(P, p, c, lane, cell_start, full, off_hi, off_lo, rows, [&](int j, int k, int kimg) {
            const int2 tj = __ldg(&tag[j]);
            if (tj.x != b || (ti.y == P.fw_mol && tj.y == P.fw_mol)) return;
            R rx, ry, rz, r2, qj;
            pair_sep<MIXED>(P, j, k, kimg, rows, xi32, xi64, pos64, pos32, rx, ry, rz, r2, qj);
            bool too_close, clip;
            pair_flags<MIXED>(P, r2, oi, j, kimg, sorted, site, too_close, clip);
            if (clip) r2 = cut100;
            PairGrad<NP, R> g;
            pair_grad<PT, EW, R>(r2, pp, alpha, norm, g);
            if (ti.y != tj.y) {
#pragma unroll
               for (int q = 0; q < NP; q++) ge[q] += g.du[q];
               gqe += qj * g.uc;
               gae += qj * g.duc;
            }
            if (A.loss) {
               R vjx, vjy, vjz;
               if (MIXED) {
                  const float4 v = __ldg(&res32[j]);
                  vjx = v.x; vjy = v.y; vjz = v.z;
               } else {
                  const double4 v = res64[j];
                  vjx = v.x; vjy = v.y; vjz = v.z;
               }
               const R wi = vix * rx + viy * ry + viz * rz;            // v_i . r
               const R ws = wi - (vjx * rx + vjy * ry + vjz * rz);      // (v_i - v_j) . r
#pragma unroll
               for (int q = 0; q < NP; q++) gl[q] -= g.df[q] * wi;
               gql -= qj * g.fc * ws;
               gal -= qj * g.dfc * wi;
            }
         });
         double *se = s_acc + ((size_t)ti.x * P.max_id + b) * NP;
#pragma unroll
         for (int q = 0; q < NP; q++) {
            const R s = warp_sum(ge[q]);
            if (lane == 0) atomicAdd(se + q, 0.5 * (double)s);
         }
         if (A.loss) {
#pragma unroll
            for (int q = 0; q < NP; q++) {
               const R s = warp_sum(gl[q]);
               if (lane == 0) atomicAdd(se + T + q, (double)s);
            }
         }
      }
      gqe = warp_sum(gqe);
      gql = warp_sum(gql);
      gae = warp_sum(gae);
      gal = warp_sum(gal);
      if (lane == 0) {
         gq[oi] = (double)gqe;
         gq[N + oi] = (double)gql;
         atomicAdd(s_acc + 2 * T, 0.5 * (double)qi * (double)gae);
         atomicAdd(s_acc + 2 * T + 1, (double)qi * (double)gal);
      }
   }
   __syncthreads();
   for (int q = threadIdx.x; q < A.nslot; q += blockDim.x) gpart[(size_t)blockIdx.x * A.nslot + q] = s_acc[q];
}

// Slot sums over blocks, in block order.
__global__ void k_adj_slots(const double *__restrict__ gpart, int nblocks, int nslot, double *__restrict__ slots)
{
   const int q = blockIdx.x * blockDim.x + threadIdx.x;
   if (q >= nslot) return;
   double s = 0.0;
   for (int b = 0; b < nblocks; b++) s += gpart[(size_t)b * nslot + q];
   slots[q] = s;
}

// --------------------------------------------------------------------- RDF
// Site-pair distance histogram (rdf_inner + rdf_accum, src/force.c:1010-1103,
// src/rdf.c:94-107): the same warp-per-site walk over the strict stencil at
// the RDF limit, r^2 in FP64 with the reference's operation order from the
// original co-ordinates, bin = (int)(rbin sqrt(r^2)) kept when < nbins.
// Counts per (id_i, id_j, bin) in a shared-memory histogram per block when it
// fits (HIST_SMEM), else directly in global memory.
constexpr int HIST_SMEM = 8192;

__global__ void __launch_bounds__(PAIR_WARPS * 32)
k_rdf(RsParams P, const int *__restrict__ cell_start, const int *__restrict__ slot_cell,
      const int4 *__restrict__ full, const int2 *__restrict__ tag, const int *__restrict__ sorted,
      const double *__restrict__ site, double rbin, int nbins, unsigned long long *__restrict__ counts)
{
   __shared__ unsigned int hist[HIST_SMEM];
   __shared__ int s_inc[PAIR_WARPS][32 * WALK_E], s_jb[PAIR_WARPS][32 * WALK_E], s_info[PAIR_WARPS][32 * WALK_E];
   const int nh = P.max_id * P.max_id * nbins;
   const bool in_smem = nh <= HIST_SMEM;
   if (in_smem)
      for (int q = threadIdx.x; q < nh; q += blockDim.x) hist[q] = 0u;
   __syncthreads();
   const int N = P.nsites;
   const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int p = blockIdx.x * PAIR_WARPS + w;
   const WalkRows rows{s_inc[w], s_jb[w], s_info[w], nullptr, nullptr};
   if (p < N) {
      const int c = slot_cell[p];
      const int oi = sorted[p];
      const int2 ti = tag[p];
      const int idi = ti.x;
      const double xi = site[oi], yi = site[N + oi], zi = site[2 * N + oi];
      walk_stencil<false>(P, p, c, lane, cell_start, full, nullptr, nullptr, rows, [&](int j, int, int kimg) {
         if (ti.y == P.fw_mol && __ldg(&tag[j]).y == P.fw_mol) return;
         const int oj = sorted[j];
         const double *rl = P.reloc[kimg];
         const double rx = __dadd_rn(__dsub_rn(site[oj], xi), rl[0]);
         const double ry = __dadd_rn(__dsub_rn(site[N + oj], yi), rl[1]);
         const double rz = __dadd_rn(__dsub_rn(site[2 * N + oj], zi), rl[2]);
         const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
         const int bin = __double2int_rz(__dmul_rn(rbin, sqrt(r2)));
         if (bin < nbins) {
            const int q = (idi * P.max_id + __ldg(&tag[j]).x) * nbins + bin;
            if (in_smem)
               atomicAdd(&hist[q], 1u);
            else
               atomicAdd(&counts[q], 1ull);
         }
      });
   }
   __syncthreads();
   if (in_smem)
      for (int q = threadIdx.x; q < nh; q += blockDim.x)
         if (hist[q]) atomicAdd(&counts[q], (unsigned long long)hist[q]);
}

// -------------------------------------------------------------- host side
static RsParams make_params(mdgpu_ctx *c)
{
   RsParams P;
   memset(&P, 0, sizeof P);
   const RsGeom &g = c->rs;
   P.nsites = c->nsites;
   P.fw_mol = c->fw_mol;
   P.fw_site0 = c->fw_site0;
   P.nmol_ent = c->nmols_nf;
   P.nent = c->ctl.molpbc ? c->nmols_nf + (c->nsites - c->fw_site0) : c->nsites;
   P.nx = g.nx; P.ny = g.ny; P.nz = g.nz; P.ncells = g.ncells;
   P.rn[0] = 1.0 / g.nx; P.rn[1] = 1.0 / g.ny; P.rn[2] = 1.0 / g.nz;
   P.nfull = (int)g.full.size();
   P.ncols = (int)g.cols.size();
   P.max_id = c->max_id;
   P.molpbc = c->ctl.molpbc;
   P.strict = c->ctl.strict_cutoff;
   P.ptype = c->ptype;
   for (int i = 0; i < 9; i++) P.hinv[i] = g.hinv[i];
   for (int i = 0; i < 9; i++) P.h[i] = g.h[i];
   for (int k = 0; k < 27; k++)
      for (int r = 0; r < 3; r++) P.reloc[k][r] = g.reloc[k][r];
   P.cut2 = g.cut2;
   P.cut100 = g.cut100;
   P.alpha = c->ctl.alpha;
   P.norm = 2.0 * c->ctl.alpha / sqrt(PI);
   P.cut2f = (float)g.cut2;
   P.bandf = 1e-4f;
   P.alphaf = (float)P.alpha;
   P.normf = (float)P.norm;
   return P;
}

mdgpu_status rs_prepare(mdgpu_ctx *c)
{
   RsDev &d = c->rd;
   const RsGeom &g = c->rs;
   const int N = c->nsites;
   cudaStream_t st = c->stream;
#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_check(c, e_, #x); } while (0)
   if (c->sys_dirty) {
      CK(d.siteid.ensure(N));
      CK(d.molmap.ensure(N));
      CK(d.chg.ensure(N));
      CK(d.ent_mol.ensure(2 * (size_t)c->nmols));
      CK(cudaMemcpyAsync(d.siteid.p, c->site_id.data(), N * sizeof(int), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.molmap.p, c->molmap.data(), N * sizeof(int), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.chg.p, c->chg.data(), N * sizeof(double), cudaMemcpyHostToDevice, st));
      std::vector<int> mf(2 * (size_t)c->nmols);
      for (int m = 0; m < c->nmols; m++) {
         mf[m] = c->mol_first[m];
         mf[c->nmols + m] = c->mol_nsites[m];
      }
      CK(cudaMemcpyAsync(d.ent_mol.p, mf.data(), mf.size() * sizeof(int), cudaMemcpyHostToDevice, st));
      const size_t np = (size_t)c->max_id * c->max_id * NPOTP;
      CK(d.pot64.ensure(np));
      CK(d.pot32.ensure(np));
      std::vector<float> p32(np);
      for (size_t i = 0; i < np; i++) p32[i] = (float)c->potpar[i];
      CK(cudaMemcpyAsync(d.pot64.p, c->potpar.data(), np * sizeof(double), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.pot32.p, p32.data(), np * sizeof(float), cudaMemcpyHostToDevice, st));
      // interaction classes: identifiers joined when they interact (both
      // charged, or a potential with a nonzero parameter either way); the
      // group holding the charged identifiers (else the most populous) is
      // class 0, every other group class 1
      {
         const int M = c->max_id, npar = pot_nparams(c->ptype);
         std::vector<int> grp(M), pop(M, 0);
         std::vector<char> charged(M, 0);
         for (int i = 0; i < N; i++) {
            pop[c->site_id[i]]++;
            if (c->chg[i] != 0.0) charged[c->site_id[i]] = 1;
         }
         for (int a = 0; a < M; a++) grp[a] = a;
         auto root = [&](int a) { while (grp[a] != a) a = grp[a] = grp[grp[a]]; return a; };
         for (int a = 0; a < M; a++)
            for (int b = 0; b < M; b++) {
               bool link = charged[a] && charged[b];
               for (int k = 0; k < npar && !link; k++)
                  link = c->potpar[((size_t)a * M + b) * NPOTP + k] != 0.0;
               if (link) grp[root(a)] = root(b);
            }
         int g0 = -1, best = -1;
         std::vector<int> gpop(M, 0);
         for (int a = 0; a < M; a++) gpop[root(a)] += pop[a];
         for (int a = 0; a < M; a++)
            if (charged[a]) g0 = root(a);
         if (g0 < 0)
            for (int a = 0; a < M; a++)
               if (gpop[root(a)] > best) best = gpop[g0 = root(a)];
         c->cls_of_id.assign(2 * (size_t)M, 0);   // second half: every identifier in class 0
         c->ncls = 1;
         for (int a = 0; a < M; a++)
            if (pop[a] > 0 && root(a) != g0) {
               c->cls_of_id[a] = 1;
               c->ncls = 2;
            }
         for (int a = 0; a < M; a++)
            if (pop[a] == 0) c->cls_of_id[a] = 0;
         CK(d.cls_of_id.ensure(2 * (size_t)M));
         CK(cudaMemcpyAsync(d.cls_of_id.p, c->cls_of_id.data(), 2 * (size_t)M * sizeof(int),
                            cudaMemcpyHostToDevice, st));
      }
      CK(cudaStreamSynchronize(st));
      CK(d.cell_of.ensure(N));
      CK(d.sorted.ensure(N));
      CK(d.pos64.ensure(N));
      CK(d.pos32.ensure(N));
      CK(d.tag.ensure(N));
      CK(d.slot_cell.ensure(N));
   }
   if (c->rs_valid && !c->rs_uploaded) {
      CK(d.cell_count.ensure(g.ncells + 1));
      CK(d.cell_start.ensure(g.ncells + 1));
      CK(d.blocksum.ensure((g.ncells + 1 + 1023) / 1024 + 2));
      CK(d.full.ensure(g.full.size()));
      CK(d.off_hi.ensure(g.full.size()));
      CK(d.off_lo.ensure(g.full.size()));
      CK(cudaMemcpyAsync(d.full.p, g.full.data(), g.full.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.off_hi.p, g.off_hi.data(), g.off_hi.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.off_lo.p, g.off_lo.data(), g.off_lo.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
      CK(d.cols.ensure(g.cols.size()));
      CK(d.col_base.ensure(g.col_base.size()));
      std::vector<float4> coff(2 * g.coff_hi.size());
      for (size_t e = 0; e < g.coff_hi.size(); e++) {
         coff[2 * e] = g.coff_hi[e];
         coff[2 * e + 1] = g.coff_lo[e];
      }
      CK(d.coff.ensure(coff.size()));
      CK(cudaMemcpyAsync(d.cols.p, g.cols.data(), g.cols.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.col_base.p, g.col_base.data(), g.col_base.size() * sizeof(int), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.coff.p, coff.data(), coff.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
      CK(d.cs.ensure(2 * ((size_t)g.ncells + 1)));
      CK(cudaStreamSynchronize(st));
      c->rs_uploaded = true;
   }
   const int nb = (N + PAIR_WARPS - 1) / PAIR_WARPS;
   CK(d.part.ensure((size_t)nb * 8));
   if (c->sys_dirty) {
      CK(d.cls_pre.ensure((size_t)N + 1));
      CK(d.cls_bsum.ensure(((size_t)N + 1 + 1023) / 1024 + 2));
      CK(d.sortc.ensure(N));
      CK(d.cellc.ensure(N));
      CK(d.posc.ensure(N));
      CK(d.tagc.ensure(N));
   }
   return MDGPU_OK;
}

template <int PT, bool EW, bool MIXED, int MODE>
static cudaError_t launch_pairs_t(const RsParams &P, mdgpu_ctx *c, double *force, DevOut *out,
                                  unsigned long long *keys, long long key_cap, size_t smem)
{
   RsDev &d = c->rd;
   const int nb = (P.nsites + PAIR_WARPS - 1) / PAIR_WARPS;
   auto kfn = k_pairs<PT, EW, MIXED, MODE>;
   if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   kfn<<<nb, PAIR_WARPS * 32, smem, c->stream>>>(P, d.cell_start.p, d.slot_cell.p, d.full.p, d.off_hi.p, d.off_lo.p,
                                     d.pos64.p, d.pos32.p, d.tag.p, d.sorted.p, c->cur_site,
                                     d.pot64.p, d.pot32.p, d.chg.p, force, d.part.p, out, keys, key_cap);
   return cudaGetLastError();
}

template <int PT>
static cudaError_t launch_pairs_pt(const RsParams &P, mdgpu_ctx *c, bool ew, bool mixed, int mode,
                                   double *force, DevOut *out, unsigned long long *keys,
                                   long long key_cap, size_t smem)
{
   if (mode == 1) return launch_pairs_t<PT, false, false, 1>(P, c, force, out, keys, key_cap, smem);
   if (mixed)
      return ew ? launch_pairs_t<PT, true, true, 0>(P, c, force, out, keys, key_cap, smem)
                : launch_pairs_t<PT, false, true, 0>(P, c, force, out, keys, key_cap, smem);
   return ew ? launch_pairs_t<PT, true, false, 0>(P, c, force, out, keys, key_cap, smem)
             : launch_pairs_t<PT, false, false, 0>(P, c, force, out, keys, key_cap, smem);
}

template <int PT, bool EW, bool MIXED>
static cudaError_t launch_adj_t(const RsParams &P, const AdjParams &A, mdgpu_ctx *c, int nblk)
{
   RsDev &d = c->rd;
   AdjDev &a = c->ad;
   k_pairs_adj<PT, EW, MIXED><<<nblk, PAIR_WARPS * 32, A.nslot * sizeof(double), c->stream>>>(
      P, A, d.cell_start.p, d.slot_cell.p, d.full.p, d.off_hi.p, d.off_lo.p, d.pos64.p, d.pos32.p, d.tag.p,
      d.sorted.p, c->cur_site, d.pot64.p, d.pot32.p, a.res64.p, a.res32.p, a.gq.p, a.gpart.p);
   return cudaGetLastError();
}

template <int PT>
static cudaError_t launch_adj_pt(const RsParams &P, const AdjParams &A, mdgpu_ctx *c, bool ew, bool mixed,
                                 int nblk)
{
   if (mixed)
      return ew ? launch_adj_t<PT, true, true>(P, A, c, nblk) : launch_adj_t<PT, false, true>(P, A, c, nblk);
   return ew ? launch_adj_t<PT, true, false>(P, A, c, nblk) : launch_adj_t<PT, false, false>(P, A, c, nblk);
}

int pot_nparams(int ptype)
{
   switch (ptype) {
   case 0: return NPar<0>::v;
   case 1: return NPar<1>::v;
   case 2: return NPar<2>::v;
   case 3: return NPar<3>::v;
   case 4: return NPar<4>::v;
   case 6: return NPar<6>::v;
   default: return 0;
   }
}

mdgpu_status rs_adjoint(mdgpu_ctx *c, bool loss)
{
   AdjDev &a = c->ad;
   cudaStream_t st = c->stream;
   RsParams P = make_params(c);
   const int N = c->nsites;
   const bool mixed = c->prec == MDGPU_MIXED;
   const int np = pot_nparams(c->ptype);
   AdjParams A;
   A.loss = loss ? 1 : 0;
   A.type_mask = 0;
   for (int id : c->site_id) A.type_mask |= 1u << id;
   A.nslot = 2 * c->max_id * c->max_id * np + 2;
   int nblk = (N + PAIR_WARPS - 1) / PAIR_WARPS;
   if (nblk > 4 * 152) nblk = 4 * 152;
   CK(a.gq.ensure(2 * (size_t)N));
   CK(a.gpart.ensure((size_t)nblk * A.nslot));
   CK(a.slots.ensure((size_t)A.nslot));
   const bool ew = c->ctl.alpha > 0.0;
   cudaError_t e;
   switch (c->ptype) {
   case 0: e = launch_adj_pt<0>(P, A, c, ew, mixed, nblk); break;
   case 1: e = launch_adj_pt<1>(P, A, c, ew, mixed, nblk); break;
   case 2: e = launch_adj_pt<2>(P, A, c, ew, mixed, nblk); break;
   case 3: e = launch_adj_pt<3>(P, A, c, ew, mixed, nblk); break;
   case 4: e = launch_adj_pt<4>(P, A, c, ew, mixed, nblk); break;
   case 6: e = launch_adj_pt<6>(P, A, c, ew, mixed, nblk); break;
   default: return fail(c, MDGPU_E_PTYPE, "KERNEL called with unknown potential type");
   }
   CK(e);
   k_adj_slots<<<(A.nslot + 255) / 256, 256, 0, st>>>(a.gpart.p, nblk, A.nslot, a.slots.p);
   CK(cudaGetLastError());
   c->launches += 2;
   return MDGPU_OK;
}

mdgpu_status rs_rdf(mdgpu_ctx *c, double limit, int nbins)
{
   RsDev &d = c->rd;
   const RsGeom &g = c->rs;
   cudaStream_t st = c->stream;
   if (!(limit > 0.0) || nbins <= 0) return fail(c, MDGPU_E_ARG, "RDF limit and bin count must be positive");
   double key[11];
   std::memcpy(key, g.h, 9 * sizeof(double));
   key[9] = limit;
   key[10] = (double)(g.nx + 1000 * (g.ny + 1000 * g.nz));
   if (d.rdf_nfull == 0 || std::memcmp(key, d.rdf_key, sizeof key) != 0) {
      std::vector<int4> full;
      mdgpu_status s = build_rdf_stencil(g.h, limit, g.nx, g.ny, g.nz, full);
      if (s == MDGPU_E_CUTOFF)
         return fail(c, s, "RDF limit > 1 * cell dimension (neighbour cells beyond one image)");
      if (s) return fail(c, s, "RDF stencil");
      CK(d.rdf_full.ensure(full.size()));
      CK(cudaMemcpyAsync(d.rdf_full.p, full.data(), full.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
      d.rdf_nfull = (int)full.size();
      std::memcpy(d.rdf_key, key, sizeof key);
   }
   const size_t nh = (size_t)c->max_id * c->max_id * nbins;
   CK(d.rdf_counts.ensure(nh));
   CK(cudaMemsetAsync(d.rdf_counts.p, 0, nh * sizeof(unsigned long long), st));
   RsParams P = make_params(c);
   P.nfull = d.rdf_nfull;
   const double rbin = (double)nbins / limit;   // src/rdf.c:99
   const int N = c->nsites;
   k_rdf<<<(N + PAIR_WARPS - 1) / PAIR_WARPS, PAIR_WARPS * 32, 0, st>>>(
      P, d.cell_start.p, d.slot_cell.p, d.rdf_full.p, d.tag.p, d.sorted.p, c->cur_site, rbin, nbins, d.rdf_counts.p);
   CK(cudaGetLastError());
   c->launches += 1;
   return MDGPU_OK;
}

mdgpu_status rs_launch(mdgpu_ctx *c, const double *d_site, const double *d_cofm, double *d_force,
                       bool cells_only, unsigned long long *d_keys, int64_t key_cap,
                       cudaEvent_t sorted_ready)
{
   RsDev &d = c->rd;
   const RsGeom &g = c->rs;
   cudaStream_t st = c->stream;
   RsParams P = make_params(c);
   const int N = c->nsites;
   DevOut *out = c->out.p;
   c->cur_site = d_site;
   phase_mark(c, MDGPU_PH_CELLS);
   CK(cudaMemsetAsync(d.cell_count.p, 0, (g.ncells + 1) * sizeof(int), st));
   const int nent = P.nent;
   k_bin<<<(nent + 255) / 256, 256, 0, st>>>(P, d_site, d_cofm, d.ent_mol.p, d.ent_mol.p + c->nmols,
                                             d.cell_of.p, d.cell_count.p, out);
   const int n = g.ncells + 1, nbs = (n + 1023) / 1024;
   k_scan_blocks<<<nbs, 1024, 0, st>>>(d.cell_count.p, d.cell_start.p, d.blocksum.p, n);
   k_scan_sums<<<1, 1024, 0, st>>>(d.blocksum.p, nbs, d.blocksum.p + nbs);
   k_scan_add<<<nbs, 1024, 0, st>>>(d.cell_start.p, d.blocksum.p, n);
   CK(cudaMemsetAsync(d.cell_count.p, 0, (g.ncells + 1) * sizeof(int), st));
   k_scatter<<<(N + 255) / 256, 256, 0, st>>>(N, d.cell_of.p, d.cell_start.p, d.cell_count.p, d.sorted.p);
   k_cellsort<<<(g.ncells + 255) / 256, 256, 0, st>>>(g.ncells, d.cell_start.p, d.sorted.p);
   // the link-cell order is all the k-space passes need from here
   if (sorted_ready) CK(cudaEventRecord(sorted_ready, st));
   const bool mixed = c->prec == MDGPU_MIXED && d_keys == nullptr;
   k_gather<<<(N + 255) / 256, 256, 0, st>>>(P, d_site, d.chg.p, d.siteid.p, d.molmap.p, d.sorted.p,
                                             d.cell_of.p, mixed ? nullptr : d.pos64.p,
                                             mixed ? d.pos32.p : nullptr, d.tag.p, d.slot_cell.p);
   CK(cudaGetLastError());
   c->launches += 7;
   phase_mark(c, MDGPU_PH_PAIRS);
   if (cells_only) return MDGPU_OK;
   return rs_pairs(c, d_force, d_keys, key_cap);
#undef CK
}

// The column walk serves the mixed form without a framework molecule or
// molecular cut-off, where every stencil column wraps the cell at most once.
static bool col_walk_ok(const mdgpu_ctx *c)
{
   static const bool off = [] {
      const char *e = std::getenv("MDGPU_PAIRS_COLUMNS");
      return e && e[0] == '0';
   }();
   return !off && c->rs.cols_ok && c->fw_mol < 0 && !c->ctl.molpbc && c->nsites < (1 << 24) &&
          c->max_id < (1 << 16) && c->rs.cols.size() > 0;
}

template <int PT, bool EW>
static cudaError_t launch_col_t(const RsParams &P, mdgpu_ctx *c, double *force, size_t smem, int nb)
{
   RsDev &d = c->rd;
   auto kfn = k_pairs_col<PT, EW>;
   if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   kfn<<<nb, PAIR_WARPS * 32, smem, c->stream>>>(P, d.cell_start.p, d.cs.p, d.cls_pre.p, d.cols.p, d.col_base.p,
                                                 d.coff.p, d.posc.p, d.tagc.p, d.cellc.p,
                                                 d.sortc.p, c->cur_site, d.pot32.p, force, d.part.p, c->out.p);
   return cudaGetLastError();
}

// Class split of the binned slots, the column-walk pair kernel and, with
// two classes, the too-close scan across them.
static mdgpu_status rs_pairs_col(mdgpu_ctx *c, const RsParams &P, double *d_force, bool ew, size_t smem)
{
#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_check(c, e_, #x); } while (0)
   RsDev &d = c->rd;
   cudaStream_t st = c->stream;
   const int N = c->nsites, M = c->max_id;
   const bool two = c->ncls == 2 && c->rs.nbr27;
   const int *cls = d.cls_of_id.p + (two ? 0 : M);
   const int n1 = N + 1, nbs = (n1 + 1023) / 1024;
   k_cls_flag<<<(n1 + 255) / 256, 256, 0, st>>>(N, d.tag.p, cls, d.cls_pre.p);
   k_scan_blocks<<<nbs, 1024, 0, st>>>(d.cls_pre.p, d.cls_pre.p, d.cls_bsum.p, n1);
   k_scan_sums<<<1, 1024, 0, st>>>(d.cls_bsum.p, nbs, d.cls_bsum.p + nbs);
   k_scan_add<<<nbs, 1024, 0, st>>>(d.cls_pre.p, d.cls_bsum.p, n1);
   const int nsplit = std::max(N, P.ncells + 1);
   k_cls_split<<<(nsplit + 255) / 256, 256, 0, st>>>(P, d.cls_pre.p, cls, d.cell_start.p, d.pos32.p, d.tag.p,
                                                    d.sorted.p, d.slot_cell.p, d.cs.p, d.posc.p, d.tagc.p,
                                                    d.sortc.p, d.cellc.p);
   CK(cudaGetLastError());
   c->launches += 5;
   // eight resident blocks per SM (the kernel's launch bounds), each warp
   // looping over home sites: the per-block set-up and energy reduction once
   // per block instead of once per four sites
   if (c->nsm <= 0) CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device));
   const int nb = std::min((N + PAIR_WARPS - 1) / PAIR_WARPS, 8 * c->nsm);
   c->rs_nblk = nb;
   cudaError_t e;
   switch (c->ptype) {
   case 0: e = ew ? launch_col_t<0, true>(P, c, d_force, smem, nb) : launch_col_t<0, false>(P, c, d_force, smem, nb); break;
   case 1: e = ew ? launch_col_t<1, true>(P, c, d_force, smem, nb) : launch_col_t<1, false>(P, c, d_force, smem, nb); break;
   case 2: e = ew ? launch_col_t<2, true>(P, c, d_force, smem, nb) : launch_col_t<2, false>(P, c, d_force, smem, nb); break;
   case 3: e = ew ? launch_col_t<3, true>(P, c, d_force, smem, nb) : launch_col_t<3, false>(P, c, d_force, smem, nb); break;
   case 4: e = ew ? launch_col_t<4, true>(P, c, d_force, smem, nb) : launch_col_t<4, false>(P, c, d_force, smem, nb); break;
   case 6: e = ew ? launch_col_t<6, true>(P, c, d_force, smem, nb) : launch_col_t<6, false>(P, c, d_force, smem, nb); break;
   default: return fail(c, MDGPU_E_PTYPE, "KERNEL called with unknown potential type");
   }
   CK(e);
   c->launches += 1;
   if (two) {
      NbCols nb;
      for (int k = 0; k < 9; k++) nb.col[k] = c->rs.nbcol[k];
      k_tooclose_x<<<(9 * N + 255) / 256, 256, 0, st>>>(P, nb, d.cs.p, d.cls_pre.p, d.cols.p, d.col_base.p, d.coff.p,
                                                    d.posc.p, d.tagc.p, d.cellc.p, d.sortc.p,
                                                    c->cur_site, c->out.p);
      CK(cudaGetLastError());
      c->launches += 1;
   }
   return MDGPU_OK;
#undef CK
}

mdgpu_status rs_count_pairs(mdgpu_ctx *c)
{
#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_check(c, e_, #x); } while (0)
   if (!c->npairs_pending) return MDGPU_OK;
   const RsParams P = make_params(c);
   cudaStream_t st = c->stream;
   DevOut *out = c->out.p;
   CK(cudaMemsetAsync(&out->npairs2, 0, sizeof(out->npairs2), st));
   k_count_col<<<(c->nsites + 255) / 256, 256, 0, st>>>(P, c->rd.cell_start.p, c->rd.cols.p, c->rd.cellc.p, out);
   CK(cudaGetLastError());
   int64_t n2 = 0;
   CK(cudaMemcpyAsync(&n2, &out->npairs2, sizeof(n2), cudaMemcpyDeviceToHost, st));
   CK(cudaStreamSynchronize(st));
   c->info.npairs = n2 / 2;
   c->npairs_pending = false;
   return MDGPU_OK;
#undef CK
}

mdgpu_status rs_pairs(mdgpu_ctx *c, double *d_force, unsigned long long *d_keys, int64_t key_cap)
{
#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_check(c, e_, #x); } while (0)
   RsDev &d = c->rd;
   cudaStream_t st = c->stream;
   RsParams P = make_params(c);
   const int N = c->nsites;
   DevOut *out = c->out.p;
   const bool mixed = c->prec == MDGPU_MIXED && d_keys == nullptr;
   const size_t potb = (size_t)c->max_id * c->max_id * NPOTP * (mixed ? sizeof(float) : sizeof(double));
   P.pot_in_smem = potb <= 96 * 1024;
   const size_t smem = P.pot_in_smem ? potb : 0;
   const bool ew = c->ctl.alpha > 0.0;
   const int mode = d_keys ? 1 : 0;
   cudaError_t e;
   c->npairs_pending = false;
   c->rs_nblk = (N + PAIR_WARPS - 1) / PAIR_WARPS;   // blocks of partial sums for the reduction
   if (mode == 0 && mixed && col_walk_ok(c)) {
      const mdgpu_status s = rs_pairs_col(c, P, d_force, ew, smem);
      if (s != MDGPU_OK) return s;
      c->npairs_pending = true;   // counted on demand (rs_count_pairs)
   } else {
   switch (c->ptype) {
   case 0: e = launch_pairs_pt<0>(P, c, ew, mixed, mode, d_force, out, d_keys, key_cap, smem); break;
   case 1: e = launch_pairs_pt<1>(P, c, ew, mixed, mode, d_force, out, d_keys, key_cap, smem); break;
   case 2: e = launch_pairs_pt<2>(P, c, ew, mixed, mode, d_force, out, d_keys, key_cap, smem); break;
   case 3: e = launch_pairs_pt<3>(P, c, ew, mixed, mode, d_force, out, d_keys, key_cap, smem); break;
   case 4: e = launch_pairs_pt<4>(P, c, ew, mixed, mode, d_force, out, d_keys, key_cap, smem); break;
   case 6: e = launch_pairs_pt<6>(P, c, ew, mixed, mode, d_force, out, d_keys, key_cap, smem); break;
   default: return fail(c, MDGPU_E_PTYPE, "KERNEL called with unknown potential type");
   }
   CK(e);
   c->launches += 1;
   }
   if (mode == 0) {
      if (c->rs_nblk <= 8 * 256) {
         k_reduce_rs1<<<1, 256, 0, st>>>(d.part.p, c->rs_nblk, out);
         c->launches += 1;
      } else {
         CK(d.part2.ensure(8 * RS_RED));
         k_reduce_rs<<<RS_RED, 256, 0, st>>>(d.part.p, c->rs_nblk, d.part2.p);
         k_reduce_rs2<<<1, 256, 0, st>>>(d.part2.p, RS_RED, out);
         c->launches += 2;
      }
      CK(cudaGetLastError());
   }
   phase_mark(c, MDGPU_PH_KPREP);
   return MDGPU_OK;
#undef CK
}

}  // namespace mdgpu
