// Reciprocal space of the mixed form on the tensor cores (tcgen05).  This
// part: the S(k) pass of ewald() (src/ewald.c:124-141, the sums of q cos(k.r)
// and q sin(k.r) over sites, 523-533) as a complex matrix product; the force
// pass (src/ewald.c:557-566) follows further down.
//
// A tensor-core item is a run of up to KT = 64 consecutive l values of one
// (h,k) column.  For item i, site j and offset t,
//     exp(i k.r_j) = seed_ij z_j(t),  seed_ij = exp(2 pi i (h u_x + k u_y + l0 u_z)),
//     z_j(t) = exp(2 pi i t u_z)
// with the 32-bit fixed-point phases u of the FP32 path, so
//     S(i, t) = sum_j (q_j seed_ij) z_j(t)
// is a product of an items x sites matrix (computed per stage on the CUDA
// cores: one polynomial sine/cosine per item and site, amortised over up to
// 64 k-vectors) and a sites x t matrix (the per-site z tables, built once
// per evaluation).  Complex arithmetic as real MMAs of N = 128: Ar and Ai
// each times the whole z operand [Zr | Zi] (rows t, then 64 + t) into D1 =
// (Ar Zr, Ar Zi) and D2 = (Ai Zr, Ai Zi), then Re S = Ar Zr - Ai Zi and
// Im S = Ar Zi + Ai Zr in the read-back.  An MMA of 128 x N x 16 costs one
// issuing thread the same time for any N up to 256 (measured:
// mdgpu_tc_rate), so the products are kept wide and issued by two threads.
//
// Precision.  Charges are scaled by a power of two to |q| < 1, and every
// FP32 operand is split into three bf16 terms on fixed grids (tc.cuh): the
// hi*hi products go to their own tensor-memory accumulators (D1, D2), where
// their sums are exact (multiples of 2^-14 below 2^10: a 1024-site partial
// of terms of magnitude < 1), so the accumulator's round-toward-zero never
// acts on them; hm, mh, hl, lh and mm go to a second pair, 2^-8 smaller.
// The terms left out and the splitting are within 2^-24 of each operand, as
// for the FP32 path.  Each CTA sums 1024 sites and writes one partial per k;
// the partials are added in compensated FP32 and FP64 by the per-k
// reduction.
//
// CTA roles (608 threads): warps 0-15 build the A operand of each 32-site
// stage (one item row and 8 sites per thread) and, at the end, read the
// accumulators back (a warp reaches tensor-memory lanes 32 (w % 4) ..);
// warp 16 streams each stage's z tables and its 32 site records (bulk
// copies, three stages in flight); warp 17 owns the tensor memory and
// issues the Ar MMAs, warp 18 the Ai MMAs.  A operands and z tables are
// triple-buffered on mbarriers, so the A operand of a stage is built while
// the MMAs of the two before it run; every wait is bounded and sets bit 3
// of the error word when it expires.
#include <atomic>
#include <cmath>

#include "mdgpu_internal.h"
#include "phase.cuh"
#include "tc.cuh"

namespace mdgpu {

constexpr int TC_KS = 32;                          // sites per stage (two MMA K-steps of 16)
constexpr int TC_NSA = 3;                          // A-operand buffers
constexpr int TC_NSB = 3;                          // z-table buffers (bulk copies in flight)
constexpr int TC_TERM = 128 * TC_KS * 2;           // one 128-row bf16 operand of a stage: 8 KB
constexpr int TC_ABYTES = 6 * TC_TERM;             // Ar, Ai x (hi, mid, lo)
constexpr int TC_BBYTES = 3 * TC_TERM;             // [Zr | Zi] x (hi, mid, lo)
constexpr int TC_CHUNK = 1024;                     // sites per CTA (one partial per k)
constexpr int TC_PBYTES = TC_KS * 16;              // a stage's site records (u_x, u_y, u_z, q)
constexpr int TC_AOFF = 0, TC_BOFF = TC_AOFF + TC_NSA * TC_ABYTES, TC_POFF = TC_BOFF + TC_NSB * TC_BBYTES;
constexpr int TC_SMEM = TC_POFF + TC_NSB * TC_PBYTES;
constexpr int TC_LBO = 16 * 128;                   // 8-column groups of a 128-row operand
constexpr int TC_ERR = 8;                          // error-word bit: a stage wait expired
constexpr int TC_AW = 16;                          // operand / read-back warps
constexpr int TC_THREADS = 32 * (TC_AW + 3);       // and a bulk-copy warp, two MMA warps

static_assert(TC_AOFF % 1024 == 0 && TC_BOFF % 1024 == 0 && TC_POFF % 16 == 0, "operand buffers stay aligned");
static_assert(TC_SMEM <= 227 * 1024, "one CTA's shared memory");
static_assert(TC_CHUNK % TC_KS == 0, "chunks hold whole stages");
static_assert(KT == 4 * KI && KT <= 64, "an item is four KI runs, Zr and Zi fit 128 rows");

__device__ __forceinline__ void tc_abort(int *flag, int *err, int bit = TC_ERR)
{
   *(volatile int *)flag = 1;
   atomicOr(err, bit);
}

__device__ __forceinline__ bool tc_aborted(const int *flag)
{
   return *(const volatile int *)flag != 0;
}

// Grid: (item tiles of 128, site chunks of TC_CHUNK).  part[chunk][k].
__global__ void __launch_bounds__(TC_THREADS, 1)
k_sfac_tc(const int4 *__restrict__ item, const int4 *__restrict__ item_k0, const int4 *__restrict__ ph,
          const uint4 *__restrict__ ztab, int np, int nk, float qscale, float qunscale, float2 *__restrict__ part,
          int *__restrict__ err)
{
   using namespace tc;
   extern __shared__ __align__(1024) unsigned char sm[];
   __shared__ __align__(8) uint64_t full_b[TC_NSB], empty_b[TC_NSB], full_a[TC_NSA], empty_a[TC_NSA], accf;
   __shared__ unsigned int tmem_s;
   __shared__ int abort_s;
   const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
   const int tile = blockIdx.x, chunk = blockIdx.y;
   const int s0 = chunk * TC_CHUNK;
   const int nst = (min(np, s0 + TC_CHUNK) - s0) / TC_KS;
   const int ncols = (item[tile * 128].w + 15) & ~15;   // the tile's largest count, rounded up
   if (ncols == 0 || nst <= 0) return;                  // (uniform over the CTA)
   if (tid == 0) {
      for (int s = 0; s < TC_NSB; s++) {
         bar_init(&full_b[s], 1);
         bar_init(&empty_b[s], 2);   // released by both MMA issuers
      }
      for (int s = 0; s < TC_NSA; s++) {
         bar_init(&full_a[s], TC_AW);
         bar_init(&empty_a[s], 2);
      }
      bar_init(&accf, 2);
      abort_s = 0;
      bar_init_fence();
   }
   __syncwarp();
   if (w == TC_AW + 1) tmem_alloc(&tmem_s, 512);
   fence_before_sync();
   __syncthreads();
   fence_after_sync();
   const unsigned int tmem = tmem_s;

   if (w == TC_AW) {
      // ---- bulk copies: each stage's z tables and site records
      if (lane == 0) {
         int issued = 0;
         for (int st = 0; st < nst; st++) {
            const int s = st % TC_NSB;
            if (st >= TC_NSB && !bar_wait(&empty_b[s], (unsigned int)(st / TC_NSB - 1) & 1u)) {
               tc_abort(&abort_s, err);
               break;
            }
            if (tc_aborted(&abort_s)) break;
            bar_expect_tx(&full_b[s], TC_BBYTES + TC_PBYTES);
            bulk_load(sm + TC_BOFF + s * TC_BBYTES, ztab + (size_t)(s0 / TC_KS + st) * (TC_BBYTES / 16), TC_BBYTES,
                      &full_b[s]);
            bulk_load(sm + TC_POFF + s * TC_PBYTES, ph + s0 + st * TC_KS, TC_PBYTES, &full_b[s]);
            issued = st + 1;
         }
         // copies still in flight complete before the CTA's shared memory goes
         for (int st = issued > TC_NSB ? issued - TC_NSB : 0; st < issued; st++)
            bar_wait(&full_b[st % TC_NSB], (unsigned int)(st / TC_NSB) & 1u);
      }
   } else if (w == TC_AW + 1 || w == TC_AW + 2) {
      // ---- MMA issue: warp TC_AW + 1 multiplies Ar, warp TC_AW + 2 Ai, by the
      // whole z operand [Zr | Zi] (N = 128) into D1 = (Ar Zr, Ar Zi) and
      // D2 = (Ai Zr, Ai Zi)
      const int ic = w - TC_AW - 1;
      if (lane == 0) {
         const unsigned int idn = idesc_bf16(128, 128, false);
         const int ta[6] = {0, 0, 1, 0, 2, 1}, tb[6] = {0, 1, 0, 2, 0, 1};
         for (int st = 0; st < nst; st++) {
            const int sa = st % TC_NSA, sb = st % TC_NSB;
            if (!bar_wait(&full_a[sa], (unsigned int)(st / TC_NSA) & 1u) ||
                !bar_wait(&full_b[sb], (unsigned int)(st / TC_NSB) & 1u)) {
               tc_abort(&abort_s, err);
               break;
            }
            fence_after_sync();
            const unsigned int a = saddr(sm + TC_AOFF + sa * TC_ABYTES) + 3 * ic * TC_TERM;
            const unsigned int b = saddr(sm + TC_BOFF + sb * TC_BBYTES);
#pragma unroll
            for (int ks = 0; ks < TC_KS / 16; ks++)
#pragma unroll
               for (int p = 0; p < 6; p++)
                  mma_f16(tmem + 128u * ic + (p == 0 ? 0u : 256u),
                           sdesc(a + ta[p] * TC_TERM + ks * 2 * TC_LBO, TC_LBO, 128),
                           sdesc(b + tb[p] * TC_TERM + ks * 2 * TC_LBO, TC_LBO, 128), idn, st > 0 || ks > 0 || p > 1);
            mma_commit(&empty_a[sa]);
            mma_commit(&empty_b[sb]);
         }
         mma_commit(&accf);   // also after an abort: the readers wait on it
      }
   } else {
      // ---- A operand: q_j seed_ij for this thread's item row and the
      // stage's sites 8 qq .. 8 qq + 7 (one column group)
      const int m = tid & 127, qq = tid >> 7;
      const int4 hd = item[tile * 128 + m];
      const unsigned int H = (unsigned int)hd.x, K = (unsigned int)hd.y, L = (unsigned int)hd.z;
      for (int st = 0; st < nst; st++) {
         const int s = st % TC_NSA, sb = st % TC_NSB;
         if (tc_aborted(&abort_s)) break;
         if ((st >= TC_NSA && !bar_wait(&empty_a[s], (unsigned int)(st / TC_NSA - 1) & 1u)) ||
             !bar_wait(&full_b[sb], (unsigned int)(st / TC_NSB) & 1u)) {
            tc_abort(&abort_s, err);
            break;
         }
         unsigned char *A = sm + TC_AOFF + s * TC_ABYTES;
         const int4 *P = reinterpret_cast<const int4 *>(sm + TC_POFF + sb * TC_PBYTES) + 8 * qq;
         unsigned int hr[4], mr[4], lr[4], hi[4], mi[4], li[4];
#pragma unroll
         for (int jp = 0; jp < 4; jp++) {
            const int4 v0 = P[2 * jp], v1 = P[2 * jp + 1];
            f2x sv, cv;   // the two sites as the lanes of paired FP32 instructions
            sincos_poly2(H * (unsigned int)v0.x + K * (unsigned int)v0.y + L * (unsigned int)v0.z,
                         H * (unsigned int)v1.x + K * (unsigned int)v1.y + L * (unsigned int)v1.z, sv, cv);
            const f2x q = pk2(__int_as_float(v0.w) * qscale, __int_as_float(v1.w) * qscale);
            split3(mul2(cv, q), hr[jp], mr[jp], lr[jp]);
            split3(mul2(sv, q), hi[jp], mi[jp], li[jp]);
         }
         unsigned char *row = A + qq * TC_LBO + (m >> 3) * 128 + (m & 7) * 16;
         *reinterpret_cast<uint4 *>(row) = make_uint4(hr[0], hr[1], hr[2], hr[3]);
         *reinterpret_cast<uint4 *>(row + TC_TERM) = make_uint4(mr[0], mr[1], mr[2], mr[3]);
         *reinterpret_cast<uint4 *>(row + 2 * TC_TERM) = make_uint4(lr[0], lr[1], lr[2], lr[3]);
         *reinterpret_cast<uint4 *>(row + 3 * TC_TERM) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
         *reinterpret_cast<uint4 *>(row + 4 * TC_TERM) = make_uint4(mi[0], mi[1], mi[2], mi[3]);
         *reinterpret_cast<uint4 *>(row + 5 * TC_TERM) = make_uint4(li[0], li[1], li[2], li[3]);
         fence_async_smem();
         __syncwarp();
         if (lane == 0) bar_arrive(&full_a[s]);
      }
      // ---- read back: item row m (lane quarter w % 4), t in [16 qq, 16 qq + 16):
      // Re = Ar Zr - Ai Zi, Im = Ar Zi + Ai Zr, each the hh sums plus the rest
      const bool done = bar_wait(&accf, 0);
      const bool ok = __all_sync(0xffffffffu, done && !tc_aborted(&abort_s));
      if (!done && lane == 0) tc_abort(&abort_s, err);
      fence_after_sync();
      const int t0 = 16 * qq;
      if (ok && t0 < ncols) {
         const int4 k0 = item_k0[tile * 128 + m];
         const unsigned int trow = tmem + ((unsigned int)(32 * (w & 3)) << 16) + (unsigned int)t0;
         const int kr = qq == 0 ? k0.x : qq == 1 ? k0.y : qq == 2 ? k0.z : k0.w;
         // column pairs (hh sums, the rest): Ar Zr at t, Ar Zi at 64 + t,
         // Ai Zr at 128 + t, Ai Zi at 192 + t; the rest 256 further on
         auto pair_sum = [&](unsigned int col, float (&out)[16]) {
            float u[16], v[16];
            tmem_ld16(trow + col, u);
            tmem_ld16(trow + col + 256, v);
            tmem_wait2(u, v);
#pragma unroll
            for (int j = 0; j < 16; j++) out[j] = u[j] + v[j];
         };
         float re[16], im[16], x[16];
         pair_sum(0, re);
         pair_sum(192, x);
#pragma unroll
         for (int j = 0; j < 16; j++) re[j] -= x[j];
         pair_sum(64, im);
         pair_sum(128, x);
#pragma unroll
         for (int j = 0; j < 16; j++) im[j] += x[j];
         float2 *dst = part + (size_t)chunk * nk;
         if (kr >= 0)
#pragma unroll
            for (int j = 0; j < 16; j++)
               if (t0 + j < hd.w) dst[kr + j] = make_float2(re[j] * qunscale, im[j] * qunscale);
      }
   }
   fence_before_sync();
   __syncthreads();
   if (w == TC_AW + 1) {
      __syncwarp();
      fence_after_sync();
      tmem_dealloc(tmem, 512);
   }
}

// The structure-factor product into part32 ([chunks][nk]); returns the
// number of chunks.
int ks_sfac_tc(cudaStream_t st, int nsites, int nk, const KsDev &d, int ntiles, double qmax, int *err)
{
   const int np = (nsites + TC_KS - 1) / TC_KS * TC_KS;
   const int nchunks = (np + TC_CHUNK - 1) / TC_CHUNK;
   // charges scaled by a power of two to |q| <= 1 (exact), undone on the partials
   int e = 0;
   std::frexp(qmax > 0 ? qmax : 1.0, &e);
   const float qs = std::ldexp(1.0f, e);
   k_sfac_tc<<<dim3(ntiles, nchunks), TC_THREADS, TC_SMEM, st>>>(d.tc_item.p, d.tc_k0.p, d.ph32.p, d.ztab.p, np, nk,
                                                          1.0f / qs, qs, d.part32.p, err);
   return nchunks;
}

size_t ks_tc_ztab_len(int nsites)
{
   const size_t np = (size_t)(nsites + TC_KS - 1) / TC_KS * TC_KS;
   return np / TC_KS * (TC_BBYTES / 16);
}

int ks_tc_chunks(int nsites)
{
   const int np = (nsites + TC_KS - 1) / TC_KS * TC_KS;
   return (np + TC_CHUNK - 1) / TC_CHUNK;
}


// ------------------------------------------------------------- forces
// The force pass of ewald() (src/ewald.c:557-566): for a charged site j,
//     F_j = q_j sum_k k (sin(k.r_j) A_k - cos(k.r_j) B_k) = q_j sum_k k Im(e_jk U_k),
// U_k = A_k - i B_k.  Over a tensor-core item (seed_ij, offsets t, k-vector
// (kx, ky, kz0 + t dkz)):
//     W1_ij = sum_t z_j(t) U_t,  W2_ij = sum_t t z_j(t) U_t,
//     F_j += q_j (kx f1, ky f1, kz0 f1 + dkz f2),  f1,2 = Im(seed_ij W1,2_ij).
// W is a product of the sites x t z tables (K = 128: the 64 cosines, then
// the 64 sines) and four coefficient rows per item,
//     W1re = [A | B],  W1im = [-B | A],  W2re = [tA | tB],  W2im = [-tB | tA],
// each row scaled by a power of two to |v| <= 1 (the scale is folded into
// the item's force coefficients).  Operands are three bf16 terms on fixed
// grids as in the structure factor, six term products (hh into one
// accumulator, the rest into another): the k-space force on a site is a
// near-cancelling sum over k, and two fp16 terms (2^-22 per operand, three
// products) raised the force error of the fixtures to 1.1e-5.  A CTA holds
// one 128-site tile's z tables (96 KB) at a time and streams the
// coefficient rows of 32 items (N = 128) per tile of items, two K-steps per
// stage (only the K-steps an item tile's longest item needs; one barrier
// wait and one commit per 12 MMAs: at one K-step per stage the issuing
// threads' waits cost 6 % of the pass); tensor memory holds two
// accumulator pairs, so the epilogue of one item tile (16 warps, four per
// tensor-memory lane quarter, 8 items each: the seed sine/cosine per item
// and site, the k-vector weights, Kahan-compensated FP32 force sums)
// overlaps the MMAs of the next.
constexpr int FTC_NI = 32;                         // items per item tile (4 rows each: N = 128)
constexpr int FTC_NSB = 2;                         // coefficient stages in flight per ring (two rings)
constexpr int FTC_ATERM = 128 * 128 * 2;           // one term of a site tile's z tables: 32 KB
constexpr int FTC_ABYTES = 3 * FTC_ATERM;          // 96 KB
constexpr int FTC_BTERM = 128 * 16 * 2;            // one term of a coefficient stage: 4 KB
constexpr int FTC_BBYTES = 3 * FTC_BTERM;          // 12 KB
constexpr int FTC_SBYTES = 2 * FTC_BBYTES;         // a stage: two K-steps (24 KB), one wait and commit per 12 MMAs
constexpr int FTC_EG = 4;                          // epilogue warps per tensor-memory lane quarter
constexpr int FTC_IPW = FTC_NI / FTC_EG;           // items of a tile per epilogue warp
constexpr int FTC_EW = 4 * FTC_EG;                 // epilogue warps
constexpr int FTC_SMEM = FTC_ABYTES + 2 * FTC_NSB * FTC_SBYTES + 2 * FTC_EG * 128 * 3 * 4 + FTC_EW * FTC_IPW * 32;
constexpr int FTC_THREADS = 32 * (FTC_EW + 4);     // epilogue warps, two bulk-copy warps, two MMA warps
static_assert(FTC_IPW % 4 == 0, "an epilogue warp reads its items' columns 16 at a time");
constexpr int FTC_SPLITS = 2;                      // force slots per site (two CTAs at most per site tile)
constexpr int FTC_ERR = 16;                        // error-word bit: a force-pass wait expired

// Coefficient rows of each item from the per-k (A, B, kz): one warp per
// item.  Layout per (item tile, K-step of 16): [term][column group 2][row
// group 16][8 rows][8 K] bf16, row 4 i + c for item i of the tile.
__global__ void __launch_bounds__(256)
k_utab_tc(int nitems, const int4 *__restrict__ item, const int4 *__restrict__ item_k0,
          const float2 *__restrict__ kxy, const float4 *__restrict__ kd, float dkz, uint4 *__restrict__ utab,
          float4 *__restrict__ coef)
{
   __shared__ float sv[8][64][4];
   const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int i = blockIdx.x * 8 + wl;
   if (i >= nitems) return;   // (warp-uniform)
   const int4 hd = item[i], k0 = item_k0[i];
   float a[2], b[2], kz0 = 0.f, m1 = 0.f, m2 = 0.f;
#pragma unroll
   for (int h = 0; h < 2; h++) {
      const int t = lane + 32 * h;
      a[h] = b[h] = 0.f;
      if (t < hd.w) {
         const int run = t >> 4;
         const int kr = run == 0 ? k0.x : run == 1 ? k0.y : run == 2 ? k0.z : k0.w;
         const float4 v = kd[kr + (t & 15)];
         a[h] = v.x;
         b[h] = v.y;
         if (t == 0) kz0 = v.z;
      }
      m1 = fmaxf(m1, fmaxf(fabsf(a[h]), fabsf(b[h])));
      m2 = fmaxf(m2, (float)t * fmaxf(fabsf(a[h]), fabsf(b[h])));
   }
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) {
      m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
      m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
   }
   kz0 = __shfl_sync(0xffffffffu, kz0, 0);
   // powers of two at or above the rows' largest magnitude
   int e1 = 0, e2 = 0;
   if (m1 > 0.f) frexpf(m1, &e1);
   if (m2 > 0.f) frexpf(m2, &e2);
   const float s1 = ldexpf(1.f, e1), s2 = ldexpf(1.f, e2), i1 = ldexpf(1.f, -e1), i2 = ldexpf(1.f, -e2);
#pragma unroll
   for (int h = 0; h < 2; h++) {
      const int t = lane + 32 * h;
      sv[wl][t][0] = a[h] * i1;
      sv[wl][t][1] = b[h] * i1;
      sv[wl][t][2] = (float)t * a[h] * i2;
      sv[wl][t][3] = (float)t * b[h] * i2;
   }
   __syncwarp();
   const int tile = i / FTC_NI, il = i % FTC_NI;
#pragma unroll
   for (int h = 0; h < 2; h++) {
      const int id = lane + 32 * h, c = id & 3, g = id >> 2;   // row c of the item, column group g
      const bool zi = g >= 8;                                  // the sine half of K
      const int t0 = 8 * (g & 7);
      // W1re = [A | B], W1im = [-B | A], W2re = [tA | tB], W2im = [-tB | tA]
      const int src = (c & 2) + (zi ? ((c & 1) ? 0 : 1) : ((c & 1) ? 1 : 0));
      const float sg = (!zi && (c & 1)) ? -1.f : 1.f;
      float v[8];
#pragma unroll
      for (int e = 0; e < 8; e++) v[e] = sg * sv[wl][t0 + e][src];
      unsigned int hh[4], mm[4], ll[4];
#pragma unroll
      for (int j = 0; j < 4; j++) tc::split3(v[2 * j], v[2 * j + 1], hh[j], mm[j], ll[j]);
      const int n = 4 * il + c, ks = g >> 1, kg = g & 1;
      const size_t base =
          ((size_t)tile * 8 + ks) * (FTC_BBYTES / 16) + kg * 128 + (n >> 3) * 8 + (n & 7);
      utab[base] = make_uint4(hh[0], hh[1], hh[2], hh[3]);
      utab[base + FTC_BTERM / 16] = make_uint4(mm[0], mm[1], mm[2], mm[3]);
      utab[base + 2 * FTC_BTERM / 16] = make_uint4(ll[0], ll[1], ll[2], ll[3]);
   }
   if (lane == 0) {
      const float2 k = kxy[i];
      coef[i] = hd.w > 0 ? make_float4(k.x * s1, k.y * s1, kz0 * s1, dkz * s2) : make_float4(0.f, 0.f, 0.f, 0.f);
   }
}

__device__ __forceinline__ void kahan_add_tc(float &s, float &c, float x)
{
   const float y = x - c;
   const float t = s + y;
   c = (t - s) - y;
   s = t;
}

// Work ranges of the persistent force pass.  Unit u is (site tile u / ntl,
// item tile u % ntl); CTA c takes units ustart[c] .. ustart[c + 1] - 1, a
// contiguous run over the site tiles.  The runs split the units' weights
// (an item tile's K-steps plus one for its epilogue) evenly over G CTAs,
// with G <= the number of site tiles (or G = twice that, each CTA then half
// a tile), so no run lies strictly inside a site tile and a tile is shared
// by two CTAs at most.  One block; pre (after ustart[G]) holds the prefix
// weights of the item tiles.
__global__ void k_ftc_ranges(const int4 *__restrict__ item, int ntl, int nsite_tiles, int G, int *__restrict__ ustart)
{
   int *pre = ustart + G + 1;
   if (threadIdx.x == 0) {
      int sum = 0;
      pre[0] = 0;
      for (int t = 0; t < ntl; t++) {
         sum += 2 * ((item[t * FTC_NI].w + 15) >> 4) + 1;
         pre[t + 1] = sum;
      }
   }
   __syncthreads();
   const long long wt = pre[ntl], wall = wt * nsite_tiles;
   for (int c = threadIdx.x; c <= G; c += blockDim.x) {
      const long long target = (long long)c * wall / G;
      const long long tile = target / wt, rem = target - tile * wt;
      int lo = 0, hi = ntl;   // the first item tile whose prefix weight reaches rem
      while (lo < hi) {
         const int mid = (lo + hi) >> 1;
         if (pre[mid] >= rem)
            hi = mid;
         else
            lo = mid + 1;
      }
      ustart[c] = (int)(tile * ntl + lo);
   }
}

// Persistent: one CTA per work range (k_ftc_ranges).  Per site tile of the
// range the CTA loads its z tables once (after the MMAs of the previous tile
// have completed) and runs its item tiles as before; the epilogue writes the
// tile's forces into slot 0 of fpart, or slot 1 when the range starts inside
// the tile (and zeros into slot 1 when the range covers the whole tile).
__global__ void __launch_bounds__(FTC_THREADS, 1)
k_force_tc(const int4 *__restrict__ item, const float4 *__restrict__ coef, int nitems,
           const int4 *__restrict__ ph, const uint4 *__restrict__ zsite, const uint4 *__restrict__ utab,
           const double *__restrict__ chg, const int *__restrict__ slots, int n, const int *__restrict__ ustart,
           double *__restrict__ fpart, int *__restrict__ err)
{
   using namespace tc;
   extern __shared__ __align__(1024) unsigned char sm[];
   __shared__ __align__(8) uint64_t full_a, a_free, full_b[2][FTC_NSB], empty_b[2][FTC_NSB], acc_full[2],
       acc_empty[2], done[2];
   __shared__ unsigned int tmem_s;
   __shared__ int abort_s;
   const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
   const int ntl = nitems / FTC_NI;   // item tiles per site tile
   const int u0 = ustart[blockIdx.x], u1 = ustart[blockIdx.x + 1];
   if (u1 <= u0) return;              // an empty range (uniform)
   const int T0 = u0 / ntl, T1 = (u1 - 1) / ntl;
   // the range's units of site tile T: ua(T) .. ue(T) - 1; local index u - u0
   auto ua = [&](int T) { return max(u0, T * ntl); };
   auto ue = [&](int T) { return min(u1, (T + 1) * ntl); };
   unsigned char *A = sm, *Bs = sm + FTC_ABYTES;
   // [2][FTC_EG][128][3]: per epilogue group, a site tile's force sums (by tile parity)
   float *red = reinterpret_cast<float *>(sm + FTC_ABYTES + 2 * FTC_NSB * FTC_SBYTES);
   // per epilogue warp: its items' (h, k, l0, count) and force coefficients
   int4 *sitem = reinterpret_cast<int4 *>(sm + FTC_ABYTES + 2 * FTC_NSB * FTC_SBYTES + 2 * FTC_EG * 128 * 3 * 4);
   if (tid == 0) {
      bar_init(&full_a, 1);
      bar_init(&a_free, 2);
      for (int p = 0; p < 2; p++)
         for (int s = 0; s < FTC_NSB; s++) {
            bar_init(&full_b[p][s], 1);
            bar_init(&empty_b[p][s], 1);
         }
      for (int b = 0; b < 2; b++) {
         bar_init(&acc_full[b], 1);
         bar_init(&acc_empty[b], FTC_EW);
      }
      bar_init(&done[0], 1);
      bar_init(&done[1], 1);
      abort_s = 0;
      bar_init_fence();
   }
   __syncwarp();
   if (w == FTC_EW + 2) tmem_alloc(&tmem_s, 512);   // two buffers x (hh sums, smaller terms) x 128 columns
   fence_before_sync();
   __syncthreads();
   fence_after_sync();
   const unsigned int tmem = tmem_s;
   // K-steps of a unit's item tile: ceil(longest count / 16) in each half of K
   auto khalf = [&](int u) { return (item[(u % ntl) * FTC_NI].w + 15) >> 4; };

   if (w == FTC_EW || w == FTC_EW + 1) {
      // ---- bulk copies: warp FTC_EW + p streams the coefficient rows of the
      // range's units of local parity p into ring p; warp FTC_EW also loads
      // each site tile's z tables
      const int p = w - FTC_EW;
      if (lane == 0) {
         int g = 0, na = 0;
         bool stop = false;
         for (int T = T0; T <= T1 && !stop; T++) {
            if (p == 0) {
               if (T > T0 && !bar_wait(&a_free, (unsigned int)(T - T0 - 1) & 1u)) {
                  tc_abort(&abort_s, err, FTC_ERR);
                  break;
               }
               bar_expect_tx(&full_a, FTC_ABYTES);
               bulk_load(A, zsite + (size_t)T * (FTC_ABYTES / 16), FTC_ABYTES, &full_a);
               na++;
            }
            for (int u = ua(T); u < ue(T) && !stop; u++) {
               if (((u - u0) & 1) != p) continue;
               const int kh = khalf(u), nt = u % ntl;
               // stage sq: K-steps q = 2 sq, 2 sq + 1 (the unit's 2 kh K-steps
               // are the kh lowest of each half of K)
               for (int sq = 0; sq < kh; sq++) {
                  const int s = g % FTC_NSB;
                  if (g >= FTC_NSB && !bar_wait(&empty_b[p][s], (unsigned int)(g / FTC_NSB - 1) & 1u)) {
                     tc_abort(&abort_s, err, FTC_ERR);
                     stop = true;
                     break;
                  }
                  if (tc_aborted(&abort_s)) {
                     stop = true;
                     break;
                  }
                  bar_expect_tx(&full_b[p][s], FTC_SBYTES);
                  for (int h = 0; h < 2; h++) {
                     const int q = 2 * sq + h, ks = q < kh ? q : 4 + q - kh;
                     bulk_load(Bs + (p * FTC_NSB + s) * FTC_SBYTES + h * FTC_BBYTES,
                               utab + ((size_t)nt * 8 + ks) * (FTC_BBYTES / 16), FTC_BBYTES, &full_b[p][s]);
                  }
                  g++;
               }
            }
         }
         // copies still in flight complete before the CTA's shared memory goes
         if (na > 0) bar_wait(&full_a, (unsigned int)(na - 1) & 1u);
         for (int q = g > FTC_NSB ? g - FTC_NSB : 0; q < g; q++)
            bar_wait(&full_b[p][q % FTC_NSB], (unsigned int)(q / FTC_NSB) & 1u);
      }
   } else if (w == FTC_EW + 2 || w == FTC_EW + 3) {
      // ---- MMA issue: warp FTC_EW + 2 + p takes the units of local parity
      // p into tensor-memory buffer p (one issuing thread sustains half the
      // tensor pipe's rate at N = 128; two keep it busy)
      const int p = w - FTC_EW - 2;
      const unsigned int idn = idesc_bf16(128, 128, false);
      const int ta[6] = {0, 0, 1, 0, 2, 1}, tb[6] = {0, 1, 0, 2, 0, 1};
      const unsigned int a0 = saddr(A), b0 = saddr(Bs + p * FTC_NSB * FTC_SBYTES);
      bool ok = true;
      int g = 0, jj = 0;
      for (int T = T0; T <= T1; T++) {
         if (T > T0) {
            // both issuers are past the previous site tile: its z tables go
            // once their MMAs complete
            __syncwarp();
            asm volatile("bar.sync 1, 64;" : : : "memory");
            if (lane == 0) mma_commit(&a_free);
         }
         if (lane != 0) continue;
         if (ok && !bar_wait(&full_a, (unsigned int)(T - T0) & 1u)) {
            tc_abort(&abort_s, err, FTC_ERR);
            ok = false;
         }
         fence_after_sync();
         for (int u = ua(T); u < ue(T); u++) {
            if (((u - u0) & 1) != p) continue;
            if (ok && (tc_aborted(&abort_s) ||
                       (jj >= 1 && !bar_wait(&acc_empty[p], (unsigned int)(jj - 1) & 1u)))) {
               tc_abort(&abort_s, err, FTC_ERR);
               ok = false;
            }
            fence_after_sync();
            const int kh = ok ? khalf(u) : 0;
            for (int sq = 0; sq < kh; sq++) {
               const int s = g % FTC_NSB;
               if (!bar_wait(&full_b[p][s], (unsigned int)(g / FTC_NSB) & 1u)) {
                  tc_abort(&abort_s, err, FTC_ERR);
                  ok = false;
                  break;
               }
               fence_after_sync();
#pragma unroll
               for (int h = 0; h < 2; h++) {
                  const int q = 2 * sq + h, ks = q < kh ? q : 4 + q - kh;
                  const unsigned int bs = b0 + s * FTC_SBYTES + h * FTC_BBYTES;
#pragma unroll
                  for (int t = 0; t < 6; t++) {
                     const uint64_t ad = sdesc(a0 + ta[t] * FTC_ATERM + ks * 4096, 2048, 128);
                     const uint64_t bd = sdesc(bs + tb[t] * FTC_BTERM, 2048, 128);
                     mma_f16(tmem + p * 256 + (t == 0 ? 0 : 128), ad, bd, idn, q > 0 || t > 1);
                  }
               }
               mma_commit(&empty_b[p][s]);
               g++;
            }
            mma_commit(&acc_full[p]);
            jj++;
         }
      }
      if (lane == 0) {
         mma_commit(&done[p]);
         bar_wait(&done[p], 0);   // every MMA complete before the tensor memory is released
      }
   } else {
      // ---- epilogue: site row r of each site tile, items ig * FTC_IPW .. of
      // each item tile
      const int r = 32 * (w & 3) + lane, ig = w >> 2;
      const unsigned int trow = tmem + ((unsigned int)(32 * (w & 3)) << 16);
      int4 *wi = sitem + w * 2 * FTC_IPW;   // [FTC_IPW] items, then [FTC_IPW] coefficients
      const float4 *wc = reinterpret_cast<const float4 *>(wi + FTC_IPW);
      bool live = true;
      for (int T = T0; T <= T1; T++) {
         const int i = T * 128 + r;
         const int4 v = i < n ? ph[i] : make_int4(0, 0, 0, 0);
         const unsigned int ux = (unsigned int)v.x, uy = (unsigned int)v.y, uz = (unsigned int)v.z;
         float Fx = 0.f, Fy = 0.f, Fz = 0.f, Cx = 0.f, Cy = 0.f, Cz = 0.f;
         for (int u = ua(T); u < ue(T) && live; u++) {
            const int j = u - u0, b = j & 1;
            const int it0 = (u % ntl) * FTC_NI + ig * FTC_IPW;
            // this unit's item records, fetched while its MMAs run
            __syncwarp();
            if (lane < FTC_IPW)
               wi[lane] = item[it0 + lane];
            else if (lane < 2 * FTC_IPW)
               reinterpret_cast<float4 *>(wi)[lane] = coef[it0 + lane - FTC_IPW];
            __syncwarp();
            const bool got = !tc_aborted(&abort_s) && bar_wait(&acc_full[b], (unsigned int)(j >> 1) & 1u);
            if (!__all_sync(0xffffffffu, got && !tc_aborted(&abort_s))) {
               if (lane == 0) tc_abort(&abort_s, err, FTC_ERR);
               live = false;
               break;
            }
            fence_after_sync();
            // the warp's accumulator columns (hh sums plus the rest) into
            // registers, then the buffer goes back to its MMA warp at once:
            // the next unit's MMAs into it overlap this unit's arithmetic
            float wv[FTC_IPW / 4][16];
#pragma unroll
            for (int grp = 0; grp < FTC_IPW / 4; grp++) {
               float mv[16], cv[16];
               const unsigned int col = (unsigned int)(b * 256 + 4 * FTC_IPW * ig + 16 * grp);
               tmem_ld16(trow + col, mv);
               tmem_ld16(trow + col + 128, cv);
               tmem_wait2(mv, cv);
#pragma unroll
               for (int c = 0; c < 16; c++) wv[grp][c] = mv[c] + cv[c];
            }
            fence_before_sync();
            __syncwarp();
            if (lane == 0) bar_arrive(&acc_empty[b]);
            float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll
            for (int grp = 0; grp < FTC_IPW / 4; grp++) {
#pragma unroll
               for (int e = 0; e < 4; e++) {
                  const int4 hd = wi[4 * grp + e];
                  // padding items come last; a tile of padding only issues no
                  // MMAs, so its buffer holds an earlier unit's sums (uniform)
                  if (hd.w == 0) continue;
                  const float4 cf = wc[4 * grp + e];
                  float sn, cs;
                  sincos_poly((unsigned int)hd.x * ux + (unsigned int)hd.y * uy + (unsigned int)hd.z * uz, &sn,
                              &cs);
                  const float w1r = wv[grp][4 * e], w1i = wv[grp][4 * e + 1];
                  const float w2r = wv[grp][4 * e + 2], w2i = wv[grp][4 * e + 3];
                  const float f1 = fmaf(cs, w1i, sn * w1r), f2 = fmaf(cs, w2i, sn * w2r);
                  fx = fmaf(cf.x, f1, fx);
                  fy = fmaf(cf.y, f1, fy);
                  fz = fmaf(cf.z, f1, fmaf(cf.w, f2, fz));
               }
            }
            kahan_add_tc(Fx, Cx, fx);
            kahan_add_tc(Fy, Cy, fy);
            kahan_add_tc(Fz, Cz, fz);
         }
         float *rt = red + (size_t)(T & 1) * FTC_EG * 128 * 3;
         float *rr = rt + ((size_t)ig * 128 + r) * 3;
         rr[0] = Fx - Cx;
         rr[1] = Fy - Cy;
         rr[2] = Fz - Cz;
         // the four groups' sums of this site tile, then its output slot
         __syncwarp();
         asm volatile("bar.sync 2, %0;" : : "n"(FTC_EW * 32) : "memory");
         if (w < 4 && i < n && !tc_aborted(&abort_s)) {
            const double q = chg[slots[i]];
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for (int g = 0; g < FTC_EG; g++) {
               const float *rg = rt + ((size_t)g * 128 + r) * 3;
               sx += (double)rg[0];
               sy += (double)rg[1];
               sz += (double)rg[2];
            }
            double *dst = fpart + (u0 > T * ntl ? 3 * (size_t)n : 0);
            dst[i] = q * sx;
            dst[n + i] = q * sy;
            dst[2 * (size_t)n + i] = q * sz;
            if (u0 <= T * ntl && u1 >= (T + 1) * ntl) {
               double *z = fpart + 3 * (size_t)n;
               z[i] = 0.0;
               z[n + i] = 0.0;
               z[2 * (size_t)n + i] = 0.0;
            }
         }
      }
   }
   fence_before_sync();
   __syncthreads();
   if (w == FTC_EW + 2) {
      __syncwarp();
      fence_after_sync();
      tmem_dealloc(tmem, 512);
   }
}

int ks_force_tc_splits(int) { return FTC_SPLITS; }

// Both z tables, cos and sin of 2 pi t u_z for t = 0..63, split into three
// bf16 terms:
//   ztab, the structure factor's B operand per 32-site stage (np sites, a
//     multiple of TC_KS): [term][column group (8 sites)][row group][8 rows]
//     [8 sites], rows 0..63 the cosines and 64..127 the sines;
//   zsite, the force pass's A operand per 128-site tile: [term][column group
//     16][row group 16][8 rows (sites)][8 t], column groups 0..7 the
//     cosines, 8..15 the sines.
// A block of 256 threads takes 32 sites (one stage, a quarter of a tile).
// Each thread computes the values of one site and 8 t (each value once),
// writes them to zsite and to shared memory, from where the block writes
// ztab.  Also zeroes the site records past n (padding sites have no
// charge).
__global__ void __launch_bounds__(256) k_ztabs_tc(int n, int np, int4 *__restrict__ ph, uint4 *__restrict__ ztab,
                                                  uint4 *__restrict__ zsite)
{
   __shared__ float sv[32][129];   // [site][t: cosines, then sines] (padded row)
   const int tid = threadIdx.x, sl = tid >> 3, tg = tid & 7;
   const int i = blockIdx.x * 32 + sl;   // site (the grid covers the 128-site tiles)
   const unsigned int uz = i < n ? (unsigned int)ph[i].z : 0u;
   float c[8], sn[8];
#pragma unroll
   for (int e = 0; e < 8; e++) sincos_rev32((unsigned int)(8 * tg + e) * uz, &sn[e], &c[e]);
   unsigned int h[4], m[4], l[4];
   const int tile = i >> 7, r = i & 127;
   const size_t zb = (size_t)tile * (FTC_ABYTES / 16) + (r >> 3) * 8 + (r & 7);
#pragma unroll
   for (int j = 0; j < 4; j++) tc::split3(c[2 * j], c[2 * j + 1], h[j], m[j], l[j]);
   zsite[zb + tg * 128] = make_uint4(h[0], h[1], h[2], h[3]);
   zsite[zb + tg * 128 + FTC_ATERM / 16] = make_uint4(m[0], m[1], m[2], m[3]);
   zsite[zb + tg * 128 + 2 * FTC_ATERM / 16] = make_uint4(l[0], l[1], l[2], l[3]);
#pragma unroll
   for (int j = 0; j < 4; j++) tc::split3(sn[2 * j], sn[2 * j + 1], h[j], m[j], l[j]);
   zsite[zb + (8 + tg) * 128] = make_uint4(h[0], h[1], h[2], h[3]);
   zsite[zb + (8 + tg) * 128 + FTC_ATERM / 16] = make_uint4(m[0], m[1], m[2], m[3]);
   zsite[zb + (8 + tg) * 128 + 2 * FTC_ATERM / 16] = make_uint4(l[0], l[1], l[2], l[3]);
#pragma unroll
   for (int e = 0; e < 8; e++) {
      sv[sl][8 * tg + e] = c[e];
      sv[sl][64 + 8 * tg + e] = sn[e];
   }
   if (i >= n && i < np) ph[i] = make_int4(0, 0, 0, 0);
   __syncthreads();
   // B operand of the stage: (8 sites q8, row) per thread, two each
   const int stage = blockIdx.x;
   if (stage * TC_KS >= np) return;   // past the structure factor's padded sites (uniform)
#pragma unroll
   for (int k = 0; k < 2; k++) {
      const int id = tid + 256 * k, q8 = id >> 7, row = id & 127;
      float v[8];
#pragma unroll
      for (int e = 0; e < 8; e++) v[e] = sv[8 * q8 + e][row];
#pragma unroll
      for (int j = 0; j < 4; j++) tc::split3(v[2 * j], v[2 * j + 1], h[j], m[j], l[j]);
      const size_t base = (size_t)stage * (TC_BBYTES / 16) + q8 * (TC_LBO / 16) + (row >> 3) * 8 + (row & 7);
      ztab[base] = make_uint4(h[0], h[1], h[2], h[3]);
      ztab[base + TC_TERM / 16] = make_uint4(m[0], m[1], m[2], m[3]);
      ztab[base + 2 * TC_TERM / 16] = make_uint4(l[0], l[1], l[2], l[3]);
   }
}

// Host side.  Per-site operand tables (after k_prep): the z tables as the
// structure factor's B operand and as the force pass's A operand.
void ks_tables_tc(cudaStream_t st, int nsites, const KsDev &d)
{
   const int np = (nsites + TC_KS - 1) / TC_KS * TC_KS;
   const int np128 = (nsites + 127) / 128 * 128;
   k_ztabs_tc<<<np128 / 32, 256, 0, st>>>(nsites, np, d.ph32.p, d.ztab.p, d.zsite.p);
}

// The force pass's coefficient rows (after the per-k reduction).
void ks_coef_tc(cudaStream_t st, const KsDev &d, int nitems_padded, float dkz)
{
   k_utab_tc<<<(nitems_padded + 7) / 8, 256, 0, st>>>(nitems_padded, d.tc_item.p, d.tc_k0.p, d.tc_kxy.p,
                                                      d.kdat32.p, dkz, d.utab.p, d.tc_coef.p);
}

int ks_force_tc(cudaStream_t st, int nsites, KsDev &d, int nitems_padded, int nsm, const double *chg,
                const int *slots, double *fpart, int *err)
{
   const int T = (nsites + 127) / 128, ntl = nitems_padded / FTC_NI;
   const int G = 2 * T <= nsm ? 2 * T : std::min(nsm, T);
   int launches = 1;
   if (d.tc_rkey[0] != T || d.tc_rkey[1] != ntl || d.tc_rkey[2] != G || d.tc_rver != d.tc_ver) {
      if (d.tc_ustart.ensure((size_t)G + ntl + 2) != cudaSuccess) return -1;
      k_ftc_ranges<<<1, 256, 0, st>>>(d.tc_item.p, ntl, T, G, d.tc_ustart.p);
      d.tc_rkey[0] = T;
      d.tc_rkey[1] = ntl;
      d.tc_rkey[2] = G;
      d.tc_rver = d.tc_ver;
      launches++;
   }
   k_force_tc<<<G, FTC_THREADS, FTC_SMEM, st>>>(d.tc_item.p, d.tc_coef.p, nitems_padded, d.ph32.p, d.zsite.p,
                                                d.utab.p, chg, slots, nsites, d.tc_ustart.p, fpart, err);
   return launches;
}

size_t ks_tc_zsite_len(int nsites)
{
   return (size_t)((nsites + 127) / 128) * (FTC_ABYTES / 16);
}

size_t ks_tc_utab_len(int nitems_padded)
{
   return (size_t)(nitems_padded / FTC_NI) * 8 * (FTC_BBYTES / 16);
}

// Shared-memory sizes of the tensor-core kernels, set once per device
// outside any stream capture (from ks_prepare).
// (contexts may be created from several host threads: the per-device flags
// are atomic, and setting the attribute twice is harmless)
cudaError_t ks_tc_init(int device)
{
   static std::atomic<unsigned long long> done{0};
   const unsigned long long bit = device >= 0 && device < 64 ? 1ull << device : 0ull;
   if (bit && (done.load() & bit)) return cudaSuccess;
   cudaError_t e = cudaFuncSetAttribute(k_sfac_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
   if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_force_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, FTC_SMEM);
   if (e == cudaSuccess && bit) done.fetch_or(bit);
   return e;
}

}  // namespace mdgpu
