// Reciprocal-space Ewald sum without any allocation: mdgpu_ewald_kspace_noalloc.
//
// Some callers cannot call cudaMalloc: hosts that hand out all device memory
// from their own fixed pools and forbid libraries to allocate behind their
// back, and step loops that must not take the allocator's locks, synchronise
// the device, or risk an out-of-memory failure part-way through a run.  For
// them this entry point runs the reciprocal-space kernels of the force path
// with every intermediate array -- the k-vector list included, which a small
// kernel builds from the cell matrix, alpha and the k-cutoff passed by value
// -- carved out of one file-scope static device array of fixed size
// (MDGPU_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the library
// until the process exits).  The caller passes the inputs and outputs in its
// own device memory; no host buffer is read after the call returns.
//
// Limits (calls beyond them are rejected with MDGPU_E_CAPACITY):
//   nsites <= MDGPU_NOALLOC_MAX_SITES, k-vectors <= MDGPU_NOALLOC_MAX_KVEC.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (which may load the module onto that device) and
// keeps it for the life of the process: it assumes the device's primary
// context stays the same (no cudaDeviceReset in between).  Make that first
// call before any stream capture.  Every call shares the same scratch:
// calls that overlap on the GPU -- on different streams, or from different
// host threads -- race and corrupt each other.
#include <atomic>
#include <cmath>
#include <cstring>

#include "mdgpu_internal.h"

namespace mdgpu {
// kernels of the reciprocal-space pass (kspace.cu)
__global__ void k_prep(int N, int ns, const int *sorted, const double *site, const double *chg, double hi0,
                       double hi1, double hi2, double hi3, double hi4, double hi5, double hi6,
                       double hi7, double hi8, int mixed, int4 *ph32, float2 *z32, float2 *zp32,
                       ulonglong2 *ph64a, ulonglong2 *ph64b, double2 *z64);
__global__ void k_sfac32(const int4 *item, const int *item_k0, int nitems, const int4 *ph,
                         const float2 *zp, int N, int chunk, int nk, float2 *part, int *err);
__global__ void k_kfinal(const double *blk, int nblocks, DevOut *out);
__global__ void k_force32(const int4 *item, const int *item_k0, const float2 *item_kxy, int nitems,
                          int nk, int per_split, const float4 *kd, const int4 *ph, const float2 *zz,
                          const double *chg, const int *sorted, int N, int obase, float dkz, double *fpart);
__global__ void k_fsum(int n3, int nsplit, const double *fpart, double *force, int accumulate);
}  // namespace mdgpu

namespace {

using namespace mdgpu;

constexpr int MAX_SITES = MDGPU_NOALLOC_MAX_SITES;
constexpr int MAX_KVEC = MDGPU_NOALLOC_MAX_KVEC;
constexpr int MAX_CHUNKS = 16;
constexpr int MAX_SPLITS = 4;
// site ordering grid: at most OG^3 cells, counted by ORDER_WARPS warps with
// 16-bit counts and slot offsets
constexpr int OG = 16;
constexpr int ORDER_WARPS = 4;
static_assert(MAX_SITES <= 65535, "the ordering counts are 16-bit");

constexpr size_t al(size_t x) { return (x + 255) / 256 * 256; }
// byte offsets of the scratch regions
constexpr size_t O_OUT = 0;
constexpr size_t O_ITEM = O_OUT + al(sizeof(DevOut));
constexpr size_t O_K0 = O_ITEM + al(sizeof(int4) * MAX_KVEC);
constexpr size_t O_KXY = O_K0 + al(sizeof(int) * (MAX_KVEC + 1));
constexpr size_t O_KVEC = O_KXY + al(sizeof(float2) * MAX_KVEC);
constexpr size_t O_COEF = O_KVEC + al(sizeof(double) * 3 * MAX_KVEC);
constexpr size_t O_COEF2 = O_COEF + al(sizeof(double) * MAX_KVEC);
constexpr size_t O_KDAT = O_COEF2 + al(sizeof(double) * MAX_KVEC);
constexpr size_t O_PH = O_KDAT + al(sizeof(float4) * MAX_KVEC);
constexpr size_t O_Z = O_PH + al(sizeof(int4) * MAX_SITES);
constexpr size_t O_ZP = O_Z + al(sizeof(float2) * MAX_SITES);
constexpr size_t O_SORT = O_ZP + al(sizeof(float2) * MAX_SITES * KI);
constexpr size_t O_KEY = O_SORT + al(sizeof(int) * MAX_SITES);
constexpr size_t O_PART = O_KEY + al(sizeof(int) * MAX_SITES);
constexpr size_t O_FPART = O_PART + al(sizeof(float2) * MAX_CHUNKS * MAX_KVEC);
constexpr size_t O_BLK = O_FPART + al(sizeof(double) * MAX_SPLITS * 3 * MAX_SITES);
constexpr size_t O_END = O_BLK + al(sizeof(double) * 8 * ((MAX_KVEC + 255) / 256));
static_assert(O_END <= MDGPU_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

// error bits of the result record set here (the shared kernels use 1 and 4)
constexpr int ERR_KLIST = 64;   // the device k-list disagrees with the host's count

// The k-vector list's geometry, by value: 2 pi h^-1 (upper triangle), the
// cut, alpha's exponent factor and the energy prefactor 2 / (eps0 V).
struct KlArgs {
   double hp0, hp1, hp2, hp4, hp5, hp8;
   double kcsq, r4a, pref;
   int hmax, kmax, lmax;
   int nk, ni;   // the host's counts (capacity already checked)
};

// Column c of the enumeration: (h, k) in the order of src/ewald.c:441-461,
// h = 0 taking k >= 0 only.
__host__ __device__ inline void kl_column(const KlArgs &a, int c, int &hh, int &k)
{
   if (c <= a.kmax) {
      hh = 0;
      k = c;
   } else {
      const int w = 2 * a.kmax + 1, cc = c - (a.kmax + 1);
      hh = 1 + cc / w;
      k = cc % w - a.kmax;
   }
}

// One column of the k-list: its k-vectors (l ascending, kept where
// |k|^2 < k_cutoff^2) grouped into items of up to KI consecutive l.  Counts
// them (WRITE false) or writes them from k index nk and item index ni on.
// Every product and sum is rounded separately, as the host computes it
// (its code is built without contraction), so both see the same cut.
template <bool WRITE>
__host__ __device__ inline void kl_scan_column(const KlArgs &a, int hh, int k, int &nk, int &ni,
                                               int4 *item, int *k0, float2 *kxy, double *kvec,
                                               double *coef, double *coef2)
{
#ifdef __CUDA_ARCH__
#define KL_MUL(x, y) __dmul_rn(x, y)
#define KL_ADD(x, y) __dadd_rn(x, y)
#else
#define KL_MUL(x, y) ((x) * (y))
#define KL_ADD(x, y) ((x) + (y))
#endif
   const double dh = (double)hh, dk = (double)k;
   const double kx = KL_MUL(dh, a.hp0);
   const double ky = KL_ADD(KL_MUL(dh, a.hp1), KL_MUL(dk, a.hp4));
   const double kzt = KL_ADD(KL_MUL(dh, a.hp2), KL_MUL(dk, a.hp5));
   const double ksq = KL_ADD(KL_MUL(kx, kx), KL_MUL(ky, ky));
   int prev_l = -1000000, cur = 0;
   for (int l = (hh == 0 && k == 0 ? 1 : -a.lmax); l <= a.lmax; l++) {
      const double kz = KL_ADD(kzt, KL_MUL((double)l, a.hp8));
      const double ks = KL_ADD(ksq, KL_MUL(kz, kz));
      if (!(ks < a.kcsq)) continue;
      const bool extend = prev_l == l - 1 && cur > 0 && cur < KI;
      if (!extend) {
         if (WRITE && ni < a.ni) {
            item[ni] = make_int4(hh, k, l, 1);
            k0[ni] = nk;
            kxy[ni] = make_float2((float)kx, (float)ky);
         }
         ni++;
         cur = 1;
      } else {
         if (WRITE && ni - 1 < a.ni) item[ni - 1].w++;
         cur++;
      }
      prev_l = l;
      if (WRITE && nk < a.nk) {
         kvec[nk] = kx;
         kvec[a.nk + nk] = ky;
         kvec[2 * a.nk + nk] = kz;
         const double e = KL_MUL(ks, a.r4a);
#ifdef __CUDA_ARCH__
         coef[nk] = __ddiv_rn(__dmul_rn(a.pref, exp(e)), ks);
         coef2[nk] = __ddiv_rn(__dmul_rn(2.0, __dsub_rn(1.0, e)), ks);
#endif
      }
      nk++;
   }
#undef KL_MUL
#undef KL_ADD
}

// Builds the k-vector list on the device (one block of 1024 threads): each
// thread takes a run of consecutive columns, counts them, a block scan gives
// every run its first k and item index, then the runs are written.  The
// totals are checked against the host's counts (ERR_KLIST on a mismatch;
// nothing is written past them).
__global__ void __launch_bounds__(1024)
k_klist_na(KlArgs a, int4 *__restrict__ item, int *__restrict__ k0, float2 *__restrict__ kxy,
           double *__restrict__ kvec, double *__restrict__ coef, double *__restrict__ coef2,
           DevOut *__restrict__ out)
{
   __shared__ int wk[32], wi[32];
   const int ncol = (a.hmax + 1) * (2 * a.kmax + 1) - a.kmax;
   const int per = (ncol + blockDim.x - 1) / blockDim.x;
   const int c0 = min(ncol, (int)threadIdx.x * per), c1 = min(ncol, c0 + per);
   int nk = 0, ni = 0;
   for (int c = c0; c < c1; c++) {
      int hh, k;
      kl_column(a, c, hh, k);
      kl_scan_column<false>(a, hh, k, nk, ni, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
   }
   // block-wide exclusive scan of (nk, ni)
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   int sk = nk, si = ni;
   for (int o = 1; o < 32; o <<= 1) {
      const int tk = __shfl_up_sync(0xffffffffu, sk, o), ti = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) {
         sk += tk;
         si += ti;
      }
   }
   if (lane == 31) {
      wk[w] = sk;
      wi[w] = si;
   }
   __syncthreads();
   if (w == 0) {
      int vk = wk[lane], vi = wi[lane];
      for (int o = 1; o < 32; o <<= 1) {
         const int tk = __shfl_up_sync(0xffffffffu, vk, o), ti = __shfl_up_sync(0xffffffffu, vi, o);
         if (lane >= o) {
            vk += tk;
            vi += ti;
         }
      }
      wk[lane] = vk;
      wi[lane] = vi;
   }
   __syncthreads();
   int ok = sk - nk + (w > 0 ? wk[w - 1] : 0), oi = si - ni + (w > 0 ? wi[w - 1] : 0);
   if (threadIdx.x == 0 && (wk[31] != a.nk || wi[31] != a.ni)) atomicOr(&out->err, ERR_KLIST);
   for (int c = c0; c < c1; c++) {
      int hh, k;
      kl_column(a, c, hh, k);
      kl_scan_column<true>(a, hh, k, ok, oi, item, k0, kxy, kvec, coef, coef2);
   }
}

// Orders the sites by a cell grid (g^3 cells of the fractional
// co-ordinates, about two sites a cell; ascending site index inside a
// cell), one block of ORDER_WARPS warps: a structure-factor chunk is then a
// compact, nearly neutral region, so its FP32 partial sum stays small even
// where the whole sum cancels (an ionic crystal listed species by species
// would otherwise give chunks of a single charge sign).  Warp w owns sites
// [w S, (w + 1) S): it counts them per cell, one scan over (cell, warp)
// gives each warp its first slot per cell, and the warp places its sites in
// order.  sorted[slot] = site.
__global__ void __launch_bounds__(ORDER_WARPS * 32)
k_order_na(int N, const double *__restrict__ site, double hi0, double hi1, double hi2, double hi4,
           double hi5, double hi8, int g, int *__restrict__ key, int *__restrict__ sorted)
{
   __shared__ unsigned short tab[OG * OG * OG * ORDER_WARPS];   // [cell][warp]: count, then first slot
   __shared__ int wsum[ORDER_WARPS];
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   const int ncell = g * g * g, nt = ncell * ORDER_WARPS;
   for (int j = threadIdx.x; j < nt; j += blockDim.x) tab[j] = 0;
   __syncthreads();
   const int S = (N + ORDER_WARPS - 1) / ORDER_WARPS, s0 = min(N, w * S), s1 = min(N, s0 + S);
   const unsigned int lt = (1u << lane) - 1u;
   for (int b = s0; b < s1; b += 32) {
      const int i = b + lane;
      int kk = -1;
      if (i < s1) {
         const double x = site[i], y = site[N + i], z = site[2 * (size_t)N + i];
         double f[3] = {hi0 * x + hi1 * y + hi2 * z, hi4 * y + hi5 * z, hi8 * z};
         int cc[3];
         for (int d = 0; d < 3; d++) {
            double u = f[d] - floor(f[d]);
            int v = (u == u) ? (int)(u * g) : 0;   // a NaN co-ordinate goes to cell 0
            cc[d] = v < 0 ? 0 : (v >= g ? g - 1 : v);
         }
         kk = (cc[0] * g + cc[1]) * g + cc[2];
         key[i] = kk;
      }
      const unsigned int peers = __match_any_sync(0xffffffffu, kk);
      if (kk >= 0 && (peers & lt) == 0) tab[kk * ORDER_WARPS + w] += (unsigned short)__popc(peers);
      __syncwarp();
   }
   __syncthreads();
   // exclusive scan over tab in (cell, warp) order: a run of entries per thread
   const int per = (nt + blockDim.x - 1) / blockDim.x;
   const int j0 = min(nt, (int)threadIdx.x * per), j1 = min(nt, j0 + per);
   int tot = 0;
   for (int j = j0; j < j1; j++) tot += tab[j];
   int sc = tot;
   for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, sc, o);
      if (lane >= o) sc += t;
   }
   if (lane == 31) wsum[w] = sc;
   __syncthreads();
   int run = sc - tot;
   for (int v = 0; v < w; v++) run += wsum[v];
   for (int j = j0; j < j1; j++) {
      const int cnt = tab[j];
      tab[j] = (unsigned short)run;
      run += cnt;
   }
   __syncthreads();
   for (int b = s0; b < s1; b += 32) {
      const int i = b + lane;
      const int kk = i < s1 ? key[i] : -1;
      const unsigned int peers = __match_any_sync(0xffffffffu, kk);
      if (kk >= 0) sorted[tab[kk * ORDER_WARPS + w] + __popc(peers & lt)] = i;
      __syncwarp();
      if (kk >= 0 && (peers & lt) == 0) tab[kk * ORDER_WARPS + w] += (unsigned short)__popc(peers);
      __syncwarp();
   }
}

// A structure-factor tile that never arrived, or a k-list that does not
// match the host's, leaves the forces undefined: they are overwritten with
// NaN (the energy too, in k_add_energy), so a caller that checks only the
// forces sees the failure.
__global__ void k_poison_na(int n3, const DevOut *__restrict__ o, double *__restrict__ force)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n3 && (o->err & (4 | ERR_KLIST))) force[i] = __longlong_as_double(0x7ff8000000000000ll);
}

// per k: S(k) from the chunk partials (FP64, fixed order), energy, stress and
// the force coefficients A = coeff Re S, B = coeff Im S (src/ewald.c:525-553);
// per-block energy/stress partials into blk
__global__ void __launch_bounds__(256)
k_kreduce_na(int nk, int nchunks, const float2 *__restrict__ part, const double *__restrict__ kvec,
             const double *__restrict__ coeff, const double *__restrict__ coeff2,
             float4 *__restrict__ kd, double *__restrict__ blk)
{
   __shared__ double red[8][8];
   const int k = blockIdx.x * blockDim.x + threadIdx.x;
   double v[7] = {0, 0, 0, 0, 0, 0, 0};
   if (k < nk) {
      double C = 0.0, S = 0.0;
      for (int c = 0; c < nchunks; c++) {
         const float2 p = part[(size_t)c * nk + k];
         C += (double)p.x;
         S += (double)p.y;
      }
      const double kx = kvec[k], ky = kvec[nk + k], kz = kvec[2 * nk + k];
      const double cf = coeff[k], cf2 = coeff2[k], pek = 0.5 * cf * (C * C + S * S);
      v[0] = pek;
      v[1] = pek - pek * cf2 * kx * kx;
      v[2] = -(pek * cf2 * kx * ky);
      v[3] = -(pek * cf2 * kx * kz);
      v[4] = pek - pek * cf2 * ky * ky;
      v[5] = -(pek * cf2 * ky * kz);
      v[6] = pek - pek * cf2 * kz * kz;
      kd[k] = make_float4((float)(cf * C), (float)(cf * S), (float)kz, 0.f);
   }
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   for (int j = 0; j < 7; j++) {
      double s = v[j];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) red[j][w] = s;
   }
   __syncthreads();
   if (threadIdx.x < 7) {
      double s = 0.0;
      for (int j = 0; j < (int)(blockDim.x >> 5); j++) s += red[threadIdx.x][j];
      blk[blockIdx.x * 8 + threadIdx.x] = s;
   }
}

// adds the k-space energy and stress upper triangle into the caller's outputs
__global__ void k_add_energy(const DevOut *o, double *pe, double *stress)
{
   if (threadIdx.x != 0) return;
   // a structure-factor tile that never arrived, or a mismatched k-list,
   // leaves the energy undefined
   *pe += (o->err & (4 | ERR_KLIST)) ? __longlong_as_double(0x7ff8000000000000ll) : o->pe_k;
   stress[0] += o->st_k[0];
   stress[1] += o->st_k[1];
   stress[2] += o->st_k[2];
   stress[4] += o->st_k[3];
   stress[5] += o->st_k[4];
   stress[8] += o->st_k[5];
}

}  // namespace

// The scratch itself.
static __device__ __align__(256) unsigned char mdgpu_noalloc_scratch[MDGPU_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int MAX_DEVICES = 64;
// device address of the array, per device (looked up once per device)
std::atomic<unsigned char *> g_scratch[MAX_DEVICES];
}  // namespace

extern "C" mdgpu_status mdgpu_ewald_kspace_noalloc(const double *h, int nsites, const double *d_site,
                                                   const double *d_chg, double alpha, double k_cutoff,
                                                   double *d_force, double *d_pe, double *d_stress,
                                                   void *stream)
{
   if (!h || nsites <= 0 || !d_site || !d_chg || !d_force || !d_pe || !d_stress)
      return MDGPU_E_ARG;
   if (!(alpha > 0.0) || !(k_cutoff > 0.0)) return MDGPU_E_ARG;
   if (h[3] != 0.0 || h[6] != 0.0 || h[7] != 0.0 || !(det3(h) > 0.0)) return MDGPU_E_UNSUPPORTED;
   if (nsites > MAX_SITES) return MDGPU_E_CAPACITY;
   cudaStream_t st = (cudaStream_t)stream;

   // set-up, once per device, with that device current
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return MDGPU_E_CUDA;
   unsigned char *S = g_scratch[dev].load();
   if (!S) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, mdgpu_noalloc_scratch) != cudaSuccess || !p) {
         cudaGetLastError();
         return MDGPU_E_CUDA;
      }
      S = (unsigned char *)p;
      g_scratch[dev].store(S);
   }

   // the k-list's geometry (src/ewald.c:441-461, 510-511), and its size
   // counted here so that the capacity check is made before any launch;
   // the list itself is built on the device from these values
   const double kc = k_cutoff;
   double hinv[9];
   inv3(h, hinv);
   KlArgs ka;
   ka.hp0 = 2 * PI * hinv[0];
   ka.hp1 = 2 * PI * hinv[1];
   ka.hp2 = 2 * PI * hinv[2];
   ka.hp4 = 2 * PI * hinv[4];
   ka.hp5 = 2 * PI * hinv[5];
   ka.hp8 = 2 * PI * hinv[8];
   ka.hmax = (int)std::floor(kc / (2 * PI) * h[0]);
   ka.kmax = (int)std::floor(kc / (2 * PI) * std::sqrt(h[1] * h[1] + h[4] * h[4]));
   ka.lmax = (int)std::floor(kc / (2 * PI) * std::sqrt(h[2] * h[2] + h[5] * h[5] + h[8] * h[8]));
   ka.kcsq = kc * kc;
   ka.r4a = -1.0 / (4.0 * alpha * alpha);
   ka.pref = 2.0 / (0.25 / PI * det3(h));
   ka.nk = ka.ni = 0;
   if ((double)(ka.hmax + 1) * (2.0 * ka.kmax + 1) * (2.0 * ka.lmax + 1) > 1e7) return MDGPU_E_CAPACITY;
   {
      const int ncol = (ka.hmax + 1) * (2 * ka.kmax + 1) - ka.kmax;
      int nk = 0, ni = 0;
      for (int c = 0; c < ncol && nk <= MAX_KVEC; c++) {
         int hh, k;
         kl_column(ka, c, hh, k);
         kl_scan_column<false>(ka, hh, k, nk, ni, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
      }
      if (nk > MAX_KVEC) return MDGPU_E_CAPACITY;
      ka.nk = nk;
      ka.ni = ni;
   }
   const int nk = ka.nk, ni = ka.ni;
   if (nk == 0) return MDGPU_OK;

   DevOut *out = (DevOut *)(S + O_OUT);
   int4 *item = (int4 *)(S + O_ITEM);
   int *k0 = (int *)(S + O_K0);
   float2 *kxy = (float2 *)(S + O_KXY);
   double *kvec = (double *)(S + O_KVEC);
   double *coef = (double *)(S + O_COEF), *coef2 = (double *)(S + O_COEF2);
   float4 *kdat = (float4 *)(S + O_KDAT);
   int4 *ph = (int4 *)(S + O_PH);
   float2 *z = (float2 *)(S + O_Z), *zp = (float2 *)(S + O_ZP);
   int *sorted = (int *)(S + O_SORT), *key = (int *)(S + O_KEY);
   float2 *part = (float2 *)(S + O_PART);
   double *fpart = (double *)(S + O_FPART), *blk = (double *)(S + O_BLK);

   // the result record must start at zero (the last call left its values);
   // every other region is written in full before it is read
   if (cudaMemsetAsync(out, 0, sizeof(DevOut), st) != cudaSuccess) return MDGPU_E_CUDA;
   k_klist_na<<<1, 1024, 0, st>>>(ka, item, k0, kxy, kvec, coef, coef2, out);

   const int N = nsites;
   // sites in the order of a cell grid, about two sites a cell
   int g = (int)std::lround(std::cbrt(N / 2.0));
   g = g < 1 ? 1 : (g > OG ? OG : g);
   k_order_na<<<1, ORDER_WARPS * 32, 0, st>>>(N, d_site, hinv[0], hinv[1], hinv[2], hinv[4], hinv[5], hinv[8], g, key,
                                  sorted);
   k_prep<<<(N + 255) / 256, 256, 0, st>>>(N, N, sorted, d_site, d_chg, hinv[0], hinv[1], hinv[2], hinv[3],
                                           hinv[4], hinv[5], hinv[6], hinv[7], hinv[8], 1, ph, z, zp,
                                           nullptr, nullptr, nullptr);
   int chunks = (N + 63) / 64;
   if (chunks > MAX_CHUNKS) chunks = MAX_CHUNKS;
   const int chunk = ((N + chunks - 1) / chunks + 31) / 32 * 32;
   chunks = (N + chunk - 1) / chunk;
   k_sfac32<<<dim3((ni + 127) / 128, chunks), 128, 0, st>>>(item, k0, ni, ph, zp, N, chunk, nk, part, &out->err);
   const int nbk = (nk + 255) / 256;
   k_kreduce_na<<<nbk, 256, 0, st>>>(nk, chunks, part, kvec, coef, coef2, kdat, blk);
   k_kfinal<<<1, 256, 0, st>>>(blk, nbk, out);
   int splits = (ni + 7) / 8;
   if (splits > MAX_SPLITS) splits = MAX_SPLITS;
   if (splits < 1) splits = 1;
   const int per_split = (ni + splits - 1) / splits;
   splits = (ni + per_split - 1) / per_split;
   k_force32<<<dim3((N + 2 * FT_THREADS - 1) / (2 * FT_THREADS), splits), FT_THREADS, 0, st>>>(
      item, k0, kxy, ni, nk, per_split, kdat, ph, zp, d_chg, sorted, N, 0, (float)ka.hp8, fpart);
   k_fsum<<<(3 * N + 255) / 256, 256, 0, st>>>(3 * N, splits, fpart, d_force, 1);
   k_poison_na<<<(3 * N + 255) / 256, 256, 0, st>>>(3 * N, out, d_force);
   k_add_energy<<<1, 32, 0, st>>>(out, d_pe, d_stress);
   const cudaError_t e = cudaGetLastError();
   return e == cudaSuccess ? MDGPU_OK : MDGPU_E_CUDA;
}
