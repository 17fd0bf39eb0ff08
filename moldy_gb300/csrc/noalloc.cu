// Reciprocal-space Ewald sum without any allocation: mdgpu_ewald_kspace_noalloc.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA stream is
// being captured into a graph (allocation is not a capturable operation),
// hosts that hand out all device memory from their own fixed pools and forbid
// libraries to allocate behind their back, and step loops that must not take
// the allocator's locks or risk an out-of-memory failure part-way through a
// run.  For them this entry point runs the reciprocal-space kernels of the
// force path with every intermediate array carved out of one file-scope
// static device array of fixed size (MDGPU_NOALLOC_SCRATCH_BYTES, held by
// every GPU that loads the library until the process exits), and the
// k-vector list built in fixed static host buffers.  The caller passes the
// inputs and outputs in its own device memory.
//
// Limits (calls beyond them are rejected with MDGPU_E_CAPACITY):
//   nsites <= MDGPU_NOALLOC_MAX_SITES, k-vectors <= MDGPU_NOALLOC_MAX_KVEC.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (which may load the module onto that device); make
// that first call before any stream capture.  Every call shares the same
// scratch and host buffers: calls that overlap -- on different streams, or
// from different host threads -- race and corrupt each other.
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
constexpr size_t O_PART = O_SORT + al(sizeof(int) * MAX_SITES);
constexpr size_t O_FPART = O_PART + al(sizeof(float2) * MAX_CHUNKS * MAX_KVEC);
constexpr size_t O_BLK = O_FPART + al(sizeof(double) * MAX_SPLITS * 3 * MAX_SITES);
constexpr size_t O_END = O_BLK + al(sizeof(double) * 8 * ((MAX_KVEC + 255) / 256));
static_assert(O_END <= MDGPU_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

// host-side k-list in fixed static buffers (same enumeration and prefactors
// as the allocating path: ewald(), src/ewald.c:441-461, 510-511)
int4 h_item[MAX_KVEC];
int h_k0[MAX_KVEC + 1];
float2 h_kxy[MAX_KVEC];
double h_kvec[3 * MAX_KVEC], h_coef[MAX_KVEC], h_coef2[MAX_KVEC];

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

__global__ void k_iota(int n, int *a)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) a[i] = i;
}

// adds the k-space energy and stress upper triangle into the caller's outputs
__global__ void k_add_energy(const DevOut *o, double *pe, double *stress)
{
   if (threadIdx.x != 0) return;
   // a structure-factor tile that never arrived leaves the energy undefined
   *pe += (o->err & 4) ? __longlong_as_double(0x7ff8000000000000ll) : o->pe_k;
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
unsigned char *g_scratch[MAX_DEVICES];   // device address of the array, per device
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
   if (!g_scratch[dev]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, mdgpu_noalloc_scratch) != cudaSuccess || !p) {
         cudaGetLastError();
         return MDGPU_E_CUDA;
      }
      g_scratch[dev] = (unsigned char *)p;
   }
   unsigned char *S = g_scratch[dev];

   // k-vector list into the static host buffers
   const double kc = k_cutoff;
   const int hmax = (int)std::floor(kc / (2 * PI) * h[0]);
   const int kmax = (int)std::floor(kc / (2 * PI) * std::sqrt(h[1] * h[1] + h[4] * h[4]));
   const int lmax = (int)std::floor(kc / (2 * PI) * std::sqrt(h[2] * h[2] + h[5] * h[5] + h[8] * h[8]));
   double hinv[9], hp[9];
   inv3(h, hinv);
   for (int i = 0; i < 9; i++) hp[i] = 2 * PI * hinv[i];
   const double kcsq = kc * kc, vol = det3(h), r4a = -1.0 / (4.0 * alpha * alpha), eps0 = 0.25 / PI;
   int nk = 0, ni = 0;
   for (int hh = 0; hh <= hmax; hh++)
      for (int k = (hh == 0 ? 0 : -kmax); k <= kmax; k++) {
         const double kx = hh * hp[0] + k * hp[3], ky = hh * hp[1] + k * hp[4];
         const double kzt = hh * hp[2] + k * hp[5], ksq = kx * kx + ky * ky;
         int prev_l = -1000000;
         for (int l = (hh == 0 && k == 0 ? 1 : -lmax); l <= lmax; l++) {
            const double kz = kzt + l * hp[8];
            if (!(kz * kz + ksq < kcsq)) continue;
            if (nk >= MAX_KVEC) return MDGPU_E_CAPACITY;
            const bool extend = ni > 0 && prev_l == l - 1 && h_item[ni - 1].x == hh &&
                                h_item[ni - 1].y == k && h_item[ni - 1].w < KI;
            if (extend) {
               h_item[ni - 1].w++;
            } else {
               h_item[ni] = make_int4(hh, k, l, 1);
               h_k0[ni] = nk;
               h_kxy[ni] = make_float2((float)kx, (float)ky);
               ni++;
            }
            prev_l = l;
            const double ks = kx * kx + ky * ky + kz * kz;
            h_kvec[nk] = kx;
            h_kvec[MAX_KVEC + nk] = ky;
            h_kvec[2 * MAX_KVEC + nk] = kz;
            h_coef[nk] = 2.0 / (eps0 * vol) * std::exp(ks * r4a) / ks;
            h_coef2[nk] = 2.0 * (1.0 - ks * r4a) / ks;
            nk++;
         }
      }
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
   int *sorted = (int *)(S + O_SORT);
   float2 *part = (float2 *)(S + O_PART);
   double *fpart = (double *)(S + O_FPART), *blk = (double *)(S + O_BLK);

   cudaError_t e = cudaSuccess;
   auto up = [&](void *dst, const void *src, size_t bytes) {
      if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
   };
   up(item, h_item, sizeof(int4) * ni);
   up(k0, h_k0, sizeof(int) * ni);
   up(kxy, h_kxy, sizeof(float2) * ni);
   // k-vector components are laid out [3][nk] for the kernels
   up(kvec, h_kvec, sizeof(double) * nk);
   up(kvec + nk, h_kvec + MAX_KVEC, sizeof(double) * nk);
   up(kvec + 2 * nk, h_kvec + 2 * MAX_KVEC, sizeof(double) * nk);
   up(coef, h_coef, sizeof(double) * nk);
   up(coef2, h_coef2, sizeof(double) * nk);
   // the result record must start at zero; every other region is written
   // in full before it is read
   if (e == cudaSuccess) e = cudaMemsetAsync(out, 0, sizeof(DevOut), st);
   if (e != cudaSuccess) return MDGPU_E_CUDA;

   const int N = nsites;
   // site order: as given (no link-cell binning in this variant)
   k_iota<<<(N + 255) / 256, 256, 0, st>>>(N, sorted);
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
      item, k0, kxy, ni, nk, per_split, kdat, ph, zp, d_chg, sorted, N, 0, (float)hp[8], fpart);
   k_fsum<<<(3 * N + 255) / 256, 256, 0, st>>>(3 * N, splits, fpart, d_force, 1);
   k_add_energy<<<1, 32, 0, st>>>(out, d_pe, d_stress);
   e = cudaGetLastError();
   return e == cudaSuccess ? MDGPU_OK : MDGPU_E_CUDA;
}
