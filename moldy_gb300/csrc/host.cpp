// Host-side set-up of the force path: link-cell partition and neighbour-cell
// stencil, the half-sphere k-vector list, and the first-call constants
// (intramolecular correction, Ewald self and sheet energies).  All of it is
// integer or O(stencil) / O(k-list) FP64 work done once per cell shape; the
// per-site and per-pair work runs in the CUDA kernels.  Built with
// -ffp-contract=off: every expression is evaluated in the written order, as
// the reference's binning and cut-off decisions require.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "mdgpu_internal.h"

namespace mdgpu {

// 3x3 determinant and inverse by the adjoint method, in the evaluation
// order of det()/invert() (src/matrix.c:163-194).
double det3(const double *a)
{
   double d = 0.0;
   for (int i = 0; i < 3; i++) {
      int j = (i + 1) % 3, k = (i + 2) % 3;
      d += a[i] * (a[3 + j] * a[6 + k] - a[3 + k] * a[6 + j]);
   }
   return d;
}

void inv3(const double *a, double *b)
{
   double d = 1.0 / det3(a);
   for (int i = 0; i < 3; i++) {
      int j = (i + 1) % 3, k = (i + 2) % 3;
      for (int l = 0; l < 3; l++) {
         int m = (l + 1) % 3, n = (l + 2) % 3;
         b[3 * l + i] = d * (a[3 * j + m] * a[3 * k + n] - a[3 * j + n] * a[3 * k + m]);
      }
   }
}

static double col_norm(const double *m, int c)
{
   return std::sqrt(m[c] * m[c] + m[3 + c] * m[3 + c] + m[6 + c] * m[6 + c]);
}

static double lattice_dist2(const double *G, int ix, int iy, int iz, int nx, int ny, int nz)
{
   double s[3] = {(double)ix / nx, (double)iy / ny, (double)iz / nz}, dist = 0.0;
   for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) dist += s[i] * G[3 * i + j] * s[j];
   return dist;
}

// Half-space neighbour-cell stencil: cells whose origin lies within the
// cutoff of the reference cell's origin (neighbour_list,
// src/force.c:167-226), or in strict mode every cell with a corner-corner or
// face-face contact closer than the cutoff (strict_neighbour_list,
// src/force.c:273-421).  Offsets come out in the reference's order.
static mdgpu_status build_stencil(const double *h, double cutoff, int nx, int ny, int nz,
                                  bool strict, std::vector<int> &out)
{
   double htr[9], G[9], htrinv[9];
   for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) htr[3 * i + j] = h[3 * j + i];
   for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
         G[3 * i + j] = htr[3 * i] * h[j] + htr[3 * i + 1] * h[3 + j] + htr[3 * i + 2] * h[6 + j];
   inv3(htr, htrinv);
   int mx = (int)std::ceil(cutoff * nx * col_norm(htrinv, 0));
   int my = (int)std::ceil(cutoff * ny * col_norm(htrinv, 1));
   int mz = (int)std::ceil(cutoff * nz * col_norm(htrinv, 2));
   out.clear();
   auto beyond = [&](int ix, int iy, int iz) {
      return ix > nx || ix < -nx || iy > ny || iy < -ny || iz > nz || iz < -nz;
   };
   if (!strict) {
      for (int ix = 0; ix < mx; ix++)
         for (int iy = (ix == 0 ? 0 : -my); iy < my; iy++)
            for (int iz = (ix == 0 && iy == 0 ? 0 : -mz); iz < mz; iz++)
               if (lattice_dist2(G, ix, iy, iz, nx, ny, nz) < cutoff * cutoff) {
                  if (beyond(ix, iy, iz)) return MDGPU_E_CUTOFF;
                  out.push_back(ix);
                  out.push_back(iy);
                  out.push_back(iz);
               }
      return MDGPU_OK;
   }
   const int sy = 2 * my + 2, sz = 2 * mz + 2;
   std::vector<char> map((size_t)(mx + 1) * sy * sz, 0);
   auto at = [&](int x, int y, int z) -> char & {
      return map[((size_t)x * sy + (y + my + 1)) * sz + (z + mz + 1)];
   };
   for (int ix = 0; ix < mx; ix++)
      for (int iy = (ix == 0 ? 0 : -my); iy < my; iy++)
         for (int iz = (ix == 0 && iy == 0 ? 0 : -mz); iz < mz; iz++)
            if (lattice_dist2(G, ix, iy, iz, nx, ny, nz) < cutoff * cutoff)
               for (int i = 0; i <= 1; i++)
                  for (int j = -1; j <= 1; j++)
                     for (int k = -1; k <= 1; k++) at(ix + i, iy + j, iz + k) = 1;
   const int nxyz[3] = {nx, ny, nz}, mxyz[3] = {mx, my, mz};
   for (int a = 0; a < 3; a++) {  // face-face contacts along each axis
      int b = (a + 1) % 3, c = (b + 1) % 3, fc[4][3];
      double proj[3] = {0.0, 0.0, 0.0}, modabc = 0.0;
      for (int i = 0; i < 3; i++) {
         modabc += htrinv[3 * i + a];
         proj[i] += htrinv[3 * i + a] * htrinv[3 * i + (a + i) % 3];
      }
      for (int i = 0; i < 3; i++) proj[i] *= (mxyz[a] - 1) * nxyz[i] / (nxyz[a] * modabc);
      for (int i = 0; i < 3; i++) fc[0][i] = fc[1][i] = fc[2][i] = fc[3][i] = (int)std::floor(proj[i]);
      fc[0][a] = fc[1][a] = fc[2][a] = fc[3][a] = mxyz[a];
      fc[1][b] = fc[3][b] = (int)std::ceil(proj[b]);
      fc[2][c] = fc[3][c] = (int)std::ceil(proj[c]);
      for (int i = 0; i < 4; i++)
         if (fc[i][0] < 0)
            for (int j = 0; j < 3; j++) fc[i][j] = -fc[i][j];
      for (int i = 0; i < 4; i++)
         if (fc[i][0] >= 0 && fc[i][0] <= mx && fc[i][1] >= -my - 1 && fc[i][1] <= my &&
             fc[i][2] >= -mz - 1 && fc[i][2] <= mz)
            at(fc[i][0], fc[i][1], fc[i][2]) = 1;
   }
   for (int ix = 0; ix <= mx; ix++)
      for (int iy = (ix == 0 ? 0 : -my - 1); iy <= my; iy++)
         for (int iz = (ix == 0 && iy == 0 ? 0 : -mz - 1); iz <= mz; iz++)
            if (at(ix, iy, iz)) {
               if (beyond(ix, iy, iz)) return MDGPU_E_CUTOFF;
               out.push_back(ix);
               out.push_back(iy);
               out.push_back(iz);
            }
   return MDGPU_OK;
}

// The full stencil regrouped by (dx, dy): each run of consecutive dz is one
// column, so that the cells a column covers around a home cell are
// consecutive in the link-cell order (cell index cz + nz (cy + ny cx)) and
// their sites one contiguous range of slots.  Columns in (dx, dy) order;
// the offset vectors of a column's cells are laid out in dz order.
static void build_columns(RsGeom &g)
{
   std::vector<int4> e(g.full.begin(), g.full.end());
   std::sort(e.begin(), e.end(), [](const int4 &a, const int4 &b) {
      return a.x != b.x ? a.x < b.x : a.y != b.y ? a.y < b.y : a.z < b.z;
   });
   g.cols.clear();
   g.col_base.clear();
   g.coff_hi.clear();
   g.coff_lo.clear();
   g.cols_ok = true;
   bool have[27] = {false};
   for (size_t i = 0; i < e.size(); i++) {
      const int4 d = e[i];
      if (std::abs(d.x) <= 1 && std::abs(d.y) <= 1 && std::abs(d.z) <= 1)
         have[9 * (d.x + 1) + 3 * (d.y + 1) + (d.z + 1)] = true;
      const bool extend = !g.cols.empty() && g.cols.back().x == d.x && g.cols.back().y == d.y &&
                          g.cols.back().z + g.cols.back().w == d.z;
      if (extend) {
         g.cols.back().w++;
      } else {
         g.cols.push_back(make_int4(d.x, d.y, d.z, 1));
         g.col_base.push_back((int)g.coff_hi.size());
      }
      double v[3];
      for (int r = 0; r < 3; r++)
         v[r] = g.h[3 * r] * ((double)d.x / g.nx) + g.h[3 * r + 1] * ((double)d.y / g.ny) +
                g.h[3 * r + 2] * ((double)d.z / g.nz);
      float hi[3], lo[3];
      for (int r = 0; r < 3; r++) {
         hi[r] = (float)v[r];
         lo[r] = (float)(v[r] - (double)hi[r]);
      }
      g.coff_hi.push_back(make_float4(hi[0], hi[1], hi[2], 0.f));
      g.coff_lo.push_back(make_float4(lo[0], lo[1], lo[2], 0.f));
   }
   for (const int4 &c : g.cols)
      if (c.w > g.nz) g.cols_ok = false;
   // cell thickness along each lattice direction: 1 / (n_i |row i of h^-1|)
   bool thick = true;
   const int n[3] = {g.nx, g.ny, g.nz};
   for (int r = 0; r < 3; r++) {
      const double rn = std::sqrt(g.hinv[3 * r] * g.hinv[3 * r] + g.hinv[3 * r + 1] * g.hinv[3 * r + 1] +
                                  g.hinv[3 * r + 2] * g.hinv[3 * r + 2]);
      if (!(1.0 / (n[r] * rn) >= 0.5)) thick = false;
   }
   g.nbr27 = thick;
   for (int k = 0; k < 27; k++) g.nbr27 = g.nbr27 && have[k];
   // the column holding (dx, dy, -1 .. 1) for each neighbour column
   for (int d = 0; d < 9; d++) {
      const int dx = d / 3 - 1, dy = d % 3 - 1;
      g.nbcol[d] = -1;
      for (size_t i = 0; i < g.cols.size(); i++) {
         const int4 cd = g.cols[i];
         if (cd.x == dx && cd.y == dy && cd.z <= -1 && cd.z + cd.w - 1 >= 1) g.nbcol[d] = (int)i;
      }
      if (g.nbcol[d] < 0) g.nbr27 = false;
   }
   if (g.nz < 3) g.nbr27 = false;
}

mdgpu_status build_rs_geom(const double *h, const mdgpu_control &ctl, RsGeom &g)
{
   double subcell = ctl.subcell;
   if (subcell <= 0.0) subcell = ctl.cutoff / 5.0;           // src/force.c:1153
   g.nx = (int)(h[0] / subcell + 0.5);                        // src/force.c:1154-1156
   g.ny = (int)(h[4] / subcell + 0.5);
   g.nz = (int)(h[8] / subcell + 0.5);
   if (g.nx < 1 || g.ny < 1 || g.nz < 1) return MDGPU_E_ARG;
   g.ncells = g.nx * g.ny * g.nz;
   mdgpu_status s = build_stencil(h, ctl.cutoff, g.nx, g.ny, g.nz, ctl.strict_cutoff != 0, g.half);
   if (s != MDGPU_OK) return s;
   g.n_half = (int)g.half.size() / 3;
   for (int i = 0; i < 9; i++) g.h[i] = h[i];
   inv3(h, g.hinv);
   int t = 0;
   for (int ii = -1; ii <= 1; ii++)
      for (int jj = -1; jj <= 1; jj++)
         for (int kk = -1; kk <= 1; kk++, t++)
            for (int r = 0; r < 3; r++)
               g.reloc[t][r] = h[3 * r] * ii + h[3 * r + 1] * jj + h[3 * r + 2] * kk;
   const int n[3] = {g.nx, g.ny, g.nz};
   for (int r = 0; r < 3; r++)
      for (int cidx = 0; cidx < 3; cidx++) g.origin_step[3 * r + cidx] = h[3 * r + cidx] / n[cidx];
   // full stencil: the zero offset, then each half-space offset and its mirror
   g.full.clear();
   g.off_hi.clear();
   g.off_lo.clear();
   auto push = [&](int dx, int dy, int dz, int zero) {
      g.full.push_back(make_int4(dx, dy, dz, zero));
      double v[3];
      for (int r = 0; r < 3; r++)
         v[r] = h[3 * r] * ((double)dx / g.nx) + h[3 * r + 1] * ((double)dy / g.ny) +
                h[3 * r + 2] * ((double)dz / g.nz);
      float hi[3], lo[3];
      for (int r = 0; r < 3; r++) {
         hi[r] = (float)v[r];
         lo[r] = (float)(v[r] - (double)hi[r]);
      }
      g.off_hi.push_back(make_float4(hi[0], hi[1], hi[2], 0.f));
      g.off_lo.push_back(make_float4(lo[0], lo[1], lo[2], 0.f));
   };
   for (int e = 0; e < g.n_half; e++) {
      int dx = g.half[3 * e], dy = g.half[3 * e + 1], dz = g.half[3 * e + 2];
      if (dx == 0 && dy == 0 && dz == 0) {
         push(0, 0, 0, 1);
      } else {
         push(dx, dy, dz, 0);
         push(-dx, -dy, -dz, 0);
      }
   }
   g.cut2 = ctl.cutoff * ctl.cutoff;
   g.cut100 = 10000.0 * g.cut2;                               // src/force.c:831-832
   build_columns(g);
   return MDGPU_OK;
}

// Strict stencil for the radial distribution function (src/force.c:1307-1308:
// strict_neighbour_list at the RDF limit on the force call's cell grid),
// with each half-space offset followed by its mirror.
mdgpu_status build_rdf_stencil(const double *h, double limit, int nx, int ny, int nz, std::vector<int4> &full)
{
   std::vector<int> half;
   mdgpu_status s = build_stencil(h, limit, nx, ny, nz, true, half);
   if (s != MDGPU_OK) return s;
   full.clear();
   for (size_t e = 0; e < half.size() / 3; e++) {
      const int dx = half[3 * e], dy = half[3 * e + 1], dz = half[3 * e + 2];
      if (dx == 0 && dy == 0 && dz == 0) {
         full.push_back(make_int4(0, 0, 0, 1));
      } else {
         full.push_back(make_int4(dx, dy, dz, 0));
         full.push_back(make_int4(-dx, -dy, -dz, 0));
      }
   }
   return MDGPU_OK;
}

// k-vectors in the half sphere |k| < k_c, in the order ewald() builds them
// (src/ewald.c:441-461), grouped into items of up to KI consecutive l values
// of one (h,k) column; plus the per-k prefactors (src/ewald.c:510-511).
mdgpu_status build_klist(const double *h, const mdgpu_control &ctl, KList &kl)
{
   const double kc = ctl.k_cutoff, alpha = ctl.alpha;
   kl.hmax = (int)std::floor(kc / (2 * PI) * h[0]);
   kl.kmax = (int)std::floor(kc / (2 * PI) * std::sqrt(h[1] * h[1] + h[4] * h[4]));
   kl.lmax = (int)std::floor(kc / (2 * PI) * std::sqrt(h[2] * h[2] + h[5] * h[5] + h[8] * h[8]));
   double hinvp[9];
   inv3(h, hinvp);
   for (int i = 0; i < 9; i++) kl.hinv[i] = hinvp[i];
   for (int i = 0; i < 9; i++) hinvp[i] = 2 * PI * hinvp[i];
   kl.dkz = hinvp[8];
   const double kcsq = kc * kc;
   kl.vol = det3(h);
   const double r4a = -1.0 / (4.0 * alpha * alpha);
   const double eps0 = 0.25 / PI;
   kl.item.clear();
   kl.item_k0.clear();
   kl.item_kxy.clear();
   kl.kz.clear();
   kl.coeff.clear();
   kl.coeff2.clear();
   int nk = 0;
   std::vector<int4> cols;         // (h, k, l0, count) of each column
   std::vector<int> col_item;      // its first item (before the sort)
   std::vector<float2> col_kxy;
   for (int hh = 0; hh <= kl.hmax; hh++)
      for (int k = (hh == 0 ? 0 : -kl.kmax); k <= kl.kmax; k++) {
         double kx = hh * hinvp[0] + k * hinvp[3];
         double ky = hh * hinvp[1] + k * hinvp[4];
         double kzt = hh * hinvp[2] + k * hinvp[5];
         double ksq = kx * kx + ky * ky;
         int prev_l = -1000000;
         for (int l = (hh == 0 && k == 0 ? 1 : -kl.lmax); l <= kl.lmax; l++) {
            double kz = kzt + l * hinvp[8];
            if (kz * kz + ksq < kcsq) {
               bool extend = !kl.item.empty() && prev_l == l - 1 && kl.item.back().x == hh &&
                             kl.item.back().y == k && kl.item.back().w < KI;
               if (extend)
                  kl.item.back().w++;
               else {
                  if (prev_l != l - 1) {   // a new column
                     cols.push_back(make_int4(hh, k, l, 0));
                     col_item.push_back((int)kl.item.size());
                     col_kxy.push_back(make_float2((float)kx, (float)ky));
                  }
                  kl.item.push_back(make_int4(hh, k, l, 1));
                  kl.item_k0.push_back(nk);
                  kl.item_kxy.push_back(make_double2(kx, ky));
               }
               prev_l = l;
               double ks = kx * kx + ky * ky + kz * kz;
               kl.kz.push_back(kz);
               kl.coeff.push_back(2.0 / (eps0 * kl.vol) * std::exp(ks * r4a) / ks);
               kl.coeff2.push_back(2.0 * (1.0 - ks * r4a) / ks);
               nk++;
            }
         }
      }
   kl.nk = nk;
   kl.nitems = (int)kl.item.size();
   // Items with the same k count side by side, full ones first: a warp (or a
   // block, in the force pass) then meets one count at a time and the full
   // items take a path with no per-k predicate.  Only the order of the sum
   // over k changes.
   std::vector<int> order(kl.nitems);
   for (int i = 0; i < kl.nitems; i++) order[i] = i;
   std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return kl.item[a].w > kl.item[b].w; });
   KList o;
   o.item.reserve(kl.nitems);
   std::vector<int> new_k0(kl.nitems), pre_w(kl.nitems);
   for (int i = 0; i < kl.nitems; i++) pre_w[i] = kl.item[i].w;
   int k0 = 0;
   for (int i : order) {
      const int4 it = kl.item[i];
      new_k0[i] = k0;
      o.item.push_back(it);
      o.item_k0.push_back(k0);
      o.item_kxy.push_back(kl.item_kxy[i]);
      for (int t = 0; t < it.w; t++) {
         const int k = kl.item_k0[i] + t;
         o.kz.push_back(kl.kz[k]);
         o.coeff.push_back(kl.coeff[k]);
         o.coeff2.push_back(kl.coeff2[k]);
      }
      k0 += it.w;
   }
   kl.item.swap(o.item);
   kl.item_k0.swap(o.item_k0);
   kl.item_kxy.swap(o.item_kxy);
   kl.kz.swap(o.kz);
   kl.coeff.swap(o.coeff);
   kl.coeff2.swap(o.coeff2);
   // Tensor-core items: each column cut into runs of KT from its first l,
   // so run r holds the column's KI items 4r .. 4r+3 (contiguous k each).
   kl.tc_item.clear();
   kl.tc_k0.clear();
   kl.tc_kxy.clear();
   for (size_t c = 0; c < cols.size(); c++) {
      const int f = col_item[c], e = c + 1 < cols.size() ? col_item[c + 1] : kl.nitems;
      int total = 0;
      for (int i = f; i < e; i++) total += pre_w[i];
      for (int r = 0; r * KT < total; r++) {
         int ki[4];
         for (int j = 0; j < 4; j++) {
            const int run = 4 * r + j;
            ki[j] = run * KI < total ? new_k0[f + run] : -1;
         }
         kl.tc_item.push_back(make_int4(cols[c].x, cols[c].y, cols[c].z + r * KT, std::min(KT, total - r * KT)));
         kl.tc_k0.push_back(make_int4(ki[0], ki[1], ki[2], ki[3]));
         kl.tc_kxy.push_back(col_kxy[c]);
      }
   }
   kl.tc_nitems = (int)kl.tc_item.size();
   {
      std::vector<int> ord(kl.tc_nitems);
      for (int i = 0; i < kl.tc_nitems; i++) ord[i] = i;
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return kl.tc_item[a].w > kl.tc_item[b].w; });
      std::vector<int4> it2, k02;
      std::vector<float2> kxy2;
      for (int i : ord) {
         it2.push_back(kl.tc_item[i]);
         k02.push_back(kl.tc_k0[i]);
         kxy2.push_back(kl.tc_kxy[i]);
      }
      while (it2.size() % 128) {
         it2.push_back(make_int4(0, 0, 0, 0));
         k02.push_back(make_int4(-1, -1, -1, -1));
         kxy2.push_back(make_float2(0.f, 0.f));
      }
      kl.tc_item.swap(it2);
      kl.tc_k0.swap(k02);
      kl.tc_kxy.swap(kxy2);
   }
   return MDGPU_OK;
}

// ---- pair potential at one distance (kernel() for one pair, poteval) -----
#define AS1 0.254829592
#define AS2 -0.284496736
#define AS3 1.421413741
#define AS4 -1.453152027
#define AS5 1.061405429
#define ASP 0.3275911
#define ASPOLY(t) ((t) * (AS1 + (t) * (AS2 + (t) * (AS3 + (t) * (AS4 + (t) * AS5)))))

double host_poteval(const double *p, double r, int ptype, double chgsq, double alpha)
{
   // poteval (src/force.c:632-650): kernel() on one pair of squared
   // distance rr = r*r, neighbour charge chgsq, reference charge 1.
   const double rr = r * r, norm = 2.0 * alpha / std::sqrt(PI);
   double pe = 0.0, t = 0.0, ef = 0.0, rs_r, r_r, rv, r4, r6, r8, r12, e1, e2, e3;
   if (alpha > 0.0) {
      rv = std::sqrt(rr);
      double ar = alpha * rv;
      t = 1.0 / (1.0 + ASP * ar);
      ef = chgsq * 1.0 * std::exp(-(ar * ar));
      r_r = 1.0 / rv;
      t = ASPOLY(t) * ef * r_r;
      rs_r = r_r * r_r;
      switch (ptype) {
      case 0:
         r6 = (p[1] * p[1]) * rs_r;
         r6 = r6 * r6 * r6;
         r12 = r6 * r6;
         pe += t + p[0] * (r12 - r6);
         break;
      case 1:
         e1 = p[1] * std::exp(-p[2] * rv);
         r6 = p[0] * (rs_r * rs_r * rs_r);
         pe += t - r6 + e1;
         break;
      case 2:
         e1 = p[0] * std::exp(-p[1] * rv);
         e2 = -p[2] * std::exp(-p[3] * rv);
         pe += t + e1 + e2;
         break;
      case 3:
         e1 = p[0] * std::exp(-p[1] * rv);
         r4 = rs_r * rs_r;
         r6 = rs_r * r4;
         r8 = p[5] * (r4 * r4);
         r12 = p[2] * (r6 * r6);
         r4 *= p[3];
         r6 *= p[4];
         pe += t + e1 + r12 - r4 - r6 - r8;
         break;
      case 4:
         r4 = rs_r * rs_r;
         r6 = rs_r * r4;
         r12 = p[2] * (r6 * r6);
         r6 *= p[1];
         r4 *= p[0];
         pe += t + r4 + r6 + r12;
         break;
      case 6:
         e1 = p[0] * std::exp((p[1] - rv) * p[2]);
         r6 = p[3] * (rs_r * rs_r * rs_r);
         e2 = p[4] * std::exp(-2.0 * p[5] * (rv - p[6]));
         e3 = -p[4] * 2.0 * std::exp(-p[5] * (rv - p[6]));
         pe += t + e1 - r6 + e2 + e3;
         break;
      default:
         return NAN;
      }
   } else {
      switch (ptype) {
      case 0:
         rs_r = 1.0 / rr;
         r6 = (p[1] * p[1]) * rs_r;
         r6 = r6 * r6 * r6;
         r12 = r6 * r6;
         pe += p[0] * (r12 - r6);
         break;
      case 1:
         rv = std::sqrt(rr);
         r_r = 1.0 / rv;
         e1 = p[1] * std::exp(-p[2] * rv);
         rs_r = r_r * r_r;
         r6 = p[0] * rs_r * rs_r * rs_r;
         pe += -r6 + e1;
         break;
      case 2:
         rv = std::sqrt(rr);
         e1 = p[0] * std::exp(-p[1] * rv);
         e2 = -p[2] * std::exp(-p[3] * rv);
         pe += e1 + e2;
         break;
      case 3:
         rv = std::sqrt(rr);
         r_r = 1.0 / rv;
         e1 = p[0] * std::exp(-p[1] * rv);
         rs_r = r_r * r_r;
         r4 = rs_r * rs_r;
         r6 = rs_r * r4;
         r8 = p[5] * (r4 * r4);
         r12 = p[2] * (r6 * r6);
         r4 *= p[3];
         r6 *= p[4];
         pe += e1 + r12 - r4 - r6 - r8;
         break;
      case 4:
         rv = std::sqrt(rr);
         r_r = 1.0 / rv;
         rs_r = r_r * r_r;
         r4 = rs_r * rs_r;
         r6 = rs_r * r4;
         r12 = (r6 * r6) * p[2];
         r6 *= p[1];
         r4 *= p[0];
         pe += r4 + r6 + r12;
         break;
      case 6:
         rv = std::sqrt(rr);
         r_r = 1.0 / rv;
         rs_r = r_r * r_r;
         e1 = p[0] * std::exp((p[1] - rv) * p[2]);
         r6 = p[3] * (rs_r * rs_r * rs_r);
         e2 = p[4] * std::exp(-2.0 * p[5] * (rv - p[6]));
         e3 = -p[4] * 2.0 * std::exp(-p[5] * (rv - p[6]));
         pe += e1 - r6 + e2 + e3;
         break;
      default:
         return NAN;
      }
   }
   return pe;
}

// Intramolecular energy of every non-framework species, summed over its
// molecules (pe_intra, src/force.c:654-668; force.c:1156-1171).
double intramolecular_energy(const std::vector<mdgpu_species> &spec,
                             const std::vector<int> &spec_ids, const std::vector<double> &spec_pf,
                             const double *potpar, int max_id, int ptype,
                             const std::vector<double> &chg, double alpha)
{
   double eintra = 0.0;
   size_t so = 0, isite = 0;
   for (const auto &s : spec) {
      if (!s.framework) {
         const int *ids = spec_ids.data() + so;
         const double *pf = spec_pf.data() + 3 * so;
         const double *q = chg.data() + isite;
         double e = 0.0;
         for (int a = 0; a < s.nsites; a++)
            for (int b = a + 1; b < s.nsites; b++) {
               const double *u = pf + 3 * b, *v = pf + 3 * a;
               double r = std::sqrt((u[0] - v[0]) * (u[0] - v[0]) + (u[1] - v[1]) * (u[1] - v[1]) +
                                    (u[2] - v[2]) * (u[2] - v[2]));
               e += host_poteval(potpar + ((size_t)ids[a] * max_id + ids[b]) * NPOTP, r, ptype,
                                 q[b] * q[a], alpha);
            }
         eintra += s.nmols * e;
      }
      so += s.nsites;
      isite += (size_t)s.nsites * s.nmols;
   }
   return eintra;
}

static double as_erf(double x)
{
   double t = 1.0 / (1.0 + ASP * x);
   if (x >= 0.0) return 1.0 - ASPOLY(t) * std::exp(-x * x);
   return -as_erf(-x);
}

// d/dx of the A&S erfc approximation t P(t) e^{-x^2}, t = 1/(1 + p x), x >= 0.
static double as_derfc(double x)
{
   const double t = 1.0 / (1.0 + ASP * x);
   const double pt = AS1 + t * (AS2 + t * (AS3 + t * (AS4 + t * AS5)));
   const double dpt = AS2 + t * (2.0 * AS3 + t * (3.0 * AS4 + t * 4.0 * AS5));
   return std::exp(-x * x) * (-ASP * t * t * (pt + t * dpt) - 2.0 * x * t * pt);
}

// Gradient of the energy terms ewald() adds besides the k sum,
// -self + sheet/V (src/ewald.c:367-433): with respect to each site charge
// (added into g_chg[nsites]) and alpha (added into *g_alpha).  The self
// energy covers the species before the framework, if any
// (src/ewald.c:372-397); its intramolecular part is taken per molecule with
// its own charges (the reference evaluates the first molecule of each
// species, whose charges every molecule of the species shares).  A
// framework's net charge q_f adds pi q_f^2 / (2 alpha^2) to the sheet term
// (src/ewald.c:405-413); a net system charge sq subtracts pi sq^2 / (2
// alpha^2) (src/ewald.c:417-422).
void ewald_self_sheet_grad(const std::vector<mdgpu_species> &spec, const std::vector<double> &spec_pf,
                           const std::vector<double> &chg, double alpha, double vol, double *g_chg,
                           double *g_alpha)
{
   const double rpi = 1.0 / std::sqrt(PI);
   double ga = 0.0, sq = 0.0, qf = 0.0;
   size_t isite = 0, so = 0, fw0 = chg.size();
   bool in_fw = false;
   for (const auto &sp : spec) {
      const int ns = sp.nsites;
      const double *pf = spec_pf.data() + 3 * so;
      in_fw = in_fw || sp.framework;
      if (in_fw && fw0 == chg.size()) fw0 = isite;
      for (int m = 0; m < sp.nmols; m++) {
         const double *q = chg.data() + isite;
         for (int a = 0; a < ns; a++) {
            sq += q[a];
            if (in_fw) {
               qf += q[a];
               continue;
            }
            g_chg[isite + a] -= 2.0 * alpha * rpi * q[a];
            ga -= rpi * q[a] * q[a];
            for (int b = a + 1; b < ns; b++) {
               const double *u = pf + 3 * a, *v = pf + 3 * b;
               const double r = std::sqrt((u[0] - v[0]) * (u[0] - v[0]) + (u[1] - v[1]) * (u[1] - v[1]) +
                                          (u[2] - v[2]) * (u[2] - v[2]));
               const double e = as_erf(alpha * r) / r;
               g_chg[isite + a] -= q[b] * e;
               g_chg[isite + b] -= q[a] * e;
               ga += q[a] * q[b] * as_derfc(alpha * r);   // d erf/dx = -d erfc/dx
            }
         }
         isite += ns;
      }
      so += ns;
   }
   if (in_fw) {   // sheet += pi q_f^2 / (2 alpha^2)
      const double dq = PI * qf / (alpha * alpha * vol);
      for (size_t i = fw0; i < isite; i++) g_chg[i] += dq;
      ga -= PI * qf * qf / (alpha * alpha * alpha * vol);
   }
   const double conv_q = (4.07497263794495e-14 * 1.0e-3 * 1.05482230112e-05) / 1.60217733e-19;
   if (std::fabs(sq) * conv_q > 1.0e-5) {   // sheet -= pi (sum q)^2 / (2 alpha^2)
      const double dq = -PI * sq / (alpha * alpha * vol);
      for (size_t i = 0; i < isite; i++) g_chg[i] += dq;
      ga += PI * sq * sq / (alpha * alpha * alpha * vol);
   }
   *g_alpha += ga;
}

// Ewald self energy and charged-system sheet correction (src/ewald.c:367-425).
void ewald_self_sheet(const std::vector<mdgpu_species> &spec, const std::vector<double> &spec_pf,
                      const std::vector<double> &chg, double alpha, double *self, double *sheet,
                      int *nsitesxf)
{
   double se = 0.0, sh = 0.0, sq = 0.0, sqsq = 0.0;
   size_t ssite = 0, so = 0, s = 0;
   for (; s < spec.size() && !spec[s].framework; s++) {
      double intra = 0.0;
      const int ns = spec[s].nsites;
      const double *pf = spec_pf.data() + 3 * so;
      for (int a = 0; a < ns; a++)
         for (int b = a + 1; b < ns; b++) {
            const double *u = pf + 3 * a, *v = pf + 3 * b;
            double r = std::sqrt((u[0] - v[0]) * (u[0] - v[0]) + (u[1] - v[1]) * (u[1] - v[1]) +
                                 (u[2] - v[2]) * (u[2] - v[2]));
            intra += chg[ssite + a] * chg[ssite + b] * as_erf(alpha * r) / r;
         }
      se += spec[s].nmols * intra;
      ssite += (size_t)ns * spec[s].nmols;
      so += ns;
   }
   const bool frame_flag = s != spec.size();
   const size_t nxf = ssite;
   size_t i = 0;
   for (; i < nxf; i++) {
      sq += chg[i];
      sqsq += chg[i] * chg[i];
   }
   se += alpha / std::sqrt(PI) * sqsq;
   const double sqxf = sq;
   for (; i < chg.size(); i++) sq += chg[i];
   const double conv_q = (4.07497263794495e-14 * 1.0e-3 * 1.05482230112e-05) / 1.60217733e-19;
   if (frame_flag) sh = PI * (sq - sqxf) * (sq - sqxf) / (2.0 * (alpha * alpha));
   if (std::fabs(sq) * conv_q > 1.0e-5) sh -= PI * (sq * sq) / (2.0 * (alpha * alpha));
   *self = se;
   *sheet = sh;
   *nsitesxf = (int)nxf;
}


// -int_rc^inf r^2 U(r) dr of the short-range part (dist_pot, src/kernel.c:103-150)
static double dist_pot(const double *p, double rc, int ptype)
{
   const double tol = 1.0e-7;   // BPAR_TOL, src/kernel.c:97
   const double rc3 = rc * rc * rc;
   switch (ptype) {
   case 0:
      {
      const double t = p[1] * p[1] / rc;
      return p[0] * (t * t * t) / 3.0;
   }
   case 1:
      if (p[2] > tol)
         return p[0] / (3.0 * rc3) -
                p[1] * std::exp(-p[2] * rc) * (rc * rc / p[2] + 2 * rc / (p[2] * p[2]) + 2.0 / (p[2] * p[2] * p[2]));
      return p[0] / (3.0 * rc3);
   case 2:
      if (p[3] > tol)
         return p[2] * (rc * rc / p[3] + 2 * rc / (p[3] * p[3]) + 2.0 / (p[3] * p[3] * p[3])) * std::exp(-p[3] * rc);
      return 0.0;
   case 3: {
      const double tail = -p[2] / (9.0 * rc3 * rc3 * rc3) + p[3] / rc + p[4] / (3.0 * rc3) + p[5] / (5.0 * rc * rc * rc3);
      if (p[1] > tol)
         return -p[0] * std::exp(-p[1] * rc) * (rc * rc / p[1] + 2 * rc / (p[1] * p[1]) + 2.0 / (p[1] * p[1] * p[1])) +
                tail;
      return tail;
   }
   case 6:
      if (p[5] != 0.0)
         return p[3] / (3.0 * rc3) + 2.0 * p[4] * (rc * rc / p[5] + 2 * rc / (p[5] * p[5]) + 2.0 / (p[5] * p[5] * p[5])) *
                                        std::exp(-p[5] * (rc - p[6]));
      return p[3] / (3.0 * rc3);
   case 4:
      return -p[0] / rc - p[1] / rc3 / 3.0 - p[2] / (rc3 * rc3 * rc3) / 9.0;
   default:
      return 0.0;
   }
}

static double distant_impl(const mdgpu_ctx *c, bool pressure)
{
   const int M = c->max_id;
   std::vector<long long> count(M, 0);
   size_t so = 0;
   for (const auto &sp : c->spec) {
      for (int k = 0; k < sp.nsites; k++) count[c->spec_ids[so + k]] += sp.nmols;
      so += sp.nsites;
   }
   const double rc = c->ctl.cutoff;
   double cst = 0.0;
   for (int id = 1; id < M; id++)
      for (int jd = 1; jd < M; jd++) {
         const double *p = c->potpar.data() + ((size_t)id + (size_t)M * jd) * NPOTP;
         cst -= 2 * PI * (double)count[id] * (double)count[jd] * dist_pot(p, rc, c->ptype);
         if (pressure)
            cst += 2.0 / 3.0 * PI * (double)count[id] * (double)count[jd] * (rc * rc * rc) *
                   host_poteval(p, rc, c->ptype, 0.0, c->ctl.alpha);
      }
   return cst;
}

double distant_const(const mdgpu_ctx *c) { return distant_impl(c, false); }
double distant_pconst(const mdgpu_ctx *c) { return distant_impl(c, true); }

}  // namespace mdgpu
