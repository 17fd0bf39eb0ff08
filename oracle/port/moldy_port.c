/*
 * moldy_port.c -- TEST INFRASTRUCTURE ONLY: C restatement of Moldy's force
 * path, used as the parity oracle and as the timed CPU baseline.  Each
 * function cites the reference code it restates.  Built with
 * -ffp-contract=off so that every floating-point expression is evaluated in
 * the order written (no fused multiply-adds), which the binning and the
 * strict-cutoff clamp need to reproduce the reference bit for bit.
 */
#include "moldy_port.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define PI_        3.14159265358979323846
#define NPOTP_     8
#define XTRA       1        /* image cells beyond the MD cell, src/force.c:90  */
#define NIMG       27
#define TOO_CLOSE_ 0.25     /* src/force.c:89                                 */
#define NMULT_     2.0      /* src/force.c:88                                 */
#define ALPHAMIN_  1e-7     /* src/defs.h:181                                 */
/* Abramowitz & Stegun 7.1.26 constants (src/kernel.c:88-96, src/auxil.c:577-583) */
#define AS1  0.254829592
#define AS2 -0.284496736
#define AS3  1.421413741
#define AS4 -1.453152027
#define AS5  1.061405429
#define ASP  0.3275911
#define ASPOLY(t) ((t)*(AS1 + (t)*(AS2 + (t)*(AS3 + (t)*(AS4 + (t)*AS5)))))

/* charge conversion, src/defs.h:201-235 */
#define CONVQ_ ((4.07497263794495e-14 * 1.0e-3 * 1.05482230112e-05) / 1.60217733e-19)

static double wall(void)
{
   struct timespec t;
   clock_gettime(CLOCK_MONOTONIC, &t);
   return t.tv_sec + 1e-9 * t.tv_nsec;
}

/* ---- 3x3 algebra, evaluated in the same order as src/matrix.c ---------- */
static double det3(const double a[3][3])
{
   double d = 0.0;
   int i;
   for (i = 0; i < 3; i++) {
      int j = (i + 1) % 3, k = (i + 2) % 3;
      d += a[0][i] * (a[1][j] * a[2][k] - a[1][k] * a[2][j]);
   }
   return d;
}

static int inv3(const double a[3][3], double b[3][3])
{
   double d = det3(a);
   int i, l;
   if (d == 0.0) return -1;
   d = 1.0 / d;
   for (i = 0; i < 3; i++) {
      int j = (i + 1) % 3, k = (i + 2) % 3;
      for (l = 0; l < 3; l++) {
         int m = (l + 1) % 3, n = (l + 2) % 3;
         b[l][i] = d * (a[j][m] * a[k][n] - a[j][n] * a[k][m]);
      }
   }
   return 0;
}

static void mul3(const double a[3][3], const double b[3][3], double c[3][3])
{
   int i, j;
   for (i = 0; i < 3; i++)
      for (j = 0; j < 3; j++)
         c[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
}

static void tr3(const double a[3][3], double b[3][3])
{
   int i, j;
   for (i = 0; i < 3; i++)
      for (j = 0; j < 3; j++)
         b[i][j] = a[j][i];
}

/* ---- link-cell geometry ------------------------------------------------ */
typedef struct { int d[3]; } off3;

/* Cell index of one fractional co-ordinate with the edge fix-ups of
 * cellbin() (src/force.c:119-137); *bad counts out-of-range values. */
static int bin1(double s, int n, double fn, double eps, int *bad)
{
   int ib;
   if (s < -0.5 + eps || s >= 0.5 - eps) {
      if (s < -0.5 + eps && s >= -0.5 - eps)
         s = -0.5;
      else if (s >= 0.5 - eps && s <= 0.5 + eps)
         s = 0.5 - eps;
      else
         (*bad)++;
   }
   ib = (int)floor((s + 0.5) * fn);
   if (ib >= n || ib < 0) {
      (*bad)++;
      ib = ib < 0 ? 0 : n - 1;
   }
   return ib;
}

static double col_norm(const double m[3][3], int c)
{
   return sqrt(m[0][c] * m[0][c] + m[1][c] * m[1][c] + m[2][c] * m[2][c]);
}

/* s . G . s with the loop order of neighbour_list (src/force.c:191-196). */
static double lattice_dist2(const double G[3][3], int ix, int iy, int iz, int nx, int ny, int nz)
{
   double s[3], dist = 0.0;
   int i, j;
   s[0] = (double)ix / nx;
   s[1] = (double)iy / ny;
   s[2] = (double)iz / nz;
   for (i = 0; i < 3; i++)
      for (j = 0; j < 3; j++)
         dist += s[i] * G[i][j] * s[j];
   return dist;
}

/* Half-space stencil of cell offsets.  Lazy mode keeps offsets whose lattice
 * vector is shorter than the cutoff (neighbour_list, src/force.c:167-226);
 * strict mode adds every cell sharing a corner-corner or face-face contact
 * closer than the cutoff (strict_neighbour_list, src/force.c:273-421).
 * Returns the count, or PORT_E_CUTOFF when a cell lies beyond one image. */
static int build_stencil(const double h[3][3], double cutoff, int nx, int ny, int nz,
                         int strict, off3 **out)
{
   double G[3][3], htr[3][3], htrinv[3][3];
   int mx, my, mz, ix, iy, iz, n = 0, cap;
   off3 *list;
   tr3(h, htr);
   mul3(htr, h, G);
   inv3(htr, htrinv);
   mx = (int)ceil(cutoff * nx * col_norm(htrinv, 0));
   my = (int)ceil(cutoff * ny * col_norm(htrinv, 1));
   mz = (int)ceil(cutoff * nz * col_norm(htrinv, 2));
   if (!strict) {
      cap = 4 * mx * my * mz + 1;
      list = (off3 *)malloc(sizeof(off3) * cap);
      for (ix = 0; ix < mx; ix++)
         for (iy = (ix == 0 ? 0 : -my); iy < my; iy++)
            for (iz = (ix == 0 && iy == 0 ? 0 : -mz); iz < mz; iz++)
               if (lattice_dist2(G, ix, iy, iz, nx, ny, nz) < cutoff * cutoff) {
                  if (ix > XTRA * nx || ix < -XTRA * nx || iy > XTRA * ny || iy < -XTRA * ny ||
                      iz > XTRA * nz || iz < -XTRA * nz) {
                     free(list);
                     return PORT_E_CUTOFF;
                  }
                  list[n].d[0] = ix; list[n].d[1] = iy; list[n].d[2] = iz;
                  n++;
               }
   } else {
      /* occupancy map over ix in [0,mx], iy in [-my-1,my], iz in [-mz-1,mz] */
      int sy = 2 * my + 2, sz = 2 * mz + 2, i, j, k, a;
      char *map = (char *)calloc((size_t)(mx + 1) * sy * sz, 1);
#define MAP(x, y, z) map[((size_t)(x) * sy + ((y) + my + 1)) * sz + ((z) + mz + 1)]
      int mxyz[3], nxyz[3];
      for (ix = 0; ix < mx; ix++)
         for (iy = (ix == 0 ? 0 : -my); iy < my; iy++)
            for (iz = (ix == 0 && iy == 0 ? 0 : -mz); iz < mz; iz++)
               if (lattice_dist2(G, ix, iy, iz, nx, ny, nz) < cutoff * cutoff)
                  for (i = 0; i <= 1; i++)
                     for (j = -1; j <= 1; j++)
                        for (k = -1; k <= 1; k++)
                           MAP(ix + i, iy + j, iz + k) = 1;
      nxyz[0] = nx; nxyz[1] = ny; nxyz[2] = nz;
      mxyz[0] = mx; mxyz[1] = my; mxyz[2] = mz;
      for (a = 0; a < 3; a++) {            /* face-face contacts, force.c:353-394 */
         int b = (a + 1) % 3, c = (b + 1) % 3, fc[4][3];
         double proj[3] = {0.0, 0.0, 0.0}, modabc = 0.0;
         for (i = 0; i < 3; i++) {
            modabc += htrinv[i][a];
            proj[i] += htrinv[i][a] * htrinv[i][(a + i) % 3];
         }
         for (i = 0; i < 3; i++)
            proj[i] *= (mxyz[a] - 1) * nxyz[i] / (nxyz[a] * modabc);
         for (i = 0; i < 3; i++)
            fc[0][i] = fc[1][i] = fc[2][i] = fc[3][i] = (int)floor(proj[i]);
         fc[0][a] = fc[1][a] = fc[2][a] = fc[3][a] = mxyz[a];
         fc[1][b] = fc[3][b] = (int)ceil(proj[b]);
         fc[2][c] = fc[3][c] = (int)ceil(proj[c]);
         for (i = 0; i < 4; i++)
            if (fc[i][0] < 0)
               for (j = 0; j < 3; j++) fc[i][j] = -fc[i][j];
         for (i = 0; i < 4; i++)
            if (fc[i][0] >= 0 && fc[i][0] <= mx && fc[i][1] >= -my - 1 && fc[i][1] <= my &&
                fc[i][2] >= -mz - 1 && fc[i][2] <= mz)
               MAP(fc[i][0], fc[i][1], fc[i][2]) = 1;
      }
      cap = (mx + 1) * sy * sz;
      list = (off3 *)malloc(sizeof(off3) * cap);
      for (ix = 0; ix <= mx; ix++)
         for (iy = (ix == 0 ? 0 : -my - 1); iy <= my; iy++)
            for (iz = (ix == 0 && iy == 0 ? 0 : -mz - 1); iz <= mz; iz++)
               if (MAP(ix, iy, iz)) {
                  if (ix > XTRA * nx || ix < -XTRA * nx || iy > XTRA * ny || iy < -XTRA * ny ||
                      iz > XTRA * nz || iz < -XTRA * nz) {
                     free(list);
                     free(map);
                     return PORT_E_CUTOFF;
                  }
                  list[n].d[0] = ix; list[n].d[1] = iy; list[n].d[2] = iz;
                  n++;
               }
#undef MAP
      free(map);
   }
   *out = list;
   return n;
}

/* ---- pair potentials (src/kernel.c:157-463) ---------------------------- */
/* Evaluates pairs [j0, j1): force[j] = -U'(r)/r, returns sum of U.  p[k][j]
 * holds parameter k of the pair (isite, nab[j]). */
static int pair_kernel(int j0, int j1, double *force, double *pe, const double *r2,
                       const double *qj, double qi, double norm, double alpha, int ptype,
                       double *const *p)
{
   double ppe = 0.0, t, ar, r, r_r, rs_r, r4, r6, r8, r12, ef, e1, e2, e3;
   const double *p0 = p[0], *p1 = p[1], *p2 = p[2], *p3 = p[3], *p4 = p[4], *p5 = p[5],
                *p6 = p[6];
   int j;
   if (alpha > 0.0) {
      for (j = j0; j < j1; j++) {
         r = sqrt(r2[j]);
         ar = alpha * r;
         t = 1.0 / (1.0 + ASP * ar);
         ef = qj[j] * qi * exp(-(ar * ar));
         r_r = 1.0 / r;
         t = ASPOLY(t) * ef * r_r;          /* q_i q_j erfc(alpha r) / r */
         ef = t + norm * ef;
         rs_r = r_r * r_r;
         switch (ptype) {
         case 0:
            r6 = (p1[j] * p1[j]) * rs_r;
            r6 = r6 * r6 * r6;
            r12 = r6 * r6;
            ppe += t + p0[j] * (r12 - r6);
            force[j] = rs_r * (6.0 * p0[j] * (2 * r12 - r6) + ef);
            break;
         case 1:
            e1 = p1[j] * exp(-p2[j] * r);
            r6 = p0[j] * (rs_r * rs_r * rs_r);
            ppe += t - r6 + e1;
            force[j] = rs_r * (-6.0 * r6 + ef) + p2[j] * e1 * r_r;
            break;
         case 2:
            e1 = p0[j] * exp(-p1[j] * r);
            e2 = -p2[j] * exp(-p3[j] * r);
            ppe += t + e1 + e2;
            force[j] = (p1[j] * e1 + p3[j] * e2) * r_r + ef * rs_r;
            break;
         case 3:
            e1 = p0[j] * exp(-p1[j] * r);
            r4 = rs_r * rs_r;
            r6 = rs_r * r4;
            r8 = p5[j] * (r4 * r4);
            r12 = p2[j] * (r6 * r6);
            r4 *= p3[j];
            r6 *= p4[j];
            ppe += t + e1 + r12 - r4 - r6 - r8;
            force[j] = rs_r * (12.0 * r12 - 4.0 * r4 - 6.0 * r6 - 8.0 * r8 + ef) + p1[j] * e1 * r_r;
            break;
         case 4:
            r4 = rs_r * rs_r;
            r6 = rs_r * r4;
            r12 = p2[j] * (r6 * r6);
            r6 *= p1[j];
            r4 *= p0[j];
            ppe += t + r4 + r6 + r12;
            force[j] = rs_r * (4.0 * r4 + 6.0 * r6 + 12.0 * r12 + ef);
            break;
         case 6:
            e1 = p0[j] * exp((p1[j] - r) * p2[j]);
            r6 = p3[j] * (rs_r * rs_r * rs_r);
            e2 = p4[j] * exp(-2.0 * p5[j] * (r - p6[j]));
            e3 = -p4[j] * 2.0 * exp(-p5[j] * (r - p6[j]));
            ppe += t + e1 - r6 + e2 + e3;
            force[j] = rs_r * (-6.0 * r6 + ef) + r_r * (p2[j] * e1 + (2.0 * p5[j]) * e2 + p5[j] * e3);
            break;
         default:
            return PORT_E_PTYPE;
         }
      }
   } else {
      for (j = j0; j < j1; j++) {
         switch (ptype) {
         case 0:
            rs_r = 1.0 / r2[j];
            r6 = (p1[j] * p1[j]) * rs_r;
            r6 = r6 * r6 * r6;
            r12 = r6 * r6;
            ppe += p0[j] * (r12 - r6);
            force[j] = rs_r * 6.0 * p0[j] * (2 * r12 - r6);
            break;
         case 1:
            r = sqrt(r2[j]);
            r_r = 1.0 / r;
            e1 = p1[j] * exp(-p2[j] * r);
            rs_r = r_r * r_r;
            r6 = p0[j] * rs_r * rs_r * rs_r;
            ppe += -r6 + e1;
            force[j] = -rs_r * 6.0 * r6 + p2[j] * e1 * r_r;
            break;
         case 2:
            r = sqrt(r2[j]);
            r_r = 1.0 / r;
            e1 = p0[j] * exp(-p1[j] * r);
            e2 = -p2[j] * exp(-p3[j] * r);
            ppe += e1 + e2;
            force[j] = (p1[j] * e1 + p3[j] * e2) * r_r;
            break;
         case 3:
            r = sqrt(r2[j]);
            r_r = 1.0 / r;
            e1 = p0[j] * exp(-p1[j] * r);
            rs_r = r_r * r_r;
            r4 = rs_r * rs_r;
            r6 = rs_r * r4;
            r8 = p5[j] * (r4 * r4);
            r12 = p2[j] * (r6 * r6);
            r4 *= p3[j];
            r6 *= p4[j];
            ppe += e1 + r12 - r4 - r6 - r8;
            force[j] = rs_r * (12.0 * r12 - 4.0 * r4 - 6.0 * r6 - 8.0 * r8) + p1[j] * e1 * r_r;
            break;
         case 4:
            r = sqrt(r2[j]);
            r_r = 1.0 / r;
            rs_r = r_r * r_r;
            r4 = rs_r * rs_r;
            r6 = rs_r * r4;
            r12 = (r6 * r6) * p2[j];
            r6 *= p1[j];
            r4 *= p0[j];
            ppe += r4 + r6 + r12;
            force[j] = rs_r * (4.0 * r4 + 6.0 * r6 + 12.0 * r12);
            break;
         case 6:
            r = sqrt(r2[j]);
            r_r = 1.0 / r;
            rs_r = r_r * r_r;
            e1 = p0[j] * exp((p1[j] - r) * p2[j]);
            r6 = p3[j] * (rs_r * rs_r * rs_r);
            e2 = p4[j] * exp(-2.0 * p5[j] * (r - p6[j]));
            e3 = -p4[j] * 2.0 * exp(-p5[j] * (r - p6[j]));
            ppe += e1 - r6 + e2 + e3;
            force[j] = rs_r * (-6.0 * r6) + r_r * (p2[j] * e1 + (2.0 * p5[j]) * e2 + p5[j] * e3);
            break;
         default:
            return PORT_E_PTYPE;
         }
      }
   }
   *pe += ppe;
   return PORT_OK;
}

double port_poteval(const double *potpar, double r, int ptype, double chgsq, double alpha)
{
   /* poteval (src/force.c:632-650): one pair at distance r, reference charge 1 */
   double pe = 0.0, f, rr = r * r, q = chgsq, norm = 2.0 * alpha / sqrt(PI_);
   double pv[NPOTP_], *pp[NPOTP_];
   int i;
   for (i = 0; i < NPOTP_; i++) {
      pv[i] = potpar[i];
      pp[i] = &pv[i];
   }
   pair_kernel(0, 1, &f, &pe, &rr, &q, 1.0, norm, alpha, ptype, pp);
   return pe;
}

/* ---- shared set-up of one real-space call ------------------------------ */
typedef struct {
   const port_system *sys;
   const double *x, *y, *z;
   double *chg;              /* per-site charges                     */
   int *id, *molmap;
   int nx, ny, nz, ncells, n_nabors;
   off3 *nabor;
   int *ent_site, *ent_num;  /* cell entries (sites, or molecules)   */
   int *ent_fw;              /* entry belongs to the framework       */
   int n_frame_types;        /* 1, or 2 with a framework (force.c:445-458) */
   int *cell_start, *cell_ent;/* entries of each cell, LIFO order     */
   double reloc[NIMG][3];
   int64_t nab_cap;
   double norm;
   int nthreads;
   int32_t *pairs;
   int64_t pairs_cap;
} rs_shared;

typedef struct {
   rs_shared *sh;
   int tid;
   double *f;                /* [3][N] private forces                */
   double pe;
   double gforce[NIMG][3];
   int64_t npairs, ntoo_close, nab_max;
   int err;
} rs_thread;

static void *force_inner(void *arg)
{
   rs_thread *T = (rs_thread *)arg;
   rs_shared *S = T->sh;
   const port_system *sys = S->sys;
   int N = sys->nsites, nx = S->nx, ny = S->ny, nz = S->nz, max_id = sys->max_id;
   int64_t cap = S->nab_cap > 0 ? S->nab_cap : 1;
   int *nab = (int *)malloc(sizeof(int) * cap), *tr = (int *)malloc(sizeof(int) * cap);
   double *bx = (double *)malloc(sizeof(double) * cap * 16);
   double *by = bx + cap, *bz = by + cap, *bq = bz + cap, *fjx = bq + cap, *fjy = fjx + cap,
          *fjz = fjy + cap, *rx = fjz + cap, *ry = rx + cap, *rz = ry + cap, *r2 = rz + cap,
          *fij = r2 + cap;
   double *pbuf = (double *)malloc(sizeof(double) * cap * NPOTP_), *pv[NPOTP_];
   double cut2 = sys->cutoff * sys->cutoff, cut100 = 10000.0 * cut2;
   double *fx = T->f, *fy = T->f + N, *fz = T->f + 2 * N;
   int icell, k, j;
   for (k = 0; k < NPOTP_; k++) pv[k] = pbuf + (size_t)k * cap;
   memset(T->gforce, 0, sizeof T->gforce);
   for (icell = T->tid; icell < S->ncells; icell += S->nthreads) {   /* force.c:856 */
      int ix = icell / (ny * nz), iy = icell / nz - ny * ix, iz = icell - nz * (iy + ny * ix);
      int64_t nnab = 0;
      int jnab, e, jmin, jmax, ft, nfnab0 = 0;
      if (S->cell_start[icell] == S->cell_start[icell + 1]) continue;
      /* site neighbour list (src/force.c:521-569): non-framework sites of
       * every stencil cell, then framework sites of every stencil cell but
       * the cell's own */
      for (ft = 0; ft < S->n_frame_types; ft++) {
         for (jnab = ft == 0 ? 0 : 1; jnab < S->n_nabors; jnab++) {
            int ex = ix + S->nabor[jnab].d[0] + nx, ey = iy + S->nabor[jnab].d[1] + ny,
                ez = iz + S->nabor[jnab].d[2] + nz;
            int ii = ex / nx, jj = ey / ny, kk = ez / nz;
            int jc = (ez - kk * nz) + nz * ((ey - jj * ny) + ny * (ex - ii * nx));
            int ktrans = 9 * ii + 3 * jj + kk;
            for (e = S->cell_start[jc]; e < S->cell_start[jc + 1]; e++) {
               int ent = S->cell_ent[e], s;
               if (S->ent_fw[ent] != ft) continue;
               for (s = 0; s < S->ent_num[ent]; s++) {
                  if (nnab >= cap) { T->err = PORT_E_TONAB; goto done; }
                  nab[nnab] = S->ent_site[ent] + s;
                  tr[nnab] = ktrans;
                  nnab++;
               }
            }
         }
         if (ft == 0) nfnab0 = (int)nnab;
      }
      if (nnab > T->nab_max) T->nab_max = nnab;
      for (j = 0; j < nnab; j++) {                  /* gathers, force.c:877-884 */
         bx[j] = S->x[nab[j]];
         by[j] = S->y[nab[j]];
         bz[j] = S->z[nab[j]];
         bq[j] = S->chg[nab[j]];
         fjx[j] = fjy[j] = fjz[j] = 0.0;
      }
      jmin = 0;
      jmax = (int)nnab;
      for (e = S->cell_start[icell]; e < S->cell_start[icell + 1]; e++) {
         int ent = S->cell_ent[e], isite;
         if (S->ent_fw[ent]) {                       /* force.c:904-908 */
            jmin = 0;
            jmax = nfnab0;
         } else {
            jmax = (int)nnab;
         }
         for (isite = S->ent_site[ent]; isite < S->ent_site[ent] + S->ent_num[ent]; isite++) {
            double xi = S->x[isite], yi = S->y[isite], zi = S->z[isite];
            double si0 = 0.0, si1 = 0.0, si2 = 0.0;
            const double *prow = sys->potpar + (size_t)S->id[isite] * max_id * NPOTP_;
            if (!S->ent_fw[ent]) jmin++;             /* force.c:916-917 */
            for (j = jmin; j < jmax; j++) {
               const double *pp = prow + (size_t)S->id[nab[j]] * NPOTP_;
               for (k = 0; k < NPOTP_; k++) pv[k][j] = pp[k];
            }
            for (j = jmin; j < jmax; j++) {          /* mk_r_sqr, force.c:692-711 */
               const double *rl = S->reloc[tr[j]];
               double a = bx[j] - xi + rl[0], b = by[j] - yi + rl[1], c = bz[j] - zi + rl[2];
               r2[j] = a * a + b * b + c * c;
               rx[j] = a; ry[j] = b; rz[j] = c;
            }
            for (j = jmin; j < jmax; j++)            /* TOO_CLOSE, force.c:939-949 */
               if (r2[j] < TOO_CLOSE_ && S->molmap[isite] != S->molmap[nab[j]])
                  T->ntoo_close++;
            if (sys->strict_cutoff && !sys->molpbc)  /* force.c:951-954 */
               for (j = jmin; j < jmax; j++)
                  if (r2[j] > cut2) r2[j] = cut100;
            T->err = pair_kernel(jmin, jmax, fij, &T->pe, r2, bq, S->chg[isite], S->norm,
                                 sys->alpha, sys->ptype, pv);
            if (T->err) goto done;
            for (j = jmin; j < jmax; j++) {          /* mk_forces, force.c:717-743 */
               double cx = fij[j] * rx[j], cy = fij[j] * ry[j], cz = fij[j] * rz[j];
               si0 -= cx; si1 -= cy; si2 -= cz;
               fjx[j] += cx; fjy[j] += cy; fjz[j] += cz;
            }
            fx[isite] += si0; fy[isite] += si1; fz[isite] += si2;
            if (S->pairs) {                          /* single-threaded only */
               if (T->npairs + (jmax - jmin) > S->pairs_cap) { T->err = PORT_E_PAIRCAP; goto done; }
               for (j = jmin; j < jmax; j++) {
                  int32_t *q = S->pairs + 3 * (T->npairs + (j - jmin));
                  q[0] = isite; q[1] = nab[j]; q[2] = tr[j];
               }
            }
            T->npairs += jmax - jmin;
         }
      }
      for (j = 0; j < nnab; j++) {                  /* scatter_forces, force.c:750-778 */
         double *g = T->gforce[tr[j]];
         fx[nab[j]] += fjx[j]; fy[nab[j]] += fjy[j]; fz[nab[j]] += fjz[j];
         g[0] += fjx[j]; g[1] += fjy[j]; g[2] += fjz[j];
      }
   }
done:
   free(nab); free(tr); free(bx); free(pbuf);
   return NULL;
}

/* Intramolecular energy of one molecule (pe_intra, src/force.c:654-668). */
static double mol_intra(const port_system *sys, const int *ids, const double *pf, int ns)
{
   double e = 0.0;
   int a, b;
   for (a = 0; a < ns; a++)
      for (b = a + 1; b < ns; b++) {
         const double *u = pf + 3 * b, *v = pf + 3 * a;
         double r = sqrt((u[0] - v[0]) * (u[0] - v[0]) + (u[1] - v[1]) * (u[1] - v[1]) +
                         (u[2] - v[2]) * (u[2] - v[2]));
         e += port_poteval(sys->potpar + ((size_t)ids[a] * sys->max_id + ids[b]) * NPOTP_, r,
                           sys->ptype, sys->site_charge[ids[b]] * sys->site_charge[ids[a]],
                           sys->alpha);
      }
   return e;
}

int port_force_calc(const port_system *sys, const double *site, double *site_force,
                    double *pe, double *stress, int nthreads, int32_t *pairs,
                    int64_t pairs_cap, port_info *info)
{
   rs_shared S;
   rs_thread *T;
   pthread_t *th;
   int N = sys->nsites, i, s, m, t, err = 0, bad = 0;
   double subcell = sys->subcell, hm[3][3], hinv[3][3], eps = 8.0 * 2.220446049250313e-16;
   double eintra = 0.0, vol, md, s00 = 0, s01 = 0, s02 = 0, s11 = 0, s12 = 0, s22 = 0;
   int nent = 0, *cnt, nsmax = 0, so = 0, isite = 0, imol = 0;
   const double *x = site, *y = site + N, *z = site + 2 * N;
   port_info dummy;
   if (!info) info = &dummy;
   memset(info, 0, sizeof *info);
   if (!sys || N <= 0 || nthreads < 1 || (pairs && nthreads != 1)) return PORT_E_ARG;
   if (sys->ptype < 0 || sys->ptype > 6 || sys->ptype == 5) return PORT_E_PTYPE;
   memset(&S, 0, sizeof S);
   S.sys = sys; S.x = x; S.y = y; S.z = z; S.nthreads = nthreads;
   S.pairs = pairs; S.pairs_cap = pairs_cap;
   S.norm = 2.0 * sys->alpha / sqrt(PI_);
   /* subcell partition, force.c:1150-1155 */
   if (subcell <= 0.0) subcell = sys->cutoff / 5.0;
   S.nx = (int)(sys->h[0][0] / subcell + 0.5);
   S.ny = (int)(sys->h[1][1] / subcell + 0.5);
   S.nz = (int)(sys->h[2][2] / subcell + 0.5);
   if (S.nx < 1 || S.ny < 1 || S.nz < 1) return PORT_E_ARG;
   S.ncells = S.nx * S.ny * S.nz;
   info->nx = S.nx; info->ny = S.ny; info->nz = S.nz;
   /* intramolecular correction, force.c:1156-1171 */
   for (s = 0; s < sys->nspecies; s++) {
      if (!sys->spec_framework[s])   /* force.c:1159-1163 */
         eintra += sys->spec_nmols[s] * mol_intra(sys, sys->spec_site_id + so, sys->spec_pf + 3 * so,
                                               sys->spec_nsites[s]);
      so += sys->spec_nsites[s];
   }
   info->eintra = eintra;
   *pe -= eintra;
   /* per-site ids, charges, molecule map (force.c:1175-1190, accel.c:480-484) */
   S.id = (int *)malloc(sizeof(int) * N);
   S.molmap = (int *)malloc(sizeof(int) * N);
   S.chg = (double *)malloc(sizeof(double) * N);
   so = 0;
   for (s = 0; s < sys->nspecies; s++) {
      for (m = 0; m < sys->spec_nmols[s]; m++, imol++)
         for (i = 0; i < sys->spec_nsites[s]; i++, isite++) {
            S.id[isite] = sys->spec_site_id[so + i];
            S.chg[isite] = sys->site_charge[S.id[isite]];
            S.molmap[isite] = imol;
         }
      so += sys->spec_nsites[s];
   }
   /* fill_cells (force.c:426-486): entries are sites, or whole molecules
    * binned by centre of mass in molecular-cutoff mode */
   memcpy(hm, sys->h, sizeof hm);
   inv3(hm, hinv);
   S.ent_site = (int *)malloc(sizeof(int) * N);
   S.ent_num = (int *)malloc(sizeof(int) * N);
   S.ent_fw = (int *)malloc(sizeof(int) * N);
   S.n_frame_types = 1;
   {
      int *ent_cell = (int *)malloc(sizeof(int) * N);
      double fnx = S.nx, fny = S.ny, fnz = S.nz;
      isite = 0; imol = 0;
      for (s = 0; s < sys->nspecies; s++)
         for (m = 0; m < sys->spec_nmols[s]; m++, imol++) {
            if (sys->spec_framework[s]) S.n_frame_types = 2;
            if (!sys->molpbc || sys->spec_framework[s]) {
               for (i = 0; i < sys->spec_nsites[s]; i++, isite++) {
                  double a0 = x[isite], a1 = y[isite], a2 = z[isite], s0, s1, s2;
                  s0 = hinv[0][0] * a0 + hinv[0][1] * a1 + hinv[0][2] * a2;
                  s1 = hinv[1][0] * a0 + hinv[1][1] * a1 + hinv[1][2] * a2;
                  s2 = hinv[2][0] * a0 + hinv[2][1] * a1 + hinv[2][2] * a2;
                  ent_cell[nent] = bin1(s2, S.nz, fnz, eps, &bad) +
                                   S.nz * (bin1(s1, S.ny, fny, eps, &bad) +
                                           S.ny * bin1(s0, S.nx, fnx, eps, &bad));
                  S.ent_site[nent] = isite;
                  S.ent_num[nent] = 1;
                  S.ent_fw[nent] = sys->spec_framework[s] ? 1 : 0;
                  nent++;
               }
            } else {
               const double *c = sys->c_of_m + 3 * imol;
               ent_cell[nent] = bin1(c[2], S.nz, fnz, eps, &bad) +
                                S.nz * (bin1(c[1], S.ny, fny, eps, &bad) +
                                        S.ny * bin1(c[0], S.nx, fnx, eps, &bad));
               S.ent_site[nent] = isite;
               S.ent_num[nent] = sys->spec_nsites[s];
               S.ent_fw[nent] = 0;
               nent++;
               isite += sys->spec_nsites[s];
            }
         }
      /* counting sort of entries by cell; each cell read back newest-first,
       * the order of the reference's LIFO linked lists */
      cnt = (int *)calloc(S.ncells + 1, sizeof(int));
      S.cell_start = (int *)malloc(sizeof(int) * (S.ncells + 1));
      S.cell_ent = (int *)malloc(sizeof(int) * (nent > 0 ? nent : 1));
      for (i = 0; i < nent; i++) cnt[ent_cell[i]] += S.ent_num[i] ? 1 : 0;
      S.cell_start[0] = 0;
      for (i = 0; i < S.ncells; i++) S.cell_start[i + 1] = S.cell_start[i] + cnt[i];
      for (i = 0; i < S.ncells; i++) cnt[i] = S.cell_start[i + 1];
      for (i = 0; i < nent; i++) S.cell_ent[--cnt[ent_cell[i]]] = i;
      /* max_density (force.c:491-507) */
      for (i = 0; i < S.ncells; i++) {
         int e, ns = 0;
         for (e = S.cell_start[i]; e < S.cell_start[i + 1]; e++) ns += S.ent_num[S.cell_ent[e]];
         if (ns > nsmax) nsmax = ns;
      }
      free(cnt);
      free(ent_cell);
   }
   if (bad) { err = PORT_E_RANGE; goto out; }
   vol = det3(hm);
   md = nsmax * S.ncells / vol;
   /* neighbour cells (force.c:1222-1227) */
   S.n_nabors = build_stencil(hm, sys->cutoff, S.nx, S.ny, S.nz, sys->strict_cutoff, &S.nabor);
   if (S.n_nabors < 0) { err = S.n_nabors; S.nabor = NULL; goto out; }
   info->n_nabors = S.n_nabors;
   /* site-list capacity (force.c:1231-1235) */
   if (sys->strict_cutoff)
      S.nab_cap = (int)(NMULT_ * 4.19 * ((sys->cutoff + subcell) * (sys->cutoff + subcell) *
                                         (sys->cutoff + subcell)) * md);
   else
      S.nab_cap = (int)(NMULT_ * 4.19 * (sys->cutoff * sys->cutoff * sys->cutoff) * md);
   info->n_nab_cap = S.nab_cap;
   /* image translation table (force.c:1282-1293) */
   t = 0;
   {
      int ii, jj, kk;
      for (ii = -XTRA; ii <= XTRA; ii++)
         for (jj = -XTRA; jj <= XTRA; jj++)
            for (kk = -XTRA; kk <= XTRA; kk++, t++) {
               S.reloc[t][0] = sys->h[0][0] * ii + sys->h[0][1] * jj + sys->h[0][2] * kk;
               S.reloc[t][1] = sys->h[1][0] * ii + sys->h[1][1] * jj + sys->h[1][2] * kk;
               S.reloc[t][2] = sys->h[2][0] * ii + sys->h[2][1] * jj + sys->h[2][2] * kk;
            }
   }
   T = (rs_thread *)calloc(nthreads, sizeof(rs_thread));
   th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
   for (t = 0; t < nthreads; t++) {
      T[t].sh = &S;
      T[t].tid = t;
      T[t].f = (double *)calloc(3 * (size_t)N, sizeof(double));
   }
   if (nthreads == 1) {
      T[0].pe = *pe;                 /* same summation order as the reference */
      *pe = 0.0;
      force_inner(&T[0]);
   } else {
      for (t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, force_inner, &T[t]);
      for (t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
   }
   for (t = 0; t < nthreads; t++) {
      if (T[t].err && !err) err = T[t].err;
      info->npairs += T[t].npairs;
      info->n_too_close += T[t].ntoo_close;
      if (T[t].nab_max > info->n_nab_max) info->n_nab_max = T[t].nab_max;
   }
   if (!err) {
      /* virial from the accumulated site forces plus the image forces,
       * force.c:973-1000; site_force already holding values contributes too */
      double *fx = site_force, *fy = site_force + N, *fz = site_force + 2 * N;
      for (t = 0; t < nthreads; t++) {
         double *f = T[t].f;
         for (i = 0; i < N; i++) {
            fx[i] += f[i];
            fy[i] += f[N + i];
            fz[i] += f[2 * N + i];
         }
         *pe += T[t].pe;
      }
      for (i = 0; i < N; i++) {
         s00 += x[i] * fx[i];
         s01 += y[i] * fx[i];
         s02 += z[i] * fx[i];
         s11 += y[i] * fy[i];
         s12 += z[i] * fy[i];
         s22 += z[i] * fz[i];
      }
      for (t = 0; t < nthreads; t++) {
         int k;
         for (k = 0; k < NIMG; k++) {
            s00 += S.reloc[k][0] * T[t].gforce[k][0];
            s01 += S.reloc[k][1] * T[t].gforce[k][0];
            s02 += S.reloc[k][2] * T[t].gforce[k][0];
            s11 += S.reloc[k][1] * T[t].gforce[k][1];
            s12 += S.reloc[k][2] * T[t].gforce[k][1];
            s22 += S.reloc[k][2] * T[t].gforce[k][2];
         }
      }
      stress[0] += s00; stress[1] += s01; stress[2] += s02;
      stress[4] += s11; stress[5] += s12; stress[8] += s22;
   }
   for (t = 0; t < nthreads; t++) free(T[t].f);
   free(T);
   free(th);
out:
   free(S.id); free(S.molmap); free(S.chg); free(S.ent_site); free(S.ent_num); free(S.ent_fw);
   free(S.cell_start); free(S.cell_ent); free(S.nabor);
   return err;
}

/* ---- reciprocal space (src/ewald.c) ------------------------------------ */
/* 4 interleaved accumulators with a one-element delay: the summation order
 * of sum() (src/auxil.c:222-256). */
static double sum4(int n, const double *x)
{
   double sa = 0, sb = 0, sc = 0, sd = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0;
   int i;
   for (i = 0; i < n - 3; i += 4) {
      s1 += sa; sa = x[i];
      s2 += sb; sb = x[i + 1];
      s3 += sc; sc = x[i + 2];
      s4 += sd; sd = x[i + 3];
   }
   s1 += sa; s2 += sb; s3 += sc; s4 += sd;
   for (; i < n; i++) s1 += x[i];
   return s1 + s2 + s3 + s4;
}

/* erf by Abramowitz & Stegun 7.1.26 (src/auxil.c:586-593). */
static double as_erf(double x)
{
   double t = 1.0 / (1.0 + ASP * x);
   if (x >= 0.0) return 1.0 - ASPOLY(t) * exp(-x * x);
   return -as_erf(-x);
}

typedef struct { double kx, ky, kz; int h, k, l; } kvec;

typedef struct {
   const port_system *sys;
   int N, nxf, hmax, kmax, lmax;
   double **chx, **shx, **cky, **sky, **clz, **slz;  /* [h][site] */
   kvec *kl;
   int64_t k0, k1;
   double vol, r4a;
   int nthreads;
} ew_shared;

typedef struct {
   ew_shared *sh;
   int tid;
   double *f;              /* private forces [3][N] */
   double pe, st[6];
   double *pe_direct;      /* single-thread: accumulate straight into *pe */
   double *stress_direct;
   double *f_direct;
} ew_thread;

/* cos/sin(h a*.r) tables by the addition formula, seeded with libm at h=1
 * (trig_recur, src/ewald.c:148-193). */
static void trig_table(double **c, double **s, const double *ks, const double *x,
                       const double *y, const double *z, int hmax, int n0, int n1)
{
   int h, i;
   for (i = n0; i < n1; i++) { c[0][i] = 1.0; s[0][i] = 0.0; }
   if (hmax < 1) return;
   for (i = n0; i < n1; i++) {
      double kr = ks[0] * x[i] + ks[1] * y[i] + ks[2] * z[i];
      c[1][i] = cos(kr);
      s[1][i] = sin(kr);
   }
   for (h = 2; h <= hmax; h++)
      for (i = n0; i < n1; i++) {
         double cc = c[h - 1][i] * c[1][i] - s[h - 1][i] * s[1][i];
         s[h][i] = s[h - 1][i] * c[1][i] + c[h - 1][i] * s[1][i];
         c[h][i] = cc;
      }
}

static void *ewald_block(void *arg)
{
   ew_thread *T = (ew_thread *)arg;
   ew_shared *S = T->sh;
   int N = S->N, nxf = S->nxf, is;
   int64_t nk = S->k1 - S->k0, per = (nk + S->nthreads - 1) / S->nthreads;
   int64_t b = S->k0 + T->tid * per, e = b + per, p;
   double *qc = (double *)malloc(sizeof(double) * N * 4), *qs = qc + N, *cxy = qs + N,
          *sxy = cxy + N;
   double *fx, *fy, *fz, *pe, *st;
   double st_local[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
   int hl = -1000000, kl = -1000000;
   if (e > S->k1) e = S->k1;
   if (T->f_direct) { fx = T->f_direct; } else { fx = T->f; }
   fy = fx + N; fz = fy + N;
   pe = T->pe_direct ? T->pe_direct : &T->pe;
   st = T->stress_direct ? T->stress_direct : st_local;   /* row-major 3x3 */
   for (p = b; p < e; p++) {                          /* ewald.c:497-580 */
      const kvec *kv = S->kl + p;
      int h = kv->h, k = kv->k, l = kv->l;
      double kx = kv->kx, ky = kv->ky, kz = kv->kz;
      double ksq = kx * kx + ky * ky + kz * kz;
      double coeff = 2.0 / ((0.25 / PI_) * S->vol) * exp(ksq * S->r4a) / ksq;
      double coeff2 = 2.0 * (1.0 - ksq * S->r4a) / ksq;
      const double *chx = S->chx[h], *shx = S->shx[h], *cky = S->cky[abs(k)],
                   *sky = S->sky[abs(k)], *clz = S->clz[abs(l)], *slz = S->slz[abs(l)];
      double cn, sn, cf, sf, ck, sk, pek;
      if (h != hl || k != kl) {                      /* qsincos, ewald.c:95-142 */
         if (k >= 0)
            for (is = 0; is < N; is++) {
               double c = chx[is] * cky[is] - shx[is] * sky[is];
               sxy[is] = shx[is] * cky[is] + chx[is] * sky[is];
               cxy[is] = c;
            }
         else
            for (is = 0; is < N; is++) {
               double c = chx[is] * cky[is] + shx[is] * sky[is];
               sxy[is] = shx[is] * cky[is] - chx[is] * sky[is];
               cxy[is] = c;
            }
      }
      hl = h; kl = k;
      if (l >= 0)
         for (is = 0; is < N; is++) {
            double c = cxy[is] * clz[is] - sxy[is] * slz[is];
            qs[is] = sxy[is] * clz[is] + cxy[is] * slz[is];
            qc[is] = c;
         }
      else
         for (is = 0; is < N; is++) {
            double c = cxy[is] * clz[is] + sxy[is] * slz[is];
            qs[is] = sxy[is] * clz[is] - cxy[is] * slz[is];
            qc[is] = c;
         }
      cn = sum4(nxf, qc);
      sn = sum4(nxf, qs);
      cf = sum4(N - nxf, qc + nxf);
      sf = sum4(N - nxf, qs + nxf);
      ck = cn + cf;
      sk = sn + sf;
      pek = 0.5 * coeff * (cn * (cn + cf + cf) + sn * (sn + sf + sf));
      *pe += pek;
      sk *= coeff; ck *= coeff; sn *= coeff; cn *= coeff;
      st[0] += pek - pek * coeff2 * kx * kx;
      st[1] -= pek * coeff2 * kx * ky;
      st[2] -= pek * coeff2 * kx * kz;
      st[4] += pek - pek * coeff2 * ky * ky;
      st[5] -= pek * coeff2 * ky * kz;
      st[8] += pek - pek * coeff2 * kz * kz;
      for (is = 0; is < nxf; is++) {
         double fc = qs[is] * ck - qc[is] * sk;
         double a = fx[is] + kx * fc, bb = fy[is] + ky * fc;
         fz[is] += kz * fc;
         fx[is] = a;
         fy[is] = bb;
      }
      for (is = nxf; is < N; is++) {
         double fc = qs[is] * cn - qc[is] * sn;
         double a = fx[is] + kx * fc, bb = fy[is] + ky * fc;
         fz[is] += kz * fc;
         fx[is] = a;
         fy[is] = bb;
      }
   }
   if (!T->stress_direct) {
      T->st[0] = st[0]; T->st[1] = st[1]; T->st[2] = st[2];
      T->st[3] = st[4]; T->st[4] = st[5]; T->st[5] = st[8];
   }
   free(qc);
   return NULL;
}

int port_ewald(const port_system *sys, const double *site, double *site_force, double *pe,
               double *stress, int nthreads, int64_t k_first, int64_t k_last, port_info *info)
{
   ew_shared S;
   int N = sys->nsites, s, i, t, h, k, l, nk = 0, so = 0, ssite = 0, frame_flag;
   double hm[3][3], hinvp[3][3], alpha = sys->alpha, kcsq = sys->k_cutoff * sys->k_cutoff;
   double self = 0.0, sheet = 0.0, sq = 0.0, sqsq = 0.0, sqxf;
   double *q, *tables;
   const double *x = site, *y = site + N, *z = site + 2 * N;
   port_info dummy;
   if (!info) info = &dummy;
   if (!sys || N <= 0 || nthreads < 1) return PORT_E_ARG;
   if (alpha <= ALPHAMIN_) return PORT_OK;
   info->t_setup = wall();
   memset(&S, 0, sizeof S);
   S.sys = sys; S.N = N; S.nthreads = nthreads;
   memcpy(hm, sys->h, sizeof hm);
   S.vol = det3(hm);
   S.r4a = -1.0 / (4.0 * alpha * alpha);
   /* k-space extent (ewald.c:306-308); ewald.c's moda/modb/modc are h00,
    * |column 1| and |column 2| of h (ewald.c:70-72) */
   S.hmax = (int)floor(sys->k_cutoff / (2 * PI_) * sys->h[0][0]);
   S.kmax = (int)floor(sys->k_cutoff / (2 * PI_) *
                       sqrt(sys->h[0][1] * sys->h[0][1] + sys->h[1][1] * sys->h[1][1]));
   S.lmax = (int)floor(sys->k_cutoff / (2 * PI_) *
                       sqrt(sys->h[0][2] * sys->h[0][2] + sys->h[1][2] * sys->h[1][2] +
                            sys->h[2][2] * sys->h[2][2]));
   info->hmax = S.hmax; info->kmax = S.kmax; info->lmax = S.lmax;
   q = (double *)malloc(sizeof(double) * N);
   {
      int isite = 0, m;
      for (s = 0; s < sys->nspecies; s++) {
         for (m = 0; m < sys->spec_nmols[s]; m++)
            for (i = 0; i < sys->spec_nsites[s]; i++)
               q[isite++] = sys->site_charge[sys->spec_site_id[so + i]];
         so += sys->spec_nsites[s];
      }
   }
   /* self and sheet energies (ewald.c:367-425) */
   so = 0;
   for (s = 0; s < sys->nspecies && !sys->spec_framework[s]; s++) {
      double intra = 0.0;
      int a, b, ns = sys->spec_nsites[s];
      const double *pf = sys->spec_pf + 3 * so;
      for (a = 0; a < ns; a++)
         for (b = a + 1; b < ns; b++) {
            const double *u = pf + 3 * a, *v = pf + 3 * b;
            double r = sqrt((u[0] - v[0]) * (u[0] - v[0]) + (u[1] - v[1]) * (u[1] - v[1]) +
                            (u[2] - v[2]) * (u[2] - v[2]));
            intra += q[ssite + a] * q[ssite + b] * as_erf(alpha * r) / r;
         }
      self += sys->spec_nmols[s] * intra;
      ssite += ns * sys->spec_nmols[s];
      so += ns;
   }
   S.nxf = ssite;
   frame_flag = s != sys->nspecies;
   for (i = 0; i < S.nxf; i++) {
      sq += q[i];
      sqsq += q[i] * q[i];
   }
   self += alpha / sqrt(PI_) * sqsq;
   sqxf = sq;
   for (; i < N; i++) sq += q[i];
   if (frame_flag) sheet = PI_ * (sq - sqxf) * (sq - sqxf) / (2.0 * (alpha * alpha));
   if (fabs(sq) * CONVQ_ > 1.0e-5) sheet -= PI_ * (sq * sq) / (2.0 * (alpha * alpha));
   info->self_energy = self;
   info->sheet_energy = sheet;
   *pe -= self;
   *pe += sheet / S.vol;
   for (i = 0; i < 3; i++) stress[4 * i] += sheet / S.vol;
   /* reciprocal lattice and the half-sphere k list (ewald.c:435-461) */
   inv3(hm, hinvp);
   for (i = 0; i < 9; i++) hinvp[i / 3][i % 3] = 2 * PI_ * hinvp[i / 3][i % 3];
   S.kl = (kvec *)malloc(sizeof(kvec) * 4 * (size_t)(S.hmax + 1) * (S.kmax + 1) * (S.lmax + 1));
   for (h = 0; h <= S.hmax; h++)
      for (k = (h == 0 ? 0 : -S.kmax); k <= S.kmax; k++) {
         double kx = h * hinvp[0][0] + k * hinvp[1][0];
         double ky = h * hinvp[0][1] + k * hinvp[1][1];
         double kzt = h * hinvp[0][2] + k * hinvp[1][2];
         double ksq = kx * kx + ky * ky;
         for (l = (h == 0 && k == 0 ? 1 : -S.lmax); l <= S.lmax; l++) {
            double kz = kzt + l * hinvp[2][2];
            if (kz * kz + ksq < kcsq) {
               S.kl[nk].h = h; S.kl[nk].k = k; S.kl[nk].l = l;
               S.kl[nk].kx = kx; S.kl[nk].ky = ky; S.kl[nk].kz = kz;
               nk++;
            }
         }
      }
   info->nkvec = nk;
   S.k0 = k_first < 0 ? 0 : (k_first > nk ? nk : k_first);
   S.k1 = (k_last < 0 || k_last > nk) ? nk : k_last;
   if (S.k1 < S.k0) S.k1 = S.k0;
   /* trig tables, q folded into the l tables (ewald.c:469-481) */
   {
      int nt = S.hmax + S.kmax + S.lmax + 3, j = 0;
      tables = (double *)malloc(sizeof(double) * 2 * (size_t)nt * N);
      S.chx = (double **)malloc(sizeof(double *) * 2 * nt);
      S.shx = S.chx + (S.hmax + 1);
      S.cky = S.shx + (S.hmax + 1);
      S.sky = S.cky + (S.kmax + 1);
      S.clz = S.sky + (S.kmax + 1);
      S.slz = S.clz + (S.lmax + 1);
      for (i = 0; i < 2 * nt; i++) S.chx[i] = tables + (size_t)i * N;
      (void)j;
      trig_table(S.chx, S.shx, hinvp[0], x, y, z, S.hmax, 0, N);
      trig_table(S.cky, S.sky, hinvp[1], x, y, z, S.kmax, 0, N);
      trig_table(S.clz, S.slz, hinvp[2], x, y, z, S.lmax, 0, N);
      for (l = 0; l <= S.lmax; l++)
         for (i = 0; i < N; i++) {
            S.clz[l][i] *= q[i];
            S.slz[l][i] *= q[i];
         }
   }
   info->t_setup = wall() - info->t_setup;
   {
      ew_thread *T = (ew_thread *)calloc(nthreads, sizeof(ew_thread));
      pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
      double t0 = wall();
      if (nthreads == 1) {
         T[0].sh = &S;
         T[0].f_direct = site_force;
         T[0].pe_direct = pe;
         T[0].stress_direct = stress;
         ewald_block(&T[0]);
      } else {
         for (t = 0; t < nthreads; t++) {
            T[t].sh = &S;
            T[t].tid = t;
            T[t].f = (double *)calloc(3 * (size_t)N, sizeof(double));
            pthread_create(&th[t], NULL, ewald_block, &T[t]);
         }
         for (t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
         for (t = 0; t < nthreads; t++) {
            for (i = 0; i < 3 * N; i++) site_force[i] += T[t].f[i];
            *pe += T[t].pe;
            stress[0] += T[t].st[0]; stress[1] += T[t].st[1]; stress[2] += T[t].st[2];
            stress[4] += T[t].st[3]; stress[5] += T[t].st[4]; stress[8] += T[t].st[5];
            free(T[t].f);
         }
      }
      info->t_kloop = wall() - t0;
      free(T);
      free(th);
   }
   free(tables);
   free(S.chx);
   free(S.kl);
   free(q);
   return PORT_OK;
}
