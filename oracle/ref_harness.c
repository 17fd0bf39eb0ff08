/*
 * ref_harness.c -- TEST INFRASTRUCTURE ONLY.  Drives the reference's own
 * force_calc() (src/force.c:1108) and ewald() (src/ewald.c:280), compiled
 * unmodified from the reference sources into oracle/_ref/libmoldyref.so by
 * oracle/build_ref.sh, on one configuration read from an MDSYS1 file
 * (moldy_gb300/system.py:write_mdsys), and writes the site forces, energies
 * and stress of each call to an output file.
 *
 * Pair-set capture: the reference library is built with -fPIC, so its calls
 * to site_neighbour_list() (src/force.c:521) and kernel() (src/kernel.c:157)
 * go through the PLT and are interposed by the definitions below, which call
 * the originals via dlsym(RTLD_NEXT) and record, for every kernel() call
 * made from force_inner (src/force.c:960), the pairs
 * (isite = nab[jmin-1], nab[j], pbctrans[j]) for j in [jmin, jmax)
 * (the cell's own sites come first in nab and jmin advances once per site,
 * src/force.c:889-917).  A framework site is called with jmin = 0 against
 * the non-framework sites [0, nfnab[0]) (src/force.c:904-908); the
 * framework entries head each cell's list (framework species come last and
 * the lists are LIFO), so they are taken in the cell's list order, read
 * from the cell list handed to site_neighbour_list.  kernel() calls made by poteval() during the
 * first-call intramolecular correction happen before any neighbour list
 * exists and are not recorded.
 *
 * Only the tests and the fixture generator run this program; it is never on
 * the product path and is not built on machines without the reference.
 *
 * With MDGPU_REF_RDF="limit nbins" in the environment the first force_calc
 * call also accumulates the reference's radial distribution histogram
 * (rdf_inner/rdf_accum, src/force.c:1010-1103, src/rdf.c:94-107, after
 * init_rdf) and the histogram (rdf_ptr's float array) is appended to the
 * output as int64 size + float[size].
 *
 * usage: moldy_ref_harness in.mdsys out.bin [repeats]
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <time.h>
#include "defs.h"
#include "structs.h"

contr_mt control;
int ithread = 0, nthreads = 1;

void force_calc(real **site, real **site_force, system_mt *system, spec_mt *species,
                real *chg, pot_mt *potpar, double *pe, mat_mt stress);
void ewald(real **site, real **site_force, system_mp system, spec_mt *species,
           real *chg, double *pe, mat_mt stress);
void init_rdf(system_mp system);
gptr *rdf_ptr(int *size);

/* ---- pair capture ------------------------------------------------------ */
/* a link-cell entry (src/force.c:42-46) */
typedef struct cell_s {
   int isite, num, frame_type;
   struct cell_s *next;
} cell_entry;
static int      fw_queue[4096], fw_head = 0, fw_n = 0;
static int      cap_on = 0;
static int     *cap_nab = NULL, *cap_trans = NULL;
static int64_t  cap_n = 0, cap_cap = 0;
static int32_t *cap_pairs = NULL;

typedef int (*snl_fn)(int *, int *, int, int *, int, int, int, int, int, int, int, int,
                      int *, void *, int (*)[2]);
int site_neighbour_list(int *nab, int *pbctrans, int n_nab_sites, int *nfnab,
                        int n_frame_types, int n_nabors, int ix, int iy, int iz,
                        int nx, int ny, int nz, int *nabor, void *cell, int (*pbclookup)[2])
{
   static snl_fn orig = NULL;
   if (!orig) orig = (snl_fn)dlsym(RTLD_NEXT, "site_neighbour_list");
   cap_nab = nab;
   cap_trans = pbctrans;
   fw_head = fw_n = 0;
   if (n_frame_types > 1) {
      const cell_entry *e = ((cell_entry **)cell)[iz + nz * (iy + ny * ix)];
      for (; e; e = e->next)
         if (e->frame_type) {
            int k;
            for (k = 0; k < e->num && fw_n < 4096; k++) fw_queue[fw_n++] = e->isite + k;
         }
   }
   return orig(nab, pbctrans, n_nab_sites, nfnab, n_frame_types, n_nabors, ix, iy, iz,
               nx, ny, nz, nabor, cell, pbclookup);
}

typedef void (*kern_fn)(int, int, real *, double *, real *, real *, double, double,
                        double, int, real **);
void kernel(int jmin, int nnab, real *forceij, double *pe, real *r_sqr, real *nab_chg,
            double chg, double norm, double alpha, int ptype, real **pot)
{
   static kern_fn orig = NULL;
   int j;
   if (!orig) orig = (kern_fn)dlsym(RTLD_NEXT, "kernel");
   if (cap_on && cap_nab && (jmin > 0 || fw_head < fw_n)) {
      int isite = jmin > 0 ? cap_nab[jmin - 1] : fw_queue[fw_head++];
      for (j = jmin; j < nnab; j++) {
         if (cap_n >= cap_cap) {
            cap_cap = cap_cap ? 2 * cap_cap : (1 << 20);
            cap_pairs = (int32_t *)realloc(cap_pairs, (size_t)cap_cap * 3 * sizeof(int32_t));
            if (!cap_pairs) { fprintf(stderr, "harness: out of memory\n"); exit(2); }
         }
         cap_pairs[3 * cap_n + 0] = isite;
         cap_pairs[3 * cap_n + 1] = cap_nab[j];
         cap_pairs[3 * cap_n + 2] = cap_trans[j];
         cap_n++;
      }
   }
   orig(jmin, nnab, forceij, pe, r_sqr, nab_chg, chg, norm, alpha, ptype, pot);
}

/* ---- input ------------------------------------------------------------- */
static void rd(void *p, size_t sz, size_t n, FILE *f)
{
   if (fread(p, sz, n, f) != n) { fprintf(stderr, "harness: short read\n"); exit(2); }
}

static double now(void)
{
   struct timespec t;
   clock_gettime(CLOCK_MONOTONIC, &t);
   return t.tv_sec + 1e-9 * t.tv_nsec;
}

int main(int argc, char **argv)
{
   FILE *f, *o;
   char magic[8];
   int hdr[8], i, s, repeats = 1, r;
   double cd[4], hm[9];
   system_mt sys;
   spec_mt *species;
   pot_mt *potpar;
   double *site_charge, *chg, *sites, *cofm, *fr, *fe;
   real *site[3], *f_real[3], *f_ew[3];
   double pe[2], t0, t_force = 0, t_ewald = 0;
   mat_mt stress_r, stress_e, hmat;
   int nsites, nmols, nspecies, max_id;

   if (argc < 3) { fprintf(stderr, "usage: %s in.mdsys out.bin [repeats]\n", argv[0]); return 2; }
   if (argc > 3) repeats = atoi(argv[3]);
   f = fopen(argv[1], "rb");
   if (!f) { perror(argv[1]); return 2; }
   rd(magic, 1, 8, f);
   if (memcmp(magic, "MDSYS1", 6)) { fprintf(stderr, "harness: bad magic\n"); return 2; }
   rd(hdr, 4, 8, f);
   rd(cd, 8, 4, f);
   rd(hm, 8, 9, f);
   nsites = hdr[0]; nmols = hdr[1]; nspecies = hdr[2]; max_id = hdr[3];

   memset(&control, 0, sizeof control);
   control.strict_cutoff = hdr[5];
   control.molpbc = hdr[6];
   control.cutoff = cd[0];
   control.subcell = cd[1];
   control.alpha = cd[2];
   control.k_cutoff = cd[3];
   control.page_width = 132;
   control.page_length = 1000000;
   cap_on = hdr[7];
   {
      const char *e = getenv("MDGPU_REF_RDF");
      double lim;
      int nb;
      if (e && sscanf(e, "%lf %d", &lim, &nb) == 2) {
         control.limit = lim;
         control.nbins = nb;
         control.rdf_interval = 1;   /* step 0 is an RDF step (src/force.c:1302-1304) */
         control.begin_rdf = 0;
         control.istep = 0;
      }
   }

   memset(&sys, 0, sizeof sys);
   sys.nsites = nsites; sys.nmols = nmols; sys.nspecies = nspecies; sys.max_id = max_id;
   sys.ptype = hdr[4];
   {
      static const int npar[] = {2, 3, 4, 6, 3, 1, 7};
      sys.n_potpar = npar[sys.ptype];
   }
   for (i = 0; i < 9; i++) hmat[i / 3][i % 3] = hm[i];
   sys.h = hmat;

   species = (spec_mt *)calloc(nspecies, sizeof(spec_mt));
   for (s = 0; s < nspecies; s++) {
      int sh[4];
      rd(sh, 4, 4, f);
      species[s].nsites = sh[0];
      species[s].nmols = sh[1];
      species[s].framework = sh[2];
      species[s].site_id = (int *)malloc(sizeof(int) * (sh[0] + 1));
      rd(species[s].site_id, 4, sh[0], f);
      species[s].p_f_sites = (vec_mt *)malloc(sizeof(vec_mt) * sh[0]);
      rd(species[s].p_f_sites, 8, 3 * sh[0], f);
   }
   potpar = (pot_mt *)calloc((size_t)max_id * max_id, sizeof(pot_mt));
   for (i = 0; i < max_id * max_id; i++) rd(potpar[i].p, 8, NPOTP, f);
   site_charge = (double *)malloc(sizeof(double) * max_id);
   rd(site_charge, 8, max_id, f);
   sites = (double *)malloc(sizeof(double) * 3 * nsites);
   rd(sites, 8, 3 * (size_t)nsites, f);
   cofm = (double *)malloc(sizeof(double) * 3 * nmols);
   rd(cofm, 8, 3 * (size_t)nmols, f);
   fclose(f);
   sys.c_of_m = (vec_mt *)cofm;

   chg = (double *)malloc(sizeof(double) * nsites);
   {
      int k = 0, m, j;
      for (s = 0; s < nspecies; s++)
         for (m = 0; m < species[s].nmols; m++)
            for (j = 0; j < species[s].nsites; j++)
               chg[k++] = site_charge[species[s].site_id[j]];
   }
   fr = (double *)calloc(3 * (size_t)nsites, sizeof(double));
   fe = (double *)calloc(3 * (size_t)nsites, sizeof(double));
   for (i = 0; i < 3; i++) {
      site[i] = sites + (size_t)i * nsites;
      f_real[i] = fr + (size_t)i * nsites;
      f_ew[i] = fe + (size_t)i * nsites;
   }

   if (control.rdf_interval > 0) init_rdf(&sys);
   for (r = 0; r < repeats; r++) {
      if (r > 0) control.rdf_interval = 0;   /* one accumulation only */
      memset(fr, 0, sizeof(double) * 3 * nsites);
      memset(fe, 0, sizeof(double) * 3 * nsites);
      memset(stress_r, 0, sizeof stress_r);
      memset(stress_e, 0, sizeof stress_e);
      pe[0] = pe[1] = 0.0;
      cap_nab = NULL;
      if (r > 0) cap_on = 0;   /* pairs are recorded on the first call only */
      t0 = now();
      force_calc(site, f_real, &sys, species, chg, potpar, &pe[0], stress_r);
      if (r > 0) t_force += now() - t0;
      if (control.alpha > ALPHAMIN) {
         t0 = now();
         ewald(site, f_ew, &sys, species, chg, &pe[1], stress_e);
         if (r > 0) t_ewald += now() - t0;
      }
   }
   if (repeats > 1)
      printf("HARNESS_TIMING force_calc %.9f ewald %.9f\n", t_force / (repeats - 1),
             t_ewald / (repeats - 1));

   o = fopen(argv[2], "wb");
   if (!o) { perror(argv[2]); return 2; }
   fwrite(fr, 8, 3 * (size_t)nsites, o);
   fwrite(&pe[0], 8, 1, o);
   fwrite(stress_r, 8, 9, o);
   fwrite(fe, 8, 3 * (size_t)nsites, o);
   fwrite(&pe[1], 8, 1, o);
   fwrite(stress_e, 8, 9, o);
   {
      int64_t n = hdr[7] ? cap_n : -1;
      fwrite(&n, 8, 1, o);
      if (n > 0) fwrite(cap_pairs, 4, 3 * (size_t)n, o);
   }
   if (getenv("MDGPU_REF_RDF")) {
      int size = 0;
      float *h = (float *)rdf_ptr(&size);
      int64_t n = size;
      fwrite(&n, 8, 1, o);
      fwrite(h, 4, (size_t)size, o);
   }
   fclose(o);
   return 0;
}
