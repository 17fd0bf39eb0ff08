/*
 * ref_abi_driver.c -- calls libmoldy_gb300's drop-in entry points exactly as
 * the reference's time step does (eval_forces, src/accel.c:398-535):
 * a global `control` record, the reference's structs (include/moldy_ref_abi.h),
 * force_calc() into zeroed site_force/pe[0]/stress, then ewald() with pe+1.
 * It also supplies note()/message() in the reference's output format
 * (src/output.c:131-190), which the library prints through.
 *
 * Reads one configuration in the MDSYS1 layout (moldy_gb300/system.py) and
 * writes forces/energies/stress in the layout of oracle/ref_harness.c, so the
 * tests compare it with the reference's golden outputs.
 *
 * With DRIVER_RDF="limit nbins" in the environment the first call is an RDF
 * step (control.rdf_interval = 1 at istep 0): the library adds the pair
 * histogram into the driver's RDF array, which stands in for the
 * reference's rdf.c (rdf_ptr, src/rdf.c:58-62, with init_rdf's layout), and
 * the array is appended to the output as int64 size + float[size].
 *
 * usage: ref_abi_driver in.mdsys out.bin
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include "moldy_ref_abi.h"

contr_mt control;
int ithread = 0, nthreads = 1;

void note(char *text, ...)
{
   va_list ap;
   va_start(ap, text);
   printf(" *I* ");
   vprintf(text, ap);
   printf("\n");
   va_end(ap);
}

void message(int *nerrs, ...)
{
   static const char *sev_txt[] = {" *I* ", " *W* ", " *E* ", " *F* "};
   va_list ap;
   char *buff, *format;
   int sev;
   va_start(ap, nerrs);
   buff = va_arg(ap, char *);
   sev = va_arg(ap, int);
   format = va_arg(ap, char *);
   printf("%s", sev_txt[sev & 3]);
   vprintf(format, ap);
   printf("\n");
   va_end(ap);
   (void)buff;
   if (sev == 3) {
      fflush(stdout);
      exit(3);
   }
}

static float *rdf_base = NULL;
static int rdf_size = 0;

void *rdf_ptr(int *size)
{
   *size = rdf_size;
   return rdf_base;
}

static void rd(void *p, size_t sz, size_t n, FILE *f)
{
   if (fread(p, sz, n, f) != n) {
      fprintf(stderr, "driver: short read\n");
      exit(2);
   }
}

int main(int argc, char **argv)
{
   FILE *f, *o;
   char magic[8];
   int hdr[8], i, s, nsites, nmols, nspecies, max_id;
   double cd[4], hm[9], *site_charge, *chg, *sites, *cofm, *fr, *pe;
   system_mt sys;
   spec_mt *species;
   pot_mt *potpar;
   mat_mt hmat, stress_r, stress_e;
   real *site[3], *force_r[3];
   double pes[2] = {0.0, 0.0};
   int64_t npairs = -1;

   if (argc < 3) return 2;
   f = fopen(argv[1], "rb");
   if (!f) return 2;
   rd(magic, 1, 8, f);
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
   if (getenv("DRIVER_RDF")) {
      double lim;
      int nb;
      if (sscanf(getenv("DRIVER_RDF"), "%lf %d", &lim, &nb) == 2) {
         control.limit = lim;
         control.nbins = nb;
         control.rdf_interval = 1;
         control.begin_rdf = 0;
         control.istep = 0;
         rdf_size = nb * max_id * (max_id - 1) / 2;
         rdf_base = (float *)calloc(rdf_size, sizeof(float));
      }
   }
   memset(&sys, 0, sizeof sys);
   sys.nsites = nsites; sys.nmols = nmols; sys.nspecies = nspecies; sys.max_id = max_id;
   sys.ptype = hdr[4];
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
      species[s].p_f_sites = (vec_mp)malloc(sizeof(vec_mt) * sh[0]);
      rd(species[s].p_f_sites, 8, 3 * sh[0], f);
   }
   potpar = (pot_mt *)calloc((size_t)max_id * max_id, sizeof(pot_mt));
   for (i = 0; i < max_id * max_id; i++) rd(potpar[i].p, 8, MDGPU_NPOTP, f);
   site_charge = (double *)malloc(sizeof(double) * max_id);
   rd(site_charge, 8, max_id, f);
   sites = (double *)malloc(sizeof(double) * 3 * nsites);
   rd(sites, 8, 3 * (size_t)nsites, f);
   cofm = (double *)malloc(sizeof(double) * 3 * nmols);
   rd(cofm, 8, 3 * (size_t)nmols, f);
   fclose(f);
   sys.c_of_m = (vec_mp)cofm;
   chg = (double *)malloc(sizeof(double) * nsites);
   {
      int k = 0, m, j;
      for (s = 0; s < nspecies; s++)
         for (m = 0; m < species[s].nmols; m++)
            for (j = 0; j < species[s].nsites; j++) chg[k++] = site_charge[species[s].site_id[j]];
   }
   /* separate real-space and reciprocal-space force arrays, as the golden
    * fixtures hold them separately */
   fr = (double *)calloc(6 * (size_t)nsites, sizeof(double));
   for (i = 0; i < 3; i++) {
      site[i] = sites + (size_t)i * nsites;
      force_r[i] = fr + (size_t)i * nsites;
   }
   memset(stress_r, 0, sizeof stress_r);
   memset(stress_e, 0, sizeof stress_e);
   force_calc(site, force_r, &sys, species, chg, potpar, &pes[0], stress_r);
   if (control.alpha > 1e-7) {
      real *force_e[3];
      for (i = 0; i < 3; i++) force_e[i] = fr + (size_t)(3 + i) * nsites;
      ewald(site, force_e, &sys, species, chg, &pes[1], stress_e);
   }
   pe = pes;
   o = fopen(argv[2], "wb");
   if (!o) return 2;
   fwrite(fr, 8, 3 * (size_t)nsites, o);
   fwrite(&pe[0], 8, 1, o);
   fwrite(stress_r, 8, 9, o);
   fwrite(fr + 3 * (size_t)nsites, 8, 3 * (size_t)nsites, o);
   fwrite(&pe[1], 8, 1, o);
   fwrite(stress_e, 8, 9, o);
   fwrite(&npairs, 8, 1, o);
   if (rdf_base) {
      int64_t n = rdf_size;
      fwrite(&n, 8, 1, o);
      fwrite(rdf_base, 4, (size_t)rdf_size, o);
      control.rdf_interval = 0;   /* the second call below is not an RDF step */
   }
   fclose(o);
   /* a second step on the same arrays: the notes must not repeat */
   memset(fr, 0, 6 * sizeof(double) * (size_t)nsites);
   pes[0] = pes[1] = 0.0;
   force_calc(site, force_r, &sys, species, chg, potpar, &pes[0], stress_r);
   printf("DRIVER second call pe %.17g\n", pes[0]);
   return 0;
}
