/*
 * ref_examples.c -- TEST INFRASTRUCTURE ONLY.  Runs the reference's own
 * start-up (start_up, src/startup.c:851) on one of the reference's example
 * control files and writes the resulting configuration as an MDSYS1 file
 * (the layout of moldy_gb300/system.py:write_mdsys), with site co-ordinates
 * built by the reference's make_sites (src/algorith.c:169) exactly as
 * eval_forces does before its force_calc call (src/accel.c:500-514).  Lets
 * the fixture generator replay the reference's shipped example runs.
 *
 * usage: moldy_ref_examples control-file out.mdsys
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "defs.h"
#include "structs.h"

contr_mt control;
int ithread = 0, nthreads = 1;

void start_up(char *, char *, system_mp, spec_mp *, site_mp *, pot_mp *, restrt_mt *, int *,
              boolean *);
void make_sites(mat_mt, vec_mp, quat_mp, vec_mp, real **, int, int, int);

int main(int argc, char **argv)
{
   system_mt sys;
   spec_mt *species;
   site_mt *site_info;
   pot_mt *potpar;
   restrt_mt hdr;
   int backup = 0, s, i, isite = 0;
   boolean new_ens = 0;
   FILE *o;
   real *site[3];
   double *buf;
   int ints[8];
   double cd[4];

   if (argc < 3) { fprintf(stderr, "usage: %s control out.mdsys\n", argv[0]); return 2; }
   memset(&sys, 0, sizeof sys);
   start_up(argv[1], "", &sys, &species, &site_info, &potpar, &hdr, &backup, &new_ens);
   buf = (double *)malloc(sizeof(double) * 3 * sys.nsites);
   for (i = 0; i < 3; i++) site[i] = buf + (size_t)i * sys.nsites;
   for (s = 0; s < sys.nspecies; s++) {
      real *sp[3];
      for (i = 0; i < 3; i++) sp[i] = site[i] + isite;
      make_sites(sys.h, species[s].c_of_m, species[s].quat, species[s].p_f_sites, sp,
                 species[s].nmols, species[s].nsites, control.molpbc ? MOLPBC : SITEPBC);
      isite += species[s].nmols * species[s].nsites;
   }
   o = fopen(argv[2], "wb");
   if (!o) { perror(argv[2]); return 2; }
   fwrite("MDSYS1\0\0", 1, 8, o);
   ints[0] = sys.nsites; ints[1] = sys.nmols; ints[2] = sys.nspecies; ints[3] = sys.max_id;
   ints[4] = sys.ptype; ints[5] = control.strict_cutoff; ints[6] = control.molpbc; ints[7] = 0;
   fwrite(ints, 4, 8, o);
   cd[0] = control.cutoff; cd[1] = control.subcell; cd[2] = control.alpha; cd[3] = control.k_cutoff;
   fwrite(cd, 8, 4, o);
   fwrite(sys.h, 8, 9, o);
   for (s = 0; s < sys.nspecies; s++) {
      int sh[4];
      sh[0] = species[s].nsites; sh[1] = species[s].nmols; sh[2] = species[s].framework; sh[3] = 0;
      fwrite(sh, 4, 4, o);
      fwrite(species[s].site_id, 4, species[s].nsites, o);
      fwrite(species[s].p_f_sites, 8, 3 * species[s].nsites, o);
   }
   for (i = 0; i < sys.max_id * sys.max_id; i++) fwrite(potpar[i].p, 8, NPOTP, o);
   for (i = 0; i < sys.max_id; i++) fwrite(&site_info[i].charge, 8, 1, o);
   fwrite(buf, 8, 3 * (size_t)sys.nsites, o);
   fwrite(sys.c_of_m, 8, 3 * (size_t)sys.nmols, o);
   fclose(o);
   return 0;
}
