/*
 * ref_md.c -- TEST INFRASTRUCTURE ONLY.  Runs the reference's own
 * constant-energy dynamics (do_step, src/accel.c:626-827, with
 * eval_forces, force_calc, ewald and the leapfrog of src/leapfrog.c) from a
 * given state, and records the conserved quantity do_step evaluates at the
 * half kick (H_0, src/accel.c:718-727; asked for every step) with the two
 * potential-energy parts, then the final state.  The golden trajectories of
 * the GPU integrator's tests come from here.
 *
 * usage: moldy_ref_md in.mdstate out.bin [dump-name level interval ndumps title]
 *
 * With the optional arguments the reference's own periodic dump (dump(),
 * src/dump.c:278-499, called from do_step, src/accel.c:811-820) writes its
 * files from step 1 (begin-dump 1) into the working directory; species are
 * named spec0, spec1, ... and carry the molecular charge and dipole that
 * the reference's start-up computes (src/startup.c:487-496, 571-580).
 *
 * in.mdstate (little-endian, written by oracle/md.py):
 *   "MDSTAT1\0"
 *   int32  nsites nmols nspecies max_id ptype strict molpbc nosym nsteps 0
 *   f64    cutoff subcell alpha k_cutoff step
 *   f64    h[3][3]
 *   per species: int32 nsites nmols framework rdof; int32 site_id[nsites];
 *                f64 p_f_sites[nsites][3]; f64 mass inertia[3]
 *   f64    potpar[max_id*max_id][8]; f64 charge[max_id]
 *   f64    c_of_m[nmols][3] mom[nmols][3] quat[nmols_r][4] amom[nmols_r][4]
 * out.bin: f64 per step (H_0, pe[0], pe[1]); then c_of_m, mom, quat, amom;
 *   then f64 seconds per step.
 *
 * Constant temperature (the Nose-Poincare thermostat of do_step,
 * src/accel.c:673-684, 696-700, 757-791):
 *   MOLDY_REF_CONST_TEMP="T Q"  const-temp 1 at temperature T (K) with
 *     thermostat mass Q (control.ttmass); H_0 is set on the first step only
 *     and each step's record adds the thermostat variable and momentum
 *     (H_0, pe[0], pe[1], ts, tsmom).
 *
 * Constant pressure (the Parrinello-Rahman cell dynamics of do_step,
 * src/accel.c:686-704, 759-783):
 *   MOLDY_REF_CONST_PRESSURE="mode P W mask"  const-pressure mode (1
 *     anisotropic, 2 uniform) at pressure P with cell mass W and strain mask;
 *     each step's record then adds h and its momentum (row-major 3x3 each).
 *
 * Restart files (the reference's own writer and reader, src/restart.c):
 *   MOLDY_REF_RESTART_OUT=path  after the run, write_restart (native
 *     format, src/restart.c:435-548) saves the whole state to path;
 *   MOLDY_REF_RESTART_IN=path   before the run, the dynamic state (centres
 *     of mass, momenta, quaternions, angular momenta) is taken from the
 *     restart file at path instead, read back by the reference's start-up
 *     sequence: re_re_header, re_re_sysdef, allocate_dynamics,
 *     init_averages, read_restart (src/startup.c:1001-1023).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <math.h>
#include "defs.h"
#include "structs.h"

contr_mt control;
int ithread = 0, nthreads = 1;

void do_step(system_mt *, spec_mt *, site_mt *, pot_mt *, vec_mt (*)[2], double *, real *, mat_mt,
             restrt_mt *, int, int);
void write_restart(char *, restrt_mt *, system_mp, spec_mp, site_mp, pot_mp);
void re_re_header(FILE *, restrt_mt *, contr_mt *);
void re_re_sysdef(FILE *, char *, system_mp, spec_mp *, site_mp *, pot_mp *);
void allocate_dynamics(system_mp, spec_mt *);
void init_averages(int, char *, long int, long int, int *);
void read_restart(FILE *, char *, system_mp, int);

static void rd(void *p, size_t sz, size_t n, FILE *f)
{
   if (fread(p, sz, n, f) != n) { fprintf(stderr, "ref_md: short read\n"); exit(2); }
}

int main(int argc, char **argv)
{
   FILE *f, *o;
   char magic[8];
   int hdr[10], s, i, nsteps, nq = 0, imol = 0, iq = 0;
   double cd[5];
   system_mt sys;
   spec_mt *species;
   site_mt *site_info;
   pot_mt *potpar;
   restrt_mt rh;
   double pe[NPE];
   real dip[3];
   mat_mt stress;
   vec_mt (*msq)[2];
   struct timespec t0, t1;

   if (argc < 3) { fprintf(stderr, "usage: %s in.mdstate out.bin [dump-name level interval ndumps title]\n", argv[0]); return 2; }
   f = fopen(argv[1], "rb");
   if (!f) { perror(argv[1]); return 2; }
   rd(magic, 1, 8, f);
   if (memcmp(magic, "MDSTAT1", 7)) { fprintf(stderr, "ref_md: bad magic\n"); return 2; }
   rd(hdr, 4, 10, f);
   rd(cd, 8, 5, f);
   memset(&sys, 0, sizeof sys);
   memset(&control, 0, sizeof control);
   memset(&rh, 0, sizeof rh);
   sys.nsites = hdr[0]; sys.nmols = hdr[1]; sys.nspecies = hdr[2]; sys.max_id = hdr[3];
   sys.ptype = hdr[4];
   {
      /* parameter count of each potential type (src/kernel.c:61-68) */
      static const int npar[7] = {2, 3, 4, 6, 3, 0, 7};
      if (sys.ptype < 0 || sys.ptype > 6 || npar[sys.ptype] == 0) { fprintf(stderr, "ref_md: ptype\n"); return 2; }
      sys.n_potpar = npar[sys.ptype];
   }
   control.strict_cutoff = hdr[5]; control.molpbc = hdr[6]; control.nosymmetric_rot = hdr[7];
   nsteps = hdr[8];
   control.cutoff = cd[0]; control.subcell = cd[1]; control.alpha = cd[2]; control.k_cutoff = cd[3];
   control.step = cd[4];
   control.ttmass = 1.0; control.pmass = 1.0;   /* unused at constant energy, kept finite */
   control.print_interval = 1000000000;
   sys.h = (mat_mp)calloc(1, sizeof(mat_mt));
   sys.hmom = (mat_mp)calloc(1, sizeof(mat_mt));
   sys.hmomp = (mat_mp)calloc(1, sizeof(mat_mt));
   rd(sys.h, 8, 9, f);
   sys.ts = 1.0; sys.tsmom = 0.0;
   species = (spec_mt *)calloc(sys.nspecies, sizeof(spec_mt));
   for (s = 0; s < sys.nspecies; s++) {
      int sh[4];
      double mi[4];
      spec_mt *sp = species + s;
      rd(sh, 4, 4, f);
      sp->nsites = sh[0]; sp->nmols = sh[1]; sp->framework = sh[2]; sp->rdof = sh[3];
      sp->site_id = (int *)malloc(sizeof(int) * sp->nsites);
      sp->p_f_sites = (vec_mp)malloc(sizeof(vec_mt) * sp->nsites);
      rd(sp->site_id, 4, sp->nsites, f);
      rd(sp->p_f_sites, 8, 3 * sp->nsites, f);
      rd(mi, 8, 4, f);
      sp->mass = mi[0]; sp->inertia[0] = mi[1]; sp->inertia[1] = mi[2]; sp->inertia[2] = mi[3];
      if (sp->rdof > 0) nq += sp->nmols;
      /* degrees of freedom as start_up counts them (src/startup.c:483-485,
         570, 591): no translation for a framework */
      sys.d_of_f += (sp->framework ? 0 : 3 * sp->nmols) + sp->rdof * sp->nmols;
   }
   sys.d_of_f -= 3;
   sys.nmols_r = nq;
   potpar = (pot_mt *)calloc((size_t)sys.max_id * sys.max_id, sizeof(pot_mt));
   for (i = 0; i < sys.max_id * sys.max_id; i++) rd(potpar[i].p, 8, NPOTP, f);
   site_info = (site_mt *)calloc(sys.max_id, sizeof(site_mt));
   for (i = 0; i < sys.max_id; i++) rd(&site_info[i].charge, 8, 1, f);
   sys.c_of_m = (vec_mp)malloc(sizeof(vec_mt) * sys.nmols);
   sys.mom = (vec_mp)malloc(sizeof(vec_mt) * sys.nmols);
   sys.momp = (vec_mp)calloc(sys.nmols, sizeof(vec_mt));
   sys.quat = (quat_mp)malloc(sizeof(quat_mt) * (nq ? nq : 1));
   sys.amom = (quat_mp)malloc(sizeof(quat_mt) * (nq ? nq : 1));
   sys.amomp = (quat_mp)calloc(nq ? nq : 1, sizeof(quat_mt));
   rd(sys.c_of_m, 8, 3 * (size_t)sys.nmols, f);
   rd(sys.mom, 8, 3 * (size_t)sys.nmols, f);
   if (nq) {
      rd(sys.quat, 8, 4 * (size_t)nq, f);
      rd(sys.amom, 8, 4 * (size_t)nq, f);
   }
   fclose(f);
   /* species arrays point into the whole-system ones (src/startup.c:640-660) */
   for (s = 0; s < sys.nspecies; s++) {
      spec_mt *sp = species + s;
      sp->c_of_m = sys.c_of_m + imol;
      sp->mom = sys.mom + imol;
      sp->momp = sys.momp + imol;
      if (sp->rdof > 0) {
         sp->quat = sys.quat + iq;
         sp->amom = sys.amom + iq;
         sp->amomp = sys.amomp + iq;
         iq += sp->nmols;
      }
      imol += sp->nmols;
   }
   if (argc >= 8) {
      strncpy(control.dump_file, argv[3], L_name - 3);
      control.dump_level = atoi(argv[4]);
      control.dump_interval = atol(argv[5]);
      control.maxdumps = atoi(argv[6]);
      strncpy(control.title, argv[7], L_name - 1);
      control.begin_dump = 1;
      for (s = 0; s < sys.nspecies; s++) {
         spec_mt *sp = species + s;
         double dip[3] = {0.0, 0.0, 0.0};
         int k;
         sprintf(sp->name, "spec%d", s);
         sp->charge = 0.0;
         for (i = 0; i < sp->nsites; i++) {
            sp->charge += site_info[sp->site_id[i]].charge;
            for (k = 0; k < 3; k++) dip[k] += sp->p_f_sites[i][k] * site_info[sp->site_id[i]].charge;
         }
         sp->dipole = sp->rdof > 0 ? sqrt(dip[0] * dip[0] + dip[1] * dip[1] + dip[2] * dip[2]) : 0.0;
      }
   }
   control.roll_interval = 10;
   if (getenv("MOLDY_REF_RESTART_IN")) {
      const char *rin = getenv("MOLDY_REF_RESTART_IN");
      FILE *rf = fopen(rin, "rb");
      restrt_mt rhdr;
      contr_mt rctl;
      system_mt rsys;
      spec_mp rspec;
      site_mp rsite;
      pot_mp rpot;
      int avc = 0;
      if (!rf) { perror(rin); return 2; }
      memset(&rsys, 0, sizeof rsys);
      re_re_header(rf, &rhdr, &rctl);
      re_re_sysdef(rf, rhdr.vsn, &rsys, &rspec, &rsite, &rpot);
      allocate_dynamics(&rsys, rspec);
      init_averages(rsys.nspecies, rhdr.vsn, rctl.roll_interval, rctl.roll_interval, &avc);
      read_restart(rf, rhdr.vsn, &rsys, avc);
      fclose(rf);
      if (rsys.nmols != sys.nmols || rsys.nmols_r != sys.nmols_r) {
         fprintf(stderr, "ref_md: restart file does not match the system\n");
         return 2;
      }
      memcpy(sys.c_of_m, rsys.c_of_m, sizeof(vec_mt) * sys.nmols);
      memcpy(sys.mom, rsys.mom, sizeof(vec_mt) * sys.nmols);
      if (nq) {
         memcpy(sys.quat, rsys.quat, sizeof(quat_mt) * nq);
         memcpy(sys.amom, rsys.amom, sizeof(quat_mt) * nq);
      }
   } else if (getenv("MOLDY_REF_RESTART_OUT")) {
      int avc = 0;
      init_averages(sys.nspecies, (char *)0, control.roll_interval, control.roll_interval, &avc);
   }
   msq = (vec_mt(*)[2])calloc(sys.nspecies, sizeof(vec_mt[2]));
   o = fopen(argv[2], "wb");
   if (!o) { perror(argv[2]); return 2; }
   clock_gettime(CLOCK_MONOTONIC, &t0);
   {
      const char *ct = getenv("MOLDY_REF_CONST_TEMP");
      const char *cp = getenv("MOLDY_REF_CONST_PRESSURE");
      if (ct && sscanf(ct, "%lf %lf", &control.temp, &control.ttmass) == 2) control.const_temp = 1;
      if (cp && sscanf(cp, "%d %lf %lf %d", &control.const_pressure, &control.pressure, &control.pmass,
                       &control.strain_mask) != 4) control.const_pressure = 0;
   }
   for (control.istep = 1; control.istep <= nsteps; control.istep++) {
      double rec[23];
      const int ens = control.const_temp || control.const_pressure;
      do_step(&sys, species, site_info, potpar, msq, pe, dip, stress, &rh, 0, ens ? 0 : 1);
      rec[0] = sys.H_0; rec[1] = pe[0]; rec[2] = pe[1]; rec[3] = sys.ts; rec[4] = sys.tsmom;
      memcpy(rec + 5, sys.h, 9 * sizeof(double));
      memcpy(rec + 14, sys.hmom, 9 * sizeof(double));
      fwrite(rec, 8, control.const_pressure ? 23 : ens ? 5 : 3, o);
   }
   clock_gettime(CLOCK_MONOTONIC, &t1);
   if (getenv("MOLDY_REF_RESTART_OUT")) {
      char *rout = getenv("MOLDY_REF_RESTART_OUT");
      snprintf(control.temp_file, sizeof control.temp_file, "%s.tmp", rout);
      strncpy(control.backup_file, "none", sizeof control.backup_file);
      write_restart(rout, &rh, &sys, species, site_info, potpar);
   }
   fwrite(sys.c_of_m, 8, 3 * (size_t)sys.nmols, o);
   fwrite(sys.mom, 8, 3 * (size_t)sys.nmols, o);
   if (nq) {
      fwrite(sys.quat, 8, 4 * (size_t)nq, o);
      fwrite(sys.amom, 8, 4 * (size_t)nq, o);
   }
   {
      double sec = ((t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec)) / (nsteps > 0 ? nsteps : 1);
      fwrite(&sec, 8, 1, o);
   }
   fclose(o);
   return 0;
}
