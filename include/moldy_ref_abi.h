/*
 * moldy_ref_abi.h -- drop-in entry points of libmoldy_gb300.so with the
 * reference's own signatures.
 *
 * Linking Moldy's objects against libmoldy_gb300.so in place of force.o and
 * ewald.o makes the reference's time step (eval_forces, src/accel.c:398-617)
 * call the GPU path.  The three functions below replace:
 *
 *   force_calc  src/force.c:1108-1320  (prototype src/accel.c:74-76)
 *   ewald       src/ewald.c:280-589    (prototype src/accel.c:80-81)
 *   poteval     src/force.c:632-650    (prototype src/accel.c:77)
 *
 * They read the caller's global `control` record (src/main.c:83) and report
 * through the caller's note()/message() (src/output.c:131-190) when those
 * are linked in; an error the reference treats as FATAL ends the process
 * with exit status 3, as message(FATAL) does.  Precision is chosen with the
 * environment variable MDGPU_PRECISION=fp64|mixed (default mixed) and the
 * device with MDGPU_DEVICE (default 0).
 *
 * The struct layouts below must match the caller's src/structs.h byte for
 * byte (they are the reference's ABI, restated field by field with the
 * same types and order); tests/test_abi.py checks every offset against the
 * reference's own header where the reference is available.
 */
#ifndef MOLDY_REF_ABI_H
#define MOLDY_REF_ABI_H

#ifdef __cplusplus
extern "C" {
#endif

#ifndef STRUCT_ALREADY            /* the reference's structs.h include guard */
typedef double real;
typedef int boolean;
typedef real vec_mt[3];
typedef vec_mt *vec_mp;
typedef real quat_mt[4];
typedef quat_mt *quat_mp;
typedef real mat_mt[3][3];
typedef vec_mt *mat_mp;

#define MDGPU_L_NAME 128          /* src/defs.h:159 */
#define MDGPU_L_SPEC 32           /* src/defs.h:160 */
#define MDGPU_L_SITE 8            /* src/defs.h:161 */
#define MDGPU_NPOTP 8             /* src/defs.h:144 */

typedef struct {                  /* contr_mt, src/structs.h:27-85 */
   char title[MDGPU_L_NAME];
   long istep, nsteps;
   double step;
   boolean print_sysdef, new_sysdef, molpbc, reset_averages;
   int scale_options;
   boolean surface_dipole, lattice_start;
   char sysdef[MDGPU_L_NAME], restart_file[MDGPU_L_NAME], save_file[MDGPU_L_NAME],
        dump_file[MDGPU_L_NAME], backup_file[MDGPU_L_NAME], temp_file[MDGPU_L_NAME];
   int spare[20];
   boolean nosymmetric_rot;
   double ewald_accuracy;
   double ttmass, rtmass;
   int const_pressure;
   int const_temp;
   boolean xdr_write, strict_cutoff;
   int strain_mask;
   int nbins;
   unsigned long seed;
   int page_width, page_length;
   long scale_interval, scale_end, begin_average, average_interval, begin_dump, dump_offset,
        dump_interval;
   int dump_level, maxdumps;
   long backup_interval, roll_interval, print_interval, begin_rdf, rdf_interval, rdf_out;
   double temp, pressure, pmass, cutoff, subcell, density, alpha, k_cutoff, limit, cpu_limit;
} contr_mt;

typedef struct {                  /* system_mt, src/structs.h:87-118 */
   int nsites, nmols, nmols_r, nspecies, max_id, d_of_f;
   int ptype, n_potpar;
   vec_mp c_of_m, mom, momp;
   quat_mp quat, amom, amomp;
   mat_mp h, hmom, hmomp;
   real ts, tsmom;
   real H_0;
   real rs, rsmom;
} system_mt, *system_mp;

typedef struct {                  /* spec_mt, src/structs.h:121-145 */
   real inertia[3], mass, dipole, charge;
   int nsites, nmols;
   int rdof, framework;
   char name[MDGPU_L_SPEC];
   int *site_id;
   vec_mp p_f_sites;
   vec_mp c_of_m, mom, momp;
   quat_mp quat, amom, amomp;
} spec_mt, *spec_mp;

typedef struct {                  /* pot_mt, src/structs.h:156-161 */
   int flag;
   int pad;
   real p[MDGPU_NPOTP];
} pot_mt, *pot_mp;
#endif /* STRUCT_ALREADY */

void force_calc(real **site, real **site_force, system_mt *system, spec_mt *species,
                real *chg, pot_mt *potpar, double *pe, mat_mt stress);
void ewald(real **site, real **site_force, system_mp system, spec_mt *species, real *chg,
           double *pe, mat_mt stress);
double poteval(real *potpar, double r, int ptype, double chgsq);

#ifdef __cplusplus
}
#endif
#endif
