/*
 * moldy_port.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A C restatement of Moldy's real-space link-cell force loop
 * (src/force.c:119-1320), pair-potential kernel (src/kernel.c:157-463) and
 * reciprocal-space Ewald sum (src/ewald.c:95-589).  It is the parity checker
 * the tests compare the CUDA path against, and the CPU baseline bench.py
 * times.  It is never linked into, or called by, the product library.
 *
 * Differences from the reference that do not change results:
 *  - no first-call statics: the intramolecular correction and the Ewald
 *    self/sheet energies are recomputed on every call;
 *  - FATAL/ERROR messages become negative return codes;
 *  - threads stride over link cells and block the k-vector list exactly as
 *    the reference's replicated-data ranks do (src/force.c:856,
 *    src/ewald.c:495-496), each with private accumulators that are summed at
 *    the end.
 */
#ifndef MOLDY_PORT_H
#define MOLDY_PORT_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
   int nsites, nmols, nspecies, max_id, ptype;
   const int *spec_nsites;     /* [nspecies] sites per molecule             */
   const int *spec_nmols;      /* [nspecies]                                */
   const int *spec_framework;  /* [nspecies]                                */
   const int *spec_site_id;    /* concatenated per-species site ids         */
   const double *spec_pf;      /* concatenated principal-frame sites [][3]  */
   const double *potpar;       /* [max_id*max_id][8]                        */
   const double *site_charge;  /* [max_id] charge of each site id           */
   const double *c_of_m;       /* [nmols][3] fractional centres of mass     */
   double h[3][3];
   double cutoff, subcell, alpha, k_cutoff;
   int strict_cutoff, molpbc;
} port_system;

typedef struct {
   int nx, ny, nz, n_nabors;          /* subcells and half neighbour list   */
   int hmax, kmax, lmax, nkvec;       /* k-space extent and k-vector count  */
   double eintra, self_energy, sheet_energy;
   int64_t npairs;                    /* evaluated site pairs               */
   int64_t n_too_close;               /* TOOCLS warnings                    */
   int64_t n_nab_max, n_nab_cap;      /* largest site list vs. its capacity */
   double t_setup, t_kloop;           /* ewald: set-up and k-loop wall time */
} port_info;

enum {
   PORT_OK = 0,
   PORT_E_ARG = -1,
   PORT_E_CUTOFF = -2,       /* stencil reaches beyond one image (CUTOFF)     */
   PORT_E_RANGE = -3,        /* co-ordinate out of range in binning           */
   PORT_E_TONAB = -4,        /* neighbour-site list capacity exceeded (TONAB)  */
   PORT_E_PTYPE = -5,        /* unknown potential type (UNKPTY)               */
   PORT_E_FRAMEWORK = -6,    /* (not returned: frameworks are restated too)  */
   PORT_E_NOMEM = -7,
   PORT_E_PAIRCAP = -8       /* pair output buffer too small                  */
};

/* Real-space part: adds into site_force[3][nsites] (SoA), *pe and the stress
 * upper triangle (row-major [9]).  pairs (optional) receives one
 * (isite, jsite, image) triplet per evaluated pair, image in 0..26 as
 * 9*(ix+1)+3*(iy+1)+(iz+1). */
int port_force_calc(const port_system *sys, const double *site, double *site_force,
                    double *pe, double *stress, int nthreads,
                    int32_t *pairs, int64_t pairs_cap, port_info *info);

/* Reciprocal-space part over k-vectors [k_first, k_last) of the list
 * (k_last < 0 means all); adds into site_force, *pe and stress. */
int port_ewald(const port_system *sys, const double *site, double *site_force,
               double *pe, double *stress, int nthreads, int64_t k_first, int64_t k_last,
               port_info *info);

/* Potential at one distance (src/force.c:632-650), alpha as the control. */
double port_poteval(const double *potpar, double r, int ptype, double chgsq, double alpha);

#ifdef __cplusplus
}
#endif
#endif
