/*
 * moldy_gb300.h -- extended C ABI of the GB300 force path (libmoldy_gb300.so).
 *
 * The library evaluates Moldy's real-space link-cell forces (force_calc,
 * src/force.c:1108) and reciprocal-space Ewald forces (ewald,
 * src/ewald.c:280) with hand-written sm_103a CUDA kernels.  This header is
 * the status-returning interface: no reference structs, plain pointers and
 * sizes, every call returns an mdgpu_status.  The drop-in entry points with
 * the reference's own signatures are declared in moldy_ref_abi.h.
 *
 * Units are Moldy's program units (src/defs.h:213-236).  Site arrays are
 * structure-of-arrays: site[0..2] (or one contiguous [3][nsites] block).
 * h is the 3x3 cell matrix, row-major (h[i][j] at h[3*i+j]), upper
 * triangular as ewald() presumes (src/ewald.c:439).
 */
#ifndef MOLDY_GB300_H
#define MOLDY_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mdgpu_ctx mdgpu_ctx;

typedef enum {
   MDGPU_OK = 0,
   MDGPU_E_ARG = 1,          /* invalid argument or call order                   */
   MDGPU_E_CUDA = 2,         /* a CUDA runtime call failed                       */
   MDGPU_E_UNSUPPORTED = 3,  /* option outside the implemented path (a framework
                                species listed before another species,
                                non-upper-triangular h)                          */
   MDGPU_E_CUTOFF = 4,       /* neighbour cells beyond one image: the reference's
                                FATAL CUTOFF (src/force.c:203-206)               */
   MDGPU_E_RANGE = 5,        /* site co-ordinate outside the cell when binning
                                (src/force.c:126-135)                            */
   MDGPU_E_PTYPE = 6,        /* unknown potential type (UNKPTY, src/kernel.c:183)*/
   MDGPU_E_CAPACITY = 7,     /* an output buffer or internal limit is too small  */
   MDGPU_E_NOMEM = 8,        /* device allocation failed                         */
   MDGPU_E_IO = 9            /* a dump file could not be opened or written       */
} mdgpu_status;

typedef enum {
   MDGPU_FP64 = 0,           /* all arithmetic in FP64                           */
   MDGPU_MIXED = 1           /* FP32 pair and k-space arithmetic, FP64
                                accumulation of forces, energies and stress      */
} mdgpu_precision;

/* One molecular species (the fields of spec_mt the force path reads,
 * src/structs.h:121-145).  Species are listed in the reference's order. */
typedef struct {
   int nsites;                  /* sites per molecule                         */
   int nmols;                   /* molecules of this species                  */
   int framework;               /* nonzero: framework species (last, 1 mol.)  */
   const int *site_id;          /* [nsites] site identifiers (1..max_id-1)    */
   const double *p_f_sites;     /* [nsites][3] principal-frame co-ordinates   */
} mdgpu_species;

/* Everything about the system that does not change from step to step. */
typedef struct {
   int nspecies;
   const mdgpu_species *species;
   int max_id;                  /* dimension of the potential table           */
   int ptype;                   /* potential type, src/kernel.c:61-68 order   */
   const double *potpar;        /* [max_id*max_id][8], [id_i*max_id + id_j]   */
   const double *chg;           /* [nsites] site charges (src/accel.c:480-484)*/
} mdgpu_system;

/* The control-file keys on the path (src/startup.c:143-202). */
typedef struct {
   double cutoff;               /* real-space cutoff, Å                       */
   double subcell;              /* link-cell side, 0 = cutoff/5               */
   double alpha;                /* Ewald alpha; <= 1e-7 disables k-space      */
   double k_cutoff;             /* k-space cutoff, Å^-1                       */
   int strict_cutoff;           /* strict-cutoff keyword                      */
   int molpbc;                  /* molecular-cutoff keyword                   */
} mdgpu_control;

/* Counters and constants of the last call (mirrors the reference's notes). */
typedef struct {
   int nx, ny, nz;              /* subcells                                   */
   int n_nabors;                /* half neighbour-cell list (reference prints
                                   twice this, src/force.c:219-221)           */
   int nkvec, hmax, kmax, lmax;
   double eintra;               /* intramolecular correction (program units)  */
   double self_energy, sheet_energy;
   int64_t npairs;              /* evaluated site pairs (reference count)     */
   int64_t n_too_close;         /* pairs closer than 0.5 Å in different mols  */
   int32_t too_close[16][2];    /* the first of them, canonical orientation   */
   int64_t launches;            /* kernels launched by this context so far    */
} mdgpu_info;

/* Phases of one evaluation, for mdgpu_phase_times. */
enum {
   MDGPU_PH_CELLS = 0,          /* binning, cell sort, per-slot records       */
   MDGPU_PH_PAIRS = 1,          /* real-space pair kernel and its reduction   */
   MDGPU_PH_KPREP = 2,          /* per-site fixed-point phases                */
   MDGPU_PH_SFAC = 3,           /* structure factor partial sums              */
   MDGPU_PH_KREDUCE = 4,        /* per-k energy, stress, force coefficients   */
   MDGPU_PH_KFORCE = 5,         /* reciprocal-space site forces               */
   MDGPU_PH_FINAL = 6,          /* force partial sums, energy/stress record   */
   MDGPU_NPHASES = 7
};

/* Context on one CUDA device.  Not thread-safe: one host thread per context. */
mdgpu_status mdgpu_create(mdgpu_ctx **ctx, int device, mdgpu_precision precision);
void mdgpu_destroy(mdgpu_ctx *ctx);
const char *mdgpu_last_error(const mdgpu_ctx *ctx);
mdgpu_status mdgpu_set_precision(mdgpu_ctx *ctx, mdgpu_precision precision);
/* Runs every kernel on `stream` (a cudaStream_t) from now on; NULL restores
 * the context's own stream. */
mdgpu_status mdgpu_set_stream(mdgpu_ctx *ctx, void *stream);
mdgpu_status mdgpu_get_stream(mdgpu_ctx *ctx, void **stream);

/* Describe the system.  Copies what it needs; the first force call after
 * this recomputes the first-call constants (intramolecular correction,
 * Ewald self energy), as a fresh reference run would. */
mdgpu_status mdgpu_set_system(mdgpu_ctx *ctx, const mdgpu_system *sys);
mdgpu_status mdgpu_set_control(mdgpu_ctx *ctx, const mdgpu_control *ctl);

/* Real-space part with force_calc's semantics (src/force.c:1108-1320): adds
 * into site_force[3][nsites], *pe and the stress upper triangle.  site and
 * site_force are host arrays; c_of_m ([nmols][3] fractional) is read only in
 * molecular-cutoff mode and may be NULL otherwise. */
mdgpu_status mdgpu_force_calc(mdgpu_ctx *ctx, const double *h, double *const site[3],
                              double *const site_force[3], const double *c_of_m,
                              double *pe, double *stress);

/* Reciprocal-space part with ewald's semantics (src/ewald.c:280-589). */
mdgpu_status mdgpu_ewald(mdgpu_ctx *ctx, const double *h, double *const site[3],
                         double *const site_force[3], double *pe, double *stress);

/* Both parts in one call on host arrays: site_soa [3][nsites] in, force_out
 * [3][nsites] overwritten with the total site force, pe_out[2] = real-space
 * and reciprocal-space energy, stress_out[9] the upper-triangular virial
 * (lower triangle zero).  c_of_m as for mdgpu_force_calc. */
mdgpu_status mdgpu_forces(mdgpu_ctx *ctx, const double *h, const double *site_soa,
                          const double *c_of_m, double *force_out, double *pe_out,
                          double *stress_out);

/* As mdgpu_forces with every array already in device memory.  Asynchronous
 * on the context's stream; nothing is copied to or from the host.  Returns
 * MDGPU_E_RANGE/MDGPU_E_CUTOFF only on the next synchronising call. */
mdgpu_status mdgpu_forces_device(mdgpu_ctx *ctx, const double *h, const double *d_site_soa,
                                 const double *d_c_of_m, double *d_force_out,
                                 double *d_pe_out, double *d_stress_out);

/* Waits for the context's stream and reports device-side errors of earlier
 * asynchronous calls (binning range, too-close pairs are counted in info). */
mdgpu_status mdgpu_synchronize(mdgpu_ctx *ctx);

/* The record of the last evaluation.  The mixed form's pair kernel leaves
 * the pair count (npairs) out of its loop; this call then counts it over the
 * binned sites the evaluation left, waiting for the context's stream. */
mdgpu_status mdgpu_get_info(mdgpu_ctx *ctx, mdgpu_info *info);

/* Diagnostic phase timing.  While enabled, every evaluation records CUDA
 * events between its phases on the context's stream; mdgpu_phase_times waits
 * for the last evaluation and returns the milliseconds of each phase
 * (MDGPU_NPHASES values; phases that did not run read 0). */
mdgpu_status mdgpu_set_phase_timing(mdgpu_ctx *ctx, int enable);
mdgpu_status mdgpu_phase_times(mdgpu_ctx *ctx, double *ms);

/* Diagnostic: the evaluated real-space pair set of the given configuration
 * as canonical keys (i << 37 | j << 5 | image, i <= j, image as
 * moldy_gb300/pairset.py), unsorted.  *count receives the number of pairs;
 * MDGPU_E_CAPACITY if it exceeds cap (keys then holds the first cap). */
mdgpu_status mdgpu_pair_keys(mdgpu_ctx *ctx, const double *h, const double *site_soa,
                             const double *c_of_m, uint64_t *keys, int64_t cap,
                             int64_t *count);

/* Radial-distribution histogram of one configuration, as force_calc
 * accumulates it on RDF steps (rdf_inner/rdf_accum, src/force.c:1010-1103,
 * src/rdf.c:94-107): every site pair the strict neighbour-cell list at
 * `limit` reaches (on the cell grid of the force cutoff and subcell), bin =
 * (int)(nbins/limit * r), kept when below nbins; pairs within a molecule
 * included.  counts ([max_id][max_id][nbins], symmetric) receives the number
 * of unordered pairs of each identifier pair per bin, exact.  The
 * reference-signature force_calc adds these counts into the caller's own
 * RDF array on RDF steps. */
mdgpu_status mdgpu_rdf_counts(mdgpu_ctx *ctx, const double *h, const double *site_soa,
                              const double *c_of_m, double limit, int nbins, uint64_t *counts);

/* Reciprocal-space Ewald sum that allocates nothing.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc: hosts that own all
 * device memory through their own pools, and step loops that must not take
 * the allocator's locks, synchronise the device or fail for lack of memory
 * mid-run.  Adds the k-space forces into d_force[3][nsites], the k-space
 * energy (without the self and sheet terms of ewald(), src/ewald.c:367-433)
 * into *d_pe and the stress upper triangle into d_stress[9]; every pointer is
 * the caller's device memory, h is on the host and read during the call
 * only, charges d_chg[nsites] are in program units.  FP32-mixed arithmetic;
 * the sites are ordered by a cell grid inside the scratch, so ionic systems
 * listed species by species keep FP32 accuracy.  Intermediates, the k-vector
 * list included, live in a static device array of
 * MDGPU_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit; nsites above MDGPU_NOALLOC_MAX_SITES or more than
 * MDGPU_NOALLOC_MAX_KVEC k-vectors return MDGPU_E_CAPACITY.  The first call
 * on a device looks the array up (cudaGetSymbolAddress) and keeps its address
 * for the process (the device's primary context must stay the same); make
 * that first call before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (other streams, other host threads) race.  A
 * device-side failure (a bounded wait that expired) is not seen by the
 * returned status, which covers the launches only: it leaves NaN in *d_pe and
 * in the forces.  Runs on `stream` (a cudaStream_t, NULL for the default
 * stream) of the current device. */
#define MDGPU_NOALLOC_MAX_SITES 16384
#define MDGPU_NOALLOC_MAX_KVEC 8192
#define MDGPU_NOALLOC_SCRATCH_BYTES (6u << 20)
mdgpu_status mdgpu_ewald_kspace_noalloc(const double *h, int nsites, const double *d_site,
                                        const double *d_chg, double alpha, double k_cutoff,
                                        double *d_force, double *d_pe, double *d_stress,
                                        void *stream);

/* ---- Adjoint: parameter gradients.  No counterpart in the reference. -----
 *
 * The parameters are the potential table (max_id*max_id*MDGPU_NPOTP
 * doubles, the layout of mdgpu_system.potpar), the per-site charges
 * (nsites, program units) and the Ewald alpha; the cutoffs and the k-vector
 * list stay fixed.  Table entry [a][b] is the one the force on a site of
 * identifier a from a site of identifier b reads: for a symmetric table the
 * derivative with respect to a shared parameter p_ab = p_ba (a != b) is
 * grad[a][b][k] + grad[b][a][k].  Entries k beyond the potential type's
 * parameter count read 0.  The energy is pe[0] + pe[1] of mdgpu_forces; the
 * force-matching loss of reference forces f_ref is
 *    L = weight * sum_i |F_i - f_ref_i|^2
 * and its gradient sum_i 2 weight (F_i - f_ref_i) . dF_i/dtheta comes from
 * Hessian-vector products through the real-space pairs (their link-cell walk
 * recomputed, no stored pair list) and the k-space sum.  Both calls run the
 * forward evaluation first, in the context's precision.  A framework
 * molecule is handled as the forward path handles it: no framework-framework
 * terms, its net charge in the sheet term.  Limits: max_id <=
 * MDGPU_ADJ_MAX_ID; in strict-cutoff mode no molecule may be larger than the
 * cutoff (MDGPU_E_UNSUPPORTED otherwise). */
#define MDGPU_NPOTP 8
#define MDGPU_ADJ_MAX_ID 16
typedef struct {
   const double *potpar;        /* [max_id*max_id][8] or NULL: unchanged      */
   const double *chg;           /* [nsites] or NULL: unchanged                */
   double alpha;                /* > 0: new alpha; <= 0: unchanged            */
} mdgpu_params;

typedef struct {
   double *potpar;              /* out [max_id*max_id][8], or NULL            */
   double *chg;                 /* out [nsites], or NULL                      */
   double alpha;                /* out                                        */
} mdgpu_grad;

/* Replaces the parameters of the system and control record. */
mdgpu_status mdgpu_set_params(mdgpu_ctx *ctx, const mdgpu_params *params);

/* Energy and its gradient at params (NULL: the current ones) for the
 * configuration site_soa [3][nsites] (c_of_m as for mdgpu_forces). */
mdgpu_status mdgpu_energy_grad(mdgpu_ctx *ctx, const mdgpu_params *params, const double *h,
                               const double *site_soa, const double *c_of_m, double *energy,
                               mdgpu_grad *grad);

/* Force-matching loss against f_ref_soa [3][nsites] and its gradient. */
mdgpu_status mdgpu_fm_loss_grad(mdgpu_ctx *ctx, const mdgpu_params *params, const double *h,
                                const double *site_soa, const double *c_of_m,
                                const double *f_ref_soa, double weight, double *loss,
                                mdgpu_grad *grad);

/* ---- Rigid-molecule dynamics on the GPU.  No counterpart in the reference
 * as an entry point: the constant-energy step of do_step (src/accel.c:626-827,
 * thermostat and barostat off) with this library's forces, every step on
 * the device.  Per step: half drift of centres of mass (fractional
 * co-ordinates, periodic wrap) and quaternions (the reference's symplectic
 * rotational splitting, src/leapfrog.c:246-392), site co-ordinates, forces,
 * molecular forces and principal-frame torques, two half kicks with the
 * kinetic energy between them, half drift.  State layout is the
 * reference's: c_of_m and mom [nmols][3] (fractional centres of mass and
 * scaled momenta h^T h m ds/dt), quat and amom [nmols_r][4] for the
 * molecules of rotating species in species order (amom[0] unused, [1..3]
 * principal angular momenta).  A framework molecule (rdof 0) is held fixed
 * as do_step holds it: its momentum is zeroed after the kicks
 * (src/accel.c:748-755).  The Nose-Poincare thermostat of const-temp runs
 * (mdgpu_md_set_thermostat) and the Parrinello-Rahman cell dynamics of
 * const-pressure runs (mdgpu_md_set_barostat) are available. */
typedef struct {
   const double *mass;          /* [nspecies] molecular mass, amu             */
   const double *inertia;       /* [nspecies][3] principal moments of inertia */
   const int *rdof;             /* [nspecies] rotational degrees of freedom   */
   double step;                 /* timestep, ps                               */
   int nosymmetric_rot;         /* the nosymmetric-rot control key            */
} mdgpu_dynamics;

/* Loads the dynamic state (h as for mdgpu_forces; quat/amom may be NULL
 * when no species rotates). */
mdgpu_status mdgpu_md_init(mdgpu_ctx *ctx, const mdgpu_dynamics *dyn, const double *h,
                           const double *c_of_m, const double *mom, const double *quat,
                           const double *amom);

/* Advances nsteps steps.  energies ([nsteps][4], or NULL) receives per step
 * the real-space energy with the distant-potential correction (pe[0] of
 * eval_forces), the reciprocal-space energy (pe[1]) and the translational
 * and rotational kinetic energies at the half kick (the point where do_step
 * evaluates its conserved quantity).  MDGPU_E_RANGE if a site left the
 * cell or a quaternion lost its normalisation (QNORM2). */
mdgpu_status mdgpu_md_run(mdgpu_ctx *ctx, int nsteps, double *energies);

/* Replaces the dynamic state (same layout as mdgpu_md_init; any pointer may
 * be NULL to keep that part), e.g. after a host-side velocity rescaling.
 * Cheaper than mdgpu_md_init: the tables and the captured step stay. */
mdgpu_status mdgpu_md_set_state(mdgpu_ctx *ctx, const double *c_of_m, const double *mom,
                                const double *quat, const double *amom);

/* Copies the current state back (any pointer may be NULL). */
mdgpu_status mdgpu_md_get_state(mdgpu_ctx *ctx, double *c_of_m, double *mom, double *quat,
                                double *amom);

/* Constant temperature: the steps of mdgpu_md_run then integrate the
 * Nose-Poincare thermostat as do_step does under const-temp 1
 * (src/accel.c:673-684, 696-700, 757-791; leapf_nose_therm,
 * src/leapfrog.c:465-472; the thermostat momentum terms of leapf_quat,
 * src/leapfrog.c:308-329, 365-386): positions, rotations and kicks scaled
 * by the thermostat variable s, its momentum driven by the kinetic
 * energies, the potential energy and d_of_f kB temp (d_of_f as start_up
 * counts it from the species of mdgpu_md_init).  temp in K, ttmass the
 * thermostat mass in program units (the reference's control.ttmass after
 * its unit conversion), ts and tsmom the variable and momentum to start
 * from (the reference's start: 1 and 0).  H_0 is evaluated on the first
 * step after this call, as do_step evaluates it on a run's first step.
 * enable 0 returns to constant energy.  Call after mdgpu_md_init.  The
 * energy records then hold the kinetic energies divided by s^2 (trans_ke,
 * rot_ke). */
mdgpu_status mdgpu_md_set_thermostat(mdgpu_ctx *ctx, int enable, double temp, double ttmass, double ts,
                                     double tsmom);

/* out[3] = ts, tsmom, H_0 after the last step. */
mdgpu_status mdgpu_md_get_thermostat(mdgpu_ctx *ctx, double *out);

/* Constant pressure: the steps of mdgpu_md_run then integrate the
 * Parrinello-Rahman cell dynamics as do_step does under const-pressure
 * (src/accel.c:686-704, 759-783; gleap_cell and update_hmom,
 * src/leapfrog.c:474-535): mode 1 anisotropic, 2 uniform dilation (the
 * reference's const-pressure 1 and 2), pressure and pmass (the cell mass W)
 * in program units as the reference's control record holds them after its
 * unit conversion, strain_mask its strain-mask (bit 3i+j set: element (i,j)
 * of h held fixed; the reference's default 200 keeps h upper triangular, as
 * the force path needs), hmom the cell momentum to start from ([3][3]
 * row-major, NULL for zero).  The kinetic and virial stress are reduced on
 * the device each step and h advances on the host, so each step runs its
 * launches directly and the force path rebuilds its cell grid and k-vector
 * list for the new h.  Combines with the thermostat.  H_0 (with the cell's
 * kinetic energy and pressure x volume terms) is evaluated on the next step.
 * mode 0 returns to constant volume; MDGPU_E_UNSUPPORTED with molecular
 * cut-offs.  Call after mdgpu_md_init. */
mdgpu_status mdgpu_md_set_barostat(mdgpu_ctx *ctx, int mode, double pressure, double pmass, int strain_mask,
                                   const double *hmom);

/* The current cell h and its momentum ([3][3] each, row-major; either may be
 * NULL). */
mdgpu_status mdgpu_md_get_barostat(mdgpu_ctx *ctx, double *h, double *hmom);

/* ---- Dump records (the periodic dump of do_step, src/accel.c:811-820,
 * and its conversion, dump_convert, src/dump.c:550-620).  A record is
 * FP32 and its contents follow the bits of dump_level:
 *   bit 0: Cartesian centres of mass h s [nmols][3], quaternions
 *          [nmols_r][4], h [3][3], thermostat variable ts (1 here), total
 *          potential energy pe[0] + pe[1];
 *   bit 1: centre-of-mass velocities [nmols][3], principal angular
 *          velocities [nmols_r][3], h momentum [3][3] and thermostat
 *          momentum (both 0 here);
 *   bit 3: molecular forces [nmols][3], principal-frame torques
 *          [nmols_r][3], the virial stress [3][3] of eval_forces (site
 *          virial, molecular correction, distant-pressure term).
 * Size in floats: mdgpu_dump_size (DUMP_SIZE, src/defs.h:294-297). */
int mdgpu_dump_size(int dump_level, int nmols, int nmols_r);

/* Advances nsteps steps as mdgpu_md_run and, after step k (1-based) with
 * k >= first and (k - first) % interval == 0, converts the state into the
 * next record of records ([nrec][mdgpu_dump_size] floats, caller-owned,
 * nrec the number of such steps).  The conversion runs on the device; the
 * records are copied back in batches. */
mdgpu_status mdgpu_md_run_dump(mdgpu_ctx *ctx, int nsteps, int first, int interval, int dump_level,
                               double *energies, float *records);

/* ---- Dump files (src/dump.c).  A sequence of files named from a template
 * holding a printf integer conversion (the file number; "%d" is appended
 * when there is none), each a header (dump_mt), the system description
 * (dump_sysinfo_mt with one mol_mt per species) and up to maxdumps records;
 * the header's record count is rewritten after every record, as dump()
 * does.  Native files are the struct images of an LP64 build of the
 * reference; XDR files are its big-endian XDR encoding (src/xdr.c:150-183),
 * with "(XDR)" after the version.  A file that exists already is not
 * overwritten (MDGPU_E_IO): the reference would try other names. */
typedef struct {                /* mol_mt, src/structs.h:220-230              */
   float inertia[3];
   float mass;
   float dipole;                /* |sum of q p| over the principal-frame sites */
   float charge;                /* molecular charge                           */
   int nmols, rdof, framework;
   char name[32];
} mdgpu_dump_species;

typedef struct {
   const char *title;           /* run title (up to 127 characters)           */
   long istep;                  /* step of the first record                   */
   long dump_interval;
   int dump_level;
   int maxdumps;                /* records per file                           */
   float deltat;                /* timestep * dump_interval                   */
   int nmols, nmols_r, nspecies;
   const mdgpu_dump_species *species;   /* [nspecies]                        */
   int xdr;                     /* 1: XDR encoding                            */
   unsigned long dump_init;     /* sequence stamp (0: the current time)       */
   unsigned long restart_timestamp;
} mdgpu_dump_info;

typedef struct mdgpu_dumpfile mdgpu_dumpfile;

/* Opens a sequence; *df is set even on failure (for mdgpu_dump_errmsg)
 * unless out of memory. */
mdgpu_status mdgpu_dump_open(mdgpu_dumpfile **df, const char *name_template, const mdgpu_dump_info *info);
/* Appends one record (mdgpu_dump_size floats), starting the next file of
 * the sequence when the current one holds maxdumps. */
mdgpu_status mdgpu_dump_append(mdgpu_dumpfile *df, const float *record);
/* Name of the file the last record went to. */
const char *mdgpu_dump_filename(const mdgpu_dumpfile *df);
const char *mdgpu_dump_errmsg(const mdgpu_dumpfile *df);
void mdgpu_dump_close(mdgpu_dumpfile *df);

/* Measures the device's dense FMA throughput (TFLOP/s, FMA = 2 flops):
 * mode 0 scalar FP32 (FFMA), 1 FP64 (DFMA), 2 FP32 as paired (f32x2)
 * instructions.  The roofline denominators of the force kernels, whose
 * bound is the FMA pipe.  No counterpart in the reference. */
mdgpu_status mdgpu_fma_peak(int device, int fp64, double *tflops);

/* Tensor-core operand probe: one 128 x n x 16 MMA pair (bf16, or fp16 if
 * flags & 8), D = A0 B0^T then (unless flags & 4) D += A1 B1^T (A1 negated
 * if flags & 2), FP32 accumulation, in the operand layout the
 * reciprocal-space tensor-core kernels use (flags & 1 exchanges the
 * descriptor's two offset fields).  a0, a1: 128 x 16 16-bit patterns,
 * row-major; b0, b1: n x 16; d: 128 x n.
 * n a multiple of 16 in 16..128.  No counterpart in the reference. */
mdgpu_status mdgpu_tc_probe(int device, const unsigned short *a0, const unsigned short *b0,
                            const unsigned short *a1, const unsigned short *b1, int n, int flags, float *d);
/* Tensor-core issue rate: in one CTA per SM (two if two_per_sm), issuers
 * threads issue reps 128 x n x 16 bf16 MMAs in all over nacc accumulators
 * each; bf16 TFLOP/s over the device.  n a multiple of 16 in 16..256,
 * issuers 1..4, issuers * nacc * n <= 512 (256 with two CTAs per SM).  No
 * counterpart in the reference. */
mdgpu_status mdgpu_tc_rate(int device, int n, int reps, int nacc, int issuers, int two_per_sm, double *tflops);

/* Potential at one distance (poteval, src/force.c:632-650): reference-site
 * charge 1, neighbour charge chgsq, Ewald alpha as given. */
double mdgpu_poteval(const double *potpar, double r, int ptype, double chgsq, double alpha);

/* The link-cell stencil for cell h (row-major) and the control values (host
 * only, no device needed): grid = (nx, ny, nz); half[3 i ..] = the
 * reference's half-space neighbour offsets (dx, dy, dz) in its order, the
 * zero offset included (*nhalf of them, the NABORS count); cols[5 c ..] =
 * the column walk's regrouping of the full stencil (the half-space offsets,
 * their mirrors and zero) into runs of consecutive dz, (dx, dy, dz0, len,
 * base) sorted by (dx, dy, dz0); coff[6 (base + t) ..] = the FP32 hi and lo
 * parts of the cell offset h (dx/nx, dy/ny, (dz0 + t)/nz) of each run's
 * t-th cell.  Any of half, cols, coff may be NULL; MDGPU_E_CAPACITY if a
 * list exceeds cap entries; MDGPU_E_CUTOFF as for the force call.  No
 * counterpart in the reference. */
mdgpu_status mdgpu_stencil_columns(const double *h, const mdgpu_control *ctl, int *grid, int *half, int *nhalf,
                                   int *cols, float *coff, int *ncols, int cap);

/* The tensor-core work items of the k-list for cell h (row-major) and the
 * control values (host only, no device needed): runs of up to 64 l values of
 * one (h, k) column, largest count first, padded with empty runs to a
 * multiple of 128.  items[4 i ..] = (h, k, l0, count); k0[4 i + r] = index of
 * the run's r-th 16 k-vectors in the k-list order the passes use (-1 past
 * its end).  *nitems and *nk (k-vectors) are set; MDGPU_E_CAPACITY if nitems
 * exceeds cap.  No counterpart in the reference. */
mdgpu_status mdgpu_tc_items(const double *h, const mdgpu_control *ctl, int *items, int *k0, int cap,
                            int *nitems, int *nk);

#ifdef __cplusplus
}
#endif
#endif
