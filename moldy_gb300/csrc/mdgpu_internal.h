// Internal declarations of libmoldy_gb300: the context, the host-side
// geometry (link-cell stencil, k-vector list) and the launch functions of
// the real-space (realspace.cu) and reciprocal-space (kspace.cu) kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/moldy_gb300.h"

namespace mdgpu {

constexpr int NPOTP = 8;          // parameters per potential (src/defs.h:144)
constexpr int KI = 16;            // k-vectors per k-space work item
constexpr int KT = 64;            // k-vectors per tensor-core structure-factor item (4 KI runs)
constexpr int FT_THREADS = 128;   // k_force32: threads per block, two sites each
constexpr double PI = 3.14159265358979323846;
constexpr double ALPHAMIN = 1e-7; // src/defs.h:181
constexpr double TOO_CLOSE = 0.25;// r^2 warning threshold, src/force.c:89
constexpr int MAX_TOO_CLOSE_REC = 16;

// ---- host-side geometry of one real-space call -------------------------
struct RsGeom {
   int nx = 0, ny = 0, nz = 0, ncells = 0;
   int n_half = 0;                 // half-space stencil (reference list)
   std::vector<int> half;          // 3 ints per offset, reference order
   std::vector<int4> full;         // (dx,dy,dz,is_zero) both half-spaces
   std::vector<float4> off_hi, off_lo;  // h.(d/n) as float hi + lo parts
   double h[9];
   double hinv[9];                 // src/matrix.c invert() of h
   double reloc[27][3];            // image translations, src/force.c:1282-1293
   double origin_step[9];          // h / n (column j scaled by 1/n_j)
   double cut2 = 0, cut100 = 0;
   double key[12];                 // h, cutoff, subcell, strict: cache key
   // The full stencil as columns: offsets of one (dx, dy) with consecutive
   // dz form one column (dx, dy, dz_min, length); col_base[i] indexes the
   // column's first entry in coff_hi/coff_lo, which hold the cell-offset
   // vectors of its dz values in order (FP32 hi + lo parts).  cols_ok: every
   // column is at most nz long (so it wraps the periodic cell at most once).
   std::vector<int4> cols;
   std::vector<int> col_base;
   std::vector<float4> coff_hi, coff_lo;
   bool cols_ok = false;
   // every offset of the 27-cell neighbourhood is in the stencil and each
   // cell is at least 0.5 A thick (any pair closer than the too-close
   // distance lies in neighbouring cells)
   bool nbr27 = false;
   int nbcol[9] = {0};             // column of each (dx, dy) in [-1, 1]^2 (when nbr27)
};

// Builds the stencil and cell geometry; returns MDGPU_E_CUTOFF as the
// reference's FATAL CUTOFF would fire.
mdgpu_status build_rs_geom(const double *h, const mdgpu_control &ctl, RsGeom &g);
mdgpu_status build_rdf_stencil(const double *h, double limit, int nx, int ny, int nz, std::vector<int4> &full);

// ---- host-side k-vector list ---------------------------------------------
struct KList {
   int hmax = 0, kmax = 0, lmax = 0, nk = 0, nitems = 0;
   std::vector<int4> item;         // (h, k, l0, count)
   std::vector<int> item_k0;       // index of the item's first k-vector
   std::vector<double2> item_kxy;  // (kx, ky) of the item's (h,k) column
   std::vector<double> kz;         // per k-vector
   double dkz = 0;                 // kz step from l to l + 1 (2 pi hinv[2][2])
   std::vector<double> coeff, coeff2;  // src/ewald.c:510-511
   double key[12];                 // h, k_cutoff, alpha
   double vol = 0;
   double hinv[9];
   // tensor-core structure factor: runs of up to KT l values of a column,
   // largest count first, padded with empty runs to a multiple of 128
   std::vector<int4> tc_item;      // (h, k, l0, count)
   std::vector<int4> tc_k0;        // first k index of each KI run of the item (-1 past its end)
   std::vector<float2> tc_kxy;     // (kx, ky) of the item's column
   int tc_nitems = 0;              // before padding
};

mdgpu_status build_klist(const double *h, const mdgpu_control &ctl, KList &kl);

// ---- first-call constants (host, FP64, reference arithmetic) -------------
double host_poteval(const double *potpar, double r, int ptype, double chgsq, double alpha);
double intramolecular_energy(const std::vector<mdgpu_species> &spec,
                             const std::vector<int> &spec_ids, const std::vector<double> &spec_pf,
                             const double *potpar, int max_id, int ptype,
                             const std::vector<double> &chg, double alpha);
void ewald_self_sheet(const std::vector<mdgpu_species> &spec, const std::vector<double> &spec_pf,
                      const std::vector<double> &chg, double alpha, double *self,
                      double *sheet, int *nsitesxf);
void ewald_self_sheet_grad(const std::vector<mdgpu_species> &spec, const std::vector<double> &spec_pf,
                           const std::vector<double> &chg, double alpha, double vol, double *g_chg,
                           double *g_alpha);
// Constant of the distant-potential correction (distant_const,
// src/accel.c:293-328 with dist_pot, src/kernel.c:103-150): energy x volume.
double distant_const(const mdgpu_ctx *c);
// The pressure form (iflag 1 of the same function, src/accel.c:316-320).
double distant_pconst(const mdgpu_ctx *c);
double det3(const double *a);
void inv3(const double *a, double *b);

// ---- device buffers ----------------------------------------------------------
// Owned by the context: freed by release() or when the context is deleted
// (on its device: mdgpu_destroy selects it first).
template <typename T>
struct DBuf {
   T *p = nullptr;
   size_t n = 0;
   DBuf() = default;
   DBuf(const DBuf &) = delete;
   DBuf &operator=(const DBuf &) = delete;
   ~DBuf() { release(); }
   cudaError_t ensure(size_t want) {
      if (want <= n && p) return cudaSuccess;
      if (p) cudaFree(p);
      p = nullptr;
      n = 0;
      cudaError_t e = cudaMalloc(&p, (want ? want : 1) * sizeof(T));
      if (e == cudaSuccess) n = want;
      return e;
   }
   void release() {
      if (p) cudaFree(p);
      p = nullptr;
      n = 0;
   }
};

// Device-resident outputs of one evaluation (all FP64).
struct DevOut {
   double pe_rs;          // sum of pair energies (before eintra)
   double vir_rs[6];      // xx xy xz yy yz zz
   double pe_k;           // sum of k-space energies (before self/sheet)
   double st_k[6];
   double vir_in[6];      // sum x_i (x) f_in_i, reference-semantics calls only
   int err;               // bit 0: co-ordinate out of range; bit 2: a
                          // structure-factor tile copy timed out
   int n_too_close;
   int64_t npairs2;       // full-list pair evaluations (2x reference count)
   int too_close[MAX_TOO_CLOSE_REC][2];
};

struct RsDev {
   DBuf<int> cell_of, cell_count, cell_start, slot_cell, sorted, blocksum;
   DBuf<double4> pos64;    // sorted: x, y, z, q
   DBuf<float4> pos32;     // sorted: x - cell origin (x, y, z), q
   DBuf<int2> tag;         // sorted: site id, molecule
   DBuf<int> molmap, siteid, ent_mol;
   DBuf<double> chg, cofm;
   DBuf<int4> full;
   DBuf<float4> off_hi, off_lo;
   DBuf<double> pot64;
   DBuf<float> pot32;
   DBuf<double> part;      // per-block partial energies/virials
   DBuf<double> part2;     // their first-level sums
   DBuf<unsigned long long> keys;
   DBuf<int4> rdf_full;    // RDF stencil (strict, at the RDF limit)
   // column walk of the mixed pair kernel (k_pairs_col): the stencil's
   // columns and their offsets; the slots re-laid class by class (class 0:
   // the sites that interact with charged sites; class 1: the rest), each
   // class in link-cell order, with per-class cell starts cs[2][ncells+1]
   DBuf<int4> cols;
   DBuf<int> col_base;
   DBuf<float4> coff;      // [e][2]: the column offsets' hi and lo parts side by side (32 B per entry)
   DBuf<int> cls_of_id, cls_pre, cs, sortc, cellc, cls_bsum;
   DBuf<float4> posc;
   DBuf<int2> tagc;
   DBuf<unsigned long long> rdf_counts;
   double rdf_key[11] = {0};
   int rdf_nfull = 0;
};

struct KsDev {
   DBuf<int4> item;
   DBuf<int> item_k0;
   DBuf<double2> item_kxy64;
   DBuf<float2> item_kxy32;
   DBuf<double> kz64, coeff, coeff2;
   DBuf<float4> kdat32;    // per k: (A_k, B_k, kz, 0)
   DBuf<double4> kdat64;
   DBuf<int4> ph32;        // per site: fixed-point phases (32-bit) + q bits
   DBuf<float2> z32;       // per site: exp(2 pi i s_z)
   DBuf<float2> zp32;      // per site: exp(2 pi i t s_z), t = 0..KI-1
   DBuf<ulonglong2> ph64a; // per site: (ux, uy) 64-bit phases
   DBuf<ulonglong2> ph64b; // per site: (uz, q bits)
   DBuf<double2> z64;
   DBuf<float2> part32;    // [chunks][nk] structure-factor partials
   DBuf<double2> part64;
   DBuf<double> fpart;     // [splits][3][N] force partials
   DBuf<double> blk;       // per-block energy/stress partials
   DBuf<double> blk2;      // their first-level sums
   DBuf<unsigned int> kcount;   // k_kfinal_part: blocks finished (the last one sums the slices)
   // framework molecule: framework-charge channel, its structure factor,
   // negated framework coefficients, its sites' records held compactly
   DBuf<int> fslot, sortedc;
   DBuf<int4> phf32, phc32;
   DBuf<ulonglong2> phf64b, pac64, pbc64;
   DBuf<float2> partf32, zpc32;
   DBuf<double2> partf64, zc64;
   DBuf<float4> kdatf32;
   DBuf<double4> kdatf64;
   DBuf<double> fpartf;
   // charged sites only (a site without charge adds nothing to S(k) and
   // gets no k-space force): their slots in link-cell order
   DBuf<int> kslots, kscan, kbsum;
   // tensor-core structure factor: its items and the per-site z tables as
   // split bf16 MMA operands (kspace_tc.cu)
   DBuf<int4> tc_item, tc_k0;
   DBuf<float2> tc_kxy;
   DBuf<uint4> ztab;       // structure factor: z tables as the B operand, per 16 sites
   DBuf<uint4> zsite;      // force pass: z tables as the A operand, per 128 sites
   DBuf<uint4> utab;       // force pass: per-item coefficient rows (B operand)
   DBuf<float4> tc_coef;   // per item: kx s1, ky s1, kz0 s1, dkz s2 (row scales s)
   DBuf<int> tc_ustart;    // force pass: the CTAs' work ranges (k_ftc_ranges)
   long long tc_ver = 0;   // uploads of tc_item so far
   int tc_rkey[3] = {-1, -1, -1};   // (site tiles, item tiles, CTAs) of tc_ustart
   long long tc_rver = -1;          // tc_ver of tc_ustart
};

// Buffers of the adjoint (parameter-gradient) passes.
struct AdjDev {
   DBuf<double4> res64;    // per slot: residual weight v of the site (FP64 form)
   DBuf<float4> res32;     // per slot: the same in FP32 (mixed form)
   DBuf<double> fref;      // [3][N] reference forces
   DBuf<double> gq;        // [2][N] dE/dq, dG/dq per site
   DBuf<double> gpart;     // per-block real-space gradient slots
   DBuf<double> slots;     // summed real-space slots
   DBuf<double> scal;      // loss, k-space dE/dalpha, dG/dalpha
   DBuf<double> lpart;     // per-block loss partials
   DBuf<int4> phv32;       // [3][N] mixed-form phases with weight q v_a
                           // ([6][N] with a framework: its sites' weights after)
   DBuf<ulonglong2> phv64; // [3][N] (u_z, weight q v_a) for the FP64 form
   DBuf<float2> partv32;   // [3][chunks][nk] weighted structure-factor partials
                           // ([6][chunks][nk] with a framework)
   DBuf<double2> partv64;
   DBuf<float4> kadj32;    // per k: A, B, P, Q
   DBuf<double4> kadj64;
   DBuf<float4> kadjf32;   // per k: the framework sites' A, B, P, Q, negated
   DBuf<double4> kadjf64;
   DBuf<float4> resc32;    // the framework sites' residual weights, compacted
   DBuf<double4> resc64;
   DBuf<double> gkpartf;   // [splits][2][nf] framework correction partials
   DBuf<float> kz32;       // per k: k_z
   DBuf<double> gkpart;    // [splits][2][N] k-space charge-gradient partials
   DBuf<double> blk;       // per-block k-space dE/dalpha, dG/dalpha
};

// Rigid-molecule dynamics (integrate.cu): one species' constants.
struct MdSpec {
   double mass;
   double inertia[3], rinertia[3];   // principal moments and their inverses
   int nsites, pf0;                  // sites per molecule, first principal-frame site
   int framework;                    // fixed framework: momentum zeroed after the kicks
};

struct MdHost {
   bool ready = false;
   std::vector<MdSpec> spec;
   double h[9];
   double half = 0;                  // dt / 2
   double dist = 0;                  // distant-potential constant (energy x volume)
   double distp = 0;                 // distant-pressure constant (stress x volume)
   int nosym = 0, saxis = 0, nmols_r = 0;
   // one captured step (CUDA graph), replayed by mdgpu_md_run
   cudaGraphExec_t graph = nullptr;
   uint64_t graph_gen = 0;
   int64_t graph_launches = 0;       // kernels one replay launches
   int graph_cap = 0;                // record capacity it was captured with
   uint64_t warm_gen = 0;            // configuration of the last direct step
   // constant temperature (mdgpu_md_set_thermostat)
   int d_of_f = 0;                   // degrees of freedom as start_up counts them
   bool therm = false;
   double temp = 0, ttmass = 0, gkt = 0, ahalf = 0;
   // constant pressure (mdgpu_md_set_barostat): mode 1 anisotropic, 2
   // uniform dilation; h (above) and its momentum advance on the host
   int baro = 0, strain_mask = 0;
   double pressure = 0, pmass = 0;
   double hmom[9] = {0};
   std::vector<double> kpart_h;      // host copies of block sums
};

struct MdDev {
   DBuf<double> cofm, mom, quat, amom;   // [nmols][3], [nmols][3], [nmols_r][4] x2
   DBuf<int> counter;                    // index of the next energy record
   DBuf<int> mol_spec, mol_q, mol_site0, site_mol, site_pf;
   DBuf<double> pf;                      // principal-frame sites of every species
   DBuf<MdSpec> spec;
   DBuf<double> kpart, energies;
   DBuf<int> err;
   DBuf<double> molf, molt;              // molecular forces, principal torques
   DBuf<double> vpart, virc;             // virial correction (dump records)
   DBuf<float> rec;                      // batch of dump records
   DBuf<double> therm;                   // s, its momentum, H_0, H_0 evaluated
   DBuf<double> tpart;                   // block sums of the thermostat momentum's increments
   DBuf<double> kdpart;                  // block sums of the kinetic stress (constant pressure)
};

}  // namespace mdgpu

struct mdgpu_ctx {
   int device = 0;
   int nsm = 0;        // multiprocessors of the device (read when first needed)
   cudaStream_t own_stream = nullptr, stream = nullptr;
   mdgpu_precision prec = MDGPU_MIXED;
   std::string err;

   // system
   bool have_system = false, have_control = false;
   int nsites = 0, nmols = 0, max_id = 0, ptype = 0;
   // the framework molecule (species flagged framework come last; the
   // reference supports one framework molecule, src/force.c:1218-1220):
   // its index, its first site and the count of molecules before it
   int fw_mol = -1, fw_site0 = 0, nmols_nf = 0;
   std::vector<mdgpu_species> spec;
   std::vector<int> spec_ids;       // concatenated per-species site ids
   std::vector<double> spec_pf;     // concatenated principal-frame sites
   std::vector<int> site_id, molmap, mol_first, mol_nsites;
   std::vector<double> chg, potpar;
   mdgpu_control ctl{};
   bool sys_dirty = true;           // device copies out of date

   // first-call constants (recomputed after set_system)
   bool have_eintra = false, have_self = false;
   double eintra = 0, self_energy = 0, sheet_energy = 0;
   int nsitesxf = 0;

   // cached geometry
   mdgpu::RsGeom rs;
   bool rs_valid = false, rs_uploaded = false;
   mdgpu::KList kl;
   bool kl_valid = false, kl_uploaded = false;
   bool npairs_pending = false;   // the last real-space pass left the pair count to rs_count_pairs
   int rs_nblk = 0;               // blocks (energy/virial partials) of the last real-space pass

   mdgpu::RsDev rd;
   mdgpu::KsDev kd;
   mdgpu::AdjDev ad;
   mdgpu::MdHost mdh;
   mdgpu::MdDev md;
   mdgpu::DBuf<double> site, force, force_in, cofm_in, small;
   const double *cur_site = nullptr;   // site array of the launch in progress
   std::vector<double> last_cofm;      // centres of mass of the last force_calc
   mdgpu::DBuf<mdgpu::DevOut> out;
   mdgpu::DevOut *h_out = nullptr;  // pinned mirror
   double *h_stage = nullptr;       // pinned staging for 6*nsites doubles
   size_t h_stage_n = 0;

   mdgpu_info info{};
   int64_t launches = 0;
   bool timing = false;
   // the k-space passes run over every site, not only the charged ones
   // (the adjoint's backward passes read every site's phases)
   bool ks_all_sites = false;
   // mixed form: structure factor on the tensor cores (MDGPU_KSPACE_TC=0
   // at context creation selects the CUDA-core pass)
   bool tc_sfac = true;
   uint64_t ncharged_gen = 0;       // configuration the count below is for
   int ncharged = 0;                // sites with a nonzero charge
   double qmax = 0;                 // and their largest |q|
   cudaEvent_t ev[MDGPU_NPHASES + 1] = {};
   // second (high-priority) stream: the k-space passes run on it beside
   // the pair kernel
   cudaStream_t side_stream = nullptr;
   cudaEvent_t ev_fork = nullptr, ev_pairs = nullptr, ev_join = nullptr;
   bool ev_marked[MDGPU_NPHASES + 1] = {};
   bool have_nabor_note = false;
   // interaction classes of the site identifiers (realspace.cu): class 0
   // holds the identifiers that interact with charged sites, class 1 the
   // rest; pairs across the classes add exactly nothing.  ncls 1 when
   // every identifier is in class 0.
   std::vector<int> cls_of_id;
   int ncls = 1;
   // bumped by every call that changes what a captured step would launch
   // (system, control, parameters, precision, stream, dynamics state)
   uint64_t gen = 1;
   int note_nx = 0, note_ny = 0, note_nz = 0, note_nabors = 0;
};

namespace mdgpu {
// realspace.cu
mdgpu_status rs_prepare(mdgpu_ctx *c);   // upload geometry/system tables
// cells_only: bin and order the sites (the k-space passes stream them in
// link-cell order) without the pair kernel.
// sorted_ready (or null): recorded on the stream once the link-cell order
// (c->rd.sorted) is complete, before the per-slot records.
mdgpu_status rs_launch(mdgpu_ctx *c, const double *d_site, const double *d_cofm,
                       double *d_force, bool cells_only, unsigned long long *d_keys,
                       int64_t key_cap, cudaEvent_t sorted_ready = nullptr);
// Real-space adjoint over the slots binned by the last rs_launch: gradients
// into c->ad.gq ([2][N], written) and c->ad.slots; residual weights from
// c->ad.res64/res32 when loss.
mdgpu_status rs_adjoint(mdgpu_ctx *c, bool loss);
// The pair kernel and its energy/virial reduction over the sites binned by
// the last rs_launch, on c->stream (rs_launch without cells_only runs both).
mdgpu_status rs_pairs(mdgpu_ctx *c, double *d_force, unsigned long long *d_keys, int64_t key_cap);
// The reference's evaluated pair count of the last real-space pass into
// c->info.npairs, when that pass left it out (the column walk); waits for
// the context's stream.
mdgpu_status rs_count_pairs(mdgpu_ctx *c);
int pot_nparams(int ptype);     // parameters the potential type reads
// Site-pair distance histogram of the sites binned by the last rs_launch:
// full-list counts [max_id][max_id][nbins] into c->rd.rdf_counts (zeroed
// first); each unordered pair appears once from each side.
mdgpu_status rs_rdf(mdgpu_ctx *c, double limit, int nbins);
// kspace.cu
mdgpu_status ks_prepare(mdgpu_ctx *c);
// join: an event the final force sum waits for (the pair kernel running on
// another stream writes d_force first), or null.
mdgpu_status ks_launch(mdgpu_ctx *c, const double *d_site, double *d_force, bool accumulate,
                       cudaEvent_t join = nullptr);
struct KsShape {
   int chunks, chunk, splits, per_split;
};
// Chunks of the structure-factor pass and k-splits of a per-site pass
// (ipt items per thread, spt sites per thread).
KsShape ks_shape(int N, int nitems, int ipt, int spt);
// Reciprocal-space passes on the tensor cores (kspace_tc.cu), mixed form:
// per-site operand tables (after k_prep); the structure factor into part32
// ([chunks][nk], returns the number of chunks); the force pass's per-item
// coefficient rows (after the per-k reduction); the force pass, F_slot * q
// into fpart[split][3][nsites] (returns the number of splits).
void ks_tables_tc(cudaStream_t st, int nsites, const KsDev &d);
int ks_sfac_tc(cudaStream_t st, int nsites, int nk, const KsDev &d, int ntiles, double qmax, int *err);
void ks_coef_tc(cudaStream_t st, const KsDev &d, int nitems_padded, float dkz);
int ks_force_tc(cudaStream_t st, int nsites, KsDev &d, int nitems_padded, int nsm, const double *chg,
                const int *slots, double *fpart, int *err);
int ks_force_tc_splits(int nsites);
cudaError_t ks_tc_init(int device);
size_t ks_tc_ztab_len(int nsites);
int ks_tc_chunks(int nsites);
size_t ks_tc_zsite_len(int nsites);
size_t ks_tc_utab_len(int nitems_padded);
cudaError_t ks_tc_init(int device);
size_t ks_tc_ztab_len(int nsites);
int ks_tc_chunks(int nsites);
// api.cu
mdgpu_status fail(mdgpu_ctx *c, mdgpu_status s, const std::string &msg);
mdgpu_status cuda_check(mdgpu_ctx *c, cudaError_t e, const char *what);
// Cell geometry, k-list and first-call constants current for h and the
// control record, device tables uploaded.
mdgpu_status ensure_ready(mdgpu_ctx *c, const double *h, bool need_rs, bool need_ks);
// Copies the device result record back, waits, reports device-side errors.
mdgpu_status sync_out(mdgpu_ctx *c);

// Marks the boundary before phase `i` (MDGPU_NPHASES marks the end).
inline void phase_mark(mdgpu_ctx *c, int i)
{
   if (!c->timing) return;
   if (!c->ev[i]) cudaEventCreate(&c->ev[i]);
   cudaEventRecord(c->ev[i], c->stream);
   c->ev_marked[i] = true;
}
}  // namespace mdgpu
