// libmoldy_gb300 C ABI: the status-returning mdgpu_* interface
// (include/moldy_gb300.h) and the drop-in entry points with the reference's
// own signatures (include/moldy_ref_abi.h).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/moldy_ref_abi.h"
#include "mdgpu_internal.h"

using namespace mdgpu;

namespace mdgpu {

mdgpu_status fail(mdgpu_ctx *c, mdgpu_status s, const std::string &msg)
{
   if (c) c->err = msg;
   return s;
}

mdgpu_status cuda_check(mdgpu_ctx *c, cudaError_t e, const char *what)
{
   if (e == cudaSuccess) return MDGPU_OK;
   std::string m = std::string(what) + ": " + cudaGetErrorString(e);
   return fail(c, e == cudaErrorMemoryAllocation ? MDGPU_E_NOMEM : MDGPU_E_CUDA, m);
}

// kJ/mol per program energy unit and elementary charges per program charge
// unit (src/defs.h:201-235), for the reference's log lines.
static const double CONV_E = 0.001 * 6.0221367e23 * 1.6605402e-27 * 1.0e4;
static const double CONV_Q = (4.07497263794495e-14 * 1.0e-3 * 1.05482230112e-05) / 1.60217733e-19;

__global__ void k_finalize(const DevOut *out, double eintra, double self, double sheet_v,
                           int has_ewald, double *pe_out, double *stress_out)
{
   if (threadIdx.x != 0) return;
   pe_out[0] = -eintra + out->pe_rs;
   pe_out[1] = has_ewald ? (-self + sheet_v) + out->pe_k : 0.0;
   const double *v = out->vir_rs, *s = out->st_k;
   const double d = has_ewald ? sheet_v : 0.0;
   const double e = has_ewald ? 1.0 : 0.0;
   stress_out[0] = v[0] + e * s[0] + d;
   stress_out[1] = v[1] + e * s[1];
   stress_out[2] = v[2] + e * s[2];
   stress_out[3] = 0.0;
   stress_out[4] = v[3] + e * s[3] + d;
   stress_out[5] = v[4] + e * s[4];
   stress_out[6] = 0.0;
   stress_out[7] = 0.0;
   stress_out[8] = v[5] + e * s[5] + d;
}

// f += f_in and sum_i x_i (x) f_in_i, the part of the reference's virial
// loop (src/force.c:973-981) that sees forces already in site_force.
__global__ void k_add_in(int N, const double *__restrict__ site, const double *__restrict__ fin,
                         double *__restrict__ f, double *__restrict__ part)
{
   __shared__ double red[6][8];
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   double v[6] = {0, 0, 0, 0, 0, 0};
   if (i < N) {
      double fx = fin[i], fy = fin[N + i], fz = fin[2 * N + i];
      double x = site[i], y = site[N + i], z = site[2 * N + i];
      f[i] += fx;
      f[N + i] += fy;
      f[2 * N + i] += fz;
      v[0] = x * fx; v[1] = y * fx; v[2] = z * fx; v[3] = y * fy; v[4] = z * fy; v[5] = z * fz;
   }
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   for (int k = 0; k < 6; k++) {
      double s = v[k];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) red[k][w] = s;
   }
   __syncthreads();
   if (threadIdx.x < 6) {
      double s = 0;
      for (int j = 0; j < (int)(blockDim.x >> 5); j++) s += red[threadIdx.x][j];
      part[blockIdx.x * 8 + threadIdx.x] = s;
   }
}

__global__ void k_sum_in(const double *__restrict__ part, int nb, DevOut *out)
{
   int k = threadIdx.x;
   if (k >= 6) return;
   double s = 0;
   for (int b = 0; b < nb; b++) s += part[b * 8 + k];
   out->vir_in[k] = s;
}

}  // namespace mdgpu

// ---------------------------------------------------------------- helpers
// The intramolecular correction force_calc subtracts (src/force.c:1170-1171).
// The FP64 form evaluates every intramolecular pair's energy and subtracts
// it, as the reference does; the mixed form leaves those energies out of the
// pair sum instead (same value, without an FP32 cancellation), so nothing is
// subtracted.
static double eintra_subtracted(const mdgpu_ctx *c)
{
   return c->prec == MDGPU_FP64 ? c->eintra : 0.0;
}

static bool same(const double *a, const double *b, int n)
{
   return std::memcmp(a, b, sizeof(double) * n) == 0;
}

static mdgpu_status check_h(mdgpu_ctx *c, const double *h)
{
   if (!h) return fail(c, MDGPU_E_ARG, "h is NULL");
   if (h[3] != 0.0 || h[6] != 0.0 || h[7] != 0.0)
      return fail(c, MDGPU_E_UNSUPPORTED,
                  "the cell matrix must be upper triangular (the reference's Ewald sum presumes it)");
   if (!(det3(h) > 0.0)) return fail(c, MDGPU_E_ARG, "the cell matrix is singular");
   return MDGPU_OK;
}

// Cell geometry and k-list for this h and control, rebuilt only when either
// changed; the first-call constants on first use after set_system.
mdgpu_status mdgpu::ensure_ready(mdgpu_ctx *c, const double *h, bool need_rs, bool need_ks)
{
   if (!c->have_system) return fail(c, MDGPU_E_ARG, "mdgpu_set_system has not been called");
   if (!c->have_control) return fail(c, MDGPU_E_ARG, "mdgpu_set_control has not been called");
   mdgpu_status s = check_h(c, h);
   if (s) return s;
   if (c->ptype < 0 || c->ptype > 6 || c->ptype == 5)
      return fail(c, MDGPU_E_PTYPE, "KERNEL called with unknown potential type " + std::to_string(c->ptype));
   double rkey[12];
   std::memcpy(rkey, h, 9 * sizeof(double));
   rkey[9] = c->ctl.cutoff;
   rkey[10] = c->ctl.subcell;
   rkey[11] = c->ctl.strict_cutoff;
   if (need_rs && (!c->rs_valid || !same(rkey, c->rs.key, 12))) {
      c->rs_valid = false;
      s = build_rs_geom(h, c->ctl, c->rs);
      if (s == MDGPU_E_CUTOFF)
         return fail(c, s, "Cutoff radius > 1 * cell dimension (neighbour cells beyond one image)");
      if (s) return fail(c, s, "invalid cell partition (check subcell and h)");
      std::memcpy(c->rs.key, rkey, sizeof rkey);
      c->rs_valid = true;
      c->rs_uploaded = false;
   }
   const bool ew = c->ctl.alpha > ALPHAMIN;
   if (need_ks && ew) {
      double kkey[12];
      std::memcpy(kkey, h, 9 * sizeof(double));
      kkey[9] = c->ctl.k_cutoff;
      kkey[10] = c->ctl.alpha;
      kkey[11] = 0;
      if (!c->kl_valid || !same(kkey, c->kl.key, 12)) {
         c->kl_valid = false;
         s = build_klist(h, c->ctl, c->kl);
         if (s) return fail(c, s, "k-vector list");
         std::memcpy(c->kl.key, kkey, sizeof kkey);
         c->kl_valid = true;
         c->kl_uploaded = false;
      }
      if (!c->have_self) {
         ewald_self_sheet(c->spec, c->spec_pf, c->chg, c->ctl.alpha, &c->self_energy,
                          &c->sheet_energy, &c->nsitesxf);
         c->have_self = true;
      }
   }
   if (need_rs && !c->have_eintra) {
      c->eintra = intramolecular_energy(c->spec, c->spec_ids, c->spec_pf, c->potpar.data(), c->max_id,
                                        c->ptype, c->chg, c->ctl.alpha);
      c->have_eintra = true;
   }
   cudaError_t e = cudaSetDevice(c->device);
   if (e != cudaSuccess) return cuda_check(c, e, "cudaSetDevice");
   const int N = c->nsites;
   if (c->site.ensure(3 * (size_t)N) || c->force.ensure(3 * (size_t)N) ||
       c->force_in.ensure(3 * (size_t)N) || c->cofm_in.ensure(3 * (size_t)c->nmols + 3) ||
       c->out.ensure(1))
      return fail(c, MDGPU_E_NOMEM, "device allocation failed");
   s = rs_prepare(c);
   if (s) return s;
   if (need_ks && ew) {
      s = ks_prepare(c);
      if (s) return s;
   }
   c->sys_dirty = false;
   return MDGPU_OK;
}

static void fill_info(mdgpu_ctx *c)
{
   const DevOut &o = *c->h_out;
   mdgpu_info &I = c->info;
   I.nx = c->rs.nx;
   I.ny = c->rs.ny;
   I.nz = c->rs.nz;
   I.n_nabors = c->rs.n_half;
   I.nkvec = c->kl_valid ? c->kl.nk : 0;
   I.hmax = c->kl.hmax;
   I.kmax = c->kl.kmax;
   I.lmax = c->kl.lmax;
   I.eintra = c->eintra;
   I.self_energy = c->self_energy;
   I.sheet_energy = c->sheet_energy;
   I.npairs = o.npairs2 / 2;
   I.n_too_close = o.n_too_close;
   for (int k = 0; k < MAX_TOO_CLOSE_REC; k++) {
      I.too_close[k][0] = o.too_close[k][0];
      I.too_close[k][1] = o.too_close[k][1];
   }
}

// Copies the device result record back and reports device-side errors.
mdgpu_status mdgpu::sync_out(mdgpu_ctx *c)
{
   cudaError_t e = cudaMemcpyAsync(c->h_out, c->out.p, sizeof(DevOut), cudaMemcpyDeviceToHost, c->stream);
   if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
   if (e != cudaSuccess) return cuda_check(c, e, "synchronise");
   fill_info(c);
   if (c->h_out->err & 1)
      return fail(c, MDGPU_E_RANGE, "Co-ordinate out of range in BIN (fill_cells)");
   if (c->h_out->err & 4)
      return fail(c, MDGPU_E_CUDA, "a structure-factor tile copy did not complete (bounded wait expired)");
   if (c->h_out->err & 8)
      return fail(c, MDGPU_E_CUDA, "a tensor-core structure-factor stage did not complete (bounded wait expired)");
   if (c->h_out->err & 16)
      return fail(c, MDGPU_E_CUDA, "a tensor-core force-pass stage did not complete (bounded wait expired)");
   return MDGPU_OK;
}

#define CKR(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_check(c, e_, #x); } while (0)

static mdgpu_status upload_sites(mdgpu_ctx *c, double *const site[3], const double *c_of_m)
{
   const size_t N = c->nsites;
   for (int k = 0; k < 3; k++)
      CKR(cudaMemcpyAsync(c->site.p + k * N, site[k], N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   if (c->ctl.molpbc) {
      if (!c_of_m) return fail(c, MDGPU_E_ARG, "molecular cutoff needs the centres of mass");
      c->last_cofm.assign(c_of_m, c_of_m + 3 * (size_t)c->nmols);
      CKR(cudaMemcpyAsync(c->cofm_in.p, c->last_cofm.data(), 3 * c->nmols * sizeof(double),
                          cudaMemcpyHostToDevice, c->stream));
   }
   return MDGPU_OK;
}

// ------------------------------------------------------------------ C ABI
extern "C" {

mdgpu_status mdgpu_create(mdgpu_ctx **out, int device, mdgpu_precision precision)
{
   if (!out) return MDGPU_E_ARG;
   *out = nullptr;
   if (precision != MDGPU_FP64 && precision != MDGPU_MIXED) return MDGPU_E_ARG;
   int n = 0;
   if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
      cudaGetLastError();
      return MDGPU_E_CUDA;
   }
   if (device < 0 || device >= n) return MDGPU_E_ARG;
   mdgpu_ctx *c = new mdgpu_ctx();
   int lo_pri = 0, hi_pri = 0;
   c->device = device;
   c->prec = precision;
   if (const char *v = getenv("MDGPU_KSPACE_TC")) c->tc_sfac = atoi(v) != 0;
   if (cudaSetDevice(device) != cudaSuccess ||
       cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
       cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri) != cudaSuccess ||
       cudaStreamCreateWithPriority(&c->side_stream, cudaStreamNonBlocking, hi_pri) != cudaSuccess ||
       cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&c->ev_pairs, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
       cudaMallocHost((void **)&c->h_out, sizeof(DevOut)) != cudaSuccess) {
      cudaGetLastError();
      if (c->ev_fork) cudaEventDestroy(c->ev_fork);
      if (c->ev_pairs) cudaEventDestroy(c->ev_pairs);
      if (c->ev_join) cudaEventDestroy(c->ev_join);
      if (c->side_stream) cudaStreamDestroy(c->side_stream);
      if (c->own_stream) cudaStreamDestroy(c->own_stream);
      delete c;
      return MDGPU_E_CUDA;
   }
   std::memset(c->h_out, 0, sizeof(DevOut));
   c->stream = c->own_stream;
   *out = c;
   return MDGPU_OK;
}

void mdgpu_destroy(mdgpu_ctx *c)
{
   if (!c) return;
   cudaSetDevice(c->device);
   cudaStreamSynchronize(c->stream);
   RsDev &r = c->rd;
   r.cell_of.release(); r.cell_count.release(); r.cell_start.release(); r.slot_cell.release();
   r.sorted.release(); r.blocksum.release(); r.pos64.release(); r.pos32.release(); r.tag.release();
   r.molmap.release(); r.siteid.release(); r.ent_mol.release(); r.chg.release(); r.cofm.release();
   r.full.release(); r.off_hi.release(); r.off_lo.release(); r.pot64.release(); r.pot32.release();
   r.part.release(); r.part2.release(); r.keys.release();
   KsDev &k = c->kd;
   k.item.release(); k.item_k0.release(); k.item_kxy64.release(); k.item_kxy32.release();
   k.kz64.release(); k.coeff.release(); k.coeff2.release(); k.kdat32.release(); k.kdat64.release();
   k.ph32.release(); k.z32.release(); k.zp32.release(); k.ph64a.release(); k.ph64b.release(); k.z64.release();
   k.part32.release(); k.part64.release(); k.fpart.release(); k.blk.release();
   AdjDev &a = c->ad;
   a.res64.release(); a.res32.release(); a.fref.release(); a.gq.release(); a.gpart.release();
   a.slots.release(); a.scal.release(); a.lpart.release(); a.phv32.release(); a.phv64.release();
   a.partv32.release(); a.partv64.release(); a.kadj32.release(); a.kadj64.release(); a.kz32.release();
   a.gkpart.release(); a.blk.release();
   c->site.release(); c->force.release(); c->force_in.release(); c->cofm_in.release(); c->out.release();
   c->small.release();
   if (c->mdh.graph) cudaGraphExecDestroy(c->mdh.graph);
   MdDev &m = c->md;
   m.cofm.release(); m.mom.release(); m.quat.release(); m.amom.release(); m.counter.release();
   m.mol_spec.release(); m.mol_q.release(); m.mol_site0.release(); m.site_mol.release(); m.site_pf.release();
   m.pf.release(); m.spec.release(); m.kpart.release(); m.energies.release(); m.err.release();
   m.molf.release(); m.molt.release(); m.vpart.release(); m.virc.release(); m.rec.release();
   if (c->h_out) cudaFreeHost(c->h_out);
   for (auto &e : c->ev)
      if (e) cudaEventDestroy(e);
   if (c->ev_fork) cudaEventDestroy(c->ev_fork);
   if (c->ev_pairs) cudaEventDestroy(c->ev_pairs);
   if (c->ev_join) cudaEventDestroy(c->ev_join);
   if (c->side_stream) cudaStreamDestroy(c->side_stream);
   if (c->own_stream) cudaStreamDestroy(c->own_stream);
   delete c;
}

const char *mdgpu_last_error(const mdgpu_ctx *c)
{
   return c ? c->err.c_str() : "no context";
}

mdgpu_status mdgpu_set_precision(mdgpu_ctx *c, mdgpu_precision p)
{
   if (!c || (p != MDGPU_FP64 && p != MDGPU_MIXED)) return MDGPU_E_ARG;
   c->prec = p;
   c->gen++;
   return MDGPU_OK;
}

mdgpu_status mdgpu_set_stream(mdgpu_ctx *c, void *stream)
{
   if (!c) return MDGPU_E_ARG;
   c->stream = stream ? (cudaStream_t)stream : c->own_stream;
   c->gen++;
   return MDGPU_OK;
}

mdgpu_status mdgpu_get_stream(mdgpu_ctx *c, void **stream)
{
   if (!c || !stream) return MDGPU_E_ARG;
   *stream = (void *)c->stream;
   return MDGPU_OK;
}

static mdgpu_status set_system_impl(mdgpu_ctx *c, const mdgpu_system *s, bool keep_constants)
{
   if (!c || !s || s->nspecies <= 0 || !s->species || s->max_id <= 0 || !s->potpar || !s->chg)
      return fail(c, MDGPU_E_ARG, "invalid system description");
   int nsites = 0, nmols = 0;
   for (int i = 0; i < s->nspecies; i++) {
      const mdgpu_species &sp = s->species[i];
      if (sp.nsites <= 0 || sp.nmols < 0 || !sp.site_id || !sp.p_f_sites)
         return fail(c, MDGPU_E_ARG, "invalid species description");
      for (int k = 0; k < sp.nsites; k++)
         if (sp.site_id[k] < 0 || sp.site_id[k] >= s->max_id)
            return fail(c, MDGPU_E_ARG, "site identifier out of range");
      nsites += sp.nsites * sp.nmols;
      nmols += sp.nmols;
   }
   if (nsites <= 0) return fail(c, MDGPU_E_ARG, "system has no sites");
   c->nsites = nsites;
   c->nmols = nmols;
   c->max_id = s->max_id;
   c->ptype = s->ptype;
   c->spec.assign(s->species, s->species + s->nspecies);
   c->spec_ids.clear();
   c->spec_pf.clear();
   c->site_id.resize(nsites);
   c->molmap.resize(nsites);
   c->mol_first.resize(nmols);
   c->mol_nsites.resize(nmols);
   int isite = 0, imol = 0;
   for (auto &sp : c->spec) {
      c->spec_ids.insert(c->spec_ids.end(), sp.site_id, sp.site_id + sp.nsites);
      c->spec_pf.insert(c->spec_pf.end(), sp.p_f_sites, sp.p_f_sites + 3 * sp.nsites);
      for (int m = 0; m < sp.nmols; m++, imol++) {
         c->mol_first[imol] = isite;
         c->mol_nsites[imol] = sp.nsites;
         for (int k = 0; k < sp.nsites; k++, isite++) {
            c->site_id[isite] = sp.site_id[k];
            c->molmap[isite] = imol;
         }
      }
   }
   // the species records must not point into caller memory after return
   size_t so = 0;
   for (auto &sp : c->spec) {
      sp.site_id = nullptr;
      sp.p_f_sites = nullptr;
      so += sp.nsites;
   }
   // frameworks: after every other species, one framework molecule at most
   c->fw_mol = -1;
   c->fw_site0 = nsites;
   c->nmols_nf = nmols;
   {
      int isite2 = 0, imol2 = 0, nfw = 0;
      bool seen_fw = false;
      for (const auto &sp : c->spec) {
         if (sp.framework) {
            if (!seen_fw) {
               c->fw_mol = imol2;
               c->fw_site0 = isite2;
               c->nmols_nf = imol2;
            }
            seen_fw = true;
            nfw += sp.nmols;
         } else if (seen_fw) {
            return fail(c, MDGPU_E_UNSUPPORTED, "framework species must come after all other species");
         }
         isite2 += sp.nsites * sp.nmols;
         imol2 += sp.nmols;
      }
      if (nfw > 1) return fail(c, MDGPU_E_UNSUPPORTED, "Multiple framework molecules are not supported");
   }
   c->chg.assign(s->chg, s->chg + nsites);
   c->potpar.assign(s->potpar, s->potpar + (size_t)s->max_id * s->max_id * NPOTP);
   c->have_system = true;
   c->gen++;
   c->sys_dirty = true;
   c->rs_uploaded = false;
   if (!keep_constants) {
      c->have_eintra = false;
      c->have_self = false;
   }
   return MDGPU_OK;
}

mdgpu_status mdgpu_set_system(mdgpu_ctx *c, const mdgpu_system *s)
{
   return set_system_impl(c, s, false);
}

mdgpu_status mdgpu_set_control(mdgpu_ctx *c, const mdgpu_control *ctl)
{
   if (!c || !ctl) return MDGPU_E_ARG;
   if (!(ctl->cutoff > 0.0)) return fail(c, MDGPU_E_ARG, "cutoff must be positive");
   if (ctl->alpha > ALPHAMIN && !(ctl->k_cutoff > 0.0))
      return fail(c, MDGPU_E_ARG, "k_cutoff must be positive when alpha > 1e-7");
   const bool eintra_changes = c->have_control && c->ctl.alpha != ctl->alpha;
   c->ctl = *ctl;
   c->have_control = true;
   c->gen++;
   if (eintra_changes) {
      c->have_eintra = false;
      c->have_self = false;
   }
   return MDGPU_OK;
}

mdgpu_status mdgpu_forces_device(mdgpu_ctx *c, const double *h, const double *d_site,
                                 const double *d_cofm, double *d_force, double *d_pe,
                                 double *d_stress)
{
   if (!c || !d_site || !d_force || !d_pe || !d_stress) return fail(c, MDGPU_E_ARG, "NULL argument");
   if (c->have_control && c->ctl.molpbc && !d_cofm)
      return fail(c, MDGPU_E_ARG, "molecular cutoff needs the centres of mass");
   mdgpu_status s = ensure_ready(c, h, true, true);
   if (s) return s;
   for (bool &m : c->ev_marked) m = false;
   CKR(cudaMemsetAsync(c->out.p, 0, sizeof(DevOut), c->stream));
   const bool ew = c->ctl.alpha > ALPHAMIN;
   // With Ewald, the k-space passes (FP32-pipe-bound) run on a second,
   // high-priority stream beside the pair kernel (latency- and integer-bound),
   // so their blocks fill the SMs as pair blocks retire; the k-space force
   // sum waits for the pair kernel's forces.  Phase timing keeps the order.
   const bool overlap = ew && !c->timing;
   // overlap: the fork event is recorded as soon as the link-cell order is
   // complete, so the per-slot records of the pair kernel are built beside
   // the first k-space passes
   s = rs_launch(c, d_site, d_cofm, d_force, overlap, nullptr, 0, overlap ? c->ev_fork : nullptr);
   if (s) return s;
   if (overlap) {
      cudaStream_t main = c->stream;
      CKR(cudaStreamWaitEvent(c->side_stream, c->ev_fork, 0));
      s = rs_pairs(c, d_force, nullptr, 0);
      if (s) return s;
      CKR(cudaEventRecord(c->ev_pairs, main));
      c->stream = c->side_stream;
      s = ks_launch(c, d_site, d_force, true, c->ev_pairs);
      c->stream = main;
      if (s) return s;
      CKR(cudaEventRecord(c->ev_join, c->side_stream));
      CKR(cudaStreamWaitEvent(main, c->ev_join, 0));
   } else if (ew) {
      s = ks_launch(c, d_site, d_force, true);
      if (s) return s;
   } else {
      phase_mark(c, MDGPU_PH_FINAL);
   }
   k_finalize<<<1, 32, 0, c->stream>>>(c->out.p, eintra_subtracted(c), c->self_energy,
                                       ew ? c->sheet_energy / c->kl.vol : 0.0, ew ? 1 : 0, d_pe, d_stress);
   CKR(cudaGetLastError());
   c->launches += 1;
   phase_mark(c, MDGPU_NPHASES);
   return MDGPU_OK;
}

mdgpu_status mdgpu_forces(mdgpu_ctx *c, const double *h, const double *site_soa, const double *c_of_m,
                          double *force_out, double *pe_out, double *stress_out)
{
   if (!c || !site_soa || !force_out || !pe_out || !stress_out) return fail(c, MDGPU_E_ARG, "NULL argument");
   mdgpu_status s = ensure_ready(c, h, true, true);
   if (s) return s;
   const size_t N = c->nsites;
   CKR(cudaMemcpyAsync(c->site.p, site_soa, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   if (c->ctl.molpbc) {
      if (!c_of_m) return fail(c, MDGPU_E_ARG, "molecular cutoff needs the centres of mass");
      CKR(cudaMemcpyAsync(c->cofm_in.p, c_of_m, 3 * c->nmols * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   }
   CKR(c->small.ensure(16));
   double *d_small = c->small.p;   // pe[2] then stress[9]
   s = mdgpu_forces_device(c, h, c->site.p, c->cofm_in.p, c->force.p, d_small, d_small + 2);
   if (s) return s;
   CKR(cudaMemcpyAsync(force_out, c->force.p, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
   double small[11];
   CKR(cudaMemcpyAsync(small, d_small, sizeof small, cudaMemcpyDeviceToHost, c->stream));
   s = sync_out(c);
   if (s) return s;
   pe_out[0] = small[0];
   pe_out[1] = small[1];
   std::memcpy(stress_out, small + 2, 9 * sizeof(double));
   return MDGPU_OK;
}

mdgpu_status mdgpu_force_calc(mdgpu_ctx *c, const double *h, double *const site[3],
                              double *const site_force[3], const double *c_of_m, double *pe,
                              double *stress)
{
   if (!c || !site || !site_force || !pe || !stress) return fail(c, MDGPU_E_ARG, "NULL argument");
   mdgpu_status s = ensure_ready(c, h, true, false);
   if (s) return s;
   const size_t N = c->nsites;
   s = upload_sites(c, site, c_of_m);
   if (s) return s;
   for (int k = 0; k < 3; k++)
      CKR(cudaMemcpyAsync(c->force_in.p + k * N, site_force[k], N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   CKR(cudaMemsetAsync(c->out.p, 0, sizeof(DevOut), c->stream));
   s = rs_launch(c, c->site.p, c->cofm_in.p, c->force.p, false, nullptr, 0, nullptr);
   if (s) return s;
   const int nb = (int)((N + 255) / 256);
   CKR(c->rd.part.ensure((size_t)nb * 8 > c->rd.part.n ? (size_t)nb * 8 : c->rd.part.n));
   k_add_in<<<nb, 256, 0, c->stream>>>((int)N, c->site.p, c->force_in.p, c->force.p, c->rd.part.p);
   k_sum_in<<<1, 32, 0, c->stream>>>(c->rd.part.p, nb, c->out.p);
   CKR(cudaGetLastError());
   for (int k = 0; k < 3; k++)
      CKR(cudaMemcpyAsync(site_force[k], c->force.p + k * N, N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
   s = sync_out(c);
   if (s) return s;
   const DevOut &o = *c->h_out;
   *pe -= eintra_subtracted(c);
   *pe += o.pe_rs;
   const int idx[6] = {0, 1, 2, 4, 5, 8};
   for (int k = 0; k < 6; k++) stress[idx[k]] += o.vir_rs[k] + o.vir_in[k];
   return MDGPU_OK;
}

mdgpu_status mdgpu_ewald(mdgpu_ctx *c, const double *h, double *const site[3],
                         double *const site_force[3], double *pe, double *stress)
{
   if (!c || !site || !site_force || !pe || !stress) return fail(c, MDGPU_E_ARG, "NULL argument");
   if (!c->have_control) return fail(c, MDGPU_E_ARG, "mdgpu_set_control has not been called");
   if (!(c->ctl.alpha > ALPHAMIN)) return MDGPU_OK;
   mdgpu_status s = ensure_ready(c, h, true, true);
   if (s) return s;
   const size_t N = c->nsites;
   for (int k = 0; k < 3; k++) {
      CKR(cudaMemcpyAsync(c->site.p + k * N, site[k], N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      CKR(cudaMemcpyAsync(c->force.p + k * N, site_force[k], N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   }
   if (c->ctl.molpbc) {   // binning by molecule: the centres of mass are on the host record only
      if (c->last_cofm.size() != 3 * (size_t)c->nmols)
         return fail(c, MDGPU_E_ARG, "molecular cutoff needs the centres of mass (call force_calc first)");
      CKR(cudaMemcpyAsync(c->cofm_in.p, c->last_cofm.data(), 3 * c->nmols * sizeof(double),
                          cudaMemcpyHostToDevice, c->stream));
   }
   CKR(cudaMemsetAsync(c->out.p, 0, sizeof(DevOut), c->stream));
   s = rs_launch(c, c->site.p, c->cofm_in.p, c->force.p, true, nullptr, 0, nullptr);
   if (s) return s;
   s = ks_launch(c, c->site.p, c->force.p, true);
   if (s) return s;
   for (int k = 0; k < 3; k++)
      CKR(cudaMemcpyAsync(site_force[k], c->force.p + k * N, N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
   s = sync_out(c);
   if (s) return s;
   const DevOut &o = *c->h_out;
   const double sv = c->sheet_energy / c->kl.vol;
   *pe -= c->self_energy;
   *pe += sv;
   for (int i = 0; i < 3; i++) stress[4 * i] += sv;
   *pe += o.pe_k;
   const int idx[6] = {0, 1, 2, 4, 5, 8};
   for (int k = 0; k < 6; k++) stress[idx[k]] += o.st_k[k];
   return MDGPU_OK;
}

// Unordered per-type-pair counts from the full-list counts of rs_rdf.
static void rdf_unordered(const std::vector<unsigned long long> &full, int M, int nbins, uint64_t *out)
{
   for (int a = 0; a < M; a++)
      for (int b = 0; b < M; b++)
         for (int k = 0; k < nbins; k++) {
            const size_t ab = ((size_t)a * M + b) * nbins + k, ba = ((size_t)b * M + a) * nbins + k;
            out[ab] = a == b ? full[ab] / 2 : (full[ab] + full[ba]) / 2;
         }
}

static mdgpu_status rdf_download(mdgpu_ctx *c, int nbins, std::vector<unsigned long long> &full)
{
   full.resize((size_t)c->max_id * c->max_id * nbins);
   CKR(cudaMemcpyAsync(full.data(), c->rd.rdf_counts.p, full.size() * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, c->stream));
   return sync_out(c);
}

mdgpu_status mdgpu_rdf_counts(mdgpu_ctx *c, const double *h, const double *site_soa, const double *c_of_m,
                              double limit, int nbins, uint64_t *counts)
{
   if (!c || !site_soa || !counts) return fail(c, MDGPU_E_ARG, "NULL argument");
   mdgpu_status s = ensure_ready(c, h, true, false);
   if (s) return s;
   const size_t N = c->nsites;
   CKR(cudaMemcpyAsync(c->site.p, site_soa, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   if (c->ctl.molpbc) {
      if (!c_of_m) return fail(c, MDGPU_E_ARG, "molecular cutoff needs the centres of mass");
      CKR(cudaMemcpyAsync(c->cofm_in.p, c_of_m, 3 * c->nmols * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   }
   CKR(cudaMemsetAsync(c->out.p, 0, sizeof(DevOut), c->stream));
   if ((s = rs_launch(c, c->site.p, c->cofm_in.p, c->force.p, true, nullptr, 0, nullptr)) != MDGPU_OK) return s;
   if ((s = rs_rdf(c, limit, nbins)) != MDGPU_OK) return s;
   std::vector<unsigned long long> full;
   if ((s = rdf_download(c, nbins, full)) != MDGPU_OK) return s;
   rdf_unordered(full, c->max_id, nbins, counts);
   return MDGPU_OK;
}

mdgpu_status mdgpu_synchronize(mdgpu_ctx *c)
{
   if (!c) return MDGPU_E_ARG;
   return sync_out(c);
}

mdgpu_status mdgpu_get_info(mdgpu_ctx *c, mdgpu_info *info)
{
   if (!c || !info) return MDGPU_E_ARG;
   if (c->npairs_pending) {
      cudaSetDevice(c->device);
      const mdgpu_status s = rs_count_pairs(c);
      if (s != MDGPU_OK) return s;
   }
   *info = c->info;
   info->launches = c->launches;
   return MDGPU_OK;
}

mdgpu_status mdgpu_set_phase_timing(mdgpu_ctx *c, int enable)
{
   if (!c) return MDGPU_E_ARG;
   c->timing = enable != 0;
   return MDGPU_OK;
}

mdgpu_status mdgpu_phase_times(mdgpu_ctx *c, double *ms)
{
   if (!c || !ms) return MDGPU_E_ARG;
   for (int i = 0; i < MDGPU_NPHASES; i++) ms[i] = 0.0;
   if (!c->ev_marked[MDGPU_NPHASES]) return fail(c, MDGPU_E_ARG, "no timed evaluation recorded");
   CKR(cudaEventSynchronize(c->ev[MDGPU_NPHASES]));
   for (int i = 0; i < MDGPU_NPHASES; i++) {
      if (!c->ev_marked[i]) continue;
      int j = i + 1;
      while (j < MDGPU_NPHASES && !c->ev_marked[j]) j++;
      float t = 0.f;
      CKR(cudaEventElapsedTime(&t, c->ev[i], c->ev[j]));
      ms[i] = t;
   }
   return MDGPU_OK;
}

mdgpu_status mdgpu_pair_keys(mdgpu_ctx *c, const double *h, const double *site_soa, const double *c_of_m,
                             uint64_t *keys, int64_t cap, int64_t *count)
{
   if (!c || !site_soa || !keys || !count || cap < 0) return fail(c, MDGPU_E_ARG, "NULL argument");
   mdgpu_status s = ensure_ready(c, h, true, false);
   if (s) return s;
   const size_t N = c->nsites;
   CKR(cudaMemcpyAsync(c->site.p, site_soa, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   if (c->ctl.molpbc) {
      if (!c_of_m) return fail(c, MDGPU_E_ARG, "molecular cutoff needs the centres of mass");
      CKR(cudaMemcpyAsync(c->cofm_in.p, c_of_m, 3 * c->nmols * sizeof(double), cudaMemcpyHostToDevice, c->stream));
   }
   CKR(c->rd.keys.ensure(cap > 0 ? (size_t)cap : 1));
   CKR(cudaMemsetAsync(c->out.p, 0, sizeof(DevOut), c->stream));
   s = rs_launch(c, c->site.p, c->cofm_in.p, c->force.p, false, c->rd.keys.p, cap, nullptr);
   if (s) return s;
   s = sync_out(c);
   if (s) return s;
   const int64_t n = c->h_out->npairs2;   // counts canonical pairs in this mode
   *count = n;
   c->info.npairs = n;
   const int64_t ncopy = n < cap ? n : cap;
   if (ncopy > 0)
      CKR(cudaMemcpy(keys, c->rd.keys.p, ncopy * sizeof(uint64_t), cudaMemcpyDeviceToHost));
   return n > cap ? fail(c, MDGPU_E_CAPACITY, "pair key buffer too small") : MDGPU_OK;
}

double mdgpu_poteval(const double *potpar, double r, int ptype, double chgsq, double alpha)
{
   return host_poteval(potpar, r, ptype, chgsq, alpha);
}

mdgpu_status mdgpu_tc_items(const double *h, const mdgpu_control *ctl, int *items, int *k0, int cap,
                            int *nitems, int *nk)
{
   if (!h || !ctl || !nitems || !nk || cap < 0) return MDGPU_E_ARG;
   KList kl;
   mdgpu_status s = build_klist(h, *ctl, kl);
   if (s) return s;
   const int n = (int)kl.tc_item.size();
   *nitems = n;
   *nk = kl.nk;
   if (n > cap) return MDGPU_E_CAPACITY;
   for (int i = 0; i < n; i++) {
      if (items) {
         items[4 * i] = kl.tc_item[i].x;
         items[4 * i + 1] = kl.tc_item[i].y;
         items[4 * i + 2] = kl.tc_item[i].z;
         items[4 * i + 3] = kl.tc_item[i].w;
      }
      if (k0) {
         k0[4 * i] = kl.tc_k0[i].x;
         k0[4 * i + 1] = kl.tc_k0[i].y;
         k0[4 * i + 2] = kl.tc_k0[i].z;
         k0[4 * i + 3] = kl.tc_k0[i].w;
      }
   }
   return MDGPU_OK;
}

mdgpu_status mdgpu_stencil_columns(const double *h, const mdgpu_control *ctl, int *grid, int *half, int *nhalf,
                                   int *cols, float *coff, int *ncols, int cap)
{
   if (!h || !ctl || !grid || !nhalf || !ncols || cap < 0) return MDGPU_E_ARG;
   RsGeom g;
   mdgpu_status s = build_rs_geom(h, *ctl, g);
   if (s) return s;
   grid[0] = g.nx;
   grid[1] = g.ny;
   grid[2] = g.nz;
   *nhalf = g.n_half;
   *ncols = (int)g.cols.size();
   if (g.n_half > cap || (int)g.cols.size() > cap || (int)g.coff_hi.size() > cap) return MDGPU_E_CAPACITY;
   if (half)
      for (int i = 0; i < 3 * g.n_half; i++) half[i] = g.half[i];
   for (size_t i = 0; i < g.cols.size(); i++)
      if (cols) {
         cols[5 * i] = g.cols[i].x;
         cols[5 * i + 1] = g.cols[i].y;
         cols[5 * i + 2] = g.cols[i].z;
         cols[5 * i + 3] = g.cols[i].w;
         cols[5 * i + 4] = g.col_base[i];
      }
   if (coff)
      for (size_t e = 0; e < g.coff_hi.size(); e++) {
         const float4 a = g.coff_hi[e], b = g.coff_lo[e];
         const float v[6] = {a.x, a.y, a.z, b.x, b.y, b.z};
         for (int r = 0; r < 6; r++) coff[6 * e + r] = v[r];
      }
   return MDGPU_OK;
}

// ------------------------------------------------ reference signatures
// The caller's globals and log functions (src/main.c:83-84,
// src/output.c:131-190), bound if the executable defines them.
extern contr_mt control __attribute__((weak));
extern int nthreads __attribute__((weak));
void note(char *, ...) __attribute__((weak));
void *rdf_ptr(int *size) __attribute__((weak));   // src/rdf.c:58-62
void message(int *, ...) __attribute__((weak));

}  // extern "C"

namespace {

mdgpu_ctx *g_ctx = nullptr;
bool g_first_rs = true, g_first_ew = true;
int g_onx = 0, g_ony = 0, g_onz = 0, g_onabor = 0;

[[noreturn]] void ref_fatal(const char *fmt, ...)
{
   char buf[512];
   va_list ap;
   va_start(ap, fmt);
   std::vsnprintf(buf, sizeof buf, fmt, ap);
   va_end(ap);
   if (&control != nullptr && &message != nullptr) message(nullptr, nullptr, 3, (char *)"%s", buf);   // FATAL exits
   std::printf(" *F* %s\n", buf);
   std::fflush(stdout);
   std::exit(3);
}

void ref_note(const char *fmt, ...)
{
   char buf[512];
   va_list ap;
   va_start(ap, fmt);
   std::vsnprintf(buf, sizeof buf, fmt, ap);
   va_end(ap);
   if (&control != nullptr && &note != nullptr)
      note((char *)"%s", buf);
   else
      std::printf(" *I* %s\n", buf);
}

// message(..., INFO, ...) of the reference (src/output.c:131-168)
void ref_info(const char *fmt, ...)
{
   char buf[512];
   va_list ap;
   va_start(ap, fmt);
   std::vsnprintf(buf, sizeof buf, fmt, ap);
   va_end(ap);
   if (&control != nullptr && &message != nullptr)
      message(nullptr, nullptr, 0, (char *)"%s", buf);
   else
      std::printf(" *I* %s\n", buf);
}

void ref_warn(const char *fmt, ...)
{
   char buf[512];
   va_list ap;
   va_start(ap, fmt);
   std::vsnprintf(buf, sizeof buf, fmt, ap);
   va_end(ap);
   if (&control != nullptr && &message != nullptr)
      message(nullptr, nullptr, 1, (char *)"%s", buf);
   else
      std::printf(" *W* %s\n", buf);
}

mdgpu_ctx *ref_ctx()
{
   if (g_ctx) return g_ctx;
   const char *pe = std::getenv("MDGPU_PRECISION");
   mdgpu_precision prec = (pe && std::strcmp(pe, "fp64") == 0) ? MDGPU_FP64 : MDGPU_MIXED;
   const char *de = std::getenv("MDGPU_DEVICE");
   int dev = de ? std::atoi(de) : 0;
   if (mdgpu_create(&g_ctx, dev, prec) != MDGPU_OK)
      ref_fatal("moldy_gb300: no usable CUDA device %d for the GPU force path", dev);
   return g_ctx;
}

// Maps the reference's structs onto the mdgpu description; the context's
// system is replaced only when something in it changed.  First-call
// constants are kept, as the reference keeps them in statics.
void ref_sync(mdgpu_ctx *c, system_mt *system, spec_mt *species, real *chg, pot_mt *potpar, double *h)
{
   if (&control == nullptr) ref_fatal("moldy_gb300: the calling program defines no 'control' record");
   if (&nthreads != nullptr && nthreads != 1)
      ref_fatal("moldy_gb300: the GPU force path runs in one process (nthreads=%d)", nthreads);
   for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) h[3 * i + j] = system->h[i][j];
   const int ns = system->nspecies, max_id = system->max_id;
   std::vector<mdgpu_species> sp(ns);
   int nsites = 0;
   for (int s = 0; s < ns; s++) {
      sp[s].nsites = species[s].nsites;
      sp[s].nmols = species[s].nmols;
      sp[s].framework = species[s].framework;
      sp[s].site_id = species[s].site_id;
      sp[s].p_f_sites = &species[s].p_f_sites[0][0];
      nsites += species[s].nsites * species[s].nmols;
   }
   if (nsites != system->nsites) ref_fatal("moldy_gb300: species table does not add up to nsites");
   // ewald() receives no potential table: keep the one force_calc supplied
   std::vector<double> pot((size_t)max_id * max_id * NPOTP, 0.0);
   if (potpar) {
      for (int i = 0; i < max_id * max_id; i++)
         for (int k = 0; k < NPOTP; k++) pot[(size_t)i * NPOTP + k] = potpar[i].p[k];
   } else if (c->have_system && c->max_id == max_id) {
      pot = c->potpar;
   }
   bool changed = !c->have_system || c->nsites != nsites || c->max_id != max_id ||
                  c->ptype != system->ptype || (int)c->spec.size() != ns ||
                  std::memcmp(c->chg.data(), chg, nsites * sizeof(double)) != 0 ||
                  std::memcmp(c->potpar.data(), pot.data(), pot.size() * sizeof(double)) != 0;
   if (!changed) {
      size_t so = 0;
      for (int s = 0; s < ns && !changed; s++) {
         changed = c->spec[s].nsites != sp[s].nsites || c->spec[s].nmols != sp[s].nmols ||
                   c->spec[s].framework != sp[s].framework ||
                   std::memcmp(c->spec_ids.data() + so, sp[s].site_id, sp[s].nsites * sizeof(int)) != 0 ||
                   std::memcmp(c->spec_pf.data() + 3 * so, sp[s].p_f_sites, 3 * sp[s].nsites * sizeof(double)) != 0;
         so += sp[s].nsites;
      }
   }
   if (changed) {
      mdgpu_system d{ns, sp.data(), max_id, system->ptype, pot.data(), chg};
      if (set_system_impl(c, &d, true) != MDGPU_OK) ref_fatal("moldy_gb300: %s", c->err.c_str());
   }
   mdgpu_control ctl{control.cutoff, control.subcell, control.alpha, control.k_cutoff,
                     control.strict_cutoff, control.molpbc};
   if (!c->have_control || std::memcmp(&ctl, &c->ctl, sizeof ctl) != 0) {
      c->ctl = ctl;
      c->have_control = true;
   }
}

void ref_check(mdgpu_ctx *c, mdgpu_status s)
{
   if (s == MDGPU_OK) return;
   if (s == MDGPU_E_PTYPE) ref_fatal("KERNEL called with unknown potential type %d", c->ptype);
   if (s == MDGPU_E_CUTOFF)
      ref_fatal("Cutoff radius > %d * cell dimension.\n  -  Increase table size IMCELL_XTRA in \"force.c\"", 1);
   ref_fatal("moldy_gb300: %s", c->err.c_str());
}

}  // namespace

extern "C" {

// Adds this configuration's pair counts into the caller's RDF histogram the
// way rdf_accum does (src/rdf.c:94-107): each counted pair adds 1/density to
// a float bin, evaluated as (float)((double)bin + 1/density).  Every addend
// of a bin is the same, so repeating the addition count times gives the
// reference's value whatever order its pairs came in.
static void ref_rdf_accumulate(mdgpu_ctx *c, system_mt *system)
{
   const int nbins = control.nbins, M = c->max_id;
   mdgpu_status s = rs_rdf(c, control.limit, nbins);
   std::vector<unsigned long long> full;
   if (s == MDGPU_OK) s = rdf_download(c, nbins, full);
   ref_check(c, s);
   std::vector<uint64_t> cnt(full.size());
   rdf_unordered(full, M, nbins, cnt.data());
   int size = 0;
   float *base = (float *)rdf_ptr(&size);
   const double hm[9] = {system->h[0][0], system->h[0][1], system->h[0][2], system->h[1][0], system->h[1][1],
                         system->h[1][2], system->h[2][0], system->h[2][1], system->h[2][2]};
   const double density = system->nsites / det3(hm);
   const double invrho = 1.0 / density;
   float *bin = base;
   for (int a = 1; a < M; a++)          // init_rdf's layout, src/rdf.c:71-91
      for (int b = a; b < M; b++, bin += nbins) {
         if (bin + nbins > base + size) ref_fatal("moldy_gb300: RDF array smaller than expected");
         for (int k = 0; k < nbins; k++) {
            float v = bin[k];
            for (uint64_t n = cnt[((size_t)a * M + b) * nbins + k]; n > 0; n--) v = (float)((double)v + invrho);
            bin[k] = v;
         }
      }
}

void force_calc(real **site, real **site_force, system_mt *system, spec_mt *species, real *chg,
                pot_mt *potpar, double *pe, mat_mt stress)
{
   mdgpu_ctx *c = ref_ctx();
   double h[9];
   ref_sync(c, system, species, chg, potpar, h);
   // force_calc also accumulates the radial distribution function on RDF
   // steps (src/force.c:1302-1313): the histogram is taken on the GPU over
   // the cells this call binned and added into the caller's rdf array
   const bool rdf_step = control.rdf_interval > 0 && control.istep >= control.begin_rdf &&
                         control.istep % control.rdf_interval == 0;
   if (rdf_step && !rdf_ptr)
      ref_fatal("moldy_gb300: RDF accumulation needs the caller's rdf.c (rdf_ptr)");
   double st[9];
   for (int i = 0; i < 9; i++) st[i] = stress[i / 3][i % 3];
   mdgpu_status s = mdgpu_force_calc(c, h, site, site_force, &system->c_of_m[0][0], pe, st);
   if (g_first_rs && c->have_eintra) {
      ref_note("Intramolecular potential energy correction = %g", c->eintra * CONV_E);
      g_first_rs = false;
   }
   if (c->rs_valid) {
      if (c->rs.n_half != g_onabor) ref_note("Neighbour list contains %d cells", 2 * c->rs.n_half);
      g_onabor = c->rs.n_half;
   }
   ref_check(c, s);
   if (c->rs.nx != g_onx || c->rs.ny != g_ony || c->rs.nz != g_onz) {
      ref_note("MD cell divided into %d subcells (%dx%dx%d)", c->rs.ncells, c->rs.nx, c->rs.ny, c->rs.nz);
      g_onx = c->rs.nx;
      g_ony = c->rs.ny;
      g_onz = c->rs.nz;
   }
   for (int k = 0; k < c->info.n_too_close && k < MAX_TOO_CLOSE_REC; k++)
      ref_warn("Sites %d and %d closer than %fA.", c->info.too_close[k][0], c->info.too_close[k][1],
               std::sqrt(TOO_CLOSE));
   if (c->info.n_too_close > MAX_TOO_CLOSE_REC)
      ref_warn("%lld further site pairs closer than %fA.",
               (long long)(c->info.n_too_close - MAX_TOO_CLOSE_REC), std::sqrt(TOO_CLOSE));
   for (int i = 0; i < 9; i++) stress[i / 3][i % 3] = st[i];
   if (rdf_step) ref_rdf_accumulate(c, system);
}

void ewald(real **site, real **site_force, system_mp system, spec_mt *species, real *chg, double *pe,
           mat_mt stress)
{
   mdgpu_ctx *c = ref_ctx();
   double h[9];
   ref_sync(c, system, species, chg, nullptr, h);
   double st[9];
   for (int i = 0; i < 9; i++) st[i] = stress[i / 3][i % 3];
   mdgpu_status s = mdgpu_ewald(c, h, site, site_force, pe, st);
   if (g_first_ew && c->have_self) {
      const double q_net = [&] {
         double t = 0;
         for (double v : c->chg) t += v;
         return t;
      }();
      if (c->fw_mol >= 0) {   // charged framework (src/ewald.c:405-413)
         double q_fw = 0;
         for (size_t i = (size_t)c->fw_site0; i < c->chg.size(); i++) q_fw += c->chg[i];
         const double corr = 3.14159265358979323846 * q_fw * q_fw / (2.0 * c->ctl.alpha * c->ctl.alpha);
         ref_info("Framework has net electric charge of %.2g - correction of %g kJmol(-1) added to self energy",
                  q_fw * CONV_Q, corr / c->kl.vol * CONV_E);
      }
      if (std::fabs(q_net) * CONV_Q > 1.0e-5) {
         const double corr = 3.14159265358979323846 * q_net * q_net / (2.0 * c->ctl.alpha * c->ctl.alpha);
         ref_warn("System has net electric charge of %.2g - correction of %g kJmol(-1) added to self energy",
                  q_net * CONV_Q, corr / c->kl.vol * CONV_E);
      }
      ref_note("Ewald self-energy = %f kJ/mol", c->self_energy * CONV_E);
      if (c->kl_valid) ref_note("%d K-vectors included in reciprocal-space sum", c->kl.nk);
      g_first_ew = false;
   }
   ref_check(c, s);
   for (int i = 0; i < 9; i++) stress[i / 3][i % 3] = st[i];
}

double poteval(real *potpar, double r, int ptype, double chgsq)
{
   const double alpha = (&control != nullptr) ? control.alpha : 0.0;
   return host_poteval(potpar, r, ptype, chgsq, alpha);
}

}  // extern "C"
