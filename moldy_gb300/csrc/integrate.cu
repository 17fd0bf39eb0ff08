// Rigid-molecule dynamics on the GPU: the step of do_step (src/accel.c:626-827),
// all in FP64 and, at constant volume, all on the device, so a run of many
// steps moves no per-step data to the host.  The Nose-Poincare thermostat and
// the Parrinello-Rahman cell are described with their kernels below.
//
// One step (the symplectic leapfrog of src/leapfrog.c):
//   k_md_drift   half-step of the centres of mass (leapf_com,
//                src/leapfrog.c:133-146, with the periodic wrap of escape(),
//                src/leapfrog.c:117-128) and of the quaternions and principal
//                angular momenta (leapf_quat, src/leapfrog.c:246-392: the
//                Dullweber-Leimkuhler-McLachlan rotational splitting,
//                symmetric-top variant unless nosymmetric_rot)
//                the first half step also writes the site co-ordinates from
//                the new centres of mass and quaternions (make_sites,
//                src/algorith.c:169-215), one thread per molecule
//   forces       the force path of this library (real space + k space)
//   k_md_kick    molecular forces and principal-frame torques (mol_force,
//                mol_torque, src/algorith.c:111-160), two half kicks of the
//                momenta (leapf_mom, leapf_amom, src/leapfrog.c:149-157,
//                395-406), the kinetic energy between them -- where do_step
//                evaluates its conserved quantity (src/accel.c:718-727)
//   k_md_record  per-step energies (potential with the distant-potential
//                correction of eval_forces, src/accel.c:608-611; kinetic)
//   k_md_drift   second half-step of the co-ordinates.
// Matrix-vector products and axpy updates keep the reference's operation
// order without fused multiply-adds (src/matrix.c mat_vec_mul, mvaxpy).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "mdgpu_internal.h"

namespace mdgpu {

constexpr double INERTIA_MIN = 1.0e-14;   // src/defs.h:298
constexpr double AMOM_EPS = 8.0e-37;      // 8 * DBL_MIN as src/leapfrog.c:88-90 defines it
constexpr double QNORM_TOL = 1.0e-4;      // TOLERANCE, src/leapfrog.c:78

// FP64 products and sums in the reference's operation order; the compiler
// fuses a product into the following sum (FMA, one rounding instead of
// two), as a build of the reference for a CPU with FMA does: these kernels
// are bound by the FP64 pipe, and the fused form takes about a third fewer
// of its instructions.
#define DM(a, b) ((a) * (b))
#define DA(a, b) ((a) + (b))
#define DS(a, b) ((a) - (b))

struct MdStepParams {
   int nmols, nsites, molpbc, nosym, saxis, o1, o2;
   double h[9], hinv[9];
   double kick[9];      // 0.5 dt h^T (leapf_mom's scaled transpose)
   double half;         // 0.5 dt
   // constant temperature (Nose-Poincare): therm 1; ginv = (h^T h)^-1 for
   // leapf_com's (step / (mass s)) G^-1; Q the thermostat mass; gkt = d_of_f
   // kB T and ahalf = 0.5 dt d_of_f kB T, in the reference's operation order
   int therm;
   double ginv[9];
   double Q, gkt, ahalf, dt;
   // constant pressure (Parrinello-Rahman): baro 1.  The cell's terms of
   // H_0 (ke_cell, pressure x volume), increments of the thermostat
   // momentum made on the host by the cell's half steps (dsm_mid before H_0,
   // dsm_end at the step's end), and h's momentum for dump records.
   int baro;
   double kecell, pv, dsm_mid, dsm_end, W;
   double hmom[9];
};

// Device record of the thermostat: the variable s, its momentum, H_0 and
// whether H_0 has been evaluated since the thermostat was set.
enum { TH_S = 0, TH_SMOM = 1, TH_H0 = 2, TH_H0SET = 3 };

// q <- p * q-style products of src/quaterns.c:38-127 (r may alias p or q)
__device__ __forceinline__ void qmul(const double *p, const double *q, double *r)
{
   const double p0 = p[0], p1 = p[1], p2 = p[2], p3 = p[3];
   const double q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
   r[0] = DS(DS(DS(DM(p0, q0), DM(p1, q1)), DM(p2, q2)), DM(p3, q3));
   r[1] = DA(DS(DA(DM(p1, q0), DM(p0, q1)), DM(p3, q2)), DM(p2, q3));
   r[2] = DS(DA(DA(DM(p2, q0), DM(p3, q1)), DM(p0, q2)), DM(p1, q3));
   r[3] = DA(DA(DS(DM(p3, q0), DM(p2, q1)), DM(p1, q2)), DM(p0, q3));
}
__device__ __forceinline__ void qconjmul(const double *p, const double *q, double *r)
{
   const double pc[4] = {p[0], -p[1], -p[2], -p[3]};
   qmul(pc, q, r);
}

// rot = (cos a, sin a along `axis`), a = 0.5 step rinertia amom[axis+1]
// (make_rot, src/leapfrog.c:206-219), then amom <- rot^-1 amom rot,
// quat <- quat rot (rot_substep, src/leapfrog.c:236-243).
// The products of rot_substep with rot = (c, s along one axis): qmul's
// terms with a zero factor left out (adding or subtracting a zero product
// leaves every nonzero value unchanged, so the results are qmul's), the
// remaining terms in qmul's order.  a = axis + 1.
//   r = (c - s e_a) * q   (q_conj_mul of rot and q)
__device__ __forceinline__ void qmul_conjrot_left(double c, double s, int a, const double *q, double *r)
{
   const double p0 = c, pa = -s;
   const double q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
   if (a == 1) {
      r[0] = DS(DM(p0, q0), DM(pa, q1));
      r[1] = DA(DM(pa, q0), DM(p0, q1));
      r[2] = DS(DM(p0, q2), DM(pa, q3));
      r[3] = DA(DM(pa, q2), DM(p0, q3));
   } else if (a == 2) {
      r[0] = DS(DM(p0, q0), DM(pa, q2));
      r[1] = DA(DM(p0, q1), DM(pa, q3));
      r[2] = DA(DM(pa, q0), DM(p0, q2));
      r[3] = DS(DM(p0, q3), DM(pa, q1));
   } else {
      r[0] = DS(DM(p0, q0), DM(pa, q3));
      r[1] = DS(DM(p0, q1), DM(pa, q2));
      r[2] = DA(DM(pa, q1), DM(p0, q2));
      r[3] = DA(DM(pa, q0), DM(p0, q3));
   }
}
//   r = p * (c + s e_a)
__device__ __forceinline__ void qmul_rot_right(const double *p, double c, double s, int a, double *r)
{
   const double p0 = p[0], p1 = p[1], p2 = p[2], p3 = p[3], q0 = c, qa = s;
   if (a == 1) {
      r[0] = DS(DM(p0, q0), DM(p1, qa));
      r[1] = DA(DM(p1, q0), DM(p0, qa));
      r[2] = DA(DM(p2, q0), DM(p3, qa));
      r[3] = DS(DM(p3, q0), DM(p2, qa));
   } else if (a == 2) {
      r[0] = DS(DM(p0, q0), DM(p2, qa));
      r[1] = DS(DM(p1, q0), DM(p3, qa));
      r[2] = DA(DM(p2, q0), DM(p0, qa));
      r[3] = DA(DM(p3, q0), DM(p1, qa));
   } else {
      r[0] = DS(DM(p0, q0), DM(p3, qa));
      r[1] = DA(DM(p1, q0), DM(p2, qa));
      r[2] = DS(DM(p2, q0), DM(p1, qa));
      r[3] = DA(DM(p3, q0), DM(p0, qa));
   }
}

// sin and cos of a rotation angle.  The angles of a time step are small:
// for |x| <= 1/8 the Taylor series of sin and cos about 0 (through x^11 and
// x^10, Horner form in x^2; the first term left out is below 1e-20
// relative) costs a third of the general routine on the FP64 pipe, which
// bounds the integrator's kernels; larger angles take the general routine.
__device__ __forceinline__ void sincos_step(double x, double *s, double *c)
{
   if (fabs(x) <= 0.125) {
      const double x2 = x * x;
      const double ps = fma(fma(fma(fma(-1.0 / 39916800.0, x2, 1.0 / 362880.0), x2, -1.0 / 5040.0), x2,
                                1.0 / 120.0), x2, -1.0 / 6.0);
      *s = fma(x * x2, ps, x);
      const double pc = fma(fma(fma(fma(-1.0 / 3628800.0, x2, 1.0 / 40320.0), x2, -1.0 / 720.0), x2,
                                1.0 / 24.0), x2, -0.5);
      *c = fma(x2, pc, 1.0);
   } else {
      sincos(x, s, c);
   }
}

__device__ __forceinline__ void rot_axis(double step, int axis, double rin, double *amom, double *quat)
{
   const double angle = DM(DM(DM(0.5, step), rin), amom[axis + 1]);
   double sa, ca;
   sincos_step(angle, &sa, &ca);
   const int a = axis + 1;
   double t[4];
   qmul_conjrot_left(ca, sa, a, amom, t);
   qmul_rot_right(t, ca, sa, a, amom);
   qmul_rot_right(quat, ca, sa, a, t);
   for (int k = 0; k < 4; k++) quat[k] = t[k];
}

// Rotation about the angular momentum by 0.5 step rinertia |L|
// (make_rot_amom, src/leapfrog.c:222-235), applied to the quaternion only.
__device__ __forceinline__ void rot_amom(double step, double rin, const double *amom, double *quat)
{
   const double samom = sqrt(DA(DA(DM(amom[1], amom[1]), DM(amom[2], amom[2])), DM(amom[3], amom[3])));
   const double ramom = 1.0 / DA(samom, AMOM_EPS);
   const double angle = DM(DM(DM(0.5, step), rin), samom);
   double sa, ca;
   sincos_step(angle, &sa, &ca);
   const double rot[4] = {ca, DM(DM(sa, ramom), amom[1]), DM(DM(sa, ramom), amom[2]), DM(DM(sa, ramom), amom[3])};
   qmul(quat, rot, quat);
}

// Rotation matrix of a quaternion (q_to_rot, src/quaterns.c:129-160).
__device__ __forceinline__ void q_to_rot(const double *q, double *r)
{
   const double q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
   const double a01 = DM(DM(2.0, q0), q1), a02 = DM(DM(2.0, q0), q2), a03 = DM(DM(2.0, q0), q3);
   const double a12 = DM(DM(2.0, q1), q2), a13 = DM(DM(2.0, q1), q3), a23 = DM(DM(2.0, q2), q3);
   r[1] = DS(a12, a03);
   r[2] = DA(a13, a02);
   r[3] = DA(a12, a03);
   r[5] = DS(a23, a01);
   r[6] = DS(a13, a02);
   r[7] = DA(a23, a01);
   const double s0 = DM(q0, q0), s1 = DM(q1, q1), s2 = DM(q2, q2), s3 = DM(q3, q3);
   r[0] = DS(DS(DA(s0, s1), s2), s3);
   r[4] = DS(DA(DS(s0, s1), s2), s3);
   r[8] = DA(DS(DS(s0, s1), s2), s3);
}

__device__ __forceinline__ void matvec(const double *m, double a0, double a1, double a2, double *o)
{
   o[0] = DA(DA(DM(m[0], a0), DM(m[1], a1)), DM(m[2], a2));
   o[1] = DA(DA(DM(m[3], a0), DM(m[4], a1)), DM(m[5], a2));
   o[2] = DA(DA(DM(m[6], a0), DM(m[7], a1)), DM(m[8], a2));
}

// Site co-ordinates of one molecule (make_sites, src/algorith.c:169-215):
// site = R(q) p + h s, wrapped into the cell unless molecular cut-offs are
// in use.  q null: a molecule without rotational freedom.
__device__ __forceinline__ void mol_sites(const MdStepParams &P, const double *c_s, const double *q, int nsites,
                                          const double *__restrict__ pf, int site0, double *__restrict__ site)
{
   const int N = P.nsites;
   double c[3], R[9];
   matvec(P.h, c_s[0], c_s[1], c_s[2], c);
   if (q) q_to_rot(q, R);
   for (int t = 0; t < nsites; t++) {
      const double *p = pf + 3 * t;
      double r[3];
      if (q) {
         matvec(R, p[0], p[1], p[2], r);
      } else {
         r[0] = p[0];
         r[1] = p[1];
         r[2] = p[2];
      }
      double x = DA(r[0], c[0]), y = DA(r[1], c[1]), z = DA(r[2], c[2]);
      if (!P.molpbc) {
         const double *hi = P.hinv, *h = P.h;
         const double tx = floor(DA(DA(DA(DM(hi[0], x), DM(hi[1], y)), DM(hi[2], z)), 0.5));
         const double ty = floor(DA(DA(DA(DM(hi[3], x), DM(hi[4], y)), DM(hi[5], z)), 0.5));
         const double tz = floor(DA(DA(DA(DM(hi[6], x), DM(hi[7], y)), DM(hi[8], z)), 0.5));
         x = DS(x, DA(DA(DM(h[0], tx), DM(h[1], ty)), DM(h[2], tz)));
         y = DS(y, DA(DA(DM(h[3], tx), DM(h[4], ty)), DM(h[5], tz)));
         z = DS(z, DA(DA(DM(h[6], tx), DM(h[7], ty)), DM(h[8], tz)));
      }
      site[site0 + t] = x;
      site[N + site0 + t] = y;
      site[2 * (size_t)N + site0 + t] = z;
   }
}

// Half step of the co-ordinates (leapf_all_coords, src/accel.c:360-372).
// Under the thermostat (therm non-null) the steps are scaled by its
// variable s, and each block writes to tpart its share of the thermostat
// momentum's increments: 0.5 dt times the translational kinetic energy
// before the step (do_step's H3 half step, src/accel.c:696-700) and the
// rotational kinetic energies leapf_quat adds between its rotations
// (src/leapfrog.c:308-329, 365-386).
__global__ void __launch_bounds__(128)
k_md_drift(MdStepParams P, const MdSpec *__restrict__ spec, const int *__restrict__ mol_spec,
           const int *__restrict__ mol_q, double *__restrict__ cofm, const double *__restrict__ mom,
           double *__restrict__ quat, double *__restrict__ amom, int *__restrict__ err,
           const double *__restrict__ therm, double *__restrict__ tpart,
           const int *__restrict__ mol_site0 = nullptr, const double *__restrict__ pf = nullptr,
           double *__restrict__ site = nullptr)
{
   __shared__ double sh[128];
   const int m = blockIdx.x * blockDim.x + threadIdx.x;
   const double sv = therm ? therm[TH_S] : 1.0;
   double dsm = 0.0;   // this molecule's increment of the thermostat momentum
   if (m < P.nmols) {
   const MdSpec &S = spec[mol_spec[m]];
   // leapf_com: c += (step/(mass s)) G^-1 mom, then the periodic wrap
   double gd[9];
   const double sc = P.half / (S.mass * sv);
   for (int i = 0; i < 9; i++) gd[i] = DM(sc, P.ginv[i]);
   const double *a = gd;
   double *c = cofm + 3 * (size_t)m;
   const double x0 = mom[3 * (size_t)m], x1 = mom[3 * (size_t)m + 1], x2 = mom[3 * (size_t)m + 2];
   const double y0 = DA(DA(DA(c[0], DM(a[0], x0)), DM(a[1], x1)), DM(a[2], x2));
   const double y1 = DA(DA(DA(c[1], DM(a[3], x0)), DM(a[4], x1)), DM(a[5], x2));
   const double y2 = DA(DA(DA(c[2], DM(a[6], x0)), DM(a[7], x1)), DM(a[8], x2));
   if (therm && P.therm) {
      // trans_ke (src/algorith.c:221-239) of the momenta before the step
      const double *hi = P.hinv;
      double v[3];
      v[0] = DA(DA(DM(hi[0], x0), DM(hi[3], x1)), DM(hi[6], x2));
      v[1] = DA(DA(DM(hi[1], x0), DM(hi[4], x1)), DM(hi[7], x2));
      v[2] = DA(DA(DM(hi[2], x0), DM(hi[5], x1)), DM(hi[8], x2));
      dsm = P.half * ((v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / (2.0 * S.mass * (sv * sv)));
   }
   c[0] = DS(y0, floor(DA(y0, 0.5)));
   c[1] = DS(y1, floor(DA(y1, 0.5)));
   c[2] = DS(y2, floor(DA(y2, 0.5)));
   const int qi = mol_q[m];
   if (qi >= 0) {
   double q[4], L[4];
   for (int k = 0; k < 4; k++) {
      q[k] = quat[4 * (size_t)qi + k];
      L[k] = amom[4 * (size_t)qi + k];
   }
   // leapf_quat's step over s (stepdts); s = 1 at constant energy
   const double st = P.half / sv;
   const double *ri = S.rinertia;
   // 2 (rot_ke) s^2 / (amom . amom / I) of rot_ke, src/algorith.c:244-258
   auto rke = [&]() {
      double k = 0.0;
      for (int i = 0; i < 3; i++)
         if (S.inertia[i] > INERTIA_MIN) k += L[i + 1] * L[i + 1] / S.inertia[i];
      return k;
   };
   if (P.nosym) {   // leapf_quat_a, src/leapfrog.c:338-392
      const double st2 = P.half / (sv * sv);   // stepdts2
      rot_axis(0.5 * st, 0, ri[0], L, q);
      if (therm && P.therm) dsm += 0.25 * st2 * ri[0] * (L[1] * L[1]) + 0.25 * st2 * ri[1] * (L[2] * L[2]);
      rot_axis(0.5 * st, 1, ri[1], L, q);
      if (therm && P.therm) dsm += 0.5 * st2 * ri[2] * (L[3] * L[3]);
      rot_axis(st, 2, ri[2], L, q);
      rot_axis(0.5 * st, 1, ri[1], L, q);
      if (therm && P.therm) dsm += 0.25 * st2 * ri[1] * (L[2] * L[2]) + 0.25 * st2 * ri[0] * (L[1] * L[1]);
      rot_axis(0.5 * st, 0, ri[0], L, q);
   } else {         // leapf_quat_b, src/leapfrog.c:253-333
      const int sx = P.saxis, o1 = P.o1, o2 = P.o2;
      rot_axis(0.5 * st, o1, DS(ri[o1], ri[o2]), L, q);
      if (therm && P.therm) dsm += 0.5 * P.half * (0.5 * rke() / (sv * sv));
      rot_axis(st, sx, DS(ri[sx], ri[o2]), L, q);
      rot_amom(st, ri[o2], L, q);
      if (therm && P.therm) dsm += 0.5 * P.half * (0.5 * rke() / (sv * sv));
      rot_axis(0.5 * st, o1, DS(ri[o1], ri[o2]), L, q);
   }
   // normalise, src/leapfrog.c:99-114
   double norm = 0.0;
   for (int k = 0; k < 4; k++) norm = DA(norm, DM(q[k], q[k]));
   norm = sqrt(norm);
   if (fabs(norm - 1.0) > QNORM_TOL) atomicOr(err, 2);
   double qn[4];
   const double rnorm = 1.0 / norm;   // one division (the FP64 pipe bounds this kernel)
   for (int k = 0; k < 4; k++) {
      qn[k] = DM(q[k], rnorm);
      quat[4 * (size_t)qi + k] = qn[k];
      amom[4 * (size_t)qi + k] = L[k];
   }
   // the step's sites from the new centre of mass and orientation (the
   // values stored above), when the force evaluation follows
   if (site) mol_sites(P, c, qn, S.nsites, pf + 3 * (size_t)S.pf0, mol_site0[m], site);
   } else if (site) {
      mol_sites(P, c, nullptr, S.nsites, pf + 3 * (size_t)S.pf0, mol_site0[m], site);
   }
   }
   if (!therm) return;
   // fixed-shape block sum of the increments
   sh[threadIdx.x] = dsm;
   __syncthreads();
   for (int w = 64; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
      __syncthreads();
   }
   if (threadIdx.x == 0) tpart[blockIdx.x] = sh[0];
}

// One thread per molecule: force and principal-frame torque from the site
// forces, two half kicks, and the kinetic energy between them (block sums
// of the translational and rotational parts in kpart).
__global__ void __launch_bounds__(256)
k_md_kick(MdStepParams P, const MdSpec *__restrict__ spec, const int *__restrict__ mol_spec,
          const int *__restrict__ mol_q, const int *__restrict__ mol_site0, const double *__restrict__ pf,
          const double *__restrict__ force, const double *__restrict__ quat, double *__restrict__ mom,
          double *__restrict__ amom, double *__restrict__ kpart, double *__restrict__ molf,
          double *__restrict__ molt, const double *__restrict__ therm)
{
   __shared__ double sh[2][256];
   const int m = blockIdx.x * blockDim.x + threadIdx.x;
   const int N = P.nsites;
   double ket = 0.0, ker = 0.0;
   // leapf_all_momenta (src/accel.c:376-387): the half kicks scaled by the
   // thermostat variable, leapf_mom(step s) and leapf_amom(step s)
   double kick[9], hs = P.half;
   if (therm) {
      hs = P.half * therm[TH_S];
      for (int i = 0; i < 3; i++)
         for (int j = 0; j < 3; j++) kick[3 * i + j] = DM(hs, P.h[3 * j + i]);
   } else {
      for (int i = 0; i < 9; i++) kick[i] = P.kick[i];
   }
   if (m < P.nmols) {
      const MdSpec &S = spec[mol_spec[m]];
      const int s0 = mol_site0[m];
      double F[3] = {0.0, 0.0, 0.0};
      for (int k = 0; k < 3; k++)
         for (int s = 0; s < S.nsites; s++) F[k] = DA(F[k], force[(size_t)k * N + s0 + s]);
      const int qi = mol_q[m];
      double T[3] = {0.0, 0.0, 0.0};
      if (qi >= 0) {
         double R[9], Rt[9];
         q_to_rot(quat + 4 * (size_t)qi, R);
         for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) Rt[3 * a + b] = R[3 * b + a];
         const double *p = pf + 3 * (size_t)S.pf0;
         // each site's force in the principal frame once, then the torque
         // components summed over the sites in the reference's order
         for (int s = 0; s < S.nsites; s++) {
            double f[3];
            matvec(Rt, force[s0 + s], force[(size_t)N + s0 + s], force[2 * (size_t)N + s0 + s], f);
            for (int i = 0, j = 1, k = 2; i < 3; i++, j = (j + 1) % 3, k = (k + 1) % 3)
               T[i] = DA(T[i], DS(DM(p[3 * s + j], f[k]), DM(p[3 * s + k], f[j])));
         }
         for (int k = 0; k < 3; k++) molt[3 * (size_t)qi + k] = T[k];
      }
      for (int k = 0; k < 3; k++) molf[3 * (size_t)m + k] = F[k];
      const double *a = kick;
      double *pm = mom + 3 * (size_t)m;
      double x[3] = {pm[0], pm[1], pm[2]};
      for (int half = 0; half < 2; half++) {
         const double y0 = DA(DA(DA(x[0], DM(a[0], F[0])), DM(a[1], F[1])), DM(a[2], F[2]));
         const double y1 = DA(DA(DA(x[1], DM(a[3], F[0])), DM(a[4], F[1])), DM(a[5], F[2]));
         const double y2 = DA(DA(DA(x[2], DM(a[6], F[0])), DM(a[7], F[1])), DM(a[8], F[2]));
         x[0] = y0;
         x[1] = y1;
         x[2] = y2;
         double L[3] = {0.0, 0.0, 0.0};
         if (qi >= 0) {
            double *am = amom + 4 * (size_t)qi;
            for (int k = 0; k < 3; k++) {
               am[k + 1] = DA(am[k + 1], DM(hs, T[k]));
               L[k] = am[k + 1];
            }
         }
         if (half == 0) {
            // trans_ke, rot_ke (src/algorith.c:221-258) at the half kick
            double v[3];
            const double *hi = P.hinv;
            v[0] = DA(DA(DM(hi[0], x[0]), DM(hi[3], x[1])), DM(hi[6], x[2]));
            v[1] = DA(DA(DM(hi[1], x[0]), DM(hi[4], x[1])), DM(hi[7], x[2]));
            v[2] = DA(DA(DM(hi[2], x[0]), DM(hi[5], x[1])), DM(hi[8], x[2]));
            ket = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / (2.0 * S.mass);
            if (qi >= 0)
               for (int k = 0; k < 3; k++)
                  if (S.inertia[k] > INERTIA_MIN) ker += 0.5 * L[k] * L[k] / S.inertia[k];
         }
      }
      // the framework constraint of do_step (src/accel.c:748-755): after the
      // kicks (and after the kinetic energy at the half kick) a framework
      // molecule's momentum is zero
      pm[0] = S.framework ? 0.0 : x[0];
      pm[1] = S.framework ? 0.0 : x[1];
      pm[2] = S.framework ? 0.0 : x[2];
   }
   // fixed-shape block sums
   sh[0][threadIdx.x] = ket;
   sh[1][threadIdx.x] = ker;
   __syncthreads();
   for (int w = 128; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) {
         sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
         sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
      }
      __syncthreads();
   }
   if (threadIdx.x == 0) {
      kpart[2 * blockIdx.x] = sh[0][0];
      kpart[2 * blockIdx.x + 1] = sh[1][0];
   }
}

// Energy record of the step (one block of 128 threads): the kinetic-energy
// block sums reduced in a fixed order; the record index is a device counter
// so that a captured step replays unchanged.
// Under the thermostat it also takes the first half step's increments of
// the thermostat momentum (tpart, nbt block sums), evaluates H_0 when it
// has not been since the thermostat was set (do_step does at its first
// step, src/accel.c:718-727), and applies the potential-energy term of the
// thermostat momentum (src/accel.c:757-758).
__global__ void __launch_bounds__(128)
k_md_record(int *__restrict__ counter, int cap, const double *__restrict__ pe, const double *__restrict__ kpart,
            int nb, double dist_v, const DevOut *__restrict__ out, double *__restrict__ energies,
            int *__restrict__ err, MdStepParams P, double *__restrict__ therm, const double *__restrict__ tpart,
            int nbt)
{
   __shared__ double sh[3][128];
   const int t = threadIdx.x;
   double kt = 0.0, kr = 0.0, ds = 0.0;
   for (int b = t; b < nb; b += 128) {
      kt += kpart[2 * b];
      kr += kpart[2 * b + 1];
   }
   if (therm && P.therm)
      for (int b = t; b < nbt; b += 128) ds += tpart[b];
   sh[0][t] = kt;
   sh[1][t] = kr;
   sh[2][t] = ds;
   __syncthreads();
   for (int w = 64; w > 0; w >>= 1) {
      if (t < w) {
         sh[0][t] += sh[0][t + w];
         sh[1][t] += sh[1][t + w];
         sh[2][t] += sh[2][t + w];
      }
      __syncthreads();
   }
   if (t != 0) return;
   double ket = sh[0][0], ker = sh[1][0];
   const double pe_tot = (pe[0] + dist_v) + pe[1];
   if (therm) {
      // trans_ke and rot_ke divide by s^2 (src/algorith.c:238, 257)
      const double s = therm[TH_S], s2 = s * s;
      ket /= s2;
      ker /= s2;
      double smom = P.therm ? (therm[TH_SMOM] + sh[2][0]) + P.dsm_mid : 0.0;
      if (therm[TH_H0SET] == 0.0) {
         // src/accel.c:718-727; without the thermostat its terms are zero
         double h0 = (ket + ker) + pe_tot;
         if (P.therm) h0 = (h0 + smom * smom / (2.0 * P.Q)) + P.gkt * log(s);
         h0 = h0 + P.kecell;
         if (P.baro) h0 += P.pv;
         therm[TH_H0] = h0;
         therm[TH_H0SET] = 1.0;
      }
      if (P.therm) {
         smom -= P.dt * (pe_tot - therm[TH_H0]);
         therm[TH_SMOM] = smom;
      }
   }
   const int step = *counter;
   *counter = step + 1;
   if (out->err & 1) *err |= 1;
   if (step >= cap) return;
   double *e = energies + 4 * (size_t)step;
   e[0] = pe[0] + dist_v;
   e[1] = pe[1];
   e[2] = ket;
   e[3] = ker;
}

// The thermostat's own half steps (one thread): at the start of a step,
// leapf_nose_therm (src/leapfrog.c:465-472) then the d_of_f kB T term
// (src/accel.c:680-682); at its end (end != 0) the second half step's
// increments (tpart, nbt block sums) are added first, then the term and
// leapf_nose_therm in the reverse order (src/accel.c:787-790).
__global__ void __launch_bounds__(128)
k_md_therm(MdStepParams P, double *__restrict__ therm, const double *__restrict__ tpart, int nbt, int end)
{
   __shared__ double sh[128];
   const int t = threadIdx.x;
   double ds = 0.0;
   if (end)
      for (int b = t; b < nbt; b += 128) ds += tpart[b];
   sh[t] = ds;
   __syncthreads();
   for (int w = 64; w > 0; w >>= 1) {
      if (t < w) sh[t] += sh[t + w];
      __syncthreads();
   }
   if (t != 0) return;
   double s = therm[TH_S], smom = therm[TH_SMOM];
   auto nose = [&]() {
      const double scale = (1.0 + smom * P.half / (2.0 * P.Q));
      smom /= scale;
      s *= scale * scale;
   };
   if (!end) {
      nose();
      smom -= P.ahalf * (1.0 + log(s));
   } else {
      smom += sh[0] + P.dsm_end;
      smom -= P.ahalf * (1.0 + log(s));
      nose();
   }
   therm[TH_S] = s;
   therm[TH_SMOM] = smom;
}

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_check(c, e_, #x); } while (0)

// Kinetic part of the stress (stress_kin / energy_dyad, src/accel.c:348-356,
// src/algorith.c:261-284): per block the sums over molecules of
// v_i v_j / (mass s^2) with v = h^-T mom the real momenta, nine components.
__global__ void __launch_bounds__(128)
k_md_kedyad(MdStepParams P, const MdSpec *__restrict__ spec, const int *__restrict__ mol_spec,
            const double *__restrict__ mom, const double *__restrict__ therm, double *__restrict__ part)
{
   __shared__ double sh[9][128];
   const int m = blockIdx.x * blockDim.x + threadIdx.x;
   double d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
   if (m < P.nmols) {
      const MdSpec &S = spec[mol_spec[m]];
      const double s = therm ? therm[TH_S] : 1.0;
      const double *hi = P.hinv;
      const double x0 = mom[3 * (size_t)m], x1 = mom[3 * (size_t)m + 1], x2 = mom[3 * (size_t)m + 2];
      double v[3];
      v[0] = DA(DA(DM(hi[0], x0), DM(hi[3], x1)), DM(hi[6], x2));
      v[1] = DA(DA(DM(hi[1], x0), DM(hi[4], x1)), DM(hi[7], x2));
      v[2] = DA(DA(DM(hi[2], x0), DM(hi[5], x1)), DM(hi[8], x2));
      const double r = 1.0 / (S.mass * (s * s));
      for (int i = 0; i < 3; i++)
         for (int j = 0; j < 3; j++) d[3 * i + j] = v[i] * v[j] * r;
   }
   for (int k = 0; k < 9; k++) sh[k][threadIdx.x] = d[k];
   __syncthreads();
   for (int w = 64; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w)
         for (int k = 0; k < 9; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
      __syncthreads();
   }
   if (threadIdx.x < 9) part[9 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// ------------------------------------------------------------ dump records
// Sum over sites of f (x) d, d = R(q) p the site's offset from its centre of
// mass: the site-to-molecular virial correction of eval_forces
// (src/accel.c:576-601), sum f.r - sum F.R over sites and molecules, which is
// this sum.  Block partials [9], then one block sums them in fixed order.
__global__ void __launch_bounds__(256)
k_md_virc(MdStepParams P, const int *__restrict__ site_mol, const int *__restrict__ site_pf,
          const double *__restrict__ pf, const int *__restrict__ mol_q, const double *__restrict__ quat,
          const double *__restrict__ force, double *__restrict__ part)
{
   __shared__ double sh[9][256];
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const int N = P.nsites, t = threadIdx.x;
   double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
   if (i < N) {
      const int m = site_mol[i];
      const double *p = pf + 3 * (size_t)site_pf[i];
      const int qi = mol_q[m];
      double d[3] = {p[0], p[1], p[2]};
      if (qi >= 0) {
         double R[9];
         q_to_rot(quat + 4 * (size_t)qi, R);
         matvec(R, p[0], p[1], p[2], d);
      }
      const double f[3] = {force[i], force[(size_t)N + i], force[2 * (size_t)N + i]};
      for (int a = 0; a < 3; a++)
         for (int b = 0; b < 3; b++) v[3 * a + b] = f[a] * d[b];
   }
   for (int k = 0; k < 9; k++) sh[k][t] = v[k];
   __syncthreads();
   for (int w = 128; w > 0; w >>= 1) {
      if (t < w)
         for (int k = 0; k < 9; k++) sh[k][t] += sh[k][t + w];
      __syncthreads();
   }
   if (t < 9) part[9 * (size_t)blockIdx.x + t] = sh[t][0];
}

__global__ void __launch_bounds__(256) k_md_virc2(const double *__restrict__ part, int nb, double *__restrict__ virc)
{
   __shared__ double sh[9][256];
   const int t = threadIdx.x;
   double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
   for (int b = t; b < nb; b += 256)
      for (int k = 0; k < 9; k++) v[k] += part[9 * (size_t)b + k];
   for (int k = 0; k < 9; k++) sh[k][t] = v[k];
   __syncthreads();
   for (int w = 128; w > 0; w >>= 1) {
      if (t < w)
         for (int k = 0; k < 9; k++) sh[k][t] += sh[k][t + w];
      __syncthreads();
   }
   if (t < 9) virc[t] = sh[t][0];
}

// Offsets of the parts of a record (-1: absent), in dump_convert's order.
struct DumpLayout {
   int pos, quat, h, vel, avel, hmom, frc, trq, st;
};

static int dump_layout(int level, int n, int nr, DumpLayout &L)
{
   int o = 0;
   L = DumpLayout{-1, -1, -1, -1, -1, -1, -1, -1, -1};
   if (level & 1) {
      L.pos = o;
      L.quat = o + 3 * n;
      L.h = L.quat + 4 * nr;   // then ts, pe
      o = L.h + 11;
   }
   if (level & 2) {
      L.vel = o;
      L.avel = o + 3 * n;
      L.hmom = L.avel + 3 * nr;   // then tsmom
      o = L.hmom + 10;
   }
   if (level & 8) {
      L.frc = o;
      L.trq = o + 3 * n;
      L.st = L.trq + 3 * nr;
      o = L.st + 9;
   }
   return o;
}

// One thread per molecule: the state after the step converted as
// dump_convert does (src/dump.c:550-620): h s, quaternions; velocities
// h^-T mom / m (ts = 1, zero h momentum); principal angular velocities
// amom / I; molecular forces and torques.  Thread 0 adds h, ts, the total
// potential energy, the zero h and thermostat momenta, and the stress.
__global__ void k_md_dump(MdStepParams P, DumpLayout L, const MdSpec *__restrict__ spec,
                          const int *__restrict__ mol_spec, const int *__restrict__ mol_q,
                          const double *__restrict__ cofm, const double *__restrict__ mom,
                          const double *__restrict__ quat, const double *__restrict__ amom,
                          const double *__restrict__ molf, const double *__restrict__ molt,
                          const double *__restrict__ small, const double *__restrict__ virc, double dist_v,
                          double distp_v, float *__restrict__ rec, const double *__restrict__ therm)
{
   const int m = blockIdx.x * blockDim.x + threadIdx.x;
   // thermostat variable and momentum, h's momentum (1, 0, 0 at constant
   // energy and volume)
   const double ts = therm ? therm[TH_S] : 1.0, tsmom = (therm && P.therm) ? therm[TH_SMOM] : 0.0;
   if (m == 0) {
      if (L.h >= 0) {
         for (int k = 0; k < 9; k++) rec[L.h + k] = (float)P.h[k];
         rec[L.h + 9] = (float)ts;
         rec[L.h + 10] = (float)(DA(DA(small[0], dist_v), small[1]));
      }
      if (L.hmom >= 0) {
         for (int k = 0; k < 9; k++) rec[L.hmom + k] = (float)P.hmom[k];
         rec[L.hmom + 9] = (float)tsmom;
      }
      if (L.st >= 0) {
         // force_calc and ewald fill the upper triangle; eval_forces mirrors
         // it, subtracts the molecular correction and adds the distant
         // pressure term on the diagonal
         double S[9];
         for (int k = 0; k < 9; k++) S[k] = small[2 + k];
         for (int i = 0; i < 3; i++)
            for (int j = i + 1; j < 3; j++) S[3 * j + i] = S[3 * i + j];
         for (int k = 0; k < 9; k++) S[k] = DS(S[k], virc[k]);
         for (int i = 0; i < 3; i++) S[4 * i] = DA(S[4 * i], distp_v);
         for (int k = 0; k < 9; k++) rec[L.st + k] = (float)S[k];
      }
   }
   if (m >= P.nmols) return;
   const MdSpec &S = spec[mol_spec[m]];
   const int qi = mol_q[m];
   const double *s = cofm + 3 * (size_t)m;
   if (L.pos >= 0) {
      double r[3];
      matvec(P.h, s[0], s[1], s[2], r);
      for (int k = 0; k < 3; k++) rec[L.pos + 3 * m + k] = (float)r[k];
      if (qi >= 0)
         for (int k = 0; k < 4; k++) rec[L.quat + 4 * qi + k] = (float)quat[4 * (size_t)qi + k];
   }
   if (L.vel >= 0) {
      // dr/dt = h^-T mom / (m s) + (1/W) hmom s_c (the second term is zero
      // at constant volume)
      const double *x = mom + 3 * (size_t)m, *hi = P.hinv;
      const double rm = 1.0 / (S.mass * ts);
      double hw[9];
      for (int k = 0; k < 9; k++) hw[k] = P.baro ? DM(1.0 / P.W, P.hmom[k]) : 0.0;
      for (int i = 0; i < 3; i++) {
         const double v = DA(DA(DM(hi[i], x[0]), DM(hi[3 + i], x[1])), DM(hi[6 + i], x[2]));
         rec[L.vel + 3 * m + i] =
            (float)DA(DA(DA(DM(v, rm), DM(hw[3 * i], s[0])), DM(hw[3 * i + 1], s[1])), DM(hw[3 * i + 2], s[2]));
      }
      if (qi >= 0)
         for (int i = 0; i < 3; i++)
            rec[L.avel + 3 * qi + i] = (float)DM(DM(amom[4 * (size_t)qi + i + 1], 1.0 / ts), S.rinertia[i]);
   }
   if (L.frc >= 0) {
      for (int k = 0; k < 3; k++) rec[L.frc + 3 * m + k] = (float)molf[3 * (size_t)m + k];
      if (qi >= 0)
         for (int k = 0; k < 3; k++) rec[L.trq + 3 * qi + k] = (float)molt[3 * (size_t)qi + k];
   }
}

// (h^T h)^-1, the G^-1 of leapf_com (src/leapfrog.c:137-140)
static void gram_inverse(const double *h, double *Gi)
{
   double ht[9], G[9];
   for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) ht[3 * i + j] = h[3 * j + i];
   for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
         G[3 * i + j] = ht[3 * i] * h[j] + ht[3 * i + 1] * h[3 + j] + ht[3 * i + 2] * h[6 + j];
   inv3(G, Gi);
}

static void step_params(const mdgpu_ctx *c, MdStepParams &P)
{
   const MdHost &H = c->mdh;
   std::memset(&P, 0, sizeof P);
   P.nmols = c->nmols;
   P.nsites = c->nsites;
   P.molpbc = c->ctl.molpbc;
   P.nosym = H.nosym;
   P.saxis = H.saxis;
   P.o1 = (H.saxis + 1) % 3;
   P.o2 = (H.saxis + 2) % 3;
   std::memcpy(P.h, H.h, sizeof P.h);
   inv3(H.h, P.hinv);
   // leapf_mom: step * h^T, step = dt/2 (each of the two half kicks)
   for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) P.kick[3 * i + j] = H.half * H.h[3 * j + i];
   P.half = H.half;
   P.therm = H.therm ? 1 : 0;
   gram_inverse(H.h, P.ginv);
   P.Q = H.ttmass;
   P.gkt = H.gkt;
   P.ahalf = H.ahalf;
   P.dt = 2.0 * H.half;
   P.baro = H.baro ? 1 : 0;
   P.W = H.pmass;
   std::memcpy(P.hmom, H.hmom, sizeof P.hmom);
}

}  // namespace mdgpu

using namespace mdgpu;

extern "C" mdgpu_status mdgpu_md_init(mdgpu_ctx *c, const mdgpu_dynamics *dyn, const double *h,
                                      const double *c_of_m, const double *mom, const double *quat,
                                      const double *amom)
{
   if (!c || !dyn || !h || !c_of_m || !mom || !dyn->mass || !dyn->inertia || !dyn->rdof)
      return fail(c, MDGPU_E_ARG, "NULL argument");
   if (!c->have_system || !c->have_control)
      return fail(c, MDGPU_E_ARG, "mdgpu_set_system and mdgpu_set_control come first");
   if (!(dyn->step > 0.0)) return fail(c, MDGPU_E_ARG, "the timestep must be positive");
   mdgpu_status s = ensure_ready(c, h, true, true);
   if (s) return s;
   MdHost &H = c->mdh;
   const int nsp = (int)c->spec.size();
   H.spec.assign(nsp, MdSpec{});
   std::vector<int> mol_spec(c->nmols), mol_q(c->nmols), mol_site0(c->nmols), site_mol(c->nsites),
      site_pf(c->nsites);
   std::memcpy(H.h, h, sizeof H.h);
   H.half = 0.5 * dyn->step;
   H.nosym = dyn->nosymmetric_rot ? 1 : 0;
   H.therm = false;
   H.baro = 0;
   std::memset(H.hmom, 0, sizeof H.hmom);
   H.d_of_f = -3;   // start_up's count (src/startup.c:483-485, 570, 591)
   int nq = 0, m = 0, site = 0, pf0 = 0;
   H.saxis = -1;
   for (int k = 0; k < nsp; k++) {
      MdSpec &S = H.spec[k];
      const mdgpu_species &sp = c->spec[k];
      S.mass = dyn->mass[k];
      if (!(S.mass > 0.0)) return fail(c, MDGPU_E_ARG, "species mass must be positive");
      for (int i = 0; i < 3; i++) S.inertia[i] = dyn->inertia[3 * k + i];
      for (int i = 0; i < 3; i++) {
         const double *I = S.inertia;
         S.rinertia[i] = I[i] / (I[(i + 1) % 3] + I[(i + 2) % 3]) < INERTIA_MIN ? 0.0 : 1.0 / I[i];
      }
      S.nsites = sp.nsites;
      S.pf0 = pf0;
      S.framework = sp.framework ? 1 : 0;
      if (S.framework && dyn->rdof[k] > 0) return fail(c, MDGPU_E_ARG, "a framework species cannot rotate");
      const bool rot = dyn->rdof[k] > 0;
      H.d_of_f += (S.framework ? 0 : 3 * sp.nmols) + dyn->rdof[k] * sp.nmols;
      if (rot && H.saxis < 0) {
         // near-symmetry axis, chosen once from the first rotating species
         // as leapf_quat_b's static first-call choice does (src/leapfrog.c:282-297)
         double idmin = 1e37;
         for (int i = 0; i < 3; i++) {
            const double idiff = std::fabs(S.rinertia[(i + 1) % 3] - S.rinertia[(i + 2) % 3]);
            if (idiff < idmin) {
               idmin = idiff;
               H.saxis = i;
            }
         }
      }
      for (int j = 0; j < sp.nmols; j++, m++) {
         mol_spec[m] = k;
         mol_q[m] = rot ? nq++ : -1;
         mol_site0[m] = site;
         for (int t = 0; t < sp.nsites; t++, site++) {
            site_mol[site] = m;
            site_pf[site] = pf0 + t;
         }
      }
      pf0 += sp.nsites;
   }
   if (H.saxis < 0) H.saxis = 0;
   if (nq > 0 && (!quat || !amom)) return fail(c, MDGPU_E_ARG, "rotating species need quaternions and angular momenta");
   H.nmols_r = nq;
   H.dist = distant_const(c);
   H.distp = distant_pconst(c);
   if (H.graph) {
      cudaGraphExecDestroy(H.graph);
      H.graph = nullptr;
   }
   c->gen++;
   MdDev &D = c->md;
   cudaStream_t st = c->stream;
   CK(D.cofm.ensure(3 * (size_t)c->nmols));
   CK(D.mom.ensure(3 * (size_t)c->nmols));
   CK(D.quat.ensure(4 * (size_t)nq + 4));
   CK(D.amom.ensure(4 * (size_t)nq + 4));
   CK(D.mol_spec.ensure(c->nmols));
   CK(D.mol_q.ensure(c->nmols));
   CK(D.mol_site0.ensure(c->nmols));
   CK(D.site_mol.ensure(c->nsites));
   CK(D.site_pf.ensure(c->nsites));
   CK(D.pf.ensure(c->spec_pf.size()));
   CK(D.spec.ensure(nsp));
   CK(D.kpart.ensure(2 * (size_t)((c->nmols + 255) / 256)));
   CK(D.molf.ensure(3 * (size_t)c->nmols));
   CK(D.molt.ensure(3 * (size_t)nq + 3));
   CK(D.err.ensure(1));
   CK(D.counter.ensure(1));
   CK(D.therm.ensure(4));
   CK(D.tpart.ensure(2 * (size_t)((c->nmols + 127) / 128)));
   CK(cudaMemcpyAsync(D.cofm.p, c_of_m, 3 * (size_t)c->nmols * sizeof(double), cudaMemcpyHostToDevice, st));
   CK(cudaMemcpyAsync(D.mom.p, mom, 3 * (size_t)c->nmols * sizeof(double), cudaMemcpyHostToDevice, st));
   if (nq) {
      CK(cudaMemcpyAsync(D.quat.p, quat, 4 * (size_t)nq * sizeof(double), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(D.amom.p, amom, 4 * (size_t)nq * sizeof(double), cudaMemcpyHostToDevice, st));
   }
   CK(cudaMemcpyAsync(D.mol_spec.p, mol_spec.data(), c->nmols * sizeof(int), cudaMemcpyHostToDevice, st));
   CK(cudaMemcpyAsync(D.mol_q.p, mol_q.data(), c->nmols * sizeof(int), cudaMemcpyHostToDevice, st));
   CK(cudaMemcpyAsync(D.mol_site0.p, mol_site0.data(), c->nmols * sizeof(int), cudaMemcpyHostToDevice, st));
   CK(cudaMemcpyAsync(D.site_mol.p, site_mol.data(), c->nsites * sizeof(int), cudaMemcpyHostToDevice, st));
   CK(cudaMemcpyAsync(D.site_pf.p, site_pf.data(), c->nsites * sizeof(int), cudaMemcpyHostToDevice, st));
   CK(cudaMemcpyAsync(D.pf.p, c->spec_pf.data(), c->spec_pf.size() * sizeof(double), cudaMemcpyHostToDevice, st));
   CK(cudaMemcpyAsync(D.spec.p, H.spec.data(), nsp * sizeof(MdSpec), cudaMemcpyHostToDevice, st));
   CK(cudaMemsetAsync(D.err.p, 0, sizeof(int), st));
   {
      const double th0[4] = {1.0, 0.0, 0.0, 0.0};   // s = 1, no momentum, H_0 not evaluated
      CK(cudaMemcpyAsync(D.therm.p, th0, sizeof th0, cudaMemcpyHostToDevice, st));
   }
   CK(cudaStreamSynchronize(st));
   H.ready = true;
   return MDGPU_OK;
}

// Enqueues one step on the context's stream.
static mdgpu_status md_enqueue_step(mdgpu_ctx *c, const MdStepParams &P, int cap, double dist_v,
                                    bool virc = false)
{
   const MdHost &H = c->mdh;
   MdDev &D = c->md;
   cudaStream_t st = c->stream;
   const int N = c->nsites, M = c->nmols, nbm = (M + 255) / 256, nbd = (M + 127) / 128;
   double *th = P.therm ? D.therm.p : nullptr;
   if (th) {
      k_md_therm<<<1, 128, 0, st>>>(P, th, nullptr, 0, 0);
      c->launches += 1;
   }
   // half drift, and the sites of the force evaluation from its result
   k_md_drift<<<nbd, 128, 0, st>>>(P, D.spec.p, D.mol_spec.p, D.mol_q.p, D.cofm.p, D.mom.p, D.quat.p, D.amom.p,
                                   D.err.p, th, D.tpart.p, D.mol_site0.p, D.pf.p, c->site.p);
   CK(cudaGetLastError());
   c->launches += 1;
   mdgpu_status s = mdgpu_forces_device(c, H.h, c->site.p, D.cofm.p, c->force.p, c->small.p, c->small.p + 2);
   if (s) return s;
   if (virc) {
      // molecular correction of the virial, with the quaternions of this
      // force evaluation (the drift after the kick moves them)
      const int nbs = (N + 255) / 256;
      k_md_virc<<<nbs, 256, 0, st>>>(P, D.site_mol.p, D.site_pf.p, D.pf.p, D.mol_q.p, D.quat.p, c->force.p,
                                     D.vpart.p);
      k_md_virc2<<<1, 256, 0, st>>>(D.vpart.p, nbs, D.virc.p);
      c->launches += 2;
   }
   k_md_kick<<<nbm, 256, 0, st>>>(P, D.spec.p, D.mol_spec.p, D.mol_q.p, D.mol_site0.p, D.pf.p, c->force.p,
                                  D.quat.p, D.mom.p, D.amom.p, D.kpart.p, D.molf.p, D.molt.p, th);
   k_md_record<<<1, 128, 0, st>>>(D.counter.p, cap, c->small.p, D.kpart.p, nbm, dist_v, c->out.p, D.energies.p,
                                 D.err.p, P, th, D.tpart.p, nbd);
   k_md_drift<<<nbd, 128, 0, st>>>(P, D.spec.p, D.mol_spec.p, D.mol_q.p, D.cofm.p, D.mom.p, D.quat.p, D.amom.p,
                                   D.err.p, th, D.tpart.p + nbd);
   CK(cudaGetLastError());
   c->launches += 3;
   if (th) {
      k_md_therm<<<1, 128, 0, st>>>(P, th, D.tpart.p + nbd, nbd, 1);
      CK(cudaGetLastError());
      c->launches += 1;
   }
   return MDGPU_OK;
}

// ---- constant pressure: the cell's part of do_step, on the host (its
// state is nine numbers and its updates need the whole system's kinetic and
// virial stress, reduced on the device and copied back each step).
// Matrices row-major 3x3; the operation order of src/leapfrog.c and
// src/algorith.c, built without contraction.

// cofactors of h (mk_sigma, src/algorith.c:287-294)
static void mk_sigma_h(const double *h, double *sg)
{
   for (int i = 0, j = 1, k = 2; i < 3; i++, j = (j + 1) % 3, k = (k + 1) % 3)
      for (int l = 0, m = 1, n = 2; l < 3; l++, m = (m + 1) % 3, n = (n + 1) % 3)
         sg[3 * i + l] = h[3 * j + m] * h[3 * k + n] - h[3 * k + m] * h[3 * j + n];
}

// src/algorith.c:296-306
static double ke_cell_h(const double *hmom, double w)
{
   double s = 0;
   for (int i = 0; i < 9; i++) s += hmom[i] * hmom[i];
   return 0.5 / w * s;
}

static double trace_sqr_h(const double *a)
{
   double sum = 0.0;
   for (int i = 0; i < 9; i++) sum += a[i] * a[i];
   return sum;
}

// leapf_hmom (src/leapfrog.c:422-437): masked elements of h's momentum held
// at zero
static void leapf_hmom_h(double step, double *hmom, const double *sigma, double s, double pressure, int mask)
{
   const double r = 0.5 * step * s * pressure;
   for (int i = 0; i < 9; i++) {
      if (mask & 1)
         hmom[i] = 0;
      else
         hmom[i] -= r * sigma[i];
      mask >>= 1;
   }
}

// gleap_cell (src/leapfrog.c:474-507); the thermostat momentum's changes
// go to *dsmom
static void gleap_cell_h(double step, double pmass, double s, double pressure, int mask, double *h, double *hmom,
                         double *dsmom, bool therm, bool uniform)
{
   double sigma[9];
   double vol = det3(h);
   if (uniform) {
      leapf_hmom_h(step, hmom, h, 3.0 * vol * s / trace_sqr_h(h), pressure, mask);
   } else {
      mk_sigma_h(h, sigma);
      leapf_hmom_h(step, hmom, sigma, s, pressure, mask);
   }
   if (therm) *dsmom -= 0.5 * step * (ke_cell_h(hmom, pmass) + pressure * vol);
   // leapf_h (src/leapfrog.c:441-449)
   const double r = step * s / pmass;
   for (int i = 0; i < 9; i++) h[i] += r * hmom[i];
   vol = det3(h);
   if (therm) *dsmom -= 0.5 * step * (ke_cell_h(hmom, pmass) + pressure * vol);
   if (uniform) {
      leapf_hmom_h(step, hmom, h, 3.0 * vol * s / trace_sqr_h(h), pressure, mask);
   } else {
      mk_sigma_h(h, sigma);
      leapf_hmom_h(step, hmom, sigma, s, pressure, mask);
   }
}

// update_hmom (src/leapfrog.c:515-535): stress_part is a stress times the
// volume
static void update_hmom_h(double step, double s, const double *h, const double *stress_part, double *hmom,
                          bool uniform)
{
   double tmp[9];
   if (uniform) {
      const double f = step * s * (stress_part[0] + stress_part[4] + stress_part[8]) / trace_sqr_h(h);
      for (int i = 0; i < 9; i++) tmp[i] = f * h[i];
   } else {
      const double vol = det3(h);
      double sigma[9], prod[9];
      mk_sigma_h(h, sigma);
      for (int i = 0; i < 3; i++)
         for (int j = 0; j < 3; j++)
            prod[3 * i + j] = stress_part[3 * i] * sigma[j] + stress_part[3 * i + 1] * sigma[3 + j] +
                              stress_part[3 * i + 2] * sigma[6 + j];
      const double f = step * s / vol;
      for (int i = 0; i < 9; i++) tmp[i] = f * prod[i];
   }
   for (int i = 0; i < 9; i++) hmom[i] = hmom[i] + tmp[i];
}

// Kinetic stress (stress_kin) of the current momenta: device block sums,
// summed here in block order.
static mdgpu_status ke_dyad_h(mdgpu_ctx *c, const MdStepParams &P, double *dyad)
{
   MdDev &D = c->md;
   cudaStream_t st = c->stream;
   const int nbd = (c->nmols + 127) / 128;
   k_md_kedyad<<<nbd, 128, 0, st>>>(P, D.spec.p, D.mol_spec.p, D.mom.p, D.therm.p, D.kdpart.p);
   CK(cudaGetLastError());
   c->launches += 1;
   std::vector<double> &hp = c->mdh.kpart_h;
   hp.resize(9 * (size_t)nbd);
   CK(cudaMemcpyAsync(hp.data(), D.kdpart.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
   CK(cudaStreamSynchronize(st));
   for (int k = 0; k < 9; k++) dyad[k] = 0.0;
   for (int b = 0; b < nbd; b++)
      for (int k = 0; k < 9; k++) dyad[k] += hp[9 * (size_t)b + k];
   return MDGPU_OK;
}

// One step of do_step under constant pressure (and, when set, constant
// temperature), src/accel.c:673-791 in order: thermostat half step, cell
// half step (gleap_cell), kinetic-stress half kick of h's momentum, half
// drift, forces with the molecular virial, two half kicks and H_0, the
// virial-stress kick of h's momentum, the second kinetic-stress half kick,
// half drift, cell half step, thermostat half step.  Launched directly
// (h changes every step, and with it the cell grid and the k-vector list
// the force path rebuilds on the host).
static mdgpu_status md_baro_step(mdgpu_ctx *c, int cap)
{
   MdHost &H = c->mdh;
   MdDev &D = c->md;
   cudaStream_t st = c->stream;
   const int N = c->nsites, M = c->nmols, nbm = (M + 255) / 256, nbd = (M + 127) / 128;
   const bool uni = H.baro == 2, therm = H.therm;
   const double dt = 2.0 * H.half;
   double *th = D.therm.p;
   MdStepParams P;
   step_params(c, P);
   double ts = 1.0;
   if (therm) {
      k_md_therm<<<1, 128, 0, st>>>(P, th, nullptr, 0, 0);
      CK(cudaGetLastError());
      c->launches += 1;
      CK(cudaMemcpyAsync(&ts, th + TH_S, sizeof(double), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
   }
   double dsm_mid = 0.0, dsm_end = 0.0, dyad[9];
   gleap_cell_h(0.5 * dt, H.pmass, ts, H.pressure, H.strain_mask, H.h, H.hmom, &dsm_mid, therm, uni);
   step_params(c, P);
   mdgpu_status s = ke_dyad_h(c, P, dyad);
   if (s) return s;
   update_hmom_h(0.5 * dt, ts, H.h, dyad, H.hmom, uni);
   // half drift, and the sites of the force evaluation from its result
   k_md_drift<<<nbd, 128, 0, st>>>(P, D.spec.p, D.mol_spec.p, D.mol_q.p, D.cofm.p, D.mom.p, D.quat.p, D.amom.p,
                                   D.err.p, th, D.tpart.p, D.mol_site0.p, D.pf.p, c->site.p);
   CK(cudaGetLastError());
   c->launches += 1;
   if ((s = mdgpu_forces_device(c, H.h, c->site.p, D.cofm.p, c->force.p, c->small.p, c->small.p + 2)) != MDGPU_OK)
      return s;
   const int nbs = (N + 255) / 256;
   k_md_virc<<<nbs, 256, 0, st>>>(P, D.site_mol.p, D.site_pf.p, D.pf.p, D.mol_q.p, D.quat.p, c->force.p, D.vpart.p);
   k_md_virc2<<<1, 256, 0, st>>>(D.vpart.p, nbs, D.virc.p);
   const double vol = det3(H.h);
   P.kecell = ke_cell_h(H.hmom, H.pmass);
   P.pv = H.pressure * vol;
   P.dsm_mid = dsm_mid;
   std::memcpy(P.hmom, H.hmom, sizeof P.hmom);
   k_md_kick<<<nbm, 256, 0, st>>>(P, D.spec.p, D.mol_spec.p, D.mol_q.p, D.mol_site0.p, D.pf.p, c->force.p,
                                  D.quat.p, D.mom.p, D.amom.p, D.kpart.p, D.molf.p, D.molt.p, th);
   k_md_record<<<1, 128, 0, st>>>(D.counter.p, cap, c->small.p, D.kpart.p, nbm, H.dist / vol, c->out.p,
                                 D.energies.p, D.err.p, P, th, D.tpart.p, nbd);
   CK(cudaGetLastError());
   c->launches += 4;
   // the virial stress of eval_forces (src/accel.c:573-611): force_calc's
   // and ewald's upper triangle mirrored, the molecular correction
   // subtracted, the distant pressure added on the diagonal
   double sm[11], vc[9], S[9];
   CK(cudaMemcpyAsync(sm, c->small.p, sizeof sm, cudaMemcpyDeviceToHost, st));
   CK(cudaMemcpyAsync(vc, D.virc.p, sizeof vc, cudaMemcpyDeviceToHost, st));
   CK(cudaStreamSynchronize(st));
   for (int k = 0; k < 9; k++) S[k] = sm[2 + k];
   for (int i = 0; i < 3; i++)
      for (int j = i + 1; j < 3; j++) S[3 * j + i] = S[3 * i + j];
   for (int k = 0; k < 9; k++) S[k] -= vc[k];
   for (int i = 0; i < 3; i++) S[4 * i] += H.distp / vol;
   update_hmom_h(dt, ts, H.h, S, H.hmom, uni);
   if ((s = ke_dyad_h(c, P, dyad)) != MDGPU_OK) return s;
   update_hmom_h(0.5 * dt, ts, H.h, dyad, H.hmom, uni);
   k_md_drift<<<nbd, 128, 0, st>>>(P, D.spec.p, D.mol_spec.p, D.mol_q.p, D.cofm.p, D.mom.p, D.quat.p, D.amom.p,
                                   D.err.p, th, D.tpart.p + nbd);
   CK(cudaGetLastError());
   c->launches += 1;
   gleap_cell_h(0.5 * dt, H.pmass, ts, H.pressure, H.strain_mask, H.h, H.hmom, &dsm_end, therm, uni);
   if (therm) {
      P.dsm_end = dsm_end;
      k_md_therm<<<1, 128, 0, st>>>(P, th, D.tpart.p + nbd, nbd, 1);
      CK(cudaGetLastError());
      c->launches += 1;
   }
   return MDGPU_OK;
}

// Captures one step as a CUDA graph (after a step has run, so every buffer
// is allocated and every table uploaded: nothing in the step allocates or
// synchronises any more).
static mdgpu_status md_capture(mdgpu_ctx *c, const MdStepParams &P, int cap, double dist_v)
{
   MdHost &H = c->mdh;
   cudaStream_t st = c->stream;
   if (H.graph) {
      cudaGraphExecDestroy(H.graph);
      H.graph = nullptr;
   }
   const int64_t l0 = c->launches;
   CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
   mdgpu_status s = md_enqueue_step(c, P, cap, dist_v);
   cudaGraph_t g = nullptr;
   const cudaError_t e = cudaStreamEndCapture(st, &g);
   if (s) {
      if (g) cudaGraphDestroy(g);
      return s;
   }
   CK(e);
   // the node priorities captured from the streams (the k-space passes run
   // on a high-priority stream beside the pair kernel) only apply with
   // this flag
   const cudaError_t ei = cudaGraphInstantiateWithFlags(&H.graph, g, cudaGraphInstantiateFlagUseNodePriority);
   cudaGraphDestroy(g);
   CK(ei);
   H.graph_launches = c->launches - l0;
   c->launches = l0;
   H.graph_gen = c->gen;
   return MDGPU_OK;
}

// nsteps steps; with records, a dump record after step k (1-based) when
// k >= first and (k - first) % interval == 0, converted on the device into a
// batch buffer that is copied back whenever it fills.
static mdgpu_status md_run_impl(mdgpu_ctx *c, int nsteps, double *energies, int first, int interval,
                                int level, float *records)
{
   if (!c || nsteps < 0) return fail(c, MDGPU_E_ARG, "invalid argument");
   if (!c->mdh.ready) return fail(c, MDGPU_E_ARG, "mdgpu_md_init has not been called");
   MdHost &H = c->mdh;
   MdDev &D = c->md;
   cudaStream_t st = c->stream;
   DumpLayout DL;
   const int dsize = records ? dump_layout(level, c->nmols, H.nmols_r, DL) : 0;
   if (records) {
      if (first < 1 || interval < 1) return fail(c, MDGPU_E_ARG, "dump steps need first >= 1 and interval >= 1");
      if (dsize == 0) return fail(c, MDGPU_E_ARG, "dump level selects nothing (bits 0, 1, 3)");
   }
   mdgpu_status s = ensure_ready(c, H.h, true, true);
   if (s) return s;
   MdStepParams P;
   step_params(c, P);
   const int cap = nsteps > 0 ? nsteps : 1;
   if (D.energies.n < 4 * (size_t)cap) {
      // a larger record buffer moves the pointer a captured step holds
      CK(D.energies.ensure(4 * (size_t)cap));
      H.graph_gen = 0;
   }
   CK(c->small.ensure(16));
   const int nrec = records && nsteps >= first ? (nsteps - first) / interval + 1 : 0;
   int batch = 0;
   if (H.baro) {
      CK(D.vpart.ensure(9 * (size_t)((c->nsites + 255) / 256)));
      CK(D.virc.ensure(9));
      CK(D.kdpart.ensure(9 * (size_t)((c->nmols + 127) / 128)));
   }
   if (nrec > 0) {
      // device batch of records: up to 256 MiB
      batch = (int)std::min<size_t>((size_t)nrec, std::max<size_t>(1, ((size_t)64 << 20) / (size_t)dsize));
      CK(D.rec.ensure((size_t)batch * dsize));
      if (level & 8) {
         CK(D.vpart.ensure(9 * (size_t)((c->nsites + 255) / 256)));
         CK(D.virc.ensure(9));
      }
   }
   CK(cudaMemsetAsync(D.counter.p, 0, sizeof(int), st));
   const double vol = det3(H.h);
   double dist_v = H.dist / vol, distp_v = H.distp / vol;
   int r = 0, r_done = 0;
   for (int i = 0; i < nsteps; i++) {
      const int k = i + 1;
      const bool dump = nrec > 0 && k >= first && (k - first) % interval == 0;
      // a step runs directly until one has run since the configuration last
      // changed (every buffer is then allocated); later ones replay a
      // captured step (a step whose record needs the virial correction also
      // runs directly)
      const bool virc = dump && (level & 8);
      const bool replay = (i > 0 || H.warm_gen == c->gen) && !c->timing && !virc && !H.baro;
      if (H.baro) {
         // constant pressure: every step direct, h and the tables change
         if ((s = md_baro_step(c, cap)) != MDGPU_OK) return s;
         step_params(c, P);
         const double v = det3(H.h);
         dist_v = H.dist / v;
         distp_v = H.distp / v;
         c->gen++;
      } else if (replay && (!H.graph || H.graph_gen != c->gen || H.graph_cap != cap)) {
         if ((s = md_capture(c, P, cap, dist_v)) != MDGPU_OK) return s;
         H.graph_cap = cap;
      }
      if (H.baro) {
      } else if (replay) {
         CK(cudaGraphLaunch(H.graph, st));
         c->launches += H.graph_launches;
      } else {
         if ((s = md_enqueue_step(c, P, cap, dist_v, virc)) != MDGPU_OK) return s;
         H.warm_gen = c->gen;
      }
      if (dump) {
         const int M = c->nmols;
         k_md_dump<<<(M + 127) / 128, 128, 0, st>>>(P, DL, D.spec.p, D.mol_spec.p, D.mol_q.p, D.cofm.p, D.mom.p,
                                                    D.quat.p, D.amom.p, D.molf.p, D.molt.p, c->small.p,
                                                    D.virc.p, dist_v, distp_v,
                                                    D.rec.p + (size_t)(r % batch) * dsize,
                                                    (H.therm || H.baro) ? D.therm.p : nullptr);
         CK(cudaGetLastError());
         c->launches += 1;
         r++;
         if (r % batch == 0 || r == nrec) {
            const int nb = r - r_done;
            CK(cudaMemcpyAsync(records + (size_t)r_done * dsize, D.rec.p, (size_t)nb * dsize * sizeof(float),
                               cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            r_done = r;
         }
      }
   }
   int err = 0;
   if (energies && nsteps > 0)
      CK(cudaMemcpyAsync(energies, D.energies.p, 4 * (size_t)nsteps * sizeof(double), cudaMemcpyDeviceToHost, st));
   CK(cudaMemcpyAsync(&err, D.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
   if ((s = sync_out(c)) != MDGPU_OK) return s;
   if (err & 1) return fail(c, MDGPU_E_RANGE, "Co-ordinate out of range in BIN (fill_cells)");
   if (err & 2) return fail(c, MDGPU_E_RANGE, "quaternion normalisation error (QNORM2)");
   return MDGPU_OK;
}

extern "C" mdgpu_status mdgpu_md_run(mdgpu_ctx *c, int nsteps, double *energies)
{
   return md_run_impl(c, nsteps, energies, 0, 0, 0, nullptr);
}

extern "C" mdgpu_status mdgpu_md_run_dump(mdgpu_ctx *c, int nsteps, int first, int interval, int dump_level,
                                          double *energies, float *records)
{
   if (!records) return fail(c, MDGPU_E_ARG, "NULL records");
   return md_run_impl(c, nsteps, energies, first, interval, dump_level, records);
}

// DUMP_SIZE, src/defs.h:294-297
extern "C" int mdgpu_dump_size(int level, int nmols, int nmols_r)
{
   DumpLayout L;
   return dump_layout(level, nmols, nmols_r, L);
}

extern "C" mdgpu_status mdgpu_md_set_state(mdgpu_ctx *c, const double *c_of_m, const double *mom,
                                           const double *quat, const double *amom)
{
   if (!c) return MDGPU_E_ARG;
   if (!c->mdh.ready) return fail(c, MDGPU_E_ARG, "mdgpu_md_init has not been called");
   MdDev &D = c->md;
   cudaStream_t st = c->stream;
   const size_t M = c->nmols, Q = c->mdh.nmols_r;
   // into the buffers a captured step reads: the capture stays valid
   if (c_of_m) CK(cudaMemcpyAsync(D.cofm.p, c_of_m, 3 * M * sizeof(double), cudaMemcpyHostToDevice, st));
   if (mom) CK(cudaMemcpyAsync(D.mom.p, mom, 3 * M * sizeof(double), cudaMemcpyHostToDevice, st));
   if (quat && Q) CK(cudaMemcpyAsync(D.quat.p, quat, 4 * Q * sizeof(double), cudaMemcpyHostToDevice, st));
   if (amom && Q) CK(cudaMemcpyAsync(D.amom.p, amom, 4 * Q * sizeof(double), cudaMemcpyHostToDevice, st));
   CK(cudaStreamSynchronize(st));
   return MDGPU_OK;
}

extern "C" mdgpu_status mdgpu_md_get_state(mdgpu_ctx *c, double *c_of_m, double *mom, double *quat,
                                           double *amom)
{
   if (!c) return MDGPU_E_ARG;
   if (!c->mdh.ready) return fail(c, MDGPU_E_ARG, "mdgpu_md_init has not been called");
   MdDev &D = c->md;
   cudaStream_t st = c->stream;
   const size_t M = c->nmols, Q = c->mdh.nmols_r;
   if (c_of_m) CK(cudaMemcpyAsync(c_of_m, D.cofm.p, 3 * M * sizeof(double), cudaMemcpyDeviceToHost, st));
   if (mom) CK(cudaMemcpyAsync(mom, D.mom.p, 3 * M * sizeof(double), cudaMemcpyDeviceToHost, st));
   if (quat && Q) CK(cudaMemcpyAsync(quat, D.quat.p, 4 * Q * sizeof(double), cudaMemcpyDeviceToHost, st));
   if (amom && Q) CK(cudaMemcpyAsync(amom, D.amom.p, 4 * Q * sizeof(double), cudaMemcpyDeviceToHost, st));
   CK(cudaStreamSynchronize(st));
   return MDGPU_OK;
}

// Boltzmann's constant in program units (kB of src/defs.h:226, the
// CODATA 1986 values and the amu, A, ps units, evaluated in that order).
static const double KB_PROG = 1.380658e-23 / (1.6605402e-27 * (1.0e-10 / 1.0e-12) * (1.0e-10 / 1.0e-12));

extern "C" mdgpu_status mdgpu_md_set_thermostat(mdgpu_ctx *c, int enable, double temp, double ttmass, double ts,
                                                double tsmom)
{
   if (!c) return MDGPU_E_ARG;
   if (!c->mdh.ready) return fail(c, MDGPU_E_ARG, "mdgpu_md_init has not been called");
   MdHost &H = c->mdh;
   if (!enable) {
      H.therm = false;
      const double v[4] = {1.0, 0.0, 0.0, 0.0};
      CK(cudaMemcpyAsync(c->md.therm.p, v, sizeof v, cudaMemcpyHostToDevice, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      c->gen++;
      return MDGPU_OK;
   }
   if (!(ttmass > 0.0) || !(temp >= 0.0) || !(ts > 0.0))
      return fail(c, MDGPU_E_ARG, "thermostat: ttmass and ts must be positive, temp not negative");
   H.therm = true;
   H.temp = temp;
   H.ttmass = ttmass;
   const double dt = 2.0 * H.half;
   H.gkt = (double)H.d_of_f * KB_PROG * temp;
   H.ahalf = 0.5 * dt * (double)H.d_of_f * KB_PROG * temp;
   const double v[4] = {ts, tsmom, 0.0, 0.0};
   CK(cudaMemcpyAsync(c->md.therm.p, v, sizeof v, cudaMemcpyHostToDevice, c->stream));
   CK(cudaStreamSynchronize(c->stream));
   c->gen++;
   return MDGPU_OK;
}

extern "C" mdgpu_status mdgpu_md_get_thermostat(mdgpu_ctx *c, double *out)
{
   if (!c || !out) return MDGPU_E_ARG;
   if (!c->mdh.ready) return fail(c, MDGPU_E_ARG, "mdgpu_md_init has not been called");
   double v[4];
   CK(cudaMemcpyAsync(v, c->md.therm.p, sizeof v, cudaMemcpyDeviceToHost, c->stream));
   CK(cudaStreamSynchronize(c->stream));
   out[0] = v[0];
   out[1] = v[1];
   out[2] = v[2];
   return MDGPU_OK;
}

extern "C" mdgpu_status mdgpu_md_set_barostat(mdgpu_ctx *c, int mode, double pressure, double pmass, int strain_mask,
                                              const double *hmom)
{
   if (!c) return MDGPU_E_ARG;
   if (!c->mdh.ready) return fail(c, MDGPU_E_ARG, "mdgpu_md_init has not been called");
   MdHost &H = c->mdh;
   if (mode == 0) {
      H.baro = 0;
      std::memset(H.hmom, 0, sizeof H.hmom);
      c->gen++;
      return MDGPU_OK;
   }
   if (mode != 1 && mode != 2) return fail(c, MDGPU_E_ARG, "barostat: mode 1 (anisotropic) or 2 (uniform)");
   if (!(pmass > 0.0) || !(pressure >= 0.0))
      return fail(c, MDGPU_E_ARG, "barostat: the cell mass must be positive, the pressure not negative");
   if (c->ctl.molpbc) return fail(c, MDGPU_E_UNSUPPORTED, "barostat with molecular cut-offs");
   H.baro = mode;
   H.pressure = pressure;
   H.pmass = pmass;
   H.strain_mask = strain_mask;
   if (hmom) std::memcpy(H.hmom, hmom, sizeof H.hmom);
   else std::memset(H.hmom, 0, sizeof H.hmom);
   // H_0 is evaluated on the next step (with the thermostat's state kept)
   double th[4];
   CK(cudaMemcpyAsync(th, c->md.therm.p, sizeof th, cudaMemcpyDeviceToHost, c->stream));
   CK(cudaStreamSynchronize(c->stream));
   th[TH_H0SET] = 0.0;
   CK(cudaMemcpyAsync(c->md.therm.p, th, sizeof th, cudaMemcpyHostToDevice, c->stream));
   CK(cudaStreamSynchronize(c->stream));
   c->gen++;
   return MDGPU_OK;
}

extern "C" mdgpu_status mdgpu_md_get_barostat(mdgpu_ctx *c, double *h, double *hmom)
{
   if (!c) return MDGPU_E_ARG;
   if (!c->mdh.ready) return fail(c, MDGPU_E_ARG, "mdgpu_md_init has not been called");
   if (h) std::memcpy(h, c->mdh.h, 9 * sizeof(double));
   if (hmom) std::memcpy(hmom, c->mdh.hmom, 9 * sizeof(double));
   return MDGPU_OK;
}
