"""Analytic gradients of the reference's energy and forces, in numpy (FP64).

TEST INFRASTRUCTURE ONLY: the checker for the GPU adjoint
(include/moldy_gb300.h, mdgpu_energy_grad / mdgpu_fm_loss_grad).  The
product path never imports this module.

The functions differentiate exactly the expressions the reference
evaluates, on the reference's own pair set (taken from the C restatement,
oracle/port):

* pair terms of kernel() (src/kernel.c:157-463): LJ, 6-exp, MCY, generic,
  HIW and Morse forms, plus the real-space Ewald term q_i q_j erfc(a r)/r
  with erfc by the A&S 7.1.26 polynomial (src/kernel.c:182-186) and the
  force factor (erfc(a r)/r + 2a/sqrt(pi) exp(-a^2 r^2))/r^2;
* the k-space sum of ewald() (src/ewald.c:495-566) over the half sphere,
  coeff_k = 8 pi/V exp(-k^2/4a^2)/k^2 (src/ewald.c:510), without the
  framework-framework part when a framework molecule is present;
* the self and sheet terms (src/ewald.c:367-433), the charged-framework
  sheet term included.

Conventions (the GPU library's): the gradient entry [a, b, k] of the
potential table is the derivative with respect to potpar[a*max_id + b][k] as
the force on a site of identifier a from a site of identifier b reads it,
each ordered evaluation carrying half the pair energy; intramolecular pairs
are left out of the energy (the reference subtracts them again as the
intramolecular correction, src/force.c:652-668) and kept in the forces.
The loss is L = w sum_i |F_i - F_ref_i|^2 with F the forces of force_calc
plus ewald.

Their correctness is pinned by central finite differences of the C
restatement's energies and forces (tests/test_adjoint_oracle.py).
"""
from __future__ import annotations

import math
from typing import Dict, Tuple

import numpy as np

from . import port

AS = (0.254829592, -0.284496736, 1.421413741, -1.453152027, 1.061405429)
ASP = 0.3275911
CONV_Q = (4.07497263794495e-14 * 1.0e-3 * 1.05482230112e-05) / 1.60217733e-19


def _as_erfc(x):
    t = 1.0 / (1.0 + ASP * x)
    pt = AS[0] + t * (AS[1] + t * (AS[2] + t * (AS[3] + t * AS[4])))
    return t * pt * np.exp(-x * x)


def _as_derfc(x):
    """d/dx of the A&S erfc t P(t) e^{-x^2}, t = 1/(1 + p x)."""
    t = 1.0 / (1.0 + ASP * x)
    pt = AS[0] + t * (AS[1] + t * (AS[2] + t * (AS[3] + t * AS[4])))
    dpt = AS[1] + t * (2 * AS[2] + t * (3 * AS[3] + t * 4 * AS[4]))
    return np.exp(-x * x) * (-ASP * t * t * (pt + t * dpt) - 2.0 * x * t * pt)


def pair_terms(ptype: int, r: np.ndarray, p: np.ndarray):
    """Short-range U, f = -U'/r, dU/dp [npar, n], df/dp [npar, n] for
    parameters p [n, 8] (src/kernel.c forms)."""
    rr = 1.0 / r
    rs = rr * rr
    P = [p[:, k] for k in range(8)]
    if ptype == 0:
        s6 = (P[1] * P[1] * rs) ** 3
        s12 = s6 * s6
        t5 = P[1] ** 5 * rs ** 3
        u = P[0] * (s12 - s6)
        f = rs * 6 * P[0] * (2 * s12 - s6)
        du = [s12 - s6, 6 * P[0] * t5 * (2 * s6 - 1)]
        df = [rs * 6 * (2 * s12 - s6), rs * 36 * P[0] * t5 * (4 * s6 - 1)]
    elif ptype == 1:
        E = np.exp(-P[2] * r)
        r6 = rs ** 3
        u = -P[0] * r6 + P[1] * E
        f = rs * (-6 * P[0] * r6) + P[2] * P[1] * E * rr
        du = [-r6, E, -r * P[1] * E]
        df = [-6 * rs * r6, P[2] * E * rr, P[1] * E * (rr - P[2])]
    elif ptype == 2:
        E1, E3 = np.exp(-P[1] * r), np.exp(-P[3] * r)
        e1, e2 = P[0] * E1, -P[2] * E3
        u = e1 + e2
        f = (P[1] * e1 + P[3] * e2) * rr
        du = [E1, -r * e1, -E3, -r * e2]
        df = [P[1] * E1 * rr, e1 * (rr - P[1]), -P[3] * E3 * rr, e2 * (rr - P[3])]
    elif ptype == 3:
        E1 = np.exp(-P[1] * r)
        e1 = P[0] * E1
        r4, r6 = rs * rs, rs ** 3
        r8, r12 = r4 * r4, r6 * r6
        u = e1 + P[2] * r12 - P[3] * r4 - P[4] * r6 - P[5] * r8
        f = rs * (12 * P[2] * r12 - 4 * P[3] * r4 - 6 * P[4] * r6 - 8 * P[5] * r8) + P[1] * e1 * rr
        du = [E1, -r * e1, r12, -r4, -r6, -r8]
        df = [P[1] * E1 * rr, e1 * (rr - P[1]), 12 * rs * r12, -4 * rs * r4, -6 * rs * r6, -8 * rs * r8]
    elif ptype == 4:
        r4, r6 = rs * rs, rs ** 3
        r12 = r6 * r6
        u = P[0] * r4 + P[1] * r6 + P[2] * r12
        f = rs * (4 * P[0] * r4 + 6 * P[1] * r6 + 12 * P[2] * r12)
        du = [r4, r6, r12]
        df = [4 * rs * r4, 6 * rs * r6, 12 * rs * r12]
    elif ptype == 6:
        E1 = np.exp((P[1] - r) * P[2])
        e1 = P[0] * E1
        r6 = rs ** 3
        d6 = r - P[6]
        E2, E3 = np.exp(-2 * P[5] * d6), np.exp(-P[5] * d6)
        e2, e3 = P[4] * E2, -2 * P[4] * E3
        u = e1 - P[3] * r6 + e2 + e3
        f = rs * (-6 * P[3] * r6) + rr * (P[2] * e1 + 2 * P[5] * e2 + P[5] * e3)
        du = [E1, P[2] * e1, (P[1] - r) * e1, -r6, E2 - 2 * E3, -d6 * (2 * e2 + e3), P[5] * (2 * e2 + e3)]
        df = [rr * P[2] * E1, rr * P[2] ** 2 * e1, rr * e1 * (1 + P[2] * (P[1] - r)), -6 * rs * r6,
              2 * P[5] * rr * (E2 - E3), rr * (2 * e2 + e3 - d6 * P[5] * (4 * e2 + e3)),
              rr * P[5] ** 2 * (4 * e2 + e3)]
    else:
        raise ValueError(f"unknown potential type {ptype}")
    return u, f, np.array(du), np.array(df)


def coulomb_terms(r: np.ndarray, alpha: float):
    """Per unit q_i q_j: uc = erfc(a r)/r, fc = (uc + norm e^{-a^2 r^2})/r^2
    and their alpha derivatives (A&S erfc, differentiated as such)."""
    x = alpha * r
    ex = np.exp(-x * x)
    uc = _as_erfc(x) / r
    norm = 2.0 * alpha / math.sqrt(math.pi)
    fc = (uc + norm * ex) / (r * r)
    de = _as_derfc(x)
    duc = de
    dfc = (de + 2.0 / math.sqrt(math.pi) * ex * (1.0 - 2.0 * x * x)) / (r * r)
    return uc, fc, duc, dfc


def kvectors(sysm) -> Tuple[np.ndarray, np.ndarray]:
    """The reference's half-sphere k-vector list (src/ewald.c:456-511):
    k [nk, 3] and coeff [nk]."""
    h = np.asarray(sysm.h, np.float64)
    c = sysm.control
    kc, alpha = c.k_cutoff, c.alpha
    hmax = int(math.floor(kc / (2 * math.pi) * h[0, 0]))
    kmax = int(math.floor(kc / (2 * math.pi) * math.sqrt(h[0, 1] ** 2 + h[1, 1] ** 2)))
    lmax = int(math.floor(kc / (2 * math.pi) * math.sqrt(h[0, 2] ** 2 + h[1, 2] ** 2 + h[2, 2] ** 2)))
    hinv = np.linalg.inv(h)
    hh, kk, ll = np.meshgrid(np.arange(0, hmax + 1), np.arange(-kmax, kmax + 1), np.arange(-lmax, lmax + 1),
                             indexing="ij")
    hh, kk, ll = hh.ravel(), kk.ravel(), ll.ravel()
    keep = (hh > 0) | ((hh == 0) & (kk > 0)) | ((hh == 0) & (kk == 0) & (ll > 0))
    hkl = np.stack([hh[keep], kk[keep], ll[keep]], 1).astype(np.float64)
    kv = 2 * math.pi * hkl @ hinv
    ksq = np.sum(kv * kv, 1)
    kv, ksq = kv[ksq < kc * kc], ksq[ksq < kc * kc]
    vol = float(np.linalg.det(h))
    coeff = 8.0 * math.pi / vol * np.exp(-ksq / (4 * alpha * alpha)) / ksq
    return kv, coeff


def _framework_mask(sysm) -> np.ndarray:
    """True for the sites of the framework species (the last species, one
    molecule; src/force.c:1215-1222)."""
    m = np.zeros(sysm.nsites, bool)
    base = 0
    for sp in sysm.species:
        n = sp.nsites * sp.nmols
        m[base:base + n] = bool(sp.framework)
        base += n
    return m


def _self_sheet_grad(sysm, gq: np.ndarray) -> float:
    """Adds d(-self + sheet/V)/dq_i into gq; returns d/dalpha.  The self
    energy covers the species before the framework (src/ewald.c:372-397); a
    framework's net charge q_f adds pi q_f^2/(2 alpha^2) to the sheet term
    (src/ewald.c:405-413), a net system charge sq subtracts pi sq^2/(2
    alpha^2) (src/ewald.c:417-422)."""
    alpha = sysm.control.alpha
    q = sysm.chg()
    fw = _framework_mask(sysm)
    rpi = 1.0 / math.sqrt(math.pi)
    ga = -rpi * float(np.sum(q[~fw] * q[~fw]))
    gq[~fw] -= 2.0 * alpha * rpi * q[~fw]
    base = 0
    for sp in sysm.species:
        if sp.framework:
            break
        ns, pf = sp.nsites, np.asarray(sp.p_f_sites, np.float64)
        for a in range(ns):
            for b in range(a + 1, ns):
                r = float(np.linalg.norm(pf[a] - pf[b]))
                e = (1.0 - _as_erfc(alpha * r)) / r
                ia = base + a + ns * np.arange(sp.nmols)
                ib = base + b + ns * np.arange(sp.nmols)
                gq[ia] -= q[ib] * e
                gq[ib] -= q[ia] * e
                ga += float(np.sum(q[ia] * q[ib])) * float(_as_derfc(alpha * r))
        base += ns * sp.nmols
    vol = sysm.volume()
    if fw.any():
        qf = float(np.sum(q[fw]))
        gq[fw] += math.pi * qf / (alpha * alpha * vol)
        ga -= math.pi * qf * qf / (alpha ** 3 * vol)
    sq = float(np.sum(q))
    if abs(sq) * CONV_Q > 1e-5:
        gq += -math.pi * sq / (alpha * alpha * vol)
        ga += math.pi * sq * sq / (alpha ** 3 * vol)
    return ga


def _forces(sysm, nthreads: int = 1) -> Tuple[np.ndarray, float]:
    rs = port.force_calc(sysm, nthreads=nthreads)
    f, pe = rs.force, rs.pe
    if sysm.control.alpha > 1e-7:
        ks = port.ewald(sysm, nthreads=nthreads)
        f, pe = f + ks.force, pe + ks.pe
    return f, pe


def gradients(sysm, f_ref=None, weight: float = 1.0) -> Tuple[float, Dict[str, np.ndarray]]:
    """(E, grads) with f_ref None, else (L, grads) of the force-matching loss.
    grads: potpar [M, M, 8], chg [N], alpha, and alpha_parts: the real-space,
    k-space and self/sheet parts of the alpha derivative (the Ewald sum does
    not depend on alpha in the converged limit, so these nearly cancel)."""
    loss = f_ref is not None
    M, N = sysm.max_id, sysm.nsites
    x = np.asarray(sysm.site, np.float64)
    q = sysm.chg()
    ids = sysm.site_ids()
    mol = sysm.molmap()
    pot = np.asarray(sysm.potpar, np.float64).reshape(M, M, 8)
    ctl = sysm.control
    alpha = ctl.alpha
    ew = alpha > 1e-7
    F, E = _forces(sysm)
    v = 2.0 * weight * (F - np.asarray(f_ref)) if loss else np.zeros((3, N))
    value = weight * float(np.sum((F - f_ref) ** 2)) if loss else E

    gp = np.zeros((M, M, 8))
    gq = np.zeros(N)
    ga = 0.0
    parts = [0.0, 0.0, 0.0]
    # ---- real space, on the reference's pair set
    pr = port.force_calc(sysm, want_pairs=True).pairs
    i, j, img = pr[:, 0].astype(np.int64), pr[:, 1].astype(np.int64), pr[:, 2].astype(np.int64)
    n = np.stack([img // 9 - 1, (img // 3) % 3 - 1, img % 3 - 1], 1).astype(np.float64)
    d = (x[:, j] - x[:, i]).T + n @ np.asarray(sysm.h, np.float64).T
    r2 = np.sum(d * d, 1)
    if ctl.strict_cutoff and not ctl.molpbc:
        r2 = np.where(r2 > ctl.cutoff ** 2, 1e4 * ctl.cutoff ** 2, r2)
    r = np.sqrt(r2)
    a, b = ids[i], ids[j]
    npar = {0: 2, 1: 3, 2: 4, 3: 6, 4: 3, 6: 7}[sysm.ptype]
    _, _, du_ab, df_ab = pair_terms(sysm.ptype, r, pot[a, b])
    _, _, du_ba, df_ba = pair_terms(sysm.ptype, r, pot[b, a])
    inter = mol[i] != mol[j]
    vi, vj = v[:, i].T, v[:, j].T
    wi = np.sum(vi * d, 1)           # v_i . d
    wj = -np.sum(vj * d, 1)          # v_j . (-d)
    ws = wi + wj                     # (v_i - v_j) . d
    for k in range(npar):
        if loss:
            np.add.at(gp, (a, b, k), -df_ab[k] * wi)
            np.add.at(gp, (b, a, k), -df_ba[k] * wj)
        else:
            np.add.at(gp, (a, b, k), np.where(inter, 0.5 * du_ab[k], 0.0))
            np.add.at(gp, (b, a, k), np.where(inter, 0.5 * du_ba[k], 0.0))
    if ew:
        uc, fc, duc, dfc = coulomb_terms(r, alpha)
        if loss:
            np.add.at(gq, i, -q[j] * fc * ws)
            np.add.at(gq, j, -q[i] * fc * ws)
            parts[0] = float(np.sum(-q[i] * q[j] * dfc * ws))
        else:
            np.add.at(gq, i, np.where(inter, q[j] * uc, 0.0))
            np.add.at(gq, j, np.where(inter, q[i] * uc, 0.0))
            parts[0] = float(np.sum(np.where(inter, q[i] * q[j] * duc, 0.0)))

    # ---- reciprocal space.  With a framework molecule the framework-
    # framework part |S_f|^2 is left out (src/ewald.c:528-579): non-framework
    # sites see the whole S(k), framework sites the non-framework part only.
    if ew:
        kv, cf = kvectors(sysm)
        ksq = np.sum(kv * kv, 1)
        dcf = cf * ksq / (2.0 * alpha ** 3)
        fw = _framework_mask(sysm)
        ph = x.T @ kv.T                  # [N, nk]
        cs, sn = np.cos(ph), np.sin(ph)
        C, S = q @ cs, q @ sn
        Cf, Sf = q[fw] @ cs[fw], q[fw] @ sn[fw]
        A, B = cf * C, cf * S
        Af, Bf = cf * Cf, cf * Sf
        if loss:
            kvv = v.T @ kv.T             # k . v_i
            Tc, Ts = (q[:, None] * kvv * cs).sum(0), (q[:, None] * kvv * sn).sum(0)
            Tcf = (q[fw, None] * kvv[fw] * cs[fw]).sum(0)
            Tsf = (q[fw, None] * kvv[fw] * sn[fw]).sum(0)
            P, Q = cf * Tc, cf * Ts
            Pf, Qf = cf * Tcf, cf * Tsf
            gq += cs @ Q - sn @ P + np.sum(kvv * (A * sn - B * cs), 1)
            gq[fw] -= cs[fw] @ Qf - sn[fw] @ Pf + np.sum(kvv[fw] * (Af * sn[fw] - Bf * cs[fw]), 1)
            parts[1] = float(np.sum(dcf * (C * Ts - S * Tc - (Cf * Tsf - Sf * Tcf))))
        else:
            gq += cs @ A + sn @ B
            gq[fw] -= cs[fw] @ Af + sn[fw] @ Bf
            parts[1] = float(np.sum(0.5 * dcf * (C * C + S * S - Cf * Cf - Sf * Sf)))
            parts[2] = _self_sheet_grad(sysm, gq)
    ga = parts[0] + parts[1] + parts[2]
    return value, {"potpar": gp, "chg": gq, "alpha": ga, "alpha_parts": parts}


def energy(sysm) -> float:
    """pe[0] + pe[1] of the C restatement (FP64)."""
    return _forces(sysm)[1]


def fm_loss(sysm, f_ref, weight: float = 1.0, nthreads: int = 1) -> float:
    F, _ = _forces(sysm, nthreads)
    return weight * float(np.sum((F - f_ref) ** 2))
