"""GPU adjoint (mdgpu_energy_grad, mdgpu_fm_loss_grad) against the analytic
oracle (oracle/adjoint.py, itself pinned by finite differences) and against
central finite differences of the FP64 C restatement, plus the torch
fitting harness (moldy_gb300/fitting.py)."""
import dataclasses
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["syn_water864_strict", "syn_water864_molpbc", "syn_water864_mcy", "ex_mgclh2o", "ex_quartz",
         "syn_generic216", "syn_hiw216", "syn_morse216", "syn_argon500_strict", "syn_rocksalt512", "ex_clay",
         "syn_waterwall"]

# FP64: the oracle's own rounding level.  Mixed: FP32 pair and k-space
# arithmetic; the bar for the fitted gradients is 1e-4 relative.
TOL = {"fp64": 1e-9, "mixed": 2e-5}
# The alpha derivative is the small difference of its real-space, k-space
# and self parts (the converged Ewald sum does not depend on alpha; the
# parts are up to 900x the total here): it is held to these tolerances of
# the parts' magnitude.  The mixed form's parts carry the FP32 error of the
# structure factors.
ATOL = {"fp64": 1e-10, "mixed": 5e-6}


def _load(name):
    """A golden fixture, or syn_waterwall: 245 rigid waters over a neutral
    checkerboard framework of 64 sites (charges +-0.4 e), built in place."""
    from moldy_gb300 import system
    if name == "syn_waterwall":
        return system.water_on_framework()
    return system.load_npz(os.path.join(GOLDEN, name + ".npz"))[0]


def _perturbed(sysm, seed=5):
    rng = np.random.default_rng(seed)
    M = sysm.max_id
    p = np.array(sysm.potpar, np.float64).reshape(M, M, 8)
    fac = rng.uniform(0.95, 1.05, (M, M, 8))
    fac = np.triu(fac.transpose(2, 0, 1)).transpose(1, 2, 0)
    fac = fac + np.transpose(fac, (1, 0, 2)) - fac * np.eye(M)[:, :, None]
    q = np.array(sysm.site_charge, np.float64) * rng.uniform(0.95, 1.05, M)
    ctl = dataclasses.replace(sysm.control, alpha=sysm.control.alpha * (1.02 if sysm.control.alpha > 1e-7 else 1))
    return dataclasses.replace(sysm, potpar=(p * fac).reshape(M * M, 8), site_charge=q, control=ctl)


def _close(g, g0, tol, what, alpha_scale=0.0, alpha_tol=None):
    """Table and charge gradients within tol of the largest entry; alpha
    within alpha_tol of |dE/dalpha| + alpha_scale (the magnitude of the
    parts it is the difference of)."""
    for k in ("potpar", "chg"):
        a, b = np.asarray(g[k]), np.asarray(g0[k])
        scale = max(np.max(np.abs(b)), 1e-300)
        err = np.max(np.abs(a - b)) / scale
        assert err <= tol, (what, k, err)
    at = 5 * tol if alpha_tol is None else alpha_tol
    assert abs(g["alpha"] - g0["alpha"]) <= at * (abs(g0["alpha"]) + alpha_scale), \
        (what, "alpha", g["alpha"], g0["alpha"], alpha_scale)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", CASES)
def test_energy_grad_matches_oracle(port_built, name, prec):
    from moldy_gb300 import ForceField
    from oracle import adjoint
    sysm = _load(name)
    E0, g0 = adjoint.gradients(sysm)
    ff = ForceField(sysm, precision=prec)
    E, g = ff.energy_grad()
    assert abs(E - E0) <= (1e-11 if prec == "fp64" else 1e-5) * abs(E0)
    _close(g, g0, TOL[prec], (name, prec, "energy"), np.sum(np.abs(g0["alpha_parts"])), ATOL[prec])
    ff.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", CASES)
def test_loss_grad_matches_oracle(port_built, name, prec):
    from moldy_gb300 import ForceField
    from oracle import adjoint
    base = _load(name)
    f_ref, _ = adjoint._forces(base)
    sysm = _perturbed(base)
    w = 1.0 / f_ref.size
    L0, g0 = adjoint.gradients(sysm, f_ref, w)
    ff = ForceField(sysm, precision=prec)
    L, g = ff.fm_loss_grad(f_ref, w)
    assert abs(L - L0) <= (1e-10 if prec == "fp64" else 1e-4) * L0
    _close(g, g0, TOL[prec] * (1 if prec == "fp64" else 5), (name, prec, "loss"),
           np.sum(np.abs(g0["alpha_parts"])), ATOL[prec])
    ff.close()


def test_set_params_matches_fresh_system(port_built):
    """Parameters changed through set_params give what a fresh context with
    those parameters gives."""
    from moldy_gb300 import ForceField
    base = _load("syn_water864_strict")
    pert = _perturbed(base)
    ff = ForceField(base, precision="fp64")
    ff.forces()
    ff.set_params(pert.potpar, pert.chg(), pert.control.alpha)
    E1, g1 = ff.energy_grad()
    ff2 = ForceField(pert, precision="fp64")
    E2, g2 = ff2.energy_grad()
    assert E1 == pytest.approx(E2, rel=1e-13)
    _close(g1, g2, 1e-12, "set_params")


def _water_theta_grads(ff_grad, base):
    """Chain rule from the table/charge gradients to (eps, sigma, q_H, alpha)
    of the water model (p0 = 4 eps / CONV_E, p1 = sigma, q_M = -2 q_H)."""
    from moldy_gb300.system import CONV_E, CONV_Q
    ids = base.site_ids()
    gp, gq = ff_grad["potpar"], ff_grad["chg"]
    return np.array([gp[1, 1, 0] * 4.0 / CONV_E, gp[1, 1, 1],
                     (np.sum(gq[ids == 2]) - 2.0 * np.sum(gq[ids == 3])) / CONV_Q, ff_grad["alpha"]])


@pytest.mark.parametrize("nside,nframes", [(8, 2), (16, 4)])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_water_fit_gradients_match_oracle_finite_differences(port_built, prec, nside, nframes):
    """Rigid water, 2048 sites over two seeded frames and the force-matching
    workload's size, 16,384 sites (4096 molecules) over four: the
    force-matching loss with epsilon, sigma and q_H scaled by seeded factors
    in [0.9, 1.1] (q_M = -2 q_H), reference forces at the original
    parameters.  The GPU gradient with respect to (epsilon, sigma, q_H,
    alpha), through the torch harness, is within 1e-4 relative of central
    finite differences of the FP64 C restatement (step 1e-5 relative)."""
    import torch

    from moldy_gb300 import ForceField, system
    from moldy_gb300.fitting import FitProblem, ForceMatchLoss, water_frames, water_tables
    from oracle import adjoint

    threads = os.cpu_count() or 1
    base = system.water(nside=nside, seed=11)
    frames = water_frames(base, nframes, seed=12)
    theta0 = np.array([0.6485, 3.154, 0.52, base.control.alpha])
    rng = np.random.default_rng(13)
    theta = theta0 * np.append(rng.uniform(0.9, 1.1, 3), 1.0)

    def sys_at(t, fr):
        pot, chg = water_tables(*[torch.tensor(v, dtype=torch.float64) for v in t[:3]], base)
        ctl = dataclasses.replace(base.control, alpha=float(t[3]))
        M = base.max_id
        qid = np.zeros(M)
        qid[2], qid[3] = t[2] / system.CONV_Q, -2 * t[2] / system.CONV_Q
        return dataclasses.replace(fr, potpar=pot.numpy(), site_charge=qid, control=ctl)

    f_refs = [adjoint._forces(sys_at(theta0, fr), threads)[0] for fr in frames]
    w = 1.0 / (len(frames) * f_refs[0].size)

    def oracle_loss(t):
        return sum(adjoint.fm_loss(sys_at(t, fr), f, w, threads) for fr, f in zip(frames, f_refs))

    fd = np.zeros(4)
    for k in range(4):
        h = 1e-5 * theta[k]
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd[k] = (oracle_loss(tp) - oracle_loss(tm)) / (2 * h)

    ff = ForceField(sys_at(theta, frames[0]), precision=prec)
    pb = FitProblem(ff, [f.site for f in frames], [f.c_of_m for f in frames], f_refs, w)
    t = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in theta]
    pot, chg = water_tables(t[0], t[1], t[2], base)
    L = ForceMatchLoss.apply(pot, chg, t[3], pb)
    L.backward()
    g = np.array([float(x.grad) for x in t])
    assert L.item() == pytest.approx(oracle_loss(theta), rel=1e-10 if prec == "fp64" else 1e-4)
    rel = np.abs(g - fd) / np.abs(fd)
    assert np.all(rel < 1e-4), (prec, g, fd, rel)
    # the C ABI's own gradient, chained by hand, agrees with autograd's
    gsum = sum(_water_theta_grads(ff.fm_loss_grad(f, w, fr.site, fr.c_of_m)[1], base)
               for fr, f in zip(frames, f_refs))
    assert np.allclose(gsum, g, rtol=1e-12, atol=0)
    ff.close()
