"""The analytic-gradient oracle (oracle/adjoint.py) against central finite
differences of the C restatement's energies and forces, on CPU.

This pins the gradient expressions the GPU adjoint is then compared with:
every potential form, the real-space and k-space Ewald terms, the self and
sheet terms, strict-cutoff and molecular-cutoff pair sets.
"""
import dataclasses
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = ["syn_water864_strict", "syn_water864_molpbc", "syn_water864_mcy", "ex_mgclh2o", "ex_quartz",
         "syn_generic216", "syn_hiw216", "syn_morse216", "syn_argon500_strict", "syn_rocksalt512", "ex_clay",
         "syn_waterwall"]


def _load(name):
    """A golden fixture, or syn_waterwall: 245 rigid waters over a neutral
    checkerboard framework of 64 sites (charges +-0.4 e), built in place."""
    from moldy_gb300 import system
    if name == "syn_waterwall":
        return system.water_on_framework()
    return system.load_npz(os.path.join(GOLDEN, name + ".npz"))[0]


def _with(sysm, potpar=None, site_charge=None, alpha=None):
    s = dataclasses.replace(sysm)
    if potpar is not None:
        s.potpar = potpar
    if site_charge is not None:
        s.site_charge = site_charge
    if alpha is not None:
        s.control = dataclasses.replace(sysm.control, alpha=alpha)
    return s


def _params(sysm):
    """(kind, index) of every parameter the system's terms depend on."""
    M = sysm.max_id
    pot = np.asarray(sysm.potpar).reshape(M, M, 8)
    out = []
    for a in range(M):
        for b in range(a, M):
            for k in range(sysm.n_potpar):
                if pot[a, b, k] != 0.0:
                    out.append(("pot", (a, b, k)))
    if sysm.control.alpha > 1e-7:
        out += [("chg", i) for i in range(M) if sysm.site_charge[i] != 0.0]
        out.append(("alpha", None))
    return out


def _shift(sysm, kind, idx, dx):
    M = sysm.max_id
    if kind == "pot":
        a, b, k = idx
        p = np.array(sysm.potpar, np.float64).reshape(M, M, 8)
        p[a, b, k] += dx
        if a != b:
            p[b, a, k] += dx
        return _with(sysm, potpar=p.reshape(M * M, 8))
    if kind == "chg":
        q = np.array(sysm.site_charge, np.float64)
        q[idx] += dx
        return _with(sysm, site_charge=q)
    return _with(sysm, alpha=sysm.control.alpha + dx)


def _value(sysm, kind, idx):
    if kind == "pot":
        return float(np.asarray(sysm.potpar).reshape(sysm.max_id, sysm.max_id, 8)[idx])
    if kind == "chg":
        return float(sysm.site_charge[idx])
    return sysm.control.alpha


def _analytic(sysm, g, kind, idx):
    if kind == "pot":
        a, b, k = idx
        return g["potpar"][a, b, k] + (g["potpar"][b, a, k] if a != b else 0.0)
    if kind == "chg":
        return float(np.sum(g["chg"][sysm.site_ids() == idx]))
    return g["alpha"]


def _fd(f, sysm, kind, idx, rel=1e-5):
    h = rel * abs(_value(sysm, kind, idx))
    return (f(_shift(sysm, kind, idx, h)) - f(_shift(sysm, kind, idx, -h))) / (2 * h)


def _perturbed(sysm, seed=5):
    """Parameters scaled by seeded factors in [0.95, 1.05]."""
    rng = np.random.default_rng(seed)
    M = sysm.max_id
    p = np.array(sysm.potpar, np.float64).reshape(M, M, 8)
    fac = rng.uniform(0.95, 1.05, (M, M, 8))
    fac = np.triu(fac.transpose(2, 0, 1)).transpose(1, 2, 0)
    fac = fac + np.transpose(fac, (1, 0, 2)) - fac * np.eye(M)[:, :, None]
    q = np.array(sysm.site_charge, np.float64) * rng.uniform(0.95, 1.05, M)
    alpha = sysm.control.alpha * (1.02 if sysm.control.alpha > 1e-7 else 1.0)
    return _with(sysm, potpar=(p * fac).reshape(M * M, 8), site_charge=q, alpha=alpha)


@pytest.mark.parametrize("name", CASES)
def test_energy_gradient_matches_finite_differences(port_built, name):
    from oracle import adjoint
    sysm = _load(name)
    E, g = adjoint.gradients(sysm)
    assert np.isclose(E, adjoint.energy(sysm), rtol=1e-12, atol=0)
    for kind, idx in _params(sysm):
        fd = _fd(adjoint.energy, sysm, kind, idx)
        an = _analytic(sysm, g, kind, idx)
        # rounding of the energies, amplified by the 2h of the difference
        noise = 1e-7 * abs(E) / abs(_value(sysm, kind, idx))
        assert abs(an - fd) <= 2e-6 * abs(fd) + noise, (name, kind, idx, an, fd)


@pytest.mark.parametrize("name", CASES)
def test_loss_gradient_matches_finite_differences(port_built, name):
    from oracle import adjoint
    base = _load(name)
    f_ref, _ = adjoint._forces(base)
    sysm = _perturbed(base)
    w = 1.0 / f_ref.size
    L, g = adjoint.gradients(sysm, f_ref, w)
    assert L > 0
    assert np.isclose(L, adjoint.fm_loss(sysm, f_ref, w), rtol=1e-12)
    loss = lambda s: adjoint.fm_loss(s, f_ref, w)   # noqa: E731
    for kind, idx in _params(sysm):
        fd = _fd(loss, sysm, kind, idx)
        an = _analytic(sysm, g, kind, idx)
        noise = 1e-7 * L / abs(_value(sysm, kind, idx))
        assert abs(an - fd) <= 2e-5 * abs(fd) + noise, (name, kind, idx, an, fd)
