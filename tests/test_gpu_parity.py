"""Parity of the CUDA path with the reference on the golden fixtures.

Every fixture under tests/golden/ holds one configuration and the
reference's own outputs on it (real-space and Ewald site forces, energies,
stress, pair-set digest, logged constants).  The GPU path, called through the
C ABI, must reproduce:
  * the evaluated pair set exactly (canonical keys, moldy_gb300/pairset.py);
  * in FP64 form: site forces, energies and stress to 1e-12 relative;
  * in mixed form: site forces to 1e-5 relative RMS (the stated target) and
    energies and stress to 1e-5 relative;
  * the reference's logged constants (subcells, neighbour cells, k-vectors,
    self energy, intramolecular correction).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from moldy_gb300 import pairset
from moldy_gb300.system import CONV_E, load_npz

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def force_scale(z, n):
    """RMS force of the fixture; a perfect lattice has zero net forces, so
    its scale falls back to the energy per site over a length of 1 Å."""
    f = z["force_real"] + z["force_ewald"]
    rms = float(np.sqrt((f ** 2).sum() / n))
    return max(rms, abs(float(z["pe_real"])) / n)


def check_force(got, want, scale, n, tol):
    den = float(np.sqrt((want ** 2).sum() / n))
    if den > 1e-3 * scale:
        assert rel_rms(got, want) < tol, rel_rms(got, want)
    else:   # forces vanish by symmetry: compare on the fixture's force scale
        err = float(np.sqrt(((got - want) ** 2).sum() / n))
        assert err < tol * scale, (err, scale)


def rel(a, b):
    return abs(a - b) / abs(b)


def stress_err(got, want):
    return float(np.abs(np.triu(got) - np.triu(want)).max() / np.abs(want).max())


@pytest.fixture(scope="module")
def lib():
    from moldy_gb300 import _lib
    return _lib.load()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", golden_files())
def test_reference_semantics_parity(name, prec, lib):
    from moldy_gb300.forcefield import ForceField
    sysm, z = load_npz(os.path.join(GOLDEN, name + ".npz"))
    n = sysm.nsites
    tol = FP64_TOL if prec == "fp64" else MIXED_TOL
    scale = force_scale(z, n)
    ff = ForceField(sysm, precision=prec)
    try:
        fr, per, sr = ff.force_calc()
        check_force(fr, z["force_real"], scale, n, tol if prec == "fp64" else MIXED_TOL)
        assert rel(per, float(z["pe_real"])) < tol
        assert stress_err(sr, z["stress_real"]) < tol
        info = ff.info()
        assert info["npairs"] == int(z["npairs"])
        assert info["nx"] * info["ny"] * info["nz"] == int(z["log_ncells"])
        assert 2 * info["n_nabors"] == int(z["log_nabor_cells"])
        assert f"{info['eintra'] * CONV_E:g}" == f"{float(z['log_eintra_kjmol']):g}"
        if sysm.control.alpha > 1e-7:
            fe, pee, se = ff.ewald()
            check_force(fe, z["force_ewald"], scale, n, tol)
            assert rel(pee, float(z["pe_ewald"])) < tol
            assert stress_err(se, z["stress_ewald"]) < tol
            info = ff.info()
            assert info["nkvec"] == int(z["log_nkvec"])
            assert f"{info['self_energy'] * CONV_E:f}" == f"{float(z['log_self_energy_kjmol']):f}"
        # both parts in one call
        f, pe, st = ff.forces()
        check_force(f, z["force_real"] + z["force_ewald"], scale, n, tol)
        assert rel(pe[0], float(z["pe_real"])) < tol
        if sysm.control.alpha > 1e-7:
            assert rel(pe[1], float(z["pe_ewald"])) < tol
        assert stress_err(st, z["stress_real"] + z["stress_ewald"]) < tol
    finally:
        ff.close()


@pytest.mark.parametrize("name", golden_files())
def test_pair_set_bit_exact(name, lib):
    from moldy_gb300.forcefield import ForceField
    sysm, z = load_npz(os.path.join(GOLDEN, name + ".npz"))
    ff = ForceField(sysm, precision="fp64")
    try:
        keys = ff.pair_keys()
    finally:
        ff.close()
    cnt, dig = pairset.digest(keys)
    assert cnt == int(z["npairs"])
    assert dig == int(z["pair_digest"][0])
    if "pair_keys" in z:
        assert np.array_equal(keys, z["pair_keys"])


def test_accumulates_like_the_reference(lib):
    """force_calc/ewald add into site_force, pe and stress; the virial sees
    forces already present (src/force.c:973-981)."""
    from moldy_gb300.forcefield import ForceField
    from oracle import port
    sysm, z = load_npz(os.path.join(GOLDEN, "syn_water864_strict.npz"))
    rng = np.random.default_rng(5)
    f0 = rng.normal(0, 100.0, size=(3, sysm.nsites))
    s0 = rng.normal(0, 1e3, size=9)
    ff = ForceField(sysm, precision="fp64")
    try:
        f, pe, st = ff.force_calc(site_force=f0, pe=12.5, stress=s0)
    finally:
        ff.close()
    # the oracle with the same pre-filled arrays
    import ctypes as C
    L = port.lib()
    ps = port.PortSystem(sysm)
    site = np.ascontiguousarray(sysm.site)
    fo = f0.copy()
    peo = np.array([12.5])
    sto = s0.copy()
    info = port.PortInfo()
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    assert L.port_force_calc(C.byref(ps.s), dp(site), dp(fo), dp(peo), dp(sto), 1, None, 0, C.byref(info)) == 0
    assert rel_rms(f, fo) < 1e-12
    assert rel(pe, peo[0]) < 1e-12
    assert np.abs(st.reshape(9) - sto).max() / np.abs(sto).max() < 1e-12


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_too_close_pairs_counted_like_the_reference(port_built, prec, tol):
    """Molecules moved so that sites come closer than the reference's
    too-close distance (r^2 < 0.25 A^2, src/force.c:939-949): an O by another
    molecule's H (a pair with no interaction at all -- O carries no charge
    and LJ acts O-O only) and an H by another molecule's M.  The count of such pairs is the
    reference's, and the forces still match the oracle."""
    import dataclasses

    from moldy_gb300 import system
    from moldy_gb300.forcefield import ForceField
    base = system.water(nside=6, seed=3)
    site = np.array(base.site, copy=True)
    # whole molecules moved (their own geometry kept): the O of molecule 7
    # by an H of molecule 0, an H of molecule 9 by the M of molecule 0
    for mol, own, other, d in ((7, 0, 1, (0.3, 0.0, 0.0)), (9, 1, 3, (0.0, 0.35, 0.0))):
        shift = site[:, other] + np.array(d) - site[:, 4 * mol + own]
        site[:, 4 * mol:4 * mol + 4] += shift[:, None]
    sysm = dataclasses.replace(base, site=site)
    r = port_built.force_calc(sysm)
    assert r.info.n_too_close >= 2
    ff = ForceField(sysm, precision=prec)
    try:
        f, pe, _ = ff.force_calc()
        info = ff.info()
    finally:
        ff.close()
    assert info["n_too_close"] == r.info.n_too_close
    for a, b in info["too_close"]:
        d = site[:, a] - site[:, b]
        assert float(d @ d) < 0.25
    assert rel_rms(f, r.force) < tol, rel_rms(f, r.force)
    assert rel(pe, r.pe) < tol
