"""The reciprocal-space entry point that allocates nothing.

mdgpu_ewald_kspace_noalloc serves callers that cannot call cudaMalloc (hosts
that own all device memory through their own pools, step loops that must not
allocate mid-run): all of its intermediates, the k-vector list included, live
in one static device array inside the library.  Here it is called through the
C ABI on device buffers the test owns, twice in a row, and must agree within
the mixed-precision tolerance of the parity tests with the allocating entry
point (mdgpu_ewald) and with the reference's own reciprocal-space forces:
water, and ionic crystals listed species by species (all cations, then all
anions), where FP32 partial sums over sites in the caller's order would be of
one sign -- the entry point orders the sites by a cell grid inside its scratch.
This file is collected last, so a run that stops at the first failure has
already run every other test.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN
from moldy_gb300.system import load_npz

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5
E_CAPACITY = 7


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def _kspace_part(sysm, pe_ewald, st_ewald):
    """The k-space energy and stress of ewald() semantics (its self and sheet
    terms, src/ewald.c:367-433, taken out), with the constants the allocating
    path computes for the same system."""
    from moldy_gb300.forcefield import ForceField
    ff = ForceField(sysm, precision="mixed")
    try:
        ff.ewald()
        info = ff.info()
    finally:
        ff.close()
    sheet_v = info["sheet_energy"] / float(np.linalg.det(sysm.h))
    return pe_ewald - (-info["self_energy"] + sheet_v), st_ewald - np.diag([sheet_v] * 3)


def _noalloc_calls(sysm, ncalls=2):
    """(forces, energy, stress) of ncalls consecutive calls on fresh outputs."""
    torch = pytest.importorskip("torch")
    from moldy_gb300 import _lib
    L = _lib.load()
    dev = torch.device("cuda", 0)
    n = sysm.nsites
    d_site = torch.from_numpy(np.ascontiguousarray(sysm.site)).to(dev)
    d_chg = torch.from_numpy(np.ascontiguousarray(sysm.chg())).to(dev)
    h = np.ascontiguousarray(sysm.h, np.float64).reshape(9)
    c = sysm.control
    res = []
    for call in range(ncalls):
        d_force = torch.zeros((3, n), dtype=torch.float64, device=dev)
        d_pe = torch.zeros(1, dtype=torch.float64, device=dev)
        d_st = torch.zeros(9, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = L.mdgpu_ewald_kspace_noalloc(_dp(h), n, C.c_void_p(d_site.data_ptr()),
                                          C.c_void_p(d_chg.data_ptr()), c.alpha, c.k_cutoff,
                                          C.c_void_p(d_force.data_ptr()), C.c_void_p(d_pe.data_ptr()),
                                          C.c_void_p(d_st.data_ptr()), None)
        torch.cuda.synchronize()
        assert st == 0, f"call {call}: status {st}"
        res.append((d_force.cpu().numpy(), float(d_pe.cpu().numpy()[0]), d_st.cpu().numpy().reshape(3, 3)))
    return res


def _check(res, f_ref, pe_ref, st_ref):
    for call, (f, pe, stv) in enumerate(res):
        assert np.isfinite(f).all() and np.isfinite(pe), call
        err = _rel_rms(f, f_ref)
        assert err < MIXED_TOL, (call, err)
        assert abs(pe - pe_ref) / abs(pe_ref) < MIXED_TOL, (call, pe, pe_ref)
        assert np.abs(np.triu(stv - st_ref)).max() / np.abs(st_ref).max() < MIXED_TOL, call


def test_noalloc_kspace_matches_allocating_path_on_two_calls():
    from moldy_gb300.forcefield import ForceField
    sysm, _ = load_npz(os.path.join(GOLDEN, "syn_water2048.npz"))
    ff = ForceField(sysm, precision="mixed")
    try:
        f_ref, pe_ref, st_ref = ff.ewald()
    finally:
        ff.close()
    pe_k, st_k = _kspace_part(sysm, pe_ref, st_ref)
    _check(_noalloc_calls(sysm), f_ref, pe_k, st_k)


@pytest.mark.parametrize("name", ["syn_rocksalt512", "ex_quartz", "ex_mgclh2o"])
def test_noalloc_species_ordered_against_the_reference(name):
    """Ionic systems as the reference lists them, species by species (rock
    salt; quartz in its triclinic cell; MgCl2 in water), against the
    reference's own ewald() output in the golden fixtures."""
    sysm, gold = load_npz(os.path.join(GOLDEN, name + ".npz"))
    q = sysm.chg()
    assert (q[: sysm.nsites // 4] * q[0] >= 0).all() or name == "ex_mgclh2o"
    pe_k, st_k = _kspace_part(sysm, float(gold["pe_ewald"]), np.asarray(gold["stress_ewald"]))
    _check(_noalloc_calls(sysm), np.asarray(gold["force_ewald"]), pe_k, st_k)


def test_noalloc_rock_salt_4096_against_the_oracle(port_built):
    """4096 ions, cations first, against the FP64 C restatement (k-cutoff
    1.9 / A: 5,000-odd k-vectors, inside the entry point's limit)."""
    from moldy_gb300 import system
    from oracle import port
    sysm = system.rock_salt(ncell=8, k_cutoff=1.9)
    e = port.ewald(sysm, nthreads=os.cpu_count() or 1)
    pe_k, st_k = _kspace_part(sysm, e.pe, e.stress)
    _check(_noalloc_calls(sysm), e.force, pe_k, st_k)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from moldy_gb300 import _lib
    L = _lib.load()
    h = np.diag([50.0, 50.0, 50.0]).reshape(9)
    too_many = 16384 + 1
    st = L.mdgpu_ewald_kspace_noalloc(_dp(h), too_many, C.c_void_p(8), C.c_void_p(8), 0.3, 2.0,
                                      C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), None)
    assert st == E_CAPACITY
    # more k-vectors than the scratch holds: a k-cutoff far above the workloads'
    st = L.mdgpu_ewald_kspace_noalloc(_dp(h), 1000, C.c_void_p(8), C.c_void_p(8), 0.3, 6.0,
                                      C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), None)
    assert st == E_CAPACITY
