"""The reciprocal-space entry point that allocates nothing.

mdgpu_ewald_kspace_noalloc serves callers that cannot call cudaMalloc (code
under CUDA stream capture, hosts that own all device memory through their own
pools, step loops that must not allocate mid-run): all of its intermediates
live in one static device array inside the library.  Here it is called through
the C ABI on device buffers the test owns, twice in a row, and must agree with
the allocating entry point (mdgpu_ewald) within the mixed-precision tolerance
of the parity tests.  This file is collected last, so a run that stops at the
first failure has already run every other test.
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


def test_noalloc_kspace_matches_allocating_path_on_two_calls():
    torch = pytest.importorskip("torch")
    from moldy_gb300 import _lib
    from moldy_gb300.forcefield import ForceField

    sysm, _ = load_npz(os.path.join(GOLDEN, "syn_water2048.npz"))
    n = sysm.nsites
    # allocating path: ewald() semantics on host arrays
    ff = ForceField(sysm, precision="mixed")
    try:
        f_ref, pe_ref, st_ref = ff.ewald()
        info = ff.info()
    finally:
        ff.close()
    vol = float(np.linalg.det(sysm.h))
    sheet_v = info["sheet_energy"] / vol
    pe_k_ref = pe_ref - (-info["self_energy"] + sheet_v)       # k-space part only
    st_k_ref = st_ref - np.diag([sheet_v] * 3)

    L = _lib.load()
    dev = torch.device("cuda", 0)
    d_site = torch.from_numpy(np.ascontiguousarray(sysm.site)).to(dev)
    d_chg = torch.from_numpy(np.ascontiguousarray(sysm.chg())).to(dev)
    h = np.ascontiguousarray(sysm.h, np.float64).reshape(9)
    c = sysm.control
    for call in range(2):
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
        f = d_force.cpu().numpy()
        err = float(np.sqrt(((f - f_ref) ** 2).sum() / (f_ref ** 2).sum()))
        assert err < MIXED_TOL, (call, err)
        pe = float(d_pe.cpu().numpy()[0])
        assert abs(pe - pe_k_ref) / abs(pe_k_ref) < MIXED_TOL, (call, pe, pe_k_ref)
        stv = d_st.cpu().numpy().reshape(3, 3)
        assert np.abs(np.triu(stv - st_k_ref)).max() / np.abs(st_k_ref).max() < MIXED_TOL, call


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from moldy_gb300 import _lib
    L = _lib.load()
    h = np.diag([50.0, 50.0, 50.0]).reshape(9)
    too_many = 16384 + 1
    st = L.mdgpu_ewald_kspace_noalloc(_dp(h), too_many, C.c_void_p(8), C.c_void_p(8), 0.3, 2.0,
                                      C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), None)
    assert st == E_CAPACITY
