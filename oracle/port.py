"""ctypes binding of the C restatement (oracle/port/moldy_port.c).

TEST INFRASTRUCTURE ONLY: the tests call it as the parity checker, and
bench.py's CPU-baseline leg and reference arm time it.  The product path
never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

PORT_ERRORS = {-1: "bad argument", -2: "cutoff beyond one image (CUTOFF)",
               -3: "co-ordinate out of range", -4: "neighbour-list capacity (TONAB)",
               -5: "unknown potential type", -6: "frameworks unsupported",
               -7: "out of memory", -8: "pair buffer too small"}


class _Sys(C.Structure):
    _fields_ = [("nsites", C.c_int), ("nmols", C.c_int), ("nspecies", C.c_int),
                ("max_id", C.c_int), ("ptype", C.c_int),
                ("spec_nsites", C.POINTER(C.c_int)), ("spec_nmols", C.POINTER(C.c_int)),
                ("spec_framework", C.POINTER(C.c_int)), ("spec_site_id", C.POINTER(C.c_int)),
                ("spec_pf", C.POINTER(C.c_double)), ("potpar", C.POINTER(C.c_double)),
                ("site_charge", C.POINTER(C.c_double)), ("c_of_m", C.POINTER(C.c_double)),
                ("h", C.c_double * 9), ("cutoff", C.c_double), ("subcell", C.c_double),
                ("alpha", C.c_double), ("k_cutoff", C.c_double),
                ("strict_cutoff", C.c_int), ("molpbc", C.c_int)]


class PortInfo(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("n_nabors", C.c_int),
                ("hmax", C.c_int), ("kmax", C.c_int), ("lmax", C.c_int), ("nkvec", C.c_int),
                ("eintra", C.c_double), ("self_energy", C.c_double), ("sheet_energy", C.c_double),
                ("npairs", C.c_int64), ("n_too_close", C.c_int64),
                ("n_nab_max", C.c_int64), ("n_nab_cap", C.c_int64),
                ("t_setup", C.c_double), ("t_kloop", C.c_double)]


_libs = {}


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib(fast: bool = False):
    name = "libmoldy_port_fast.so" if fast else "libmoldy_port.so"
    if name not in _libs:
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        dp, i64 = C.POINTER(C.c_double), C.c_int64
        L.port_force_calc.argtypes = [C.POINTER(_Sys), dp, dp, dp, dp, C.c_int,
                                      C.POINTER(C.c_int32), i64, C.POINTER(PortInfo)]
        L.port_ewald.argtypes = [C.POINTER(_Sys), dp, dp, dp, dp, C.c_int, i64, i64,
                                 C.POINTER(PortInfo)]
        L.port_poteval.argtypes = [dp, C.c_double, C.c_int, C.c_double, C.c_double]
        L.port_poteval.restype = C.c_double
        _libs[name] = L
    return _libs[name]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class PortSystem:
    """Holds the flattened arrays of a System alive for the C calls."""

    def __init__(self, sysm):
        self.sysm = sysm
        sp = sysm.species
        self.spec_nsites = np.array([s.nsites for s in sp], np.int32)
        self.spec_nmols = np.array([s.nmols for s in sp], np.int32)
        self.spec_fw = np.array([int(s.framework) for s in sp], np.int32)
        self.spec_ids = np.concatenate([s.site_id for s in sp]).astype(np.int32)
        self.spec_pf = np.ascontiguousarray(np.concatenate([s.p_f_sites for s in sp]), np.float64)
        self.potpar = np.ascontiguousarray(sysm.potpar, np.float64)
        self.site_charge = np.ascontiguousarray(sysm.site_charge, np.float64)
        self.c_of_m = np.ascontiguousarray(sysm.c_of_m, np.float64)
        c = sysm.control
        s = _Sys()
        s.nsites, s.nmols, s.nspecies = sysm.nsites, sysm.nmols, len(sp)
        s.max_id, s.ptype = sysm.max_id, sysm.ptype
        s.spec_nsites, s.spec_nmols = _ip(self.spec_nsites), _ip(self.spec_nmols)
        s.spec_framework, s.spec_site_id = _ip(self.spec_fw), _ip(self.spec_ids)
        s.spec_pf, s.potpar = _dp(self.spec_pf), _dp(self.potpar)
        s.site_charge, s.c_of_m = _dp(self.site_charge), _dp(self.c_of_m)
        for i in range(9):
            s.h[i] = float(sysm.h[i // 3, i % 3])
        s.cutoff, s.subcell, s.alpha, s.k_cutoff = c.cutoff, c.subcell, c.alpha, c.k_cutoff
        s.strict_cutoff, s.molpbc = int(c.strict_cutoff), int(c.molpbc)
        self.s = s


@dataclass
class PortResult:
    force: np.ndarray        # [3, N]
    pe: float
    stress: np.ndarray       # [3, 3], upper triangle
    info: PortInfo
    pairs: Optional[np.ndarray] = None


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"oracle port error {rc}: {PORT_ERRORS.get(rc, '?')}")


def force_calc(sysm, nthreads: int = 1, want_pairs: bool = False, fast: bool = False,
               pairs_cap: Optional[int] = None) -> PortResult:
    L = lib(fast)
    ps = PortSystem(sysm)
    n = sysm.nsites
    site = np.ascontiguousarray(sysm.site, np.float64)
    f = np.zeros((3, n))
    pe = np.zeros(1)
    st = np.zeros(9)
    info = PortInfo()
    pairs = None
    pp, cap = None, 0
    if want_pairs:
        cap = pairs_cap or 600 * n + 100000
        pairs = np.zeros((cap, 3), np.int32)
        pp = pairs.ctypes.data_as(C.POINTER(C.c_int32))
    _check(L.port_force_calc(C.byref(ps.s), _dp(site), _dp(f), _dp(pe), _dp(st), nthreads,
                             pp, cap, C.byref(info)))
    if want_pairs:
        pairs = pairs[:info.npairs].copy()
    return PortResult(f, float(pe[0]), st.reshape(3, 3), info, pairs)


def ewald(sysm, nthreads: int = 1, k_first: int = 0, k_last: int = -1, fast: bool = False) -> PortResult:
    L = lib(fast)
    ps = PortSystem(sysm)
    n = sysm.nsites
    site = np.ascontiguousarray(sysm.site, np.float64)
    f = np.zeros((3, n))
    pe = np.zeros(1)
    st = np.zeros(9)
    info = PortInfo()
    _check(L.port_ewald(C.byref(ps.s), _dp(site), _dp(f), _dp(pe), _dp(st), nthreads,
                        k_first, k_last, C.byref(info)))
    return PortResult(f, float(pe[0]), st.reshape(3, 3), info)


def poteval(potpar8, r: float, ptype: int, chgsq: float, alpha: float) -> float:
    p = np.ascontiguousarray(potpar8, np.float64)
    return lib().port_poteval(_dp(p), r, ptype, chgsq, alpha)
