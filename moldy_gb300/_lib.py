"""ctypes binding of libmoldy_gb300.so (include/moldy_gb300.h).

The library is built in-tree by moldy_gb300/build.py.  Loading fails loudly
when it is missing: there is no CPU fallback for the force path.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmoldy_gb300.so")

STATUS = {0: "MDGPU_OK", 1: "MDGPU_E_ARG", 2: "MDGPU_E_CUDA", 3: "MDGPU_E_UNSUPPORTED",
          4: "MDGPU_E_CUTOFF", 5: "MDGPU_E_RANGE", 6: "MDGPU_E_PTYPE", 7: "MDGPU_E_CAPACITY",
          8: "MDGPU_E_NOMEM", 9: "MDGPU_E_IO"}
FP64, MIXED = 0, 1

#: every function include/*.h declares, with the library that must export it
EXPORTS = ["mdgpu_create", "mdgpu_destroy", "mdgpu_last_error", "mdgpu_set_precision",
           "mdgpu_set_stream", "mdgpu_get_stream", "mdgpu_set_system", "mdgpu_set_control",
           "mdgpu_force_calc", "mdgpu_ewald", "mdgpu_forces", "mdgpu_forces_device",
           "mdgpu_synchronize", "mdgpu_get_info", "mdgpu_pair_keys", "mdgpu_poteval",
           "mdgpu_set_phase_timing", "mdgpu_phase_times", "mdgpu_fma_peak", "mdgpu_tc_probe", "mdgpu_tc_rate", "mdgpu_tc_items", "mdgpu_stencil_columns",
           "mdgpu_ewald_kspace_noalloc", "mdgpu_set_params", "mdgpu_energy_grad",
           "mdgpu_fm_loss_grad", "mdgpu_md_init", "mdgpu_md_run", "mdgpu_md_get_state", "mdgpu_md_set_state",
           "mdgpu_md_set_thermostat", "mdgpu_md_get_thermostat", "mdgpu_md_set_barostat",
           "mdgpu_md_get_barostat",
           "mdgpu_rdf_counts", "mdgpu_dump_size", "mdgpu_md_run_dump", "mdgpu_dump_open",
           "mdgpu_dump_append", "mdgpu_dump_filename", "mdgpu_dump_errmsg", "mdgpu_dump_close",
           "force_calc", "ewald", "poteval"]


class MdgpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Species(C.Structure):
    _fields_ = [("nsites", C.c_int), ("nmols", C.c_int), ("framework", C.c_int),
                ("site_id", C.POINTER(C.c_int)), ("p_f_sites", C.POINTER(C.c_double))]


class SystemDesc(C.Structure):
    _fields_ = [("nspecies", C.c_int), ("species", C.POINTER(Species)), ("max_id", C.c_int),
                ("ptype", C.c_int), ("potpar", C.POINTER(C.c_double)), ("chg", C.POINTER(C.c_double))]


class ControlDesc(C.Structure):
    _fields_ = [("cutoff", C.c_double), ("subcell", C.c_double), ("alpha", C.c_double),
                ("k_cutoff", C.c_double), ("strict_cutoff", C.c_int), ("molpbc", C.c_int)]


class Info(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("n_nabors", C.c_int),
                ("nkvec", C.c_int), ("hmax", C.c_int), ("kmax", C.c_int), ("lmax", C.c_int),
                ("eintra", C.c_double), ("self_energy", C.c_double), ("sheet_energy", C.c_double),
                ("npairs", C.c_int64), ("n_too_close", C.c_int64),
                ("too_close", (C.c_int32 * 2) * 16), ("launches", C.c_int64)]


class Params(C.Structure):
    _fields_ = [("potpar", C.POINTER(C.c_double)), ("chg", C.POINTER(C.c_double)), ("alpha", C.c_double)]


class Grad(C.Structure):
    _fields_ = [("potpar", C.POINTER(C.c_double)), ("chg", C.POINTER(C.c_double)), ("alpha", C.c_double)]


class Dynamics(C.Structure):
    _fields_ = [("mass", C.POINTER(C.c_double)), ("inertia", C.POINTER(C.c_double)),
                ("rdof", C.POINTER(C.c_int)), ("step", C.c_double), ("nosymmetric_rot", C.c_int)]


class DumpSpecies(C.Structure):
    """mol_mt of the reference's dump header (src/structs.h:220-230)."""
    _fields_ = [("inertia", C.c_float * 3), ("mass", C.c_float), ("dipole", C.c_float),
                ("charge", C.c_float), ("nmols", C.c_int), ("rdof", C.c_int), ("framework", C.c_int),
                ("name", C.c_char * 32)]


class DumpInfo(C.Structure):
    _fields_ = [("title", C.c_char_p), ("istep", C.c_long), ("dump_interval", C.c_long),
                ("dump_level", C.c_int), ("maxdumps", C.c_int), ("deltat", C.c_float),
                ("nmols", C.c_int), ("nmols_r", C.c_int), ("nspecies", C.c_int),
                ("species", C.POINTER(DumpSpecies)), ("xdr", C.c_int), ("dump_init", C.c_ulong),
                ("restart_timestamp", C.c_ulong)]


NPOTP = 8
ADJ_MAX_ID = 16
NPHASES = 7
PHASES = ["cells", "pairs", "kprep", "sfac", "kreduce", "kforce", "final"]


_lib = None


def load():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m moldy_gb300.build` "
                          "(the force path has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.c_int
    dpp = C.POINTER(dp)
    sig = {
        "mdgpu_create": ([C.POINTER(vp), ip, ip], ip),
        "mdgpu_destroy": ([vp], None),
        "mdgpu_last_error": ([vp], C.c_char_p),
        "mdgpu_set_precision": ([vp, ip], ip),
        "mdgpu_set_stream": ([vp, vp], ip),
        "mdgpu_get_stream": ([vp, C.POINTER(vp)], ip),
        "mdgpu_set_system": ([vp, C.POINTER(SystemDesc)], ip),
        "mdgpu_set_control": ([vp, C.POINTER(ControlDesc)], ip),
        "mdgpu_force_calc": ([vp, dp, dpp, dpp, dp, dp, dp], ip),
        "mdgpu_ewald": ([vp, dp, dpp, dpp, dp, dp], ip),
        "mdgpu_forces": ([vp, dp, dp, dp, dp, dp, dp], ip),
        "mdgpu_forces_device": ([vp, dp, vp, vp, vp, vp, vp], ip),
        "mdgpu_synchronize": ([vp], ip),
        "mdgpu_get_info": ([vp, C.POINTER(Info)], ip),
        "mdgpu_pair_keys": ([vp, dp, dp, dp, C.POINTER(C.c_uint64), C.c_int64,
                             C.POINTER(C.c_int64)], ip),
        "mdgpu_poteval": ([dp, C.c_double, ip, C.c_double, C.c_double], C.c_double),
        "mdgpu_set_phase_timing": ([vp, ip], ip),
        "mdgpu_phase_times": ([vp, dp], ip),
        "mdgpu_fma_peak": ([ip, ip, dp], ip),
        "mdgpu_tc_probe": ([ip, vp, vp, vp, vp, ip, ip, vp], ip),
        "mdgpu_tc_rate": ([ip, ip, ip, ip, ip, ip, dp], ip),
        "mdgpu_tc_items": ([dp, C.POINTER(ControlDesc), vp, vp, ip, C.POINTER(ip), C.POINTER(ip)], ip),
        "mdgpu_stencil_columns": ([dp, C.POINTER(ControlDesc), vp, vp, C.POINTER(ip), vp, vp, C.POINTER(ip), ip],
                                  ip),
        "mdgpu_ewald_kspace_noalloc": ([dp, ip, vp, vp, C.c_double, C.c_double, vp, vp, vp, vp], ip),
        "mdgpu_set_params": ([vp, C.POINTER(Params)], ip),
        "mdgpu_md_init": ([vp, C.POINTER(Dynamics), dp, dp, dp, dp, dp], ip),
        "mdgpu_md_run": ([vp, ip, dp], ip),
        "mdgpu_md_get_state": ([vp, dp, dp, dp, dp], ip),
        "mdgpu_md_set_state": ([vp, dp, dp, dp, dp], ip),
        "mdgpu_md_set_thermostat": ([vp, ip, C.c_double, C.c_double, C.c_double, C.c_double], ip),
        "mdgpu_md_get_thermostat": ([vp, dp], ip),
        "mdgpu_md_set_barostat": ([vp, ip, C.c_double, C.c_double, ip, dp], ip),
        "mdgpu_md_get_barostat": ([vp, dp, dp], ip),
        "mdgpu_dump_size": ([ip, ip, ip], ip),
        "mdgpu_md_run_dump": ([vp, ip, ip, ip, ip, dp, C.POINTER(C.c_float)], ip),
        "mdgpu_dump_open": ([C.POINTER(vp), C.c_char_p, C.POINTER(DumpInfo)], ip),
        "mdgpu_dump_append": ([vp, C.POINTER(C.c_float)], ip),
        "mdgpu_dump_filename": ([vp], C.c_char_p),
        "mdgpu_dump_errmsg": ([vp], C.c_char_p),
        "mdgpu_dump_close": ([vp], None),
        "mdgpu_rdf_counts": ([vp, dp, dp, dp, C.c_double, ip, C.POINTER(C.c_uint64)], ip),
        "mdgpu_energy_grad": ([vp, C.POINTER(Params), dp, dp, dp, dp, C.POINTER(Grad)], ip),
        "mdgpu_fm_loss_grad": ([vp, C.POINTER(Params), dp, dp, dp, dp, C.c_double, dp, C.POINTER(Grad)], ip),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L
