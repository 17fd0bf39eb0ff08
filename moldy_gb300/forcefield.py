"""Host-side interface of the GPU force path, mirroring Moldy's own entry
points for it: ``force_calc`` (src/force.c:1108), ``ewald``
(src/ewald.c:280) and ``poteval`` (src/force.c:632), with the same argument
meaning and accumulate-into semantics, over the C ABI of libmoldy_gb300.so.

Errors the reference reports as FATAL (unknown potential type, cutoff beyond
one periodic image, co-ordinates outside the cell) raise
:class:`moldy_gb300._lib.MdgpuError` here.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np

from . import _lib
from ._lib import MdgpuError
from .system import System


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class ForceField:
    """One GPU context bound to one :class:`System` description.

    ``precision`` is ``"fp64"`` or ``"mixed"`` (FP32 pair and k-space
    arithmetic, FP64 accumulation)."""

    def __init__(self, sysm: System, precision: str = "mixed", device: int = 0):
        self.L = _lib.load()
        self._prec = {"fp64": _lib.FP64, "mixed": _lib.MIXED}[precision]
        ctx = C.c_void_p()
        st = self.L.mdgpu_create(C.byref(ctx), device, self._prec)
        if st != 0:
            raise MdgpuError(st, f"cannot create a context on CUDA device {device}")
        self.ctx = ctx
        self.sysm = None
        self.set_system(sysm)

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "ctx", None):
            self.L.mdgpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != 0:
            raise MdgpuError(st, self.L.mdgpu_last_error(self.ctx).decode())

    # -- configuration -----------------------------------------------------
    def set_system(self, sysm: System):
        """Describe the system (and control keys); the next call recomputes
        the first-call constants as a fresh reference run does."""
        self.sysm = sysm
        sp = sysm.species
        self._ids = [np.ascontiguousarray(s.site_id, np.int32) for s in sp]
        self._pf = [np.ascontiguousarray(s.p_f_sites, np.float64) for s in sp]
        arr = (_lib.Species * len(sp))()
        for k, s in enumerate(sp):
            arr[k].nsites, arr[k].nmols, arr[k].framework = s.nsites, s.nmols, int(s.framework)
            arr[k].site_id = self._ids[k].ctypes.data_as(C.POINTER(C.c_int))
            arr[k].p_f_sites = _dp(self._pf[k])
        self._spec = arr
        self._pot = np.ascontiguousarray(sysm.potpar, np.float64)
        self._chg = np.ascontiguousarray(sysm.chg(), np.float64)
        d = _lib.SystemDesc(len(sp), arr, sysm.max_id, sysm.ptype, _dp(self._pot), _dp(self._chg))
        self._check(self.L.mdgpu_set_system(self.ctx, C.byref(d)))
        self.set_control(sysm.control)

    def set_control(self, c):
        d = _lib.ControlDesc(c.cutoff, c.subcell, c.alpha, c.k_cutoff, int(c.strict_cutoff), int(c.molpbc))
        self._check(self.L.mdgpu_set_control(self.ctx, C.byref(d)))

    def set_precision(self, precision: str):
        self._prec = {"fp64": _lib.FP64, "mixed": _lib.MIXED}[precision]
        self._check(self.L.mdgpu_set_precision(self.ctx, self._prec))

    def set_stream(self, stream_ptr: int):
        self._check(self.L.mdgpu_set_stream(self.ctx, C.c_void_p(stream_ptr)))

    # -- evaluation ----------------------------------------------------------
    def _h(self):
        return np.ascontiguousarray(self.sysm.h, np.float64).reshape(9)

    def force_calc(self, site: Optional[np.ndarray] = None, site_force: Optional[np.ndarray] = None,
                   pe: float = 0.0, stress: Optional[np.ndarray] = None):
        """Real-space part with force_calc's semantics: returns
        (site_force + F_real, pe + U_real - eintra, stress + virial)."""
        site = np.ascontiguousarray(self.sysm.site if site is None else site, np.float64)
        n = site.shape[1]
        f = np.zeros((3, n)) if site_force is None else np.array(site_force, np.float64, copy=True)
        st = np.zeros(9) if stress is None else np.array(stress, np.float64, copy=True).reshape(9)
        pe_a = np.array([pe], np.float64)
        sp = (C.POINTER(C.c_double) * 3)(*[_dp(site[k]) for k in range(3)])
        fp = (C.POINTER(C.c_double) * 3)(*[_dp(f[k]) for k in range(3)])
        cm = np.ascontiguousarray(self.sysm.c_of_m, np.float64)
        self._check(self.L.mdgpu_force_calc(self.ctx, _dp(self._h()), sp, fp, _dp(cm), _dp(pe_a), _dp(st)))
        return f, float(pe_a[0]), st.reshape(3, 3)

    def ewald(self, site: Optional[np.ndarray] = None, site_force: Optional[np.ndarray] = None,
              pe: float = 0.0, stress: Optional[np.ndarray] = None):
        """Reciprocal-space part with ewald's semantics."""
        site = np.ascontiguousarray(self.sysm.site if site is None else site, np.float64)
        n = site.shape[1]
        f = np.zeros((3, n)) if site_force is None else np.array(site_force, np.float64, copy=True)
        st = np.zeros(9) if stress is None else np.array(stress, np.float64, copy=True).reshape(9)
        pe_a = np.array([pe], np.float64)
        sp = (C.POINTER(C.c_double) * 3)(*[_dp(site[k]) for k in range(3)])
        fp = (C.POINTER(C.c_double) * 3)(*[_dp(f[k]) for k in range(3)])
        self._check(self.L.mdgpu_ewald(self.ctx, _dp(self._h()), sp, fp, _dp(pe_a), _dp(st)))
        return f, float(pe_a[0]), st.reshape(3, 3)

    def forces(self, site: Optional[np.ndarray] = None, c_of_m: Optional[np.ndarray] = None
               ) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Both parts in one call: (total site force [3,N], pe[2], stress[3,3])."""
        site = np.ascontiguousarray(self.sysm.site if site is None else site, np.float64)
        cm = np.ascontiguousarray(self.sysm.c_of_m if c_of_m is None else c_of_m, np.float64)
        f = np.empty_like(site)
        pe = np.zeros(2)
        st = np.zeros(9)
        self._check(self.L.mdgpu_forces(self.ctx, _dp(self._h()), _dp(site), _dp(cm), _dp(f), _dp(pe), _dp(st)))
        return f, pe, st.reshape(3, 3)

    def forces_device(self, d_site: int, d_force: int, d_pe: int, d_stress: int, d_cofm: int = 0):
        """Device-pointer variant (asynchronous on the context's stream)."""
        self._check(self.L.mdgpu_forces_device(self.ctx, _dp(self._h()), C.c_void_p(d_site),
                                               C.c_void_p(d_cofm or None), C.c_void_p(d_force),
                                               C.c_void_p(d_pe), C.c_void_p(d_stress)))

    def synchronize(self):
        self._check(self.L.mdgpu_synchronize(self.ctx))

    def set_phase_timing(self, on: bool):
        self._check(self.L.mdgpu_set_phase_timing(self.ctx, int(on)))

    def phase_times(self) -> dict:
        """Milliseconds of each phase of the last evaluation (CUDA events)."""
        ms = np.zeros(_lib.NPHASES)
        self._check(self.L.mdgpu_phase_times(self.ctx, _dp(ms)))
        return dict(zip(_lib.PHASES, ms.tolist()))

    def pair_keys(self, site: Optional[np.ndarray] = None, cap: Optional[int] = None) -> np.ndarray:
        """Sorted canonical keys of the evaluated pair set (moldy_gb300.pairset)."""
        site = np.ascontiguousarray(self.sysm.site if site is None else site, np.float64)
        cm = np.ascontiguousarray(self.sysm.c_of_m, np.float64)
        cap = cap or 400 * site.shape[1] + 100000
        keys = np.empty(cap, np.uint64)
        cnt = C.c_int64()
        st = self.L.mdgpu_pair_keys(self.ctx, _dp(self._h()), _dp(site), _dp(cm),
                                    keys.ctypes.data_as(C.POINTER(C.c_uint64)), cap, C.byref(cnt))
        if st == 7:
            return self.pair_keys(site, cap=int(cnt.value) + 1)
        self._check(st)
        return np.sort(keys[:cnt.value])

    def rdf_counts(self, limit: float, nbins: int, site: Optional[np.ndarray] = None,
                   c_of_m: Optional[np.ndarray] = None) -> np.ndarray:
        """Unordered site-pair counts [max_id, max_id, nbins] of the
        reference's RDF accumulation (bin = int(nbins/limit * r))."""
        site = np.ascontiguousarray(self.sysm.site if site is None else site, np.float64)
        cm = np.ascontiguousarray(self.sysm.c_of_m if c_of_m is None else c_of_m, np.float64)
        M = self.sysm.max_id
        out = np.zeros(M * M * nbins, np.uint64)
        self._check(self.L.mdgpu_rdf_counts(self.ctx, _dp(self._h()), _dp(site), _dp(cm), float(limit), int(nbins),
                                            out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out.reshape(M, M, nbins)

    # -- adjoint -------------------------------------------------------------
    def _params(self, potpar, chg, alpha):
        keep = []
        P = _lib.Params(None, None, float(alpha) if alpha is not None else 0.0)
        if potpar is not None:
            a = np.ascontiguousarray(potpar, np.float64).reshape(-1)
            if a.size != self.sysm.max_id ** 2 * _lib.NPOTP:
                raise ValueError("potpar must hold max_id*max_id*8 values")
            keep.append(a)
            P.potpar = _dp(a)
        if chg is not None:
            a = np.ascontiguousarray(chg, np.float64).reshape(-1)
            if a.size != self.sysm.nsites:
                raise ValueError("chg must hold one charge per site")
            keep.append(a)
            P.chg = _dp(a)
        return P, keep

    def set_params(self, potpar=None, chg=None, alpha=None):
        """Replace the potential table, the site charges and/or alpha (None
        keeps the current value); the cutoffs and the k-vector list stay."""
        P, keep = self._params(potpar, chg, alpha)
        self._check(self.L.mdgpu_set_params(self.ctx, C.byref(P)))

    def _grad_call(self, loss: bool, site, c_of_m, f_ref=None, weight=1.0):
        site = np.ascontiguousarray(self.sysm.site if site is None else site, np.float64)
        cm = np.ascontiguousarray(self.sysm.c_of_m if c_of_m is None else c_of_m, np.float64)
        M, N = self.sysm.max_id, site.shape[1]
        gp = np.zeros(M * M * _lib.NPOTP)
        gq = np.zeros(N)
        G = _lib.Grad(_dp(gp), _dp(gq), 0.0)
        val = np.zeros(1)
        if loss:
            fr = np.ascontiguousarray(f_ref, np.float64)
            self._check(self.L.mdgpu_fm_loss_grad(self.ctx, None, _dp(self._h()), _dp(site), _dp(cm), _dp(fr),
                                                  float(weight), _dp(val), C.byref(G)))
        else:
            self._check(self.L.mdgpu_energy_grad(self.ctx, None, _dp(self._h()), _dp(site), _dp(cm), _dp(val),
                                                 C.byref(G)))
        return float(val[0]), {"potpar": gp.reshape(M, M, _lib.NPOTP), "chg": gq, "alpha": float(G.alpha)}

    def energy_grad(self, site: Optional[np.ndarray] = None, c_of_m: Optional[np.ndarray] = None):
        """Potential energy pe[0] + pe[1] and its gradient with respect to
        the potential table ([max_id, max_id, 8]; entry [a, b] as the force
        on a site of id a from one of id b reads it), the site charges and
        alpha, at the current parameters."""
        return self._grad_call(False, site, c_of_m)

    def fm_loss_grad(self, f_ref: np.ndarray, weight: float = 1.0, site: Optional[np.ndarray] = None,
                     c_of_m: Optional[np.ndarray] = None):
        """Force-matching loss weight * sum |F - f_ref|^2 and its gradient
        (same layout as energy_grad)."""
        return self._grad_call(True, site, c_of_m, f_ref, weight)

    def info(self) -> dict:
        i = _lib.Info()
        self._check(self.L.mdgpu_get_info(self.ctx, C.byref(i)))
        return {k: getattr(i, k) for k, _ in _lib.Info._fields_ if k != "too_close"} | {
            "too_close": [(i.too_close[k][0], i.too_close[k][1]) for k in range(min(16, i.n_too_close))]}


def poteval(potpar, r: float, ptype: int, chgsq: float, alpha: float) -> float:
    """Potential at one distance (poteval, src/force.c:632-650)."""
    p = np.ascontiguousarray(potpar, np.float64)
    return _lib.load().mdgpu_poteval(_dp(p), r, ptype, chgsq, alpha)
