"""Constant-energy rigid-molecule dynamics on the GPU (mdgpu_md_*), with the
per-species constants and the seeded thermal start it needs.

The integrator is the reference's leapfrog step (do_step, src/accel.c:626-827,
thermostat and barostat off; src/leapfrog.c); the state is held in the
reference's layout -- fractional centres of mass, scaled momenta
mom = h^T (m v), quaternions and principal-frame angular momenta -- so a
state moves between the two unchanged.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional

import numpy as np

from . import _lib
from .forcefield import ForceField, _dp
from .system import System

#: Boltzmann's constant in program units, amu Å^2 ps^-2 K^-1 (src/defs.h:201,226)
KB = 1.380658e-23 / (1.6605402e-27 * 1.0e4)


@dataclasses.dataclass
class Dynamics:
    """Per-species constants of the equations of motion."""
    mass: np.ndarray              # [nspecies] amu
    inertia: np.ndarray           # [nspecies, 3] principal moments, amu Å^2
    rdof: np.ndarray              # [nspecies] rotational degrees of freedom
    step: float                   # timestep, ps
    nosymmetric_rot: bool = False


@dataclasses.dataclass
class MDState:
    c_of_m: np.ndarray            # [nmols, 3] fractional centres of mass
    mom: np.ndarray               # [nmols, 3] scaled momenta
    quat: np.ndarray              # [nmols_r, 4]
    amom: np.ndarray              # [nmols_r, 4], [:, 1:] principal angular momenta


def species_dynamics(sysm: System, step: float, nosymmetric_rot: bool = False) -> Dynamics:
    """Masses, principal moments and rotational freedom of every species from
    the site masses, with the principal-frame site co-ordinates as given
    (the inertia tensor must be diagonal in that frame).  A moment below
    1e-14 of the sum of the other two counts as zero (src/startup.c:540-560)."""
    if sysm.site_mass is None:
        raise ValueError("the system has no site masses")
    mass, inertia, rdof = [], [], []
    for sp in sysm.species:
        m = np.asarray(sysm.site_mass, np.float64)[sp.site_id]
        p = np.asarray(sp.p_f_sites, np.float64)
        M = float(m.sum())
        com = (m[:, None] * p).sum(0) / M if M > 0 else np.zeros(3)
        if sp.nsites > 1 and np.max(np.abs(com)) > 1e-8:
            raise ValueError(f"species {sp.name}: principal-frame sites are not centred on the centre of mass")
        I = np.array([np.sum(m * (p[:, 1] ** 2 + p[:, 2] ** 2)), np.sum(m * (p[:, 0] ** 2 + p[:, 2] ** 2)),
                      np.sum(m * (p[:, 0] ** 2 + p[:, 1] ** 2))])
        off = np.array([np.sum(m * p[:, 0] * p[:, 1]), np.sum(m * p[:, 0] * p[:, 2]), np.sum(m * p[:, 1] * p[:, 2])])
        # a framework does not rotate (src/startup.c:557-561): its sites stay
        # as given, only centred on the centre of mass
        if sp.nsites > 1 and not sp.framework and np.max(np.abs(off)) > 1e-8 * max(I.max(), 1e-30):
            raise ValueError(f"species {sp.name}: principal-frame sites are not on the principal axes")
        nz = sum(1 for i in range(3) if I[i] <= 1e-14 * (I[(i + 1) % 3] + I[(i + 2) % 3]))
        mass.append(M)
        inertia.append(I)
        rdof.append(0 if sp.nsites == 1 or sp.framework else 3 - nz)
    return Dynamics(np.array(mass), np.array(inertia), np.array(rdof, np.int32), float(step), nosymmetric_rot)


def thermal_state(sysm: System, dyn: Dynamics, temp: float, seed: int) -> MDState:
    """Seeded Maxwell-Boltzmann momenta at ``temp`` K with zero total linear
    momentum (framework molecules at rest); principal angular momenta
    L_i = I_i w_i with w_i Gaussian of variance kT/I_i.  Orientations are
    the system's (identity if it has none)."""
    rng = np.random.default_rng(seed)
    h = np.asarray(sysm.h, np.float64)
    nm = sysm.nmols
    masses = np.concatenate([np.full(sp.nmols, dyn.mass[k]) for k, sp in enumerate(sysm.species)])
    moving = np.concatenate([np.full(sp.nmols, not sp.framework) for sp in sysm.species])
    p = rng.normal(0.0, 1.0, (nm, 3)) * np.sqrt(KB * temp * masses)[:, None]
    p[~moving] = 0.0                                # a framework is held fixed
    p[moving] -= p[moving].sum(0) / max(int(moving.sum()), 1)
    mom = p @ h                                     # h^T p per molecule
    nq = int(sum(sp.nmols for k, sp in enumerate(sysm.species) if dyn.rdof[k] > 0))
    amom = np.zeros((nq, 4))
    row = 0
    for k, sp in enumerate(sysm.species):
        if dyn.rdof[k] <= 0:
            continue
        I = dyn.inertia[k]
        sd = np.sqrt(KB * temp * np.where(I > 1e-14, I, 0.0))
        amom[row:row + sp.nmols, 1:] = rng.normal(0.0, 1.0, (sp.nmols, 3)) * sd
        row += sp.nmols
    quat = np.zeros((nq, 4))
    quat[:, 0] = 1.0
    if sysm.quat is not None and nq:
        quat = np.array(sysm.quat, np.float64).reshape(nq, 4)
    return MDState(np.array(sysm.c_of_m, np.float64), mom, quat, amom)


def total_energy(energies: np.ndarray) -> np.ndarray:
    """Conserved quantity per step from mdgpu_md_run's records."""
    return energies.sum(axis=1)


class MolecularDynamics:
    """A dynamics run on one ForceField's GPU context."""

    def __init__(self, ff: ForceField, dyn: Dynamics, state: MDState):
        self.ff = ff
        self.L = ff.L
        sysm = ff.sysm
        self._dyn = (np.ascontiguousarray(dyn.mass, np.float64),
                     np.ascontiguousarray(dyn.inertia, np.float64).reshape(-1),
                     np.ascontiguousarray(dyn.rdof, np.int32))
        self.nq = int(sum(sp.nmols for k, sp in enumerate(sysm.species) if dyn.rdof[k] > 0))
        d = _lib.Dynamics(_dp(self._dyn[0]), _dp(self._dyn[1]),
                          self._dyn[2].ctypes.data_as(C.POINTER(C.c_int)), float(dyn.step),
                          int(dyn.nosymmetric_rot))
        cm = np.ascontiguousarray(state.c_of_m, np.float64)
        mo = np.ascontiguousarray(state.mom, np.float64)
        qu = np.ascontiguousarray(state.quat, np.float64)
        am = np.ascontiguousarray(state.amom, np.float64)
        h = np.ascontiguousarray(sysm.h, np.float64).reshape(9)
        ff._check(self.L.mdgpu_md_init(ff.ctx, C.byref(d), _dp(h), _dp(cm), _dp(mo),
                                       _dp(qu) if self.nq else None, _dp(am) if self.nq else None))

    def run(self, nsteps: int) -> np.ndarray:
        """Advance nsteps; returns per-step [pe_real, pe_ewald, ke_trans, ke_rot]."""
        e = np.zeros((max(nsteps, 1), 4))
        self.ff._check(self.L.mdgpu_md_run(self.ff.ctx, int(nsteps), _dp(e)))
        return e[:nsteps]

    def run_dump(self, nsteps: int, interval: int, level: int, first: int = 1):
        """Advance nsteps as run() and return (energies, records): a dump
        record ([mdgpu_dump_size] float32, the layout of dump_convert,
        src/dump.c:550-620) after step k when k >= first and
        (k - first) % interval == 0, converted on the GPU."""
        nrec = (nsteps - first) // interval + 1 if nsteps >= first else 0
        size = self.L.mdgpu_dump_size(int(level), self.ff.sysm.nmols, self.nq)
        rec = np.zeros((max(nrec, 1), max(size, 1)), np.float32)
        e = np.zeros((max(nsteps, 1), 4))
        self.ff._check(self.L.mdgpu_md_run_dump(self.ff.ctx, int(nsteps), int(first), int(interval), int(level),
                                                _dp(e), rec.ctypes.data_as(C.POINTER(C.c_float))))
        return e[:nsteps], rec[:nrec]

    def set_state(self, state: MDState) -> None:
        """Replaces the dynamic state on the GPU (mdgpu_md_set_state)."""
        cm = np.ascontiguousarray(state.c_of_m, np.float64)
        mo = np.ascontiguousarray(state.mom, np.float64)
        qu = np.ascontiguousarray(state.quat, np.float64)
        am = np.ascontiguousarray(state.amom, np.float64)
        self.ff._check(self.L.mdgpu_md_set_state(self.ff.ctx, _dp(cm), _dp(mo), _dp(qu) if self.nq else None,
                                                 _dp(am) if self.nq else None))

    def set_thermostat(self, temp: float, ttmass: float, ts: float = 1.0, tsmom: float = 0.0,
                       enable: bool = True) -> None:
        """Constant temperature (mdgpu_md_set_thermostat): the Nose-Poincare
        thermostat of do_step under const-temp, temp in K, ttmass in program
        units; H_0 is evaluated on the next step."""
        self.ff._check(self.L.mdgpu_md_set_thermostat(self.ff.ctx, int(enable), float(temp), float(ttmass),
                                                      float(ts), float(tsmom)))

    def set_barostat(self, mode: int, pressure: float, pmass: float, strain_mask: int = 200,
                     hmom: Optional[np.ndarray] = None) -> None:
        """Constant pressure (mdgpu_md_set_barostat): the Parrinello-Rahman
        cell dynamics of do_step, mode 1 anisotropic or 2 uniform (0 off),
        pressure and cell mass W in program units, the reference's strain
        mask."""
        hm = None if hmom is None else np.ascontiguousarray(hmom, np.float64).reshape(9)
        self.ff._check(self.L.mdgpu_md_set_barostat(self.ff.ctx, int(mode), float(pressure), float(pmass),
                                                    int(strain_mask), _dp(hm) if hm is not None else None))

    def cell(self):
        """(h, its momentum) now, [3, 3] each."""
        h, hm = np.zeros(9), np.zeros(9)
        self.ff._check(self.L.mdgpu_md_get_barostat(self.ff.ctx, _dp(h), _dp(hm)))
        return h.reshape(3, 3), hm.reshape(3, 3)

    def thermostat(self):
        """(ts, tsmom, H_0) after the last step."""
        out = np.zeros(3)
        self.ff._check(self.L.mdgpu_md_get_thermostat(self.ff.ctx, _dp(out)))
        return float(out[0]), float(out[1]), float(out[2])

    def state(self) -> MDState:
        sysm = self.ff.sysm
        cm, mo = np.zeros((sysm.nmols, 3)), np.zeros((sysm.nmols, 3))
        qu, am = np.zeros((self.nq, 4)), np.zeros((self.nq, 4))
        self.ff._check(self.L.mdgpu_md_get_state(self.ff.ctx, _dp(cm), _dp(mo),
                                                 _dp(qu) if self.nq else None, _dp(am) if self.nq else None))
        return MDState(cm, mo, qu, am)


def ns_per_day(steps_per_s: float, step_ps: float) -> float:
    return steps_per_s * step_ps * 86400.0 / 1000.0


def drift_per_ns(energies: np.ndarray, step_ps: float, nmols: Optional[int] = None) -> float:
    """Least-squares slope of the conserved quantity, per ns (per molecule
    when nmols is given), in program energy units."""
    H = total_energy(energies)
    t = np.arange(len(H)) * step_ps * 1e-3
    slope = float(np.polyfit(t, H, 1)[0]) if len(H) > 1 else 0.0
    return slope / nmols if nmols else slope



def restart_state(data: bytes, nspecies: int, nmols: int, nmols_r: int) -> MDState:
    """The dynamic state held in a restart file the reference wrote in its
    native format, to start GPU dynamics from (mdgpu_md_init/set_state).

    The file is a sequence of records, each an unsigned long byte count
    (8 bytes, little-endian on LP64 hosts) followed by that many bytes
    (cwrite, src/restart.c:183-191).  write_restart (src/restart.c:435-548)
    writes the header, the control record, the system record, the species
    records, then per species the principal-frame sites and site ids, the
    site table and the potential table, and then the dynamic variables:
    c_of_m, mom, momp, and with rotating molecules quat, amom, amomp."""
    recs, o = [], 0
    while o + 8 <= len(data):
        n = int.from_bytes(data[o:o + 8], "little")
        recs.append((o + 8, n))
        o += 8 + n
    first = 3 + 1 + 2 * nspecies + 2          # header, control, system, species, per-species pairs, sites, pots

    def arr(k, shape):
        off, n = recs[first + k]
        want = 8 * int(np.prod(shape))
        if n != want:
            raise ValueError(f"restart record {first + k}: {n} bytes, expected {want}")
        return np.frombuffer(data, "<f8", count=want // 8, offset=off).reshape(shape).copy()

    cm, mo = arr(0, (nmols, 3)), arr(1, (nmols, 3))
    if nmols_r > 0:
        qu, am = arr(3, (nmols_r, 4)), arr(4, (nmols_r, 4))
    else:
        qu, am = np.zeros((0, 4)), np.zeros((0, 4))
    return MDState(cm, mo, qu, am)
