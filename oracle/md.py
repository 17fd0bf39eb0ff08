"""Runs the reference's own constant-energy dynamics (oracle/ref_md.c, do_step
of src/accel.c:626-827 compiled from the reference sources by
oracle/build_ref.sh) from a given state.

TEST INFRASTRUCTURE ONLY: it makes the golden trajectories the GPU
integrator is checked against (tests/golden/make_md_golden.py).  The product
path never imports this module.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile
from typing import Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")


def write_mdstate(path: str, sysm, dyn, state, nsteps: int) -> None:
    c = sysm.control
    with open(path, "wb") as f:
        f.write(b"MDSTAT1\0")
        f.write(struct.pack("<10i", sysm.nsites, sysm.nmols, len(sysm.species), sysm.max_id, sysm.ptype,
                            int(c.strict_cutoff), int(c.molpbc), int(dyn.nosymmetric_rot), int(nsteps), 0))
        f.write(struct.pack("<5d", c.cutoff, c.subcell, c.alpha, c.k_cutoff, dyn.step))
        f.write(np.ascontiguousarray(sysm.h, "<f8").tobytes())
        for k, sp in enumerate(sysm.species):
            f.write(struct.pack("<4i", sp.nsites, sp.nmols, int(sp.framework), int(dyn.rdof[k])))
            f.write(np.ascontiguousarray(sp.site_id, "<i4").tobytes())
            f.write(np.ascontiguousarray(sp.p_f_sites, "<f8").tobytes())
            f.write(struct.pack("<4d", dyn.mass[k], *dyn.inertia[k]))
        f.write(np.ascontiguousarray(sysm.potpar, "<f8").tobytes())
        f.write(np.ascontiguousarray(sysm.site_charge, "<f8").tobytes())
        for a in (state.c_of_m, state.mom, state.quat, state.amom):
            f.write(np.ascontiguousarray(a, "<f8").tobytes())


def run(sysm, dyn, state, nsteps: int, fast: bool = False, dump=None, restart_out=None, restart_in=None,
        const_temp=None, const_pressure=None):
    """(records [nsteps, 3] = (H_0, pe[0], pe[1]) per step, final MDState,
    seconds per step).  The reference prints its notes to stdout.

    dump = (name, level, interval, ndumps, title) has the reference write
    its dump files (from step 1); they are returned as a fourth item,
    {file name: bytes}.  restart_out: path the reference's write_restart
    saves the final state to; restart_in: a restart file whose dynamic
    state, read back by the reference's own reader, replaces `state`.
    const_temp = (T, Q): the reference's Nose-Poincare thermostat at T (K)
    with thermostat mass Q; the records are then [nsteps, 5] = (H_0, pe[0],
    pe[1], ts, tsmom).  const_pressure = (mode, pressure, W, strain_mask):
    the reference's Parrinello-Rahman cell dynamics (mode 1 anisotropic, 2
    uniform); the records are then [nsteps, 23], h and its momentum
    (row-major 3x3 each) after (H_0, pe[0], pe[1], ts, tsmom)."""
    from moldy_gb300.dynamics import MDState
    exe = os.path.join(REF, "moldy_ref_md_fast" if fast else "moldy_ref_md")
    if not os.path.exists(exe):
        raise FileNotFoundError(f"{exe}: build it with oracle/build_ref.sh")
    nm, nq = sysm.nmols, len(state.quat)
    with tempfile.TemporaryDirectory() as d:
        pin, pout = os.path.join(d, "in.mdstate"), os.path.join(d, "out.bin")
        write_mdstate(pin, sysm, dyn, state, nsteps)
        args = [exe, pin, pout] + ([str(x) for x in dump] if dump else [])
        env = dict(os.environ)
        if restart_out:
            env["MOLDY_REF_RESTART_OUT"] = os.path.abspath(restart_out)
        if restart_in:
            env["MOLDY_REF_RESTART_IN"] = os.path.abspath(restart_in)
        if const_temp:
            env["MOLDY_REF_CONST_TEMP"] = "%.17g %.17g" % tuple(const_temp)
        if const_pressure:
            env["MOLDY_REF_CONST_PRESSURE"] = "%d %.17g %.17g %d" % tuple(const_pressure)
        subprocess.run(args, check=True, cwd=d, stdout=subprocess.DEVNULL, env=env)
        raw = np.fromfile(pout, "<f8")
        files = {}
        if dump:
            for fn in sorted(os.listdir(d)):
                if fn not in ("in.mdstate", "out.bin"):
                    with open(os.path.join(d, fn), "rb") as fh:
                        files[fn] = fh.read()
    w = 23 if const_pressure else 5 if const_temp else 3
    o = w * nsteps
    rec = raw[:o].reshape(nsteps, w)
    cm = raw[o:o + 3 * nm].reshape(nm, 3)
    o += 3 * nm
    mo = raw[o:o + 3 * nm].reshape(nm, 3)
    o += 3 * nm
    qu = raw[o:o + 4 * nq].reshape(nq, 4)
    o += 4 * nq
    am = raw[o:o + 4 * nq].reshape(nq, 4)
    o += 4 * nq
    if dump:
        return rec, MDState(cm, mo, qu, am), float(raw[o]), files
    return rec, MDState(cm, mo, qu, am), float(raw[o])
