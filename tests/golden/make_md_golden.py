"""Generate the dynamics fixtures tests/golden/md_*.npz from the reference's
own constant-energy integrator (do_step, driven by oracle/ref_md.c, built in
place from the reference sources by oracle/build_ref.sh).

Each short fixture holds a System, the per-species constants (mass,
principal moments, rotational freedom), the timestep, a seeded thermal
start (moldy_gb300.dynamics.thermal_state), the reference's per-step
records (H_0 at the half kick, pe[0], pe[1]) and its final state.

The drift fixtures (md_drift_*) hold the reference's conserved quantity
every step of a long run (10^4 steps of 2048-site water at 1 fs, lazy and
strict cutoffs; 1000 steps of 500-atom argon at 10 fs) and its CPU time per
step, for the energy-drift comparison.

The framework fixture (md_waterwall) holds rigid water over a fixed,
charged framework molecule: the reference zeroes the framework's momentum
after each step's kicks (src/accel.c:748-755).

The constant-temperature fixtures (md_nvt_*) hold runs of the reference's
Nose-Poincare thermostat (const-temp 1): per step (H_0, pe[0], pe[1], ts,
tsmom).

The constant-pressure fixtures (md_npt_*) hold runs of the reference's
Parrinello-Rahman cell dynamics (const-pressure 1 and 2, the second with the
thermostat): per step (H_0, pe[0], pe[1], ts, tsmom, h[3][3], hmom[3][3]).

The restart fixture (md_restart_water864) holds a restart file the
reference's write_restart saved after 10 steps from the thermal start, the
state those steps reached, and the reference's next 10 steps from that file
as its own reader (re_re_header, re_re_sysdef, read_restart) reads it back.

usage: python tests/golden/make_md_golden.py [--skip-drift] [--only NAME | --only drift-extra |
                                                --only drift-more]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import dataclasses  # noqa: E402

import numpy as np  # noqa: E402

from moldy_gb300 import system as S  # noqa: E402
from moldy_gb300.dynamics import species_dynamics, thermal_state  # noqa: E402
from oracle import md  # noqa: E402


def case(sysm, step, temp, seed, nsteps, nosym=False):
    dyn = species_dynamics(sysm, step, nosym)
    st = thermal_state(sysm, dyn, temp, seed)
    rec, fin, sec = md.run(sysm, dyn, st, nsteps)
    return dyn, st, rec, fin, sec


def save(name, sysm, dyn, st, rec, fin, sec, temp, seed, **extra):
    S.save_npz(os.path.join(HERE, name + ".npz"), sysm,
               md_mass=dyn.mass, md_inertia=dyn.inertia, md_rdof=dyn.rdof, md_step=dyn.step,
               md_nosym=int(dyn.nosymmetric_rot), md_temp=temp, md_seed=seed,
               c_of_m0=st.c_of_m, mom0=st.mom, quat0=st.quat, amom0=st.amom,
               ref_rec=rec, c_of_m1=fin.c_of_m, mom1=fin.mom, quat1=fin.quat, amom1=fin.amom,
               ref_sec_per_step=sec, **extra)
    print(name, sysm.nsites, "sites", len(rec), "steps", "%.3g s/step" % sec)


def _drift_more(job):
    strict, tag, seed = job
    w2 = S.water(nside=8, seed=11)
    s = dataclasses.replace(w2, control=dataclasses.replace(w2.control, strict_cutoff=strict))
    dyn, st, rec, fin, sec = case(s, 0.001, 300.0, seed, 10000)
    save("md_drift_water2048" + ("_strict" if strict else "") + "_" + tag, s, dyn, st, rec[::10], fin, sec, 300.0,
         seed, rec_stride=10)


def main():
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    ww = S.water_on_framework()
    if only in (None, "md_waterwall"):
        save("md_waterwall", ww, *case(ww, 0.001, 300.0, 9, 30), 300.0, 9)
    if only == "drift-more":
        # five more thermal starts of each water drift run, kept every 10th
        # step (the drift is a least-squares slope over the whole run), so
        # that each mean is taken over eight starts
        import multiprocessing as mp
        jobs = [(strict, tag, seed) for strict in (False, True)
                for tag, seed in (("d", 42), ("e", 52), ("f", 62), ("g", 72), ("h", 82))]
        with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
            pool.map(_drift_more, jobs)
        return
    if only == "drift-extra":
        # two more independent thermal starts of each drift run: the drift of
        # a 10^4-step run is a noisy quantity, compared as a mean over starts
        w2 = S.water(nside=8, seed=11)
        for strict in (False, True):
            s = dataclasses.replace(w2, control=dataclasses.replace(w2.control, strict_cutoff=strict))
            for tag, seed in (("b", 22), ("c", 32)):
                dyn, st, rec, fin, sec = case(s, 0.001, 300.0, seed, 10000)
                save("md_drift_water2048" + ("_strict" if strict else "") + "_" + tag, s, dyn, st, rec, fin, sec,
                     300.0, seed)
        return
    if only in (None, "md_nvt"):
        # constant temperature: the reference's Nose-Poincare thermostat
        # (const-temp 1, 250 K from a 300 K start, thermostat mass 1e4 in
        # program units -- the reference's default of 100 kJ/mol ps^2), both
        # rotational splittings
        w = S.water(nside=6, seed=3)
        ws = dataclasses.replace(w, control=dataclasses.replace(w.control, strict_cutoff=True))
        for name, sysm, seed, nosym in (("md_nvt_water864", w, 15, False), ("md_nvt_water864_strict_nosym", ws, 16, True)):
            dyn = species_dynamics(sysm, 0.001, nosym)
            st = thermal_state(sysm, dyn, 300.0, seed)
            rec, fin, sec = md.run(sysm, dyn, st, 30, const_temp=(250.0, 1.0e4))
            save(name, sysm, dyn, st, rec, fin, sec, 300.0, seed, nvt_temp=250.0, nvt_ttmass=1.0e4)
    if only in (None, "md_npt"):
        # constant pressure: the reference's Parrinello-Rahman cell dynamics
        # (const-pressure 1 with its default strain mask 200, and 2, uniform
        # dilation, under the thermostat too); pressure 0, cell mass 1e3 in
        # program units
        w = S.water(nside=6, seed=3)
        for name, seed, mode, mask, nvt in (("md_npt_water864", 17, 1, 200, None),
                                            ("md_npt_water864_uniform_nvt", 18, 2, 0, (250.0, 1.0e4))):
            dyn = species_dynamics(w, 0.001)
            st = thermal_state(w, dyn, 300.0, seed)
            rec, fin, sec = md.run(w, dyn, st, 30, const_temp=nvt, const_pressure=(mode, 0.0, 1.0e3, mask))
            extra = dict(npt_mode=mode, npt_pressure=0.0, npt_pmass=1.0e3, npt_mask=mask)
            if nvt:
                extra.update(nvt_temp=nvt[0], nvt_ttmass=nvt[1])
            save(name, w, dyn, st, rec, fin, sec, 300.0, seed, **extra)
    if only in (None, "md_restart_water864"):
        # the reference's restart file after 10 steps (its own
        # write_restart) and its continuation read back from that file
        import tempfile
        w = S.water(nside=6, seed=3)
        dyn = species_dynamics(w, 0.001)
        st = thermal_state(w, dyn, 300.0, 14)
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "water.rst")
            rec1, fin1, sec = md.run(w, dyn, st, 10, restart_out=path)
            rec2, fin2, _ = md.run(w, dyn, st, 10, restart_in=path)
            with open(path, "rb") as f:
                rst = np.frombuffer(f.read(), np.uint8)
        save("md_restart_water864", w, dyn, st, rec2, fin2, sec, 300.0, 14, restart_file=rst, ref_rec_before=rec1,
             c_of_m_restart=fin1.c_of_m, mom_restart=fin1.mom, quat_restart=fin1.quat, amom_restart=fin1.amom)
    if only is not None:
        return
    w = S.water(nside=6, seed=3)
    save("md_water864", w, *case(w, 0.001, 300.0, 4, 30), 300.0, 4)
    ws = dataclasses.replace(w, control=dataclasses.replace(w.control, strict_cutoff=True))
    save("md_water864_strict_nosym", ws, *case(ws, 0.001, 300.0, 5, 30, nosym=True), 300.0, 5)
    wm = S.water(nside=6, seed=3, molpbc=True)
    save("md_water864_molpbc", wm, *case(wm, 0.001, 300.0, 6, 30), 300.0, 6)
    ar = S.argon_fcc()
    save("md_argon500", ar, *case(ar, 0.01, 120.0, 7, 50), 120.0, 7)
    rs = S.rock_salt(ncell=4)
    save("md_rocksalt512", rs, *case(rs, 0.002, 300.0, 8, 30), 300.0, 8)
    if "--skip-drift" in sys.argv:
        return
    w2 = S.water(nside=8, seed=11)
    for strict in (False, True):
        s = dataclasses.replace(w2, control=dataclasses.replace(w2.control, strict_cutoff=strict))
        dyn, st, rec, fin, sec = case(s, 0.001, 300.0, 12, 10000)
        save("md_drift_water2048" + ("_strict" if strict else ""), s, dyn, st, rec, fin, sec, 300.0, 12)
    dyn, st, rec, fin, sec = case(ar, 0.01, 120.0, 13, 1000)
    save("md_drift_argon500", ar, dyn, st, rec, fin, sec, 120.0, 13)


if __name__ == "__main__":
    main()
