"""Dump records converted on the GPU during dynamics (mdgpu_md_run_dump)
against the records the reference's own dump() wrote from the same start
(tests/golden/dump_*.npz), and the files the library's writer makes from
them against the reference's files."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["dump_water864", "dump_argon500", "dump_rocksalt512", "dump_waterwall"]


def _setup(name, prec):
    from moldy_gb300 import ForceField, system
    from moldy_gb300.dynamics import Dynamics, MDState, MolecularDynamics
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    files = {k[5:]: z[k].tobytes() for k in z.files if k.startswith("file:")}
    sysm, m = system.load_npz(os.path.join(GOLDEN, str(z["md_fixture"]) + ".npz"))
    dyn = Dynamics(m["md_mass"], m["md_inertia"].reshape(-1, 3), m["md_rdof"], float(m["md_step"]),
                   bool(m["md_nosym"]))
    st0 = MDState(m["c_of_m0"], m["mom0"], m["quat0"], m["amom0"])
    ff = ForceField(sysm, precision=prec)
    return z, files, sysm, dyn, st0, ff, MolecularDynamics(ff, dyn, st0)


def _ref_records(files, tmp_path):
    from moldy_gb300.dumpfile import read_dump
    recs = []
    for fn in sorted(files):
        p = tmp_path / ("ref_" + fn)
        p.write_bytes(files[fn])
        recs.append(read_dump(str(p)).records)
    return np.concatenate(recs)


# per part: tolerance relative to the part's largest magnitude
TOL = {"fp64": dict(default=2e-6), "mixed": dict(default=2e-6, force=1e-4, torque=1e-4, stress=1e-4, pe=1e-5)}


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", CASES)
def test_records_match_reference(name, prec, tmp_path):
    from moldy_gb300.dumpfile import split_record
    z, files, sysm, dyn, st0, ff, md = _setup(name, prec)
    level, interval, steps = int(z["level"]), int(z["interval"]), int(z["steps"])
    e, rec = md.run_dump(steps, interval, level)
    ff.close()
    ref = _ref_records(files, tmp_path)
    assert rec.shape == ref.shape
    tol = TOL[prec]
    for r, (a, b) in enumerate(zip(rec, ref)):
        pa, pb = split_record(a, level, sysm.nmols, md.nq), split_record(b, level, sysm.nmols, md.nq)
        for key in pb:
            scale = float(np.max(np.abs(pb[key]))) if pb[key].size else 0.0
            t = tol.get(key, tol["default"])
            err = float(np.max(np.abs(pa[key] - pb[key]))) if pb[key].size else 0.0
            assert err <= t * scale + 1e-30, (r, key, err, scale)


def test_dumping_leaves_the_trajectory_unchanged():
    """A run with records (level 8 steps run outside the captured graph)
    gives bit-identical energies and state to a plain run."""
    z, files, sysm, dyn, st0, ff, md = _setup("dump_water864", "mixed")
    e1, _ = md.run_dump(20, 3, 11)
    s1 = md.state()
    ff.close()
    from moldy_gb300 import ForceField
    from moldy_gb300.dynamics import MolecularDynamics
    ff2 = ForceField(sysm, precision="mixed")
    md2 = MolecularDynamics(ff2, dyn, st0)
    e2 = md2.run(20)
    s2 = md2.state()
    ff2.close()
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_array_equal(s1.c_of_m, s2.c_of_m)
    np.testing.assert_array_equal(s1.amom, s2.amom)


def test_files_from_gpu_records(tmp_path):
    """GPU records through the writer: the header and system description
    bytes equal the reference's (outside the uninitialised and clock
    fields), the records agree as above."""
    from moldy_gb300.dumpfile import DumpWriter, read_dump, species_info
    z, files, sysm, dyn, st0, ff, md = _setup("dump_water864", "fp64")
    level, interval, steps, nd = int(z["level"]), int(z["interval"]), int(z["steps"]), int(z["ndumps"])
    _, rec = md.run_dump(steps, interval, level)
    ff.close()
    sp = species_info(sysm, dyn, names=["spec0"])
    out = tmp_path / "gpu"
    out.mkdir()
    with DumpWriter(str(out / "run%02d.dmp"), sp, level, interval, nd, dyn.step, sysm.nmols, md.nq,
                    istep=1, title=str(z["title"])) as w:
        for r in rec:
            w.append(r)
    for fn in sorted(files):
        a, b = files[fn], (out / fn).read_bytes()
        assert len(a) == len(b)
        hdr = 208 + 16 + 68
        A, B = np.frombuffer(a[:hdr], np.uint8), np.frombuffer(b[:hdr], np.uint8)
        keep = np.ones(hdr, bool)
        keep[a.index(b"\0"):128] = False
        keep[176:192] = False
        n = a.index(b"\0", 208 + 16 + 36)
        keep[n:208 + 16 + 68] = False
        assert not np.any((A != B) & keep)
        p = tmp_path / ("ref_" + fn)
        p.write_bytes(a)
        ours, theirs = read_dump(str(out / fn)), read_dump(str(p))
        assert ours.ndumps == theirs.ndumps and ours.istep == theirs.istep
        scale = np.max(np.abs(theirs.records), axis=0) + 1e-30
        assert np.max(np.abs(ours.records - theirs.records) / scale) < 1e-4
