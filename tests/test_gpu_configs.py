"""The measured configurations at full size, against the FP64 C restatement
of the reference (the oracle, bit-exact with the reference on every fixture):

* rock salt, 32,768 ions (16^3 fcc cells, a = 5.64 Å, Buckingham + Ewald,
  alpha 0.35, rc 10 Å, k-cutoff 1.59 Å^-1: 24,970 k-vectors): the FP32-mixed
  form within 1e-5 relative RMS force error of the FP64 oracle;
* 2048-site water (512 rigid molecules, alpha 0.3, rc 9 Å, k-cutoff for
  1e-5): both forms;
* 131,072-site water (the benchmark workload, 69,876 k-vectors): both
  forms' total forces (real space + reciprocal space), energies and stress
  against the oracle run on every host core, and the mixed form against the
  FP64 GPU form."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def oracle_forces(sysm, threads=None):
    from oracle import port
    threads = threads or os.cpu_count() or 1
    r = port.force_calc(sysm, nthreads=threads)
    e = port.ewald(sysm, nthreads=threads)
    return r.force + e.force, r.pe, e.pe


@pytest.fixture(scope="module")
def water131k(port_built):
    """The benchmark configuration and the oracle's real-space and
    reciprocal-space results for it (about 3 s on 16 host threads)."""
    from moldy_gb300 import system
    from oracle import port
    sysm = system.water(nside=32, seed=7)
    threads = os.cpu_count() or 1
    return sysm, port.force_calc(sysm, nthreads=threads), port.ewald(sysm, nthreads=threads)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_rock_salt_32768(port_built, prec, tol):
    from moldy_gb300 import ForceField, system
    sysm = system.rock_salt(ncell=16, k_cutoff=1.59)
    f0, pr, pk = oracle_forces(sysm)
    ff = ForceField(sysm, precision=prec)
    f, pe, _ = ff.forces()
    assert ff.info()["nkvec"] == 24970
    ff.close()
    assert rel_rms(f, f0) < tol, rel_rms(f, f0)
    assert abs(pe[0] - pr) < tol * abs(pr)
    assert abs(pe[1] - pk) < tol * abs(pk)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_water_2048(port_built, prec, tol):
    from moldy_gb300 import ForceField, system
    sysm = system.water(nside=8)
    f0, pr, pk = oracle_forces(sysm)
    ff = ForceField(sysm, precision=prec)
    f, pe, _ = ff.forces()
    ff.close()
    assert rel_rms(f, f0) < tol, rel_rms(f, f0)
    assert abs((pe[0] + pe[1]) - (pr + pk)) < tol * (abs(pr) + abs(pk))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_water_131072_total_forces_against_the_oracle(water131k, prec, tol):
    """The headline workload: both parts and their sum against the oracle
    (src/force.c:1108-1320 and src/ewald.c:280-589 restated)."""
    from moldy_gb300 import ForceField
    sysm, r, e = water131k
    ff = ForceField(sysm, precision=prec)
    fr, per, str_ = ff.force_calc()
    fk, pek, stk = ff.ewald()
    f, pe, st = ff.forces()
    nk = ff.info()["nkvec"]
    ff.close()
    assert nk == 69876 == e.info.nkvec
    ftot = r.force + e.force
    assert rel_rms(f, ftot) < tol, rel_rms(f, ftot)
    assert rel_rms(fr, r.force) < tol, rel_rms(fr, r.force)
    assert rel_rms(fk, e.force) < tol, rel_rms(fk, e.force)
    assert abs(pe[0] - r.pe) < tol * abs(r.pe)
    assert abs(pe[1] - e.pe) < tol * abs(e.pe)
    assert abs(per - r.pe) < tol * abs(r.pe) and abs(pek - e.pe) < tol * abs(e.pe)
    s_ref = r.stress + e.stress
    s_gpu = np.triu(np.asarray(st).reshape(3, 3))
    assert np.abs(s_gpu - np.triu(s_ref)).max() < tol * np.abs(s_ref).max()
    for got, want in ((str_, r.stress), (stk, e.stress)):
        assert np.abs(np.triu(got) - np.triu(want)).max() < tol * np.abs(want).max()


def test_water_131072_mixed_against_fp64():
    from moldy_gb300 import ForceField, system
    sysm = system.water(nside=32, seed=7)
    ff = ForceField(sysm, precision="fp64")
    f64, pe64, _ = ff.forces()
    ff.set_precision("mixed")
    f32, pe32, _ = ff.forces()
    ff.close()
    assert rel_rms(f32, f64) < 1e-5, rel_rms(f32, f64)
    assert abs(pe32.sum() - pe64.sum()) < 1e-5 * abs(pe64.sum())
