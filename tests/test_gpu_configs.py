"""The measured configurations at full size, against the FP64 C restatement
of the reference (the oracle, bit-exact with the reference on every fixture):

* rock salt, 32,768 ions (16^3 fcc cells, a = 5.64 Å, Buckingham + Ewald,
  alpha 0.35, rc 10 Å, k-cutoff 1.59 Å^-1: 24,970 k-vectors): the FP32-mixed
  form within 1e-5 relative RMS force error of the FP64 oracle;
* 2048-site water (512 rigid molecules, alpha 0.3, rc 9 Å, k-cutoff for
  1e-5): both forms;
* 131,072-site water (the benchmark workload): the mixed form against the
  FP64 GPU form (the oracle takes ~3 s there; its real-space part alone is
  compared)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def oracle_forces(sysm, threads=16):
    from oracle import port
    r = port.force_calc(sysm, nthreads=threads)
    e = port.ewald(sysm, nthreads=threads)
    return r.force + e.force, r.pe, e.pe


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


def test_water_131072_mixed_against_fp64(port_built):
    from moldy_gb300 import ForceField, system
    sysm = system.water(nside=32, seed=7)
    ff = ForceField(sysm, precision="fp64")
    f64, pe64, _ = ff.forces()
    fr64, per64, _ = ff.force_calc()
    ff.set_precision("mixed")
    f32, pe32, _ = ff.forces()
    ff.close()
    assert rel_rms(f32, f64) < 1e-5, rel_rms(f32, f64)
    assert abs(pe32.sum() - pe64.sum()) < 1e-5 * abs(pe64.sum())
    from oracle import port
    r = port.force_calc(sysm, nthreads=16)
    assert rel_rms(fr64, r.force) < 1e-12
    assert abs(per64 - r.pe) < 1e-12 * abs(r.pe)
