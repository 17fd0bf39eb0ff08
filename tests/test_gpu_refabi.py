"""The drop-in path: a C program that calls force_calc()/ewald() with the
reference's signatures, structs and globals (tests/ref_abi_driver.c), linked
against libmoldy_gb300.so, reproduces the reference's golden outputs and its
log lines."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from moldy_gb300.system import load_npz, write_mdsys

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver():
    from moldy_gb300 import build
    lib = build.build()
    out = os.path.join(ROOT, "moldy_gb300", "_build", "ref_abi_driver")
    subprocess.run(["gcc", "-O2", "-std=gnu99", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "ref_abi_driver.c"), "-o", out,
                    "-L", os.path.dirname(lib), "-lmoldy_gb300",
                    "-Wl,-rpath," + os.path.dirname(lib), "-rdynamic", "-lm"], check=True)
    return out


def run_driver(exe, sysm, precision, rdf=None):
    n = sysm.nsites
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.mdsys"), os.path.join(td, "out.bin")
        write_mdsys(fin, sysm)
        env = dict(os.environ, MDGPU_PRECISION=precision)
        if rdf is not None:
            env["DRIVER_RDF"] = f"{float(rdf[0])!r} {int(rdf[1])}"
        cp = subprocess.run([exe, fin, fout], capture_output=True, text=True, env=env)
        assert cp.returncode == 0, cp.stdout + cp.stderr
        d = np.fromfile(fout, dtype="<f8", count=2 * (3 * n + 10))
        if rdf is not None:
            raw = open(fout, "rb").read()
            off = 8 * (2 * (3 * n + 10) + 1)
            size = int(np.frombuffer(raw, "<i8", 1, off)[0])
            return np.frombuffer(raw, "<f4", size, off + 8).copy()
    fr = d[:3 * n].reshape(3, n)
    o = 3 * n + 10
    return (fr, d[3 * n], d[3 * n + 1:o].reshape(3, 3), d[o:o + 3 * n].reshape(3, n), d[o + 3 * n],
            d[o + 3 * n + 1:o + 3 * n + 10].reshape(3, 3), cp.stdout)


def rel(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
@pytest.mark.parametrize("name", ["ex_tip4p", "syn_water864_molpbc", "syn_rocksalt512", "syn_argon500_strict"])
def test_reference_signatures_reproduce_the_reference(driver, name, prec, tol):
    sysm, z = load_npz(os.path.join(GOLDEN, name + ".npz"))
    fr, per, sr, fe, pee, se, out = run_driver(driver, sysm, prec)
    assert rel(fr, z["force_real"]) < tol
    assert abs(per - z["pe_real"]) / abs(z["pe_real"]) < tol
    assert np.abs(sr - z["stress_real"]).max() / np.abs(z["stress_real"]).max() < tol
    if sysm.control.alpha > 1e-7:
        assert rel(fe, z["force_ewald"]) < tol
        assert abs(pee - z["pe_ewald"]) / abs(z["pe_ewald"]) < tol
        assert np.abs(se - z["stress_ewald"]).max() / np.abs(z["stress_ewald"]).max() < tol
    # the reference's log lines, in its format and order (each printed once)
    want = [str(n) for n in z["notes"] if str(n).startswith("*I*")]
    got = [l.strip() for l in out.splitlines() if l.strip().startswith("*I*")]
    assert got == want, (got, want)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["rdf_water864", "rdf_argon500"])
def test_rdf_step_fills_the_callers_histogram_like_the_reference(driver, name, prec):
    """An RDF step through the reference's force_calc signature adds into the
    caller's RDF array exactly what the reference's rdf_accum adds."""
    sysm, z = load_npz(os.path.join(GOLDEN, name + ".npz"))
    got = run_driver(driver, sysm, prec, rdf=(float(z["rdf_limit"]), int(z["rdf_nbins"])))
    assert np.array_equal(got, z["ref_rdf"]), int(np.sum(got != z["ref_rdf"]))
