"""The oracle pinned against the reference: the C restatement
(oracle/port/moldy_port.c) must reproduce the golden fixtures the reference
itself produced (tests/golden/make_golden.py), and the reference's own example
runs must reproduce the constants its shipped 1996 outputs log."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from moldy_gb300 import pairset
from moldy_gb300.system import CONV_E, load_npz


def rel_rms(a, b):
    den = float((b ** 2).sum())
    return float(np.sqrt(((a - b) ** 2).sum() / den)) if den > 0 else float(np.abs(a - b).max())


@pytest.mark.parametrize("name", golden_files())
def test_port_matches_reference_fixture(name, port_built):
    port = port_built
    sysm, z = load_npz(os.path.join(GOLDEN, name + ".npz"))
    r = port.force_calc(sysm, want_pairs=True)
    # real space: the port evaluates the same expressions in the same order
    assert rel_rms(r.force, z["force_real"]) < 1e-13
    assert abs(r.pe - float(z["pe_real"])) <= 1e-13 * abs(float(z["pe_real"]))
    assert np.abs(r.stress - z["stress_real"]).max() <= 1e-13 * np.abs(z["stress_real"]).max()
    keys = pairset.keys_from_triplets(r.pairs)
    cnt, dig = pairset.digest(keys)
    assert cnt == int(z["npairs"])
    assert dig == int(z["pair_digest"][0])
    if "pair_keys" in z:
        assert np.array_equal(keys, z["pair_keys"])
    assert r.info.n_nabors * 2 == int(z["log_nabor_cells"])
    assert r.info.nx * r.info.ny * r.info.nz == int(z["log_ncells"])
    assert f"{r.info.eintra * CONV_E:g}" == f"{float(z['log_eintra_kjmol']):g}"
    if sysm.control.alpha > 1e-7:
        e = port.ewald(sysm)
        assert rel_rms(e.force, z["force_ewald"]) < 1e-13
        assert abs(e.pe - float(z["pe_ewald"])) <= 1e-13 * abs(float(z["pe_ewald"]))
        assert e.info.nkvec == int(z["log_nkvec"])
        assert f"{e.info.self_energy * CONV_E:f}" == f"{float(z['log_self_energy_kjmol']):f}"


def test_port_threads_agree(port_built):
    port = port_built
    sysm, z = load_npz(os.path.join(GOLDEN, "syn_water2048.npz"))
    a = port.force_calc(sysm, nthreads=1)
    b = port.force_calc(sysm, nthreads=3)
    assert rel_rms(b.force, a.force) < 1e-14
    assert abs(b.pe - a.pe) < 1e-12 * abs(a.pe)
    c = port.ewald(sysm, nthreads=1)
    d = port.ewald(sysm, nthreads=3)
    assert rel_rms(d.force, c.force) < 1e-14


# Constants the reference logs in its shipped example outputs
# (src/examples/<name>-example.out, lines cited), reproduced today by the
# reference's own start-up on the same control files (ex_* fixtures).
SHIPPED = {
    "ex_water": (125, 82, 794.119798, 447),      # water-example.out:61-64
    "ex_tips2": (125, 94, 968.356089, 570),      # tips2-example.out:65-68
    "ex_tip4p": (512, 204, 1722.888659, 1102),   # tip4p-example.out:65-68
    "ex_mgclh2o": (3375, 486, 11332.778403, 1484),  # mgclh2o-example.out:79-82
    "ex_argon": (729, 912, None, None),          # argon-example.out:59-60
}


@pytest.mark.parametrize("name", sorted(SHIPPED))
def test_port_reproduces_shipped_example_constants(name, port_built):
    port = port_built
    sysm, _ = load_npz(os.path.join(GOLDEN, name + ".npz"))
    ncells, nab, self_e, nk = SHIPPED[name]
    r = port.force_calc(sysm)
    assert r.info.nx * r.info.ny * r.info.nz == ncells
    assert 2 * r.info.n_nabors == nab
    if self_e is not None:
        e = port.ewald(sysm)
        assert f"{e.info.self_energy * CONV_E:f}" == f"{self_e:f}"
        assert e.info.nkvec == nk


def test_port_rejects_what_the_reference_rejects(port_built):
    port = port_built
    sysm, _ = load_npz(os.path.join(GOLDEN, "syn_water864_strict.npz"))
    bad = sysm.with_sites(sysm.site * 3.0)        # co-ordinates outside the cell
    with pytest.raises(RuntimeError, match="out of range"):
        port.force_calc(bad)
    import dataclasses
    big = dataclasses.replace(sysm, control=dataclasses.replace(sysm.control, cutoff=40.0))
    with pytest.raises(RuntimeError, match="CUTOFF"):
        port.force_calc(big)
