"""The two-stream force evaluation (pair kernel beside the high-priority
k-space passes) against the one-stream order phase timing uses, and
single-step dynamics calls (captured-step replay) against one long call:
the same kernels in the same per-buffer order, so the results are
bit-identical."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("make", ["water", "rock_salt"])
def test_two_streams_match_one_stream(make, prec):
    from moldy_gb300 import ForceField, system
    sysm = system.water(nside=8, seed=5) if make == "water" else system.rock_salt(ncell=4)
    ff = ForceField(sysm, precision=prec)
    f1, pe1, st1 = ff.forces()           # two streams
    ff.set_phase_timing(True)
    f2, pe2, st2 = ff.forces()           # one stream, in order
    ff.set_phase_timing(False)
    f3, pe3, st3 = ff.forces()
    ff.close()
    np.testing.assert_array_equal(f1, f2)
    np.testing.assert_array_equal(pe1, pe2)
    np.testing.assert_array_equal(st1, st2)
    np.testing.assert_array_equal(f1, f3)


def test_single_step_calls_match_one_run():
    from moldy_gb300 import ForceField, system
    from moldy_gb300.dynamics import MolecularDynamics, species_dynamics, thermal_state
    sysm = system.water(nside=6, seed=3)
    dyn = species_dynamics(sysm, 0.001)
    st0 = thermal_state(sysm, dyn, 300.0, seed=4)
    runs = []
    for single in (False, True):
        ff = ForceField(sysm, precision="mixed")
        md = MolecularDynamics(ff, dyn, st0)
        if single:
            e = np.concatenate([md.run(1) for _ in range(12)])
        else:
            e = md.run(12)
        runs.append((e, md.state()))
        ff.close()
    (e1, s1), (e2, s2) = runs
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_array_equal(s1.c_of_m, s2.c_of_m)
    np.testing.assert_array_equal(s1.mom, s2.mom)
    np.testing.assert_array_equal(s1.quat, s2.quat)
    np.testing.assert_array_equal(s1.amom, s2.amom)


def test_set_state_replays_the_same_trajectory():
    """mdgpu_md_set_state puts a saved state back into the buffers the
    captured step reads: the run from it repeats bit for bit."""
    from moldy_gb300 import ForceField, system
    from moldy_gb300.dynamics import MolecularDynamics, species_dynamics, thermal_state
    sysm = system.water(nside=6, seed=3)
    dyn = species_dynamics(sysm, 0.001)
    ff = ForceField(sysm, precision="mixed")
    md = MolecularDynamics(ff, dyn, thermal_state(sysm, dyn, 300.0, seed=4))
    md.run(5)
    s5 = md.state()
    e1 = md.run(6)
    s11 = md.state()
    md.set_state(s5)
    e2 = md.run(6)
    s11b = md.state()
    ff.close()
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_array_equal(s11.c_of_m, s11b.c_of_m)
    np.testing.assert_array_equal(s11.amom, s11b.amom)
