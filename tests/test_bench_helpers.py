"""Host-side accounting of bench.py: the tensor-core items it counts for the
MMA work cover the reference's k-vector set exactly (the oracle's ewald()
k-vector count), each item at most 64 k-vectors."""
import numpy as np
import pytest


@pytest.mark.parametrize("make", ["water", "rock_salt", "ions"])
def test_tc_items_cover_the_k_list(make):
    import bench
    from moldy_gb300 import system
    from oracle import port
    if make == "water":
        sysm = system.water(nside=6, seed=3)
    elif make == "rock_salt":
        sysm = system.rock_salt(ncell=3)
    else:
        sysm = system.generic_ions(system.GENPOT, n=27, L=17.0)
    counts = bench.tc_item_counts(sysm)
    ref = port.ewald(sysm)
    assert sum(counts) == ref.info.nkvec
    assert max(counts) <= 64 and len(counts) % 128 == 0
    assert counts == sorted(counts, reverse=True)
    assert bench.tc_mma_flops(sysm, int(np.count_nonzero(sysm.chg())))["kforce"] > 0
