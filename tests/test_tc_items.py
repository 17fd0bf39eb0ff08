"""The tensor-core work items the library builds from the k-list
(mdgpu_tc_items, host code only, no device): they cover every k-vector of
the reference's k-list exactly once, in runs of up to 64 consecutive l of
one (h, k) column, largest first, padded to a multiple of 128; the bench's
restatement (bench.tc_item_counts) counts the same items."""
import ctypes as C

import numpy as np
import pytest


def tc_items(sysm):
    from moldy_gb300 import _lib
    L = _lib.load()
    c = sysm.control
    ctl = _lib.ControlDesc(c.cutoff, c.subcell, c.alpha, c.k_cutoff, int(c.strict_cutoff), int(c.molpbc))
    h = np.ascontiguousarray(np.asarray(sysm.h, np.float64).reshape(9))
    n, nk = C.c_int(), C.c_int()
    hp = h.ctypes.data_as(C.POINTER(C.c_double))
    assert L.mdgpu_tc_items(hp, C.byref(ctl), None, None, 0, C.byref(n), C.byref(nk)) in (0, 7)
    items = np.zeros((n.value, 4), np.int32)
    k0 = np.zeros((n.value, 4), np.int32)
    st = L.mdgpu_tc_items(hp, C.byref(ctl), items.ctypes.data_as(C.c_void_p), k0.ctypes.data_as(C.c_void_p),
                          n.value, C.byref(n), C.byref(nk))
    assert st == 0
    return items, k0, nk.value


@pytest.mark.parametrize("make", ["water", "rock_salt", "ions", "quartz"])
def test_tc_items_cover_every_k_once(make):
    import os

    import bench
    from conftest import GOLDEN
    from moldy_gb300 import system
    from oracle import port
    if make == "water":
        sysm = system.water(nside=6, seed=3)
    elif make == "rock_salt":
        sysm = system.rock_salt(ncell=3)
    elif make == "ions":
        sysm = system.generic_ions(system.GENPOT, n=27, L=17.0)
    else:   # a hexagonal cell: k_x, k_y and k_z all depend on h and k
        sysm = system.load_npz(os.path.join(GOLDEN, "ex_quartz.npz"))[0]
    items, k0, nk = tc_items(sysm)
    assert nk == port.ewald(sysm).info.nkvec
    counts = items[:, 3]
    assert len(items) % 128 == 0 and counts.max() <= 64
    assert np.all(np.diff(counts) <= 0)                       # largest first
    assert list(counts) == bench.tc_item_counts(sysm)
    seen = np.zeros(nk, np.int32)
    for (h, k, l0, w), runs in zip(items, k0):
        for r in range(4):
            m = min(16, w - 16 * r)
            if m <= 0:
                assert runs[r] == -1
                continue
            seen[runs[r]:runs[r] + m] += 1
    assert np.all(seen == 1)
    # runs of one column: same (h, k), consecutive l0 64 apart
    cols = {}
    for h, k, l0, w in items[counts > 0]:
        cols.setdefault((h, k), []).append((l0, w))
    for runs in cols.values():
        runs.sort()
        for (a, wa), (b, _) in zip(runs, runs[1:]):
            assert wa == 64 and b == a + 64
