"""The link-cell stencil and its regrouping into columns (mdgpu_stencil_columns,
host code only, no device): the grid and the half-space neighbour count are
the reference's (the C restatement's NABORS count on the same system); the
columns the mixed form's pair kernel walks cover the full stencil -- the
half-space offsets, their mirrors and the zero offset -- exactly once, as
maximal runs of consecutive dz sorted by (dx, dy, dz0); and each cell offset
is h (dx/nx, dy/ny, dz/nz) split into an FP32 hi part and the FP32 rest."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN


def stencil(sysm):
    from moldy_gb300 import _lib
    L = _lib.load()
    c = sysm.control
    ctl = _lib.ControlDesc(c.cutoff, c.subcell, c.alpha, c.k_cutoff, int(c.strict_cutoff), int(c.molpbc))
    h = np.ascontiguousarray(np.asarray(sysm.h, np.float64).reshape(9))
    hp = h.ctypes.data_as(C.POINTER(C.c_double))
    grid = np.zeros(3, np.int32)
    nhalf, ncols = C.c_int(), C.c_int()
    st = L.mdgpu_stencil_columns(hp, C.byref(ctl), grid.ctypes.data_as(C.c_void_p), None, C.byref(nhalf), None,
                                 None, C.byref(ncols), 0)
    assert st in (0, 7)
    cap = max(2 * nhalf.value + 1, 1)
    half = np.zeros((cap, 3), np.int32)
    cols = np.zeros((cap, 5), np.int32)
    coff = np.zeros((cap, 6), np.float32)
    st = L.mdgpu_stencil_columns(hp, C.byref(ctl), grid.ctypes.data_as(C.c_void_p), half.ctypes.data_as(C.c_void_p),
                                 C.byref(nhalf), cols.ctypes.data_as(C.c_void_p), coff.ctypes.data_as(C.c_void_p),
                                 C.byref(ncols), cap)
    assert st == 0
    return grid, half[:nhalf.value], cols[:ncols.value], coff


CASES = ["syn_water864_strict", "syn_water864_molpbc", "ex_quartz", "ex_mgclh2o", "syn_argon500_strict",
         "syn_rocksalt512", "ex_clay"]


@pytest.mark.parametrize("name", CASES)
def test_columns_cover_the_reference_stencil_once(name, port_built):
    from moldy_gb300 import system
    from oracle import port
    sysm = system.load_npz(os.path.join(GOLDEN, name + ".npz"))[0]
    grid, half, cols, coff = stencil(sysm)
    info = port.force_calc(sysm).info
    assert (int(grid[0]), int(grid[1]), int(grid[2])) == (info.nx, info.ny, info.nz)
    assert len(half) == info.n_nabors
    # the full stencil: zero once, every other half-space offset and its mirror
    full = {tuple(d) for d in half}
    assert (0, 0, 0) in full
    full |= {tuple(-d) for d in half}
    assert len(full) == 2 * len(half) - 1
    # the columns: sorted, maximal runs of consecutive dz, covering it once
    keys = [tuple(c[:3]) for c in cols]
    assert keys == sorted(keys)
    seen = []
    for i, (dx, dy, dz0, n, base) in enumerate(cols):
        assert n >= 1
        seen += [(dx, dy, dz0 + t) for t in range(n)]
        if i > 0:
            px, py, pz, pn, pb = cols[i - 1]
            assert base == pb + pn
            assert not (px == dx and py == dy and pz + pn == dz0), "a column split in two"
    assert len(seen) == len(set(seen)) == len(full)
    assert set(seen) == full
    # the offsets: h (d / n) as FP32 hi plus the FP32 rest
    h = np.asarray(sysm.h, np.float64)
    for dx, dy, dz0, n, base in cols:
        for t in range(n):
            v = h @ (np.array([dx, dy, dz0 + t], np.float64) / grid)
            hi, lo = coff[base + t, :3].astype(np.float64), coff[base + t, 3:].astype(np.float64)
            assert np.all(hi == v.astype(np.float32))
            assert np.all(np.abs(hi + lo - v) <= 1e-12 * max(1.0, np.abs(v).max()))
