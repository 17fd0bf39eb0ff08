"""GPU radial-distribution histogram (mdgpu_rdf_counts) against the
reference's own float histogram from one RDF step of force_calc (fixtures
made by tests/golden/make_rdf_golden.py): integer pair counts per bin,
turned into the reference's float accumulation, bit for bit."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["rdf_water864", "rdf_water864_strict", "rdf_water864_molpbc", "rdf_argon500", "rdf_rocksalt512"]


def float_accumulate(counts, invrho):
    """rdf_accum's per-pair update bin = (float)((double)bin + 1/density),
    repeated count times from zero (src/rdf.c:103-104)."""
    out = np.zeros(counts.shape, np.float32)
    flat, c = out.reshape(-1), counts.reshape(-1)
    for i in np.nonzero(c)[0]:
        v = np.float32(0.0)
        for _ in range(int(c[i])):
            v = np.float32(float(v) + invrho)
        flat[i] = v
    return out


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_rdf_matches_reference_bit_for_bit(name, prec):
    from moldy_gb300 import ForceField, system
    sysm, z = system.load_npz(os.path.join(GOLDEN, name + ".npz"))
    limit, nbins = float(z["rdf_limit"]), int(z["rdf_nbins"])
    ff = ForceField(sysm, precision=prec)   # the histogram is FP64 in both forms
    cnt = ff.rdf_counts(limit, nbins)
    ff.close()
    M = sysm.max_id
    assert np.array_equal(cnt, np.transpose(cnt, (1, 0, 2)))
    assert np.all(cnt[0] == 0) and np.all(cnt[:, 0] == 0)
    invrho = 1.0 / (sysm.nsites / float(np.linalg.det(sysm.h)))
    rows = [cnt[a, b] for a in range(1, M) for b in range(a, M)]   # init_rdf's layout
    got = float_accumulate(np.concatenate(rows), invrho)
    ref = z["ref_rdf"]
    assert got.shape == ref.shape
    assert np.array_equal(got, ref), int(np.sum(got != ref))
