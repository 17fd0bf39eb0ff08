"""Tensor-core (tcgen05) path of the mixed form's reciprocal space.

The operand probe runs one 128 x n x 16 MMA pair (bf16, the structure
factor's operands, and fp16, the force pass's) in the operand layout the
kernels use and compares it with the product computed on the host (small
integers times powers of two: every sum is exact in FP32), with and without
the A-negation flag.  The tensor-core passes (structure factor and forces)
are compared with the CUDA-core passes on the same configurations."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)


def bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


def probe(a0, b0, a1, b1, flags):
    from moldy_gb300 import _lib
    lib = _lib.load()
    n = b0.shape[0]
    d = np.zeros((128, n), np.float32)
    args = [np.ascontiguousarray(v) for v in (a0, b0, a1, b1)]
    st = lib.mdgpu_tc_probe(0, *[v.ctypes.data_as(C.c_void_p) for v in args], n, flags,
                            d.ctypes.data_as(C.c_void_p))
    assert st == 0, st
    return d


@pytest.mark.parametrize("n", [16, 48, 64, 128])
@pytest.mark.parametrize("neg", [False, True])
def test_probe_layout_and_negation(n, neg):
    rng = np.random.default_rng(n)
    mk = lambda r: bf16_bits(rng.integers(-8, 9, size=(r, 16)).astype(np.float32) * 0.125)
    a0, a1, b0, b1 = mk(128), mk(128), mk(n), mk(n)
    d = probe(a0, b0, a1, b1, 2 if neg else 0)
    A0, A1, B0, B1 = (bf16_value(v).astype(np.float64) for v in (a0, a1, b0, b1))
    ref = A0 @ B0.T + (-1.0 if neg else 1.0) * (A1 @ B1.T)
    np.testing.assert_array_equal(d, ref.astype(np.float32))


@pytest.mark.parametrize("n", [64, 128])
def test_probe_fp16_operands(n):
    """The force pass's operand type: fp16 bit patterns, flags & 8."""
    rng = np.random.default_rng(7 + n)
    mk = lambda r: (rng.integers(-64, 65, size=(r, 16)).astype(np.float16) * np.float16(0.0625))
    a0, a1, b0, b1 = mk(128), mk(128), mk(n), mk(n)
    d = probe(*(v.view(np.uint16) for v in (a0, b0, a1, b1)), 8)
    ref = a0.astype(np.float64) @ b0.astype(np.float64).T + a1.astype(np.float64) @ b1.astype(np.float64).T
    np.testing.assert_array_equal(d, ref.astype(np.float32))


@pytest.mark.parametrize("make", ["water", "rock_salt", "ex_quartz", "ex_mgclh2o", "syn_water2048",
                                  "ions27", "ions125"])
def test_tensor_core_structure_factor_matches_cuda_core_pass(make, monkeypatch):
    """ions27 / ions125: charged-site counts that are not a multiple of the
    32-site stage (padding sites with zero charge), one item tile and a
    net charge."""
    from conftest import GOLDEN
    from moldy_gb300 import ForceField, system
    if make == "water":
        sysm = system.water(nside=8, seed=5)
    elif make == "rock_salt":
        sysm = system.rock_salt(ncell=4)
    elif make.startswith("ions"):
        sysm = system.generic_ions(system.GENPOT, n=int(make[4:]), L=17.0)
    else:
        sysm = system.load_npz(os.path.join(GOLDEN, make + ".npz"))[0]
    res = {}
    for tc in ("1", "0"):
        monkeypatch.setenv("MDGPU_KSPACE_TC", tc)
        ff = ForceField(sysm, precision="mixed")
        res[tc] = ff.ewald()
        self_e = abs(ff.info()["self_energy"])
        ff.close()
    # the Ewald total is the difference of the k-space sum and the self
    # energy: FP32 errors scale with the parts (a small net-charged system
    # cancels them to 0.4 % of the self energy)
    e_scale = lambda e: abs(e) + self_e
    (f1, e1, s1), (f0, e0, s0) = res["1"], res["0"]
    if make.startswith("ions"):
        # no golden fixture: both paths against the oracle's ewald()
        from oracle import port
        ref = port.ewald(sysm)
        for name, (f, e) in (("tensor-core", (f1, e1)), ("CUDA-core", (f0, e0))):
            ef = np.sqrt(((f - ref.force) ** 2).mean()) / np.sqrt((ref.force ** 2).mean())
            ee = abs(e - ref.pe) / e_scale(ref.pe)
            print(f"{make} {name} vs oracle: force {ef:.2e}, energy {ee:.2e} of the parts")
            assert ef < 1e-5 and ee < 1e-5
    # both are FP32-level sums of the same terms; each is held to 1e-5 of
    # the reference by the parity tests
    df = np.sqrt(((f1 - f0) ** 2).mean()) / np.sqrt((f0 ** 2).mean())
    print(f"{make}: force rel RMS difference {df:.2e}, energy {abs(e1 - e0) / abs(e0):.2e}")
    assert df < 1e-5
    assert abs(e1 - e0) <= 1e-5 * e_scale(e0)
    np.testing.assert_allclose(s1, s0, rtol=1e-5, atol=1e-5 * np.abs(s0).max())
