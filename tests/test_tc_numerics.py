"""The operand splitting of the tensor-core reciprocal-space kernels
(moldy_gb300/csrc/tc.cuh), restated in numpy FP32 arithmetic: three bf16
terms on fixed grids (hi on multiples of 2^-7, mid of 2^-15, lo of 2^-23,
each grid reached by (v + C) - C with C = 1.5 2^(23 - bits)), so that

* every term is exactly representable in bf16,
* |v - hi - mid - lo| <= 2^-24 for |v| <= 1,
* sums of hi*hi products of a 1024-site chunk are exact in FP32 in any
  order (the property that makes the tensor cores' truncating FP32
  accumulation harmless for the large accumulator).
"""
import numpy as np


def round_grid(v, c):
    c = np.float32(c)
    return ((v + c).astype(np.float32) - c).astype(np.float32)


def split3(v):
    v = np.asarray(v, np.float32)
    hi = round_grid(v, 98304.0)
    r = (v - hi).astype(np.float32)
    mid = round_grid(r, 384.0)
    r2 = (r - mid).astype(np.float32)
    lo = round_grid(r2, 1.5)
    return hi, mid, lo


def bf16_exact(x):
    return np.all((np.asarray(x, np.float32).view(np.uint32) & 0xFFFF) == 0)


def test_terms_are_bf16_and_reconstruct_to_2e_minus_24():
    rng = np.random.default_rng(11)
    v = np.concatenate([rng.uniform(-1, 1, 200000), rng.uniform(-1e-4, 1e-4, 20000),
                        np.array([1.0, -1.0, 0.5, 1 - 2 ** -24, 2 ** -30, 0.0])]).astype(np.float32)
    hi, mid, lo = split3(v)
    assert bf16_exact(hi) and bf16_exact(mid) and bf16_exact(lo)
    assert np.all(np.mod(hi.astype(np.float64) * 2 ** 7, 1) == 0)
    assert np.all(np.mod(mid.astype(np.float64) * 2 ** 15, 1) == 0)
    assert np.all(np.mod(lo.astype(np.float64) * 2 ** 23, 1) == 0)
    res = v.astype(np.float64) - (hi.astype(np.float64) + mid + lo)
    assert np.abs(res).max() <= 2.0 ** -24


def test_hh_chunk_sums_are_exact_in_fp32():
    rng = np.random.default_rng(12)
    for trial in range(20):
        # a 1024-site chunk of charge-scaled seeds (|A| < 1) times z values (|Z| <= 1)
        a = rng.uniform(-0.999, 0.999, 1024).astype(np.float32)
        z = np.cos(rng.uniform(0, 2 * np.pi, 1024)).astype(np.float32)
        if trial == 0:   # all in phase: the largest partial sums
            a, z = np.full(1024, 0.99, np.float32), np.ones(1024, np.float32)
        ah, zh = split3(a)[0], split3(z)[0]
        prod = (ah * zh).astype(np.float32)          # exact: 16-bit integers times 2^-14
        exact = prod.astype(np.float64).sum()
        for order in (np.arange(1024), rng.permutation(1024)):
            acc = np.float32(0.0)
            for p in prod[order]:
                acc = np.float32(acc + p)
            assert float(acc) == exact


def _rz_add(acc, x):
    """acc + x rounded toward zero to FP32 (the tensor cores' accumulation,
    measured by mdgpu_tc_probe: 1 + 1.5 ulp -> 1, 1 - 3.5 ulp -> 1 - 4 ulp)."""
    v = float(acc) + float(x)
    f = np.float32(v)
    if abs(float(f)) > abs(v):
        f = np.nextafter(f, np.float32(0.0))
    return f


def _bf16_float_split3(v):
    """Three bf16 terms relative to each value's own exponent (round to nearest)."""
    def rn16(x):
        b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
        return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16).astype(np.uint32).view(np.float32)
    v = np.asarray(v, np.float32)
    h = rn16(v)
    r = (v - h).astype(np.float32)
    m = rn16(r)
    lo = rn16((r - m).astype(np.float32))
    return h, m, lo


def _chunk_sum(a, z, split, separate):
    """sum_j a_j z_j as the structure-factor kernel forms it: 16-site K-steps,
    six term products, each K-step's products summed exactly and added to the
    accumulator with round-toward-zero; hh into its own accumulator when
    separate, everything into one otherwise."""
    ta, tz = split(a), split(z)
    pairs = [(0, 0), (0, 1), (1, 0), (0, 2), (2, 0), (1, 1)]
    main = np.float32(0.0)
    rest = np.float32(0.0)
    for s in range(0, len(a), 16):
        for p, (i, j) in enumerate(pairs):
            step = float(np.sum(ta[i][s:s + 16].astype(np.float64) * tz[j][s:s + 16]))
            if separate and p > 0:
                rest = _rz_add(rest, step)
            else:
                main = _rz_add(main, step)
    return float(main) + float(rest)


def test_chunk_sums_with_truncating_accumulation():
    """A near-neutral 1024-site chunk (the near-cancelling sums of a crystal's
    structure factor): with fixed-grid terms and the hh accumulator apart the
    truncating accumulation stays at the FP32 level of the FP64 sum (4-8e-9 of
    the sum of |terms| here); floating bf16 terms in one accumulator drift
    toward zero (up to 7e-7 of it, 1e-5 of the chunk's near-cancelled sum --
    the energy error the first tensor-core structure factor showed)."""
    rng = np.random.default_rng(13)
    err_fixed, err_float = [], []
    for trial in range(6):
        q = np.where(rng.random(1024) < 0.5, 0.9, -0.9)
        phase = rng.uniform(0, 2 * np.pi, 1024)
        a = (q * np.cos(phase) * 0.5).astype(np.float32)   # charge-scaled seeds, |a| < 1
        z = (np.cos(rng.uniform(0, 2 * np.pi) * np.arange(1024) / 1024 + 0.3)).astype(np.float32)
        exact = float(np.sum(a.astype(np.float64) * z))
        scale = float(np.sum(np.abs(a.astype(np.float64) * z)))
        err_fixed.append(abs(_chunk_sum(a, z, split3, True) - exact) / scale)
        err_float.append(abs(_chunk_sum(a, z, _bf16_float_split3, False) - exact) / scale)
    assert max(err_fixed) < 1e-7
    assert max(err_float) > 3 * max(err_fixed)
