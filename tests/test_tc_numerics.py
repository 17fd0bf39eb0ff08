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
