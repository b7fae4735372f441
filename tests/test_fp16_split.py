"""Precision of the tensor-core kernel's operands: each fp32 value v is split into
fp16 hi = rn(v) and lo = rn(v - hi), and a product a.b is formed as
hi_a.hi_b + hi_a.lo_b + lo_a.hi_b (the lo.lo term dropped), accumulated in fp32.
Receive terms R satisfy |R| <= 1 and the spectra are scaled by a power of two below
2^14.  For |R| well inside fp16's normal range the split keeps about 22 bits; for
small |R| the lo part falls into fp16's subnormals, whose spacing (2^-24) bounds the
absolute error instead.  This emulates the split in numpy and bounds the error of
the 16-term dot products one mma k-step forms, relative to the sum of |terms|."""
import numpy as np


def _split(v):
    hi = v.astype(np.float16)
    lo = (v - hi.astype(np.float32)).astype(np.float16)
    return hi.astype(np.float32), lo.astype(np.float32)


def _dots(rng, r_lo_exp, n=16 * 4096):
    a = (rng.uniform(-1, 1, n) * 10 ** rng.uniform(r_lo_exp, 0, n)).astype(np.float32).reshape(-1, 16)
    b = (rng.uniform(-1, 1, n) * 10 ** rng.uniform(-3, 0, n) * 2.0 ** 14).astype(np.float32).reshape(-1, 16)
    ah, al = _split(a)
    bh, bl = _split(b)
    got = np.sum(ah.astype(np.float64) * bh + ah * bl.astype(np.float64) + al * bh.astype(np.float64), axis=1)
    want = np.sum(a.astype(np.float64) * b, axis=1)
    scale = np.sum(np.abs(a.astype(np.float64) * b), axis=1)
    return np.abs(got - want) / scale


def test_three_product_split_error():
    rng = np.random.default_rng(3)
    e = _dots(rng, -2)                      # |R| in [0.01, 1]
    assert np.median(e) < 2.0 ** -23 and np.max(e) < 2.0 ** -17
    e = _dots(rng, -4)                      # |R| down to 1e-4: subnormal lo parts
    assert np.median(e) < 2.0 ** -22 and np.max(e) < 2.0 ** -14
