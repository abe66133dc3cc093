"""Error model of the split-FP16 tensor-core products of the sweep kernels
(qmprs_gb300/csrc/sweep_group.cu: f16_split2, mma3).

The kernels split each scaled FP32 operand v s = hi + lo with hi = fp16(v s)
and lo = fp16(v s - hi) (round to nearest even, as __floats2half2_rn) and
take a product as lo_a hi_b + hi_a lo_b + hi_a hi_b, accumulated in FP32.
This numpy model of that arithmetic pins the bound the design states: at
most about 2^-21 relative per product (median about 2^-24) while lo is a
normal FP16 number (|v s| >= 2^-2), the same as the 3xTF32 scheme, and an
absolute error of half a subnormal spacing (2^-25) times |b| below that.
"""

import numpy as np


def _split_f16(v):
    hi = v.astype(np.float16)
    lo = (v - hi.astype(np.float32)).astype(np.float16)
    return hi.astype(np.float64), lo.astype(np.float64)


def _round_bits(x, bits, trunc=False):
    m, e = np.frexp(x)
    m = m * 2.0 ** bits
    return np.ldexp((np.trunc(m) if trunc else np.round(m)) / 2.0 ** bits, e)


def _split_tf32(v):
    # hi rounded to TF32's 11 significant bits; lo exact, then truncated to
    # 11 bits by the tensor core
    v = v.astype(np.float64)
    hi = _round_bits(v, 11)
    return hi, _round_bits(v - hi, 11, trunc=True)


def _product(a, b, split):
    ah, al = split(a)
    bh, bl = split(b)
    return al * bh + ah * bl + ah * bh


def _operands(seed, lo_exp, hi_exp):
    rng = np.random.default_rng(seed)
    n = 200000
    a = (2.0 ** rng.uniform(lo_exp, hi_exp, n) * rng.choice([-1, 1], n)).astype(np.float32)
    b = (2.0 ** rng.uniform(-2, 8, n) * rng.choice([-1, 1], n)).astype(np.float32)
    return a, b, a.astype(np.float64) * b.astype(np.float64)


def test_split_product_relative_error_in_normal_range():
    a, b, exact = _operands(0, -2, 15)
    rel = np.abs(_product(a, b, _split_f16) - exact) / np.abs(exact)
    assert rel.max() <= 2.0 ** -21
    assert np.median(rel) <= 2.0 ** -24


def test_split_product_absolute_error_below_normal_range():
    a, b, exact = _operands(1, -30, -2)
    err = np.abs(_product(a, b, _split_f16) - exact)
    assert np.all(err <= 2.0 ** -25 * np.abs(b) * 1.01 + 2.0 ** -21 * np.abs(exact))


def test_split_matches_three_tf32():
    """Both schemes carry 11 bits in hi and about 11 in lo: the same error
    distribution, the FP16 one at half the instructions."""
    a, b, exact = _operands(2, -2, 15)
    r16 = np.abs(_product(a, b, _split_f16) - exact) / np.abs(exact)
    r32 = np.abs(_product(a, b, _split_tf32) - exact) / np.abs(exact)
    assert abs(r16.max() / r32.max() - 1) < 0.1
    assert abs(np.median(r16) / np.median(r32) - 1) < 0.2
