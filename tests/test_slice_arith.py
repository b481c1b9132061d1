"""The arithmetic of the mixed-precision tensor-core contractions, restated with Python
integers (the device code is ttn_expm.cu: slice6, the level accumulation of
tc_issue_chunk and the combination of tc_drain_to_stage).

Every FP64 operand row is scaled by 2^E (E the smallest exponent with all |x| < 2^E) and
cut into six 7-bit slices; the products of slices t, u (levels t + u = 2..8) are summed
over K = 128 per level, which must stay below 2^24 so that FP32 accumulation is exact; the
levels are combined as (hi << 34) + (lo >> 1) times 2^(E_a + E_b - 55).  Checked: the
slices reconstruct each operand to 2^-42 of its row scale, every level sum fits in FP32
exactly, and dot products agree with exact rational arithmetic to the documented bound.
"""
import struct
from fractions import Fraction

import numpy as np

K, SLICES, LEVELS = 128, 6, 7


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def exp_bound(vals):
    mx = max(bits(abs(v)) for v in vals)
    if mx == 0:
        return 0
    e = mx >> 52
    return e - 1022 if e else -1074 + mx.bit_length()


def slice6(x, er):
    b = bits(x)
    e, frac = (b >> 52) & 0x7FF, b & ((1 << 52) - 1)
    q = 0
    if e or frac:
        m = (frac | (1 << 52)) if e else frac
        p = (e - 1075) if e else -1074
        sh = er - 42 - p
        q = 0 if sh >= 64 else (m >> sh if sh >= 0 else m << (-sh))
    sign = -1 if b >> 63 else 1
    return [sign * ((q >> (35 - 7 * t)) & 127) for t in range(SLICES)]


def contract(a, b):
    ea, eb = exp_bound(a), exp_bound(b)
    sa = [slice6(x, ea) for x in a]
    sb = [slice6(x, eb) for x in b]
    acc = [0] * LEVELS
    for k in range(len(a)):
        for s in range(SLICES):
            for u in range(SLICES):
                if s + u < LEVELS:
                    acc[s + u] += sa[k][s] * sb[k][u]
    hi = acc[0] * 128 + acc[1]
    lo = sum(acc[L] << (7 * (LEVELS - 1 - L)) for L in range(2, LEVELS))
    tot = (hi << 34) + (lo >> 1)
    return acc, tot, ea + eb - 55, sa, ea


def test_slices_reconstruct_operands():
    rng = np.random.default_rng(0)
    row = rng.normal(size=64) * 10.0 ** rng.uniform(-4, 4, size=64)
    er = exp_bound(row)
    for x in row:
        s = slice6(x, er)
        rec = sum(Fraction(v) * Fraction(2) ** (er - 7 * (t + 1)) for t, v in enumerate(s))
        assert abs(rec - Fraction(x)) <= Fraction(2) ** (er - 42)


def test_levels_are_exact_in_fp32_even_at_the_worst_case():
    # every operand at the top of its row scale: the largest possible level sums
    a = [1.0 - 2.0 ** -52] * K
    acc, _, _, _, _ = contract(a, a)
    assert max(abs(v) for v in acc) < 2 ** 24


def test_dot_products_against_exact_arithmetic():
    rng = np.random.default_rng(1)
    worst = 0.0
    for trial in range(25):
        a = rng.normal(size=K) * 10.0 ** rng.uniform(-3, 3, size=K) * 10.0 ** rng.uniform(-80, 80)
        b = rng.normal(size=K) * 10.0 ** rng.uniform(-3, 3, size=K) * 10.0 ** rng.uniform(-80, 80)
        if trial % 5 == 0:
            a[:7] = 0.0
        acc, tot, e2, _, _ = contract(list(a), list(b))
        assert max(abs(v) for v in acc) < 2 ** 24
        val = Fraction(tot) * Fraction(2) ** e2
        exact = sum(Fraction(x) * Fraction(y) for x, y in zip(a, b))
        scale = sum(abs(Fraction(x) * Fraction(y)) for x, y in zip(a, b))
        worst = max(worst, float(abs(val - exact) / scale))
    # rows with a 10^6 spread of magnitudes: the operands are kept to 2^-42 of their row
    # maxima, so the error relative to sum |a||b| is at most a few times 1e-11
    assert worst < 5e-11, worst
