"""Float-float exponential of the MBIS "ff" kernels, emulated on the CPU.

The device routine (``exp_ff`` in ``horton_part_gb300/csrc/hp_ff.cuh``) is
replayed step by step in NumPy float32 arithmetic (an FMA is emulated
exactly: a float32 product is exact in float64) to check the method itself,
its split constants for ln2/64 and its table, against float64 exp. The GPU
tests check the kernels end to end against the FP64 path.
"""

import numpy as np

f32 = np.float32


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def two_prod(a, b):
    p = f32(a * b)
    return p, fma(a, b, -p)


def add(a, b):
    s = two_sum(a[0], b[0])
    t = two_sum(a[1], b[1])
    s = (s[0], f32(s[1] + t[0]))
    s = fast_two_sum(*s)
    s = (s[0], f32(s[1] + t[1]))
    return fast_two_sum(*s)


def add_pos(a, b):
    s = two_sum(a[0], b[0])
    return fast_two_sum(s[0], f32(s[1] + f32(a[1] + b[1])))


def add_f(a, b):
    s = two_sum(a[0], b)
    return fast_two_sum(s[0], f32(s[1] + a[1]))


def mul(a, b):
    p, e = two_prod(a[0], b[0])
    e = fma(a[0], b[1], e)
    e = fma(a[1], b[0], e)
    return fast_two_sum(p, e)


TABLE = []
for i in range(64):
    v = 2.0 ** (i / 64.0)
    hi = f32(v)
    TABLE.append((hi, f32(v - np.float64(hi))))

L1 = f32(float.fromhex("0x1.63p-7"))
L2 = f32(float.fromhex("-0x1.bd0106p-19"))
L3 = f32(float.fromhex("0x1.cf79acp-46"))


def exp_ff(x):
    if x[0] < f32(-87.0):
        return (f32(0), f32(0))
    nf = f32(np.rint(f32(x[0] * f32(92.3324813842773))))
    n = int(nf)
    p2 = two_prod(nf, L2)
    r = two_sum(f32(x[0] - f32(nf * L1)), x[1])
    r = add_f(r, f32(-p2[0]))
    r = add_f(r, f32(-(f32(p2[1] + f32(nf * L3)))))
    sq = two_prod(r[0], r[0])
    sq = fast_two_sum(sq[0], fma(f32(2.0) * r[0], r[1], sq[1]))
    half = (f32(0.5) * sq[0], f32(0.5) * sq[1])
    c = f32(f32(r[0] * sq[0]) * fma(r[0], fma(r[0], f32(1.0 / 120.0), f32(1.0 / 24.0)), f32(1.0 / 6.0)))
    e = add_pos(r, half)
    e = add_f(e, c)
    e = add_f(e, f32(1.0))
    m = n >> 6
    i = n - (m << 6)
    v = mul(TABLE[i], e)
    scale = f32(2.0 ** max(min(m, 127), -126))
    return (f32(v[0] * scale), f32(v[1] * scale))


def split(v):
    hi = f32(v)
    return (hi, f32(v - np.float64(hi)))


def test_split_constants_reproduce_ln2_over_64():
    total = np.float64(L1) + np.float64(L2) + np.float64(L3)
    assert abs(total - np.log(2.0) / 64.0) < 1e-19
    # n * L1 must be exact for every reduction index of the argument range
    for n in (1, 63, 4097, 8064):
        assert np.float64(L1) * n == np.float64(f32(L1 * f32(n)))


def test_exp_ff_matches_float64_exp():
    """Relative error ~1e-15 down to exp(-60) ~ 1e-26; below that the low
    float becomes subnormal and only the absolute error stays tiny (such
    terms are far below the 1e-15 density cutoff of every ratio)."""
    rng = np.random.default_rng(7)
    xs = np.concatenate([-np.geomspace(1e-8, 86.9, 400), rng.uniform(-86.9, 0.0, 600), [0.0]])
    worst_rel, worst_abs = 0.0, 0.0
    for x in xs:
        hi, lo = split(x)
        v = exp_ff((hi, lo))
        got = np.float64(v[0]) + np.float64(v[1])
        ref = np.exp(np.float64(hi) + np.float64(lo))
        if x >= -60.0:
            worst_rel = max(worst_rel, abs(got - ref) / ref)
        else:
            worst_abs = max(worst_abs, abs(got - ref))
    assert worst_rel < 1e-14, worst_rel
    assert worst_abs < 1e-40, worst_abs


def test_exp_ff_underflows_to_zero_below_float_range():
    assert exp_ff(split(-90.0)) == (0.0, 0.0)
