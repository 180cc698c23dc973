"""The double-float methods of mechafm_gb300/csrc/dfloat.cuh, restated step
for step in numpy FP32 arithmetic (an FMA is the exact float64 product plus
the addend, rounded once), checked against 120-bit arithmetic (mpmath).

The relax kernel's FP64-faithful claim rests on these error levels: one
double-float operation within a few 1e-15, a chain of them (exp, the LJ
powers) within a few 1e-14 to 1e-13 relative, all far below the near-tie
margins (1e-8 of the tolerances) that send a column to the FP64
re-relaxation.  The GPU tests check the kernels themselves against FP64.
"""
import numpy as np
import pytest

mpmath = pytest.importorskip("mpmath")

f32 = np.float32


def add(a, b):
    return f32(f32(a) + f32(b))


def sub(a, b):
    return f32(f32(a) - f32(b))


def mul(a, b):
    return f32(f32(a) * f32(b))


def fma(a, b, c):
    return f32(mpmath.mpf(float(a)) * mpmath.mpf(float(b)) + mpmath.mpf(float(c)))


def two_sum(a, b):
    s = add(a, b)
    bb = sub(s, a)
    return s, add(sub(a, sub(s, bb)), sub(b, bb))


def fast_two_sum(a, b):
    s = add(a, b)
    return s, sub(b, sub(s, a))


def dadd(a, b):           # operator+ (sloppy sum, renormalised)
    s, e = two_sum(a[0], b[0])
    return fast_two_sum(s, add(e, add(a[1], b[1])))


def dadd_u(a, b):         # dfl2_add_u: no renormalisation
    s, e = two_sum(a[0], b[0])
    return s, add(e, add(a[1], b[1]))


def dmul_u(a, b):         # dfl2_mul_u
    p = mul(a[0], b[0])
    e = fma(a[0], b[0], -p)
    e = fma(a[0], b[1], e)
    return p, fma(a[1], b[0], e)


def dmulf_u(a, x):        # dfl2_mulf_u
    p = mul(a[0], x)
    return p, fma(a[1], x, fma(a[0], x, -p))


def split(x):
    h = f32(x)
    return h, f32(x - float(h))


def value(a):
    return mpmath.mpf(float(a[0])) + mpmath.mpf(float(a[1]))


LN2 = 0.69314718055994530942
LN2_HI = f32(0.693145751953125)
LN2_MID = f32(LN2 - float(LN2_HI))
LN2_LO = f32(LN2 - float(LN2_HI) - float(LN2_MID))
INV_FACT = [1.0 / float(mpmath.factorial(k)) for k in range(8)]


def dexp(x):
    """dfl2_exp for one element: Cody–Waite reduction, r / 16, degree-7
    Horner expm1, four doublings, 2^n (1 + e)."""
    n = f32(np.rint(mul(x[0], f32(1.44269504088896341))))
    r = dadd(x, (-mul(n, LN2_HI), f32(0)))
    p = mul(n, LN2_MID)
    r = dadd(r, (-p, -fma(n, LN2_MID, -p)))
    r = dadd(r, (-mul(n, LN2_LO), f32(0)))
    r = (mul(r[0], f32(0.0625)), mul(r[1], f32(0.0625)))
    q = split(INV_FACT[7])
    for k in range(6, 0, -1):
        q = dadd_u(dmul_u(q, r), split(INV_FACT[k]))
    e = dmul_u(q, r)
    for _ in range(4):
        e = dmul_u(e, dadd_u((f32(2), f32(0)), e))
    y = fast_two_sum(*dadd_u((f32(1), f32(0)), e))
    return mpmath.ldexp(value(y), int(n))


def drsqrt(a):
    """rsqrt_u: one Newton step from the FP32 approximation (here the FP32
    rounding of the exact value stands in for rsqrt.approx)."""
    y = f32(1.0 / np.sqrt(float(a[0])))
    t = dmulf_u(dmulf_u(a, y), y)
    e = sub(sub(f32(1), t[0]), t[1])
    return fast_two_sum(y, mul(mul(y, e), f32(0.5)))


@pytest.fixture(autouse=True)
def _precision():
    old = mpmath.mp.prec
    mpmath.mp.prec = 120
    yield
    mpmath.mp.prec = old


def test_exp_is_within_3e_14_relative():
    rng = np.random.default_rng(7)
    worst = 0.0
    for x in rng.uniform(-20.0, 8.0, 200):     # Morse arguments -a (r - re)
        d = split(x)
        want = mpmath.exp(value(d))
        worst = max(worst, float(abs(dexp(d) - want) / want))
    assert worst < 3e-14, worst      # measured 1.4e-14


def test_rsqrt_is_within_1e_14_relative():
    rng = np.random.default_rng(8)
    worst = 0.0
    for x in rng.uniform(1.0, 400.0, 200):     # r^2 of the tip–atom terms, A^2
        d = split(x)
        want = 1 / mpmath.sqrt(value(d))
        worst = max(worst, float(abs(value(drsqrt(d)) - want) / want))
    assert worst < 1e-14, worst


def test_unnormalised_product_chain_keeps_double_float_accuracy():
    """r^-12 from r^-1 by five unnormalised products with one
    renormalisation at r^-6 (a longer chain than any in the LJ term): within
    3e-13 of the exact power (measured 1.5e-13; the same chain of
    renormalised products 5e-14, one product 3.6e-15)."""
    rng = np.random.default_rng(9)
    worst = 0.0
    for x in rng.uniform(0.05, 0.5, 200):      # 1/r for r in 2-20 A
        ir = split(x)
        ir2 = dmul_u(ir, ir)
        ir6 = fast_two_sum(*dmul_u(dmul_u(ir2, ir2), ir2))
        ir12 = dmul_u(ir6, ir6)
        want = value(ir) ** 12
        worst = max(worst, float(abs(value(ir12) - want) / want))
    assert worst < 3e-13, worst
