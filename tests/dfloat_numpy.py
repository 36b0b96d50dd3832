"""Double-float arithmetic on numpy float32 arrays, restating csrc/dfloat.cuh for
the CPU tests (Knuth two-sum, two-product by FMA).  A helper module, not a test."""
import numpy as np

f32, f64 = np.float32, np.float64


def fma(a, b, c):
    """fmaf(a, b, c): a*b is exact in FP64 for float32 operands; one rounding to FP32
    (exact whenever c is minus the rounded product, as in two_prod)."""
    return (a.astype(f64) * b.astype(f64) + c.astype(f64)).astype(f32)


def two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def fast_two_sum(a, b):
    s = a + b
    return s, b - (s - a)


def two_prod(a, b):
    p = a * b
    return p, fma(a, b, -p)


def df(x):
    h = np.asarray(x, f64).astype(f32)
    return h, (np.asarray(x, f64) - h).astype(f32)


def add(a, b):
    sh, sl = two_sum(a[0], b[0])
    return fast_two_sum(sh, sl + (a[1] + b[1]))


def neg(a):
    return -a[0], -a[1]


def mul(a, b):
    ph, pl = two_prod(a[0], b[0])
    return fast_two_sum(ph, pl + (a[0] * b[1] + a[1] * b[0]))


def mul_f(a, b):
    ph, pl = two_prod(a[0], b)
    return fast_two_sum(ph, pl + a[1] * b)


def div(a, b):
    q1 = a[0] / b[0]
    r = add(a, neg(mul_f(b, q1)))
    return fast_two_sum(q1, r[0] / b[0])


def dot3(ah, al, b):
    """df_dot3: three double-float coefficients times three double-float values."""
    p = [two_prod(ah[k], b[k][0]) for k in range(3)]
    s01 = two_sum(p[0][0], p[1][0])
    s = two_sum(s01[0], p[2][0])
    lo = ((p[0][1] + p[1][1]) + (p[2][1] + s01[1])) + s[1]
    for k in range(3):
        lo = fma(ah[k], b[k][1], lo)
    for k in range(3):
        lo = fma(al[k], b[k][0], lo)
    return fast_two_sum(s[0], lo)
