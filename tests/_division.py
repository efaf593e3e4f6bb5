"""Division by a grid spacing with the two-term reciprocal, restated in
Python for the tests: the quotient form, the numerators whose quotient lies
near a midpoint between doubles, and the per-spacing criterion, the last
also checked exhaustively at reduced precision in exact arithmetic."""
import ctypes
import math
from fractions import Fraction as F

_libm = ctypes.CDLL("libm.so.6")
_libm.fma.restype = ctypes.c_double
_libm.fma.argtypes = [ctypes.c_double] * 3


def fma(a, b, c):
    """correctly rounded a*b + c (C99 fma)"""
    return _libm.fma(a, b, c)


def recip(h):
    y = 1.0 / h
    return y, fma(-y, h, 1.0) / h


def two_term(a, h):
    """the kernels' two-term quotient of a / h (zero numerators and the
    exponent range outside [-900, 900] take the IEEE division)"""
    if a == 0.0:
        return a
    e = math.frexp(a)[1] - 1
    if e < -900 or e > 900 or not math.isfinite(a):
        return a / h
    y, yl = recip(h)
    return fma(a, y, a * yl)


def near_midpoint(H, kmax53=1, kmax54=3, p=53):
    """numerator mantissas A in [2^(p-1), 2^p) with 2^c A - H N = k, N odd,
    0 < |k| <= kmax (c = p: A/H in [1, 2); c = p + 1: A/H in [1/2, 1))"""
    out = []
    v = (H & -H).bit_length() - 1
    for c, kmax in ((p, kmax53), (p + 1, kmax54)):
        for k in range(-kmax, kmax + 1):
            if k == 0 or k % (1 << v):
                continue
            cc = c - v
            mod = 1 << cc
            kk = k // (1 << v)
            n0 = (-kk * pow(H >> v, -1, mod)) % mod
            N = n0
            while N < (1 << (p + 1)):
                if N > (1 << p) and N & 1:
                    num = H * N + k
                    A = num >> c
                    if num % (1 << c) == 0 and (1 << (p - 1)) <= A < (1 << p) and (A >= H) == (c == p):
                        out.append(A)
                N += mod
    return out


def mantissa(h):
    m, e = math.frexp(h)
    return int(math.ldexp(m, 53)), e


def criterion(h):
    """the per-spacing check of the library, restated: the two-term form on
    every near-midpoint numerator"""
    H, e = mantissa(h)
    for A in near_midpoint(H):
        a = math.ldexp(A, e - 53)
        if two_term(a, h) != a / h:
            return False
    return True


# ---- reduced precision p, exact rationals ------------------------------------

def _rn(x, p):
    if x == 0:
        return F(0)
    s = -1 if x < 0 else 1
    x = abs(x)
    e = x.numerator.bit_length() - x.denominator.bit_length()
    if F(2) ** e > x:
        e -= 1
    m = x * F(2) ** (p - 1 - e)
    n = m.numerator // m.denominator
    r = m - n
    if r > F(1, 2) or (r == F(1, 2) and n & 1):
        n += 1
    return s * n * F(2) ** (e - p + 1)


def reduced_precision_failures(H, p):
    """numerator mantissas A for which the two-term quotient at precision p
    differs from the correctly rounded A/H (every A, exact arithmetic)"""
    h = F(H, 1 << (p - 1))
    y = _rn(1 / h, p)
    t = _rn(1 - y * h, p)
    assert t == 1 - y * h          # the fused residual is exact
    yl = _rn(t / h, p)
    bad = set()
    for A in range(1 << (p - 1), 1 << p):
        a = F(A, 1 << (p - 1))
        if _rn(a * y + _rn(a * yl, p), p) != _rn(a / h, p):
            bad.add(A)
    return bad
