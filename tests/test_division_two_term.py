"""The ENO kernels divide by a grid spacing h with the two-term quotient
RN(a y + RN(a yl)) alone (one multiply, one fused multiply-add) when the
set-up's check says that form rounds as the IEEE division for every
numerator, and with the Markstein-corrected form otherwise.  These CPU tests
pin the check: its criterion against an exhaustive search at reduced
precision, the library's check against the Python restatement, and the
flagged spacings against IEEE division on the hardest numerators (quotients
near midpoints between doubles).  CPU arithmetic rounds as the GPU's (IEEE
double, correctly rounded fma), so what holds here holds in the kernels;
tests/test_gpu_parity.py compares the kernels' quotients with these."""
import math
import random

import numpy as np
import pytest

from tests import _division as D


@pytest.mark.parametrize("p", [7, 8, 9])
def test_criterion_is_exact_at_reduced_precision(p):
    """At precision p, for every divisor mantissa H: every numerator on which
    the two-term form fails is one of the near-midpoint candidates, so
    trying the candidates decides the divisor."""
    unsafe = 0
    for H in range(1 << (p - 1), 1 << p):
        bad = D.reduced_precision_failures(H, p)
        cands = set(D.near_midpoint(H, p=p))
        assert bad <= cands, (H, sorted(bad - cands))
        unsafe += bool(bad)
    assert unsafe < (1 << (p - 1)) // 8


def _spacings(n, seed):
    rng = random.Random(seed)
    hs = [math.ldexp(rng.uniform(1.0, 2.0), rng.randint(-14, 3)) for _ in range(n)]
    # short mantissas and differences of tanh-stretched coordinates
    hs += [0.75, 1.5, 3.0 / 1024, 0.1, 0.2, 0.3, 1.0 / 3.0, 0.01]
    y = [2.0 * (1.0 + math.tanh(1.5 * (j / 256.0 - 1.0)) / math.tanh(1.5)) for j in range(257)]
    hs += [y[j + 1] - y[j] for j in range(0, 256, 7)] + [y[j + 2] - y[j - 1] for j in range(1, 254, 11)]
    return hs


@pytest.fixture(scope="module")
def lib_check():
    api = pytest.importorskip("turbins_gb300.api")
    try:
        api.load_library()
    except api.TurbError:
        pytest.skip("libturbgpu.so not built")
    return api.division_two_term_exact


def test_library_check_matches_restatement(lib_check):
    hs = _spacings(3000, 11)
    got = [lib_check(h) for h in hs]
    want = [D.criterion(h) for h in hs]
    assert got == want
    frac = sum(got) / len(got)
    assert 0.95 < frac < 1.0, frac


def test_flagged_spacings_divide_exactly(lib_check):
    """flagged spacings: the two-term form equals the IEEE quotient on every
    numerator within |k| <= 64 of a midpoint (both binades) and on random
    numerators over the exponent range; unflagged ones fail on a candidate"""
    rng = random.Random(5)
    n_flag = n_unflag = 0
    for h in _spacings(300, 12):
        H, e = D.mantissa(h)
        As = D.near_midpoint(H, 64, 64) + [rng.randrange(1 << 52, 1 << 53) for _ in range(64)]
        flagged = lib_check(h)
        fails = 0
        for A in As:
            for sh in (0, -37, 41, -400, 400):
                a = math.ldexp(A, e - 53 + sh)
                for s in (a, -a):
                    fails += D.two_term(s, h) != s / h
        if flagged:
            n_flag += 1
            assert fails == 0, h
        else:
            n_unflag += 1
            assert fails > 0, h
    assert n_flag > 0 and n_unflag > 0


def test_special_numerators(lib_check):
    h = 0.0123456789
    assert lib_check(h)
    for a in (0.0, -0.0, 5e-324, -5e-324, 1e-300, 1e300, -1e-280, float("inf"), float("-inf")):
        q, r = D.two_term(a, h), a / h
        assert np.float64(q).tobytes() == np.float64(r).tobytes(), a
    assert math.isnan(D.two_term(float("nan"), h))
