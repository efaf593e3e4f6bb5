"""CPU-only tests: the C-ABI library loads and exports every declared entry
point, argument checking fails loudly, the workload generator's invariants,
and known-answer tests of the oracle (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from turbins_gb300 import workload as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "turbins_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*)\s*(turb_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from turbins_gb300 import build
    return C.CDLL(build.build())


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_bad_arguments_fail_loudly(lib):
    ctx = C.c_void_p()
    assert lib.turb_create(None, None, C.byref(ctx)) == 1
    assert lib.turb_destroy(None) == 1
    assert lib.turb_step(None, C.c_double(1e-3), None) == 1
    assert lib.turb_ENO_compute_convective_terms(5, 10, None, None, None, None) == 1


def test_no_cpu_fallback_without_gpu(lib):
    """On a machine without a GPU the context cannot be created: the call
    returns TURB_ERR_CUDA instead of computing anything on the host."""
    from turbins_gb300 import api
    if os.environ.get("CUDA_VISIBLE_DEVICES") is None and os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    case = W.lock_exchange_case(8, 8, 8)
    with pytest.raises(api.TurbError) as e:
        api.Context(case.grid, case.params)
    assert e.value.code == 2


def test_uniform_axis_repeated_addition():
    c, f = W.uniform_axis(64, 0.0, 8.0)
    acc = 0.0
    for i in range(65):
        assert f[i] == acc
        acc += 8.0 * (1.0 / 64)
    assert len(c) == 65 and c[0] == 0.5 * 8.0 / 64


def test_tanh_axis_clusters_at_bed():
    c, f = W.tanh_axis(64, 0.0, 2.0, 1.5)
    d = np.diff(f)
    assert f[0] == 0.0 and abs(f[-1] - 2.0) < 1e-14
    assert np.all(d > 0) and d[0] < d[-1] / 3
    assert np.all((c[:-1] > f[:-1]) & (c[:-1] < f[1:]))


def test_status_box_boundaries():
    case = W.lock_exchange_case(8, 6, 4)
    st = case.grid.status
    assert np.all(st["u"][:, :, 0] == W.BOUNDARY) and np.all(st["u"][:, :, -1] == W.BOUNDARY)
    assert np.all(st["v"][:, 0, :] == W.BOUNDARY) and np.all(st["w"][0] == W.BOUNDARY)
    assert np.all(st["c"][:-1, :-1, :-1] == W.FLUID)


def test_immersed_stencils():
    case = W.turbidity_bump_case(48, 24, 8)
    g = case.grid
    for q in "uvw":
        ib = g.ib[q]
        assert ib["n"] > 0
        good = ib["nf"] == 8
        # Dirichlet: fluid coefficients are trilinear weights x ds/df (= 1)
        s = ib["fcoef"][good].sum(axis=1)
        assert np.allclose(s, ib["bcoef"][good] - 1.0)
        assert np.all(g.status[q].ravel()[ib["im"]] == W.IMMERSED)
    ib = g.ib["c"]
    good = (ib["nf"] == 8)
    sc = ib["fcoef"][good].sum(axis=1)
    assert np.all(sc <= 1e-12) and np.all(sc >= -1.0 - 1e-9)
    st = g.status["u"]
    assert (st == W.BUFFER_SOLID).sum() > 0 and (st == W.SOLID).sum() >= 0


def test_eno_known_answers(oracle_mod):
    """ENO-2 differentiates quadratics exactly, ENO-3 cubics (uniform grid)."""
    o = oracle_mod.Oracle.__new__(oracle_mod.Oracle)
    o.lib = C.CDLL(oracle_mod.build())
    x = np.linspace(0.0, 3.0, 31)
    h = x[1] - x[0]
    P = x.copy()
    for order, f, df in ((2, lambda t: 3 * t * t - t + 1, lambda t: 6 * t - 1),
                         (3, lambda t: t ** 3 - 2 * t * t + t, lambda t: 3 * t * t - 4 * t + 1)):
        for V in (np.ones_like(x), -np.ones_like(x)):
            out = o.eno_line(order, f(x), P, V)
            i = slice(order, len(x) - order)
            assert np.allclose(out[i], V[i] * df(x[i]), atol=1e-9 / h)


def test_eno_tie_and_zero_velocity(oracle_mod):
    """|D2[k]| == |D2[k+1]| picks the left stencil; V == 0 uses k = i (and
    contributes 0)."""
    o = oracle_mod.Oracle.__new__(oracle_mod.Oracle)
    o.lib = C.CDLL(oracle_mod.build())
    P = np.arange(9.0)
    D0 = np.array([0, 0, 0, 1, 0, 0, 0, 0, 0], float)   # symmetric bump: ties at i=3
    V = np.zeros(9)
    V[3] = 1.0
    out = o.eno_line(2, D0, P, V)
    # k = 2: D1[2] = 1; D2[2] = (1-0)/2, D2[3] = (-1-1)/2 -> |0.5| <= |1| picks left: c = 0.5
    assert out[3] == 1.0 * (1.0 + 0.5 * ((3 - 2) + (3 - 3)))
    assert np.all(out[[2, 4, 5, 6]] == 0.0)


def test_manufactured_poisson_second_order(oracle_mod):
    """Neumann cos*cos*cos manufactured solution (the Debugger.c form): the
    discrete solution converges at second order."""
    errs = []
    for n in (16, 32):
        case = W.lock_exchange_case(n, n, n)
        g = case.grid
        g.xc, g.xu = W.uniform_axis(n, 0.0, 1.0)
        o = oracle_mod.Oracle(g, case.params)
        X, Y, Z = np.meshgrid(g.xc, g.yc, g.zc, indexing="ij")
        k = np.pi
        ex = np.cos(k * X) * np.cos(k * Y) * np.cos(k * Z)
        ex = ex.transpose(2, 1, 0)
        b = 3 * k * k * ex
        b[g.status["c"] == W.BOUNDARY] = 0.0
        b[:-1, :-1, :-1] -= b[:-1, :-1, :-1].mean()
        case.params.p_rtol = 1e-12
        o2 = oracle_mod.Oracle(g, case.params)
        phi, it, rr = o2.pressure_solve(b, np.zeros(g.shape))
        m = np.zeros(g.shape, bool)
        m[:-1, :-1, :-1] = True
        e = (phi[m] - phi[m].mean()) - (ex[m] - ex[m].mean())
        errs.append(np.abs(e).max())
    assert errs[1] < errs[0] / 3.0


def test_projection_gate_and_nonconvergence(oracle_mod):
    case = W.lock_exchange_case(16, 8, 8)
    o = oracle_mod.Oracle(case.grid, case.params)
    rng = np.random.Generator(np.random.PCG64(1))
    u, v, w = [rng.standard_normal(case.grid.shape) * 1e-3 for _ in range(3)]
    for a, q in ((u, "u"), (v, "v"), (w, "w")):
        a[case.grid.status[q] == W.BOUNDARY] = 0.0
    b = o.pressure_rhs(1e-3, u, v, w)
    case.params.p_rtol = 1e-12
    o = oracle_mod.Oracle(case.grid, case.params)
    phi, it, rr = o.pressure_solve(b, np.zeros(case.grid.shape))
    z = np.zeros(case.grid.shape)
    o.project(1e-3, phi, b, u, v, w, z.copy(), z.copy(), z.copy())
    assert o.divergence(u, v, w)[0] <= 1e-10
    case.params.p_maxit = 1
    o = oracle_mod.Oracle(case.grid, case.params)
    phi, it, rr = o.pressure_solve(b, np.zeros(case.grid.shape))
    assert it == 1 and rr > 1e-12


def test_oracle_threads_give_same_bits(oracle_mod):
    """the oracle's parallel loops write disjoint outputs and its sums stay
    serial: two steps on 1 and on 4 threads give the same bits"""
    from tests import _cases
    case = _cases.multi_small(32, 16, 8)
    out = []
    for nt in (1, 4):
        oracle_mod.set_threads(nt)
        o = oracle_mod.Oracle(case.grid, case.params)
        s = {k: v.copy() for k, v in _cases.random_state(case, seed=3).items()}
        for _ in range(2):
            o.step(s, case.dt)
        out.append(s)
    oracle_mod.set_threads(1)
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
