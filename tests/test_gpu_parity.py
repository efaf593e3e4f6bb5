"""GPU parity of every hot-path routine against the CPU oracle, through the
C ABI.  Integer-like / element-wise and ENO results are compared bit for bit
(ENO stencil choices and fluxes are bit-identical by construction); solver
outputs are compared within the tolerances the solvers converge to."""
import numpy as np
import pytest

from tests import _cases

pytestmark = pytest.mark.gpu

F = None


@pytest.fixture(scope="module")
def api():
    from turbins_gb300 import api as A
    from turbins_gb300 import build
    build.build()
    global F
    F = A
    return A


def _pair(case, api, oracle_mod, state=None):
    ctx = api.Context(case.grid, case.params)
    orc = oracle_mod.Oracle(case.grid, case.params)
    s = state if state is not None else case.state
    ctx.load_state(s)
    return ctx, orc, s


def same(a, b):
    """bitwise equality treating +0 and -0 as equal"""
    return np.array_equal(a, b)


CASES = [("lock", lambda: _cases.lock_small(order=2)),
         ("lock3", lambda: _cases.lock_small(order=3)),
         ("bump", lambda: _cases.bump_small()),
         ("multi", lambda: _cases.multi_small())]


@pytest.mark.parametrize("order", [1, 2, 3])
def test_eno_line_bitexact(api, oracle_mod, order):
    rng = np.random.Generator(np.random.PCG64(7 + order))
    from turbins_gb300 import workload as W
    g = W.make_grid(8, 8, 8, (1.0, 1.0, 1.0))
    orc = oracle_mod.Oracle.__new__(oracle_mod.Oracle)
    orc.lib = __import__("ctypes").CDLL(oracle_mod.build())
    for n in (2 * order + 2, 37, 300):
        P = np.cumsum(rng.uniform(0.5, 1.5, n))
        D0 = rng.standard_normal(n)
        D0[n // 3: n // 3 + 5] = 0.25          # flat run -> exact ties
        V = rng.standard_normal(n)
        V[::7] = 0.0                           # V == 0 picks k = i
        a = api.ENO_compute_convective_terms(order, D0, P, V)
        b = orc.eno_line(order, D0, P, V)
        assert same(a[order:n - order], b[order:n - order])


@pytest.mark.parametrize("name,mk", CASES)
def test_cell_center_transpose_bitexact(api, oracle_mod, name, mk):
    case = mk()
    s = _cases.random_state(case)
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    ctx.Velocity_cell_center()
    ub, vb, wb = orc.cell_center(s["u"], s["v"], s["w"])
    m = np.zeros(case.grid.shape, bool)
    m[:-1, :-1, :-1] = True
    assert same(ctx.download(api.F_UBC)[m], ub[m])
    assert same(ctx.download(api.F_VBC)[m], vb[m])
    assert same(ctx.download(api.F_WBC)[m], wb[m])
    for q in "uvw":
        ctx.Velocity_transpose_velocities(q)
        A, B = orc.transpose(q, s["u"], s["v"], s["w"])
        nb = case.grid.status[q] != 7
        assert same(ctx.download(api.F_SCRATCH0)[nb], A[nb])
        assert same(ctx.download(api.F_SCRATCH1)[nb], B[nb])


def test_division_selftest(api):
    """The ENO kernels divide by grid spacings through a precomputed
    reciprocal and two Markstein corrections; that must give the IEEE
    quotient bit for bit (random, near-representable and near-midpoint
    quotients, differences of nearby values)."""
    for seed in (1, 2, 3, 4):
        bad, ex = api.selftest_division(1 << 29, seed)
        assert bad == 0, (bad, ex)


def test_two_term_division_on_device(api):
    """The kernels' two-term quotient on the GPU equals the CPU's (libm fma)
    on every pair, and the IEEE quotient wherever the set-up's check flags
    the spacing; the pairs are the near-midpoint numerators (|k| <= 8) of
    seeded spacings, where an unflagged spacing fails."""
    import math
    import random
    from tests import _division as D
    rng = random.Random(21)
    a, h, flag = [], [], []
    for _ in range(400):
        hh = math.ldexp(rng.uniform(1.0, 2.0), rng.randint(-14, 3))
        H, e = D.mantissa(hh)
        f = api.division_two_term_exact(hh)
        for A in D.near_midpoint(H, 8, 8) + [rng.randrange(1 << 52, 1 << 53) for _ in range(8)]:
            for sh in (0, -300, 300):
                for s in (1.0, -1.0):
                    a.append(s * math.ldexp(A, e - 53 + sh))
                    h.append(hh)
                    flag.append(f)
    a, h, flag = np.array(a), np.array(h), np.array(flag)
    q2, qd = api.selftest_division_pairs(a, h)
    host = np.array([D.two_term(x, y) for x, y in zip(a, h)])
    bits = lambda x: x.view(np.int64)
    assert np.array_equal(bits(q2), bits(host))
    assert np.array_equal(bits(q2[flag]), bits(qd[flag]))
    assert flag.any() and (~flag).any()
    assert (q2[~flag] != qd[~flag]).any()


@pytest.mark.parametrize("fastdiv", [1, 0])
@pytest.mark.parametrize("name,mk", CASES)
def test_convection_bitexact(api, oracle_mod, name, mk, fastdiv):
    case = mk()
    s = _cases.random_state(case, seed=3)
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    ctx.set_eno_division(fastdiv)
    for q, f in (("u", api.F_CONV_U), ("v", api.F_CONV_V), ("w", api.F_CONV_W)):
        ctx.Velocity_convective_terms(q)
        if q == "u":
            vx, (vy, vz) = s["u"], orc.transpose("u", s["u"], s["v"], s["w"])
        elif q == "v":
            A, B = orc.transpose("v", s["u"], s["v"], s["w"])
            vx, vy, vz = A, s["v"], B
        else:
            A, B = orc.transpose("w", s["u"], s["v"], s["w"])
            vx, vy, vz = A, B, s["w"]
        ref = orc.convection_vel(q, s[q], vx, vy, vz)
        got = ctx.download(f)
        assert same(got, ref), "%s conv mismatch: max %g" % (q, np.abs(got - ref).max())
    ctx.Velocity_cell_center()
    ub, vb, wb = orc.cell_center(s["u"], s["v"], s["w"])
    for ic in range(case.params.nconc):
        ctx.Conc_convective_terms(ic)
        va = vb + case.params.vs0[ic] if case.params.ctype[ic] == 2 else vb
        ref = orc.convection_conc(ic, s["c%d" % ic], ub, va, wb)
        got = ctx.download(api.F_CCONV0 + ic)
        assert same(got, ref), "c%d conv mismatch: max %g" % (ic, np.abs(got - ref).max())


@pytest.mark.parametrize("name,mk", CASES)
def test_rhs_projection_divergence_bitexact(api, oracle_mod, name, mk):
    case = mk()
    s = _cases.random_state(case, seed=5)
    dt = case.dt
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    n = case.params.nconc
    if n > 1:
        ctx.Conc_compute_total_concentration()
        ct = orc.total_concentration([s["c%d" % i] for i in range(n)])
        assert same(ctx.download(api.F_CTOT), ct)
    else:
        ct = s["c0"]
    for q, fc, fd, fb in (("u", api.F_CONV_U, "dpx", api.F_B_U), ("v", api.F_CONV_V, "dpy", api.F_B_V),
                          ("w", api.F_CONV_W, "dpz", api.F_B_W)):
        conv = 0.1 * s[q] + 0.01
        ctx.upload(fc, conv)
        ctx.Velocity_set_RHS(q, dt)
        assert same(ctx.download(fb), orc.set_rhs_vel(q, dt, s[q], conv, s[fd], ct))
    for ic in range(n):
        conv = 0.3 * s["c%d" % ic]
        ctx.upload(api.F_CCONV0 + ic, conv)
        ctx.Conc_set_RHS(ic, dt)
        assert same(ctx.download(api.F_CB0 + ic), orc.set_rhs_conc(dt, s["c%d" % ic], conv))
    ctx.Pressure_set_RHS(dt)
    pb = orc.pressure_rhs(dt, s["u"], s["v"], s["w"])
    assert same(ctx.download(api.F_PB), pb)
    ctx.Pressure_project_velocity(dt)
    u, v, w = s["u"].copy(), s["v"].copy(), s["w"].copy()
    dpx, dpy, dpz = s["dpx"].copy(), s["dpy"].copy(), s["dpz"].copy()
    orc.project(dt, s["phi"], pb, u, v, w, dpx, dpy, dpz)
    for f, ref in ((api.F_U, u), (api.F_V, v), (api.F_W, w), (api.F_DPX, dpx), (api.F_DPY, dpy), (api.F_DPZ, dpz)):
        assert same(ctx.download(f), ref)
    dm = ctx.Pressure_compute_velocity_divergence()
    dmo, div = orc.divergence(u, v, w)
    assert dm == dmo
    assert same(ctx.download(api.F_DIV), div)


@pytest.mark.parametrize("name,mk", CASES)
def test_operators(api, oracle_mod, name, mk):
    case = mk()
    s = _cases.random_state(case, seed=9)
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    dt = case.dt
    x = s["phi"]
    ctx.upload(api.F_SCRATCH0, x)
    for q in "uvw":
        ctx.helmholtz_apply(q, 0, dt, api.F_SCRATCH0, api.F_SCRATCH1)
        ref = orc.helmholtz_apply(q, 0, dt, x)
        got = ctx.download(api.F_SCRATCH1)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    for ic in range(case.params.nconc):
        ctx.helmholtz_apply("c", ic, dt, api.F_SCRATCH0, api.F_SCRATCH1)
        ref = orc.helmholtz_apply("c", ic, dt, x)
        got = ctx.download(api.F_SCRATCH1)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    ctx.pressure_apply(api.F_SCRATCH0, api.F_SCRATCH1)
    ref = orc.pressure_apply(x)
    got = ctx.download(api.F_SCRATCH1)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("name,mk", CASES)
@pytest.mark.parametrize("mode", [0, 1])
def test_pressure_solve(api, oracle_mod, name, mk, mode):
    """Mean-removed pressure within 1e-8 relative of the oracle's exact discrete
    solution; post-projection max|div u| <= 1e-10."""
    case = mk()
    # a random (strongly divergent) velocity needs a tighter relative residual
    # than a physical step to reach the absolute |div| gate
    case.params.p_rtol = 1e-12
    s = _cases.random_state(case, seed=11)
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    ctx.set_pressure_mode(mode)
    dt = case.dt
    ctx.Pressure_set_RHS(dt)
    it, rr = ctx.Pressure_solve()
    assert rr <= case.params.p_rtol
    pb = orc.pressure_rhs(dt, s["u"], s["v"], s["w"])
    case.params.p_rtol = 1e-13
    orc2 = type(orc)(case.grid, case.params)
    phi_ref, _, _ = orc2.pressure_solve(pb, s["phi"])
    phi = ctx.download(api.F_PHI)
    m = np.zeros(case.grid.shape, bool)
    m[:-1, :-1, :-1] = True
    a = phi[m] - phi[m].mean()
    b = phi_ref[m] - phi_ref[m].mean()
    assert np.abs(a - b).max() <= 1e-8 * np.abs(b).max()
    ctx.Pressure_project_velocity(dt)
    assert ctx.Pressure_compute_velocity_divergence() <= 1e-10


@pytest.mark.parametrize("name,mk", CASES + [("bump_64", lambda: _cases.bump_small(64, 40, 24))])
def test_mg_split_storage_is_bit_identical(api, oracle_mod, name, mk):
    """The FP32 multigrid levels' colour-split storage changes only where
    values live: the mixed-precision solve gives the same iterates bit for
    bit as with natural storage."""
    case = mk()
    s = _cases.random_state(case, seed=11)
    out = []
    for split in (False, True):
        ctx, orc, _ = _pair(case, api, oracle_mod, s)
        ctx.set_pressure_mode(api.PMODE_MIXED)
        ctx.set_mg_split(split)
        ctx.Pressure_set_RHS(case.dt)
        it, rr = ctx.Pressure_solve()
        out.append((it, rr, ctx.download(api.F_PHI)))
        ctx.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert same(out[0][2], out[1][2])


@pytest.mark.parametrize("name,mk", CASES[:3])
@pytest.mark.parametrize("hmode", [0, 1])
def test_helmholtz_solve(api, oracle_mod, name, mk, hmode):
    """FP64 Jacobi and FP64-residual/FP32-inner defect correction both reach
    the discrete solution of the oracle's BiCGStab (KSPIBCGS)."""
    case = mk()
    s = _cases.random_state(case, seed=13)
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    ctx.set_helmholtz_mode(hmode, 6)
    dt = case.dt
    for q, f, fb in (("u", api.F_U, api.F_B_U), ("v", api.F_V, api.F_B_V), ("w", api.F_W, api.F_B_W)):
        b = s[q] / dt + 0.1
        b[case.grid.status[q] != 3] = 0.0
        ctx.upload(fb, b)
        it = ctx.Velocity_solve(q, dt)
        x = ctx.download(f)
        case.params.vel_rtol = 1e-14
        orc2 = type(orc)(case.grid, case.params)
        xr, itr, rr = orc2.helmholtz_solve(q, 0, dt, b, s[q], method=0)
        assert np.abs(x - xr).max() <= 1e-10 * max(1.0, np.abs(xr).max())
        case.params.vel_rtol = 1e-12
    for ic in range(case.params.nconc):
        b = s["c%d" % ic] / dt
        b[case.grid.status["c"] != 3] = 0.0
        ctx.upload(api.F_CB0 + ic, b)
        ctx.Conc_solve(ic, dt)
        x = ctx.download(api.F_C0 + ic)
        case.params.vel_rtol = 1e-14
        orc2 = type(orc)(case.grid, case.params)
        xr, itr, rr = orc2.helmholtz_solve("c", ic, dt, b, s["c%d" % ic], method=0)
        assert np.abs(x - xr).max() <= 1e-10 * max(1.0, np.abs(xr).max())
        case.params.vel_rtol = 1e-12


@pytest.mark.parametrize("name,mk", CASES[:3])
def test_step_matches_oracle(api, oracle_mod, name, mk):
    """Two full TVD-RK2 steps on the GPU against the oracle's steps: the
    solvers differ (Jacobi vs BiCGStab, MG-CG variants), so fields agree to the
    solver tolerances, and the GPU divergence gate holds."""
    case = mk()
    ctx, orc, s = _pair(case, api, oracle_mod)
    so = {k: v.copy() for k, v in s.items()}
    for _ in range(2):
        st = ctx.step(case.dt)
        orc.step(so, case.dt)
        assert max(st["div_max"]) <= 1e-10
    g = ctx.state()
    # the solvers stop at relative residuals 1e-12 (Helmholtz) and 1e-10
    # (Poisson) of their right-hand sides, so differences are measured
    # against the velocity scale, not each component's own magnitude
    vscale = max(np.abs(so[k]).max() for k in ("u", "v", "w"))
    for k in ("u", "v", "w"):
        assert np.abs(g[k] - so[k]).max() <= 1e-7 * vscale, k
    assert np.abs(g["c0"] - so["c0"]).max() <= 1e-9 * np.abs(so["c0"]).max()


def _front_limit(h, alpha):
    """a limit between two heights of the alpha-weighted h(x) profile, so the
    front scan finds a crossing"""
    hw = sum(h[i] * alpha[i] for i in range(len(h)))
    for i in range(len(hw) - 2, 0, -1):
        if hw[i - 1] > hw[i]:
            return 0.5 * (hw[i - 1] + hw[i])
    return 0.05


DIAG_CASES = CASES + [("bump_64", lambda: _cases.bump_small(64, 40, 24))]


@pytest.mark.parametrize("name,mk", DIAG_CASES)
def test_deposit_and_bed_index(api, oracle_mod, name, mk):
    """Bed index and one deposited-height integration are per-node results:
    bit-identical to the oracle."""
    case = mk()
    s = _cases.random_state(case, seed=9)
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    nc = case.params.nconc
    assert np.array_equal(ctx.bed_index(), orc.interface_y_index())
    rng = np.random.default_rng(4)
    cs = [s["c%d" % i] for i in range(nc)]
    cold = [c + 0.01 * rng.standard_normal(c.shape) for c in cs]
    dep0 = rng.uniform(0.0, 0.01, (nc, case.grid.nz + 1, case.grid.nx + 1))
    for i in range(nc):
        ctx.upload(api.F_C0 + i, cold[i])
    ctx.store_old_data()
    for i in range(nc):
        ctx.upload(api.F_C0 + i, cs[i])
    ctx.set_deposit(dep0)
    ctx.deposit_integrate(case.dt)
    assert same(ctx.deposit(), orc.deposit_integrate(cs, cold, case.dt, dep0.copy()))


@pytest.mark.parametrize("name,mk", DIAG_CASES)
def test_diagnostics(api, oracle_mod, name, mk):
    """Flow integrals, heights, front location and bed rates on the GPU
    against the oracle (itself pinned to the reference's Extract.c / Conc.c):
    per-node terms are bit-identical, the device sums run in block order, so
    agreement is to 1e-12 relative, not bitwise."""
    case = mk()
    s = _cases.random_state(case, seed=9)
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    nc = case.params.nconc
    cs = [s["c%d" % i] for i in range(nc)]
    dep = np.random.default_rng(5).uniform(0.0, 0.01, (nc, case.grid.nz + 1, case.grid.nx + 1))
    ctx.set_deposit(dep)
    h0 = orc.diagnostics(s["u"], s["v"], s["w"], cs, 0.05)["ave_height"]
    limit = _front_limit(h0, case.params.alpha)
    ref = orc.diagnostics(s["u"], s["v"], s["w"], cs, limit, dep=dep)
    got = ctx.diagnostics(limit)
    for k in ("kinetic_energy", "conversion_rate", "viscous_dissipation"):
        assert abs(got[k] - ref[k]) <= 1e-12 * abs(ref[k]) + 1e-300, k
    for k in ("suspended_mass", "potential_energy", "stokes_dissipation", "conversion_rate_c", "ep_passive",
              "ep_passive_rate", "ep_rate", "sed_rate"):
        a, b = np.array(got[k]), np.array(ref[k])
        assert np.all(np.abs(a - b) <= 1e-12 * np.abs(b)), k
    hr = ref["ave_height"]
    assert np.abs(got["ave_height"] - hr).max() <= 1e-12 * np.abs(hr).max()
    assert same(got["sed_bottom"], ref["sed_bottom"])
    assert ref["front_location"] > 0.0
    assert abs(got["front_location"] - ref["front_location"]) <= 1e-9


def test_deposit_in_step(api, oracle_mod):
    """turb_deposit_enable: two steps integrate the deposit from each step's
    start and end concentrations, as the oracle does after its steps."""
    case = _cases.multi_small()
    ctx, orc, s = _pair(case, api, oracle_mod)
    so = {k: v.copy() for k, v in s.items()}
    nc = case.params.nconc
    ctx.deposit_enable(True)
    dep = np.zeros((nc, case.grid.nz + 1, case.grid.nx + 1))
    for _ in range(2):
        ctx.step(case.dt)
        cold = [so["c%d" % i].copy() for i in range(nc)]
        orc.step(so, case.dt)
        orc.deposit_integrate([so["c%d" % i] for i in range(nc)], cold, case.dt, dep)
    got = ctx.deposit()
    assert dep.max() > 0.0
    assert np.abs(got - dep).max() <= 1e-9 * dep.max()


def _golden_cases():
    import glob
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    return sorted(glob.glob(os.path.join(here, "*_eno*.npz")))


@pytest.mark.parametrize("path", _golden_cases(), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_step_matches_reference_trace(api, path):
    """Two GPU steps from the fixture's state against two steps composed of
    the reference's own routines (tests/golden/make_golden.py), solvers at
    relative residual 1e-12: fields agree to the solvers' tolerance.  The
    Helmholtz test |b - A x| <= 1e-12 |b| is global and |b| is dominated by
    the 1/dt rows, so Neumann immersed rows of the concentration (scale
    ap_solid << 1/dt) are resolved only to ~1e-7 by Jacobi (GPU) as by
    BiCGStab (reference): concentration is compared at 1e-6."""
    from tests.test_oracle_golden import load
    z, g, p, dt = load(path)
    p.p_rtol = 1e-12
    p.vel_rtol = 1e-12
    keys = ["u", "v", "w", "phi", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(p.nconc)]
    ctx = api.Context(g, p)
    ctx.load_state({k: z["in_" + k] for k in keys})
    for _ in range(2):
        st = ctx.step(dt)
        assert max(st["div_max"]) <= 1e-10
    s = ctx.state()
    vscale = max(np.abs(z["ref_step2_" + k]).max() for k in "uvw")
    for k in ("u", "v", "w"):
        assert np.abs(s[k] - z["ref_step2_" + k]).max() <= 1e-7 * vscale, k
    for i in range(p.nconc):
        ref = z["ref_step2_c%d" % i]
        assert np.abs(s["c%d" % i] - ref).max() <= 1e-6 * max(np.abs(ref).max(), 1.0)
    ctx.close()


def test_failure_paths(api, oracle_mod):
    """Non-convergence and non-finite input come back as status codes; the
    context stays usable afterwards."""
    case = _cases.bump_small()
    ctx, orc, s = _pair(case, api, oracle_mod, _cases.random_state(case, seed=17))
    case.params.p_maxit = 1
    ctx2 = api.Context(case.grid, case.params)
    ctx2.load_state(s)
    ctx2.Pressure_set_RHS(case.dt)
    with pytest.raises(api.TurbError) as e:
        ctx2.Pressure_solve()
    assert e.value.code == 3
    b = np.zeros(case.grid.shape)
    b[3, 3, 3] = np.nan
    ctx.upload(api.F_B_U, b)
    with pytest.raises(api.TurbError) as e:
        ctx.Velocity_solve("u", case.dt)
    assert e.value.code == 4
    ctx.load_state(case.state)
    st = ctx.step(case.dt)
    assert max(st["div_max"]) <= 1e-10


@pytest.mark.parametrize("name,mk", [("bump", lambda: _cases.bump_small()), ("multi", lambda: _cases.multi_small())])
def test_divergence_gate(api, oracle_mod, name, mk):
    """A strongly divergent random velocity: the relative residual 1e-10
    alone leaves max|div u| above 1e-10 after the projection; with the gate
    the solve goes on until the projected velocity meets it, and the answer
    still matches the oracle's exact solve."""
    case = mk()
    s = _cases.random_state(case, seed=11)
    dt = case.dt
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    ctx.Pressure_set_RHS(dt)
    ctx.Pressure_solve()
    ctx.Pressure_project_velocity(dt)
    ungated = ctx.Pressure_compute_velocity_divergence()
    ctx.close()
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    ctx.set_divergence_gate(1e-10)
    ctx.Pressure_set_RHS(dt)
    it, rr = ctx.Pressure_solve()
    ctx.Pressure_project_velocity(dt)
    gated = ctx.Pressure_compute_velocity_divergence()
    assert ungated > 1e-10 and ctx.divergence_gate_count() >= 1
    assert gated <= 1e-10 and rr <= case.params.p_rtol
    ctx.close()


@pytest.mark.parametrize("pmode", ["mixed", "fp64"])
def test_divergence_gate_stops_at_round_off(api, oracle_mod, pmode):
    """A gate no residual can meet (1e-30): the solve goes on down to the
    round-off floor of its residual (64 DBL_EPSILON |b|) and returns there,
    counted, instead of running into the iteration limit; the projected
    velocity is as divergence-free as the floor allows."""
    case = _cases.multi_small()
    s = _cases.random_state(case, seed=11)
    dt = case.dt
    ctx, orc, _ = _pair(case, api, oracle_mod, s)
    ctx.set_pressure_mode(api.PMODE_MIXED if pmode == "mixed" else api.PMODE_FP64)
    ctx.set_divergence_gate(1e-30)
    ctx.Pressure_set_RHS(dt)
    it, rr = ctx.Pressure_solve()
    ctx.Pressure_project_velocity(dt)
    div = ctx.Pressure_compute_velocity_divergence()
    assert ctx.divergence_gate_floor_count() == 1
    assert it < case.params.p_maxit and rr <= 64 * np.finfo(np.float64).eps
    assert div <= 1e-10
    ctx.close()


@pytest.mark.parametrize("name,mk", [("bump", lambda: _cases.bump_small()), ("multi", lambda: _cases.multi_small()),
                                     ("bump_64", lambda: _cases.bump_small(64, 40, 24))])
def test_marching_sweeps_are_bit_identical(api, oracle_mod, name, mk):
    """The kernel variants that hide latency or traffic (FP32 Jacobi and
    red-black sweeps marching along k through shared-memory plane tiles, ENO
    y / z lines walked in segments, V-cycle kernels with programmatic
    dependent launch, the coarse levels in one cluster launch, the finest
    level's sweeps two per pass on the 64x32x16 case) give the same bits as the one-point-per-thread kernels in plain
    stream order: two full steps (every convection pass and every Helmholtz
    and Poisson solve) with either."""
    case = mk()
    s = _cases.random_state(case, seed=13)
    out = []
    for variants in (0, api.KV_MARCHING | api.KV_ENO_SEGMENTS | api.KV_PDL,
                     api.KV_MARCHING | api.KV_ENO_SEGMENTS | api.KV_PDL | api.KV_CLUSTER_VCYCLE,
                     api.KV_ENO_SEGMENTS | api.KV_PDL | api.KV_SWEEP_PAIRS):
        ctx = api.Context(case.grid, case.params)
        ctx.set_sweep_kernels(variants)
        ctx.load_state(s)
        for _ in range(2):
            ctx.step(case.dt)
        out.append(ctx.state())
        ctx.close()
    for o in out[1:]:
        for k in out[0]:
            assert np.array_equal(out[0][k], o[k]), k


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("cells,tail", [(1 << 17, 4096), (1 << 20, 4096), (1 << 17, 0)])
def test_cluster_vcycle_is_bit_identical(api, mode, cells, tail):
    """The one-cluster V-cycle (every level from the first of at most `cells`
    cells in one thread-block cluster launch, phases separated by the
    cluster barrier; the single-block tail's levels in block 0 of it, or
    every level cluster-wide when the tail is off) gives the same Poisson
    iterates as a launch per half sweep, in either pressure mode, on a
    256x128x128 grid whose finest levels still run as separate launches."""
    from turbins_gb300 import workload as W
    case = W.poisson_case(256, 128, 128, (16.0, 2.0, 2.0), 1.5)
    vel = W.fourier_velocity(case.grid, 3)
    out = []
    for variants in (api.KV_ENO_SEGMENTS | api.KV_PDL, api.KV_ENO_SEGMENTS | api.KV_PDL | api.KV_CLUSTER_VCYCLE):
        ctx = api.Context(case.grid, case.params)
        ctx.set_sweep_kernels(variants)
        ctx.set_mg_cluster(cells)
        ctx.set_mg_tail(tail)
        ctx.set_pressure_mode(api.PMODE_FP64 if mode == "fp64" else api.PMODE_MIXED)
        for f, k in ((api.F_U, "u"), (api.F_V, "v"), (api.F_W, "w")):
            ctx.upload(f, vel[k])
        ctx.upload(api.F_PHI, np.zeros(case.grid.shape))
        ctx.Pressure_set_RHS(1.0)
        it, rr = ctx.Pressure_solve()
        out.append((it, rr, ctx.download(api.F_PHI)))
        ctx.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("shape,lengths,q", [((256, 128, 128), (16.0, 2.0, 2.0), 1.5),
                                             ((128, 64, 64), (1.0, 1.0, 1.0), None),
                                             ((64, 64, 40), (4.0, 2.0, 2.0), 1.5)])
def test_sweep_pairs_are_bit_identical(api, shape, lengths, q):
    """The finest FP32 level's two-sweeps-per-pass smoother (TMA-staged z
    planes, a wavefront of four half sweeps over overlapped tiles, ping-pong
    x) gives the same Poisson iterates, residual and pressure as four launches
    of one half sweep each: on a y-stretched 256x128x128 grid (blocks whose
    plane ranges cross tiles), a uniform 128x64x64 grid, and a 64x64x40 grid
    (a few planes per block, two tile rows)."""
    from turbins_gb300 import workload as W
    case = W.poisson_case(*shape, lengths, q)
    vel = W.fourier_velocity(case.grid, 5)
    out = []
    for variants in (api.KV_ENO_SEGMENTS | api.KV_PDL, api.KV_ENO_SEGMENTS | api.KV_PDL | api.KV_SWEEP_PAIRS):
        ctx = api.Context(case.grid, case.params)
        ctx.set_sweep_kernels(variants)
        ctx.set_pressure_mode(api.PMODE_MIXED)
        for f, k in ((api.F_U, "u"), (api.F_V, "v"), (api.F_W, "w")):
            ctx.upload(f, vel[k])
        rec = []
        ctx.upload(api.F_PHI, np.zeros(case.grid.shape))
        for rhs_dt in (1.0, 0.5):   # a cold start (zero guess), then a warm one
            ctx.Pressure_set_RHS(rhs_dt)
            it, rr = ctx.Pressure_solve()
            rec.append((it, rr, ctx.download(api.F_PHI)))
        out.append(rec)
        ctx.close()
    for a, b in zip(out[0], out[1]):
        assert a[0] == b[0] and a[1] == b[1]
        assert np.array_equal(a[2], b[2])
