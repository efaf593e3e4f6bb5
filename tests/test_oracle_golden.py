"""Pins the CPU oracle against the reference: golden fixtures made by the
reference's own routines (tests/golden/make_golden.py) must be reproduced bit
for bit by the oracle (matrix-vector products: to 1e-14, the reference sums
in assembled-column order)."""
import glob
import json
import os

import numpy as np
import pytest

from turbins_gb300 import workload as W

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def load(path):
    z = np.load(path, allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    nx, ny, nz = meta["nx"], meta["ny"], meta["nz"]
    g = W.Grid(nx, ny, nz, *[z["grid_" + k] for k in ("xc", "yc", "zc", "xu", "yv", "zw")])
    for q in "uvwc":
        g.status[q] = z["status_" + q]
        ib = {k: z["ib_%s_%s" % (q, k)] for k in ("im", "nf", "fidx", "fcoef", "bcoef")}
        ib["n"] = int(len(ib["im"]))
        g.ib[q] = ib
    p = W.Params(**meta["params"])
    return z, g, p, meta["dt"]


@pytest.fixture(scope="module", params=FIX, ids=[os.path.basename(f)[:-4] for f in FIX])
def fixture(request, oracle_mod):
    z, g, p, dt = load(request.param)
    return z, g, p, dt, oracle_mod.Oracle(g, p)


def test_fixtures_present():
    assert len(FIX) >= 4


def test_metrics(fixture):
    z, g, p, dt, o = fixture
    for k in ("mxc", "myc", "mzc", "mxu", "myv", "mzw"):
        assert np.array_equal(o.metrics[k], z["ref_" + k]), k


def test_eno_lines(fixture):
    z, g, p, dt, o = fixture
    for order in (1, 2, 3):
        got = o.eno_line(order, z["eno%d_D0" % order], z["eno%d_P" % order], z["eno%d_V" % order])
        ref = z["ref_eno%d" % order]
        n = len(ref)
        assert np.array_equal(got[order:n - order], ref[order:n - order])


def test_interpolations(fixture):
    z, g, p, dt, o = fixture
    u, v, w = z["in_u"], z["in_v"], z["in_w"]
    ub, vb, wb = o.cell_center(u, v, w)
    assert np.array_equal(ub, z["ref_ubc"]) and np.array_equal(vb, z["ref_vbc"]) and np.array_equal(wb, z["ref_wbc"])
    for q in "uvw":
        A, B = o.transpose(q, u, v, w)
        nb = g.status[q] != W.BOUNDARY
        assert np.array_equal(A[nb], z["ref_T%sA" % q][nb])
        assert np.array_equal(B[nb], z["ref_T%sB" % q][nb])


def test_convection(fixture):
    """restated line driver + ghost rules == reference ghost routines + ENO"""
    z, g, p, dt, o = fixture
    u, v, w = z["in_u"], z["in_v"], z["in_w"]
    vel = {"u": (u, z["ref_TuA"], z["ref_TuB"]), "v": (z["ref_TvA"], v, z["ref_TvB"]),
           "w": (z["ref_TwA"], z["ref_TwB"], w)}
    for q in "uvw":
        assert np.array_equal(o.convection_vel(q, z["in_" + q], *vel[q]), z["ref_conv_" + q]), q
    for ic in range(p.nconc):
        vb = z["ref_vbc"]
        va = vb + p.vs0[ic] if p.ctype[ic] == W.PARTICLE else vb
        got = o.convection_conc(ic, z["in_c%d" % ic], z["ref_ubc"], va, z["ref_wbc"])
        assert np.array_equal(got, z["ref_conv_c%d" % ic])


def test_rhs(fixture):
    z, g, p, dt, o = fixture
    p.buoyancy = 0   # the shipped Velocity_v_set_RHS multiplies c_term by 0.0
    o0 = type(o)(g, p)
    if p.nconc > 1:
        assert np.array_equal(o.total_concentration([z["in_c%d" % i] for i in range(p.nconc)]), z["ref_ctot"])
    for q, dk in (("u", "dpx"), ("v", "dpy"), ("w", "dpz")):
        got = o0.set_rhs_vel(q, dt, z["in_" + q], z["ref_conv_" + q], z["in_" + dk], z["ref_ctot"])
        assert np.array_equal(got, z["ref_rhs_" + q]), q
    for ic in range(p.nconc):
        got = o.set_rhs_conc(dt, z["in_c%d" % ic], z["ref_conv_c%d" % ic])
        assert np.array_equal(got, z["ref_rhs_c%d" % ic])
    p.buoyancy = 1


def test_buoyancy_term(fixture):
    """with buoyancy on, v's RHS differs from the shipped one by exactly -c_term
    (2-point interpolation of the total concentration to the v node)."""
    z, g, p, dt, o = fixture
    got = o.set_rhs_vel("v", dt, z["in_v"], z["ref_conv_v"], z["in_dpy"], z["ref_ctot"])
    ct = z["ref_ctot"]
    yc, yv = g.yc, g.yv
    m = (g.status["v"] == W.FLUID) | (g.status["v"] == W.BUFFER_SOLID)
    c0 = ct[:, :-1, :]
    c1 = ct[:, 1:, :]
    slope = (c1 - c0) / (yc[1:] - yc[:-1])[None, :, None]
    cterm = np.zeros_like(ct)
    cterm[:, 1:, :] = slope * (yv[1:] - yc[:-1])[None, :, None] + c0
    assert np.array_equal(got[m], (z["ref_rhs_v"] - cterm)[m])


def test_operators(fixture):
    z, g, p, dt, o = fixture
    x = z["in_phi"]
    for q in "uvw":
        a, b = o.helmholtz_apply(q, 0, dt, x), z["ref_lhs_" + q]
        assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max(), q
    for ic in range(p.nconc):
        a, b = o.helmholtz_apply("c", ic, dt, x), z["ref_lhs_c%d" % ic]
        assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max()
    a, b = o.pressure_apply(x), z["ref_plhs"]
    assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max()


def test_pressure_rhs_projection_divergence(fixture):
    z, g, p, dt, o = fixture
    pb = o.pressure_rhs(dt, z["in_u"], z["in_v"], z["in_w"])
    assert np.array_equal(pb, z["ref_pb"])
    arrs = [z["in_" + k].copy() for k in ("u", "v", "w", "dpx", "dpy", "dpz")]
    o.project(dt, z["in_phi"], pb, *arrs)
    for k, a in zip(("u", "v", "w", "dpx", "dpy", "dpz"), arrs):
        assert np.array_equal(a, z["ref_proj_" + k]), k
    mx, dv = o.divergence(*arrs[:3])
    assert mx == z["ref_divmax"][0]
    assert np.array_equal(dv, z["ref_div"])


def test_diagnostics(fixture):
    """to_diagnostics reproduces Extract.c / Conc.c's flow integrals, the
    spanwise-averaged heights, the front location, the bed sedimentation
    rates and, with to_deposit_integrate, the deposited heights bit for bit."""
    z, g, p, dt, o = fixture
    nc = p.nconc
    cs = [z["in_c%d" % i] for i in range(nc)]
    assert np.array_equal(o.interface_y_index(), z["ref_iy"])
    cold = [z["in_cold%d" % i] for i in range(nc)]
    dep = o.deposit_integrate(cs, cold, dt, z["in_dep0"].copy())
    assert np.array_equal(dep, z["ref_dep"])
    d = o.diagnostics(z["in_u"], z["in_v"], z["in_w"], cs, float(z["diag_front_limit"][0]), dep=dep)
    got = np.array([d["kinetic_energy"], d["conversion_rate"]] + d["suspended_mass"] + d["potential_energy"] +
                   d["stokes_dissipation"] + d["conversion_rate_c"] + [d["front_location"], d["viscous_dissipation"]] +
                   d["ep_passive"] + d["ep_passive_rate"] + d["ep_rate"] + d["sed_rate"])
    assert np.array_equal(got, z["ref_diag"])
    assert np.array_equal(d["ave_height"], z["ref_ave_height"])
    assert np.array_equal(d["sed_bottom"], z["ref_sed_bottom"])
    assert d["front_location"] > 0.0


def test_step_trace(fixture):
    """Two TVD-RK2 steps of the oracle against two steps composed of the
    reference's own routines (its RHS, LHS assembly, projection, divergence,
    ghost and ENO routines; its BiCGStab set-up for the Helmholtz solves and
    an exact pressure solve), both to relative residual 1e-12: fields agree to
    the solvers' tolerance, measured against the velocity scale."""
    z, g, p, dt, o = fixture
    p.p_rtol = 1e-12
    p.vel_rtol = 1e-12
    o2 = type(o)(g, p)
    keys = ["u", "v", "w", "phi", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(p.nconc)]
    s = {k: z["in_" + k].copy() for k in keys}
    for _ in range(2):
        o2.step(s, dt)
    vscale = max(np.abs(z["ref_step2_" + k]).max() for k in "uvw")
    for k in ("u", "v", "w"):
        assert np.abs(s[k] - z["ref_step2_" + k]).max() <= 1e-7 * vscale, k
    for i in range(p.nconc):
        ref = z["ref_step2_c%d" % i]
        assert np.abs(s["c%d" % i] - ref).max() <= 1e-9 * max(np.abs(ref).max(), 1.0)
    m = np.zeros(g.shape, bool)
    m[:-1, :-1, :-1] = True
    a = s["phi"][m] - s["phi"][m].mean()
    b = z["ref_step2_phi"][m] - z["ref_step2_phi"][m].mean()
    assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
