"""Open boundaries (inflow / convective outflow) on the GPU against the
reference's own routines with params->inflow and params->outflow on
(tests/golden/open/open_bump.npz, made by tests/golden/make_golden.py):
Inflow.c, Outflow.c and the open-face branches of the step routines.
Element-wise results are compared bit for bit; the influx and the mass
correction (block-ordered sums on the device, serial in the reference) to
1e-13 relative; operators to 1e-14."""
import json
import os

import numpy as np
import pytest

from tests.test_oracle_golden import load

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "open", "open_bump.npz")


@pytest.fixture(scope="module")
def api():
    from turbins_gb300 import api as A
    from turbins_gb300 import build
    build.build()
    return A


@pytest.fixture(scope="module")
def fx():
    z, g, p, dt = load(FIX)
    p.buoyancy = 0   # the fixture holds the shipped RHS (c_term times 0.0)
    meta = json.loads(str(z["meta"]))
    return z, g, p, dt, meta["open"]


def ctx_of(api, fx):
    z, g, p, dt, op = fx
    ctx = api.Context(g, p)
    keys = ["u", "v", "w", "phi", "dpx", "dpy", "dpz", "c0"]
    ctx.load_state({k: z["in_" + k] for k in keys})
    ctx.set_open_boundaries(1, 1, U=op["U"], transient=op["transient"], time_c=op["time_c"])
    ctx.set_open_plane("in", "u", 0, z["pl_in_u"])
    ctx.set_open_plane("in", "c", 0, z["pl_in_c"])
    for q in "uvwc":
        ctx.set_open_plane("out", q, 0, z["pl_out_" + q])
        ctx.set_open_plane("out_old", q, 0, z["pl_old_" + q])
    return ctx


def same(a, b):
    return np.array_equal(a, b)


def test_inflow_profiles(api, fx):
    z = fx[0]
    ctx = ctx_of(api, fx)
    f = ctx.Inflow_u_velocity_profile(0.3)
    ctx.Inflow_conc_profile(0, 0.3)
    assert abs(f - z["ref_influx"][0]) <= 1e-13 * abs(z["ref_influx"][0])
    assert same(ctx.open_plane("in", "u"), z["ref_inflow_u"])
    assert same(ctx.open_plane("in", "c"), z["ref_inflow_c"])
    ctx.close()


def test_convective_outflow_and_mass_correction(api, fx):
    z, g, p, dt, op = fx
    ctx = ctx_of(api, fx)
    ctx.set_influx(0.75)
    for q in "uvw":
        ctx.Outflow_vel_impose_convective_boundary(q, dt)
    ctx.Outflow_conc_impose_convective_boundary(0, dt)
    for q in "vwc":
        assert same(ctx.open_plane("out", q), z["ref_outflow_" + q]), q
    # u carries the mass correction: a block-ordered sum on the device
    assert np.abs(ctx.open_plane("out", "u") - z["ref_outflow_u"]).max() <= 1e-13 * np.abs(z["ref_outflow_u"]).max()
    ctx.close()


def test_rk_average_and_plane_copies(api, fx):
    z = fx[0]
    ctx = ctx_of(api, fx)
    ctx.rk_average_outflow(0.5, 0.5)
    for q in "uvwc":
        assert same(ctx.open_plane("out", q), z["ref_rkavg_" + q]), q
    ctx.close()
    ctx = ctx_of(api, fx)
    ctx.Outflow_copy_data_into_last_plane("u", 0, True)
    ctx.Outflow_copy_data_into_last_plane("c", 0, False)
    assert same(ctx.download(api.F_U), z["ref_toplane_u"])
    assert same(ctx.download(api.F_C0), z["ref_toplane_c"])
    ctx.Outflow_copy_data_into_2D_array("w", 0)
    assert same(ctx.open_plane("out", "w"), z["ref_fromplane_w"])
    ctx.close()


def test_step_routines_with_open_faces(api, fx):
    z, g, p, dt, op = fx
    ctx = ctx_of(api, fx)
    ctx.Velocity_cell_center()
    for f, k in ((api.F_UBC, "ubc"), (api.F_VBC, "vbc"), (api.F_WBC, "wbc")):
        assert same(ctx.download(f), z["ref_" + k]), k
    for q in "uvw":
        ctx.Velocity_transpose_velocities(q)
        ok = np.asarray(g.status[q]) != 7   # transposes are defined off the BOUNDARY nodes
        assert same(ctx.download(api.F_SCRATCH0)[ok], z["ref_T%sA" % q][ok]), q
        assert same(ctx.download(api.F_SCRATCH1)[ok], z["ref_T%sB" % q][ok]), q
    for q, f in (("u", api.F_CONV_U), ("v", api.F_CONV_V), ("w", api.F_CONV_W)):
        ctx.Velocity_convective_terms(q)
        assert same(ctx.download(f), z["ref_conv_" + q]), q
    ctx.Conc_convective_terms(0)
    assert same(ctx.download(api.F_CCONV0), z["ref_conv_c0"])
    for q, fc, fb in (("u", api.F_CONV_U, api.F_B_U), ("v", api.F_CONV_V, api.F_B_V),
                      ("w", api.F_CONV_W, api.F_B_W)):
        ctx.upload(fc, z["ref_conv_" + q])
        ctx.Velocity_set_RHS(q, dt)
        assert same(ctx.download(fb), z["ref_rhs_" + q]), q
    ctx.upload(api.F_CCONV0, z["ref_conv_c0"])
    ctx.Conc_set_RHS(0, dt)
    assert same(ctx.download(api.F_CB0), z["ref_rhs_c0"])
    for q, ic in (("u", 0), ("v", 0), ("w", 0), ("c", 0)):
        ctx.helmholtz_apply(q, ic, dt, api.F_PHI, api.F_SCRATCH0)
        y = ctx.download(api.F_SCRATCH0)
        ref = z["ref_lhs_" + (q if q != "c" else "c0")]
        assert np.abs(y - ref).max() <= 1e-14 * np.abs(ref).max(), q
    ctx.Pressure_set_RHS(dt)
    assert same(ctx.download(api.F_PB), z["ref_pb"])
    dm = ctx.Pressure_compute_velocity_divergence()
    assert dm == z["ref_divmax"][0]
    assert same(ctx.download(api.F_DIV), z["ref_div"])
    d = ctx.diagnostics()
    assert abs(d["viscous_dissipation"] - z["ref_visc"][0]) <= 1e-12 * abs(z["ref_visc"][0])
    ctx.close()


def test_steps_with_open_faces_match_reference_trace(api, fx):
    """Two GPU steps with both faces open against two steps composed of the
    reference's routines in the same order (tests/golden/make_golden.py),
    solvers at relative residual 1e-12."""
    z, g, p, dt, op = fx
    p.buoyancy = 1
    p.p_rtol = 1e-12
    p.vel_rtol = 1e-12
    try:
        ctx = ctx_of(api, fx)
        zero = np.zeros((g.nz + 1, g.ny + 1))
        ctx.set_open_plane("in", "u", 0, zero)
        ctx.set_open_plane("in", "c", 0, zero)
        for q in "uvwc":
            ctx.set_open_plane("out", q, 0, zero)
            ctx.set_open_plane("out_old", q, 0, zero)
        ctx.set_time(0.3)
        for _ in range(2):
            st = ctx.step(dt)
            assert max(st["div_max"]) <= 1e-10
        s = ctx.state()
    finally:
        p.buoyancy = 0
    vscale = max(np.abs(z["ref_step2_" + k]).max() for k in "uvw")
    for k in ("u", "v", "w"):
        assert np.abs(s[k] - z["ref_step2_" + k]).max() <= 1e-7 * vscale, k
    assert np.abs(s["c0"] - z["ref_step2_c0"]).max() <= 1e-6
    for q in "uvw":
        assert np.abs(ctx.open_plane("out", q) - z["ref_step2_out_" + q]).max() <= 1e-7 * vscale, q
    assert np.abs(ctx.open_plane("out", "c") - z["ref_step2_out_c"]).max() <= 1e-6
    assert abs(ctx.time() - (0.3 + 2 * dt)) <= 1e-15
    ctx.close()
