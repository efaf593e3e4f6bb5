"""A run whose time step changes.

The reference assembles each Helmholtz matrix once and moves its diagonal by
1/dt - 1/dt_old when dt changes (Velocity_modify_diagonal, Velocity.c:374-443;
Conc_modify_diagonal, Conc.c:293-354): IMMERSED rows never get the term, and
a change of 1/dt of at most 1e-10 is skipped.  The library forms its
operators matrix-free and keeps the 1/dt term of each system by the same
rule, so its operators equal the reference's accumulated diagonals to
rounding, also after a skipped change.  The fixture
tests/golden/dt/dt_change.npz holds the reference's operators after several
dt sequences and three steps with dt = dt0, 0.7 dt0, 1.3 dt0 through its own
routines (tests/golden/make_golden.py); the oracle (CPU) and the library
(GPU) must reproduce both.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "golden", "dt", "dt_change.npz")


def _case():
    from tests import _cases
    return _cases.bump_small(24, 12, 8)


def _load():
    z = np.load(PATH, allow_pickle=False)
    return z, json.loads(str(z["meta"]))


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _check_trace(s, z, n, nconc):
    vscale = max(np.abs(z["ref_step%d_%s" % (n, k)]).max() for k in "uvw")
    for k in ("u", "v", "w"):
        assert np.abs(s[k] - z["ref_step%d_%s" % (n, k)]).max() <= 1e-7 * vscale, (n, k)
    for i in range(nconc):
        ref = z["ref_step%d_c%d" % (n, i)]
        assert np.abs(s["c%d" % i] - ref).max() <= 1e-6 * max(np.abs(ref).max(), 1.0), (n, i)


def test_fixture_sequences():
    z, meta = _load()
    assert abs(1.0 / z["dts_tiny"][1] - 1.0 / z["dts_tiny"][0]) <= 1e-10     # below the skip threshold
    assert abs(1.0 / z["dts_up"][1] - 1.0 / z["dts_up"][0]) > 1.0
    assert len(z["dts_many"]) == 5


def kept_dt(dts):
    """the dt whose 1/dt the reference's diagonal holds (to rounding) after
    modify_diagonal ran for each entry of dts in turn: a change of 1/dt of at
    most 1e-10 leaves the diagonal alone"""
    kept = dts[0]
    for prev, dt in zip(dts[:-1], dts[1:]):
        if abs(1.0 / dt - 1.0 / prev) > 1e-10:
            kept = dt
    return float(kept)


def test_oracle_operators_after_dt_changes(oracle_mod):
    """oracle operator at the dt the reference's diagonal holds after each
    sequence == the reference's operator, to 1e-14 relative; for the
    sequence whose change is below the threshold that is the first dt"""
    z, meta = _load()
    case = _case()
    o = oracle_mod.Oracle(case.grid, case.params)
    x = z["in_phi"]
    assert kept_dt(z["dts_tiny"]) == z["dts_tiny"][0]
    for nm in ("up", "tiny", "many"):
        dt = kept_dt(z["dts_" + nm])
        for q in "uvw":
            assert _rel(o.helmholtz_apply(q, 0, dt, x), z["ref_lhs_%s_%s" % (nm, q)]) <= 1e-14, (nm, q)
        for ic in range(case.params.nconc):
            assert _rel(o.helmholtz_apply("c", ic, dt, x), z["ref_lhs_%s_c%d" % (nm, ic)]) <= 1e-14, (nm, ic)


def test_oracle_steps_with_changing_dt(oracle_mod):
    z, meta = _load()
    case = _case()
    p = case.params
    p.p_rtol = 1e-12
    p.vel_rtol = 1e-12
    o = oracle_mod.Oracle(case.grid, p)
    keys = ["u", "v", "w", "phi", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(p.nconc)]
    s = {k: z["in_" + k].copy() for k in keys}
    for n, f in enumerate(meta["steps"]):
        o.step(s, meta["dt0"] * f)
        _check_trace(s, z, n + 1, p.nconc)


@pytest.mark.gpu
def test_gpu_operators_after_dt_changes():
    from turbins_gb300 import api, build
    build.build()
    z, meta = _load()
    case = _case()
    nc = case.params.nconc
    systems = [(q, 0, "ref_lhs_%s_" + q) for q in "uvw"] + [("c", ic, "ref_lhs_%%s_c%d" % ic) for ic in range(nc)]
    for nm in ("up", "tiny", "many"):
        ctx = api.Context(case.grid, case.params)       # a run that sees this dt sequence
        ctx.upload(api.F_SCRATCH0, z["in_phi"])
        for dt in z["dts_" + nm]:
            for q, ic, key in systems:
                ctx.helmholtz_apply(q, ic, float(dt), api.F_SCRATCH0, api.F_SCRATCH1)
        for q, ic, key in systems:
            ctx.helmholtz_apply(q, ic, float(z["dts_" + nm][-1]), api.F_SCRATCH0, api.F_SCRATCH1)
            assert _rel(ctx.download(api.F_SCRATCH1), z[key % nm]) <= 1e-14, (nm, q, ic)
        ctx.close()
    # the skipped change: the library's diagonal keeps 1/dt0 exactly, so the
    # operator at dt0 (1 + 1e-14) equals the operator at dt0 bit for bit
    ctx = api.Context(case.grid, case.params)
    ctx.upload(api.F_SCRATCH0, z["in_phi"])
    d0, d1 = (float(t) for t in z["dts_tiny"])
    ctx.helmholtz_apply("u", 0, d0, api.F_SCRATCH0, api.F_SCRATCH1)
    y0 = ctx.download(api.F_SCRATCH1)
    ctx.helmholtz_apply("u", 0, d1, api.F_SCRATCH0, api.F_SCRATCH1)
    assert np.array_equal(ctx.download(api.F_SCRATCH1), y0)
    ctx.close()


@pytest.mark.gpu
def test_gpu_steps_with_changing_dt():
    """three GPU steps with dt = dt0, 0.7 dt0, 1.3 dt0 against the same steps
    through the reference's routines, after each step (tolerances of the
    two-step reference trace test)"""
    from turbins_gb300 import api, build
    build.build()
    z, meta = _load()
    case = _case()
    p = case.params
    p.p_rtol = 1e-12
    p.vel_rtol = 1e-12
    keys = ["u", "v", "w", "phi", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(p.nconc)]
    ctx = api.Context(case.grid, p)
    ctx.load_state({k: z["in_" + k] for k in keys})
    for n, f in enumerate(meta["steps"]):
        st = ctx.step(meta["dt0"] * f)
        assert max(st["div_max"]) <= 1e-10
        _check_trace(ctx.state(), z, n + 1, p.nconc)
    ctx.close()
