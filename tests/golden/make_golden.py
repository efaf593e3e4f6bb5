"""Regenerates the golden fixtures of tests/golden from the reference's own
routines (oracle/_ref, compiled from the reference checkout through the PETSc
shim).  Run in a checkout that has the reference sources:

    python tests/golden/make_golden.py

Each fixture holds a small seeded case (grid, status, immersed stencils,
parameters, state) and the reference's outputs for it.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.refcheck import Reference  # noqa: E402
from tests import _cases  # noqa: E402
from turbins_gb300.geometry import bed_heights  # noqa: E402

CASES = {
    "lock_eno2": lambda: _cases.lock_small(12, 8, 8, order=2),
    "lock_eno3": lambda: _cases.lock_small(12, 8, 8, order=3),
    "bump_eno3": lambda: _cases.bump_small(24, 12, 8),
    "multi_eno3": lambda: _cases.multi_small(24, 16, 8),
}


def dump(name, case):
    g, p = case.grid, case.params
    s = _cases.random_state(case, seed=21)
    ref = Reference(g, p)
    out = {}
    for k in ("xc", "yc", "zc", "xu", "yv", "zw"):
        out["grid_" + k] = getattr(g, k)
    for q in "uvwc":
        out["status_" + q] = g.status[q]
        for k in ("im", "nf", "fidx", "fcoef", "bcoef"):
            out["ib_%s_%s" % (q, k)] = np.asarray(g.ib[q][k])
    for k, v in s.items():
        out["in_" + k] = v
    m = ref.metrics()
    for k, v in m.items():
        out["ref_" + k] = v
    ub, vb, wb = ref.cell_center(s["u"], s["v"], s["w"])
    out["ref_ubc"], out["ref_vbc"], out["ref_wbc"] = ub, vb, wb
    vel = {}
    for q in "uvw":
        A, B = ref.transpose(q, s["u"], s["v"], s["w"])
        out["ref_T%sA" % q], out["ref_T%sB" % q] = A, B
        vel[q] = (s["u"], A, B) if q == "u" else (A, s["v"], B) if q == "v" else (A, B, s["w"])
        out["ref_conv_" + q] = ref.convection(q, 0, s[q], *vel[q])
    for ic in range(p.nconc):
        va = vb + p.vs0[ic] if p.ctype[ic] == 2 else vb
        out["ref_conv_c%d" % ic] = ref.convection("c", ic, s["c%d" % ic], ub, va, wb)
    dt = case.dt
    ct = s["c0"] if p.nconc == 1 else ref.total_concentration([s["c%d" % i] for i in range(p.nconc)])
    out["ref_ctot"] = ct
    for q, dk in (("u", "dpx"), ("v", "dpy"), ("w", "dpz")):
        out["ref_rhs_" + q] = ref.set_rhs_vel(q, dt, s[q], out["ref_conv_" + q], s[dk], ct)
    for ic in range(p.nconc):
        out["ref_rhs_c%d" % ic] = ref.set_rhs_conc(ic, dt, s["c%d" % ic], out["ref_conv_c%d" % ic])
    x = s["phi"]
    for q in "uvw":
        out["ref_lhs_" + q] = ref.lhs_apply(q, 0, dt, x)
    for ic in range(p.nconc):
        out["ref_lhs_c%d" % ic] = ref.lhs_apply("c", ic, dt, x)
    out["ref_plhs"] = ref.pressure_apply(x)
    pb = ref.pressure_rhs(dt, s["u"], s["v"], s["w"])
    out["ref_pb"] = pb
    arrs = [s[k].copy() for k in ("u", "v", "w", "dpx", "dpy", "dpz")]
    ref.project(dt, s["phi"], pb, *arrs)
    for k, a in zip(("u", "v", "w", "dpx", "dpy", "dpz"), arrs):
        out["ref_proj_" + k] = a
    mx, dv = ref.divergence(*arrs[:3])
    out["ref_divmax"] = np.array([mx])
    out["ref_div"] = dv
    # flow diagnostics; the front limit is set between two heights of the
    # alpha-weighted h(x) profile so that the fixture holds a front crossing
    cs = [s["c%d" % i] for i in range(p.nconc)]
    h = ref.diagnostics(s["u"], s["v"], s["w"], cs, 0.05)["ave_height"]
    hw = sum(h[i] * p.alpha[i] for i in range(p.nconc))
    limit = 0.05
    for i in range(g.nx - 1, 0, -1):
        if hw[i - 1] > hw[i]:
            limit = 0.5 * (hw[i - 1] + hw[i])
            break
    # bed index, one deposit integration from a perturbed start-of-step state
    out["ref_iy"] = ref.interface_y_index()
    rng = np.random.Generator(np.random.PCG64(8))
    cold = [c + 0.01 * rng.standard_normal(c.shape) for c in cs]
    dep0 = rng.uniform(0.0, 0.01, (p.nconc, g.nz + 1, g.nx + 1))
    for i in range(p.nconc):
        out["in_cold%d" % i] = cold[i]
    out["in_dep0"] = dep0
    dep = ref.deposit_integrate(cs, cold, dt, dep0.copy())
    out["ref_dep"] = dep
    d = ref.diagnostics(s["u"], s["v"], s["w"], cs, limit, dep=dep)
    out["diag_front_limit"] = np.array([limit])
    out["ref_diag"] = np.array([d["kinetic_energy"], d["conversion_rate"]] + d["suspended_mass"] +
                               d["potential_energy"] + d["stokes_dissipation"] + d["conversion_rate_c"] +
                               [d["front_location"], d["viscous_dissipation"]] + d["ep_passive"] +
                               d["ep_passive_rate"] + d["ep_rate"] + d["sed_rate"])
    out["ref_ave_height"] = d["ave_height"]
    out["ref_sed_bottom"] = d["sed_bottom"]
    # two full TVD-RK2 steps through the reference's own routines (linear
    # solves: the reference's KSP set-up, resmax 1e-12; the pressure system
    # solved exactly by the harness)
    st = {k: s[k].copy() for k in ["u", "v", "w", "phi", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(p.nconc)]}
    for _ in range(2):
        ref.step(st, dt)
    for k in ["u", "v", "w", "phi", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(p.nconc)]:
        out["ref_step2_" + k] = st[k]
    # ENO lines with ties and zero velocities
    rng = np.random.Generator(np.random.PCG64(5))
    for order in (1, 2, 3):
        n = 41
        P = np.cumsum(rng.uniform(0.5, 1.5, n))
        D0 = rng.standard_normal(n)
        D0[10:16] = 0.5
        V = rng.standard_normal(n)
        V[::5] = 0.0
        out["eno%d_D0" % order], out["eno%d_P" % order], out["eno%d_V" % order] = D0, P, V
        out["ref_eno%d" % order] = ref.eno_line(order, D0, P, V)
    meta = dict(name=name, nx=g.nx, ny=g.ny, nz=g.nz, dt=dt, params=p.__dict__)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(json.dumps(meta)), **out)


# restart set written by the reference's Resume.c (through the harness) for
# the 16x8x8 bump case: the files themselves are the fixture
RESUME_CASE = dict(nx=16, ny=8, nz=8, seed=31)
RESUME_PRIM = dict(time=0.1234567891, dt=2.5e-4, dt_old=2.4e-4, iter=17, output_iter=3)


def resume_case():
    c = RESUME_CASE
    return _cases.bump_small(c["nx"], c["ny"], c["nz"])


def dump_resume():
    case = resume_case()
    g, p = case.grid, case.params
    s = _cases.random_state(case, seed=RESUME_CASE["seed"])
    dep = np.random.Generator(np.random.PCG64(2)).uniform(0.0, 0.01, (p.nconc, g.nz + 1, g.nx + 1))
    d = os.path.join(HERE, "resume_bump")
    os.makedirs(d, exist_ok=True)
    Reference(g, p).resume_write(d, s, RESUME_PRIM, grid=True, dep=dep)
    with open(os.path.join(d, "case.json"), "w") as f:
        json.dump(dict(case=RESUME_CASE, prim=RESUME_PRIM), f)


# open boundaries: the 24x12x8 bump case with inflow and convective outflow,
# every open-face routine through the reference's own code
OPEN_ARGS = dict(U=0.8, transient=1, time_c=0.5)


def dump_open():
    case = _cases.bump_small(24, 12, 8)
    g, p = case.grid, case.params
    s = _cases.random_state(case, seed=23)
    ref = Reference(g, p)
    ref.set_open(1, 1, **OPEN_ARGS)
    rng = np.random.Generator(np.random.PCG64(9))
    shp = (g.nz + 1, g.ny + 1)
    out = {}
    for k in ("xc", "yc", "zc", "xu", "yv", "zw"):
        out["grid_" + k] = getattr(g, k)
    for q in "uvwc":
        out["status_" + q] = g.status[q]
        for k in ("im", "nf", "fidx", "fcoef", "bcoef"):
            out["ib_%s_%s" % (q, k)] = np.asarray(g.ib[q][k])
    for k, v in s.items():
        out["in_" + k] = v
    planes = {"in_u": rng.uniform(0.0, 1.0, shp), "in_c": rng.uniform(0.0, 1.0, shp)}
    for q in "uvwc":
        planes["out_" + q] = rng.uniform(-0.5, 0.5, shp)
        planes["old_" + q] = rng.uniform(-0.5, 0.5, shp)
    for k, v in planes.items():
        out["pl_" + k] = v

    def load_planes():
        ref.open_set("in", "u", 0, planes["in_u"])
        ref.open_set("in", "c", 0, planes["in_c"])
        for q in "uvwc":
            ref.open_set("out", q, 0, planes["out_" + q])
            ref.open_set("out_old", q, 0, planes["old_" + q])

    dt = case.dt
    # inflow profiles
    load_planes()
    out["ref_influx"] = np.array([ref.inflow_u(0.3)])
    ref.inflow_c(0, 0.3)
    out["ref_inflow_u"] = ref.open_get("in", "u")
    out["ref_inflow_c"] = ref.open_get("in", "c")
    # convective outflow (u with the mass correction from influx 0.75)
    load_planes()
    for q in "uvw":
        ref.outflow_impose(q, 0, dt, s[q], influx=0.75)
        out["ref_outflow_" + q] = ref.open_get("out", q)
    ref.outflow_impose("c", 0, dt, s["c0"])
    out["ref_outflow_c"] = ref.open_get("out", "c")
    # rk average of the outflow planes, plane copies
    load_planes()
    for q in "uvwc":
        ref.outflow_rk_average(q, 0, 0.5, 0.5)
        out["ref_rkavg_" + q] = ref.open_get("out", q)
    load_planes()
    out["ref_toplane_u"] = ref.outflow_to_plane("u", 0, 1, s["u"])
    out["ref_toplane_c"] = ref.outflow_to_plane("c", 0, 0, s["c0"])
    ref.outflow_from_plane("w", 0, s["w"])
    out["ref_fromplane_w"] = ref.open_get("out", "w")
    # the step routines with both faces open
    load_planes()
    ub, vb, wb = ref.cell_center(s["u"], s["v"], s["w"])
    out["ref_ubc"], out["ref_vbc"], out["ref_wbc"] = ub, vb, wb
    vel = {}
    for q in "uvw":
        A, B = ref.transpose(q, s["u"], s["v"], s["w"])
        out["ref_T%sA" % q], out["ref_T%sB" % q] = A, B
        vel[q] = (s["u"], A, B) if q == "u" else (A, s["v"], B) if q == "v" else (A, B, s["w"])
        out["ref_conv_" + q] = ref.convection(q, 0, s[q], *vel[q])
    va = vb + p.vs0[0] if p.ctype[0] == 2 else vb
    out["ref_conv_c0"] = ref.convection("c", 0, s["c0"], ub, va, wb)
    for q, dk in (("u", "dpx"), ("v", "dpy"), ("w", "dpz")):
        out["ref_rhs_" + q] = ref.set_rhs_vel(q, dt, s[q], out["ref_conv_" + q], s[dk], s["c0"])
    out["ref_rhs_c0"] = ref.set_rhs_conc(0, dt, s["c0"], out["ref_conv_c0"])
    x = s["phi"]
    for q in "uvw":
        out["ref_lhs_" + q] = ref.lhs_apply(q, 0, dt, x)
    out["ref_lhs_c0"] = ref.lhs_apply("c", 0, dt, x)
    out["ref_pb"] = ref.pressure_rhs(dt, s["u"], s["v"], s["w"])
    mx, dv = ref.divergence(s["u"], s["v"], s["w"])
    out["ref_divmax"] = np.array([mx])
    out["ref_div"] = dv
    d = ref.diagnostics(s["u"], s["v"], s["w"], [s["c0"]], 0.01)
    out["ref_visc"] = np.array([d["viscous_dissipation"]])
    # two steps with both faces open, from time 0.3 (the restated driver's
    # order: inflow planes, outflow stored, imposed per stage, RK-averaged),
    # the planes starting at zero as the reference allocates them
    for q in "uvwc":
        ref.open_set("out", q, 0, np.zeros(shp))
        ref.open_set("out_old", q, 0, np.zeros(shp))
    ref.open_set("in", "u", 0, np.zeros(shp))
    ref.open_set("in", "c", 0, np.zeros(shp))
    st = {k: s[k].copy() for k in ["u", "v", "w", "phi", "dpx", "dpy", "dpz", "c0"]}
    for n in range(2):
        ref.step(st, dt, time=0.3 + n * dt)
    for k in ["u", "v", "w", "phi", "dpx", "dpy", "dpz", "c0"]:
        out["ref_step2_" + k] = st[k]
    for q in "uvwc":
        out["ref_step2_out_" + q] = ref.open_get("out", q)
    meta = dict(name="open_bump", nx=g.nx, ny=g.ny, nz=g.nz, dt=dt, params=p.__dict__, open=OPEN_ARGS)
    np.savez_compressed(os.path.join(HERE, "open", "open_bump.npz"), meta=np.array(json.dumps(meta)), **out)


# immersed-boundary geometry: the reference's surface set-up (level-set
# reinitialisation of yc - h, q-sdf, node tagging) from the bed heights, and
# the ghost-cell stencils it builds on them
GEOM_CASES = {
    "bump": lambda: _cases.bump_small(24, 12, 8),
    "multi": lambda: _cases.multi_small(40, 20, 12),
}


def dump_geom(name, case):
    g = case.grid
    ipos = bed_heights(g, case.bed)
    ref = Reference(g, case.params)
    sdf, st = ref.geometry(ipos)
    out = {"ipos": ipos}
    for q in "uvwc":
        ib = ref.immersed(q)
        for k in ("im", "nf", "fidx", "fcoef", "bcoef", "pts"):
            out["ref_ib_%s_%s" % (q, k)] = ib[k]
    for k in ("xc", "yc", "zc", "xu", "yv", "zw"):
        out["grid_" + k] = getattr(g, k)
    for q in "cuvw":
        out["ref_sdf_" + q] = sdf[q]
        out["ref_status_" + q] = st[q]
    meta = dict(name=name, nx=g.nx, ny=g.ny, nz=g.nz)
    np.savez_compressed(os.path.join(HERE, "geom", "geom_%s.npz" % name), meta=np.array(json.dumps(meta)), **out)


# a run whose time step changes: operators after the reference's diagonal
# updates for several dt sequences (one change above the 1e-10 threshold of
# Velocity_modify_diagonal / Conc_modify_diagonal, one below it, several in
# a row) and three steps with dt = dt0, 0.7 dt0, 1.3 dt0 through the
# reference's routines
DT_SEQS = {"up": (1.0, 0.7), "tiny": (1.0, 1.0 + 1e-14), "many": (1.0, 0.7, 1.3, 1.3, 1.0)}
DT_STEPS = (1.0, 0.7, 1.3)


def dt_case():
    return _cases.bump_small(24, 12, 8)


def dump_dt():
    case = dt_case()
    g, p = case.grid, case.params
    s = _cases.random_state(case, seed=23)
    ref = Reference(g, p)
    dt0 = case.dt
    out = {}
    x = s["phi"]
    for nm, seq in DT_SEQS.items():
        dts = [dt0 * f for f in seq]
        out["dts_" + nm] = np.array(dts)
        for q in "uvw":
            out["ref_lhs_%s_%s" % (nm, q)] = ref.lhs_apply_dts(q, 0, dts, x)
        for ic in range(p.nconc):
            out["ref_lhs_%s_c%d" % (nm, ic)] = ref.lhs_apply_dts("c", ic, dts, x)
    keys = ["u", "v", "w", "phi", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(p.nconc)]
    for k in keys:
        out["in_" + k] = s[k]
    st = {k: s[k].copy() for k in keys}
    for n, f in enumerate(DT_STEPS):
        ref.step(st, dt0 * f)
        for k in keys:
            out["ref_step%d_%s" % (n + 1, k)] = st[k].copy()
    meta = dict(dt0=dt0, steps=list(DT_STEPS))
    os.makedirs(os.path.join(HERE, "dt"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "dt", "dt_change.npz"), meta=np.array(json.dumps(meta)), **out)


if __name__ == "__main__":
    if sys.argv[1:] == ["dt"]:          # only the dt-change fixture
        dump_dt()
        print("wrote dt_change")
        sys.exit(0)
    dump_dt()
    print("wrote dt_change")
    for nm, mk in CASES.items():
        dump(nm, mk())
        print("wrote", nm)
    dump_resume()
    print("wrote resume_bump")
    os.makedirs(os.path.join(HERE, "open"), exist_ok=True)
    dump_open()
    print("wrote open_bump")
    os.makedirs(os.path.join(HERE, "geom"), exist_ok=True)
    for nm, mk in GEOM_CASES.items():
        dump_geom(nm, mk())
        print("wrote geom", nm)
