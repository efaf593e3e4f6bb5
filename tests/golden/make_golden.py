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


if __name__ == "__main__":
    for nm, mk in CASES.items():
        dump(nm, mk())
        print("wrote", nm)
    dump_resume()
    print("wrote resume_bump")
