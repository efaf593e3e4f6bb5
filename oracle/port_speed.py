"""Speed of the oracle port against the reference's own compiled routines
(TEST INFRASTRUCTURE ONLY; needs oracle/_ref, i.e. the reference checkout).

The CPU arm of bench.py times the oracle port, since the reference's own C
cannot be built on the GPU machine.  This script times the element-wise routines
both implement in plain single-threaded C -- Velocity_cell_center,
Velocity_transpose_velocities, Velocity_u_set_RHS, Pressure_set_RHS,
Pressure_project_velocity, Pressure_compute_velocity_divergence -- on one
seeded state of the multi-bump workload, so that the port can be shown not
to be slower than the code it stands for.  The reference's times include
its harness's copies of the fields into and out of its vectors.

  python -m oracle.port_speed [NX NY NZ]
"""
from __future__ import annotations

import sys
import time

import numpy as np


def _time(f, n=5):
    f()
    t = time.perf_counter()
    for _ in range(n):
        f()
    return (time.perf_counter() - t) / n * 1e3


def main(nx=128, ny=64, nz=64):
    from turbins_gb300 import workload as W
    from oracle import oracle as O
    from oracle import refcheck as R
    O.build()
    if not R.available():
        raise SystemExit("oracle/_ref not built (it needs the reference checkout)")
    case = W.multi_bump_case(nx, ny, nz)
    rng = np.random.default_rng(5)
    s = {k: v + 1e-3 * rng.standard_normal(v.shape) for k, v in case.state.items()}
    orc, ref = O.Oracle(case.grid, case.params), R.Reference(case.grid, case.params)
    dt = case.dt
    u, v, w, ct = s["u"], s["v"], s["w"], s["c0"]
    conv = 0.1 * u + 0.01

    def project(o):
        st = [a.copy() for a in (u, v, w, s["dpx"], s["dpy"], s["dpz"])]
        return lambda: o.project(dt, s["phi"], s["phi"], *st)

    rows = [
        ("Velocity_cell_center", lambda o: (lambda: o.cell_center(u, v, w))),
        ("Velocity_transpose_velocities (v)", lambda o: (lambda: o.transpose("v", u, v, w))),
        ("Velocity_u_set_RHS", lambda o: (lambda: o.set_rhs_vel("u", dt, u, conv, s["dpx"], ct))),
        ("Pressure_set_RHS", lambda o: (lambda: o.pressure_rhs(dt, u, v, w))),
        ("Pressure_project_velocity", project),
        ("Pressure_compute_velocity_divergence", lambda o: (lambda: o.divergence(u, v, w))),
    ]
    print("%dx%dx%d, one core; ms per call" % (nx, ny, nz))
    print("%-38s %9s %9s %7s" % ("routine", "port", "reference", "ratio"))
    for name, mk in rows:
        a, b = _time(mk(orc)), _time(mk(ref))
        print("%-38s %9.2f %9.2f %7.2f" % (name, a, b, a / b))
    # ENO_compute_convective_terms on one 256-node line (ENO-3), both called
    # through the same kind of ctypes wrapper, so the call overhead is alike
    P = np.cumsum(rng.uniform(0.5, 1.5, 262))
    D0, V = rng.standard_normal(262), rng.standard_normal(262)
    a = _time(lambda: [orc.eno_line(3, D0, P, V) for _ in range(1000)], 3)
    b = _time(lambda: [ref.eno_line(3, D0, P, V) for _ in range(1000)], 3)
    print("%-38s %9.4f %9.4f %7.2f" % ("ENO_compute_convective_terms (line)", a / 1000, b / 1000, a / b))


if __name__ == "__main__":
    main(*[int(x) for x in sys.argv[1:4]])
