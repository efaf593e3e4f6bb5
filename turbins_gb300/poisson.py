"""Pressure-Poisson solves alone: the mixed-precision MG-CG (FP32 V-cycles
inside FP64 CG) against the plain FP64 MG-CG on seeded divergence fields.

Each right-hand side is b = -div(u)/dt (Pressure_set_RHS, Pressure.c:171-276,
dt = 1) of a random-Fourier-mode velocity (``workload.fourier_velocity``:
wave vectors 1 <= |k| <= 8, amplitude |k|^-5/3, zero mean, impermeable
walls) on a closed box with Neumann walls.  Both methods start from a zero
pressure and iterate to the same FP64 relative residual (1e-10 by default);
the solution of each is compared mean-removed over the physical cells (the
corner pin of Pressure.c:864-868 fixes only the constant).

  python -m turbins_gb300.poisson NX NY NZ [--stretch Q] [--rhs N]
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import api
from . import workload as W

SHAPES = {"cube128": ((128, 128, 128), (1.0, 1.0, 1.0), None),
          "stretched256": ((256, 128, 128), (16.0, 2.0, 2.0), 1.5)}


def _mean_removed(phi, g):
    a = phi[:g.nz, :g.ny, :g.nx]
    return a - a.mean()


def solve_set(case, seeds, rtol=1e-10, keep=False):
    """Solve the Poisson system of every seed's divergence field with both
    methods.  Returns one record per seed: iterations, final relative
    residual and device ms per solve of each method, and the largest
    difference of the mean-removed solutions relative to the FP64 one's
    largest magnitude.  keep=True adds the solutions."""
    g = case.grid
    case.params.p_rtol = rtol
    ctx = api.Context(g, case.params)
    ctx.set_pressure_guess(api.GUESS_PREVIOUS)
    zero = np.zeros(g.shape)
    modes = (("fp64", api.PMODE_FP64), ("mixed", api.PMODE_MIXED))
    out = []
    try:
        for n, seed in enumerate(seeds):
            vel = W.fourier_velocity(g, seed)
            ctx.upload(api.F_U, vel["u"])
            ctx.upload(api.F_V, vel["v"])
            ctx.upload(api.F_W, vel["w"])
            ctx.Pressure_set_RHS(1.0)
            rec = {"seed": int(seed)}
            sol = {}
            for name, mode in modes:
                ctx.set_pressure_mode(mode)
                if n == 0:                       # capture the method's graphs once, untimed
                    ctx.upload(api.F_PHI, zero)
                    ctx.Pressure_solve()
                ctx.upload(api.F_PHI, zero)
                ctx.synchronize()
                api.event_record(ctx, 6)
                it, rr = ctx.Pressure_solve()
                api.event_record(ctx, 7)
                ms = api.event_elapsed(ctx, 6, 7)
                sol[name] = ctx.download(api.F_PHI)
                rec[name] = {"iters": it, "relres": rr, "ms": ms}
            a = _mean_removed(sol["mixed"], g)
            b = _mean_removed(sol["fp64"], g)
            rec["rel_diff"] = float(np.abs(a - b).max() / np.abs(b).max())
            if keep:
                rec["phi"] = sol
            out.append(rec)
    finally:
        ctx.close()
    return out


def summary(recs):
    """iterations and ms per solve of both methods over a set of records"""
    s = {}
    for name in ("fp64", "mixed"):
        its = [r[name]["iters"] for r in recs]
        ms = [r[name]["ms"] for r in recs]
        s[name] = {"iters_mean": float(np.mean(its)), "iters_max": int(np.max(its)),
                   "ms_per_solve": float(np.mean(ms)), "relres_max": float(max(r[name]["relres"] for r in recs))}
    s["rhs"] = len(recs)
    s["max_rel_diff"] = float(max(r["rel_diff"] for r in recs))
    s["speedup"] = s["fp64"]["ms_per_solve"] / s["mixed"]["ms_per_solve"]
    return s


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("shape", choices=sorted(SHAPES))
    ap.add_argument("--rhs", type=int, default=64)
    a = ap.parse_args()
    (nx, ny, nz), lengths, q = SHAPES[a.shape]
    case = W.poisson_case(nx, ny, nz, lengths, q)
    recs = solve_set(case, range(a.rhs))
    print(json.dumps({"shape": a.shape, "grid": [nx, ny, nz], **summary(recs)}))


if __name__ == "__main__":
    main()
