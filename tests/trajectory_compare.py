"""Long-run comparison of the GPU step with the oracle on the multi-bump
workload with the reference's immersed-boundary geometry (test
infrastructure, too slow for the test suite at the headline size).

  # on a GB300: the step on the GPU, its per-step maxima, and the device-built
  # geometry (statuses, immersed stencils, lock concentrations) for the oracle
  python tests/trajectory_compare.py gpu NX NY NZ STEPS OUT [--pmode mixed|fp64]

  # on any host: the oracle on the same geometry
  python tests/trajectory_compare.py oracle NX NY NZ STEPS OUT --geom GPU_OUT [--threads N]

  # side by side
  python tests/trajectory_compare.py compare GPU_OUT ORACLE_OUT

OUT / GPU_OUT name a prefix: the gpu mode writes PREFIX.jsonl (one record per
step: max |u|, |v|, |w|, max |div u|, PCG iterations) and PREFIX_geom_Q.npz
per quantity group, the oracle mode PREFIX.jsonl.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from turbins_gb300 import workload as W  # noqa: E402

IB_KEYS = ("n", "im", "nf", "fidx", "fcoef", "bcoef")
GROUPS = ("uv", "wc")   # two files, each small enough to move between machines


def _record(n, s, st):
    return {"step": n, "umax": float(np.abs(s["u"]).max()), "vmax": float(np.abs(s["v"]).max()),
            "wmax": float(np.abs(s["w"]).max()), "div": float(max(st["div_max"])), "p": list(st["p_iters"])}


def run_gpu(a):
    from turbins_gb300 import api, geometry as G
    case = W.multi_bump_case(a.nx, a.ny, a.nz)
    G.reference_geometry(case)
    g = case.grid
    for grp in GROUPS:
        out = {}
        for q in grp:
            out["status_" + q] = g.status[q]
            for k in IB_KEYS:
                out["ib_%s_%s" % (q, k)] = np.asarray(g.ib[q][k])
        if "c" in grp:
            for k, v in case.state.items():
                if k.startswith("c"):
                    out["state_" + k] = v
        np.savez_compressed("%s_geom_%s.npz" % (a.out, grp), **out)
    ctx = api.Context(g, case.params)
    ctx.load_state(case.state)
    ctx.set_pressure_mode(api.PMODE_MIXED if a.pmode == "mixed" else api.PMODE_FP64)
    ctx.set_pressure_guess(api.GUESS_PREVIOUS)
    if a.pmode == "mixed":
        ctx.set_divergence_gate(1e-10)
    with open(a.out + ".jsonl", "w") as f:
        try:
            for n in range(1, a.steps + 1):
                st = ctx.step(case.dt)
                s = {k: ctx.download(fld) for k, fld in (("u", api.F_U), ("v", api.F_V), ("w", api.F_W))}
                f.write(json.dumps(_record(n, s, st)) + "\n")
                f.flush()
        finally:
            ctx.close()


def run_oracle(a):
    from oracle import oracle as O
    O.set_threads(a.threads)
    case = W.multi_bump_case(a.nx, a.ny, a.nz)
    g = case.grid
    for grp in GROUPS:
        z = np.load("%s_geom_%s.npz" % (a.geom, grp))
        for q in grp:
            g.status[q] = z["status_" + q]
            g.ib[q] = {k: (int(z["ib_%s_%s" % (q, k)]) if k == "n" else z["ib_%s_%s" % (q, k)]) for k in IB_KEYS}
        if "c" in grp:
            for k in list(case.state):
                if k.startswith("c"):
                    case.state[k] = z["state_" + k]
    o = O.Oracle(g, case.params)
    s = {k: v.copy() for k, v in case.state.items()}
    with open(a.out + ".jsonl", "w") as f:
        for n in range(1, a.steps + 1):
            st = o.step(s, case.dt)
            f.write(json.dumps(_record(n, s, st)) + "\n")
            f.flush()


def compare(a):
    def load(p):
        return {r["step"]: r for r in (json.loads(l) for l in open(p + ".jsonl"))}
    gpu, orc = load(a.gpu), load(a.oracle)
    print("step  max|u| gpu / oracle            max|w| gpu / oracle            rel |w|")
    for n in sorted(set(gpu) & set(orc)):
        g_, o_ = gpu[n], orc[n]
        rel = abs(g_["wmax"] - o_["wmax"]) / max(o_["wmax"], 1e-300)
        print("%4d  %.6e / %.6e  %.6e / %.6e  %.2e" % (n, g_["umax"], o_["umax"], g_["wmax"], o_["wmax"], rel))


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="mode", required=True)
    for m in ("gpu", "oracle"):
        p = sub.add_parser(m)
        p.add_argument("nx", type=int)
        p.add_argument("ny", type=int)
        p.add_argument("nz", type=int)
        p.add_argument("steps", type=int)
        p.add_argument("out")
        if m == "gpu":
            p.add_argument("--pmode", default="mixed", choices=["mixed", "fp64"])
        else:
            p.add_argument("--geom", required=True)
            p.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    p = sub.add_parser("compare")
    p.add_argument("gpu")
    p.add_argument("oracle")
    a = ap.parse_args()
    {"gpu": run_gpu, "oracle": run_oracle, "compare": compare}[a.mode](a)


if __name__ == "__main__":
    main()
