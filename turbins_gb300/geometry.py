"""Immersed-boundary geometry of a bottom surface, set up on the GPU.

The reference builds its geometry once at start-up from the bed heights
h(x, z) (MAC_grid.interface_position): a signed distance by level-set
reinitialisation, the u/v/w/c node statuses and the ghost-cell stencils of
every IMMERSED node (Surface.c, Levelset.c, Grid.c:1825-1870,
Immersed.c:546-616).  ``device_geometry`` runs that set-up through
turb_geometry / turb_geometry_stencils and, with ``apply``, puts the
statuses and stencils into a workload Grid, so that a Context created from it
solves on exactly the reference's geometry.

    python -m turbins_gb300.geometry [nx ny nz]

times the set-up of the multi-bump bed (default 512 x 256 x 256) and prints
one JSON line.
"""
from __future__ import annotations

import json
import sys
import time

import numpy as np

from . import api as A
from . import workload as W


def bed_heights(grid, bed):
    """interface_position [nz+1][nx+1]: the bed height at the cell-centre
    columns (xc[i], zc[k])"""
    return np.ascontiguousarray(bed.h(grid.xc[None, :], grid.zc[:, None])[0])


def device_geometry(grid, params, heights, apply=True, ctx=None):
    """Set up the geometry of bed heights [nz+1][nx+1] on the GPU.  Returns
    dict(sdf, status, stencils, steps, seconds); with apply the grid's
    status and ib records are replaced by the device results."""
    own = ctx is None
    if own:
        ctx = A.Context(grid, params)
    try:
        t = time.perf_counter()
        sdf, st, steps = ctx.geometry(heights)
        ib = {q: ctx.geometry_stencils(q) for q in "uvwc"}
        sec = time.perf_counter() - t
    finally:
        if own:
            ctx.close()
    if apply:
        for q in "uvwc":
            grid.status[q] = st[q]
            grid.ib[q] = {k: ib[q][k] for k in ("n", "im", "nf", "fidx", "fcoef", "bcoef")}
    return dict(sdf=sdf, status=st, stencils=ib, steps=steps, seconds=sec)


def reference_geometry(case):
    """Replace a workload case's analytic-sdf statuses and stencils with the
    reference's construction run on the GPU (level-set reinitialised sdf,
    Immersed.c stencils; bit-identical to the reference's set-up), and zero
    the concentration at the new SOLID / BOUNDARY c nodes as the lock
    initial condition does.  Returns the set-up record (seconds, reinit
    steps, IMMERSED nodes per quantity)."""
    g = case.grid
    if case.bed is None:
        return None
    r = device_geometry(g, case.params, bed_heights(g, case.bed), apply=True)
    st = g.status["c"]
    for k in case.state:
        if k.startswith("c"):
            case.state[k] = case.state[k].copy()
            case.state[k][(st == W.BOUNDARY) | (st == W.SOLID)] = 0.0
    return {"seconds": r["seconds"], "reinit_steps": r["steps"],
            "ib_nodes": {q: int(r["stencils"][q]["n"]) for q in "uvwc"}}


def main(argv):
    nx, ny, nz = (int(a) for a in argv[:3]) if len(argv) >= 3 else (512, 256, 256)
    case = W.multi_bump_case(nx, ny, nz)
    g = case.grid
    h = bed_heights(g, case.bed)
    ctx = A.Context(g, case.params)
    runs = []
    for _ in range(3):
        r = device_geometry(g, case.params, h, apply=False, ctx=ctx)
        runs.append(r["seconds"])
    out = dict(workload="multi_bump_%dx%dx%d" % (nx, ny, nz), seconds=runs, reinit_steps=r["steps"],
               ib_nodes={q: int(r["stencils"][q]["n"]) for q in "uvwc"},
               single_fluid_node={q: int((r["stencils"][q]["nf"] == 1).sum()) for q in "uvwc"})
    ctx.close()
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
