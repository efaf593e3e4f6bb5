"""Training and use of the learned initial guess of the pressure solve.

Snapshots come from the plain solver (previous-pressure guess) on small runs
of the same physics; the network is trained on the GPU by the library's own
kernels (turb_net_train: tcgen05 forward and backward, Adam) and is then
attached to a solver context of any size whose cell counts are multiples of
8.  The solver keeps a network guess only when it lowers the initial residual
below the previous pressure's, so the converged answer never depends on it.

    python -m turbins_gb300.learned --infer 256 128 128      # training + inference report
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api as A
from . import net as N
from . import workload as W


def record(case_fn, seeds, steps, capacity=None):
    """Run case_fn(seed) for `steps` steps per seed with the plain solver and
    keep the network inputs of every pressure solve.  Returns (store, ctx),
    ctx being a context on the same grid (its pressure operator defines the
    training loss)."""
    store, ctx = None, None
    for seed in seeds:
        case = case_fn(seed)
        p = case.params
        if store is None:
            store = N.Snapshots(p.nx, p.ny, p.nz, capacity or 2 * steps * len(seeds))
        if ctx is not None:
            ctx.close()
        ctx = A.Context(case.grid, case.params)
        ctx.load_state(case.state)
        N.set_snapshot_store(ctx, store)
        for _ in range(steps):
            ctx.step(case.dt)
        N.set_snapshot_store(ctx, None)
    return store, ctx


def train(store, ctx, iters=3000, lr=1e-3, seed=0, init_seed=1, w_residual=1.0, w_energy=1.0):
    """Adam on randomly drawn snapshots (lr for 70% of the steps, lr/4 after);
    returns (net, mean loss of the last phase)."""
    nx, ny, nz = ctx.params.nx, ctx.params.ny, ctx.params.nz
    net = N.Net(nx, ny, nz, train=True)
    net.init_params(init_seed)
    net.set_loss(w_residual, w_energy)
    n1 = int(0.7 * iters)
    net.train_on(ctx, store, n1, lr=lr, seed=seed)
    loss = net.train_on(ctx, store, iters - n1, lr=lr / 4, seed=seed + 1)
    return net, loss


def attach(ctx, params):
    """Network of ctx's size carrying `params`, used as the LEARNED guess."""
    p = ctx.params
    net = N.Net(p.nx, p.ny, p.nz, train=False)
    net.set_params(params)
    N.set_learned_net(ctx, net)
    ctx.set_pressure_guess(A.GUESS_LEARNED)
    return net


def multi_bump_train_case(nx=128, ny=64, nz=64, full=(512, 256, 256)):
    """Training runs for the multi-bump step on a `full` grid: the same
    physics with the x extent cut to nx / full[0] of the full domain, one bump
    field per seed.  With ny = full[1] the training grid keeps the full case's
    spacing in every direction: the z extent is cut to nz / full[2] too, and
    the number of bumps follows the domain's area (16 on the full one)."""
    if ny != full[1]:
        return lambda seed: W.multi_bump_case(nx, ny, nz, seed=100 + seed, lx=32.0 * nx / full[0])
    fx, fz = nx / full[0], nz / full[2]
    nb = max(1, int(round(16 * fx * fz)))
    return lambda seed: W.multi_bump_case(nx, ny, nz, seed=100 + seed, lx=32.0 * fx, lz=2.0 * fz, nbump=nb)


def turbidity_train_case(nx=128, ny=64, nz=64):
    """Training runs for the single-bump turbidity current: one lock-noise seed each."""
    return lambda seed: W.turbidity_bump_case(nx, ny, nz, seed=seed)


def train_default(case_fn, seeds=8, steps=250, iters=3000, lr=1e-3, w_residual=1.0, w_energy=1.0):
    t0 = time.perf_counter()
    store, ctx = record(case_fn, range(seeds), steps)
    t1 = time.perf_counter()
    net, loss = train(store, ctx, iters=iters, lr=lr, w_residual=w_residual, w_energy=w_energy)
    t2 = time.perf_counter()
    res, en = net.eval_on(ctx, store, max(0, len(store) - 64), min(64, len(store)))
    info = dict(snapshots=len(store), record_s=t1 - t0, train_s=t2 - t1, iters=iters, train_loss=loss,
                loss_weights=[w_residual, w_energy], last64_residual=res, last64_energy=en)
    params = net.get_params()
    net.close()
    store.close()
    ctx.close()
    return params, info


ARMS = {"previous": (A.GUESS_PREVIOUS, False), "projection": (A.GUESS_PROJECT, False),
        "learned": (A.GUESS_LEARNED, False), "learned_galerkin": (A.GUESS_LEARNED, True)}


def compare(case, params, steps, pmode=A.PMODE_MIXED, arms=tuple(ARMS), div_gate=1e-10):
    """Per-step PCG iterations and pressure-solve time of each guess from the
    same initial state: the previous pressure, the Galerkin fit over the
    stage's last two solutions, the network candidate, and the network
    candidate fitted together with those solutions."""
    out = {}
    for name in arms:
        mode, gal = ARMS[name]
        ctx = A.Context(case.grid, case.params)
        ctx.load_state(case.state)
        ctx.set_pressure_mode(pmode)
        ctx.set_divergence_gate(div_gate)
        net = attach(ctx, params) if mode == A.GUESS_LEARNED else None
        ctx.set_pressure_guess(mode)
        ctx.set_guess_galerkin(gal)
        for _ in range(2):
            ctx.step(case.dt)   # history for the guess
        A.profile_enable(ctx, True)
        its = []
        A.event_record(ctx, 0)
        for _ in range(steps):
            st = ctx.step(case.dt)
            its.append(list(st["p_iters"]))
        A.event_record(ctx, 1)
        ms = A.event_elapsed(ctx, 0, 1)
        prof = A.profile_read(ctx)
        tried, taken = ctx.pressure_guess_stats()
        out[name] = dict(p_iters=its, mean_iters=float(np.mean(its)), residual_ratio=ctx.pressure_guess_ratio(),
                         step_ms=ms / steps,
                         solve_ms_per_step=sum(prof[g][0] for g in ("mg", "pcg", "net")) / steps,
                         net_ms_per_step=prof["net"][0] / steps, guess_tried=tried, guess_taken=taken)
        if net is not None:
            net.close()
        ctx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--infer", type=int, nargs=3, default=[256, 128, 128])
    ap.add_argument("--train", type=int, nargs=3, default=[128, 64, 64])
    ap.add_argument("--seeds", type=int, default=8)
    ap.add_argument("--steps", type=int, default=250)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--compare-steps", type=int, default=20)
    ap.add_argument("--warm-steps", type=int, default=200, help="steps before the comparison window")
    ap.add_argument("--physics", choices=["turbidity", "multi"], default="turbidity")
    ap.add_argument("--save", default=None)
    a = ap.parse_args()
    tx, ty, tz = a.train
    mk = turbidity_train_case(tx, ty, tz) if a.physics == "turbidity" else multi_bump_train_case(tx, ty, tz)
    params, info = train_default(mk, seeds=a.seeds, steps=a.steps, iters=a.iters)
    if a.save:
        np.save(a.save, params)
    nx, ny, nz = a.infer
    case = W.turbidity_bump_case(nx, ny, nz) if a.physics == "turbidity" else \
        W.multi_bump_case(nx, ny, nz, lx=32.0 * nx / 512.0)
    ctx = A.Context(case.grid, case.params)
    ctx.load_state(case.state)
    for _ in range(a.warm_steps):
        ctx.step(case.dt)
    case.state = ctx.state()
    ctx.close()
    res = compare(case, params, a.compare_steps)
    print(json.dumps(dict(train=info, infer=[nx, ny, nz], physics=a.physics, warm_steps=a.warm_steps, **res)))


if __name__ == "__main__":
    main()
