"""The learned initial guess end to end on the GPU: snapshots recorded by the
plain solver, training with the library's own forward/backward/Adam kernels,
and what the trained network gains over the previous-pressure guess on later
steps of the same flow -- with the converged answer unchanged."""
import numpy as np
import pytest

from turbins_gb300 import workload as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    from turbins_gb300 import build
    build.build()
    from turbins_gb300 import api as A
    from turbins_gb300 import net as N
    return A, N


def _case():
    c = W.turbidity_bump_case(64, 32, 32)
    c.params.eno_order = 3
    return c


def _run(A, case, state, steps, dt, guess, net=None, galerkin=False):
    ctx = A.Context(case.grid, case.params)
    ctx.load_state(state)
    if net is not None:
        from turbins_gb300 import net as N
        N.set_learned_net(ctx, net)
    ctx.set_pressure_guess(guess)
    ctx.set_guess_galerkin(galerkin)
    iters = []
    for _ in range(steps):
        st = ctx.step(dt)
        iters.append(sum(st["p_iters"]))
        assert max(st["div_max"]) <= 1e-10
    out = ctx.state()
    tried, taken = ctx.pressure_guess_stats()
    return out, iters, tried, taken, ctx.pressure_guess_ratio()


def test_learned_guess_trains_and_gains(mods):
    A, N = mods
    case = _case()
    dt = case.dt
    nx, ny, nz = case.params.nx, case.params.ny, case.params.nz
    ctx = A.Context(case.grid, case.params)
    ctx.load_state(case.state)
    train = N.Snapshots(nx, ny, nz, 160)
    held = N.Snapshots(nx, ny, nz, 40)
    N.set_snapshot_store(ctx, train)
    for _ in range(60):
        ctx.step(dt)
    N.set_snapshot_store(ctx, held)
    for _ in range(20):
        ctx.step(dt)
    N.set_snapshot_store(ctx, None)
    assert len(train) >= 100 and len(held) >= 30
    state = ctx.state()

    net = N.Net(nx, ny, nz, train=True)
    net.init_params(1)
    net.set_loss(1.0, 1.0)
    before = net.eval_on(ctx, held, 0, len(held))
    # a near-zero output leaves the previous pressure as it is
    assert abs(before[0] - 1.0) < 0.5 and abs(before[1] - 1.0) < 0.5
    loss = net.train_on(ctx, train, 600, lr=1e-3, seed=7)
    after = net.eval_on(ctx, held, 0, len(held))
    print("held-out |r|^2 ratio before %.4f after %.4f, energy-error ratio before %.4f after %.4f (train %.4f)"
          % (before[0], after[0], before[1], after[1], loss))
    assert after[0] < 0.5 * before[0] and after[1] < before[1]

    ref, it_prev, _, _, _ = _run(A, case, state, 12, dt, A.GUESS_PREVIOUS)
    got, it_learn, tried, taken, ratio = _run(A, case, state, 12, dt, A.GUESS_LEARNED, net)
    got_g, it_gal, tried_g, taken_g, ratio_g = _run(A, case, state, 12, dt, A.GUESS_LEARNED, net, galerkin=True)
    print("PCG iterations per step: previous %s  learned %s  (guess taken %d/%d, initial residual x%.3f)  "
          "learned + Galerkin fit %s (taken %d/%d, x%.3f)"
          % (it_prev, it_learn, taken, tried, ratio, it_gal, taken_g, tried_g, ratio_g))
    # what the network gains: a lower initial residual on every solve it is
    # tried on, and no more iterations than the previous pressure; fitted
    # together with the stage's last two solutions (the energy-norm best
    # guess in their span), fewer iterations in total
    assert tried > 0 and taken == tried and ratio < 0.6
    assert sum(it_learn) <= sum(it_prev)
    assert tried_g > 0 and sum(it_gal) < sum(it_prev)
    # the guess changes the iteration count, not the converged answer
    for k in ("u", "v", "w"):
        scale = max(np.abs(ref[k]).max(), 1e-30)
        assert np.abs(got[k] - ref[k]).max() <= 1e-7 * scale, k
        assert np.abs(got_g[k] - ref[k]).max() <= 1e-7 * scale, k
    p0, p1 = ref["phi"] - ref["phi"].mean(), got["phi"] - got["phi"].mean()
    assert np.abs(p1 - p0).max() <= 1e-7 * np.abs(p0).max()
    net.close()


def test_projection_guess_keeps_the_answer(mods):
    """The Galerkin fit over the stage's last two solutions (no network):
    fields after 12 steps as with the previous-pressure guess, to the
    solvers' tolerance, in no more PCG iterations."""
    A, N = mods
    case = _case()
    ctx = A.Context(case.grid, case.params)
    ctx.load_state(case.state)
    for _ in range(20):
        ctx.step(case.dt)
    state = ctx.state()
    ctx.close()
    ref, it_prev, _, _, _ = _run(A, case, state, 12, case.dt, A.GUESS_PREVIOUS)
    got, it_proj, tried, taken, ratio = _run(A, case, state, 12, case.dt, A.GUESS_PROJECT)
    print("PCG iterations per step: previous %s  projection %s  (taken %d/%d, initial residual x%.3f)"
          % (it_prev, it_proj, taken, tried, ratio))
    assert tried > 0 and sum(it_proj) <= sum(it_prev)
    for k in ("u", "v", "w"):
        scale = max(np.abs(ref[k]).max(), 1e-30)
        assert np.abs(got[k] - ref[k]).max() <= 1e-7 * scale, k


def test_learned_mode_without_network_stages_is_the_projection(mods):
    """With the Galerkin fit on, the learned mode's stages that do not
    evaluate the network take the fit over their earlier solutions alone:
    with no network stage at all (guess stages 0) the run is the projection
    guess's, bit for bit, iteration for iteration, and the network never
    runs."""
    A, N = mods
    case = _case()
    ctx = A.Context(case.grid, case.params)
    ctx.load_state(case.state)
    for _ in range(10):
        ctx.step(case.dt)
    state = ctx.state()
    ctx.close()
    proj, it_proj, _, _, _ = _run(A, case, state, 6, case.dt, A.GUESS_PROJECT)
    nx, ny, nz = case.params.nx, case.params.ny, case.params.nz
    net = N.Net(nx, ny, nz, train=False)
    net.init_params(3)
    ctx = A.Context(case.grid, case.params)
    try:
        ctx.load_state(state)
        N.set_learned_net(ctx, net)
        ctx.set_pressure_guess(A.GUESS_LEARNED)
        ctx.set_guess_galerkin(True)
        ctx.set_guess_stages(0)
        it = [sum(ctx.step(case.dt)["p_iters"]) for _ in range(6)]
        got = ctx.state()
    finally:
        ctx.close()
        net.close()
    assert it == it_proj
    for k in proj:
        assert np.array_equal(proj[k], got[k]), k
