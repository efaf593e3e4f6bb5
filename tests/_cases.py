"""Small seeded cases shared by the parity tests (sizes the oracle finishes in
seconds)."""
import numpy as np

from turbins_gb300 import workload as W


def lock_small(nx=32, ny=16, nz=16, order=2):
    c = W.lock_exchange_case(nx, ny, nz)
    c.params.eno_order = order
    return c


def bump_small(nx=48, ny=24, nz=16, order=3):
    c = W.turbidity_bump_case(nx, ny, nz)
    c.params.eno_order = order
    return c


def multi_small(nx=64, ny=32, nz=16, order=3):
    return W.multi_bump_case(nx, ny, nz, lx=8.0)


def random_state(case, seed=1, amp=0.05):
    """Seeded smooth-plus-noise velocities so every ENO branch is exercised."""
    g = case.grid
    rng = np.random.Generator(np.random.PCG64(seed))
    s = dict(case.state)
    for k in ("u", "v", "w"):
        a = amp * rng.standard_normal(g.shape)
        st = g.status[k]
        a[st == W.BOUNDARY] = 0.0
        s[k] = a
    for k in ("dpx", "dpy", "dpz"):
        s[k] = 1e-3 * rng.standard_normal(g.shape)
    s["phi"] = 1e-2 * rng.standard_normal(g.shape)
    return s
