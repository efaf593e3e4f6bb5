"""The single-block V-cycle tail (k_vcycle_tail, turb_set_mg_tail) against
the launch-per-half-sweep V-cycle: the same per-cell operations, so two full
steps from the same state agree bit for bit, in both pressure modes, with the
tail holding every level (small grid) or only the coarse ones."""
import numpy as np
import pytest

from tests import _cases

pytestmark = pytest.mark.gpu

KEYS = ["u", "v", "w", "phi", "dpx", "dpy", "dpz", "c0"]


@pytest.fixture(scope="module")
def api():
    from turbins_gb300 import api as A
    from turbins_gb300 import build
    build.build()
    return A


def run(api, case, state, pmode, tail):
    ctx = api.Context(case.grid, case.params)
    ctx.load_state(state)
    ctx.set_pressure_mode(pmode)
    ctx.set_mg_tail(tail)
    its = [ctx.step(case.dt)["p_iters"] for _ in range(2)]
    out = {k: v for k, v in ctx.state().items() if k in KEYS}
    ctx.close()
    return out, its


@pytest.mark.parametrize("mk,tail", [(lambda: _cases.bump_small(24, 12, 8), 1 << 20),
                                     (lambda: _cases.multi_small(64, 32, 16), 4096)])
@pytest.mark.parametrize("pmode", [0, 1])
def test_tail_is_bit_identical(api, mk, tail, pmode):
    case = mk()
    state = _cases.random_state(case, seed=31)
    a, ia = run(api, case, state, pmode, tail)
    b, ib = run(api, case, state, pmode, 0)
    assert ia == ib
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k
