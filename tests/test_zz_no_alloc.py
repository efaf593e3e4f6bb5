"""The no-allocation divergence check against the regular entry point.

Some callers cannot allocate GPU memory (a step replayed inside a CUDA graph
capture, a host under a fixed memory budget, a plugin that only receives
device buffers from its host application).  turb_velocity_divergence_noalloc
serves them: it reads caller-owned device buffers and keeps its scratch in a
fixed-size array inside the library.  This test calls it through the C ABI
twice in a row and checks both calls against
turb_Pressure_compute_velocity_divergence on the same fields; the results
must be the same bits (same arithmetic, and the maximum of non-negative
values is exact).  It runs last (file name) so that a failure here never
hides the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from tests import _cases

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


@pytest.mark.parametrize("name,mk", [("lock", lambda: _cases.lock_small()), ("multi", lambda: _cases.multi_small())])
def test_noalloc_divergence_matches(name, mk):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from turbins_gb300 import api, build
    build.build()
    case = mk()
    g = case.grid
    ctx = api.Context(g, case.params)
    lib = api.load_library()
    results = []
    for call in range(2):
        s = _cases.random_state(case, seed=31 + call)
        ctx.load_state(s)
        ref_max = ctx.Pressure_compute_velocity_divergence()
        ref_div = ctx.download(api.F_DIV)
        from oracle.oracle import Oracle
        orc = Oracle(g, case.params)
        du, dv, dw = (_dev(torch, s[k], torch.float64) for k in ("u", "v", "w"))
        dst = _dev(torch, g.status["c"], torch.uint8)
        mx = [_dev(torch, orc.metrics[k], torch.float64) for k in ("mxc", "myc", "mzc")]
        ddiv = torch.full(g.shape, -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        out = C.c_double(-1.0)
        P = C.c_void_p
        rc = lib.turb_velocity_divergence_noalloc(
            C.c_int(g.nx), C.c_int(g.ny), C.c_int(g.nz), C.c_longlong(g.nx + 1), P(du.data_ptr()),
            P(dv.data_ptr()), P(dw.data_ptr()), P(dst.data_ptr()), P(mx[0].data_ptr()), P(mx[1].data_ptr()),
            P(mx[2].data_ptr()), P(ddiv.data_ptr()), C.byref(out), P(0))
        assert rc == 0, lib.turb_status_string(rc)
        got = ddiv.cpu().numpy()
        assert out.value == ref_max
        assert np.array_equal(got, ref_div)
        results.append(out.value)
    assert results[0] != results[1]   # two different fields, both checked


def test_noalloc_rejects_oversize():
    from turbins_gb300 import api, build
    build.build()
    lib = api.load_library()
    out = C.c_double()
    P = C.c_void_p
    one = P(1)
    rc = lib.turb_velocity_divergence_noalloc(C.c_int(8192), C.c_int(8192), C.c_int(8192), C.c_longlong(8193),
                                              one, one, one, one, one, one, one, one, C.byref(out), P(0))
    assert rc == 6
