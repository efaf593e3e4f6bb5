"""The no-allocation divergence check against the regular entry point.

Some callers cannot allocate GPU memory: a host that runs under a fixed
device memory budget, or a plugin that only receives device buffers from its
host application.  turb_velocity_divergence_noalloc serves them: it reads
caller-owned device buffers and keeps its scratch in a fixed-size array
inside the library.  These tests call it through the C ABI twice in a row and
check both calls against turb_Pressure_compute_velocity_divergence on the same
fields; the results must be the same bits (same arithmetic, and the maximum
of non-negative values is exact).  They cover the unpadded row pitch nx+1 and
the library's own 8-aligned pitch, a status array without the BOUNDARY ring
on the last layers (the index guard keeps every read inside the caller's
buffers and gives the same bits), and a NaN, which the maximum must keep.
The file runs last (file name) so that a failure here never hides the other
tests.
"""
import ctypes as C

import numpy as np
import pytest

from tests import _cases

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def _pitched(a, px, fill=0.0):
    nz, ny, nx1 = a.shape
    out = np.full((nz, ny, px), fill, dtype=a.dtype)
    out[:, :, :nx1] = a
    return out


def _call(lib, torch, g, s, status, metrics, px):
    """one call of the no-allocation entry point on freshly copied buffers of
    row pitch px; returns (status code, div_max, div in DA layout)"""
    du, dv, dw = (_dev(torch, _pitched(s[k], px), torch.float64) for k in ("u", "v", "w"))
    dst = _dev(torch, _pitched(status, px, fill=7), torch.uint8)
    mx = [_dev(torch, metrics[k], torch.float64) for k in ("mxc", "myc", "mzc")]
    ddiv = torch.full((g.nz + 1, g.ny + 1, px), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    out = C.c_double(-1.0)
    P = C.c_void_p
    rc = lib.turb_velocity_divergence_noalloc(
        C.c_int(g.nx), C.c_int(g.ny), C.c_int(g.nz), C.c_longlong(px), P(du.data_ptr()),
        P(dv.data_ptr()), P(dw.data_ptr()), P(dst.data_ptr()), P(mx[0].data_ptr()), P(mx[1].data_ptr()),
        P(mx[2].data_ptr()), P(ddiv.data_ptr()), C.byref(out), P(0))
    got = ddiv.cpu().numpy()
    assert np.all(got[:, :, g.nx + 1:] == -1.0)      # pad columns untouched
    return rc, out.value, got[:, :, :g.nx + 1]


def _setup(mk):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from oracle.oracle import Oracle
    from turbins_gb300 import api, build
    build.build()
    case = mk()
    ctx = api.Context(case.grid, case.params)
    return torch, api, case, ctx, api.load_library(), Oracle(case.grid, case.params).metrics


@pytest.mark.parametrize("name,mk", [("lock", lambda: _cases.lock_small()), ("multi", lambda: _cases.multi_small())])
@pytest.mark.parametrize("padded", [False, True])
def test_noalloc_divergence_matches(name, mk, padded):
    torch, api, case, ctx, lib, metrics = _setup(mk)
    g = case.grid
    px = (g.nx + 1 + 7) // 8 * 8 if padded else g.nx + 1
    results = []
    for call in range(2):
        s = _cases.random_state(case, seed=31 + call)
        ctx.load_state(s)
        ref_max = ctx.Pressure_compute_velocity_divergence()
        ref_div = ctx.download(api.F_DIV)
        rc, got_max, got = _call(lib, torch, g, s, g.status["c"], metrics, px)
        assert rc == 0, lib.turb_status_string(rc)
        assert got_max == ref_max
        assert np.array_equal(got, ref_div)
        results.append(got_max)
    assert results[0] != results[1]   # two different fields, both checked
    ctx.close()


def test_noalloc_status_without_boundary_ring():
    """A status array whose last layers (i = nx, j = ny, k = nz) are not
    BOUNDARY: the kernel still reads only inside the caller's unpadded
    buffers and returns what the valid status gives."""
    torch, api, case, ctx, lib, metrics = _setup(lambda: _cases.lock_small())
    g = case.grid
    s = _cases.random_state(case, seed=5)
    ctx.load_state(s)
    ref_max = ctx.Pressure_compute_velocity_divergence()
    ref_div = ctx.download(api.F_DIV)
    st = g.status["c"].copy()
    st[-1, :, :] = 3
    st[:, -1, :] = 3
    st[:, :, -1] = 3
    for _ in range(2):
        rc, got_max, got = _call(lib, torch, g, s, st, metrics, g.nx + 1)
        assert rc == 0, lib.turb_status_string(rc)
        assert got_max == ref_max
        assert np.array_equal(got, ref_div)
    ctx.close()


def test_noalloc_keeps_nan():
    """One NaN velocity: both entry points report a NaN maximum and the NaN
    status, and a finite field afterwards is checked normally again."""
    torch, api, case, ctx, lib, metrics = _setup(lambda: _cases.lock_small())
    g = case.grid
    s = _cases.random_state(case, seed=9)
    s["u"] = s["u"].copy()
    s["u"][g.nz // 2, g.ny // 2, g.nx // 2] = np.nan
    ctx.load_state(s)
    with pytest.raises(api.TurbError) as ei:
        ctx.Pressure_compute_velocity_divergence()
    assert ei.value.code == 4
    rc, got_max, got = _call(lib, torch, g, s, g.status["c"], metrics, g.nx + 1)
    assert rc == 4 and got_max != got_max
    assert np.isnan(got).sum() == 2     # the two cells sharing that u face
    s2 = _cases.random_state(case, seed=10)
    ctx.load_state(s2)
    ref_max = ctx.Pressure_compute_velocity_divergence()
    rc, got_max, _ = _call(lib, torch, g, s2, g.status["c"], metrics, g.nx + 1)
    assert rc == 0 and got_max == ref_max
    ctx.close()


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
