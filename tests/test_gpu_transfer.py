"""Host <-> device transfers (turb_fields_upload / turb_fields_download and
the single-field calls built on them): every field round-trips bit for bit,
with pinned and pageable host arrays, in both host-copy modes (copy engines
through staging, or the layout kernel across the host link), for field
counts that use both staging buffers more than once."""
import numpy as np
import pytest

from tests import _cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from turbins_gb300 import api as A
    from turbins_gb300 import build
    build.build()
    return A


@pytest.mark.parametrize("mode", ["dma", "kernel"])
@pytest.mark.parametrize("pinned", ["pageable", "registered", "driver"])
def test_fields_round_trip(api, pinned, mode):
    case = _cases.bump_small(24, 12, 8)
    g = case.grid
    ctx = api.Context(g, case.params)
    ctx.set_host_copy(api.HOST_COPY_DMA if mode == "dma" else api.HOST_COPY_KERNEL)
    rng = np.random.Generator(np.random.PCG64(5))
    fields = [api.F_U, api.F_V, api.F_W, api.F_PHI, api.F_DPX, api.F_DPY, api.F_DPZ, api.F_C0]
    src = [np.ascontiguousarray(rng.standard_normal(g.shape)) for _ in fields]
    dst = [np.zeros(g.shape) for _ in fields]
    if pinned == "driver":
        src2 = []
        for a in src:
            b = api.host_empty(g.shape)
            b[...] = a
            src2.append(b)
        src = src2
        dst = [api.host_empty(g.shape) for _ in fields]
    if pinned == "registered":
        for a in src + dst:
            api.host_register(a)
    try:
        ctx.upload_many(list(zip(fields, src)))
        ctx.download_many(list(zip(fields, dst)))
        for a, b in zip(src, dst):
            assert np.array_equal(a, b)
        # single-field calls see the same data
        for f, a in zip(fields, src):
            assert np.array_equal(ctx.download(f), a)
        ctx.upload(api.F_U, src[1])
        assert np.array_equal(ctx.download(api.F_U), src[1])
    finally:
        if pinned == "registered":
            for a in src + dst:
                api.host_unregister(a)
        ctx.close()


@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_matches_separate_calls(api, pinned):
    """turb_step_host (the state uploaded, one step, downloaded into the same
    arrays, the late fields' copies overlapping the step) gives the same bits
    and the same solver statistics as turb_fields_upload, turb_step and
    turb_fields_download in turn, for three steps of the immersed multi-bump
    case; with pageable arrays it is those three calls."""
    case = _cases.multi_small()
    s = _cases.random_state(case, seed=3)
    g = case.grid
    fields = [api.F_U, api.F_V, api.F_W, api.F_PHI, api.F_DPX, api.F_DPY, api.F_DPZ] + \
        [api.F_C0 + i for i in range(case.params.nconc)]
    out, stats = [], []
    for fused in (False, True):
        ctx = api.Context(g, case.params)
        try:
            ctx.load_state(s)
            bufs = [api.host_empty(g.shape) if pinned else np.zeros(g.shape) for _ in fields]
            pairs = list(zip(fields, bufs))
            ctx.download_many(pairs)
            st = []
            for _ in range(3):
                if fused:
                    st.append(ctx.step_host(case.dt, pairs))
                else:
                    ctx.upload_many(pairs)
                    st.append(ctx.step(case.dt))
                    ctx.download_many(pairs)
            out.append([b.copy() for b in bufs])
            stats.append(st)
        finally:
            ctx.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
    for a, b in zip(stats[0], stats[1]):
        for k in a:
            if k != "kernel_launches":
                assert a[k] == b[k], k
