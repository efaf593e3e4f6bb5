"""Checkpoint / resume on the GPU (turb_resume_write / turb_resume_read)
against the restart set the reference's Resume.c wrote
(tests/golden/resume_bump)."""
import filecmp
import os
import shutil

import numpy as np
import pytest

from oracle import resume_format as F
from tests import _cases
from tests.test_resume_format import GOLD, decoded, golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from turbins_gb300 import api as A
    from turbins_gb300 import build
    build.build()
    return A


def _ctx(api, case):
    ctx = api.Context(case.grid, case.params)
    ctx.load_state(case.state)
    return ctx


def test_read_reference_set(api):
    case, meta = golden()
    st, dep = decoded(case)
    ctx = _ctx(api, case)
    prim = ctx.resume_read(GOLD, grid=True, deposit=True)
    assert prim == F.read_primary(os.path.join(GOLD, "Resume_primary.dat"))
    s = ctx.state()
    for k in ("u", "v", "w", "dpx", "dpy", "dpz", "c0"):
        assert np.array_equal(s[k], st[k]), k
    assert not np.any(s["phi"])
    assert np.array_equal(ctx.deposit(), dep)
    ctx.close()


def test_write_matches_reference_bytes(api, tmp_path):
    case, meta = golden()
    st, dep = decoded(case)
    ctx = _ctx(api, case)
    ctx.load_state({k: v for k, v in st.items() if k != "status_c"})
    ctx.set_deposit(dep)
    ctx.resume_write(str(tmp_path), meta["prim"], grid=True, deposit=True)
    names = sorted(f for f in os.listdir(GOLD) if f.startswith("Resume_"))
    assert names == sorted(os.listdir(tmp_path))
    for f in names:
        assert filecmp.cmp(os.path.join(GOLD, f), os.path.join(tmp_path, f), shallow=False), f
    ctx.close()


def test_geometry_mismatch_is_refused(api, tmp_path):
    case, meta = golden()
    for f in os.listdir(GOLD):
        shutil.copy(os.path.join(GOLD, f), tmp_path)
    g = F.read_vec(os.path.join(GOLD, "Resume_gridc.bin"))
    g[np.argmax(g == 3.0)] = 5.0           # one FLUID node turned IMMERSED
    F.write_vec(os.path.join(tmp_path, "Resume_gridc.bin"), g)
    ctx = _ctx(api, case)
    before = ctx.state()
    with pytest.raises(api.TurbError) as e:
        ctx.resume_read(str(tmp_path), grid=True)
    assert e.value.code == 8
    after = ctx.state()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    ctx.close()


def test_resumed_run_repeats_uninterrupted_run(api, tmp_path):
    """3 steps, checkpoint (with the pressure), 2 more steps; a new context
    resumed from the checkpoint gives the same fields bit for bit."""
    case = _cases.multi_small()
    a = _ctx(api, case)
    a.deposit_enable(True)
    for _ in range(3):
        a.step(case.dt)
    prim = dict(time=3 * case.dt, dt=case.dt, dt_old=case.dt, iter=3, output_iter=0)
    a.resume_write(str(tmp_path), prim, deposit=True, phi=True)
    for _ in range(2):
        a.step(case.dt)
    b = api.Context(case.grid, case.params)
    b.deposit_enable(True)
    q = b.resume_read(str(tmp_path), deposit=True, phi=True)
    assert q["iter"] == 3
    for _ in range(2):
        b.step(case.dt)
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    assert np.array_equal(a.deposit(), b.deposit())
    a.close()
    b.close()
