"""Immersed-boundary geometry set-up on the GPU (turb_geometry) against the
reference's own Surface / Levelset / Grid routines
(tests/golden/geom/geom_*.npz, made by tests/golden/make_golden.py): the
reinitialised signed distance at the c nodes, its u/v/w interpolation, the
u, v, w, c node statuses and the ghost-cell stencils (Immersed.c), bit for bit.  The reinitialisation stops on an L2
change summed in block order on the device (serially in the reference); the
cases here stop far from the 1e-5 threshold, so the step count agrees."""
import json
import os

import numpy as np
import pytest

from tests import _cases

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GEOM = {
    "bump": lambda: _cases.bump_small(24, 12, 8),
    "multi": lambda: _cases.multi_small(40, 20, 12),
}


@pytest.fixture(scope="module")
def api():
    from turbins_gb300 import api as A
    from turbins_gb300 import build
    build.build()
    return A


@pytest.mark.parametrize("name", sorted(GEOM))
def test_geometry_matches_reference(api, name):
    z = np.load(os.path.join(HERE, "golden", "geom", "geom_%s.npz" % name))
    meta = json.loads(str(z["meta"]))
    case = GEOM[name]()
    g = case.grid
    assert (g.nx, g.ny, g.nz) == (meta["nx"], meta["ny"], meta["nz"])
    for k in ("xc", "yc", "zc", "xu", "yv", "zw"):
        assert np.array_equal(getattr(g, k), z["grid_" + k]), k
    ctx = api.Context(g, case.params)
    sdf, st, iters = ctx.geometry(z["ipos"])
    assert 1 <= iters <= 503
    for q in "cuvw":
        d = np.abs(sdf[q] - z["ref_sdf_" + q]).max()
        assert np.array_equal(sdf[q], z["ref_sdf_" + q]), (q, d)
    for q in "uvwc":
        bad = int((st[q] != z["ref_status_" + q]).sum())
        assert bad == 0, (q, bad)


@pytest.mark.parametrize("name", sorted(GEOM))
def test_stencils_match_reference(api, name):
    """the ghost-cell stencils turb_geometry builds on the device against the
    reference's Immersed_setup_q_immersed_nodes, every array bit for bit"""
    z = np.load(os.path.join(HERE, "golden", "geom", "geom_%s.npz" % name))
    case = GEOM[name]()
    ctx = api.Context(case.grid, case.params)
    ctx.geometry(z["ipos"])
    for q in "uvwc":
        ib = ctx.geometry_stencils(q)
        assert ib["n"] == len(z["ref_ib_%s_im" % q]), q
        for k in ("im", "nf", "fidx", "fcoef", "bcoef", "pts"):
            ref = z["ref_ib_%s_%s" % (q, k)]
            assert np.array_equal(ib[k], ref), (q, k, np.abs(ib[k].astype(float) - ref.astype(float)).max())
