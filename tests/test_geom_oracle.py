"""The numpy restatement of the reference's geometry set-up (oracle/geometry.py)
pinned to the reference's own Surface / Levelset / Grid routines through the
fixtures tests/golden/geom/geom_*.npz: sdf bit for bit, statuses exactly."""
import os

import numpy as np
import pytest

from oracle import geometry as G
from tests import _cases

HERE = os.path.dirname(os.path.abspath(__file__))
GEOM = {
    "bump": lambda: _cases.bump_small(24, 12, 8),
    "multi": lambda: _cases.multi_small(40, 20, 12),
}


@pytest.mark.parametrize("name", sorted(GEOM))
def test_geometry_oracle_matches_reference(name):
    z = np.load(os.path.join(HERE, "golden", "geom", "geom_%s.npz" % name))
    g = GEOM[name]().grid
    sdf, st, n = G.geometry(g, z["ipos"])
    assert 1 <= n <= 503
    for q in "cuvw":
        assert np.array_equal(sdf[q], z["ref_sdf_" + q]), q
    for q in "uvwc":
        assert np.array_equal(st[q], z["ref_status_" + q]), q


def test_flat_bed_keeps_the_interface():
    """a flat bed: the reinitialised sdf keeps the sign of yc - h, the c
    statuses are FLUID above h, IMMERSED in the cell row under it, SOLID below"""
    g = _cases.bump_small(24, 12, 8).grid
    h = 0.31
    ipos = np.full((g.nz + 1, g.nx + 1), h)
    sdf, st, n = G.geometry(g, ipos)
    assert 1 <= n <= 503
    yc = g.yc[:-1]
    c = sdf["c"][:-1, :-1, :-1]
    assert np.all(np.sign(c) == np.sign(yc - h)[None, :, None])
    want = np.where(yc >= h, G.FLUID, np.where(np.r_[yc[1:], np.inf] >= h, G.IMMERSED, G.SOLID))
    assert np.all(st["c"][:-1, :-1, :-1] == want[None, :, None].astype(np.uint8))


@pytest.mark.parametrize("name", sorted(GEOM))
def test_stencil_oracle_matches_reference(name):
    """Immersed_setup_q_immersed_nodes restated: node order, boxes, nearest-
    node fallbacks, Dirichlet and Neumann (Gauss-Jordan) coefficients"""
    z = np.load(os.path.join(HERE, "golden", "geom", "geom_%s.npz" % name))
    g = GEOM[name]().grid
    for q in "uvwc":
        ib = G.immersed(g, q, z["ref_sdf_" + q], z["ref_status_" + q])
        for k in ("im", "nf", "fidx", "fcoef", "bcoef", "pts"):
            assert np.array_equal(ib[k], z["ref_ib_%s_%s" % (q, k)]), (q, k)
