"""Pressure-Poisson solves alone (the mixed-precision solve of the
128^3 uniform and 256x128x128 y-stretched boxes with Neumann walls).

Right-hand sides are b = -div(u)/dt of seeded random-Fourier-mode velocities
(wave vectors 1 <= |k| <= 8, amplitude |k|^-5/3, zero mean; seeds 0..63).
The mixed method (FP32 V-cycles inside FP64 CG) and the plain FP64 MG-CG both
iterate to relative residual 1e-10 from a zero pressure, and their
mean-removed solutions must agree within 1e-8 of the FP64 solution's largest
magnitude for every right-hand side (Pressure.c:443-458 solves the same
system with GMRES + BoomerAMG; Solver.c:90-265).  A small case pins both
methods to the oracle's exact discrete solution on the same family of
right-hand sides.
"""
import numpy as np
import pytest

from turbins_gb300 import workload as W


def _div(g, vel):
    """-div(u) per cell in index space (dt = 1, unit spacings): zero sum when
    the walls are impermeable"""
    u, v, w = vel["u"], vel["v"], vel["w"]
    d = (u[:-1, :-1, 1:] - u[:-1, :-1, :-1]) + (v[:-1, 1:, :-1] - v[:-1, :-1, :-1]) + \
        (w[1:, :-1, :-1] - w[:-1, :-1, :-1])
    return d


def test_fourier_velocity_properties():
    case = W.poisson_case(24, 16, 8, (16.0, 2.0, 2.0), 1.5)
    g = case.grid
    a = W.fourier_velocity(g, 3)
    b = W.fourier_velocity(g, 3)
    c = W.fourier_velocity(g, 4)
    for q in "uvw":
        assert a[q].flags["C_CONTIGUOUS"]
        assert np.array_equal(a[q], b[q])                       # seeded
        assert not np.array_equal(a[q], c[q])
        assert np.all(a[q][g.status[q] == W.BOUNDARY] == 0.0)   # impermeable walls
        assert np.isfinite(a[q]).all() and a[q].std() > 0.1
    d = _div(g, a)
    assert abs(d.sum()) <= 1e-9 * np.abs(d).sum()               # telescoping: zero net flux


def test_fourier_velocity_spectrum():
    """a single-seed field on a periodic-size uniform grid carries no energy
    above |k| = 8 and none at k = 0"""
    g = W.make_grid(32, 32, 32, (1.0, 1.0, 1.0))
    W.tag_status(g, None)
    f = W.fourier_velocity(g, 0)["w"]
    # the w nodes at z = zw[k] are periodic samples except the BOUNDARY ring;
    # take the interior block of cell-centred x and y, all 32 zw planes
    a = f[:32, :32, :32].copy()
    spec = np.abs(np.fft.fftn(a))
    k = np.fft.fftfreq(32) * 32
    KZ, KY, KX = np.meshgrid(k, k, k, indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    # x and y samples sit at cell centres (a phase shift only); the zeroed
    # BOUNDARY ring leaks a little, so compare energy fractions
    e = spec ** 2
    assert e[kk > 9].sum() <= 0.05 * e.sum()


@pytest.mark.gpu
def test_small_case_matches_oracle():
    """both methods against the oracle's exact discrete solve of the same
    right-hand side (32x16x16 y-stretched), mean-removed within 1e-8"""
    from oracle.oracle import Oracle
    from turbins_gb300 import build, poisson
    build.build()
    case = W.poisson_case(32, 16, 16, (16.0, 2.0, 2.0), 1.5)
    recs = poisson.solve_set(case, [5], keep=True)
    g = case.grid
    vel = W.fourier_velocity(g, 5)
    case.params.p_rtol = 1e-13
    o = Oracle(g, case.params)
    pb = o.pressure_rhs(1.0, vel["u"], vel["v"], vel["w"])
    ref, _, _ = o.pressure_solve(pb, np.zeros(g.shape))
    b = poisson._mean_removed(ref, g)
    for name in ("fp64", "mixed"):
        a = poisson._mean_removed(recs[0]["phi"][name], g)
        assert np.abs(a - b).max() <= 1e-8 * np.abs(b).max(), name
        assert recs[0][name]["relres"] <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ["cube128", "stretched256"])
def test_mixed_matches_fp64_on_64_rhs(shape):
    from turbins_gb300 import build, poisson
    build.build()
    (nx, ny, nz), lengths, q = poisson.SHAPES[shape]
    case = W.poisson_case(nx, ny, nz, lengths, q)
    recs = poisson.solve_set(case, range(64))
    assert len(recs) == 64
    for r in recs:
        assert r["fp64"]["relres"] <= 1e-10 and r["mixed"]["relres"] <= 1e-10, r
        assert r["rel_diff"] <= 1e-8, r
    s = poisson.summary(recs)
    print(shape, s)
