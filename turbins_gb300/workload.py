"""Host-side set-up of a TURBINS case: MAC grid coordinates, node status,
immersed-boundary stencils and initial conditions.

This is one-time set-up, not the per-step hot path.  It restates the
reference's set-up rules so that the arrays handed to the device (and to the
CPU oracle in the tests) have the reference's meaning:

* uniform coordinates by repeated addition, Grid.c:470-591;
* imported (stretched) y coordinates and the extrapolated half cell,
  Grid.c:1241-1378 (``Grid_y.inp`` layout: ny centres then ny+1 faces);
* one-sided tanh stretching of GridGenerator.c:390-393 for the y faces;
* box BOUNDARY tags, Grid.c:1617-1685; FLUID / IMMERSED / SOLID tags from the
  signed distance, Grid.c:1424-1613; BUFFER_SOLID layers of width 2 for u, v,
  w, Grid.c:1849-1856 and 2024-2160;
* the bed offset ``h(x,z) + 2.001*dy_c[0]``, Grid.c:913 and 1118;
* ghost-cell stencils: control point on the surface, image point at 2*ds along
  the normal (Immersed.c:1063-1149), an 8-node FLUID/IMMERSED box around the
  image point (Immersed.c:1210-1402) with trilinear weights, Dirichlet rows for
  u, v, w and Neumann rows for c (Immersed.c:122-374, 838-880).

The signed distance is computed from the analytic bed (first-order normal
distance) instead of the reference's level-set reinitialisation
(Levelset.c:85-160), so stencils follow the same construction but are not
bit-identical to the reference's set-up; the per-step parity tests feed the
same stencils to both the CUDA path and the oracle.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

FLUID, SOLID, IMMERSED, BOUNDARY, BUFFER_SOLID, OUTSIDE = 3, 2, 5, 7, 11, 1
SALINITY, PARTICLE = 1, 2
QUANTITIES = "uvwc"


@dataclass
class Params:
    """Physical and numerical parameters (the reference's ``Parameters``).

    ``vs0`` holds settling speeds after the sign flip of Input.c:481 (negative
    is downward); ``alpha`` holds the buoyancy weights after the rescale of
    Input.c:454-483.
    """
    nx: int
    ny: int
    nz: int
    eno_order: int = 3
    re: float = 2000.0
    nconc: int = 1
    pe: list = field(default_factory=lambda: [2000.0])
    vs0: list = field(default_factory=lambda: [0.0])
    alpha: list = field(default_factory=lambda: [1.0])
    ctype: list = field(default_factory=lambda: [SALINITY])
    sedimentation: int = 1
    wall_noslip: list = field(default_factory=lambda: [0, 0, 0, 0, 0, 0])
    buoyancy: int = 1
    vel_rtol: float = 1e-12
    vel_maxit: int = 200
    p_rtol: float = 1e-10
    p_maxit: int = 200


def rescale_alpha(alpha):
    """Input.c:454-483: alpha_i <- (alpha_i/alpha_0) / sum_j(alpha_j/alpha_0)."""
    et = sum(a / alpha[0] for a in alpha)
    return [(a / alpha[0]) / et for a in alpha]


def uniform_axis(n, lmin, length):
    """Grid_generate_mesh_coordinates (Grid.c:470-591): faces and centres by
    repeated addition of d = L * (1/n), n+1 entries each."""
    d = length * (1.0 / n)
    faces = np.empty(n + 1)
    cent = np.empty(n + 1)
    f = lmin
    c = lmin + 0.5 * d
    for i in range(n + 1):
        faces[i] = f
        cent[i] = c
        f += d
        c += d
    return cent, faces


def tanh_axis(n, lmin, length, q):
    """One-sided tanh stretching y = L (1 + tanh(Q(eta-1))/tanh Q)
    (GridGenerator.c:390-393), clustered at lmin: faces at eta = j/n,
    centres at eta = (j+1/2)/n, half cell extrapolated as Grid.c:1290."""
    eta_f = np.arange(n + 1) / n
    eta_c = (np.arange(n) + 0.5) / n
    faces = lmin + length * (1.0 + np.tanh(q * (eta_f - 1.0)) / np.tanh(q))
    cent = np.empty(n + 1)
    cent[:n] = lmin + length * (1.0 + np.tanh(q * (eta_c - 1.0)) / np.tanh(q))
    cent[n] = cent[n - 1] + (cent[n - 1] - cent[n - 2])
    faces[0] = lmin
    return cent, faces


@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    xc: np.ndarray
    yc: np.ndarray
    zc: np.ndarray
    xu: np.ndarray
    yv: np.ndarray
    zw: np.ndarray
    status: dict = field(default_factory=dict)   # q -> uint8 [NZ,NY,NX]
    ib: dict = field(default_factory=dict)       # q -> dict of stencil arrays

    @property
    def shape(self):
        return (self.nz + 1, self.ny + 1, self.nx + 1)

    @property
    def npts(self):
        return (self.nx + 1) * (self.ny + 1) * (self.nz + 1)

    def coords(self, q):
        """(x, y, z) node coordinates of quantity q (Grid.c:1366-1378 aliases)."""
        if q == "u":
            return self.xu, self.yc, self.zc
        if q == "v":
            return self.xc, self.yv, self.zc
        if q == "w":
            return self.xc, self.yc, self.zw
        return self.xc, self.yc, self.zc


def make_grid(nx, ny, nz, lengths, ystretch=None):
    lx, ly, lz = lengths
    xc, xu = uniform_axis(nx, 0.0, lx)
    zc, zw = uniform_axis(nz, 0.0, lz)
    if ystretch:
        yc, yv = tanh_axis(ny, 0.0, ly, ystretch)
    else:
        yc, yv = uniform_axis(ny, 0.0, ly)
    return Grid(nx, ny, nz, xc, yc, zc, xu, yv, zw)


def _box_boundary(g, q):
    st = np.zeros(g.shape, np.uint8)
    st[:, :, -1] = BOUNDARY
    st[:, -1, :] = BOUNDARY
    st[-1, :, :] = BOUNDARY
    if q == "u":
        st[:, :, 0] = BOUNDARY
    if q == "v":
        st[:, 0, :] = BOUNDARY
    if q == "w":
        st[0, :, :] = BOUNDARY
    return st


def _tag_ranges(g, q):
    i0 = 1 if q == "u" else 0
    j0 = 1 if q == "v" else 0
    k0 = 1 if q == "w" else 0
    return (k0, g.nz), (j0, g.ny), (i0, g.nx)


class Bed:
    """Bed elevation h(x, z) with analytic gradient."""

    def __init__(self, bumps, offset):
        self.bumps = bumps      # list of (height, width, xc, zc or None)
        self.offset = offset

    def h(self, x, z):
        out = np.full(np.broadcast(x, z).shape, self.offset)
        gx = np.zeros_like(out)
        gz = np.zeros_like(out)
        for hgt, wid, x0, z0 in self.bumps:
            r2 = (x - x0) ** 2 + (0.0 if z0 is None else (z - z0) ** 2)
            e = hgt * np.exp(-r2 / (2.0 * wid * wid))
            out = out + e
            gx = gx + e * (-(x - x0) / (wid * wid))
            if z0 is not None:
                gz = gz + e * (-(z - z0) / (wid * wid))
        return out, gx, gz

    def sdf(self, x, y, z):
        h, gx, gz = self.h(x, z)
        nrm = np.sqrt(1.0 + gx * gx + gz * gz)
        d = (y - h) / nrm
        return d, -gx / nrm, 1.0 / nrm, -gz / nrm


def tag_status(g, bed):
    """Node status for u, v, w, c (Grid_identify_geometry, Grid.c:1825-1871)."""
    for q in QUANTITIES:
        st = _box_boundary(g, q)
        (k0, k1), (j0, j1), (i0, i1) = _tag_ranges(g, q)
        if bed is None:
            st[k0:k1, j0:j1, i0:i1] = FLUID
        else:
            x, y, z = g.coords(q)
            X = x[None, None, :]
            Y = y[None, :, None]
            Z = z[:, None, None]
            s, _, _, _ = bed.sdf(X, Y, Z)
            s = np.broadcast_to(s, g.shape).copy()
            NI, NJ, NK = g.nx, g.ny, g.nz
            sub = np.s_[k0:k1, j0:j1, i0:i1]
            ii = np.arange(i0, i1)
            jj = np.arange(j0, j1)
            kk = np.arange(k0, k1)
            sp = s[sub]
            se = s[k0:k1, j0:j1, np.minimum(ii + 1, NI - 1)]
            sw = s[k0:k1, j0:j1, np.maximum(ii - 1, 0)]
            sn = s[k0:k1, np.minimum(jj + 1, NJ - 1), :][:, :, i0:i1]
            ss = s[k0:k1, np.maximum(jj - 1, 0), :][:, :, i0:i1]
            sf = s[np.minimum(kk + 1, NK - 1)][:, j0:j1, i0:i1]
            sb = np.sign(s[np.maximum(kk - 1, 0)][:, j0:j1, i0:i1])
            imm = ((sp * se < 0) | (sp * sw < 0) | (sp * sn < 0) | (sp * ss < 0)
                   | (sp * sb < 0) | (sp * sf < 0))
            tag = np.where(sp >= 0.0, FLUID, np.where(imm, IMMERSED, SOLID)).astype(np.uint8)
            st[sub] = tag
            if q != "c":
                _buffer_solid(st, sub, 2)
        g.status[q] = st


def _buffer_solid(st, sub, width):
    """Grid_tag_q_buffer_solid_nodes (Grid.c:2024-2160): SOLID nodes with an
    IMMERSED node within +-width in every direction become BUFFER_SOLID."""
    imm = (st == IMMERSED)
    nz, ny, nx = st.shape
    near = np.zeros_like(imm)
    for dz in range(-width, width + 1):
        for dy in range(-width, width + 1):
            for dx in range(-width, width + 1):
                src = imm[max(dz, 0):nz + min(dz, 0), max(dy, 0):ny + min(dy, 0), max(dx, 0):nx + min(dx, 0)]
                near[max(-dz, 0):nz + min(-dz, 0), max(-dy, 0):ny + min(-dy, 0), max(-dx, 0):nx + min(-dx, 0)] |= src
    region = np.zeros_like(imm)
    region[sub] = True
    st[(st == SOLID) & near & region] = BUFFER_SOLID


_DIRX = np.array([0, 1, 0, 1, 0, 1, 0, 1])
_DIRY = np.array([0, 0, 1, 1, 0, 0, 1, 1])
_DIRZ = np.array([0, 0, 0, 0, 1, 1, 1, 1])


def build_immersed(g, bed):
    """Ghost-cell stencils for every IMMERSED node of u, v, w (Dirichlet) and
    c (Neumann); arrays in the layout the C-ABI takes."""
    NX, NY = g.nx + 1, g.ny + 1
    for q in QUANTITIES:
        st = g.status[q]
        kk, jj, ii = np.nonzero(st == IMMERSED)
        n = len(ii)
        rec = dict(n=n, im=np.zeros(n, np.int32), nf=np.zeros(n, np.int32),
                   fidx=np.zeros((n, 8), np.int32), fcoef=np.zeros((n, 8)),
                   bcoef=np.zeros(n))
        if bed is None or n == 0:
            g.ib[q] = rec
            continue
        x, y, z = g.coords(q)
        px, py, pz = x[ii], y[jj], z[kk]
        d, nxv, nyv, nzv = bed.sdf(px, py, pz)
        ds = np.abs(d)
        cpx, cpy, cpz = px + nxv * ds, py + nyv * ds, pz + nzv * ds
        ipx, ipy, ipz = px + nxv * 2.0 * ds, py + nyv * 2.0 * ds, pz + nzv * 2.0 * ds
        i0 = np.clip(np.searchsorted(x, ipx, "right") - 1, 0, len(x) - 2)
        j0 = np.clip(np.searchsorted(y, ipy, "right") - 1, 0, len(y) - 2)
        k0 = np.clip(np.searchsorted(z, ipz, "right") - 1, 0, len(z) - 2)
        ci = i0[:, None] + _DIRX[None, :]
        cj = j0[:, None] + _DIRY[None, :]
        ck = k0[:, None] + _DIRZ[None, :]
        cst = st[ck, cj, ci]
        good = np.all((cst == FLUID) | (cst == IMMERSED), axis=1)
        lin = ((ck * NY) + cj) * NX + ci
        im_lin = ((kk * NY) + jj) * NX + ii
        rec["im"][:] = im_lin
        df = np.sqrt((ipx - cpx) ** 2 + (ipy - cpy) ** 2 + (ipz - cpz) ** 2)
        coef = np.where((ds <= 1e-10) & (df <= 1e-10), 1.0, ds / np.where(df > 0, df, 1.0))
        x0, x7 = x[i0], x[i0 + 1]
        y0, y7 = y[j0], y[j0 + 1]
        z0, z7 = z[k0], z[k0 + 1]
        al = (x7 - ipx) / (x7 - x0)
        be = (y7 - ipy) / (y7 - y0)
        ga = (z7 - ipz) / (z7 - z0)
        w = np.stack([al * be * ga, (1 - al) * be * ga, al * (1 - be) * ga, (1 - al) * (1 - be) * ga,
                      al * be * (1 - ga), (1 - al) * be * (1 - ga), al * (1 - be) * (1 - ga),
                      (1 - al) * (1 - be) * (1 - ga)], axis=1)
        # fallback: one fluid node (the FLUID corner closest to the image point,
        # else the FLUID node straight above the immersed node)
        bad = np.nonzero(~good)[0]
        for t in bad:
            cand = [m for m in range(8) if cst[t, m] == FLUID]
            if cand:
                dist = [(x[ci[t, m]] - ipx[t]) ** 2 + (y[cj[t, m]] - ipy[t]) ** 2 + (z[ck[t, m]] - ipz[t]) ** 2
                        for m in cand]
                m = cand[int(np.argmin(dist))]
                fi, fj, fk = ci[t, m], cj[t, m], ck[t, m]
            else:
                fi, fj, fk = ii[t], jj[t], kk[t]
                while fj < g.ny - 1 and st[fk, fj, fi] != FLUID:
                    fj += 1
            lin[t, :] = 0
            lin[t, 0] = ((fk * NY) + fj) * NX + fi
            w[t, :] = 0.0
            w[t, 0] = 1.0
        nf = np.where(good, 8, 1).astype(np.int32)
        rec["nf"][:] = nf
        rec["fidx"][:] = lin.astype(np.int32)
        if q != "c":
            rec["bcoef"][:] = 1.0 + coef
            rec["fcoef"][:] = w * coef[:, None]
        else:
            rec["bcoef"][:] = -(ds + df)
            fc = -w.copy()
            selfm = (lin == im_lin[:, None]) & good[:, None]
            rows = np.nonzero(selfm.any(axis=1))[0]
            for t in rows:
                # self-included box: the normal-derivative condition replaces
                # the immersed node's own equation (Immersed.c:262-330)
                A = np.zeros((8, 8))
                r = 0
                for m in range(8):
                    if selfm[t, m]:
                        continue
                    xr, yr, zr = x[ci[t, m]] - ipx[t], y[cj[t, m]] - ipy[t], z[ck[t, m]] - ipz[t]
                    A[r] = [xr * yr * zr, xr * yr, xr * zr, yr * zr, xr, yr, zr, 1.0]
                    r += 1
                xcn, ycn, zcn = cpx[t] - ipx[t], cpy[t] - ipy[t], cpz[t] - ipz[t]
                a, b, c = nxv[t], nyv[t], nzv[t]
                A[r] = [a * ycn * zcn + b * xcn * zcn + c * xcn * ycn, ycn * a + xcn * b, zcn * a + xcn * c,
                        zcn * b + ycn * c, a, b, c, 0.0]
                Ai = np.linalg.inv(A)
                rec["bcoef"][t] = -(ds[t] + df[t]) + Ai[7, 7]
                r = 0
                for m in range(8):
                    if selfm[t, m]:
                        fc[t, m] = 0.0
                    else:
                        fc[t, m] = -Ai[7, r]
                        r += 1
            fc[~good] = np.where(np.arange(8)[None, :] == 0, -1.0, 0.0)
            rec["fcoef"][:] = fc
            rec["bcoef"][~good] = -(ds[~good] + df[~good])
        g.ib[q] = rec


@dataclass
class Case:
    name: str
    grid: Grid
    params: Params
    dt: float
    steps: int
    state: dict
    bed: object = None     # Bed of an immersed-boundary case


def _lock_ic(g, params, seed, smooth=0.02, x_lock=1.0):
    """c = 1/2 (1 - tanh((x - x_lock)/smooth)) plus seeded U(-1e-3, 1e-3) noise
    where 0 < c < 1, clipped to [0, 1]; zero at non-fluid c nodes."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = g.shape
    c = np.broadcast_to(0.5 * (1.0 - np.tanh((g.xc[None, None, :] - x_lock) / smooth)), shape).copy()
    noise = rng.uniform(-1e-3, 1e-3, size=shape)
    m = (c > 0.0) & (c < 1.0)
    c[m] += noise[m]
    np.clip(c, 0.0, 1.0, out=c)
    st = g.status["c"]
    c[(st == BOUNDARY) | (st == SOLID)] = 0.0
    return c


def _zero_state(g, nconc):
    z = lambda: np.zeros(g.shape)  # noqa: E731
    s = {k: z() for k in ("u", "v", "w", "phi", "dpx", "dpy", "dpz")}
    for i in range(nconc):
        s["c%d" % i] = z()
    return s


def lock_exchange_case(nx=64, ny=32, nz=32, seed=0):
    """Plain-method lock exchange: uniform [0,8]x[0,1]x[0,1], Re=2000, Sc=1,
    salinity, ENO-2, free-slip walls, no immersed body, dt=1e-3, 100 steps."""
    g = make_grid(nx, ny, nz, (8.0, 1.0, 1.0))
    tag_status(g, None)
    build_immersed(g, None)
    p = Params(nx, ny, nz, eno_order=2, re=2000.0, nconc=1, pe=[2000.0], vs0=[0.0],
               alpha=[1.0], ctype=[SALINITY], p_rtol=1e-10)
    s = _zero_state(g, 1)
    s["c0"] = _lock_ic(g, p, seed)
    return Case("lock_exchange_%dx%dx%d" % (nx, ny, nz), g, p, 1e-3, 100, s)


def turbidity_bump_case(nx=256, ny=128, nz=128, seed=0):
    """Turbidity current over one immersed Gaussian bump (height 0.3, width 0.5
    at x=6) on [0,16]x[0,2]x[0,2], y-stretched (tanh, 1.5), Re=2000,
    settling 0.02, dt=5e-4."""
    g = make_grid(nx, ny, nz, (16.0, 2.0, 2.0), ystretch=1.5)
    dy0 = g.yv[1] - g.yv[0]
    bed = Bed([(0.3, 0.5, 6.0, None)], 2.001 * dy0)
    tag_status(g, bed)
    build_immersed(g, bed)
    p = Params(nx, ny, nz, eno_order=3, re=2000.0, nconc=1, pe=[2000.0], vs0=[-0.02],
               alpha=[1.0], ctype=[PARTICLE], p_rtol=1e-10)
    s = _zero_state(g, 1)
    s["c0"] = _lock_ic(g, p, seed)
    return Case("turbidity_bump_%dx%dx%d" % (nx, ny, nz), g, p, 5e-4, 200, s, bed)


def multi_bump_case(nx=512, ny=256, nz=256, seed=4, lx=32.0, lz=2.0, nbump=16):
    """Full coupled step: [0,32]x[0,2]x[0,2] y-stretched, 16 seeded Gaussian
    bumps (heights U[0.05,0.3], widths U[0.2,1.0], centres x U[4,28],
    z U[0,2]), two fractions settling at 0.005 and 0.02, Re=5000, dt=2.5e-4.
    lx, lz shrink the domain (bump centres scale with it) and nbump sets the
    number of bumps, for training runs at the full case's grid spacing."""
    g = make_grid(nx, ny, nz, (lx, 2.0, lz), ystretch=1.5)
    rng = np.random.Generator(np.random.PCG64(seed))
    hs = rng.uniform(0.05, 0.3, nbump)
    ws = rng.uniform(0.2, 1.0, nbump)
    xs = rng.uniform(4.0 * lx / 32.0, 28.0 * lx / 32.0, nbump)
    zs = rng.uniform(0.0, lz, nbump)
    dy0 = g.yv[1] - g.yv[0]
    bed = Bed([(hs[i], ws[i], xs[i], zs[i]) for i in range(nbump)], 2.001 * dy0)
    tag_status(g, bed)
    build_immersed(g, bed)
    p = Params(nx, ny, nz, eno_order=3, re=5000.0, nconc=2, pe=[5000.0, 5000.0],
               vs0=[-0.005, -0.02], alpha=rescale_alpha([1.0, 1.0]),
               ctype=[PARTICLE, PARTICLE], p_rtol=1e-10)
    s = _zero_state(g, 2)
    c = _lock_ic(g, p, seed)
    s["c0"] = c.copy()
    s["c1"] = c.copy()
    return Case("multi_bump_%dx%dx%d" % (nx, ny, nz), g, p, 2.5e-4, 500, s, bed)


def poisson_case(nx, ny, nz, lengths, ystretch=None):
    """Closed box with Neumann walls and no immersed body, for pressure
    solves alone (every c node FLUID except the BOUNDARY ring)."""
    g = make_grid(nx, ny, nz, lengths, ystretch=ystretch)
    tag_status(g, None)
    build_immersed(g, None)
    p = Params(nx, ny, nz, eno_order=2, re=2000.0, nconc=1, pe=[2000.0], vs0=[0.0], alpha=[1.0],
               ctype=[SALINITY], p_rtol=1e-10, p_maxit=400)
    return Case("poisson_%dx%dx%d%s" % (nx, ny, nz, "_ystretch" if ystretch else ""), g, p, 1.0, 0,
                _zero_state(g, 1))


def fourier_velocity(g, seed, kmax=8, slope=-5.0 / 3.0):
    """Seeded random-Fourier-mode velocity on the MAC grid: each component is
    Re sum_k C_k exp(2 pi i (kx x/Lx + ky y/Ly + kz z/Lz)) over the integer
    wave vectors 1 <= |k| <= kmax, C_k = |k|^slope (a + i b)/sqrt(2) with a, b
    standard normal (PCG64(seed)), evaluated at the component's own nodes and
    set to zero on its BOUNDARY nodes (impermeable walls, so the divergence
    sums to zero).  No k = 0 mode: zero mean.  Separable evaluation: one
    contraction per direction."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ks = np.arange(-kmax, kmax + 1)
    KZ, KY, KX = np.meshgrid(ks, ks, ks, indexing="ij")
    kk = np.sqrt(KX * KX + KY * KY + KZ * KZ)
    mask = (kk >= 1.0) & (kk <= kmax)
    amp = np.where(mask, np.where(mask, kk, 1.0) ** slope, 0.0)
    lx, ly, lz = g.xu[-1] - g.xu[0], g.yv[-1] - g.yv[0], g.zw[-1] - g.zw[0]
    out = {}
    for q in "uvw":
        cz = amp * (rng.standard_normal(amp.shape) + 1j * rng.standard_normal(amp.shape)) / np.sqrt(2.0)
        x, y, z = g.coords(q)
        ex = np.exp(2j * np.pi * np.outer(ks, (x - g.xu[0]) / lx))      # [k, NX]
        ey = np.exp(2j * np.pi * np.outer(ks, (y - g.yv[0]) / ly))      # [k, NY]
        ez = np.exp(2j * np.pi * np.outer((z - g.zw[0]) / lz, ks))      # [NZ, k]
        t1 = cz @ ex                                                    # [kz, ky, NX]
        t2 = np.einsum("jb,abi->aji", ey.T, t1)                         # [kz, NY, NX]
        n = len(ks)
        f = np.ascontiguousarray((ez @ t2.reshape(n, -1)).real.reshape(g.shape))
        f[g.status[q] == BOUNDARY] = 0.0
        out[q] = f
    return out
