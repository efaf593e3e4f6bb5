"""Immersed-boundary geometry set-up of the reference, restated with numpy.

TEST INFRASTRUCTURE ONLY: the checker of the library's device geometry
set-up (turb_geometry); nothing in the product imports it.

For a bottom surface at heights h[k][i] (MAC_grid.interface_position):
* guess: phi_0 = yc[j] - h[k][i] at every DA point (Surface_initialize,
  Surface.c:96-191, Only_bottom_surface);
* Levelset_reinitialize (Levelset.c:85-151): phi = phi_0, phi_old = 0; each
  step one-sided differences Dx, Dy, Dz (Levelset_compute_derivatives,
  Levelset.c:154-258), one Godunov step on the cells i < NI, j < NJ, k < NK
  with the Russo-Smereka fix next to the interface (Levelset_do_Godunov,
  Levelset.c:265-497), the L2 change sqrt(sum |phi - phi_old|^2 dx dy dz)
  over every DA point (Levelset_is_converged, Levelset.c:500-578, summed in
  DA order), phi_old = phi; stop when the change is below 1e-5 or the counter
  passes max_iterations + 1 = 501; the fictitious time step is half the
  smallest cell width (Levelset.c:590-640); then the last planes copy their
  neighbours, x then y then z (Levelset.c:642-700);
* u/v/w sdf by 2-point interpolation from the c sdf (Surface_find_q_sdf,
  Surface.c:216-336, MyMath_interpolate_quantity MyMath.c:13-44);
* statuses (Grid_identify_geometry, Grid.c:1825-1870): box planes
  (Grid.c:1617-1672), FLUID / IMMERSED / SOLID from the sdf and its six
  neighbours with sign() on the back one (Grid.c:1424-1613), then
  BUFFER_SOLID for SOLID u/v/w nodes within +-2 of an IMMERSED node of the
  statuses before that pass, out-of-range indices OUTSIDE (Grid.c:2024-2160).
Every operation is a single IEEE double operation in the reference's order,
so the result is bit-identical to the reference compiled without
contraction.
"""
from __future__ import annotations

import numpy as np

SOLID, FLUID, IMMERSED, BOUNDARY, BUFFER_SOLID = 2, 3, 5, 7, 11


def cell_widths(f):
    """dx_c of Grid.c:633-671 from the face coordinates"""
    f = np.asarray(f, dtype=np.float64)
    d = np.zeros_like(f)
    d[1:-1] = f[2:] - f[1:-1]
    d[0] = f[1] - f[0]
    d[-1] = f[-1] - f[-2]
    return d


def face_metric(c, f, deta):
    """metric_xu of Grid_compute_metric_coefficients (Grid.c:595-708)"""
    n = len(c)
    m = np.zeros(n)
    m[1:n - 1] = deta / (c[1:n - 1] - c[0:n - 2])
    m[0] = 0.5 * deta / (c[0] - f[0])
    m[n - 1] = 0.5 * deta / (f[n - 1] - c[n - 2])
    return m


def reinitialize(g, ipos, max_iterations=500):
    """the c-node sdf and the number of Godunov steps"""
    xc, yc, zc = (np.asarray(a, dtype=np.float64) for a in (g.xc, g.yc, g.zc))
    NI, NJ, NK = g.nx, g.ny, g.nz
    NX, NY, NZ = NI + 1, NJ + 1, NK + 1
    dEta, dXi, dPhi = 1.0 / NI, 1.0 / NJ, 1.0 / NK
    a_dEta, a_dXi, a_dPhi = 1.0 / dEta, 1.0 / dXi, 1.0 / dPhi
    mxu = face_metric(xc, g.xu, dEta)
    myv = face_metric(yc, g.yv, dXi)
    mzw = face_metric(zc, g.zw, dPhi)
    dxc, dyc, dzc = cell_widths(g.xu), cell_widths(g.yv), cell_widths(g.zw)
    p0 = yc[None, :, None] - np.asarray(ipos, dtype=np.float64)[:, None, :]
    p = p0.copy()
    po = np.zeros_like(p)
    dmin = min(min(dxc[:NI].min(), 1000.0), min(dyc[:NJ].min(), 1000.0))
    dmin = min(dmin, min(dzc[:NK].min(), 1000.0))
    dt = 0.5 * dmin
    # neighbour index vectors
    ie = np.minimum(np.arange(NI) + 1, NI - 1); iw = np.maximum(np.arange(NI) - 1, 0)
    jn = np.minimum(np.arange(NJ) + 1, NJ - 1); js = np.maximum(np.arange(NJ) - 1, 0)
    kf = np.minimum(np.arange(NK) + 1, NK - 1); kb = np.maximum(np.arange(NK) - 1, 0)
    P0 = p0[:NK, :NJ, :NI]
    dx = dxc[:NI][None, None, :]
    dy = dyc[:NJ][None, :, None]
    dz = dzc[:NK][:, None, None]
    sign0 = P0 / np.sqrt(P0 * P0 + dx * dx)
    pe = p0[:NK, :NJ, ie]; pw = p0[:NK, :NJ, iw]
    pn = p0[:NK, jn, :NI]; ps = p0[:NK, js, :NI]
    pf = p0[kf, :NJ, :NI]; pb = p0[kb, :NJ, :NI]
    DX = (xc[ie] - xc[iw])[None, None, :]
    DY = (yc[jn] - yc[js])[None, :, None]
    DZ = (zc[kf] - zc[kb])[:, None, None]
    tol = 0.01
    near = ((P0 * pw < 0) | (P0 * pe < 0) | (P0 * pn < 0) | (P0 * ps < 0) | (P0 * pb < 0) | (P0 * pf < 0))
    with np.errstate(divide="ignore", invalid="ignore"):
        ddx = np.where(np.abs(DX) > tol, (pe - pw) / DX, 0.0)
        ddy = np.where(np.abs(DY) > tol, (pn - ps) / DY, 0.0)
        ddz = np.where(np.abs(DZ) > tol, (pf - pb) / DZ, 0.0)
    Dt = np.sqrt(ddx * ddx + ddy * ddy + ddz * ddz)
    Dt = np.where(Dt < tol, tol, Dt)
    Dd = P0 / Dt
    sgn = np.where(np.abs(sign0) < 1.0e-8, 0.0, np.where(sign0 > 0.0, 1.0, -1.0))
    Ds = np.sqrt(dx * dx + dy * dy + dz * dz)
    c = 0
    while True:
        Dx = np.empty_like(p); Dy = np.empty_like(p); Dz = np.empty_like(p)
        Dx[:, :, :NI - 1] = (p[:, :, 1:NI] - p[:, :, :NI - 1]) * mxu[:NI - 1] * a_dEta
        Dx[:, :, NI - 1:] = (p[:, :, NI - 1:] - p[:, :, NI - 2:NX - 1]) * mxu[NI - 2:NX - 1] * a_dEta
        Dy[:, :NJ - 1, :] = (p[:, 1:NJ, :] - p[:, :NJ - 1, :]) * myv[:NJ - 1, None] * a_dXi
        Dy[:, NJ - 1:, :] = (p[:, NJ - 1:, :] - p[:, NJ - 2:NY - 1, :]) * myv[NJ - 2:NY - 1, None] * a_dXi
        Dz[:NK - 1] = (p[1:NK] - p[:NK - 1]) * mzw[:NK - 1, None, None] * a_dPhi
        Dz[NK - 1:] = (p[NK - 1:] - p[NK - 2:NZ - 1]) * mzw[NK - 2:NZ - 1, None, None] * a_dPhi
        Dxp = Dx[:NK, :NJ, :NI]; Dxm = Dx[:NK, :NJ, iw]
        Dyp = Dy[:NK, :NJ, :NI]; Dym = Dy[:NK, js, :NI]
        Dzp = Dz[:NK, :NJ, :NI]; Dzm = Dz[kb, :NJ, :NI]
        ap, am = np.maximum(Dxm, 0.0), np.minimum(Dxm, 0.0)
        bp, bm = np.maximum(Dxp, 0.0), np.minimum(Dxp, 0.0)
        cp, cm = np.maximum(Dym, 0.0), np.minimum(Dym, 0.0)
        dp, dm = np.maximum(Dyp, 0.0), np.minimum(Dyp, 0.0)
        ep, em = np.maximum(Dzm, 0.0), np.minimum(Dzm, 0.0)
        fp, fm = np.maximum(Dzp, 0.0), np.minimum(Dzp, 0.0)
        pos = sign0 > 0.0
        tx = np.where(pos, np.maximum(ap * ap, bm * bm), np.maximum(am * am, bp * bp))
        ty = np.where(pos, np.maximum(cp * cp, dm * dm), np.maximum(cm * cm, dp * dp))
        tz = np.where(pos, np.maximum(ep * ep, fm * fm), np.maximum(em * em, fp * fp))
        H = sign0 * (np.sqrt(tx + ty + tz) - 1.0)
        Hn = (sgn * np.abs(p[:NK, :NJ, :NI]) - Dd) / Ds
        H = np.where(near, Hn, H)
        p[:NK, :NJ, :NI] = p[:NK, :NJ, :NI] + (-H) * dt
        err = np.abs(p - po)
        e2 = err * err * dxc[None, None, :] * dyc[None, :, None] * dzc[:, None, None]
        W = np.sqrt(np.cumsum(e2.ravel())[-1])
        po = p.copy()
        if c > max_iterations + 1 or W < 1.0e-5:
            break
        c += 1
    p[:, :, NX - 1] = p[:, :, NX - 2]
    p[:, NY - 1, :] = p[:, NY - 2, :]
    p[NZ - 1] = p[NZ - 2]
    return p, c + 1


def _interp2(q0, x0, q1, x1, x):
    with np.errstate(divide="ignore", invalid="ignore"):
        m = (q1 - q0) / (x1 - x0)
        return np.where(np.abs(x1 - x0) < 1.0e-8, q0, m * (x - x0) + q0)


def q_sdf(g, c):
    xc, yc, zc = g.xc, g.yc, g.zc
    u = np.empty_like(c); v = np.empty_like(c); w = np.empty_like(c)
    u[:, :, 1:] = _interp2(c[:, :, 1:], xc[1:], c[:, :, :-1], xc[:-1], g.xu[1:])
    u[:, :, 0] = _interp2(c[:, :, 0], xc[0], c[:, :, 0], xc[0], g.xu[0])
    v[:, 1:, :] = _interp2(c[:, 1:, :], yc[1:, None], c[:, :-1, :], yc[:-1, None], g.yv[1:, None])
    v[:, 0, :] = _interp2(c[:, 0, :], yc[0], c[:, 0, :], yc[0], g.yv[0])
    w[1:] = _interp2(c[1:], zc[1:, None, None], c[:-1], zc[:-1, None, None], g.zw[1:, None, None])
    w[0] = _interp2(c[0], zc[0], c[0], zc[0], g.zw[0])
    return u, v, w


def tag(g, q, s):
    NI, NJ, NK = g.nx, g.ny, g.nz
    st = np.zeros(s.shape, dtype=np.uint8)
    i0 = 1 if q == "u" else 0
    j0 = 1 if q == "v" else 0
    k0 = 1 if q == "w" else 0
    ii = np.arange(i0, NI); jj = np.arange(j0, NJ); kk = np.arange(k0, NK)
    sub = np.s_[k0:NK, j0:NJ, i0:NI]
    sp = s[sub]
    se = s[k0:NK, j0:NJ][:, :, np.minimum(ii + 1, NI - 1)]
    sw = s[k0:NK, j0:NJ][:, :, np.maximum(ii - 1, 0)]
    sn = s[k0:NK][:, np.minimum(jj + 1, NJ - 1)][:, :, i0:NI]
    ss = s[k0:NK][:, np.maximum(jj - 1, 0)][:, :, i0:NI]
    sf = s[np.minimum(kk + 1, NK - 1)][:, j0:NJ, i0:NI]
    sb = np.sign(s[np.maximum(kk - 1, 0)][:, j0:NJ, i0:NI])
    imm = (sp * se < 0) | (sp * sw < 0) | (sp * sn < 0) | (sp * ss < 0) | (sp * sb < 0) | (sp * sf < 0)
    st[sub] = np.where(sp >= 0.0, FLUID, np.where(imm, IMMERSED, SOLID))
    st[:, :, -1] = BOUNDARY; st[:, -1, :] = BOUNDARY; st[-1] = BOUNDARY
    if q == "u":
        st[:, :, 0] = BOUNDARY
    if q == "v":
        st[:, 0, :] = BOUNDARY
    if q == "w":
        st[0] = BOUNDARY
    if q != "c":
        before = st.copy()
        imm = before == IMMERSED
        Z, Y, X = imm.shape
        near = np.zeros_like(imm)
        for dz in range(-2, 3):
            for dy in range(-2, 3):
                for dx in range(-2, 3):
                    src = imm[max(dz, 0):Z + min(dz, 0), max(dy, 0):Y + min(dy, 0), max(dx, 0):X + min(dx, 0)]
                    near[max(-dz, 0):Z + min(-dz, 0), max(-dy, 0):Y + min(-dy, 0), max(-dx, 0):X + min(-dx, 0)] |= src
        region = np.zeros_like(imm)
        region[sub] = True
        st[(before == SOLID) & near & region] = BUFFER_SOLID
    return st


def geometry(g, ipos):
    """(sdf dict c/u/v/w, status dict u/v/w/c, Godunov steps)"""
    c, n = reinitialize(g, ipos)
    u, v, w = q_sdf(g, c)
    sdf = dict(c=c, u=u, v=v, w=w)
    st = {q: tag(g, q, sdf[q]) for q in "uvwc"}
    return sdf, st, n


# ---- ghost-cell stencils (Immersed.c) ---------------------------------------
DIRX = (0, 1, 0, 1, 0, 1, 0, 1)
DIRY = (0, 0, 1, 1, 0, 0, 1, 1)
DIRZ = (0, 0, 0, 0, 1, 1, 1, 1)
NOT_FOUND, GVG_INF = -1, 10000000


def node_coords(g, q):
    """xq, yq, zq of Grid.c:1350-1370: u at (xu, yc, zc), v at (xc, yv, zc),
    w at (xc, yc, zw), c at the centres"""
    return (g.xu if q == "u" else g.xc, g.yv if q == "v" else g.yc, g.zw if q == "w" else g.zc)


def _bsearch(data, v, lo, hi):
    """MyMath_binary_search, MyMath.c:384-398"""
    while lo <= hi:
        mid = (lo + hi) // 2
        if v >= data[mid]:
            if v < data[mid + 1]:
                return mid
            lo = mid + 1
        elif v < data[mid]:
            hi = mid - 1
    return -1


def _index(a, v, n):
    """Grid_get_x_index / _y_ / _z_ (Grid.c:1877-1966) with n = NI / NJ / NK"""
    if v < a[0]:
        return NOT_FOUND
    if v > a[n - 1]:
        return GVG_INF
    return _bsearch(a, v, 0, n - 1)


def _dist(a, b):
    """MyMath_get_point_point_distance, MyMath.c:105-111"""
    dx, dy, dz = a[0] - b[0], a[1] - b[1], a[2] - b[2]
    return np.sqrt(dx * dx + dy * dy + dz * dz)


def _gauss_jordan(A):
    """MyMath_GaussJordan_matrix_inv (MyMath.c:117-195), full pivoting with
    the reference's tie rule (the last maximum) and operation order"""
    n = 8
    B = [list(map(float, r)) for r in A]
    piv = [-1] * n
    irow = [0] * n
    icol = [0] * n
    in_row = in_col = -1
    for i in range(n):
        mx = 0.0
        for j in range(n):
            if piv[j] != 0:
                for k in range(n):
                    if piv[k] == -1 and abs(B[j][k]) >= mx:
                        mx = abs(B[j][k])
                        in_row, in_col = j, k
        piv[in_col] += 1
        if in_row != in_col:
            B[in_row], B[in_col] = B[in_col], B[in_row]
        irow[i], icol[i] = in_row, in_col
        a = np.float64(1.0) / np.float64(B[in_col][in_col])
        B[in_col][in_col] = 1.0
        B[in_col] = [float(np.float64(x) * a) for x in B[in_col]]
        for hh in range(n):
            if hh != in_col:
                t = B[hh][in_col]
                B[hh][in_col] = 0.0
                B[hh] = [float(np.float64(B[hh][h]) - np.float64(B[in_col][h]) * np.float64(t)) for h in range(n)]
    for h in range(n - 1, -1, -1):
        if irow[h] != icol[h]:
            for k in range(n):
                B[k][irow[h]], B[k][icol[h]] = B[k][icol[h]], B[k][irow[h]]
    return B


def immersed(g, q, sdf, st):
    """Immersed_setup_q_immersed_nodes (Immersed.c:546-616) for quantity q
    from its sdf and status arrays ([NZ][NY][NX]): returns im, nf, fidx [N,8]
    and im/fidx as DA linear indices, fcoef [N,8], bcoef, pts [N,12]
    (normal, control point, image point, node point)."""
    f = np.float64
    NI, NJ, NK = g.nx, g.ny, g.nz
    NX, NY = NI + 1, NJ + 1
    xq, yq, zq = node_coords(g, q)
    dxc, dyc, dzc = cell_widths(g.xu), cell_widths(g.yv), cell_widths(g.zw)
    ni = NI + (q == "u"); nj = NJ + (q == "v"); nk = NK + (q == "w")

    def status(i, j, k):
        if i < 0 or i > NI or j < 0 or j > NJ or k < 0 or k > NK:
            return -1
        return int(st[k, j, i])

    def grad(i, j, k):
        iw, ie = max(i - 1, 0), min(i + 1, ni - 1)
        js, jn = max(j - 1, 0), min(j + 1, nj - 1)
        kb, kf = max(k - 1, 0), min(k + 1, nk - 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            return ((sdf[k, j, ie] - sdf[k, j, iw]) / (xq[ie] - xq[iw]),
                    (sdf[k, jn, i] - sdf[k, js, i]) / (yq[jn] - yq[js]),
                    (sdf[kf, j, i] - sdf[kb, j, i]) / (zq[kf] - zq[kb]))

    kk, jj, ii = np.nonzero(st == IMMERSED)   # DA order
    N = len(ii)
    im = ((kk * NY + jj) * NX + ii).astype(np.int32)
    nf = np.zeros(N, np.int32)
    fidx = np.zeros((N, 8), np.int32)
    fcoef = np.zeros((N, 8))
    bcoef = np.zeros(N)
    pts = np.zeros((N, 12))
    for t in range(N):
        i, j, k = int(ii[t]), int(jj[t]), int(kk[t])
        P = (f(xq[i]), f(yq[j]), f(zq[k]))
        # Surface_compute_normal, Surface.c:547-615
        gx, gy, gz = grad(i, j, k)
        an = f(1.0) / np.sqrt(gx * gx + gy * gy + gz * gz)
        n = (gx * an, gy * an, gz * an)
        # Surface_find_Dn_to_surface, Surface.c:475-541
        dn = n[0] * gx + n[1] * gy + n[2] * gz
        if abs(dn) < 1.0e-2 or np.isnan(dn):
            dn = f(1.0e-2)
        D = sdf[k, j, i] / dn
        C = (P[0] - n[0] * D, P[1] - n[1] * D, P[2] - n[2] * D)
        # Immersed_find_image_point, Immersed.c:1063-1150
        ds = _dist(P, C)
        D2 = f(2.0) * ds
        I = (P[0] + n[0] * D2, P[1] + n[1] * D2, P[2] + n[2] * D2)
        # Immersed_find_box, Immersed.c:1210-1402
        tx = max(f(0.005) * dxc[i], 1e-12)
        ty = max(f(0.005) * dyc[j], 1e-12)
        tz = max(f(0.005) * dzc[k], 1e-12)
        px = (tx, -tx, tx, -tx, tx, -tx, tx, -tx)
        py = (ty, ty, -ty, -ty, ty, ty, -ty, -ty)
        pz = (tz, tz, tz, tz, -tz, -tz, -tz, -tz)
        found = False
        m = 0
        while not found and m < 8:
            ig = _index(xq, I[0] + px[m], NI)
            jg = _index(yq, I[1] + py[m], NJ)
            kg = _index(zq, I[2] + pz[m], NK)
            good = True
            for gg in range(8):
                s = status(ig + DIRX[gg], jg + DIRY[gg], kg + DIRZ[gg])
                if s != FLUID and s != IMMERSED:
                    good = False
                    break
            found = good
            if found and not (xq[ig] <= I[0] <= xq[ig + 1] and yq[jg] <= I[1] <= yq[jg + 1]
                              and zq[kg] <= I[2] <= zq[kg + 1]):
                found = False
            m += 1
        box = []
        if found:
            box = [(ig + DIRX[gg], jg + DIRY[gg], kg + DIRZ[gg]) for gg in range(8)]
        else:
            ig = min(max(_index(xq, I[0], NI), 0), NI - 1)
            jg = min(max(_index(yq, I[1], NJ), 0), NJ - 1)
            kg = min(max(_index(zq, I[2], NK), 0), NK - 1)
            dmin, gf = 1e12, -1
            for gg in range(8):
                a, b, c = ig + DIRX[gg], jg + DIRY[gg], kg + DIRZ[gg]
                if status(a, b, c) == FLUID:
                    dd = _dist(I, (xq[a], yq[b], zq[c]))
                    if dd < dmin:
                        dmin, gf = dd, gg
            if gf >= 0:
                box = [(ig + DIRX[gf], jg + DIRY[gf], kg + DIRZ[gf])]
        nfl = len(box)
        # Immersed_compute_interpolation_coef, Immersed.c:122-376
        df = _dist(I, C)
        if abs(ds) <= 1e-10 and abs(df) <= 1e-10:
            coef = f(1.0)
        else:
            coef = ds / df
        fp = [(f(xq[a]), f(yq[b]), f(zq[c])) for a, b, c in box]
        w = [f(0.0)] * 8
        if nfl == 8:
            x7, y7, z7 = fp[7]
            x0, y0, z0 = fp[0]
            al = (x7 - I[0]) / (x7 - x0)
            be = (y7 - I[1]) / (y7 - y0)
            ga = (z7 - I[2]) / (z7 - z0)
            w = [al * be * ga, (1.0 - al) * be * ga, al * (1.0 - be) * ga, (1.0 - al) * (1.0 - be) * ga,
                 al * be * (1.0 - ga), (1.0 - al) * be * (1.0 - ga), al * (1.0 - be) * (1.0 - ga),
                 (1.0 - al) * (1.0 - be) * (1.0 - ga)]
        elif nfl == 1:
            w[0] = f(1.0)
        fc = [f(0.0)] * 8
        if q != "c":
            bc = f(1.0) + coef
            for gg in range(nfl):
                fc[gg] = w[gg] * coef
        elif nfl == 1:
            bc = -(ds + df)
            fc[0] = w[0] * f(-1.0)
        else:
            A = [[0.0] * 8 for _ in range(8)]
            selfin = False
            r = 0
            for gg in range(nfl):
                if box[gg] == (i, j, k):
                    selfin = True
                else:
                    x = fp[gg][0] - I[0]
                    y = fp[gg][1] - I[1]
                    z = fp[gg][2] - I[2]
                    A[r] = [x * y * z, x * y, x * z, y * z, x, y, z, 1.0]
                    r += 1
            if selfin:
                xc_, yc_, zc_ = C[0] - I[0], C[1] - I[1], C[2] - I[2]
                nx_, ny_, nz_ = n
                A[r] = [nx_ * yc_ * zc_ + ny_ * xc_ * zc_ + nz_ * xc_ * yc_, yc_ * nx_ + xc_ * ny_,
                        zc_ * nx_ + xc_ * nz_, zc_ * ny_ + yc_ * nz_, nx_, ny_, nz_, 0.0]
            with np.errstate(divide="ignore", invalid="ignore"):
                B = _gauss_jordan(A)
            rhs = f(B[7][7]) if selfin else f(0.0)
            bc = -(ds + df) + rhs
            r = 0
            for gg in range(nfl):
                if box[gg] == (i, j, k):
                    fc[gg] = f(0.0)
                else:
                    fc[gg] = -f(B[7][r])
                    r += 1
        for gg in range(nfl):
            if np.isnan(fc[gg]) or np.isinf(fc[gg]):
                fc[gg] = f(0.0)
                bc = f(0.0)
        nf[t] = nfl
        for gg in range(nfl):
            a, b, c = box[gg]
            fidx[t, gg] = (c * NY + b) * NX + a
            fcoef[t, gg] = fc[gg]
        bcoef[t] = bc
        pts[t] = (n[0], n[1], n[2], C[0], C[1], C[2], I[0], I[1], I[2], P[0], P[1], P[2])
    return dict(n=N, im=im, nf=nf, fidx=fidx, fcoef=fcoef, bcoef=bcoef, pts=pts)
