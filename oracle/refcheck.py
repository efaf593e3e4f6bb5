"""ctypes binding of oracle/_ref/libturbins_ref.so, the reference's own
routines compiled against the PETSc shim (TEST INFRASTRUCTURE ONLY).

Used to pin the CPU oracle and to regenerate tests/golden.  Includes the
restated line driver (the reference has none) expressed with the reference's
own ghost-cell routines and ENO_compute_convective_terms.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import refbuild

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_ubyte)


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def available():
    return os.path.exists(refbuild.LIB) or refbuild.available()


class Reference:
    def __init__(self, grid, params):
        lib = C.CDLL(refbuild.build())
        lib.ref_create.restype = C.c_void_p
        lib.ref_divergence.restype = C.c_double
        for f in ("ref_set_immersed", "ref_eno_line", "ref_cell_center", "ref_transpose", "ref_ghost_cells",
                  "ref_set_rhs_vel", "ref_set_rhs_conc", "ref_total_concentration", "ref_lhs_apply",
                  "ref_pressure_apply", "ref_pressure_rhs", "ref_project", "ref_divergence", "ref_metrics"):
            getattr(lib, f).argtypes = None
        self.lib = lib
        self.g = grid
        self.p = params
        self._keep = []
        st = [np.ascontiguousarray(grid.status[q], dtype=np.uint8) for q in "uvwc"]
        self._keep += st
        n = params.nconc
        pe = np.array(list(params.pe) + [0] * 4, dtype=np.float64)[:4]
        vs = np.array(list(params.vs0) + [0] * 4, dtype=np.float64)[:4]
        al = np.array(list(params.alpha) + [0] * 4, dtype=np.float64)[:4]
        ct = np.array(list(params.ctype) + [0] * 4, dtype=np.int32)[:4]
        co = [np.ascontiguousarray(getattr(grid, k), dtype=np.float64) for k in ("xc", "yc", "zc", "xu", "yv", "zw")]
        self._keep += co + [pe, vs, al, ct]
        self.h = C.c_void_p(lib.ref_create(C.c_int(grid.nx), C.c_int(grid.ny), C.c_int(grid.nz),
                                           *[_p(a) for a in co], *[_p(s, _up) for s in st],
                                           C.c_int(params.eno_order), C.c_double(params.re), C.c_int(n), _p(pe),
                                           _p(vs), _p(al), _p(ct, _ip), C.c_int(params.sedimentation)))
        for q in "uvwc":
            ib = grid.ib.get(q)
            if ib is None:
                continue
            arrs = [np.ascontiguousarray(ib["im"], dtype=np.int32), np.ascontiguousarray(ib["nf"], dtype=np.int32),
                    np.ascontiguousarray(ib["fidx"], dtype=np.int32), np.ascontiguousarray(ib["fcoef"], dtype=np.float64),
                    np.ascontiguousarray(ib["bcoef"], dtype=np.float64)]
            self._keep += arrs
            lib.ref_set_immersed(self.h, C.c_char(q.encode()), C.c_int(int(ib["n"])), _p(arrs[0], _ip),
                                 _p(arrs[1], _ip), _p(arrs[2], _ip), _p(arrs[3]), _p(arrs[4]))

    def _z(self):
        return np.zeros(self.g.shape)

    def metrics(self):
        g = self.g
        out = [np.zeros(g.nx + 1), np.zeros(g.ny + 1), np.zeros(g.nz + 1), np.zeros(g.nx + 1), np.zeros(g.ny + 1),
               np.zeros(g.nz + 1)]
        self.lib.ref_metrics(self.h, *[_p(a) for a in out])
        return dict(zip(("mxc", "myc", "mzc", "mxu", "myv", "mzw"), out))

    def eno_line(self, order, D0, P, V):
        D0, P, V = [np.ascontiguousarray(a, dtype=np.float64) for a in (D0, P, V)]
        out = np.zeros(len(D0))
        self.lib.ref_eno_line(self.h, C.c_int(order), C.c_int(len(D0)), _p(D0), _p(P), _p(V), _p(out))
        return out

    def cell_center(self, u, v, w):
        a, b, c = self._z(), self._z(), self._z()
        self.lib.ref_cell_center(self.h, _p(u), _p(v), _p(w), _p(a), _p(b), _p(c))
        return a, b, c

    def transpose(self, q, u, v, w):
        A, B = self._z(), self._z()
        self.lib.ref_transpose(self.h, C.c_char(q.encode()), _p(u), _p(v), _p(w), _p(A), _p(B))
        return A, B

    def set_rhs_vel(self, q, dt, x, conv, dp, ctot):
        b = self._z()
        self.lib.ref_set_rhs_vel(self.h, C.c_char(q.encode()), C.c_double(dt), _p(x), _p(conv), _p(dp), _p(ctot),
                                 _p(b))
        return b

    def set_rhs_conc(self, ic, dt, c, conv):
        b = self._z()
        self.lib.ref_set_rhs_conc(self.h, C.c_int(ic), C.c_double(dt), _p(c), _p(conv), _p(b))
        return b

    def total_concentration(self, cs):
        arr = (_dp * 4)()
        for i, c in enumerate(cs):
            arr[i] = _p(c)
        out = self._z()
        self.lib.ref_total_concentration(self.h, arr, _p(out))
        return out

    def _bed_shape(self, nc):
        return (nc, self.g.nz + 1, self.g.nx + 1)

    def interface_y_index(self):
        iy = np.zeros((self.g.nz + 1, self.g.nx + 1), dtype=np.int32)
        self.lib.ref_interface_y_index(self.h, iy.ctypes.data_as(C.POINTER(C.c_int)))
        return iy

    def deposit_integrate(self, cs, cs_old, dt, dep):
        """Conc_integrate_deposited_height of every fraction on dep (in place)"""
        a, b = (_dp * 4)(), (_dp * 4)()
        for i in range(len(cs)):
            a[i], b[i] = _p(cs[i]), _p(cs_old[i])
        assert dep.shape == self._bed_shape(len(cs)) and dep.flags.c_contiguous
        self.lib.ref_deposit_integrate(self.h, a, b, C.c_double(dt), _p(dep))
        return dep

    def resume_write(self, dirname, state, prim, grid=False, dep=None):
        """Resume_write_data / Resume_write_primary_data / Resume_write_2D_data
        of state (u, v, w, dpx, dpy, dpz, c0..) into dirname"""
        nc = self.p.nconc
        keys = ["u", "v", "w", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(nc)]
        arrs = [np.ascontiguousarray(state[k], dtype=np.float64) for k in keys]
        ptrs = (_dp * len(arrs))(*[_p(a) for a in arrs])
        dp = None if dep is None else _p(np.ascontiguousarray(dep))
        rc = self.lib.ref_resume_write(self.h, dirname.encode(), ptrs, C.c_int(int(grid)), C.c_double(prim["time"]),
                                       C.c_double(prim["dt"]), C.c_double(prim["dt_old"]), C.c_int(prim["iter"]),
                                       C.c_int(prim["output_iter"]), dp)
        assert rc == 0

    def resume_read(self, dirname, grid=False, dep=True):
        nc = self.p.nconc
        keys = ["u", "v", "w", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(nc)]
        arrs = [self._z() for _ in keys]
        ptrs = (_dp * len(arrs))(*[_p(a) for a in arrs])
        prim = np.zeros(5)
        d = np.zeros((nc, self.g.nz + 1, self.g.nx + 1)) if dep else None
        rc = self.lib.ref_resume_read(self.h, dirname.encode(), ptrs, C.c_int(int(grid)), _p(prim),
                                      None if d is None else _p(d))
        assert rc == 0
        out = dict(zip(keys, arrs))
        return out, dict(time=prim[0], dt=prim[1], dt_old=prim[2], iter=int(prim[3]), output_iter=int(prim[4])), d

    def diagnostics(self, u, v, w, cs, front_limit=0.01, dep=None):
        nc = len(cs)
        arr = (_dp * 4)()
        for i, c in enumerate(cs):
            arr[i] = _p(c)
        out = np.zeros(4 + 8 * nc)
        h = np.zeros((nc, self.g.nx + 1))
        sb = np.zeros(self._bed_shape(nc))
        dp = None if dep is None else _p(np.ascontiguousarray(dep))
        self.lib.ref_diagnostics(self.h, _p(u), _p(v), _p(w), arr, C.c_double(front_limit), dp, _p(out), _p(h),
                                 _p(sb))
        e = 4 + 4 * nc
        return dict(kinetic_energy=out[0], conversion_rate=out[1],
                    suspended_mass=[out[2 + 4 * i] for i in range(nc)],
                    potential_energy=[out[3 + 4 * i] for i in range(nc)],
                    stokes_dissipation=[out[4 + 4 * i] for i in range(nc)],
                    conversion_rate_c=[out[5 + 4 * i] for i in range(nc)],
                    front_location=out[2 + 4 * nc], viscous_dissipation=out[3 + 4 * nc],
                    ep_passive=[out[e + 4 * i] for i in range(nc)],
                    ep_passive_rate=[out[e + 1 + 4 * i] for i in range(nc)],
                    ep_rate=[out[e + 2 + 4 * i] for i in range(nc)],
                    sed_rate=[out[e + 3 + 4 * i] for i in range(nc)],
                    ave_height=h, sed_bottom=sb)

    def lhs_apply(self, q, ic, dt, x):
        y = self._z()
        self.lib.ref_lhs_apply(self.h, C.c_char(q.encode()), C.c_int(ic), C.c_double(dt),
                               _p(np.ascontiguousarray(x)), _p(y))
        return y

    def lhs_apply_dts(self, q, ic, dts, x):
        """A x after the reference's diagonal updates for the time steps dts
        in turn (matrix assembled once, as in a run whose dt changes)"""
        y = self._z()
        d = np.ascontiguousarray(dts, dtype=np.float64)
        self.lib.ref_lhs_apply_dts(self.h, C.c_char(q.encode()), C.c_int(ic), C.c_int(len(d)), _p(d),
                                   _p(np.ascontiguousarray(x)), _p(y))
        return y

    def pressure_apply(self, x):
        y = self._z()
        self.lib.ref_pressure_apply(self.h, _p(np.ascontiguousarray(x)), _p(y))
        return y

    def pressure_rhs(self, dt, u, v, w):
        b = self._z()
        self.lib.ref_pressure_rhs(self.h, C.c_double(dt), _p(u), _p(v), _p(w), _p(b))
        return b

    def project(self, dt, phi, pb, u, v, w, dpx, dpy, dpz):
        self.lib.ref_project(self.h, C.c_double(dt), _p(phi), _p(pb), _p(u), _p(v), _p(w), _p(dpx), _p(dpy), _p(dpz))

    def divergence(self, u, v, w):
        d = self._z()
        m = self.lib.ref_divergence(self.h, _p(u), _p(v), _p(w), _p(d))
        return m, d

    # -- open boundaries ----------------------------------------------------
    OPEN = {"in": 0, "out": 1, "out_old": 2}

    def set_open(self, inflow, outflow, U=1.0, transient=0, time_c=1.0):
        g = self.g
        self._open = (int(inflow), int(outflow))
        self.lib.ref_set_open(self.h, int(inflow), int(outflow), C.c_double(U), int(transient), C.c_double(time_c),
                              C.c_double(g.yv[-1] - g.yv[0]), C.c_double(g.zw[-1] - g.zw[0]))

    def _plane(self):
        return np.zeros((self.g.nz + 1, self.g.ny + 1))

    def open_set(self, which, q, ic, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.lib.ref_open_set(self.h, self.OPEN[which], C.c_char(q.encode()), int(ic), _p(a))

    def open_get(self, which, q, ic=0):
        a = self._plane()
        self.lib.ref_open_get(self.h, self.OPEN[which], C.c_char(q.encode()), int(ic), _p(a))
        return a

    def inflow_u(self, time):
        self.lib.ref_inflow_u.restype = C.c_double
        return self.lib.ref_inflow_u(self.h, C.c_double(time))

    def inflow_c(self, ic, time):
        self.lib.ref_inflow_c(self.h, int(ic), C.c_double(time))

    def outflow_impose(self, q, ic, dt, x, influx=0.0):
        self.lib.ref_outflow_impose(self.h, C.c_char(q.encode()), int(ic), C.c_double(dt),
                                    _p(np.ascontiguousarray(x)), C.c_double(influx))

    def outflow_store_old(self, q, ic=0):
        self.lib.ref_outflow_store_old(self.h, C.c_char(q.encode()), int(ic))

    def outflow_rk_average(self, q, ic, old_frac, new_frac):
        self.lib.ref_outflow_rk_average(self.h, C.c_char(q.encode()), int(ic), C.c_double(old_frac),
                                        C.c_double(new_frac))

    def outflow_to_plane(self, q, ic, should_set, x):
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        self.lib.ref_outflow_to_plane(self.h, C.c_char(q.encode()), int(ic), int(should_set), _p(x))
        return x

    def outflow_from_plane(self, q, ic, x):
        self.lib.ref_outflow_from_plane(self.h, C.c_char(q.encode()), int(ic), _p(np.ascontiguousarray(x)))

    def geometry(self, ipos):
        """the reference's geometry set-up from interface heights ipos
        [NZ][NX]: returns sdf of c, u, v, w and the status of u, v, w, c"""
        g = self.g
        ipos = np.ascontiguousarray(ipos, dtype=np.float64)
        sd = [self._z() for _ in range(4)]
        st = np.zeros((4,) + g.shape, dtype=np.uint8)
        self.lib.ref_geometry(self.h, _p(ipos), _p(sd[0]), _p(sd[1]), _p(sd[2]), _p(sd[3]),
                              st.ctypes.data_as(C.c_void_p))
        return dict(c=sd[0], u=sd[1], v=sd[2], w=sd[3]), dict(u=st[0], v=st[1], w=st[2], c=st[3])

    def immersed(self, q, cap=None):
        """the reference's stencils of quantity q from the current geometry
        (after geometry()): dict of im, nf, fidx [N,8], fcoef [N,8], bcoef,
        pts [N,12] (normal, control point, image point, node point)"""
        if cap is None:
            cap = self.g.npts
        im = np.zeros(cap, np.int32)
        nf = np.zeros(cap, np.int32)
        fidx = np.zeros((cap, 8), np.int32)
        fcoef = np.zeros((cap, 8))
        bcoef = np.zeros(cap)
        pts = np.zeros((cap, 12))
        n = self.lib.ref_immersed(self.h, C.c_char(q.encode()), cap, im.ctypes.data_as(C.c_void_p),
                                  nf.ctypes.data_as(C.c_void_p), fidx.ctypes.data_as(C.c_void_p), _p(fcoef),
                                  _p(bcoef), _p(pts))
        if n > cap:
            return self.immersed(q, n)
        return dict(n=n, im=im[:n], nf=nf[:n], fidx=fidx[:n], fcoef=fcoef[:n], bcoef=bcoef[:n], pts=pts[:n])

    def c_term(self, ct):
        """the buoyancy term at v nodes that Velocity_v_set_RHS computes
        (2-point y interpolation of the total concentration, Velocity.c:1861-
        1878) and then multiplies by 0.0 (Velocity.c:1883); the restated
        driver subtracts it at FLUID / BUFFER_SOLID v nodes"""
        g = self.g
        yc, yv = g.yc, g.yv
        c0, c1 = ct[:, :-1, :], ct[:, 1:, :]
        slope = (c1 - c0) / (yc[1:] - yc[:-1])[None, :, None]
        out = np.zeros_like(ct)
        out[:, 1:, :] = slope * (yv[1:] - yc[:-1])[None, :, None] + c0
        st = g.status["v"]
        return np.where((st == 3) | (st == 11), out, 0.0)

    def solve(self, q, ic, dt, b, x):
        """the reference's Velocity_solve / Conc_solve / Pressure_solve
        (q = 'u', 'v', 'w', 'c' or 'p') from initial guess x; returns
        (solution, iterations)"""
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        its = self.lib.ref_solve(self.h, C.c_char(q.encode()), C.c_int(ic), C.c_double(dt),
                                 _p(np.ascontiguousarray(b)), _p(x))
        return x, its

    def step(self, s, dt, time=None):
        """One TVD-RK2 step through the reference's routines, in the stage
        order of the restated driver (the oracle's to_step): store old; two
        stages of {cell centre, total concentration, convection of u, v, w
        and c_i, momentum RHS, u/v/w solves, concentration RHS and solves,
        pressure RHS, pressure solve, projection, divergence}; rk average
        (0.5, 0.5).  s: dict of DA arrays, updated in place; returns the
        per-stage divergence maxima."""
        p = self.p
        nc = p.nconc
        op = getattr(self, "_open", None)
        influx = 0.0
        if op and op[0]:
            influx = self.inflow_u(time)
            for ic in range(nc):
                self.inflow_c(ic, time)
        if op and op[1]:
            for q in "uvw":
                self.outflow_store_old(q)
            for ic in range(nc):
                self.outflow_store_old("c", ic)
        old = {k: s[k].copy() for k in ["u", "v", "w"] + ["c%d" % i for i in range(nc)]}
        divs = []
        for stage in range(2):
            if op and op[1]:
                for q in "uvw":
                    self.outflow_impose(q, 0, dt, s[q], influx)
                for ic in range(nc):
                    self.outflow_impose("c", ic, dt, s["c%d" % ic])
            ub, vb, wb = self.cell_center(s["u"], s["v"], s["w"])
            cs = [s["c%d" % i] for i in range(nc)]
            ct = self.total_concentration(cs) if nc > 1 else s["c0"].copy()
            conv = {}
            A, B = self.transpose("u", s["u"], s["v"], s["w"])
            conv["u"] = self.convection("u", 0, s["u"], s["u"], A, B)
            A, B = self.transpose("v", s["u"], s["v"], s["w"])
            conv["v"] = self.convection("v", 0, s["v"], A, s["v"], B)
            A, B = self.transpose("w", s["u"], s["v"], s["w"])
            conv["w"] = self.convection("w", 0, s["w"], A, B, s["w"])
            for ic in range(nc):
                va = vb + p.vs0[ic] if p.ctype[ic] == 2 else vb
                conv["c%d" % ic] = self.convection("c", ic, s["c%d" % ic], ub, va, wb)
            bs = {q: self.set_rhs_vel(q, dt, s[q], conv[q], s[dk], ct)
                  for q, dk in (("u", "dpx"), ("v", "dpy"), ("w", "dpz"))}
            if p.buoyancy:
                bs["v"] = bs["v"] - self.c_term(ct)
            for q in "uvw":
                s[q], _ = self.solve(q, 0, dt, bs[q], s[q])
            for ic in range(nc):
                k = "c%d" % ic
                b = self.set_rhs_conc(ic, dt, s[k], conv[k])
                s[k], _ = self.solve("c", ic, dt, b, s[k])
            pb = self.pressure_rhs(dt, s["u"], s["v"], s["w"])
            s["phi"], _ = self.solve("p", 0, dt, pb, s["phi"])
            s["pb"] = pb
            self.project(dt, s["phi"], pb, s["u"], s["v"], s["w"], s["dpx"], s["dpy"], s["dpz"])
            divs.append(self.divergence(s["u"], s["v"], s["w"])[0])
        for k, a in old.items():
            s[k] = 0.5 * a + 0.5 * s[k]
        if op and op[1]:
            for q in "uvw":
                self.outflow_rk_average(q, 0, 0.5, 0.5)
            for ic in range(nc):
                self.outflow_rk_average("c", ic, 0.5, 0.5)
        return divs

    # -- restated line driver around the reference's ghost and ENO routines --
    def convection(self, q, ic, fld, vx, vy, vz):
        """conv = Vx dq/dx + Vy dq/dy + Vz dq/dz over full box lines of
        non-BOUNDARY nodes; ghosts filled by the reference routines."""
        g, r = self.g, self.p.eno_order
        nx, ny, nz = g.nx, g.ny, g.nz
        i0 = 1 if q == "u" else 0
        j0 = 1 if q == "v" else 0
        k0 = 1 if q == "w" else 0
        x, y, z = g.coords(q)
        conv = self._z()
        qc = C.c_char(q.encode())
        for d, (pos, s0, e0, vel) in enumerate(((x, i0, nx - 1, vx), (y, j0, ny - 1, vy), (z, k0, nz - 1, vz))):
            nint = e0 - s0 + 1
            nb = nint + 2 * r
            if d == 0:
                lines = [(None, j, k) for k in range(k0, nz) for j in range(j0, ny)]
            elif d == 1:
                lines = [(i, None, k) for k in range(k0, nz) for i in range(i0, nx)]
            else:
                lines = [(i, j, None) for j in range(j0, ny) for i in range(i0, nx)]
            for (i, j, k) in lines:
                sl = (slice(k, k + 1) if k is not None else slice(s0, e0 + 1),
                      slice(j, j + 1) if j is not None else slice(s0, e0 + 1),
                      slice(i, i + 1) if i is not None else slice(s0, e0 + 1))
                vals = fld[sl].ravel()
                vv = vel[sl].ravel()
                D0 = np.zeros(nb)
                P = np.zeros(nb)
                V = np.zeros(nb)
                D0[r:r + nint] = vals
                P[r:r + nint] = pos[s0:e0 + 1]
                V[r:r + nint] = vv
                # salinity top ghosts are never written by the reference:
                # pre-fill with the Neumann value (the restated driver's choice)
                D0[nb - r:] = vals[-1]
                ci = (i if i is not None else s0, j if j is not None else s0, k if k is not None else s0)
                ce = (i if i is not None else e0, j if j is not None else e0, k if k is not None else e0)
                self.lib.ref_ghost_cells(self.h, qc, C.c_int(ic), C.c_char(b"xyz"[d:d + 1]), C.c_int(ci[0]),
                                         C.c_int(ci[1]), C.c_int(ci[2]), C.c_int(ce[0]), C.c_int(ce[1]),
                                         C.c_int(ce[2]), C.c_int(nb), _p(D0), _p(P))
                out = self.eno_line(r, D0, P, V)[r:r + nint]
                if d == 0:
                    conv[sl] = out.reshape(conv[sl].shape)
                else:
                    conv[sl] = (conv[sl].ravel() + out).reshape(conv[sl].shape)
        return conv
