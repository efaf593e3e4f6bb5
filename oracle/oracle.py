"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle (turb_oracle.c) is the checker for the CUDA path and the timed CPU
baseline; only tests/, __graft_entry__.smoke() and bench.py's CPU legs load it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libturb_oracle.so")
MAXC = 4

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


def build(force=False):
    """Compile turb_oracle.c with the reference's rounding rules (no FMA
    contraction, no fast-math)."""
    src = os.path.join(HERE, "turb_oracle.c")
    deps = [src, os.path.join(HERE, "turb_oracle.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in deps):
        return LIB
    base = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-o", LIB + ".tmp", src]
    try:
        subprocess.check_call(base + ["-fopenmp", "-lm"])
    except subprocess.CalledProcessError:
        subprocess.check_call(base + ["-lm"])      # no OpenMP: the loops run serially
    os.replace(LIB + ".tmp", LIB)
    return LIB


_LOADED = None


def _lib():
    """the oracle library, loaded once; its parallel loops start with
    TURB_ORACLE_THREADS threads (default 1)"""
    global _LOADED
    if _LOADED is None:
        _LOADED = C.CDLL(build())
        _LOADED.to_set_threads(int(os.environ.get("TURB_ORACLE_THREADS", "1")))
    return _LOADED


def set_threads(n):
    """threads of the oracle's parallel loops (results are the same bits for
    any count)"""
    _lib().to_set_threads(int(n))


class _Params(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("eno_order", C.c_int),
                ("re", C.c_double), ("nconc", C.c_int), ("pe", C.c_double * MAXC),
                ("vs0", C.c_double * MAXC), ("alpha", C.c_double * MAXC), ("ctype", C.c_int * MAXC),
                ("sedimentation", C.c_int), ("wall_noslip", C.c_int * 6), ("buoyancy", C.c_int),
                ("vel_rtol", C.c_double), ("vel_maxit", C.c_int), ("p_rtol", C.c_double),
                ("p_maxit", C.c_int)]


class _IB(C.Structure):
    _fields_ = [("n", C.c_int), ("im", _ip), ("nf", _ip), ("fidx", _ip), ("fcoef", _dp), ("bcoef", _dp)]


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("NX", C.c_int), ("NY", C.c_int),
                ("NZ", C.c_int), ("dEta", C.c_double), ("dXi", C.c_double), ("dPhi", C.c_double)] + \
        [(n, _dp) for n in ("xc", "yc", "zc", "xu", "yv", "zw", "mxc", "myc", "mzc", "mxu", "myv", "mzw")] + \
        [("st", _u8p * 4), ("ib", _IB * 4)]


class _State(C.Structure):
    _fields_ = [(n, _dp) for n in ("u", "v", "w", "u_old", "v_old", "w_old", "phi", "dpx", "dpy", "dpz", "pb")] + \
        [("c", _dp * MAXC), ("c_old", _dp * MAXC)]


class _Stats(C.Structure):
    _fields_ = [("vel_iters", (C.c_int * 2) * 3), ("conc_iters", (C.c_int * 2) * MAXC),
                ("p_iters", C.c_int * 2), ("p_relres", C.c_double * 2), ("div_max", C.c_double * 2)]


def _ptr(a, t=_dp):
    """pointer to a C-contiguous array (a strided view would be read as if
    it were contiguous, so it is refused)"""
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("oracle arrays must be C-contiguous")
    return a.ctypes.data_as(t)


class _Diag(C.Structure):
    """to_diag / turb_diag"""
    _fields_ = [("ke", C.c_double), ("rate", C.c_double), ("mass", C.c_double * MAXC),
                ("ep", C.c_double * MAXC), ("stokes", C.c_double * MAXC), ("rate_c", C.c_double * MAXC),
                ("front", C.c_double), ("visc", C.c_double), ("epp", C.c_double * MAXC),
                ("epp_rate", C.c_double * MAXC), ("ep_rate", C.c_double * MAXC), ("sed", C.c_double * MAXC)]


def diag_dict(d, nc, h, sb):
    return dict(kinetic_energy=d.ke, conversion_rate=d.rate, suspended_mass=list(d.mass)[:nc],
                potential_energy=list(d.ep)[:nc], stokes_dissipation=list(d.stokes)[:nc],
                conversion_rate_c=list(d.rate_c)[:nc], front_location=d.front, viscous_dissipation=d.visc,
                ep_passive=list(d.epp)[:nc], ep_passive_rate=list(d.epp_rate)[:nc], ep_rate=list(d.ep_rate)[:nc],
                sed_rate=list(d.sed)[:nc], ave_height=h, sed_bottom=sb)


class Oracle:
    """Holds one grid + parameter set in the oracle's C layout."""

    def __init__(self, grid, params):
        self.lib = _lib()
        L = self.lib
        L.to_divergence.restype = C.c_double
        self.g = grid
        self.p = params
        self._keep = []
        cg = _Grid()
        cg.nx, cg.ny, cg.nz = grid.nx, grid.ny, grid.nz
        cg.NX, cg.NY, cg.NZ = grid.nx + 1, grid.ny + 1, grid.nz + 1
        for n in ("xc", "yc", "zc", "xu", "yv", "zw"):
            a = np.ascontiguousarray(getattr(grid, n), dtype=np.float64)
            self._keep.append(a)
            setattr(cg, n, _ptr(a))
        self.metrics = {}
        for n, ln in (("mxc", cg.NX), ("myc", cg.NY), ("mzc", cg.NZ), ("mxu", cg.NX), ("myv", cg.NY), ("mzw", cg.NZ)):
            a = np.zeros(ln)
            self._keep.append(a)
            self.metrics[n] = a
            setattr(cg, n, _ptr(a))
        for qi, q in enumerate("uvwc"):
            st = np.ascontiguousarray(grid.status[q], dtype=np.uint8)
            self._keep.append(st)
            cg.st[qi] = _ptr(st, _u8p)
            ib = grid.ib.get(q)
            if ib is not None and ib["n"] > 0:
                arrs = [np.ascontiguousarray(ib[k]) for k in ("im", "nf", "fidx", "fcoef", "bcoef")]
                arrs[0] = arrs[0].astype(np.int32)
                arrs[1] = arrs[1].astype(np.int32)
                arrs[2] = np.ascontiguousarray(arrs[2].astype(np.int32))
                arrs[3] = np.ascontiguousarray(arrs[3].astype(np.float64))
                self._keep.extend(arrs)
                cg.ib[qi].n = int(ib["n"])
                cg.ib[qi].im = _ptr(arrs[0], _ip)
                cg.ib[qi].nf = _ptr(arrs[1], _ip)
                cg.ib[qi].fidx = _ptr(arrs[2], _ip)
                cg.ib[qi].fcoef = _ptr(arrs[3])
                cg.ib[qi].bcoef = _ptr(arrs[4])
            else:
                cg.ib[qi].n = 0
        self.cg = cg
        L.to_grid_metrics(C.byref(cg))
        cp = _Params()
        cp.nx, cp.ny, cp.nz = params.nx, params.ny, params.nz
        cp.eno_order = params.eno_order
        cp.re = params.re
        cp.nconc = params.nconc
        for i in range(params.nconc):
            cp.pe[i] = params.pe[i]
            cp.vs0[i] = params.vs0[i]
            cp.alpha[i] = params.alpha[i]
            cp.ctype[i] = params.ctype[i]
        cp.sedimentation = params.sedimentation
        for i in range(6):
            cp.wall_noslip[i] = params.wall_noslip[i]
        cp.buoyancy = params.buoyancy
        cp.vel_rtol, cp.vel_maxit = params.vel_rtol, params.vel_maxit
        cp.p_rtol, cp.p_maxit = params.p_rtol, params.p_maxit
        self.cp = cp

    # -- helpers ------------------------------------------------------------
    def _z(self):
        return np.zeros(self.g.shape)

    def cell_center(self, u, v, w):
        ubc, vbc, wbc = self._z(), self._z(), self._z()
        self.lib.to_cell_center(C.byref(self.cg), _ptr(u), _ptr(v), _ptr(w), _ptr(ubc), _ptr(vbc), _ptr(wbc))
        return ubc, vbc, wbc

    def transpose(self, which, u, v, w):
        A, B = self._z(), self._z()
        self.lib.to_transpose(C.byref(self.cg), C.c_char(which.encode()), _ptr(u), _ptr(v), _ptr(w), _ptr(A), _ptr(B))
        return A, B

    def convection_vel(self, which, q, vx, vy, vz):
        out = self._z()
        self.lib.to_convection_vel(C.byref(self.cg), C.byref(self.cp), C.c_char(which.encode()), _ptr(q),
                                   _ptr(vx), _ptr(vy), _ptr(vz), _ptr(out))
        return out

    def convection_conc(self, ic, c, ubc, vadv, wbc):
        out = self._z()
        self.lib.to_convection_conc(C.byref(self.cg), C.byref(self.cp), ic, _ptr(c), _ptr(ubc), _ptr(vadv),
                                    _ptr(wbc), _ptr(out))
        return out

    def eno_line(self, order, D0, P, V):
        out = np.zeros(len(D0))
        D0 = np.ascontiguousarray(D0, dtype=np.float64)
        P = np.ascontiguousarray(P, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        self.lib.to_eno_line(order, len(D0), _ptr(D0), _ptr(P), _ptr(V), _ptr(out))
        return out

    def set_rhs_vel(self, which, dt, q, conv, dp, ctot):
        b = self._z()
        self.lib.to_set_rhs_vel(C.byref(self.cg), C.byref(self.cp), C.c_char(which.encode()), C.c_double(dt),
                                _ptr(q), _ptr(conv), _ptr(dp), _ptr(ctot), _ptr(b))
        return b

    def set_rhs_conc(self, dt, c, conv):
        b = self._z()
        self.lib.to_set_rhs_conc(C.byref(self.cg), C.c_double(dt), _ptr(c), _ptr(conv), _ptr(b))
        return b

    def helmholtz_apply(self, which, ic, dt, x):
        y = self._z()
        self.lib.to_helmholtz_apply(C.byref(self.cg), C.byref(self.cp), C.c_char(which.encode()), ic,
                                    C.c_double(dt), _ptr(x), _ptr(y))
        return y

    def helmholtz_solve(self, which, ic, dt, b, x0, method=0):
        x = np.array(x0, dtype=np.float64, copy=True)
        rr = C.c_double()
        it = self.lib.to_helmholtz_solve(C.byref(self.cg), C.byref(self.cp), C.c_char(which.encode()), ic,
                                         C.c_double(dt), _ptr(np.ascontiguousarray(b)), _ptr(x), method, C.byref(rr))
        return x, it, rr.value

    def pressure_rhs(self, dt, u, v, w):
        b = self._z()
        self.lib.to_pressure_rhs(C.byref(self.cg), C.c_double(dt), _ptr(u), _ptr(v), _ptr(w), _ptr(b))
        return b

    def pressure_apply(self, x):
        y = self._z()
        self.lib.to_pressure_apply(C.byref(self.cg), _ptr(np.ascontiguousarray(x)), _ptr(y))
        return y

    def pressure_solve(self, b, phi0):
        phi = np.array(phi0, dtype=np.float64, copy=True)
        rr = C.c_double()
        it = self.lib.to_pressure_solve(C.byref(self.cg), C.byref(self.cp), _ptr(np.ascontiguousarray(b)),
                                        _ptr(phi), C.byref(rr))
        return phi, it, rr.value

    def project(self, dt, phi, b, u, v, w, dpx, dpy, dpz):
        self.lib.to_project(C.byref(self.cg), C.byref(self.cp), C.c_double(dt), _ptr(phi), _ptr(b), _ptr(u),
                            _ptr(v), _ptr(w), _ptr(dpx), _ptr(dpy), _ptr(dpz))

    def divergence(self, u, v, w):
        d = self._z()
        mx = self.lib.to_divergence(C.byref(self.cg), _ptr(u), _ptr(v), _ptr(w), _ptr(d))
        return mx, d

    def total_concentration(self, cs):
        out = self._z()
        arr = (_dp * MAXC)()
        for i, c in enumerate(cs):
            arr[i] = _ptr(c)
        self.lib.to_total_concentration(C.byref(self.cg), C.byref(self.cp), arr, _ptr(out))
        return out

    def _bed_shape(self):
        return (self.p.nconc, self.g.nz + 1, self.g.nx + 1)

    def interface_y_index(self):
        """to_interface_y_index: [NZ][NX] bed index (-1: none)"""
        iy = np.zeros((self.g.nz + 1, self.g.nx + 1), dtype=np.int32)
        self.lib.to_interface_y_index(C.byref(self.cg), iy.ctypes.data_as(C.c_void_p))
        return iy

    def deposit_integrate(self, cs, cs_old, dt, dep, iy=None):
        """to_deposit_integrate on dep (nconc x NZ x NX) in place"""
        iy = self.interface_y_index() if iy is None else iy
        a, b = (_dp * MAXC)(), (_dp * MAXC)()
        for i in range(len(cs)):
            a[i], b[i] = _ptr(cs[i]), _ptr(cs_old[i])
        assert dep.shape == self._bed_shape() and dep.flags.c_contiguous
        self.lib.to_deposit_integrate(C.byref(self.cg), C.byref(self.cp), iy.ctypes.data_as(C.c_void_p), a, b,
                                      C.c_double(dt), _ptr(dep))
        return dep

    def diagnostics(self, u, v, w, cs, front_limit=0.01, dep=None):
        """to_diagnostics: dict of the flow integrals, the h(x) profiles and
        the bed sedimentation rates"""
        d = _Diag()
        arr = (_dp * MAXC)()
        for i, c in enumerate(cs):
            arr[i] = _ptr(c)
        nc = self.p.nconc
        h = np.zeros((nc, self.g.nx + 1))
        sb = np.zeros(self._bed_shape())
        iy = self.interface_y_index()
        dp = None if dep is None else _ptr(np.ascontiguousarray(dep))
        self.lib.to_diagnostics(C.byref(self.cg), C.byref(self.cp), _ptr(u), _ptr(v), _ptr(w), arr,
                                C.c_double(front_limit), iy.ctypes.data_as(C.c_void_p), dp, C.byref(d), _ptr(h),
                                _ptr(sb))
        return diag_dict(d, nc, h, sb)

    def step(self, state, dt):
        """One TVD-RK2 step in place on a dict of DA arrays."""
        n = self.p.nconc
        cs = _State()
        olds = {}
        for k in ("u", "v", "w", "phi", "dpx", "dpy", "dpz"):
            setattr(cs, k, _ptr(state[k]))
        for k in ("u", "v", "w"):
            olds[k] = self._z()
            setattr(cs, k + "_old", _ptr(olds[k]))
        pb = state.setdefault("pb", self._z())
        cs.pb = _ptr(pb)
        for i in range(n):
            cs.c[i] = _ptr(state["c%d" % i])
            olds["c%d" % i] = self._z()
            cs.c_old[i] = _ptr(olds["c%d" % i])
        st = _Stats()
        self.lib.to_step(C.byref(self.cg), C.byref(self.cp), C.byref(cs), C.c_double(dt), C.byref(st))
        return dict(vel_iters=[list(st.vel_iters[i]) for i in range(3)],
                    conc_iters=[list(st.conc_iters[i]) for i in range(n)],
                    p_iters=list(st.p_iters), p_relres=list(st.p_relres), div_max=list(st.div_max))
