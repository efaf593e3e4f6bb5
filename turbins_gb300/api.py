"""Python host binding of libturbgpu.so (the C ABI of include/turbins_gb300.h).

The host side mirrors the reference's routine interface: one ``Context``
holds what the reference spreads over GVG_bag, MAC_grid, Velocity, Pressure
and Concentration; its methods carry the reference routine names
(``Velocity_cell_center``, ``Pressure_solve`` ...) and raise ``TurbError``
where the reference would stop (PETScErrAct) or warn (Solver_is_converged).
There is no CPU fallback: without the CUDA library or a GPU every call fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import workload as W

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "lib", "libturbgpu.so")
MAXC = 4

F_U, F_V, F_W, F_PHI, F_DPX, F_DPY, F_DPZ, F_PB, F_DIV = range(9)
F_UBC, F_VBC, F_WBC, F_CONV_U, F_CONV_V, F_CONV_W, F_B_U, F_B_V, F_B_W, F_CTOT, F_SCRATCH0, F_SCRATCH1 = range(9, 21)
F_C0, F_CCONV0, F_CB0, F_VP0 = 32, 40, 48, 56
PMODE_FP64, PMODE_MIXED = 0, 1
HMODE_FP64, HMODE_MIXED = 0, 1
GUESS_PREVIOUS, GUESS_EXTRAPOLATE, GUESS_LEARNED, GUESS_PROJECT = 0, 1, 2, 3
KV_MARCHING, KV_ENO_SEGMENTS, KV_PDL, KV_CLUSTER_VCYCLE, KV_SWEEP_PAIRS = 1, 2, 4, 8, 16
HOST_COPY_DMA, HOST_COPY_KERNEL = 1, 2

STATUS = {0: "ok", 1: "bad argument", 2: "CUDA error", 3: "not converged", 4: "non-finite residual",
          5: "device allocation failed", 6: "scratch limit", 7: "restart file I/O", 8: "restart file mismatch"}
RESUME_GRID, RESUME_DEPOSIT, RESUME_PHI = 1, 2, 4


class TurbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


class _Params(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("eno_order", C.c_int),
                ("re", C.c_double), ("nconc", C.c_int), ("pe", C.c_double * MAXC),
                ("vs0", C.c_double * MAXC), ("alpha", C.c_double * MAXC), ("ctype", C.c_int * MAXC),
                ("sedimentation", C.c_int), ("wall_noslip", C.c_int * 6), ("buoyancy", C.c_int),
                ("vel_rtol", C.c_double), ("vel_maxit", C.c_int), ("p_rtol", C.c_double),
                ("p_maxit", C.c_int)]


class _IbDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("im", _ip), ("nf", _ip), ("fidx", _ip), ("fcoef", _dp), ("bcoef", _dp)]


class _GridDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int)] + \
        [(n, _dp) for n in ("xc", "yc", "zc", "xu", "yv", "zw")] + \
        [("status", _u8p * 4), ("ib", _IbDesc * 4)]


class StepStats(C.Structure):
    _fields_ = [("vel_iters", (C.c_int * 2) * 3), ("conc_iters", (C.c_int * 2) * MAXC),
                ("p_iters", C.c_int * 2), ("p_relres", C.c_double * 2), ("div_max", C.c_double * 2),
                ("kernel_launches", C.c_int)]

    def as_dict(self, nconc=1):
        return dict(vel_iters=[list(self.vel_iters[i]) for i in range(3)],
                    conc_iters=[list(self.conc_iters[i]) for i in range(nconc)],
                    p_iters=list(self.p_iters), p_relres=list(self.p_relres),
                    div_max=list(self.div_max), kernel_launches=self.kernel_launches)


_lib = None


def load_library():
    """Load the in-tree CUDA library; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise TurbError(2, "libturbgpu.so not built (run turbins_gb300.build.build())")
        L = C.CDLL(LIBPATH)
        L.turb_status_string.restype = C.c_char_p
        _lib = L
    return _lib


def _check(rc, what):
    if rc != 0:
        msg = load_library().turb_status_string(rc).decode()
        raise TurbError(rc, "%s: %s" % (what, msg))


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def params_struct(p: W.Params):
    cp = _Params()
    cp.nx, cp.ny, cp.nz = p.nx, p.ny, p.nz
    cp.eno_order = p.eno_order
    cp.re = p.re
    cp.nconc = p.nconc
    for i in range(p.nconc):
        cp.pe[i] = p.pe[i]
        cp.vs0[i] = p.vs0[i]
        cp.alpha[i] = p.alpha[i]
        cp.ctype[i] = p.ctype[i]
    cp.sedimentation = p.sedimentation
    for i in range(6):
        cp.wall_noslip[i] = p.wall_noslip[i]
    cp.buoyancy = p.buoyancy
    cp.vel_rtol, cp.vel_maxit = p.vel_rtol, p.vel_maxit
    cp.p_rtol, cp.p_maxit = p.p_rtol, p.p_maxit
    return cp


class Primary(C.Structure):
    """turb_primary: the scalars of Resume_primary.dat"""
    _fields_ = [("time", C.c_double), ("dt", C.c_double), ("dt_old", C.c_double), ("iter", C.c_int),
                ("output_iter", C.c_int)]

    @classmethod
    def of(cls, d):
        return cls(d["time"], d["dt"], d["dt_old"], int(d["iter"]), int(d["output_iter"]))

    def as_dict(self):
        return dict(time=self.time, dt=self.dt, dt_old=self.dt_old, iter=self.iter, output_iter=self.output_iter)


def petsc_vec_write(path, a):
    """a PETSc binary vector file (the reference's Resume_*.bin), no GPU needed"""
    a = np.ascontiguousarray(a, dtype=np.float64)
    _check(load_library().turb_petsc_vec_write(os.fsencode(path), _ptr(a), C.c_longlong(a.size)), "petsc_vec_write")


def petsc_vec_read(path, shape):
    a = np.zeros(shape)
    _check(load_library().turb_petsc_vec_read(os.fsencode(path), _ptr(a), C.c_longlong(a.size)), "petsc_vec_read")
    return a


def resume_primary_write(dirname, prim):
    _check(load_library().turb_resume_primary_write(os.fsencode(dirname), C.byref(Primary.of(prim))),
           "resume_primary_write")


def resume_primary_read(dirname):
    q = Primary()
    _check(load_library().turb_resume_primary_read(os.fsencode(dirname), C.byref(q)), "resume_primary_read")
    return q.as_dict()


def resume_2d_write(path, a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    nz, nx = a.shape
    _check(load_library().turb_resume_2d_write(os.fsencode(path), _ptr(a), nx, nz), "resume_2d_write")


def resume_2d_read(path, nz, nx):
    a = np.zeros((nz, nx))
    _check(load_library().turb_resume_2d_read(os.fsencode(path), _ptr(a), nx, nz), "resume_2d_read")
    return a


class _Diag(C.Structure):
    """turb_diag"""
    _fields_ = [("ke", C.c_double), ("rate", C.c_double), ("mass", C.c_double * MAXC),
                ("ep", C.c_double * MAXC), ("stokes", C.c_double * MAXC), ("rate_c", C.c_double * MAXC),
                ("front", C.c_double), ("visc", C.c_double), ("epp", C.c_double * MAXC),
                ("epp_rate", C.c_double * MAXC), ("ep_rate", C.c_double * MAXC), ("sed", C.c_double * MAXC)]


class Context:
    """Device-resident state of one case (turb_ctx)."""

    def __init__(self, grid: W.Grid, params: W.Params):
        L = load_library()
        self.lib = L
        self.grid = grid
        self.params = params
        keep = []
        gd = _GridDesc()
        gd.nx, gd.ny, gd.nz = grid.nx, grid.ny, grid.nz
        for n in ("xc", "yc", "zc", "xu", "yv", "zw"):
            a = np.ascontiguousarray(getattr(grid, n), dtype=np.float64)
            keep.append(a)
            setattr(gd, n, _ptr(a))
        for qi, q in enumerate("uvwc"):
            st = np.ascontiguousarray(grid.status[q], dtype=np.uint8)
            keep.append(st)
            gd.status[qi] = _ptr(st, _u8p)
            ib = grid.ib.get(q)
            if ib is not None and ib["n"] > 0:
                arrs = [np.ascontiguousarray(ib["im"], dtype=np.int32), np.ascontiguousarray(ib["nf"], dtype=np.int32),
                        np.ascontiguousarray(ib["fidx"], dtype=np.int32),
                        np.ascontiguousarray(ib["fcoef"], dtype=np.float64),
                        np.ascontiguousarray(ib["bcoef"], dtype=np.float64)]
                keep.extend(arrs)
                gd.ib[qi].n = int(ib["n"])
                gd.ib[qi].im, gd.ib[qi].nf, gd.ib[qi].fidx = _ptr(arrs[0], _ip), _ptr(arrs[1], _ip), _ptr(arrs[2], _ip)
                gd.ib[qi].fcoef, gd.ib[qi].bcoef = _ptr(arrs[3]), _ptr(arrs[4])
            else:
                gd.ib[qi].n = 0
        self._cp = params_struct(params)
        self.ctx = C.c_void_p()
        _check(L.turb_create(C.byref(gd), C.byref(self._cp), C.byref(self.ctx)), "turb_create")
        del keep

    def close(self):
        if self.ctx:
            self.lib.turb_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- transfer -------------------------------------------------------------
    def upload(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.size == self.grid.npts
        _check(self.lib.turb_field_upload(self.ctx, field, _ptr(a)), "upload")

    def download(self, field):
        a = np.empty(self.grid.shape)
        _check(self.lib.turb_field_download(self.ctx, field, _ptr(a)), "download")
        return a

    def set_host_copy(self, mode):
        """turb_set_host_copy: HOST_COPY_KERNEL (default: the layout kernel
        reads / writes page-locked host arrays in place) or HOST_COPY_DMA
        (staged copies on the copy engines)"""
        _check(self.lib.turb_set_host_copy(self.ctx, int(mode)), "set_host_copy")

    def upload_many(self, pairs):
        """turb_fields_upload: [(field, array), ...] in one overlapped call;
        the arrays must be C-contiguous float64 of the grid's shape"""
        n = len(pairs)
        f = (C.c_int * n)(*[int(fi) for fi, _ in pairs])
        for _, a in pairs:
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.grid.npts
        h = (C.c_void_p * n)(*[a.ctypes.data for _, a in pairs])
        _check(self.lib.turb_fields_upload(self.ctx, n, f, h), "fields_upload")

    def download_many(self, pairs):
        """turb_fields_download into [(field, array), ...] (C-contiguous
        float64 arrays of the grid's shape)"""
        n = len(pairs)
        f = (C.c_int * n)(*[int(fi) for fi, _ in pairs])
        for _, a in pairs:
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.grid.npts
        h = (C.c_void_p * n)(*[a.ctypes.data for _, a in pairs])
        _check(self.lib.turb_fields_download(self.ctx, n, f, h), "fields_download")

    def load_state(self, s):
        for k, f in (("u", F_U), ("v", F_V), ("w", F_W), ("phi", F_PHI), ("dpx", F_DPX), ("dpy", F_DPY),
                     ("dpz", F_DPZ)):
            if k in s:
                self.upload(f, s[k])
        for i in range(self.params.nconc):
            self.upload(F_C0 + i, s["c%d" % i])

    def state(self):
        out = {k: self.download(f) for k, f in (("u", F_U), ("v", F_V), ("w", F_W), ("phi", F_PHI), ("dpx", F_DPX),
                                                 ("dpy", F_DPY), ("dpz", F_DPZ), ("pb", F_PB))}
        for i in range(self.params.nconc):
            out["c%d" % i] = self.download(F_C0 + i)
        return out

    def set_pressure_mode(self, mode):
        _check(self.lib.turb_set_pressure_mode(self.ctx, mode), "set_pressure_mode")

    def set_pressure_guess(self, mode):
        _check(self.lib.turb_set_pressure_guess(self.ctx, mode), "set_pressure_guess")

    def reset_pressure_history(self):
        """turb_reset_pressure_history: the guesses forget earlier solutions"""
        _check(self.lib.turb_reset_pressure_history(self.ctx), "reset_pressure_history")

    def set_sweep_kernels(self, variants=KV_ENO_SEGMENTS | KV_PDL):
        """kernel variants (KV_MARCHING | KV_ENO_SEGMENTS | KV_PDL | KV_CLUSTER_VCYCLE | KV_SWEEP_PAIRS); all give the same bits"""
        _check(self.lib.turb_set_sweep_kernels(self.ctx, int(variants)), "set_sweep_kernels")

    def set_divergence_gate(self, max_div=1e-10):
        _check(self.lib.turb_set_divergence_gate(self.ctx, C.c_double(max_div)), "set_divergence_gate")

    def divergence_gate_count(self):
        n = C.c_longlong()
        _check(self.lib.turb_divergence_gate_count(self.ctx, C.byref(n)), "divergence_gate_count")
        return n.value

    def divergence_gate_floor_count(self):
        """solves the divergence gate let go at the residual's round-off floor"""
        n = C.c_longlong()
        _check(self.lib.turb_divergence_gate_floor_count(self.ctx, C.byref(n)), "divergence_gate_floor_count")
        return n.value

    def set_guess_galerkin(self, on=True):
        _check(self.lib.turb_set_guess_galerkin(self.ctx, 1 if on else 0), "set_guess_galerkin")

    def set_guess_stages(self, mask):
        _check(self.lib.turb_set_guess_stages(self.ctx, int(mask)), "set_guess_stages")

    def pressure_guess_stats(self):
        a, b = C.c_int(), C.c_int()
        _check(self.lib.turb_pressure_guess_stats(self.ctx, C.byref(a), C.byref(b)), "pressure_guess_stats")
        return a.value, b.value

    def set_mg_sweeps(self, npre, npost):
        _check(self.lib.turb_set_mg_sweeps(self.ctx, npre, npost), "set_mg_sweeps")

    def set_mg_tail(self, max_cells):
        """turb_set_mg_tail: single-block V-cycle below max_cells cells (0: off)"""
        _check(self.lib.turb_set_mg_tail(self.ctx, C.c_longlong(int(max_cells))), "set_mg_tail")

    def set_mg_cluster(self, max_cells):
        """turb_set_mg_cluster: one-cluster V-cycle below max_cells cells (0: off), with KV_CLUSTER_VCYCLE"""
        _check(self.lib.turb_set_mg_cluster(self.ctx, C.c_longlong(int(max_cells))), "set_mg_cluster")

    def set_mg_coarse_sweeps(self, from_level, npre, npost):
        """turb_set_mg_coarse_sweeps: levels >= from_level use npre / npost"""
        _check(self.lib.turb_set_mg_coarse_sweeps(self.ctx, int(from_level), int(npre), int(npost)),
               "set_mg_coarse_sweeps")

    def set_mg_split(self, on):
        """colour-split (True) or natural (False) storage of the FP32 multigrid levels"""
        _check(self.lib.turb_set_mg_split(self.ctx, int(bool(on))), "set_mg_split")

    def pressure_guess_ratio(self):
        r = C.c_double()
        _check(self.lib.turb_pressure_guess_ratio(self.ctx, C.byref(r)), "pressure_guess_ratio")
        return r.value

    def diagnostics(self, front_limit=0.01):
        """Flow integrals of the current state (turb_diagnostics): kinetic
        energy, conversion rates, viscous dissipation, and per fraction the
        suspended mass, potential energies, Stokes dissipation and
        sedimentation rate; front location (the reference's output path uses
        front_limit 0.01, Output.c:2131); spanwise-averaged heights h(x) and
        bed sedimentation rates."""
        d = _Diag()
        nc = self.params.nconc
        h = np.zeros((nc, self.grid.nx + 1))
        sb = np.zeros(self._bed_shape())
        _check(self.lib.turb_diagnostics(self.ctx, C.c_double(front_limit), C.byref(d), _ptr(h), _ptr(sb)),
               "diagnostics")
        return dict(kinetic_energy=d.ke, conversion_rate=d.rate, suspended_mass=list(d.mass)[:nc],
                    potential_energy=list(d.ep)[:nc], stokes_dissipation=list(d.stokes)[:nc],
                    conversion_rate_c=list(d.rate_c)[:nc], front_location=d.front, viscous_dissipation=d.visc,
                    ep_passive=list(d.epp)[:nc], ep_passive_rate=list(d.epp_rate)[:nc], ep_rate=list(d.ep_rate)[:nc],
                    sed_rate=list(d.sed)[:nc], ave_height=h, sed_bottom=sb)

    def _bed_shape(self):
        return (self.params.nconc, self.grid.nz + 1, self.grid.nx + 1)

    def bed_index(self):
        """turb_bed_index: [nz+1][nx+1] index of the bed node of each column (-1: none)"""
        iy = np.zeros((self.grid.nz + 1, self.grid.nx + 1), dtype=np.int32)
        _check(self.lib.turb_bed_index(self.ctx, iy.ctypes.data_as(C.c_void_p)), "bed_index")
        return iy

    def geometry(self, ipos):
        """turb_geometry: the device set-up of a bottom surface at heights
        ipos [nz+1][nx+1].  Returns (sdf, status, iterations): sdf of c, u, v,
        w and status of u, v, w, c as dicts of [nz+1][ny+1][nx+1] arrays"""
        g = self.grid
        shape = (g.nz + 1, g.ny + 1, g.nx + 1)
        ipos = np.ascontiguousarray(ipos, dtype=np.float64)
        if ipos.shape != (g.nz + 1, g.nx + 1):
            raise ValueError("ipos must be [nz+1][nx+1]")
        sd = [np.zeros(shape) for _ in range(4)]
        st = [np.zeros(shape, dtype=np.uint8) for _ in range(4)]
        sp = (C.c_void_p * 4)(*[a.ctypes.data for a in sd])
        tp = (C.c_void_p * 4)(*[a.ctypes.data for a in st])
        it = C.c_int(0)
        _check(self.lib.turb_geometry(self.ctx, ipos.ctypes.data_as(C.c_void_p), sp, tp, C.byref(it)), "geometry")
        return (dict(c=sd[0], u=sd[1], v=sd[2], w=sd[3]), dict(u=st[0], v=st[1], w=st[2], c=st[3]), it.value)

    def geometry_stencils(self, q):
        """turb_geometry_stencils: the ghost-cell stencils of quantity q
        ('u', 'v', 'w', 'c') made by the last geometry() call"""
        qi = "uvwc".index(q)
        n = C.c_int(0)
        _check(self.lib.turb_geometry_stencils(self.ctx, qi, C.byref(n), None, None, None, None, None, None),
               "geometry_stencils")
        n = n.value
        im = np.zeros(n, np.int32)
        nf = np.zeros(n, np.int32)
        fidx = np.zeros((n, 8), np.int32)
        fcoef = np.zeros((n, 8))
        bcoef = np.zeros(n)
        pts = np.zeros((n, 12))
        m = C.c_int(0)
        v = C.c_void_p
        _check(self.lib.turb_geometry_stencils(self.ctx, qi, C.byref(m), v(im.ctypes.data), v(nf.ctypes.data),
                                               v(fidx.ctypes.data), v(fcoef.ctypes.data), v(bcoef.ctypes.data),
                                               v(pts.ctypes.data)), "geometry_stencils")
        return dict(n=n, im=im, nf=nf, fidx=fidx, fcoef=fcoef, bcoef=bcoef, pts=pts)

    def deposit_integrate(self, dt):
        _check(self.lib.turb_deposit_integrate(self.ctx, C.c_double(dt)), "deposit_integrate")

    def deposit_enable(self, on=True):
        """integrate the deposited heights at the end of every step"""
        _check(self.lib.turb_deposit_enable(self.ctx, int(bool(on))), "deposit_enable")

    def deposit(self):
        out = np.zeros(self._bed_shape())
        _check(self.lib.turb_deposit_get(self.ctx, _ptr(out)), "deposit_get")
        return out

    def set_deposit(self, dep):
        dep = np.ascontiguousarray(dep, dtype=np.float64)
        if dep.shape != self._bed_shape():
            raise ValueError("deposit shape %s, expected %s" % (dep.shape, self._bed_shape()))
        _check(self.lib.turb_deposit_set(self.ctx, _ptr(dep)), "deposit_set")

    # -- open boundaries ----------------------------------------------------
    OPEN = {"in": 0, "out": 1, "out_old": 2}
    QIDX = {"u": 0, "v": 1, "w": 2, "c": 3}

    def set_open_boundaries(self, inflow, outflow, U=1.0, transient=False, time_c=1.0):
        _check(self.lib.turb_set_open_boundaries(self.ctx, int(bool(inflow)), int(bool(outflow)), C.c_double(U),
                                                 int(bool(transient)), C.c_double(time_c)), "set_open_boundaries")

    def open_plane(self, which, q, ic=0):
        a = np.zeros((self.grid.nz + 1, self.grid.ny + 1))
        _check(self.lib.turb_open_plane_get(self.ctx, self.OPEN[which], self.QIDX[q], int(ic), _ptr(a)),
               "open_plane_get")
        return a

    def set_open_plane(self, which, q, ic, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        _check(self.lib.turb_open_plane_set(self.ctx, self.OPEN[which], self.QIDX[q], int(ic), _ptr(a)),
               "open_plane_set")

    def Inflow_u_velocity_profile(self, time):
        f = C.c_double()
        _check(self.lib.turb_Inflow_u_velocity_profile(self.ctx, C.c_double(time), C.byref(f)), "inflow_u")
        return f.value

    def Inflow_conc_profile(self, ic, time):
        _check(self.lib.turb_Inflow_conc_profile(self.ctx, int(ic), C.c_double(time)), "inflow_c")

    def set_time(self, t):
        _check(self.lib.turb_set_time(self.ctx, C.c_double(t)), "set_time")

    def time(self):
        t = C.c_double()
        _check(self.lib.turb_get_time(self.ctx, C.byref(t)), "get_time")
        return t.value

    def set_influx(self, influx):
        _check(self.lib.turb_set_influx(self.ctx, C.c_double(influx)), "set_influx")

    def Outflow_vel_impose_convective_boundary(self, which, dt):
        _check(self.lib.turb_Outflow_vel_impose_convective_boundary(self.ctx, C.c_char(which.encode()),
                                                                    C.c_double(dt)), "outflow_vel")

    def Outflow_conc_impose_convective_boundary(self, ic, dt):
        _check(self.lib.turb_Outflow_conc_impose_convective_boundary(self.ctx, int(ic), C.c_double(dt)),
               "outflow_conc")

    def store_old_outflow(self):
        _check(self.lib.turb_store_old_outflow(self.ctx), "store_old_outflow")

    def rk_average_outflow(self, old_frac=0.5, new_frac=0.5):
        _check(self.lib.turb_rk_average_outflow(self.ctx, C.c_double(old_frac), C.c_double(new_frac)),
               "rk_average_outflow")

    def Outflow_copy_data_into_last_plane(self, which, ic, should_set):
        _check(self.lib.turb_Outflow_copy_data_into_last_plane(self.ctx, C.c_char(which.encode()), int(ic),
                                                               int(bool(should_set))), "copy_into_last_plane")

    def Outflow_copy_data_into_2D_array(self, which, ic):
        _check(self.lib.turb_Outflow_copy_data_into_2D_array(self.ctx, C.c_char(which.encode()), int(ic)),
               "copy_into_2d")

    def resume_write(self, dirname, prim, grid=False, deposit=False, phi=False):
        """turb_resume_write: the reference's restart set (+ options) into dirname"""
        flags = (RESUME_GRID if grid else 0) | (RESUME_DEPOSIT if deposit else 0) | (RESUME_PHI if phi else 0)
        _check(self.lib.turb_resume_write(self.ctx, os.fsencode(dirname), C.byref(Primary.of(prim)), flags),
               "resume_write")

    def resume_read(self, dirname, grid=False, deposit=False, phi=False):
        """turb_resume_read: state from a restart set; returns the primary scalars"""
        flags = (RESUME_GRID if grid else 0) | (RESUME_DEPOSIT if deposit else 0) | (RESUME_PHI if phi else 0)
        q = Primary()
        _check(self.lib.turb_resume_read(self.ctx, os.fsencode(dirname), C.byref(q), flags), "resume_read")
        return q.as_dict()

    def set_helmholtz_mode(self, mode, inner_sweeps=5):
        _check(self.lib.turb_set_helmholtz_mode(self.ctx, mode, inner_sweeps), "set_helmholtz_mode")

    def set_eno_division(self, fast):
        _check(self.lib.turb_set_eno_division(self.ctx, 1 if fast else 0), "set_eno_division")

    def synchronize(self):
        _check(self.lib.turb_synchronize(self.ctx), "synchronize")

    # -- reference routines -----------------------------------------------------
    def Velocity_cell_center(self):
        _check(self.lib.turb_Velocity_cell_center(self.ctx), "Velocity_cell_center")

    def Velocity_transpose_velocities(self, which):
        _check(self.lib.turb_Velocity_transpose_velocities(self.ctx, C.c_char(which.encode())),
               "Velocity_transpose_velocities")

    def Conc_compute_total_concentration(self):
        _check(self.lib.turb_Conc_compute_total_concentration(self.ctx), "Conc_compute_total_concentration")

    def Conc_set_particle_v_velocity(self, ic):
        _check(self.lib.turb_Conc_set_particle_v_velocity(self.ctx, ic), "Conc_set_particle_v_velocity")

    def Velocity_convective_terms(self, which):
        _check(self.lib.turb_Velocity_convective_terms(self.ctx, C.c_char(which.encode())), "convective_terms")

    def Conc_convective_terms(self, ic):
        _check(self.lib.turb_Conc_convective_terms(self.ctx, ic), "Conc_convective_terms")

    def Velocity_set_RHS(self, which, dt):
        _check(self.lib.turb_Velocity_set_RHS(self.ctx, C.c_char(which.encode()), C.c_double(dt)), "set_RHS")

    def Conc_set_RHS(self, ic, dt):
        _check(self.lib.turb_Conc_set_RHS(self.ctx, ic, C.c_double(dt)), "Conc_set_RHS")

    def Velocity_solve(self, which, dt):
        it = C.c_int()
        _check(self.lib.turb_Velocity_solve(self.ctx, C.c_char(which.encode()), C.c_double(dt), C.byref(it)),
               "Velocity_solve")
        return it.value

    def Conc_solve(self, ic, dt):
        it = C.c_int()
        _check(self.lib.turb_Conc_solve(self.ctx, ic, C.c_double(dt), C.byref(it)), "Conc_solve")
        return it.value

    def Pressure_set_RHS(self, dt):
        _check(self.lib.turb_Pressure_set_RHS(self.ctx, C.c_double(dt)), "Pressure_set_RHS")

    def Pressure_solve(self):
        it = C.c_int()
        rr = C.c_double()
        _check(self.lib.turb_Pressure_solve(self.ctx, C.byref(it), C.byref(rr)), "Pressure_solve")
        return it.value, rr.value

    def Pressure_project_velocity(self, dt):
        _check(self.lib.turb_Pressure_project_velocity(self.ctx, C.c_double(dt)), "Pressure_project_velocity")

    def Pressure_compute_velocity_divergence(self):
        d = C.c_double()
        _check(self.lib.turb_Pressure_compute_velocity_divergence(self.ctx, C.byref(d)), "divergence")
        return d.value

    def store_old_data(self):
        _check(self.lib.turb_store_old_data(self.ctx), "store_old_data")

    def rk_average(self, old_frac=0.5, new_frac=0.5):
        _check(self.lib.turb_rk_average(self.ctx, C.c_double(old_frac), C.c_double(new_frac)), "rk_average")

    def helmholtz_apply(self, which, ic, dt, fx, fy):
        _check(self.lib.turb_helmholtz_apply(self.ctx, C.c_char(which.encode()), ic, C.c_double(dt), fx, fy),
               "helmholtz_apply")

    def pressure_apply(self, fx, fy):
        _check(self.lib.turb_pressure_apply(self.ctx, fx, fy), "pressure_apply")

    def step(self, dt):
        """one step; on a solver failure the TurbError carries the step's
        statistics so far (iterations of every solve that ran) as .stats"""
        st = StepStats()
        rc = self.lib.turb_step(self.ctx, C.c_double(dt), C.byref(st))
        if rc != 0:
            try:
                _check(rc, "turb_step")
            except TurbError as e:
                e.stats = st.as_dict(self.params.nconc)
                raise
        return st.as_dict(self.params.nconc)

    def step_host(self, dt, pairs):
        """turb_step_host: upload [(field, array), ...], one step, download
        into the same arrays, with the late fields' copies overlapped"""
        n = len(pairs)
        f = (C.c_int * n)(*[int(fi) for fi, _ in pairs])
        for _, a in pairs:
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.grid.npts
        h = (C.c_void_p * n)(*[a.ctypes.data for _, a in pairs])
        st = StepStats()
        _check(self.lib.turb_step_host(self.ctx, C.c_double(dt), n, f, h, C.byref(st)), "turb_step_host")
        return st.as_dict(self.params.nconc)


def ENO_compute_convective_terms(order, D0, P, V):
    """ENO.c:103-245 on one host line, computed on the GPU."""
    L = load_library()
    D0 = np.ascontiguousarray(D0, dtype=np.float64)
    P = np.ascontiguousarray(P, dtype=np.float64)
    V = np.ascontiguousarray(V, dtype=np.float64)
    out = np.zeros(len(D0))
    _check(L.turb_ENO_compute_convective_terms(order, len(D0), _ptr(D0), _ptr(P), _ptr(V), _ptr(out)),
           "ENO_compute_convective_terms")
    return out


# ---- measurement helpers ------------------------------------------------------
PROF_GROUPS = ("eno_x", "eno_yz", "jacobi", "mg", "pcg", "inner32", "net")


def profile_enable(ctx, on=True):
    _check(ctx.lib.turb_profile_enable(ctx.ctx, 1 if on else 0), "profile_enable")


def profile_read(ctx):
    ms = (C.c_double * len(PROF_GROUPS))()
    nl = (C.c_longlong * len(PROF_GROUPS))()
    _check(ctx.lib.turb_profile_read(ctx.ctx, ms, nl), "profile_read")
    return {g: (ms[i], nl[i]) for i, g in enumerate(PROF_GROUPS)}


def event_record(ctx, slot):
    _check(ctx.lib.turb_event_record(ctx.ctx, slot), "event_record")


def event_elapsed(ctx, a, b):
    ms = C.c_double()
    _check(ctx.lib.turb_event_elapsed(ctx.ctx, a, b, C.byref(ms)), "event_elapsed")
    return ms.value


def kernel_launches(ctx):
    n = C.c_longlong()
    _check(ctx.lib.turb_kernel_launches(ctx.ctx, C.byref(n)), "kernel_launches")
    return n.value


def host_register(arr):
    _check(load_library().turb_host_register(C.c_void_p(arr.ctypes.data), C.c_size_t(arr.nbytes)), "host_register")


def host_unregister(arr):
    _check(load_library().turb_host_unregister(C.c_void_p(arr.ctypes.data)), "host_unregister")


class _PinnedBuffer:
    def __init__(self, nbytes):
        self.lib = load_library()
        self.ptr = C.c_void_p()
        _check(self.lib.turb_host_alloc(C.c_size_t(nbytes), C.byref(self.ptr)), "host_alloc")
        self.nbytes = nbytes

    def __del__(self):
        try:
            if self.ptr:
                self.lib.turb_host_free(self.ptr)
                self.ptr = C.c_void_p()
        except Exception:
            pass


def host_empty(shape, dtype=np.float64):
    """an uninitialised C-contiguous array in page-locked host memory
    (turb_host_alloc); the memory is released when the array is collected"""
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) * dt.itemsize
    buf = _PinnedBuffer(max(n, 1))
    raw = (C.c_char * buf.nbytes).from_address(buf.ptr.value)
    raw.owner = buf   # every view's base chain ends at raw, which keeps the memory
    return np.frombuffer(raw, dtype=dt, count=int(np.prod(shape))).reshape(shape)


def selftest_division(nsamples, seed=1):
    """Bitwise mismatches of the ENO kernels' division against IEEE division."""
    bad = C.c_ulonglong()
    ex = (C.c_double * 2)()
    _check(load_library().turb_selftest_division(C.c_longlong(nsamples), C.c_ulonglong(seed), C.byref(bad), ex),
           "selftest_division")
    return bad.value, (ex[0], ex[1])


def division_two_term_exact(h):
    """Whether the ENO kernels divide by spacing h with the two-term quotient
    alone (turb_division_two_term_exact; host only)."""
    f = load_library().turb_division_two_term_exact
    f.argtypes = [C.c_double]
    return bool(f(float(h)))


def selftest_division_pairs(a, h):
    """The kernels' two-term quotient and the IEEE quotient of a / h on the GPU."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    h = np.ascontiguousarray(h, dtype=np.float64)
    if a.shape != h.shape:
        raise ValueError("a and h differ in shape")
    q2, qd = np.empty_like(a), np.empty_like(a)
    _check(load_library().turb_selftest_division_pairs(C.c_longlong(a.size), _ptr(a), _ptr(h), _ptr(q2), _ptr(qd)),
           "selftest_division_pairs")
    return q2, qd


def measure_fp64_rate():
    """FP64 FMA instructions per second of the current GPU (turb_measure_fp64_rate)"""
    r = C.c_double()
    _check(load_library().turb_measure_fp64_rate(C.byref(r)), "measure_fp64_rate")
    return r.value


def profile_bytes(ctx):
    """algorithmic bytes of the timed launches per group (turb_profile_bytes)"""
    b = (C.c_double * len(PROF_GROUPS))()
    _check(ctx.lib.turb_profile_bytes(ctx.ctx, b), "profile_bytes")
    return {g: b[i] for i, g in enumerate(PROF_GROUPS)}
