// k_stencil.cu -- element-wise / 7-point FP64 kernels of the step: cell-centre
// interpolation, transposed velocities, total concentration, particle
// velocity, momentum and concentration RHS, pressure RHS, projection,
// divergence, store/average.  Every rounding is explicit (_rn intrinsics, no
// contraction) so results are bit-identical to the reference's C compiled
// without FMA contraction.
#include "turb_internal.cuh"
#include "turb_kernels.cuh"
#include "turb_div.cuh"

namespace {

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }

// MyMath_interpolate_quantity two-point branch, MyMath.c:22-40; the slope's
// division rounds as the IEEE division in every mode (see Interp2)
__device__ __forceinline__ double interp2(double q0, double q1, const Interp2 &T, int t)
{
    if (T.flat[t]) return q0;
    double a = sb(q1, q0), h = T.dx[t];
    int mode = T.div[t];
    double m = mode == 1   ? ml(a, T.rdx[t])
               : mode == 3 ? div_by_spacing_2t(a, h, T.rdx[t], T.rdxl[t])
               : mode == 2 ? div_by_spacing(a, h, T.rdx[t], T.rdxl[t])
                           : dv(a, h);
    return ad(ml(m, T.dq[t]), q0);
}

// four-point branch, MyMath.c:54-74, weights precomputed per direction
__device__ __forceinline__ double interp4(double q0, double q1, double q2, double q3, double wx0,
                                          double wx1, double wy0, double wy1)
{
    double qt = ad(ml(wx0, q2), ml(wx1, q3));
    double qb = ad(ml(wx0, q0), ml(wx1, q1));
    return ad(ml(wy0, qb), ml(wy1, qt));
}

struct Ijk {
    int i, j, k;
    bool ok;
};

// 3-D launch: blocks of 32 x 8 threads over (i, j), one z-block per k
__device__ __forceinline__ Ijk ijk_of(const Dims &d)
{
    Ijk r;
    r.i = blockIdx.x * blockDim.x + threadIdx.x;
    r.j = blockIdx.y * blockDim.y + threadIdx.y;
    r.k = blockIdx.z;
    r.ok = r.i < d.NX && r.j < d.NY;
    return r;
}

// Velocity_cell_center, Velocity.c:1476-1602 (u on the inflow / outflow
// faces from the open-boundary planes, Velocity.c:1544-1558)
__global__ void k_cell_center(Dims d, Interp2 ix, Interp2 iy, Interp2 iz, OpenBC ob, const double *__restrict__ u,
                              const double *__restrict__ v, const double *__restrict__ w,
                              double *__restrict__ ubc, double *__restrict__ vbc, double *__restrict__ wbc)
{
    Ijk t = ijk_of(d);
    if (!t.ok || t.i >= d.nx || t.j >= d.ny || t.k >= d.nz) return;
    long long p = d.at(t.i, t.j, t.k);
    double u0 = (ob.in && t.i == 0) ? ob.pl(ob.u_in, t.j, t.k) : u[p];
    double u1 = (ob.out && t.i == d.nx - 1) ? ob.pl(ob.out_f[0], t.j, t.k) : u[p + 1];
    ubc[p] = interp2(u0, u1, ix, t.i);
    vbc[p] = interp2(v[p], v[p + d.PX], iy, t.j);
    wbc[p] = interp2(w[p], w[p + d.plane], iz, t.k);
}

// Velocity_transpose_velocities, Velocity.c:3341-3663 (u from the inflow /
// outflow planes next to the open faces, Velocity.c:3491-3507, 3589-3605)
__global__ void k_transpose(Dims d, int which, const uint8_t *__restrict__ st, TransW tw, OpenBC ob,
                            const double *__restrict__ u, const double *__restrict__ v,
                            const double *__restrict__ w, double *__restrict__ A, double *__restrict__ B)
{
    Ijk t = ijk_of(d);
    if (!t.ok) return;
    long long p = d.at(t.i, t.j, t.k);
    if (st[p] == T_BOUNDARY) return;
    int i = t.i, j = t.j, k = t.k;
    long long X = 1, Y = d.PX, Z = d.plane;
    if (which == 0) {
        A[p] = interp4(v[p - X], v[p], v[p - X + Y], v[p + Y], tw.xu.w0[i], tw.xu.w1[i], tw.yc.w0[j], tw.yc.w1[j]);
        B[p] = interp4(w[p - X], w[p], w[p - X + Z], w[p + Z], tw.xu.w0[i], tw.xu.w1[i], tw.zc.w0[k], tw.zc.w1[k]);
    } else if (which == 1) {
        double q0 = u[p - Y], q1 = u[p - Y + X], q2 = u[p], q3 = u[p + X];
        if (ob.in && i == 0 && j > 0) { q0 = ob.pl(ob.u_in, j - 1, k); q2 = ob.pl(ob.u_in, j, k); }
        if (ob.out && i == d.nx - 1 && j > 0) { q1 = ob.pl(ob.out_f[0], j - 1, k); q3 = ob.pl(ob.out_f[0], j, k); }
        A[p] = interp4(q0, q1, q2, q3, tw.xc.w0[i], tw.xc.w1[i], tw.yv.w0[j], tw.yv.w1[j]);
        B[p] = interp4(w[p - Y], w[p - Y + Z], w[p], w[p + Z], tw.zc.w0[k], tw.zc.w1[k], tw.yv.w0[j], tw.yv.w1[j]);
    } else {
        double q0 = u[p - Z], q1 = u[p - Z + X], q2 = u[p], q3 = u[p + X];
        if (ob.in && i == 0 && k > 0) { q0 = ob.pl(ob.u_in, j, k - 1); q2 = ob.pl(ob.u_in, j, k); }
        if (ob.out && i == d.nx - 1 && k > 0) { q1 = ob.pl(ob.out_f[0], j, k - 1); q3 = ob.pl(ob.out_f[0], j, k); }
        A[p] = interp4(q0, q1, q2, q3, tw.xc.w0[i], tw.xc.w1[i], tw.zw.w0[k], tw.zw.w1[k]);
        B[p] = interp4(v[p - Z], v[p], v[p - Z + Y], v[p + Y], tw.zw.w0[k], tw.zw.w1[k], tw.yc.w0[j], tw.yc.w1[j]);
    }
}

// Conc_compute_total_concentration, Conc.c:1291-1314 (VecCopy/VecScale/VecAXPY)
__global__ void k_total_conc(long long n, int nc, ConcPtrs c, ConcW a, double *__restrict__ ct)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double s = ml(c.p[0][p], a.v[0]);
    for (int q = 1; q < nc; q++) s = ad(s, ml(a.v[q], c.p[q][p]));
    ct[p] = s;
}

// Conc_set_particle_v_velocity, Conc.c:734-761 (VecCopy + VecShift)
__global__ void k_shift(long long n, const double *__restrict__ x, double s, double *__restrict__ y)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    y[p] = ad(x[p], s);
}

// Velocity_{u,v,w}_set_RHS, Velocity.c:1607-2043; open boundaries add the
// known face values of the boundary-adjacent rows (u: inflow at i = 1,
// outflow at i = nx-1, Velocity.c:1691-1721; v, w: outflow at i = nx-1,
// Velocity.c:1885-1896, 2011-2022)
__global__ void k_rhs_vel(Dims d, int q, const uint8_t *__restrict__ st, double a_dt,
                          const double *__restrict__ x, const double *__restrict__ conv,
                          const double *__restrict__ dp, const double *__restrict__ ct, int buoy,
                          Interp2 iyv, OpenBC ob, double *__restrict__ b)
{
    Ijk t = ijk_of(d);
    if (!t.ok) return;
    long long p = d.at(t.i, t.j, t.k);
    int s = st[p];
    double r = 0.0;
    if (s == T_FLUID || s == T_BUFFER_SOLID) {
        r = sb(sb(ml(x[p], a_dt), conv[p]), dp[p]);
        if (q == 0) {
            if (ob.in && t.i == 1) r = ad(r, ml(ob.u_aw, ob.pl(ob.u_in, t.j, t.k)));
            if (ob.out && t.i == d.nx - 1) r = ad(r, ml(ob.u_ae, ob.pl(ob.out_f[0], t.j, t.k)));
        } else if (ob.out && t.i == d.nx - 1) {
            r = ad(r, ml(ob.vw_ae[q - 1], ob.pl(ob.out_f[q], t.j, t.k)));
        }
        if (q == 1 && buoy) {
            double c = interp2(ct[p - d.PX], ct[p], iyv, t.j);
            r = sb(r, c);
        }
    }
    b[p] = r;
}

// Conc_set_RHS, Conc.c:864-992 (inflow at i = 0, outflow at i = nx-1:
// Conc.c:938-962)
__global__ void k_rhs_conc(Dims d, int ic, const uint8_t *__restrict__ st, double a_dt,
                           const double *__restrict__ c, const double *__restrict__ conv, OpenBC ob,
                           double *__restrict__ b)
{
    Ijk t = ijk_of(d);
    if (!t.ok) return;
    long long p = d.at(t.i, t.j, t.k);
    double r = 0.0;
    if (st[p] == T_FLUID) {
        r = sb(ml(c[p], a_dt), conv[p]);
        if (ob.in && t.i == 0) r = ad(r, ml(ob.c_aw[ic], ob.pl(ob.c_in[ic], t.j, t.k)));
        if (ob.out && t.i == d.nx - 1) r = ad(r, ml(ob.c_ae[ic], ob.pl(ob.out_f[3 + ic], t.j, t.k)));
    }
    b[p] = r;
}

// Pressure_set_RHS, Pressure.c:171-276
__global__ void k_pressure_rhs(Dims d, const uint8_t *__restrict__ st, const double *__restrict__ cx,
                               const double *__restrict__ cy, const double *__restrict__ cz, double a_dt, OpenBC ob,
                               const double *__restrict__ u, const double *__restrict__ v,
                               const double *__restrict__ w, double *__restrict__ b)
{
    Ijk t = ijk_of(d);
    if (!t.ok) return;
    long long p = d.at(t.i, t.j, t.k);
    double r = 0.0;
    if (st[p] != T_BOUNDARY) {
        double ue = u[p + 1], uw = u[p];   // open faces: Pressure.c:242-248
        if (ob.in && t.i == 0) uw = ob.pl(ob.u_in, t.j, t.k);
        if (ob.out && t.i == d.nx - 1) ue = ob.pl(ob.out_f[0], t.j, t.k);
        double dudx = ml(sb(ue, uw), cx[t.i]);
        double dvdy = ml(sb(v[p + d.PX], v[p]), cy[t.j]);
        double dwdz = ml(sb(w[p + d.plane], w[p]), cz[t.k]);
        r = ml(-ad(ad(dudx, dvdy), dwdz), a_dt);
    }
    b[p] = r;
}

// Pressure_project_velocity, Pressure.c:280-439
__global__ void k_project(Dims d, ProjArgs a, const double *__restrict__ phi, const double *__restrict__ pb,
                          double *__restrict__ u, double *__restrict__ v, double *__restrict__ w,
                          double *__restrict__ dpx, double *__restrict__ dpy, double *__restrict__ dpz)
{
    Ijk t = ijk_of(d);
    if (!t.ok) return;
    long long p = d.at(t.i, t.j, t.k);
    if (a.su[p] != T_BOUNDARY) {
        double me = a.mxu[t.i];
        double dd = ml(ml(sb(phi[p], phi[p - 1]), a.a_dEta), me);
        u[p] = sb(u[p], ml(a.dt, dd));
        double lap = ml(ml(-sb(pb[p], pb[p - 1]), me), a.a_dEta);
        dpx[p] = ad(dpx[p], sb(dd, ml(a.coef, lap)));
    }
    if (a.sv[p] != T_BOUNDARY) {
        double cyv = a.cyv[t.j];
        double dd = ml(sb(phi[p], phi[p - d.PX]), cyv);
        v[p] = sb(v[p], ml(a.dt, dd));
        double lap = ml(-sb(pb[p], pb[p - d.PX]), cyv);
        dpy[p] = ad(dpy[p], sb(dd, ml(a.coef, lap)));
    }
    if (a.sw[p] != T_BOUNDARY) {
        double czw = a.czw[t.k];
        double dd = ml(sb(phi[p], phi[p - d.plane]), czw);
        w[p] = sb(w[p], ml(a.dt, dd));
        double lap = ml(-sb(pb[p], pb[p - d.plane]), czw);
        dpz[p] = ad(dpz[p], sb(dd, ml(a.coef, lap)));
    }
}

// Pressure_compute_velocity_divergence, Pressure.c:462-586 (block max)
__global__ void k_divergence(Dims d, const uint8_t *__restrict__ st, const double *__restrict__ mxc,
                             const double *__restrict__ myc, const double *__restrict__ mzc, double a_dEta,
                             double a_dXi, double a_dPhi, OpenBC ob, const double *__restrict__ u,
                             const double *__restrict__ v, const double *__restrict__ w,
                             double *__restrict__ div, double *__restrict__ part)
{
    Ijk t = ijk_of(d);
    double dc = 0.0;
    if (t.ok) {
        long long p = d.at(t.i, t.j, t.k);
        if (st[p] != T_BOUNDARY) {
            double ue = u[p + 1], uw = u[p];   // open faces: Pressure.c:541-547
            if (ob.in && t.i == 0) uw = ob.pl(ob.u_in, t.j, t.k);
            if (ob.out && t.i == d.nx - 1) ue = ob.pl(ob.out_f[0], t.j, t.k);
            double dudx = ml(ml(sb(ue, uw), a_dEta), mxc[t.i]);
            double dvdy = ml(ml(sb(v[p + d.PX], v[p]), a_dXi), myc[t.j]);
            double dwdz = ml(ml(sb(w[p + d.plane], w[p]), a_dPhi), mzc[t.k]);
            dc = fabs(ad(ad(dudx, dvdy), dwdz));
        }
        div[p] = dc;
    }
    // block max (values are >= 0; a NaN is kept)
    __shared__ double sm[32];
    int lt = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    double m = dc;
    m = turb_warp_maxbits(m);
    if ((lt & 31) == 0) sm[lt >> 5] = m;
    __syncthreads();
    if (lt < 32) {
        m = (lt < (nt >> 5)) ? sm[lt] : 0.0;
        m = turb_warp_maxbits(m);
        if (lt == 0) part[((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = m;
    }
}

__global__ void k_max_final(long long nparts, const double *__restrict__ part, double *__restrict__ out)
{
    double m = 0.0;
    for (long long t = threadIdx.x; t < nparts; t += blockDim.x) m = turb_maxbits(m, part[t]);
    __shared__ double sm[32];
    m = turb_warp_maxbits(m);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        m = turb_warp_maxbits(m);
        if (threadIdx.x == 0) *out = m;
    }
}

// Velocity_rk_average / Conc_rk_average (VecAXPBY: y = a*x + b*y)
__global__ void k_axpby(long long n, double a, const double *__restrict__ x, double b, double *__restrict__ y)
{
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    y[p] = ad(ml(a, x[p]), ml(b, y[p]));
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static const dim3 B3(32, 8, 1);
static inline dim3 grid_of(const Dims &d, int)
{
    return dim3((unsigned)((d.NX + 31) / 32), (unsigned)((d.NY + 7) / 8), (unsigned)d.NZ);
}

void launch_cell_center(cudaStream_t s, const Dims &d, Interp2 ix, Interp2 iy, Interp2 iz, const OpenBC &ob,
                        const double *u, const double *v, const double *w, double *ubc, double *vbc, double *wbc)
{
    k_cell_center<<<grid_of(d, 256), B3, 0, s>>>(d, ix, iy, iz, ob, u, v, w, ubc, vbc, wbc);
}

void launch_transpose(cudaStream_t s, const Dims &d, int which, const uint8_t *st, TransW tw, const OpenBC &ob,
                      const double *u, const double *v, const double *w, double *A, double *B)
{
    k_transpose<<<grid_of(d, 256), B3, 0, s>>>(d, which, st, tw, ob, u, v, w, A, B);
}

void launch_total_conc(cudaStream_t s, long long n, int nc, ConcPtrs c, ConcW a, double *ct)
{
    k_total_conc<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, nc, c, a, ct);
}

void launch_shift(cudaStream_t s, long long n, const double *x, double sh, double *y)
{
    k_shift<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, x, sh, y);
}

void launch_rhs_vel(cudaStream_t s, const Dims &d, int q, const uint8_t *st, double a_dt, const double *x,
                    const double *conv, const double *dp, const double *ct, int buoy, Interp2 iyv,
                    const OpenBC &ob, double *b)
{
    k_rhs_vel<<<grid_of(d, 256), B3, 0, s>>>(d, q, st, a_dt, x, conv, dp, ct, buoy, iyv, ob, b);
}

void launch_rhs_conc(cudaStream_t s, const Dims &d, int ic, const uint8_t *st, double a_dt, const double *c,
                     const double *conv, const OpenBC &ob, double *b)
{
    k_rhs_conc<<<grid_of(d, 256), B3, 0, s>>>(d, ic, st, a_dt, c, conv, ob, b);
}

void launch_pressure_rhs(cudaStream_t s, const Dims &d, const uint8_t *st, const double *cx, const double *cy,
                         const double *cz, double a_dt, const OpenBC &ob, const double *u, const double *v,
                         const double *w, double *b)
{
    k_pressure_rhs<<<grid_of(d, 256), B3, 0, s>>>(d, st, cx, cy, cz, a_dt, ob, u, v, w, b);
}

void launch_project(cudaStream_t s, const Dims &d, ProjArgs a, const double *phi, const double *pb, double *u,
                    double *v, double *w, double *dpx, double *dpy, double *dpz)
{
    k_project<<<grid_of(d, 256), B3, 0, s>>>(d, a, phi, pb, u, v, w, dpx, dpy, dpz);
}

long long divergence_parts(const Dims &d)
{
    dim3 g = grid_of(d, 256);
    return (long long)g.x * g.y * g.z;
}

void launch_divergence(cudaStream_t s, const Dims &d, const uint8_t *st, const double *mxc, const double *myc,
                       const double *mzc, double a_dEta, double a_dXi, double a_dPhi, const OpenBC &ob,
                       const double *u, const double *v, const double *w, double *div, double *part, double *out)
{
    dim3 g = grid_of(d, 256);
    k_divergence<<<g, B3, 0, s>>>(d, st, mxc, myc, mzc, a_dEta, a_dXi, a_dPhi, ob, u, v, w, div, part);
    k_max_final<<<1, 1024, 0, s>>>((long long)g.x * g.y * g.z, part, out);
}

void launch_axpby(cudaStream_t s, long long n, double a, const double *x, double b, double *y)
{
    k_axpby<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, x, b, y);
}
