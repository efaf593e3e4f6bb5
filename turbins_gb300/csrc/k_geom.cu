// k_geom.cu -- immersed-boundary geometry on the device: the signed distance
// to a bottom topography and the node status, as the reference sets them up
// (Surface.c, Levelset.c, Grid.c):
//   sdf guess yc - interface_position          Surface_initialize, Surface.c:96-195
//   level-set reinitialisation (Godunov with    Levelset_reinitialize / _compute_derivatives /
//   the Russo-Smereka subcell fix)             _do_Godunov / _is_converged, Levelset.c:85-578
//   sdf at u, v, w nodes (2-point)             Surface_find_q_sdf, Surface.c:216-336
//   box / surface / BUFFER_SOLID tagging       Grid.c:1424-1613, 1617-1672, 2024-2160
// Every operation is rounded as the reference's C (explicit _rn intrinsics,
// no contraction), so the fields and statuses are bit-identical to it; only
// the convergence norm is summed in block order.
#include <cmath>
#include "turb_geom.cuh"

namespace {

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }
// definitions.h:53-54
__device__ __forceinline__ double mx(double a, double b) { return a < b ? b : a; }
__device__ __forceinline__ double mn(double a, double b) { return a > b ? b : a; }
__device__ __forceinline__ int imx(int a, int b) { return a < b ? b : a; }
__device__ __forceinline__ int imn(int a, int b) { return a > b ? b : a; }

struct GeoIn {
    Dims d;
    const double *xc, *yc, *zc, *xu, *yv, *zw;
    const double *mxu, *myv, *mzw;
    const double *dxc, *dyc, *dzc;     // cell widths dx_c, dy_c, dz_c
    double a_dEta, a_dXi, a_dPhi;
};

// 3-D launch over all DA points: 32 x 8 threads over (i, j), one k per z block
struct P3 {
    int i, j, k;
    bool ok;
};
__device__ __forceinline__ P3 p3(const Dims &d)
{
    P3 r{(int)(blockIdx.x * blockDim.x + threadIdx.x), (int)(blockIdx.y * blockDim.y + threadIdx.y), (int)blockIdx.z,
         false};
    r.ok = r.i < d.NX && r.j < d.NY;
    return r;
}

__global__ void k_sdf_guess(GeoIn g, const double *__restrict__ ipos, double *__restrict__ p0)
{
    P3 t = p3(g.d);
    if (!t.ok) return;
    p0[g.d.at(t.i, t.j, t.k)] = sb(g.yc[t.j], ipos[(long long)t.k * g.d.NX + t.i]);
}

// Levelset_compute_derivatives: one-sided differences, forward except on the
// last two planes (NI = nx)
__global__ void k_ls_deriv(GeoIn g, const double *__restrict__ p, double *__restrict__ Dx, double *__restrict__ Dy,
                           double *__restrict__ Dz)
{
    P3 t = p3(g.d);
    if (!t.ok) return;
    const Dims &d = g.d;
    long long q = d.at(t.i, t.j, t.k);
    int NI = d.nx, NJ = d.ny, NK = d.nz;
    Dx[q] = t.i < NI - 1 ? ml(ml(sb(p[q + 1], p[q]), g.mxu[t.i]), g.a_dEta)
                         : ml(ml(sb(p[q], p[q - 1]), g.mxu[t.i - 1]), g.a_dEta);
    Dy[q] = t.j < NJ - 1 ? ml(ml(sb(p[q + d.PX], p[q]), g.myv[t.j]), g.a_dXi)
                         : ml(ml(sb(p[q], p[q - d.PX]), g.myv[t.j - 1]), g.a_dXi);
    Dz[q] = t.k < NK - 1 ? ml(ml(sb(p[q + d.plane], p[q]), g.mzw[t.k]), g.a_dPhi)
                         : ml(ml(sb(p[q], p[q - d.plane]), g.mzw[t.k - 1]), g.a_dPhi);
}

// Levelset_do_Godunov, Levelset.c:267-497, on the cells i < nx, j < ny, k < nz
__global__ void k_ls_godunov(GeoIn g, const double *__restrict__ p0, const double *__restrict__ Dx,
                             const double *__restrict__ Dy, const double *__restrict__ Dz, double dt,
                             double *__restrict__ p)
{
    P3 t = p3(g.d);
    const Dims &d = g.d;
    int NI = d.nx, NJ = d.ny, NK = d.nz;
    if (!t.ok || t.i >= NI || t.j >= NJ || t.k >= NK) return;
    int i = t.i, j = t.j, k = t.k;
    const double tol = 0.01;
    long long q = d.at(i, j, k);
    double dx = g.dxc[i];
    double pp0 = p0[q];
    double sign_0 = dv(pp0, __dsqrt_rn(ad(ml(pp0, pp0), ml(dx, dx))));
    double Dxp = Dx[q], Dxm = Dx[d.at(imx(0, i - 1), j, k)];
    double Dyp = Dy[q], Dym = Dy[d.at(i, imx(0, j - 1), k)];
    double Dzp = Dz[q], Dzm = Dz[d.at(i, j, imx(0, k - 1))];
    double ap = mx(Dxm, 0.0), am = mn(Dxm, 0.0), bp = mx(Dxp, 0.0), bm = mn(Dxp, 0.0);
    double cp = mx(Dym, 0.0), cm = mn(Dym, 0.0), dp = mx(Dyp, 0.0), dm = mn(Dyp, 0.0);
    double ep = mx(Dzm, 0.0), em = mn(Dzm, 0.0), fp = mx(Dzp, 0.0), fm = mn(Dzp, 0.0);
    double tx, ty, tz;
    if (sign_0 > 0.0) {
        tx = mx(ml(ap, ap), ml(bm, bm));
        ty = mx(ml(cp, cp), ml(dm, dm));
        tz = mx(ml(ep, ep), ml(fm, fm));
    } else {
        tx = mx(ml(am, am), ml(bp, bp));
        ty = mx(ml(cm, cm), ml(dp, dp));
        tz = mx(ml(em, em), ml(fp, fp));
    }
    double H = ml(sign_0, sb(__dsqrt_rn(ad(ad(tx, ty), tz)), 1.0));
    double p_p = pp0;
    int ie = imn(i + 1, NI - 1), jn = imn(j + 1, NJ - 1), kf = imn(k + 1, NK - 1);
    int iw = imx(i - 1, 0), js = imx(j - 1, 0), kb = imx(k - 1, 0);
    double p_e = p0[d.at(ie, j, k)], p_n = p0[d.at(i, jn, k)], p_f = p0[d.at(i, j, kf)];
    double p_w = p0[d.at(iw, j, k)], p_s = p0[d.at(i, js, k)], p_b = p0[d.at(i, j, kb)];
    double DeltaX = sb(g.xc[ie], g.xc[iw]), DeltaY = sb(g.yc[jn], g.yc[js]), DeltaZ = sb(g.zc[kf], g.zc[kb]);
    if (ml(p_p, p_w) < 0.0 || ml(p_p, p_e) < 0.0 || ml(p_p, p_n) < 0.0 || ml(p_p, p_s) < 0.0 ||
        ml(p_p, p_b) < 0.0 || ml(p_p, p_f) < 0.0) {
        double Ddx = fabs(DeltaX) > tol ? dv(sb(p_e, p_w), DeltaX) : 0.0;
        double Ddy = fabs(DeltaY) > tol ? dv(sb(p_n, p_s), DeltaY) : 0.0;
        double Ddz = fabs(DeltaZ) > tol ? dv(sb(p_f, p_b), DeltaZ) : 0.0;
        double Dt = __dsqrt_rn(ad(ad(ml(Ddx, Ddx), ml(Ddy, Ddy)), ml(Ddz, Ddz)));
        if (Dt < tol) Dt = tol;
        double D = dv(p_p, Dt);
        if (fabs(sign_0) < 1.0e-8) sign_0 = 0.0;
        else if (sign_0 > 0.0) sign_0 = 1.0;
        else sign_0 = -1.0;
        double dy = g.dyc[j], dz = g.dzc[k];
        double Ds = __dsqrt_rn(ad(ad(ml(dx, dx), ml(dy, dy)), ml(dz, dz)));
        H = dv(sb(ml(sign_0, fabs(p[q])), D), Ds);
    }
    p[q] = ad(p[q], ml(-H, dt));
}

// Levelset_is_converged (NORM2) partials: sum of |p - p_old|^2 dx dy dz over
// all DA points, per block; then Levelset_store_old_data (p_old = p)
__global__ void k_ls_err(GeoIn g, const double *__restrict__ p, double *__restrict__ po, double *__restrict__ part)
{
    P3 t = p3(g.d);
    double e2 = 0.0;
    if (t.ok) {
        long long q = g.d.at(t.i, t.j, t.k);
        double pq = p[q];
        double err = fabs(sb(pq, po[q]));
        e2 = ml(ml(ml(ml(err, err), g.dxc[t.i]), g.dyc[t.j]), g.dzc[t.k]);
        po[q] = pq;
    }
    __shared__ double sm[8];
    for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    int lt = threadIdx.y * blockDim.x + threadIdx.x;
    if ((lt & 31) == 0) sm[lt >> 5] = e2;
    __syncthreads();
    if (lt == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; w++) s += sm[w];
        part[((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void k_sum(long long n, const double *__restrict__ part, double *__restrict__ out)
{
    double s = 0.0;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) s += part[t];
    __shared__ double sm[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += sm[w];
        *out = r;
    }
}

// Levelset_update_last_planes, Levelset.c:642-700: x, then y, then z plane
__global__ void k_ls_last_x(Dims d, double *__restrict__ p)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (j < d.NY) p[d.at(d.NX - 1, j, k)] = p[d.at(d.NX - 2, j, k)];
}
__global__ void k_ls_last_y(Dims d, double *__restrict__ p)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i < d.NX) p[d.at(i, d.NY - 1, k)] = p[d.at(i, d.NY - 2, k)];
}
__global__ void k_ls_last_z(Dims d, double *__restrict__ p)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i < d.NX) p[d.at(i, j, d.NZ - 1)] = p[d.at(i, j, d.NZ - 2)];
}

// MyMath_interpolate_quantity, two points (MyMath.c:25-44)
__device__ __forceinline__ double itp2(double q0, double x0, double q1, double x1, double x)
{
    double m = dv(sb(q1, q0), sb(x1, x0));
    if (fabs(sb(x1, x0)) < 1.0e-8) return q0;
    return ad(ml(m, sb(x, x0)), q0);
}

// Surface_find_q_sdf: u, v, w sdf from the cell centres
__global__ void k_q_sdf(GeoIn g, const double *__restrict__ c, double *__restrict__ u, double *__restrict__ v,
                        double *__restrict__ w)
{
    P3 t = p3(g.d);
    if (!t.ok) return;
    const Dims &d = g.d;
    int i = t.i, j = t.j, k = t.k;
    long long q = d.at(i, j, k);
    double c0 = c[q];
    u[q] = i > 0 ? itp2(c0, g.xc[i], c[q - 1], g.xc[i - 1], g.xu[i]) : itp2(c0, g.xc[i], c0, g.xc[i], g.xu[i]);
    v[q] = j > 0 ? itp2(c0, g.yc[j], c[q - d.PX], g.yc[j - 1], g.yv[j]) : itp2(c0, g.yc[j], c0, g.yc[j], g.yv[j]);
    w[q] = k > 0 ? itp2(c0, g.zc[k], c[q - d.plane], g.zc[k - 1], g.zw[k]) : itp2(c0, g.zc[k], c0, g.zc[k], g.zw[k]);
}

// Grid_tag_q_box_boundary_nodes + Grid_tag_q_nodes_using_surface for
// quantity q (0..3: u, v, w, c)
__global__ void k_tag(Dims d, int q, const double *__restrict__ sdf, uint8_t *__restrict__ st)
{
    P3 t = p3(d);
    if (!t.ok) return;
    int i = t.i, j = t.j, k = t.k;
    long long p = d.at(i, j, k);
    bool box = i == d.NX - 1 || j == d.NY - 1 || k == d.NZ - 1 || (q == 0 && i == 0) || (q == 1 && j == 0) ||
               (q == 2 && k == 0);
    if (box) { st[p] = T_BOUNDARY; return; }
    int NI = d.nx, NJ = d.ny, NK = d.nz;
    double s_p = sdf[p];
    if (s_p >= 0.0) { st[p] = T_FLUID; return; }
    double s_e = sdf[d.at(imn(i + 1, NI - 1), j, k)], s_w = sdf[d.at(imx(i - 1, 0), j, k)];
    double s_n = sdf[d.at(i, imn(j + 1, NJ - 1), k)], s_s = sdf[d.at(i, imx(j - 1, 0), k)];
    double s_f = sdf[d.at(i, j, imn(k + 1, NK - 1))];
    double sbk = sdf[d.at(i, j, imx(k - 1, 0))];
    double s_b = sbk > 0.0 ? 1.0 : (sbk < 0.0 ? -1.0 : 0.0);   // sign(), definitions.h:57
    bool imm = ml(s_p, s_e) < 0.0 || ml(s_p, s_w) < 0.0 || ml(s_p, s_n) < 0.0 || ml(s_p, s_s) < 0.0 ||
               ml(s_p, s_b) < 0.0 || ml(s_p, s_f) < 0.0;
    st[p] = imm ? T_IMMERSED : T_SOLID;
}

// Grid_tag_q_buffer_solid_nodes: SOLID nodes with an IMMERSED node within
// +-width (statuses read before the pass, as the reference reads the local
// copy while it writes the global one)
__global__ void k_buffer(Dims d, int q, int width, const uint8_t *__restrict__ before, uint8_t *__restrict__ st)
{
    P3 t = p3(d);
    if (!t.ok) return;
    int i = t.i, j = t.j, k = t.k;
    int NI = d.nx, NJ = d.ny, NK = d.nz;
    int i0 = q == 0 ? 1 : 0, j0 = q == 1 ? 1 : 0, k0 = q == 2 ? 1 : 0;
    if (i < i0 || i >= NI || j < j0 || j >= NJ || k < k0 || k >= NK) return;
    long long p = d.at(i, j, k);
    if (before[p] != T_SOLID) return;
    for (int kz = -width; kz <= width; kz++)
        for (int ky = -width; ky <= width; ky++)
            for (int kx = -width; kx <= width; kx++) {
                int a = i + kx, b = j + ky, c = k + kz;
                if (a < 0 || a > NI || b < 0 || b > NJ || c < 0 || c > NK) continue;   // OUTSIDE
                if (before[d.at(a, b, c)] == T_IMMERSED) { st[p] = T_BUFFER_SOLID; return; }
            }
}

inline dim3 g3(const Dims &d) { return dim3((unsigned)((d.NX + 31) / 32), (unsigned)((d.NY + 7) / 8), (unsigned)d.NZ); }
const dim3 B38(32, 8, 1);

}  // namespace

long long geom_scratch_doubles(const Dims &d)
{
    dim3 g = g3(d);
    return 5 * d.n + (long long)g.x * g.y * g.z + 1;
}

cudaError_t geom_setup(cudaStream_t s, const GeomArgs &a, const double *ipos, double *scratch, uint8_t *tmp,
                       GeomOut *o)
{
    GeoIn g;
    g.d = a.d;
    g.xc = a.xc; g.yc = a.yc; g.zc = a.zc; g.xu = a.xu; g.yv = a.yv; g.zw = a.zw;
    g.mxu = a.mxu; g.myv = a.myv; g.mzw = a.mzw; g.dxc = a.dxc; g.dyc = a.dyc; g.dzc = a.dzc;
    g.a_dEta = a.a_dEta; g.a_dXi = a.a_dXi; g.a_dPhi = a.a_dPhi;
    const Dims &d = a.d;
    const dim3 G = g3(d);
    long long np = (long long)G.x * G.y * G.z;
    // phi->G_data is the c sdf output itself
    double *p = o->sdf[0], *po = scratch, *p0 = scratch + d.n, *Dx = scratch + 2 * d.n, *Dy = scratch + 3 * d.n,
           *Dz = scratch + 4 * d.n, *part = scratch + 5 * d.n, *tot = part + np;
    size_t fb = sizeof(double) * d.n;
    // Surface_initialize (only a bottom surface): yc - interface_position
    k_sdf_guess<<<G, B38, 0, s>>>(g, ipos, p0);
    cudaMemcpyAsync(p, p0, fb, cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(po, 0, fb, s);
    // Levelset_reinitialize: stop after the step whose NORM2 change is below
    // 1e-5, or once the counter passes max_iterations + 1
    int c = 0;
    double W = 0.0;
    for (;;) {
        k_ls_deriv<<<G, B38, 0, s>>>(g, p, Dx, Dy, Dz);
        k_ls_godunov<<<G, B38, 0, s>>>(g, p0, Dx, Dy, Dz, a.dt, p);
        k_ls_err<<<G, B38, 0, s>>>(g, p, po, part);
        k_sum<<<1, 1024, 0, s>>>(np, part, tot);
        double e2 = 0.0;
        cudaMemcpyAsync(&e2, tot, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        W = std::sqrt(e2);
        if (c > a.max_iterations + 1 || W < 1.0e-5) break;
        c++;
    }
    o->iterations = c + 1;
    o->last_error = W;
    // Levelset_update_last_planes, then G_c_sdf = phi
    k_ls_last_x<<<dim3((unsigned)((d.NY + 127) / 128), (unsigned)d.NZ), 128, 0, s>>>(d, p);
    k_ls_last_y<<<dim3((unsigned)((d.NX + 127) / 128), (unsigned)d.NZ), 128, 0, s>>>(d, p);
    k_ls_last_z<<<dim3((unsigned)((d.NX + 127) / 128), (unsigned)d.NY), 128, 0, s>>>(d, p);
    k_q_sdf<<<G, B38, 0, s>>>(g, p, o->sdf[1], o->sdf[2], o->sdf[3]);
    // Grid_identify_geometry: box planes + surface, then BUFFER_SOLID (width 2)
    // for u, v, w from the statuses before that pass
    const double *qs[4] = {o->sdf[1], o->sdf[2], o->sdf[3], o->sdf[0]};
    for (int q = 0; q < 4; q++) cudaMemsetAsync(o->st[q], 0, (size_t)d.n, s);
    for (int q = 0; q < 4; q++) k_tag<<<G, B38, 0, s>>>(d, q, qs[q], o->st[q]);
    for (int q = 0; q < 3; q++) {
        cudaMemcpyAsync(tmp, o->st[q], (size_t)d.n, cudaMemcpyDeviceToDevice, s);
        k_buffer<<<G, B38, 0, s>>>(d, q, 2, tmp, o->st[q]);
    }
    return cudaGetLastError();
}
