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
#include <utility>
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

// The per-point constants of Levelset_do_Godunov (Levelset.c:265-497) depend
// on phi_0 only: sign_0 = phi_0 / sqrt(phi_0^2 + dx^2) and, next to the
// interface (a sign change of phi_0 towards a neighbour), the distance
// D = phi_0 / |grad phi_0| of the Russo-Smereka fix (NaN elsewhere).  They
// are made once, with the reference's operations.
__global__ void k_ls_prep(GeoIn g, const double *__restrict__ p0, double *__restrict__ s0, double *__restrict__ nD)
{
    P3 t = p3(g.d);
    const Dims &d = g.d;
    int NI = d.nx, NJ = d.ny, NK = d.nz;
    if (!t.ok) return;
    int i = t.i, j = t.j, k = t.k;
    long long q = d.at(i, j, k);
    if (i >= NI || j >= NJ || k >= NK) {
        s0[q] = 0.0;
        nD[q] = __longlong_as_double(0x7ff8000000000000LL);
        return;
    }
    const double tol = 0.01;
    double dx = g.dxc[i];
    double pp0 = p0[q];
    s0[q] = dv(pp0, __dsqrt_rn(ad(ml(pp0, pp0), ml(dx, dx))));
    int ie = imn(i + 1, NI - 1), jn = imn(j + 1, NJ - 1), kf = imn(k + 1, NK - 1);
    int iw = imx(i - 1, 0), js = imx(j - 1, 0), kb = imx(k - 1, 0);
    double p_e = p0[d.at(ie, j, k)], p_n = p0[d.at(i, jn, k)], p_f = p0[d.at(i, j, kf)];
    double p_w = p0[d.at(iw, j, k)], p_s = p0[d.at(i, js, k)], p_b = p0[d.at(i, j, kb)];
    double DeltaX = sb(g.xc[ie], g.xc[iw]), DeltaY = sb(g.yc[jn], g.yc[js]), DeltaZ = sb(g.zc[kf], g.zc[kb]);
    double D = __longlong_as_double(0x7ff8000000000000LL);
    if (ml(pp0, p_w) < 0.0 || ml(pp0, p_e) < 0.0 || ml(pp0, p_n) < 0.0 || ml(pp0, p_s) < 0.0 ||
        ml(pp0, p_b) < 0.0 || ml(pp0, p_f) < 0.0) {
        double Ddx = fabs(DeltaX) > tol ? dv(sb(p_e, p_w), DeltaX) : 0.0;
        double Ddy = fabs(DeltaY) > tol ? dv(sb(p_n, p_s), DeltaY) : 0.0;
        double Ddz = fabs(DeltaZ) > tol ? dv(sb(p_f, p_b), DeltaZ) : 0.0;
        double Dt = __dsqrt_rn(ad(ad(ml(Ddx, Ddx), ml(Ddy, Ddy)), ml(Ddz, Ddz)));
        if (Dt < tol) Dt = tol;
        D = dv(pp0, Dt);
    }
    nD[q] = D;
}

// One reinitialisation step, Levelset_compute_derivatives
// (Levelset.c:154-258: one-sided differences, forward except on the last
// two planes) fused with Levelset_do_Godunov on the cells i < nx, j < ny,
// k < nz (the other DA points keep their value), from pc into pn; and the
// partials of Levelset_is_converged (NORM2, Levelset.c:500-578):
// |pn - p_old|^2 dx dy dz over all DA points, p_old = pc (0 before the
// first step), per block.
__global__ void __launch_bounds__(256) k_ls_step(GeoIn g, const double *__restrict__ pc, const double *__restrict__ s0,
                                                 const double *__restrict__ nD, double dt, int first,
                                                 double *__restrict__ pn, double *__restrict__ part)
{
    P3 t = p3(g.d);
    const Dims &d = g.d;
    int NI = d.nx, NJ = d.ny, NK = d.nz;
    double e2 = 0.0;
    if (t.ok) {
        int i = t.i, j = t.j, k = t.k;
        long long q = d.at(i, j, k);
        double pq = pc[q], pnew = pq;
        if (i < NI && j < NJ && k < NK) {
            auto DX = [&](int ii) {
                long long r = q + (ii - i);
                return ii < NI - 1 ? ml(ml(sb(pc[r + 1], pc[r]), g.mxu[ii]), g.a_dEta)
                                   : ml(ml(sb(pc[r], pc[r - 1]), g.mxu[ii - 1]), g.a_dEta);
            };
            auto DY = [&](int jj) {
                long long r = q + (long long)(jj - j) * d.PX;
                return jj < NJ - 1 ? ml(ml(sb(pc[r + d.PX], pc[r]), g.myv[jj]), g.a_dXi)
                                   : ml(ml(sb(pc[r], pc[r - d.PX]), g.myv[jj - 1]), g.a_dXi);
            };
            auto DZ = [&](int kk) {
                long long r = q + (long long)(kk - k) * d.plane;
                return kk < NK - 1 ? ml(ml(sb(pc[r + d.plane], pc[r]), g.mzw[kk]), g.a_dPhi)
                                   : ml(ml(sb(pc[r], pc[r - d.plane]), g.mzw[kk - 1]), g.a_dPhi);
            };
            double Dxp = DX(i), Dxm = DX(imx(0, i - 1));
            double Dyp = DY(j), Dym = DY(imx(0, j - 1));
            double Dzp = DZ(k), Dzm = DZ(imx(0, k - 1));
            double sign_0 = s0[q];
            double H;
            double D = nD[q];
            if (D == D) {
                // next to the interface: the sign function proper and the
                // distance kept from phi_0
                double sg = fabs(sign_0) < 1.0e-8 ? 0.0 : (sign_0 > 0.0 ? 1.0 : -1.0);
                double dx = g.dxc[i], dy = g.dyc[j], dz = g.dzc[k];
                double Ds = __dsqrt_rn(ad(ad(ml(dx, dx), ml(dy, dy)), ml(dz, dz)));
                H = dv(sb(ml(sg, fabs(pq)), D), Ds);
            } else {
                double tx, ty, tz;
                if (sign_0 > 0.0) {
                    double ap = mx(Dxm, 0.0), bm = mn(Dxp, 0.0), cp = mx(Dym, 0.0), dm = mn(Dyp, 0.0);
                    double ep = mx(Dzm, 0.0), fm = mn(Dzp, 0.0);
                    tx = mx(ml(ap, ap), ml(bm, bm));
                    ty = mx(ml(cp, cp), ml(dm, dm));
                    tz = mx(ml(ep, ep), ml(fm, fm));
                } else {
                    double am = mn(Dxm, 0.0), bp = mx(Dxp, 0.0), cm = mn(Dym, 0.0), dp = mx(Dyp, 0.0);
                    double em = mn(Dzm, 0.0), fp = mx(Dzp, 0.0);
                    tx = mx(ml(am, am), ml(bp, bp));
                    ty = mx(ml(cm, cm), ml(dp, dp));
                    tz = mx(ml(em, em), ml(fp, fp));
                }
                H = ml(sign_0, sb(__dsqrt_rn(ad(ad(tx, ty), tz)), 1.0));
            }
            pnew = ad(pq, ml(-H, dt));
        }
        pn[q] = pnew;
        double err = fabs(sb(pnew, first ? 0.0 : pq));
        e2 = ml(ml(ml(ml(err, err), g.dxc[i]), g.dyc[j]), g.dzc[k]);
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


// ---- ghost-cell stencils (Immersed.c) --------------------------------------

// IMMERSED nodes per (j, k) row, one thread per row
__global__ void k_ib_count(Dims d, const uint8_t *__restrict__ st, int *__restrict__ cnt)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (long long)d.NY * d.NZ) return;
    int j = (int)(r % d.NY), k = (int)(r / d.NY);
    const uint8_t *row = st + d.at(0, j, k);
    int c = 0;
    for (int i = 0; i < d.NX; i++) c += row[i] == T_IMMERSED;
    cnt[r] = c;
}

// exclusive scan of the row counts in place, total at cnt[nr]; one block
__global__ void k_ib_scan(long long nr, int *__restrict__ cnt)
{
    __shared__ int sm[1024];
    long long per = (nr + blockDim.x - 1) / blockDim.x;
    long long a = threadIdx.x * per, b = a + per < nr ? a + per : nr;
    int s = 0;
    for (long long r = a; r < b; r++) s += cnt[r];
    sm[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < (int)blockDim.x; t++) {
            int v = sm[t];
            sm[t] = run;
            run += v;
        }
        cnt[nr] = run;
    }
    __syncthreads();
    int run = sm[threadIdx.x];
    for (long long r = a; r < b; r++) {
        int v = cnt[r];
        cnt[r] = run;
        run += v;
    }
}

// node list in DA order (Immersed_set_q_immersed_indices, Immersed.c:379-447)
__global__ void k_ib_emit(Dims d, const uint8_t *__restrict__ st, const int *__restrict__ off,
                          int *__restrict__ node)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (long long)d.NY * d.NZ) return;
    int j = (int)(r % d.NY), k = (int)(r / d.NY);
    const uint8_t *row = st + d.at(0, j, k);
    int o = off[r];
    for (int i = 0; i < d.NX; i++)
        if (row[i] == T_IMMERSED) node[o++] = (int)(((long long)k * d.NY + j) * d.NX + i);
}

struct IbArgs {
    Dims d;
    int neumann;                          // c: NEUMANN, u/v/w: DIRICHLET
    int ni, nj, nk;                       // NI / NJ / NK, +1 along the node's own face axis
    const double *xq, *yq, *zq;           // node coordinates of the quantity
    const double *dxc, *dyc, *dzc;
    const double *sdf;                    // pitched DA
    const uint8_t *st;                    // pitched DA
};

__device__ __forceinline__ int ib_status(const IbArgs &a, int i, int j, int k)
{
    const Dims &d = a.d;
    if (i < 0 || i > d.nx || j < 0 || j > d.ny || k < 0 || k > d.nz) return -1;   // OUTSIDE
    return a.st[d.at(i, j, k)];
}

// MyMath_binary_search (MyMath.c:384-398) behind Grid_get_x_index
// (Grid.c:1877-1903): NOT_FOUND below q[0], GVG_INF above q[n-1]
__device__ int ib_index(const double *q, double v, int n)
{
    if (v < q[0]) return -1;
    if (v > q[n - 1]) return 10000000;
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) / 2;
        if (v >= q[mid]) {
            if (v < q[mid + 1]) return mid;
            lo = mid + 1;
        } else if (v < q[mid]) {
            hi = mid - 1;
        } else {
            return -1;   // unordered (NaN) search value: the reference loops; treat as not found
        }
    }
    return -1;
}

__device__ __forceinline__ double dist3(double ax, double ay, double az, double bx, double by, double bz)
{
    double x = sb(ax, bx), y = sb(ay, by), z = sb(az, bz);
    return __dsqrt_rn(ad(ad(ml(x, x), ml(y, y)), ml(z, z)));
}

// MyMath_GaussJordan_matrix_inv (MyMath.c:117-195) of an 8x8 matrix in place
__device__ void ib_gauss_jordan(double (*A)[8])
{
    int piv[8], irow[8], icol[8];
    for (int j = 0; j < 8; j++) piv[j] = -1;
    int in_row = -1, in_col = -1;
    for (int i = 0; i < 8; i++) {
        double mxv = 0.0;
        for (int j = 0; j < 8; j++)
            if (piv[j] != 0)
                for (int k = 0; k < 8; k++)
                    if (piv[k] == -1 && fabs(A[j][k]) >= mxv) {
                        mxv = fabs(A[j][k]);
                        in_row = j;
                        in_col = k;
                    }
        if (in_col < 0) return;   // every entry NaN: nothing the reference could pick either
        ++piv[in_col];
        if (in_row != in_col)
            for (int h = 0; h < 8; h++) {
                double t = A[in_row][h];
                A[in_row][h] = A[in_col][h];
                A[in_col][h] = t;
            }
        irow[i] = in_row;
        icol[i] = in_col;
        double ap = dv(1.0, A[in_col][in_col]);
        A[in_col][in_col] = 1.0;
        for (int h = 0; h < 8; h++) A[in_col][h] = ml(A[in_col][h], ap);
        for (int hh = 0; hh < 8; hh++)
            if (hh != in_col) {
                double t = A[hh][in_col];
                A[hh][in_col] = 0.0;
                for (int h = 0; h < 8; h++) A[hh][h] = sb(A[hh][h], ml(A[in_col][h], t));
            }
    }
    for (int h = 7; h >= 0; h--)
        if (irow[h] != icol[h])
            for (int k = 0; k < 8; k++) {
                double t = A[k][irow[h]];
                A[k][irow[h]] = A[k][icol[h]];
                A[k][icol[h]] = t;
            }
}

// one IMMERSED node: normal (Surface_compute_normal, Surface.c:547-615),
// control point (Immersed_find_control_point + Surface_find_Dn_to_surface,
// Immersed.c:891-953, Surface.c:475-541), image point (Immersed.c:1063-1150),
// surrounding box or nearest fluid node (Immersed_find_box,
// Immersed.c:1210-1402) and coefficients (Immersed_compute_interpolation_coef,
// Immersed.c:122-376)
__global__ void __launch_bounds__(128) k_ib_stencil(IbArgs a, int n, const int *__restrict__ node, GeomIb o)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const Dims &d = a.d;
    int L = node[t];
    int i = L % d.NX, j = (L / d.NX) % d.NY, k = L / (d.NX * d.NY);
    const double *xq = a.xq, *yq = a.yq, *zq = a.zq;
    double Px = xq[i], Py = yq[j], Pz = zq[k];
    auto S = [&](int ii, int jj, int kk) { return a.sdf[d.at(ii, jj, kk)]; };
    int iw = imx(i - 1, 0), ie = imn(i + 1, a.ni - 1);
    int js = imx(j - 1, 0), jn = imn(j + 1, a.nj - 1);
    int kb = imx(k - 1, 0), kf = imn(k + 1, a.nk - 1);
    double gx = dv(sb(S(ie, j, k), S(iw, j, k)), sb(xq[ie], xq[iw]));
    double gy = dv(sb(S(i, jn, k), S(i, js, k)), sb(yq[jn], yq[js]));
    double gz = dv(sb(S(i, j, kf), S(i, j, kb)), sb(zq[kf], zq[kb]));
    double an = dv(1.0, __dsqrt_rn(ad(ad(ml(gx, gx), ml(gy, gy)), ml(gz, gz))));
    double nx = ml(gx, an), ny = ml(gy, an), nz = ml(gz, an);
    double dn = ad(ad(ml(nx, gx), ml(ny, gy)), ml(nz, gz));
    if (fabs(dn) < 1.0e-2 || isnan(dn)) dn = 1.0e-2;
    double D = dv(S(i, j, k), dn);
    double Cx = sb(Px, ml(nx, D)), Cy = sb(Py, ml(ny, D)), Cz = sb(Pz, ml(nz, D));
    double ds = dist3(Px, Py, Pz, Cx, Cy, Cz);
    double D2 = ml(2.0, ds);
    double Ix = ad(Px, ml(nx, D2)), Iy = ad(Py, ml(ny, D2)), Iz = ad(Pz, ml(nz, D2));
    // the box: the image point perturbed towards each of the 8 corners
    const double tx = mx(ml(0.005, a.dxc[i]), 1e-12), ty = mx(ml(0.005, a.dyc[j]), 1e-12),
                 tz = mx(ml(0.005, a.dzc[k]), 1e-12);
    int ig = 0, jg = 0, kg = 0;
    bool found = false;
    for (int m = 0; m < 8 && !found; m++) {
        double xp = ad(Ix, (m & 1) ? -tx : tx), yp = ad(Iy, (m & 2) ? -ty : ty), zp = ad(Iz, (m & 4) ? -tz : tz);
        ig = ib_index(xq, xp, d.nx);
        jg = ib_index(yq, yp, d.ny);
        kg = ib_index(zq, zp, d.nz);
        bool good = true;
        for (int g = 0; g < 8 && good; g++) {
            int s = ib_status(a, ig + (g & 1), jg + ((g >> 1) & 1), kg + (g >> 2));
            good = s == T_FLUID || s == T_IMMERSED;
        }
        found = good && Ix >= xq[ig] && Ix <= xq[ig + 1] && Iy >= yq[jg] && Iy <= yq[jg + 1] && Iz >= zq[kg] &&
                Iz <= zq[kg + 1];
    }
    int nf = 0;
    int fi[8], fj[8], fk[8];
    if (found) {
        nf = 8;
        for (int g = 0; g < 8; g++) {
            fi[g] = ig + (g & 1);
            fj[g] = jg + ((g >> 1) & 1);
            fk[g] = kg + (g >> 2);
        }
    } else {
        ig = imn(imx(ib_index(xq, Ix, d.nx), 0), d.nx - 1);
        jg = imn(imx(ib_index(yq, Iy, d.ny), 0), d.ny - 1);
        kg = imn(imx(ib_index(zq, Iz, d.nz), 0), d.nz - 1);
        double dmin = 1e12;
        int gf = -1;
        for (int g = 0; g < 8; g++) {
            int p = ig + (g & 1), q = jg + ((g >> 1) & 1), r = kg + (g >> 2);
            if (ib_status(a, p, q, r) == T_FLUID) {
                double dd = dist3(Ix, Iy, Iz, xq[p], yq[q], zq[r]);
                if (dd < dmin) {
                    dmin = dd;
                    gf = g;
                }
            }
        }
        if (gf >= 0) {
            nf = 1;
            fi[0] = ig + (gf & 1);
            fj[0] = jg + ((gf >> 1) & 1);
            fk[0] = kg + (gf >> 2);
        }
    }
    double df = dist3(Ix, Iy, Iz, Cx, Cy, Cz);
    double coef = (fabs(ds) <= 1e-10 && fabs(df) <= 1e-10) ? 1.0 : dv(ds, df);
    double w[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (nf == 8) {
        double x7 = xq[fi[7]], y7 = yq[fj[7]], z7 = zq[fk[7]];
        double x0 = xq[fi[0]], y0 = yq[fj[0]], z0 = zq[fk[0]];
        double al = dv(sb(x7, Ix), sb(x7, x0)), be = dv(sb(y7, Iy), sb(y7, y0)), ga = dv(sb(z7, Iz), sb(z7, z0));
        double al1 = sb(1.0, al), be1 = sb(1.0, be), ga1 = sb(1.0, ga);
        w[0] = ml(ml(al, be), ga);
        w[1] = ml(ml(al1, be), ga);
        w[2] = ml(ml(al, be1), ga);
        w[3] = ml(ml(al1, be1), ga);
        w[4] = ml(ml(al, be), ga1);
        w[5] = ml(ml(al1, be), ga1);
        w[6] = ml(ml(al, be1), ga1);
        w[7] = ml(ml(al1, be1), ga1);
    } else if (nf == 1) {
        w[0] = 1.0;
    }
    double fc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    double bc;
    if (!a.neumann) {
        bc = ad(1.0, coef);
        for (int g = 0; g < nf; g++) fc[g] = ml(w[g], coef);
    } else if (nf == 1) {
        bc = -ad(ds, df);
        fc[0] = -w[0];
    } else {
        double A[8][8];
        for (int r = 0; r < 8; r++)
            for (int c = 0; c < 8; c++) A[r][c] = 0.0;
        bool self = false;
        int r = 0;
        for (int g = 0; g < nf; g++) {
            if (fi[g] == i && fj[g] == j && fk[g] == k) {
                self = true;
            } else {
                double x = sb(xq[fi[g]], Ix), y = sb(yq[fj[g]], Iy), z = sb(zq[fk[g]], Iz);
                A[r][0] = ml(ml(x, y), z);
                A[r][1] = ml(x, y);
                A[r][2] = ml(x, z);
                A[r][3] = ml(y, z);
                A[r][4] = x;
                A[r][5] = y;
                A[r][6] = z;
                A[r][7] = 1.0;
                r++;
            }
        }
        if (self) {
            double xc = sb(Cx, Ix), yc = sb(Cy, Iy), zc = sb(Cz, Iz);
            A[r][0] = ad(ad(ml(ml(nx, yc), zc), ml(ml(ny, xc), zc)), ml(ml(nz, xc), yc));
            A[r][1] = ad(ml(yc, nx), ml(xc, ny));
            A[r][2] = ad(ml(zc, nx), ml(xc, nz));
            A[r][3] = ad(ml(zc, ny), ml(yc, nz));
            A[r][4] = nx;
            A[r][5] = ny;
            A[r][6] = nz;
            A[r][7] = 0.0;
        }
        ib_gauss_jordan(A);
        bc = ad(-ad(ds, df), self ? A[7][7] : 0.0);
        r = 0;
        for (int g = 0; g < nf; g++) {
            if (fi[g] == i && fj[g] == j && fk[g] == k) {
                fc[g] = 0.0;
            } else {
                fc[g] = -A[7][r];
                r++;
            }
        }
    }
    for (int g = 0; g < nf; g++)
        if (isnan(fc[g]) || isinf(fc[g])) {
            fc[g] = 0.0;
            bc = 0.0;
        }
    o.im[t] = L;
    o.nf[t] = nf;
    for (int g = 0; g < 8; g++) {
        o.fidx[(long long)t * 8 + g] = g < nf ? (int)(((long long)fk[g] * d.NY + fj[g]) * d.NX + fi[g]) : 0;
        o.fcoef[(long long)t * 8 + g] = g < nf ? fc[g] : 0.0;
    }
    o.bcoef[t] = bc;
    if (o.pts) {
        double *p = o.pts + (long long)t * 12;
        p[0] = nx; p[1] = ny; p[2] = nz;
        p[3] = Cx; p[4] = Cy; p[5] = Cz;
        p[6] = Ix; p[7] = Iy; p[8] = Iz;
        p[9] = Px; p[10] = Py; p[11] = Pz;
    }
}

}  // namespace

long long geom_scratch_doubles(const Dims &d)
{
    dim3 g = g3(d);
    return 3 * d.n + (long long)g.x * g.y * g.z + 1;
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
    // phi ping-pongs between the c sdf output and scratch
    double *pa = o->sdf[0], *pb = scratch, *s0 = scratch + d.n, *nD = scratch + 2 * d.n, *part = scratch + 3 * d.n,
           *tot = part + np;
    // Surface_initialize (only a bottom surface): phi_0 = yc - interface_position
    k_sdf_guess<<<G, B38, 0, s>>>(g, ipos, pa);
    k_ls_prep<<<G, B38, 0, s>>>(g, pa, s0, nD);
    // Levelset_reinitialize: stop after the step whose NORM2 change is below
    // 1e-5, or once the counter passes max_iterations + 1
    int c = 0;
    double W = 0.0;
    for (;;) {
        k_ls_step<<<G, B38, 0, s>>>(g, pa, s0, nD, a.dt, c == 0, pb, part);
        k_sum<<<1, 1024, 0, s>>>(np, part, tot);
        double e2 = 0.0;
        cudaMemcpyAsync(&e2, tot, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        std::swap(pa, pb);
        W = std::sqrt(e2);
        if (c > a.max_iterations + 1 || W < 1.0e-5) break;
        c++;
    }
    o->iterations = c + 1;
    o->last_error = W;
    double *p = o->sdf[0];
    if (pa != p) cudaMemcpyAsync(p, pa, sizeof(double) * d.n, cudaMemcpyDeviceToDevice, s);
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

// IMMERSED nodes of one status array: row offsets (NY*NZ + 1 ints) and the count
cudaError_t geom_ib_count(cudaStream_t s, const Dims &d, const uint8_t *st, int *rows, int *n)
{
    long long nr = (long long)d.NY * d.NZ;
    k_ib_count<<<(unsigned)((nr + 255) / 256), 256, 0, s>>>(d, st, rows);
    k_ib_scan<<<1, 1024, 0, s>>>(nr, rows);
    cudaError_t e = cudaMemcpyAsync(n, rows + nr, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

// Immersed_setup_q_immersed_nodes (Immersed.c:546-616) for quantity q
// (0..3 = u, v, w, c) into o (o.n entries; node: o.n ints of scratch)
cudaError_t geom_ib_build(cudaStream_t s, const GeomArgs &a, int q, const double *sdf, const uint8_t *st,
                          const int *rows, int *node, const GeomIb &o)
{
    const Dims &d = a.d;
    long long nr = (long long)d.NY * d.NZ;
    if (o.n == 0) return cudaGetLastError();
    k_ib_emit<<<(unsigned)((nr + 255) / 256), 256, 0, s>>>(d, st, rows, node);
    IbArgs b;
    b.d = d;
    b.neumann = q == 3;
    b.ni = d.nx + (q == 0);
    b.nj = d.ny + (q == 1);
    b.nk = d.nz + (q == 2);
    b.xq = q == 0 ? a.xu : a.xc;
    b.yq = q == 1 ? a.yv : a.yc;
    b.zq = q == 2 ? a.zw : a.zc;
    b.dxc = a.dxc; b.dyc = a.dyc; b.dzc = a.dzc;
    b.sdf = sdf;
    b.st = st;
    k_ib_stencil<<<(unsigned)((o.n + 127) / 128), 128, 0, s>>>(b, o.n, node, o);
    return cudaGetLastError();
}
