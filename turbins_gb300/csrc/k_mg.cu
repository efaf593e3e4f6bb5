// k_mg.cu -- pressure Poisson solve: geometric-multigrid-preconditioned CG.
//
// Replaces GMRES(20) + hypre BoomerAMG (Solver.c:90-265) for the system of
// Pressure_form_LHS_matrix (Pressure.c:691-936).  CG runs in FP64 on the
// volume-weighted form S = W A (W = cell volume), which is symmetric; the
// corner pin of Pressure.c:864-868 is kept as an extra diagonal term.  The
// preconditioner is one V-cycle: red-black Gauss-Seidel smoothing (2 pre, 2
// post, reversed colour order on the way up so the cycle is symmetric),
// restriction by summing children, piecewise-constant prolongation (its
// transpose), rediscretised coarse operators built from the coarse cell
// widths (so coarsening follows the y stretching), semi-coarsening of the
// directions whose mean spacing is more than twice the finest, and a dense
// inverse on the coarsest (<= 64 cells) level.  The V-cycle is templated on
// its precision: FP64 (plain method) or FP32 inside the FP64 CG (mixed).
#include "turb_internal.cuh"
#include "turb_kernels.cuh"
#include "turb_mg.cuh"

namespace {

template <typename T>
struct LevelT {
    int nx, ny, nz;
    const T *dx, *dy, *dz, *rfx, *rfy, *rfz;
    T pin;
};

template <typename T>
__device__ __forceinline__ LevelT<T> lev_of(const MgDevLevel &L);

template <>
__device__ __forceinline__ LevelT<double> lev_of<double>(const MgDevLevel &L)
{
    LevelT<double> o{L.nx, L.ny, L.nz, L.dxd, L.dyd, L.dzd, L.rfxd, L.rfyd, L.rfzd, L.pin};
    return o;
}
template <>
__device__ __forceinline__ LevelT<float> lev_of<float>(const MgDevLevel &L)
{
    LevelT<float> o{L.nx, L.ny, L.nz, L.dxf, L.dyf, L.dzf, L.rfxf, L.rfyf, L.rfzf, (float)L.pin};
    return o;
}

// S x - evaluated as  diag*x_p - sum f*x_nb ; returns (offsum, diag)
template <typename T>
__device__ __forceinline__ void s_row(const LevelT<T> &L, const T *__restrict__ x, int i, int j, int k,
                                      T &off, T &dg)
{
    long long nx = L.nx, nxy = (long long)L.nx * L.ny;
    long long c = ((long long)k * L.ny + j) * nx + i;
    T dyz = L.dy[j] * L.dz[k], dxz = L.dx[i] * L.dz[k], dxy = L.dx[i] * L.dy[j];
    T o = 0, d = 0, f;
    if (i > 0) { f = dyz * L.rfx[i]; d += f; o += f * x[c - 1]; }
    if (i < L.nx - 1) { f = dyz * L.rfx[i + 1]; d += f; o += f * x[c + 1]; }
    if (j > 0) { f = dxz * L.rfy[j]; d += f; o += f * x[c - nx]; }
    if (j < L.ny - 1) { f = dxz * L.rfy[j + 1]; d += f; o += f * x[c + nx]; }
    if (k > 0) { f = dxy * L.rfz[k]; d += f; o += f * x[c - nxy]; }
    if (k < L.nz - 1) { f = dxy * L.rfz[k + 1]; d += f; o += f * x[c + nxy]; }
    if (i == L.nx - 1 && j == L.ny - 1 && k == L.nz - 1) d += L.pin;
    off = o;
    dg = d;
}

template <typename T>
__global__ void k_invdiag(MgDevLevel Ld, T *__restrict__ invd)
{
    LevelT<T> L = lev_of<T>(Ld);
    long long n = (long long)L.nx * L.ny * L.nz;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        int i = (int)(c % L.nx), j = (int)((c / L.nx) % L.ny), k = (int)(c / ((long long)L.nx * L.ny));
        T dyz = L.dy[j] * L.dz[k], dxz = L.dx[i] * L.dz[k], dxy = L.dx[i] * L.dy[j], d = 0;
        if (i > 0) d += dyz * L.rfx[i];
        if (i < L.nx - 1) d += dyz * L.rfx[i + 1];
        if (j > 0) d += dxz * L.rfy[j];
        if (j < L.ny - 1) d += dxz * L.rfy[j + 1];
        if (k > 0) d += dxy * L.rfz[k];
        if (k < L.nz - 1) d += dxy * L.rfz[k + 1];
        if (i == L.nx - 1 && j == L.ny - 1 && k == L.nz - 1) d += L.pin;
        invd[c] = T(1) / d;
    }
}

// red-black Gauss-Seidel half sweep; zero_init: x taken as 0 on entry (first
// sweep of a cycle, colour 0 only)
template <typename T>
__global__ void k_rbgs(MgDevLevel Ld, int color, int zero_init, const T *__restrict__ b, const T *__restrict__ invd,
                       T *__restrict__ x)
{
    LevelT<T> L = lev_of<T>(Ld);
    int i2 = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (j >= L.ny) return;
    int i = 2 * i2 + ((j + k + color) & 1);
    if (i >= L.nx) return;
    long long c = ((long long)k * L.ny + j) * L.nx + i;
    if (zero_init) { x[c] = b[c] * invd[c]; return; }
    T off, dg;
    s_row<T>(L, x, i, j, k, off, dg);
    x[c] = (b[c] + off) * invd[c];
}

template <typename T>
__global__ void k_resid(MgDevLevel Ld, const T *__restrict__ b, const T *__restrict__ x, T *__restrict__ r)
{
    LevelT<T> L = lev_of<T>(Ld);
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= L.nx || j >= L.ny) return;
    long long c = ((long long)k * L.ny + j) * L.nx + i;
    T off, dg;
    s_row<T>(L, x, i, j, k, off, dg);
    r[c] = b[c] - (dg * x[c] - off);
}

template <typename T>
__device__ __forceinline__ const T *rw_of(const Xfer1D &t);
template <>
__device__ __forceinline__ const double *rw_of<double>(const Xfer1D &t) { return t.rwd; }
template <>
__device__ __forceinline__ const float *rw_of<float>(const Xfer1D &t) { return t.rwf; }
template <typename T>
__device__ __forceinline__ const T *pw0_of(const Xfer1D &t);
template <>
__device__ __forceinline__ const double *pw0_of<double>(const Xfer1D &t) { return t.w0d; }
template <>
__device__ __forceinline__ const float *pw0_of<float>(const Xfer1D &t) { return t.w0f; }
template <typename T>
__device__ __forceinline__ const T *pw1_of(const Xfer1D &t);
template <>
__device__ __forceinline__ const double *pw1_of<double>(const Xfer1D &t) { return t.w1d; }
template <>
__device__ __forceinline__ const float *pw1_of<float>(const Xfer1D &t) { return t.w1f; }

// restriction = transpose of the linear prolongation (gather over <= 4 fine
// cells per coarsened direction)
template <typename T>
__global__ void k_restrict(MgDevLevel Lf, MgDevLevel Lc, const T *__restrict__ rf, T *__restrict__ bc)
{
    int I = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y * blockDim.y + threadIdx.y, K = blockIdx.z;
    if (I >= Lc.nx || J >= Lc.ny) return;
    long long c = ((long long)K * Lc.ny + J) * Lc.nx + I;
    const T *rwx = rw_of<T>(Lf.tx), *rwy = rw_of<T>(Lf.ty), *rwz = rw_of<T>(Lf.tz);
    int nxx = Lf.tx.rcnt[I], nyy = Lf.ty.rcnt[J], nzz = Lf.tz.rcnt[K];
    T s = 0;
    for (int c3 = 0; c3 < nzz; c3++) {
        int k = Lf.tz.rf[4 * K + c3];
        T wz = rwz[4 * K + c3];
        for (int b = 0; b < nyy; b++) {
            int j = Lf.ty.rf[4 * J + b];
            T wyz = wz * rwy[4 * J + b];
            const T *row = rf + ((long long)k * Lf.ny + j) * Lf.nx;
            for (int a = 0; a < nxx; a++) s += wyz * rwx[4 * I + a] * row[Lf.tx.rf[4 * I + a]];
        }
    }
    bc[c] = s;
}

// linear prolongation (stretching-aware weights), added to the fine iterate
template <typename T>
__global__ void k_prolong(MgDevLevel Lf, MgDevLevel Lc, const T *__restrict__ xc, T *__restrict__ xf)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= Lf.nx || j >= Lf.ny) return;
    long long c = ((long long)k * Lf.ny + j) * Lf.nx + i;
    int Ix[2] = {Lf.tx.I0[i], Lf.tx.I1[i]}, Iy[2] = {Lf.ty.I0[j], Lf.ty.I1[j]}, Iz[2] = {Lf.tz.I0[k], Lf.tz.I1[k]};
    T wx[2] = {pw0_of<T>(Lf.tx)[i], pw1_of<T>(Lf.tx)[i]};
    T wy[2] = {pw0_of<T>(Lf.ty)[j], pw1_of<T>(Lf.ty)[j]};
    T wz[2] = {pw0_of<T>(Lf.tz)[k], pw1_of<T>(Lf.tz)[k]};
    T acc = 0;
#pragma unroll
    for (int d = 0; d < 2; d++) {
        if (wz[d] == T(0)) continue;
#pragma unroll
        for (int b = 0; b < 2; b++) {
            if (wy[b] == T(0)) continue;
            const T *row = xc + ((long long)Iz[d] * Lc.ny + Iy[b]) * Lc.nx;
            T wyz = wz[d] * wy[b];
#pragma unroll
            for (int a = 0; a < 2; a++)
                if (wx[a] != T(0)) acc += wyz * wx[a] * row[Ix[a]];
        }
    }
    xf[c] += acc;
}

template <typename T>
__global__ void k_coarse(int n, const double *__restrict__ ainv, const T *__restrict__ b, T *__restrict__ x)
{
    int r = threadIdx.x;
    if (r >= n) return;
    double s = 0.0;
    for (int c = 0; c < n; c++) s += ainv[r * n + c] * (double)b[c];
    x[r] = (T)s;
}

inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }
inline dim3 g3(int nx, int ny, int nz) { return dim3((unsigned)((nx + 31) / 32), (unsigned)((ny + 7) / 8), (unsigned)nz); }
const dim3 B38(32, 8, 1);

}  // namespace

template <typename T>
void mg_setup_invdiag(cudaStream_t s, const MgDevLevel &L, T *invd)
{
    k_invdiag<T><<<1024, 256, 0, s>>>(L, invd);
}

// One V-cycle from level l: input b[l], output x[l] (x starts at zero).
template <typename T>
void mg_vcycle(cudaStream_t s, const MgHier<T> &H, int l, int npre, int npost)
{
    const MgDevLevel &L = H.lev[l];
    long long n = (long long)L.nx * L.ny * L.nz;
    if (l == H.nl - 1) {
        k_coarse<T><<<1, 64, 0, s>>>((int)n, H.coarse_inv, H.b[l], H.x[l]);
        return;
    }
    dim3 g = g3((L.nx + 1) >> 1, L.ny, L.nz);
    for (int it = 0; it < npre; it++) {
        // the first colour-0 half sweep takes x = 0 (it reads no neighbours);
        // every colour-1 point is then rewritten from colour-0 values only
        k_rbgs<T><<<g, B38, 0, s>>>(L, 0, it == 0, H.b[l], H.invd[l], H.x[l]);
        k_rbgs<T><<<g, B38, 0, s>>>(L, 1, 0, H.b[l], H.invd[l], H.x[l]);
    }
    k_resid<T><<<g3(L.nx, L.ny, L.nz), B38, 0, s>>>(L, H.b[l], H.x[l], H.r[l]);
    const MgDevLevel &C = H.lev[l + 1];
    k_restrict<T><<<g3(C.nx, C.ny, C.nz), B38, 0, s>>>(L, C, H.r[l], H.b[l + 1]);
    mg_vcycle<T>(s, H, l + 1, npre, npost);
    k_prolong<T><<<g3(L.nx, L.ny, L.nz), B38, 0, s>>>(L, C, H.x[l + 1], H.x[l]);
    for (int it = 0; it < npost; it++) {
        k_rbgs<T><<<g, B38, 0, s>>>(L, 1, 0, H.b[l], H.invd[l], H.x[l]);
        k_rbgs<T><<<g, B38, 0, s>>>(L, 0, 0, H.b[l], H.invd[l], H.x[l]);
    }
}

int mg_vcycle_launches(int nl, int npre, int npost)
{
    // per non-coarsest level: 2*npre + resid + restrict + prolong + 2*npost; coarsest: 1
    return (nl - 1) * (2 * npre + 3 + 2 * npost) + 1;
}

template void mg_setup_invdiag<double>(cudaStream_t, const MgDevLevel &, double *);
template void mg_setup_invdiag<float>(cudaStream_t, const MgDevLevel &, float *);
template void mg_vcycle<double>(cudaStream_t, const MgHier<double> &, int, int, int);
template void mg_vcycle<float>(cudaStream_t, const MgHier<float> &, int, int, int);
