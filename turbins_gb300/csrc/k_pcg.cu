// k_pcg.cu -- FP64 conjugate-gradient vector kernels for the pressure solve
// (volume-weighted system on the compact physical-cell layout).  Dot products
// reduce by warp shuffles into a fixed set of per-block partials that one
// block sums in a fixed order, so results are run-to-run deterministic.
#include "turb_internal.cuh"
#include "turb_mg.cuh"

namespace {

constexpr int NP = 4096;   // blocks of the grid-stride reductions
constexpr int BS = 256;

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void block_store(double v, double *dst)
{
    __shared__ double sm[32];
    int lt = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    v = warp_sum(v);
    if ((lt & 31) == 0) sm[lt >> 5] = v;
    __syncthreads();
    if (lt < 32) {
        double r = (lt < (nt >> 5)) ? sm[lt] : 0.0;
        r = warp_sum(r);
        if (lt == 0) *dst = r;
    }
    __syncthreads();
}

constexpr int KC = 4;   // planes per thread in the 3-D stencil kernels
__device__ __forceinline__ long long blk3() { return ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x; }

struct Cell {
    int i, j, k;
};

// (S x)_c = dz_k [cxy x_c - sum_xy a_n x_n] + (dx dy) [zs x_c - zb x_b - zf x_f]
// (+ the corner pin): the x and y face coefficients times the other cell
// widths are constants of the thread's (i, j) column and are formed once,
// the z ones are constants of a plane; absent faces have a zero coefficient
// (their neighbour index is redirected to the cell itself).  Eleven FP64
// operations per cell.
struct SCol {
    double axw, axe, ays, ayn, cxy, wz;
};

__device__ __forceinline__ SCol s_col(const MgDevLevel &L, int i, int j)
{
    SCol r;
    double dx = L.dxd[i], dy = L.dyd[j];
    double fxw = i > 0 ? L.rfxd[i] : 0.0, fxe = i < L.nx - 1 ? L.rfxd[i + 1] : 0.0;
    double fys = j > 0 ? L.rfyd[j] : 0.0, fyn = j < L.ny - 1 ? L.rfyd[j + 1] : 0.0;
    r.axw = dy * fxw;
    r.axe = dy * fxe;
    r.ays = dx * fys;
    r.ayn = dx * fyn;
    r.cxy = (r.axw + r.axe) + (r.ays + r.ayn);
    r.wz = dx * dy;
    return r;
}

// z face coefficients of one plane (zero for an absent face) and their sum
struct SPlane {
    double zb, zf, zs, dz;
};

__device__ __forceinline__ SPlane s_plane(const MgDevLevel &L, int k)
{
    SPlane r;
    r.zb = k > 0 ? L.rfzd[k] : 0.0;
    r.zf = k < L.nz - 1 ? L.rfzd[k + 1] : 0.0;
    r.zs = r.zb + r.zf;
    r.dz = L.dzd[k];
    return r;
}

// the KC planes of a block, formed once by its first threads
__device__ __forceinline__ void s_planes(const MgDevLevel &L, SPlane *sp)
{
    int t = threadIdx.y * blockDim.x + threadIdx.x, k = blockIdx.z * KC + t;
    if (t < KC && k < L.nz) sp[t] = s_plane(L, k);
    __syncthreads();
}

__device__ __forceinline__ double s_apply(const MgDevLevel &L, const SCol &a, const SPlane &z,
                                          const double *__restrict__ x, long long c, Cell q)
{
    long long nx = L.nx, nxy = (long long)L.nx * L.ny;
    double xc = x[c];
    double xw = x[c - (q.i > 0 ? 1 : 0)], xe = x[c + (q.i < L.nx - 1 ? 1 : 0)];
    double xs = x[c - (q.j > 0 ? nx : 0)], xn = x[c + (q.j < L.ny - 1 ? nx : 0)];
    double xb = x[c - (q.k > 0 ? nxy : 0)], xf = x[c + (q.k < L.nz - 1 ? nxy : 0)];
    double t = fma(a.axw, xw, fma(a.axe, xe, fma(a.ays, xs, a.ayn * xn)));
    double xy = fma(a.cxy, xc, -t);
    double sz = fma(z.zs, xc, -fma(z.zb, xb, z.zf * xf));
    double v = fma(z.dz, xy, a.wz * sz);
    if (q.i == L.nx - 1 && q.j == L.ny - 1 && q.k == L.nz - 1) v = fma(L.pin, xc, v);
    return v;
}

__global__ void k_gather(Dims d, MgDevLevel L, const double *__restrict__ phi, const double *__restrict__ pb,
                         double *__restrict__ x, double *__restrict__ bw)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= L.nx || j >= L.ny) return;
    long long c = ((long long)k * L.ny + j) * L.nx + i, p = d.at(i, j, k);
    x[c] = phi[p];
    bw[c] = (L.dxd[i] * L.dyd[j] * L.dzd[k]) * pb[p];
}

__global__ void k_scatter(Dims d, MgDevLevel L, const double *__restrict__ x, double *__restrict__ phi)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= d.NX || j >= d.NY) return;
    long long p = d.at(i, j, k);
    phi[p] = (i < L.nx && j < L.ny && k < L.nz) ? x[((long long)k * L.ny + j) * L.nx + i] : 0.0;
}

// r = W b - S x with partial |r|^2 per block (3-D launch, KC planes per thread)
__global__ void k_resid(MgDevLevel L, const double *__restrict__ bw, const double *__restrict__ x,
                        double *__restrict__ r, double *__restrict__ part)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    __shared__ SPlane sp[KC];
    s_planes(L, sp);
    double acc = 0.0;
    if (i < L.nx && j < L.ny) {
        const SCol a = s_col(L, i, j);
        for (int kk = 0; kk < KC; kk++) {
            int k = blockIdx.z * KC + kk;
            if (k >= L.nz) break;
            long long c = ((long long)k * L.ny + j) * L.nx + i;
            Cell q{i, j, k};
            double v = bw[c] - s_apply(L, a, sp[kk], x, c, q);
            r[c] = v;
            acc += v * v;
        }
    }
    block_store(acc, part + blk3());
}

// q = S p with partial p.q per block
__global__ void k_apply(MgDevLevel L, const double *__restrict__ p, double *__restrict__ q, double *__restrict__ part)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    __shared__ SPlane sp[KC];
    s_planes(L, sp);
    double acc = 0.0;
    if (i < L.nx && j < L.ny) {
        const SCol a = s_col(L, i, j);
        for (int kk = 0; kk < KC; kk++) {
            int k = blockIdx.z * KC + kk;
            if (k >= L.nz) break;
            long long c = ((long long)k * L.ny + j) * L.nx + i;
            Cell cc{i, j, k};
            double v = s_apply(L, a, sp[kk], p, c, cc);
            q[c] = v;
            acc += p[c] * v;
        }
    }
    block_store(acc, part + blk3());
}

__global__ void k_dot(long long n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ part)
{
    double acc = 0.0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        acc += a[c] * b[c];
    block_store(acc, part + blockIdx.x);
}

__global__ void k_dot2(long long n, const double *__restrict__ r, const double *__restrict__ z,
                       const double *__restrict__ ro, double *__restrict__ part)
{
    double a = 0.0, b = 0.0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double zc = z[c];
        a += r[c] * zc;
        b += ro[c] * zc;
    }
    block_store(a, part + blockIdx.x);
    block_store(b, part + NP + blockIdx.x);
}

__global__ void k_reduce(const double *__restrict__ part, int nvals, int nper, double *__restrict__ dst)
{
    for (int v = 0; v < nvals; v++) {
        double acc = 0.0;
        for (int t = threadIdx.x; t < nper; t += blockDim.x) acc += part[(long long)v * nper + t];
        block_store(acc, dst + v);
    }
}

__global__ void k_scalars(PcgScal *sc, int what)
{
    if (threadIdx.x != 0) return;
    if (what == 0) {
        sc->beta = sc->rz_old != 0.0 ? (sc->rz - sc->zr_old) / sc->rz_old : 0.0;
    } else {
        sc->alpha = sc->pq != 0.0 ? sc->rz / sc->pq : 0.0;
        sc->rz_old = sc->rz;
    }
}

__global__ void k_pupdate(long long n, const double *__restrict__ z, double *__restrict__ p, const PcgScal *sc, int first)
{
    double beta = first ? 0.0 : sc->beta;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        p[c] = first ? z[c] : z[c] + beta * p[c];
}

__global__ void k_xrupdate(long long n, double *__restrict__ x, double *__restrict__ r, double *__restrict__ ro,
                           const double *__restrict__ p, const double *__restrict__ q, const PcgScal *sc,
                           double *__restrict__ part)
{
    double alpha = sc->alpha, acc = 0.0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double rc = r[c];
        ro[c] = rc;
        x[c] += alpha * p[c];
        rc -= alpha * q[c];
        r[c] = rc;
        acc += rc * rc;
    }
    block_store(acc, part + blockIdx.x);
}

__global__ void k_lincomb(long long n, double a, const double *__restrict__ x, double b, const double *__restrict__ y,
                          double *__restrict__ out)
{
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        out[c] = a * x[c] + b * y[c];
}

__global__ void k_f2(long long n, const double *__restrict__ a, float *__restrict__ b)
{
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        b[c] = (float)a[c];
}
__global__ void k_d2(long long n, const float *__restrict__ a, double *__restrict__ b)
{
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        b[c] = (double)a[c];
}
__global__ void k_copy(long long n, const double *__restrict__ a, double *__restrict__ b)
{
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        b[c] = a[c];
}

// Galerkin fit of the initial guess (projection onto earlier solutions):
// direction m is d_m = y_m - x0 with S-image s_m = w_m - bw + r1 when w_m is
// the right-hand side y_m was solved for (S y_m = w_m to that solve's
// tolerance), or s_m = r1 - w_m when w_m is the computed residual of a
// candidate y_m.  Per block: G[a][b] = d_a . s_b and g[a] = d_a . r1, value
// v = a * GAL_MAX + b (g at GAL_MAX * GAL_MAX + a) in part[v * GAL_NP + block].
constexpr int GAL_NP = 512;
__global__ void __launch_bounds__(BS) k_gal_dots(long long n, GalDirs dd, const double *__restrict__ x0,
                                                 const double *__restrict__ r1, const double *__restrict__ bw,
                                                 double *__restrict__ part)
{
    double G[GAL_MAX][GAL_MAX] = {}, gv[GAL_MAX] = {};
    const int nd = dd.nd;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double xc = x0[c], rc = r1[c], sb = rc - bw[c];
        double d[GAL_MAX], sv[GAL_MAX];
#pragma unroll
        for (int m = 0; m < GAL_MAX; m++) {
            if (m < nd) {
                d[m] = dd.y[m][c] - xc;
                sv[m] = dd.resid[m] ? rc - dd.w[m][c] : dd.w[m][c] + sb;
            } else {
                d[m] = 0.0;
                sv[m] = 0.0;
            }
        }
#pragma unroll
        for (int a = 0; a < GAL_MAX; a++) {
            gv[a] = fma(d[a], rc, gv[a]);
#pragma unroll
            for (int b = 0; b < GAL_MAX; b++) G[a][b] = fma(d[a], sv[b], G[a][b]);
        }
    }
#pragma unroll
    for (int a = 0; a < GAL_MAX; a++) {
#pragma unroll
        for (int b = 0; b < GAL_MAX; b++) block_store(G[a][b], part + (long long)(a * GAL_MAX + b) * GAL_NP + blockIdx.x);
        block_store(gv[a], part + (long long)(GAL_MAX * GAL_MAX + a) * GAL_NP + blockIdx.x);
    }
}

// x = x0 + sum_m alpha_m (y_m - x0)
__global__ void k_gal_update(long long n, GalDirs dd, GalCoef al, const double *__restrict__ x0, double *__restrict__ x)
{
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double xc = x0[c], v = xc;
        for (int m = 0; m < dd.nd; m++) v = fma(al.a[m], dd.y[m][c] - xc, v);
        x[c] = v;
    }
}

// largest |r_c| / (dx_i dy_j dz_k): the unweighted residual b - A phi of the
// volume-weighted system, whose maximum times dt is the largest divergence
// the projection with this phi leaves.  3-D launch as k_apply (KC planes per
// thread); 1/(dx dy) once per thread and 1/dz once per plane of a block, so a
// cell costs two multiplies.  Per block maxima into part (NaN kept).
__global__ void k_rmax(MgDevLevel L, const double *__restrict__ r, double *__restrict__ part)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    __shared__ double izs[KC];
    int t = threadIdx.y * blockDim.x + threadIdx.x;
    if (t < KC && blockIdx.z * KC + t < L.nz) izs[t] = 1.0 / L.dzd[blockIdx.z * KC + t];
    __syncthreads();
    double m = 0.0;
    if (i < L.nx && j < L.ny) {
        double ixy = 1.0 / (L.dxd[i] * L.dyd[j]);
        for (int kk = 0; kk < KC; kk++) {
            int k = blockIdx.z * KC + kk;
            if (k >= L.nz) break;
            long long c = ((long long)k * L.ny + j) * L.nx + i;
            m = turb_maxbits(m, fabs(r[c]) * ixy * izs[kk]);
        }
    }
    __shared__ double sm[32];
    int lt = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    m = turb_warp_maxbits(m);
    if ((lt & 31) == 0) sm[lt >> 5] = m;
    __syncthreads();
    if (lt < 32) {
        m = lt < (nt >> 5) ? sm[lt] : 0.0;
        m = turb_warp_maxbits(m);
        if (lt == 0) part[blk3()] = m;
    }
}

__global__ void k_max_parts(const double *__restrict__ part, int n, double *__restrict__ dst)
{
    double m = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) m = turb_maxbits(m, part[t]);
    __shared__ double sm[32];
    m = turb_warp_maxbits(m);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (int)(blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
        m = turb_warp_maxbits(m);
        if (threadIdx.x == 0) *dst = m;
    }
}

long long ncell(const MgDevLevel &L) { return (long long)L.nx * L.ny * L.nz; }

}  // namespace


void pcg_gal_dots(cudaStream_t s, long long n, const GalDirs &dd, const double *x0, const double *r1,
                  const double *bw, double *part, double *dst)
{
    k_gal_dots<<<GAL_NP, BS, 0, s>>>(n, dd, x0, r1, bw, part);
    k_reduce<<<1, 1024, 0, s>>>(part, GAL_MAX * GAL_MAX + GAL_MAX, GAL_NP, dst);
}

void pcg_gal_update(cudaStream_t s, long long n, const GalDirs &dd, const GalCoef &al, const double *x0, double *x)
{
    k_gal_update<<<NP, BS, 0, s>>>(n, dd, al, x0, x);
}

int pcg_nparts() { return NP; }

static dim3 g3k(const MgDevLevel &L)
{
    return dim3((unsigned)((L.nx + 31) / 32), (unsigned)((L.ny + 7) / 8), (unsigned)((L.nz + KC - 1) / KC));
}
int pcg_stencil_parts(const MgDevLevel &L)
{
    dim3 g = g3k(L);
    return (int)(g.x * g.y * g.z);
}

void pcg_rmax(cudaStream_t s, const MgDevLevel &L0, const double *r, double *part, double *dst)
{
    k_rmax<<<g3k(L0), dim3(32, 8), 0, s>>>(L0, r, part);
    k_max_parts<<<1, 1024, 0, s>>>(part, pcg_stencil_parts(L0), dst);
}

void pcg_gather(cudaStream_t s, const Dims &d, const MgDevLevel &L0, const double *phi_da, const double *pb_da,
                double *x, double *bw)
{
    k_gather<<<dim3((L0.nx + 31) / 32, (L0.ny + 7) / 8, L0.nz), dim3(32, 8), 0, s>>>(d, L0, phi_da, pb_da, x, bw);
}

void pcg_scatter(cudaStream_t s, const Dims &d, const MgDevLevel &L0, const double *x, double *phi_da)
{
    k_scatter<<<dim3((d.NX + 31) / 32, (d.NY + 7) / 8, d.NZ), dim3(32, 8), 0, s>>>(d, L0, x, phi_da);
}

void pcg_resid(cudaStream_t s, const MgDevLevel &L0, const double *bw, const double *x, double *r, double *part)
{
    k_resid<<<g3k(L0), dim3(32, 8), 0, s>>>(L0, bw, x, r, part);
}

void pcg_apply(cudaStream_t s, const MgDevLevel &L0, const double *p, double *q, double *part)
{
    k_apply<<<g3k(L0), dim3(32, 8), 0, s>>>(L0, p, q, part);
}

void pcg_dot(cudaStream_t s, long long n, const double *a, const double *b, double *part)
{
    k_dot<<<NP, BS, 0, s>>>(n, a, b, part);
}

void pcg_dot2(cudaStream_t s, long long n, const double *r, const double *z, const double *rold, double *part)
{
    k_dot2<<<NP, BS, 0, s>>>(n, r, z, rold, part);
}

void pcg_reduce(cudaStream_t s, const double *part, int nvals, double *dst, int nper)
{
    k_reduce<<<1, 1024, 0, s>>>(part, nvals, nper > 0 ? nper : NP, dst);
}

void pcg_pupdate(cudaStream_t s, long long n, const double *z, double *p, const PcgScal *sc, int first)
{
    k_pupdate<<<NP, BS, 0, s>>>(n, z, p, sc, first);
}

void pcg_xrupdate(cudaStream_t s, long long n, double *x, double *r, double *rold, const double *p,
                  const double *q, const PcgScal *sc, double *part)
{
    k_xrupdate<<<NP, BS, 0, s>>>(n, x, r, rold, p, q, sc, part);
}

void pcg_scalars(cudaStream_t s, PcgScal *sc, int what) { k_scalars<<<1, 32, 0, s>>>(sc, what); }

void pcg_to_float(cudaStream_t s, long long n, const double *a, float *b) { k_f2<<<NP, BS, 0, s>>>(n, a, b); }
void pcg_to_double(cudaStream_t s, long long n, const float *a, double *b) { k_d2<<<NP, BS, 0, s>>>(n, a, b); }
void pcg_copy(cudaStream_t s, long long n, const double *a, double *b) { k_copy<<<NP, BS, 0, s>>>(n, a, b); }
void pcg_lincomb(cudaStream_t s, long long n, double a, const double *x, double b, const double *y, double *out)
{
    k_lincomb<<<NP, BS, 0, s>>>(n, a, x, b, y, out);
}
