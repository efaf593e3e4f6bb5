// k_pcg.cu -- FP64 conjugate-gradient vector kernels for the pressure solve
// (volume-weighted system on the compact physical-cell layout).  Dot products
// reduce by warp shuffles into a fixed set of per-block partials that one
// block sums in a fixed order, so results are run-to-run deterministic.
#include "turb_internal.cuh"
#include "turb_mg.cuh"

namespace {

constexpr int NP = 1024;   // blocks of the grid-stride reductions
constexpr int BS = 256;

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void block_store(double v, double *dst)
{
    __shared__ double sm[32];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double r = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        r = warp_sum(r);
        if (threadIdx.x == 0) *dst = r;
    }
    __syncthreads();
}

struct Cell {
    int i, j, k;
};
__device__ __forceinline__ Cell cell_of(const MgDevLevel &L, long long c)
{
    Cell o;
    o.i = (int)(c % L.nx);
    long long t = c / L.nx;
    o.j = (int)(t % L.ny);
    o.k = (int)(t / L.ny);
    return o;
}

__device__ __forceinline__ double s_apply(const MgDevLevel &L, const double *__restrict__ x, long long c, Cell q)
{
    long long nx = L.nx, nxy = (long long)L.nx * L.ny;
    double dyz = L.dyd[q.j] * L.dzd[q.k], dxz = L.dxd[q.i] * L.dzd[q.k], dxy = L.dxd[q.i] * L.dyd[q.j];
    double o = 0.0, d = 0.0, f, xc = x[c];
    if (q.i > 0) { f = dyz * L.rfxd[q.i]; d += f; o += f * x[c - 1]; }
    if (q.i < L.nx - 1) { f = dyz * L.rfxd[q.i + 1]; d += f; o += f * x[c + 1]; }
    if (q.j > 0) { f = dxz * L.rfyd[q.j]; d += f; o += f * x[c - nx]; }
    if (q.j < L.ny - 1) { f = dxz * L.rfyd[q.j + 1]; d += f; o += f * x[c + nx]; }
    if (q.k > 0) { f = dxy * L.rfzd[q.k]; d += f; o += f * x[c - nxy]; }
    if (q.k < L.nz - 1) { f = dxy * L.rfzd[q.k + 1]; d += f; o += f * x[c + nxy]; }
    if (q.i == L.nx - 1 && q.j == L.ny - 1 && q.k == L.nz - 1) d += L.pin;
    return d * xc - o;
}

__global__ void k_gather(Dims d, MgDevLevel L, const double *__restrict__ phi, const double *__restrict__ pb,
                         double *__restrict__ x, double *__restrict__ bw)
{
    long long n = (long long)L.nx * L.ny * L.nz;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        Cell q = cell_of(L, c);
        long long p = d.at(q.i, q.j, q.k);
        x[c] = phi[p];
        bw[c] = (L.dxd[q.i] * L.dyd[q.j] * L.dzd[q.k]) * pb[p];
    }
}

__global__ void k_scatter(Dims d, MgDevLevel L, const double *__restrict__ x, double *__restrict__ phi)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int k = blockIdx.y;
    int j = (int)(t / d.NX), i = (int)(t - (long long)j * d.NX);
    if (j >= d.NY) return;
    long long p = d.at(i, j, k);
    phi[p] = (i < L.nx && j < L.ny && k < L.nz) ? x[((long long)k * L.ny + j) * L.nx + i] : 0.0;
}

__global__ void k_resid(MgDevLevel L, const double *__restrict__ bw, const double *__restrict__ x,
                        double *__restrict__ r, double *__restrict__ part)
{
    long long n = (long long)L.nx * L.ny * L.nz;
    double acc = 0.0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double v = bw[c] - s_apply(L, x, c, cell_of(L, c));
        r[c] = v;
        acc += v * v;
    }
    block_store(acc, part + blockIdx.x);
}

__global__ void k_apply(MgDevLevel L, const double *__restrict__ p, double *__restrict__ q, double *__restrict__ part)
{
    long long n = (long long)L.nx * L.ny * L.nz;
    double acc = 0.0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double v = s_apply(L, p, c, cell_of(L, c));
        q[c] = v;
        acc += p[c] * v;
    }
    block_store(acc, part + blockIdx.x);
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

__global__ void k_reduce(const double *__restrict__ part, int nvals, double *__restrict__ dst)
{
    for (int v = 0; v < nvals; v++) {
        double acc = 0.0;
        for (int t = threadIdx.x; t < NP; t += blockDim.x) acc += part[v * NP + t];
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

long long ncell(const MgDevLevel &L) { return (long long)L.nx * L.ny * L.nz; }

}  // namespace

int pcg_nparts() { return NP; }

void pcg_gather(cudaStream_t s, const Dims &d, const MgDevLevel &L0, const double *phi_da, const double *pb_da,
                double *x, double *bw)
{
    k_gather<<<NP, BS, 0, s>>>(d, L0, phi_da, pb_da, x, bw);
}

void pcg_scatter(cudaStream_t s, const Dims &d, const MgDevLevel &L0, const double *x, double *phi_da)
{
    long long nij = (long long)d.NX * d.NY;
    dim3 g((unsigned)((nij + BS - 1) / BS), d.NZ);
    k_scatter<<<g, BS, 0, s>>>(d, L0, x, phi_da);
}

void pcg_resid(cudaStream_t s, const MgDevLevel &L0, const double *bw, const double *x, double *r, double *part)
{
    k_resid<<<NP, BS, 0, s>>>(L0, bw, x, r, part);
}

void pcg_apply(cudaStream_t s, const MgDevLevel &L0, const double *p, double *q, double *part)
{
    k_apply<<<NP, BS, 0, s>>>(L0, p, q, part);
}

void pcg_dot(cudaStream_t s, long long n, const double *a, const double *b, double *part)
{
    k_dot<<<NP, BS, 0, s>>>(n, a, b, part);
}

void pcg_dot2(cudaStream_t s, long long n, const double *r, const double *z, const double *rold, double *part)
{
    k_dot2<<<NP, BS, 0, s>>>(n, r, z, rold, part);
}

void pcg_reduce(cudaStream_t s, const double *part, int nvals, double *dst)
{
    k_reduce<<<1, 1024, 0, s>>>(part, nvals, dst);
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
