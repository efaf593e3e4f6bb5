// k_solve.cu -- implicit viscous / diffusive (Helmholtz) solves and the
// reductions they use.
//
// The operator is the matrix of Velocity_{u,v,w}_form_LHS_matrix /
// Conc_form_LHS_matrix plus the 1/dt diagonal of *_modify_diagonal, applied
// matrix-free: every stencil coefficient is a product of 1-D metric arrays,
// so a row needs the 1-D tables of HelmTab only.  Immersed rows are a gather
// over <= 8 precomputed (column, value) pairs.  The solver is point-Jacobi
// iteration to the reference's test ||b - A x|| <= rtol ||b|| (KSPIBCGS
// without a preconditioner in Solver.c:269-322 reaches the same discrete
// solution); the squared residual norm is reduced in the sweep itself.
#include "turb_internal.cuh"
#include "turb_kernels.cuh"

namespace {

constexpr int HB = 256;   // block size of the Helmholtz sweeps

struct RowOut {
    double diag, ax;      // diagonal coefficient and (A x)_p
};

__device__ __forceinline__ RowOut helm_row(const Dims &d, const HelmTab &h, int s, double a_dt,
                                           const double *__restrict__ x, long long p, int i, int j, int k)
{
    RowOut o;
    bool stencil = (h.q == 3) ? (s == T_FLUID) : (s == T_FLUID || s == T_BUFFER_SOLID);
    if (stencil) {
        double dg = h.apx[i] + h.apy[j] + h.apz[k] + a_dt;
        double acc = dg * x[p];
        double c;
        c = h.aw[i]; if (c != 0.0) acc = fma(c, x[p - 1], acc);
        c = h.ae[i]; if (c != 0.0) acc = fma(c, x[p + 1], acc);
        c = h.as[j]; if (c != 0.0) acc = fma(c, x[p - d.PX], acc);
        c = h.an[j]; if (c != 0.0) acc = fma(c, x[p + d.PX], acc);
        c = h.ab[k]; if (c != 0.0) acc = fma(c, x[p - d.plane], acc);
        c = h.af[k]; if (c != 0.0) acc = fma(c, x[p + d.plane], acc);
        o.diag = dg;
        o.ax = acc;
    } else {
        double dg = h.ap_solid + a_dt;
        o.diag = dg;
        o.ax = dg * x[p];
    }
    return o;
}

__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double sm[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;   // valid in thread 0
}

__global__ void k_helm_apply(Dims d, HelmTab h, const uint8_t *__restrict__ st, double a_dt,
                             const double *__restrict__ x, double *__restrict__ y)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int k = blockIdx.y;
    int j = (int)(t / d.NX), i = (int)(t - (long long)j * d.NX);
    if (j >= d.NY) return;
    long long p = d.at(i, j, k);
    int s = st[p];
    if (s == T_IMMERSED) return;
    y[p] = helm_row(d, h, s, a_dt, x, p, i, j, k).ax;
}

// immersed rows: y = diag*x_im + sum val*x_col
__global__ void k_ib_apply(IbDev ib, const double *__restrict__ x, double *__restrict__ y)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ib.n) return;
    long long im = ib.im[t];
    double acc = ib.diag[t] * x[im];
    int c = ib.cnt[t];
    for (int g = 0; g < c; g++) acc += ib.val[t * 8 + g] * x[ib.col[t * 8 + g]];
    y[im] = acc;
}

// one Jacobi sweep xn = x + (b - A x)/diag, partial sums of |b - A x|^2
__global__ void k_helm_jacobi(Dims d, HelmTab h, const uint8_t *__restrict__ st, double a_dt,
                              const double *__restrict__ b, const double *__restrict__ x,
                              double *__restrict__ xn, double *__restrict__ part)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int k = blockIdx.y;
    int j = (int)(t / d.NX), i = (int)(t - (long long)j * d.NX);
    double r2 = 0.0;
    if (j < d.NY) {
        long long p = d.at(i, j, k);
        int s = st[p];
        if (s != T_IMMERSED) {
            RowOut o = helm_row(d, h, s, a_dt, x, p, i, j, k);
            double r = b[p] - o.ax;
            xn[p] = x[p] + r / o.diag;
            r2 = r * r;
        }
    }
    double bs = block_sum(r2);
    if (threadIdx.x == 0) part[(long long)blockIdx.y * gridDim.x + blockIdx.x] = bs;
}

__global__ void k_ib_jacobi(IbDev ib, const double *__restrict__ b, const double *__restrict__ x,
                            double *__restrict__ xn, double *__restrict__ part)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double r2 = 0.0;
    if (t < ib.n) {
        long long im = ib.im[t];
        double acc = ib.diag[t] * x[im];
        int c = ib.cnt[t];
        for (int g = 0; g < c; g++) acc += ib.val[t * 8 + g] * x[ib.col[t * 8 + g]];
        double r = b[im] - acc;
        xn[im] = x[im] + r / ib.diag[t];
        r2 = r * r;
    }
    double bs = block_sum(r2);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
}

__global__ void k_sum_final(long long n, const double *__restrict__ part, double *__restrict__ out)
{
    double v = 0.0;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) v += part[t];
    double s = block_sum(v);
    if (threadIdx.x == 0) *out = s;
}

// ---- mixed-precision defect correction -----------------------------------
// outer: x <- x + e, r = b - A x in FP64 (rounded to FP32 for the inner solve)
__global__ void k_helm_resid64(Dims d, HelmTab h, const uint8_t *__restrict__ st, double a_dt,
                               const double *__restrict__ b, const double *__restrict__ x,
                               const float *__restrict__ e, double *__restrict__ xn, float *__restrict__ rf,
                               double *__restrict__ part)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int k = blockIdx.y;
    int j = (int)(t / d.NX), i = (int)(t - (long long)j * d.NX);
    double r2 = 0.0;
    if (j < d.NY) {
        long long p = d.at(i, j, k);
        int s = st[p];
        double xp = x[p] + (double)e[p];
        xn[p] = xp;
        if (s != T_IMMERSED) {
            bool stencil = (h.q == 3) ? (s == T_FLUID) : (s == T_FLUID || s == T_BUFFER_SOLID);
            double acc;
            if (stencil) {
                double dg = h.apx[i] + h.apy[j] + h.apz[k] + a_dt, c;
                acc = dg * xp;
                c = h.aw[i]; if (c != 0.0) acc = fma(c, x[p - 1] + (double)e[p - 1], acc);
                c = h.ae[i]; if (c != 0.0) acc = fma(c, x[p + 1] + (double)e[p + 1], acc);
                c = h.as[j]; if (c != 0.0) acc = fma(c, x[p - d.PX] + (double)e[p - d.PX], acc);
                c = h.an[j]; if (c != 0.0) acc = fma(c, x[p + d.PX] + (double)e[p + d.PX], acc);
                c = h.ab[k]; if (c != 0.0) acc = fma(c, x[p - d.plane] + (double)e[p - d.plane], acc);
                c = h.af[k]; if (c != 0.0) acc = fma(c, x[p + d.plane] + (double)e[p + d.plane], acc);
            } else {
                acc = (h.ap_solid + a_dt) * xp;
            }
            double r = b[p] - acc;
            rf[p] = (float)r;
            r2 = r * r;
        }
    }
    double bs = block_sum(r2);
    if (threadIdx.x == 0) part[(long long)blockIdx.y * gridDim.x + blockIdx.x] = bs;
}

__global__ void k_ib_resid64(IbDev ib, const double *__restrict__ b, const double *__restrict__ x,
                             const float *__restrict__ e, float *__restrict__ rf, double *__restrict__ part)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double r2 = 0.0;
    if (t < ib.n) {
        long long im = ib.im[t];
        double acc = ib.diag[t] * (x[im] + (double)e[im]);
        int c = ib.cnt[t];
        for (int g = 0; g < c; g++) {
            long long q = ib.col[t * 8 + g];
            acc += ib.val[t * 8 + g] * (x[q] + (double)e[q]);
        }
        double r = b[im] - acc;
        rf[im] = (float)r;
        r2 = r * r;
    }
    double bs = block_sum(r2);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
}

// inner FP32 Jacobi sweep on A e = r (first sweep from e = 0)
__global__ void k_helm_jac32(Dims d, HelmTabF h, const uint8_t *__restrict__ st, float a_dt,
                             const float *__restrict__ r, const float *__restrict__ e, float *__restrict__ en,
                             int first)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int k = blockIdx.y;
    int j = (int)(t / d.NX), i = (int)(t - (long long)j * d.NX);
    if (j >= d.NY) return;
    long long p = d.at(i, j, k);
    int s = st[p];
    if (s == T_IMMERSED) return;
    bool stencil = (h.q == 3) ? (s == T_FLUID) : (s == T_FLUID || s == T_BUFFER_SOLID);
    float dg = stencil ? (h.apx[i] + h.apy[j] + h.apz[k] + a_dt) : (h.ap_solid + a_dt);
    if (first) { en[p] = r[p] / dg; return; }
    float acc = dg * e[p], c;
    if (stencil) {
        c = h.aw[i]; if (c != 0.0f) acc = fmaf(c, e[p - 1], acc);
        c = h.ae[i]; if (c != 0.0f) acc = fmaf(c, e[p + 1], acc);
        c = h.as[j]; if (c != 0.0f) acc = fmaf(c, e[p - d.PX], acc);
        c = h.an[j]; if (c != 0.0f) acc = fmaf(c, e[p + d.PX], acc);
        c = h.ab[k]; if (c != 0.0f) acc = fmaf(c, e[p - d.plane], acc);
        c = h.af[k]; if (c != 0.0f) acc = fmaf(c, e[p + d.plane], acc);
    }
    en[p] = e[p] + (r[p] - acc) / dg;
}

__global__ void k_ib_jac32(IbDevF ib, const float *__restrict__ r, const float *__restrict__ e,
                           float *__restrict__ en, int first)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ib.n) return;
    long long im = ib.im[t];
    if (first) { en[im] = r[im] / ib.diag[t]; return; }
    float acc = ib.diag[t] * e[im];
    int c = ib.cnt[t];
    for (int g = 0; g < c; g++) acc += ib.val[t * 8 + g] * e[ib.col[t * 8 + g]];
    en[im] = e[im] + (r[im] - acc) / ib.diag[t];
}

constexpr int NPART = 1024;

__global__ void k_norm2(long long n, const double *__restrict__ x, double *__restrict__ part)
{
    double v = 0.0;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        v += x[p] * x[p];
    double s = block_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

}  // namespace

long long helm_parts(const Dims &d)
{
    long long nij = (long long)d.NX * d.NY;
    return ((nij + HB - 1) / HB) * d.NZ;
}

long long norm_parts() { return NPART; }

void launch_helm_resid64(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                         const double *b, const double *x, const float *e, double *xn, float *rf, const IbDev &ib,
                         double *part, long long nparts)
{
    long long nij = (long long)d.NX * d.NY;
    dim3 g((unsigned)((nij + HB - 1) / HB), d.NZ);
    k_helm_resid64<<<g, HB, 0, s>>>(d, h, st, a_dt, b, x, e, xn, rf, part);
    if (ib.n > 0) k_ib_resid64<<<(ib.n + 255) / 256, 256, 0, s>>>(ib, b, x, e, rf, part + nparts);
}

void launch_helm_jac32(cudaStream_t s, const Dims &d, const HelmTabF &h, const uint8_t *st, float a_dt,
                       const float *r, const float *e, float *en, const IbDevF &ib, int first)
{
    long long nij = (long long)d.NX * d.NY;
    dim3 g((unsigned)((nij + HB - 1) / HB), d.NZ);
    k_helm_jac32<<<g, HB, 0, s>>>(d, h, st, a_dt, r, e, en, first);
    if (ib.n > 0) k_ib_jac32<<<(ib.n + 255) / 256, 256, 0, s>>>(ib, r, e, en, first);
}

void launch_helm_apply(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                       const double *x, double *y, const IbDev &ib)
{
    long long nij = (long long)d.NX * d.NY;
    dim3 g((unsigned)((nij + HB - 1) / HB), d.NZ);
    k_helm_apply<<<g, HB, 0, s>>>(d, h, st, a_dt, x, y);
    if (ib.n > 0) k_ib_apply<<<(ib.n + 255) / 256, 256, 0, s>>>(ib, x, y);
}

// part must hold helm_parts(d) + (ib.n+255)/256 entries
void launch_helm_jacobi(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                        const double *b, const double *x, double *xn, const IbDev &ib, double *part,
                        long long nparts)
{
    long long nij = (long long)d.NX * d.NY;
    dim3 g((unsigned)((nij + HB - 1) / HB), d.NZ);
    k_helm_jacobi<<<g, HB, 0, s>>>(d, h, st, a_dt, b, x, xn, part);
    long long np = nparts;
    if (ib.n > 0) {
        int nbk = (ib.n + 255) / 256;
        k_ib_jacobi<<<nbk, 256, 0, s>>>(ib, b, x, xn, part + nparts);
        np += nbk;
    }
    (void)np;
}

void launch_sum_final(cudaStream_t s, long long nparts, const double *part, double *out)
{
    k_sum_final<<<1, 1024, 0, s>>>(nparts, part, out);
}

void launch_norm2(cudaStream_t s, long long n, const double *x, double *part, long long nparts, double *out)
{
    (void)nparts;
    k_norm2<<<NPART, 256, 0, s>>>(n, x, part);
    k_sum_final<<<1, 1024, 0, s>>>(NPART, part, out);
}
