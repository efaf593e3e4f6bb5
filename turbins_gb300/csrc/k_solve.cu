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

constexpr int HBX = 32, HBY = 8, KC = 4;   // 32x8 threads over (i, j), KC planes per thread
constexpr int KCJ = 2;                      // planes per thread of the FP32 Jacobi sweep

__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double sm[32];
    int lt = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((lt & 31) == 0) sm[lt >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (lt < 32) {
        r = (lt < (nt >> 5)) ? sm[lt] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;   // valid in thread (0, 0)
}

__device__ __forceinline__ long long part_index()
{
    return ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}

// offsets of the six neighbours; an absent neighbour (coefficient 0) is
// redirected to the point itself so that every load stays inside the field
struct Nb {
    long long w, e, s, n, b, f;
};
__device__ __forceinline__ Nb nb_of(const Dims &d, int i, int j, int k)
{
    Nb o;
    o.w = i > 0 ? -1 : 0;
    o.e = i < d.NX - 1 ? 1 : 0;
    o.s = j > 0 ? -(long long)d.PX : 0;
    o.n = j < d.NY - 1 ? (long long)d.PX : 0;
    o.b = k > 0 ? -d.plane : 0;
    o.f = k < d.NZ - 1 ? d.plane : 0;
    return o;
}

__device__ __forceinline__ bool is_stencil(int q, int s)
{
    return (q == 3) ? (s == T_FLUID) : (s == T_FLUID || s == T_BUFFER_SOLID);
}

// (A x)_p and the diagonal of a non-immersed row (rows of *_form_LHS_matrix
// plus 1/dt); coefficients are products of 1-D tables, zero where absent
// axy = apx[i] + apy[j], formed once per (i, j) column by the caller
__device__ __forceinline__ double helm_ax(const Dims &d, const HelmTab &h, int s, double a_dt, double axy,
                                          const double *__restrict__ x, long long p, int i, int j, int k,
                                          double &dg)
{
    if (!is_stencil(h.q, s)) {
        dg = h.ap_solid + a_dt;
        return dg * x[p];
    }
    Nb o = nb_of(d, i, j, k);
    dg = axy + (h.apz[k] + a_dt);
    double acc = dg * x[p];
    acc = fma(h.aw[i], x[p + o.w], acc);
    acc = fma(h.ae[i], x[p + o.e], acc);
    acc = fma(h.as[j], x[p + o.s], acc);
    acc = fma(h.an[j], x[p + o.n], acc);
    acc = fma(h.ab[k], x[p + o.b], acc);
    acc = fma(h.af[k], x[p + o.f], acc);
    return acc;
}

__global__ void k_helm_apply(Dims d, HelmTab h, const uint8_t *__restrict__ st, double a_dt,
                             const double *__restrict__ x, double *__restrict__ y)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const double axy = h.apx[i] + h.apy[j];
    for (int kk = 0; kk < KC; kk++) {
        int k = blockIdx.z * KC + kk;
        if (k >= d.NZ) break;
        long long p = d.at(i, j, k);
        int s = st[p];
        if (s == T_IMMERSED) continue;
        double dg;
        y[p] = helm_ax(d, h, s, a_dt, axy, x, p, i, j, k, dg);
    }
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
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    double r2 = 0.0;
    if (i < d.NX && j < d.NY) {
        const double axy = h.apx[i] + h.apy[j];
        for (int kk = 0; kk < KC; kk++) {
            int k = blockIdx.z * KC + kk;
            if (k >= d.NZ) break;
            long long p = d.at(i, j, k);
            int s = st[p];
            if (s == T_IMMERSED) continue;
            double dg, ax = helm_ax(d, h, s, a_dt, axy, x, p, i, j, k, dg);
            double r = b[p] - ax;
            xn[p] = x[p] + r / dg;
            r2 = fma(r, r, r2);
        }
    }
    double bs = block_sum(r2);
    if (threadIdx.x == 0 && threadIdx.y == 0) part[part_index()] = bs;
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
// xn = x + e over the whole field (FP64 accumulation of the FP32 correction)
__global__ void k_add_corr(long long n, const double *__restrict__ x, const float *__restrict__ e,
                           double *__restrict__ xn)
{
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        xn[p] = x[p] + (double)e[p];
}

// r = b - A x in FP64, rounded to FP32 for the inner solve; |r|^2 partials.
// The FP64 pipe bounds this kernel, so the row is accumulated as
// -(diag x - b + sum a_nb x_nb) (no separate subtraction) and apz[k] + 1/dt
// is formed once per plane of the block: nine FP64 operations per point
__global__ void k_helm_resid64(Dims d, HelmTab h, const uint8_t *__restrict__ st, double a_dt,
                               const double *__restrict__ b, const double *__restrict__ x,
                               float *__restrict__ rf, double *__restrict__ part)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    __shared__ double zdt[KC];
    {
        int t = threadIdx.y * blockDim.x + threadIdx.x, k = blockIdx.z * KC + t;
        if (t < KC) zdt[t] = k < d.NZ ? h.apz[k] + a_dt : 0.0;
    }
    __syncthreads();
    double r2 = 0.0;
    pdl_trigger();   // the immersed rows' kernel (disjoint points) may start at once
    if (i < d.NX && j < d.NY) {
        const double axy = h.apx[i] + h.apy[j];
        for (int kk = 0; kk < KC; kk++) {
            int k = blockIdx.z * KC + kk;
            if (k >= d.NZ) break;
            long long p = d.at(i, j, k);
            int s = st[p];
            if (s == T_IMMERSED) continue;
            double r;
            if (!is_stencil(h.q, s)) {
                r = b[p] - (h.ap_solid + a_dt) * x[p];
            } else {
                Nb o = nb_of(d, i, j, k);
                double acc = fma(axy + zdt[kk], x[p], -b[p]);
                acc = fma(h.aw[i], x[p + o.w], acc);
                acc = fma(h.ae[i], x[p + o.e], acc);
                acc = fma(h.as[j], x[p + o.s], acc);
                acc = fma(h.an[j], x[p + o.n], acc);
                acc = fma(h.ab[k], x[p + o.b], acc);
                acc = fma(h.af[k], x[p + o.f], acc);
                r = -acc;
            }
            rf[p] = (float)r;
            r2 = fma(r, r, r2);
        }
    }
    double bs = block_sum(r2);
    if (threadIdx.x == 0 && threadIdx.y == 0) part[part_index()] = bs;
}

__global__ void k_ib_resid64(IbDev ib, const double *__restrict__ b, const double *__restrict__ x,
                             float *__restrict__ rf, double *__restrict__ part)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double r2 = 0.0;
    if (t < ib.n) {
        long long im = ib.im[t];
        double acc = ib.diag[t] * x[im];
        int c = ib.cnt[t];
        for (int g = 0; g < c; g++) acc += ib.val[t * 8 + g] * x[ib.col[t * 8 + g]];
        double r = b[im] - acc;
        rf[im] = (float)r;
        r2 = r * r;
    }
    double bs = block_sum(r2);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    pdl_wait();   // as in k_ib_jac32: end after the stencil residual
}

// inner FP32 Jacobi sweep on A e = r (first sweep from e = 0), four points
// of a row per thread: e, r, status and the j+-1 / k+-1 neighbours are
// 16-byte (4-byte for status) loads, the x tables are padded to the pitch.
// Immersed points are left to k_ib_jac32 (not written here, so the two
// kernels may overlap); pad columns (i >= NX) are not written.
// four blocks of 32 x 8 per SM (64 registers): measured 17 % faster at
// 513x257x257 than the three that 76 registers allow
__global__ void __launch_bounds__(HBX *HBY, 4) k_helm_jac32v(Dims d, HelmTabF h, const uint8_t *__restrict__ st, float a_dt,
                              const float *__restrict__ r, const float *__restrict__ e, float *__restrict__ en,
                              int first)
{
    pdl_trigger();   // the immersed rows' kernel may start at once
    const int i0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x), j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i0 >= d.NX || j >= d.NY) return;
    const float4 apx = *reinterpret_cast<const float4 *>(h.apx + i0);
    const float4 aw = *reinterpret_cast<const float4 *>(h.aw + i0);
    const float4 ae = *reinterpret_cast<const float4 *>(h.ae + i0);
    const float apxv[4] = {apx.x, apx.y, apx.z, apx.w}, awv[4] = {aw.x, aw.y, aw.z, aw.w};
    const float aev[4] = {ae.x, ae.y, ae.z, ae.w};
    const float apyj = h.apy[j], asj = h.as[j], anj = h.an[j];
    const int nvalid = min(4, d.NX - i0);
    for (int kk = 0; kk < KCJ; kk++) {
        const int k = blockIdx.z * KCJ + kk;
        if (k >= d.NZ) break;
        const long long p = d.at(i0, j, k);
        const uchar4 s4 = *reinterpret_cast<const uchar4 *>(st + p);
        const int sv[4] = {s4.x, s4.y, s4.z, s4.w};
        const float4 r4 = *reinterpret_cast<const float4 *>(r + p);
        const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
        const float apzk = h.apz[k], abk = h.ab[k], afk = h.af[k];
        float out[4];
        if (first) {
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const bool stn = is_stencil(h.q, sv[t]);
                const float dg = stn ? __fadd_rn(__fadd_rn(__fadd_rn(apxv[t], apyj), apzk), a_dt)
                                     : __fadd_rn(h.ap_solid, a_dt);
                out[t] = __fmul_rn(rv[t], __frcp_rn(dg));
            }
        } else {
            const float4 e4 = *reinterpret_cast<const float4 *>(e + p);
            const float ev[4] = {e4.x, e4.y, e4.z, e4.w};
            const float xw = i0 > 0 ? e[p - 1] : ev[0];
            const float xe = i0 + 4 < d.NX ? e[p + 4] : ev[3];
            const float4 s_ = j > 0 ? *reinterpret_cast<const float4 *>(e + p - d.PX) : e4;
            const float4 n_ = j < d.NY - 1 ? *reinterpret_cast<const float4 *>(e + p + d.PX) : e4;
            const float4 b_ = k > 0 ? *reinterpret_cast<const float4 *>(e + p - d.plane) : e4;
            const float4 f_ = k < d.NZ - 1 ? *reinterpret_cast<const float4 *>(e + p + d.plane) : e4;
            const float sv_[4] = {s_.x, s_.y, s_.z, s_.w}, nv_[4] = {n_.x, n_.y, n_.z, n_.w};
            const float bv_[4] = {b_.x, b_.y, b_.z, b_.w}, fv_[4] = {f_.x, f_.y, f_.z, f_.w};
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const bool stn = is_stencil(h.q, sv[t]);
                const float dg = stn ? __fadd_rn(__fadd_rn(__fadd_rn(apxv[t], apyj), apzk), a_dt)
                                     : __fadd_rn(h.ap_solid, a_dt);
                float acc = __fmul_rn(dg, ev[t]);
                if (stn) {
                    acc = __fmaf_rn(awv[t], t == 0 ? xw : ev[t - 1], acc);
                    acc = __fmaf_rn(aev[t], t == 3 ? xe : ev[t + 1], acc);
                    acc = __fmaf_rn(asj, sv_[t], acc);
                    acc = __fmaf_rn(anj, nv_[t], acc);
                    acc = __fmaf_rn(abk, bv_[t], acc);
                    acc = __fmaf_rn(afk, fv_[t], acc);
                }
                out[t] = __fmaf_rn(__fadd_rn(rv[t], -acc), __frcp_rn(dg), ev[t]);
            }
        }
        const bool ib4 = sv[0] == T_IMMERSED || sv[1] == T_IMMERSED || sv[2] == T_IMMERSED || sv[3] == T_IMMERSED;
        if (nvalid == 4 && !ib4) {
            *reinterpret_cast<float4 *>(en + p) = make_float4(out[0], out[1], out[2], out[3]);
        } else {
            for (int t = 0; t < nvalid; t++)
                if (sv[t] != T_IMMERSED) en[p + t] = out[t];
        }
    }
}

// The same sweep (not the first one) marching along k: a block of 32 x 8
// threads owns a tile of 128 x 8 points of every plane of a chunk of JZ
// planes.  Each thread keeps its four points of planes k-1, k, k+1 in
// registers (e of plane k+1 is loaded while plane k is computed); the x and
// y neighbours come from the plane-k tile in shared memory, whose halo rows
// j-1, j+8 and columns are loaded by the edge threads.  e is read from
// memory about once per sweep instead of once per neighbour, and every
// point's arithmetic and neighbour substitutions are k_helm_jac32v's, so the
// results are the same bits.
constexpr int JZ = 16;                 // planes per block
constexpr int JTX = 4 * HBX + 2;       // tile row: 128 points and two halo columns
__global__ void __launch_bounds__(HBX *HBY, 3) k_helm_jac32z(Dims d, HelmTabF h, const uint8_t *__restrict__ st,
                                                          float a_dt, const float *__restrict__ r,
                                                          const float *__restrict__ e, float *__restrict__ en)
{
    __shared__ float tile[HBY + 2][JTX];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = 4 * (blockIdx.x * HBX + tx), j = blockIdx.y * HBY + ty;
    const int k0 = blockIdx.z * JZ, k1 = min(k0 + JZ, d.NZ);
    const bool act = i0 < d.NX && j < d.NY;
    const int nvalid = act ? min(4, d.NX - i0) : 0;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float apxv[4] = {}, awv[4] = {}, aev[4] = {};
    float apyj = 0.f, asj = 0.f, anj = 0.f;
    if (act) {
        const float4 apx = *reinterpret_cast<const float4 *>(h.apx + i0);
        const float4 aw = *reinterpret_cast<const float4 *>(h.aw + i0);
        const float4 ae = *reinterpret_cast<const float4 *>(h.ae + i0);
        apxv[0] = apx.x; apxv[1] = apx.y; apxv[2] = apx.z; apxv[3] = apx.w;
        awv[0] = aw.x; awv[1] = aw.y; awv[2] = aw.z; awv[3] = aw.w;
        aev[0] = ae.x; aev[1] = ae.y; aev[2] = ae.z; aev[3] = ae.w;
        apyj = h.apy[j]; asj = h.as[j]; anj = h.an[j];
    }
    const long long pj = act ? d.at(i0, j, 0) : 0;
    // the edge threads also load a halo row (j-1 for the first row of the
    // block, j+1 for the last) and a halo column (left / right of the tile)
    const int jh = ty == 0 ? j - 1 : (ty == HBY - 1 ? j + 1 : -1);
    const bool hrow = act && jh >= 0 && jh < d.NY;
    const long long ph = hrow ? d.at(i0, jh, 0) : 0;
    const bool hl = act && tx == 0 && i0 > 0, hr_ = act && tx == HBX - 1 && i0 + 4 < d.NX;
    auto in_k = [&](int k) { return act && k >= 0 && k < d.NZ; };
    auto ld4 = [&](const float *a, long long base, int k) -> float4 {
        return in_k(k) ? *reinterpret_cast<const float4 *>(a + base + (long long)k * d.plane) : z4;
    };
    // plane k0 and the planes around it; the rest is loaded one plane ahead
    float4 eb = ld4(e, pj, k0 - 1), ec = ld4(e, pj, k0), ef = ld4(e, pj, k0 + 1);
    float4 rc = ld4(r, pj, k0);
    uchar4 sc = in_k(k0) ? *reinterpret_cast<const uchar4 *>(st + pj + (long long)k0 * d.plane) : make_uchar4(0, 0, 0, 0);
    float4 hc = (hrow && k0 < d.NZ) ? ld4(e, ph, k0) : z4;
    float xlc = hl ? e[pj + (long long)k0 * d.plane - 1] : 0.f, xrc = hr_ ? e[pj + (long long)k0 * d.plane + 4] : 0.f;
    for (int k = k0; k < k1; k++) {
        const float ev[4] = {ec.x, ec.y, ec.z, ec.w};
        float *row = &tile[ty + 1][1 + 4 * tx];
        row[0] = ev[0]; row[1] = ev[1]; row[2] = ev[2]; row[3] = ev[3];
        if (hrow) {
            float *hrw = &tile[ty == 0 ? 0 : HBY + 1][1 + 4 * tx];
            hrw[0] = hc.x; hrw[1] = hc.y; hrw[2] = hc.z; hrw[3] = hc.w;
        }
        if (hl) tile[ty + 1][0] = xlc;
        if (hr_) tile[ty + 1][JTX - 1] = xrc;
        __syncthreads();
        // the next plane's loads, in flight while this plane is computed
        const int kn = k + 1;
        const float4 ef2 = ld4(e, pj, kn + 1), rn = ld4(r, pj, kn);
        const uchar4 sn = in_k(kn) ? *reinterpret_cast<const uchar4 *>(st + pj + (long long)kn * d.plane)
                                   : make_uchar4(0, 0, 0, 0);
        const float4 hn = (hrow && kn < d.NZ) ? ld4(e, ph, kn) : z4;
        const float xln = (hl && kn < d.NZ) ? e[pj + (long long)kn * d.plane - 1] : 0.f;
        const float xrn = (hr_ && kn < d.NZ) ? e[pj + (long long)kn * d.plane + 4] : 0.f;
        if (act) {
            const long long p = pj + (long long)k * d.plane;
            const int sv[4] = {sc.x, sc.y, sc.z, sc.w};
            const float rv[4] = {rc.x, rc.y, rc.z, rc.w};
            const float apzk = h.apz[k], abk = h.ab[k], afk = h.af[k];
            const float xw = i0 > 0 ? tile[ty + 1][4 * tx] : ev[0];
            const float xe = i0 + 4 < d.NX ? tile[ty + 1][4 * tx + 5] : ev[3];
            float sv_[4], nv_[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                sv_[t] = j > 0 ? tile[ty][1 + 4 * tx + t] : ev[t];
                nv_[t] = j < d.NY - 1 ? tile[ty + 2][1 + 4 * tx + t] : ev[t];
            }
            const float4 b_ = k > 0 ? eb : ec, f_ = k < d.NZ - 1 ? ef : ec;
            const float bv_[4] = {b_.x, b_.y, b_.z, b_.w}, fv_[4] = {f_.x, f_.y, f_.z, f_.w};
            float out[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const bool stn = is_stencil(h.q, sv[t]);
                const float dg = stn ? __fadd_rn(__fadd_rn(__fadd_rn(apxv[t], apyj), apzk), a_dt)
                                     : __fadd_rn(h.ap_solid, a_dt);
                float acc = __fmul_rn(dg, ev[t]);
                if (stn) {
                    acc = __fmaf_rn(awv[t], t == 0 ? xw : ev[t - 1], acc);
                    acc = __fmaf_rn(aev[t], t == 3 ? xe : ev[t + 1], acc);
                    acc = __fmaf_rn(asj, sv_[t], acc);
                    acc = __fmaf_rn(anj, nv_[t], acc);
                    acc = __fmaf_rn(abk, bv_[t], acc);
                    acc = __fmaf_rn(afk, fv_[t], acc);
                }
                out[t] = __fmaf_rn(__fadd_rn(rv[t], -acc), __frcp_rn(dg), ev[t]);
            }
            if (nvalid == 4) {
                *reinterpret_cast<float4 *>(en + p) = make_float4(out[0], out[1], out[2], out[3]);
            } else {
                for (int t = 0; t < nvalid; t++) en[p + t] = out[t];
            }
        }
        __syncthreads();
        eb = ec;
        ec = ef;
        ef = ef2;
        rc = rn;
        sc = sn;
        hc = hn;
        xlc = xln;
        xrc = xrn;
    }
}

__global__ void k_helm_jac32(Dims d, HelmTabF h, const uint8_t *__restrict__ st, float a_dt,
                             const float *__restrict__ r, const float *__restrict__ e, float *__restrict__ en,
                             int first)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    for (int kk = 0; kk < KC; kk++) {
        int k = blockIdx.z * KC + kk;
        if (k >= d.NZ) break;
        long long p = d.at(i, j, k);
        int s = st[p];
        if (s == T_IMMERSED) continue;
        bool stencil = is_stencil(h.q, s);
        float dg = stencil ? (h.apx[i] + h.apy[j] + h.apz[k] + a_dt) : (h.ap_solid + a_dt);
        float inv = __frcp_rn(dg);
        if (first) { en[p] = r[p] * inv; continue; }
        float acc = dg * e[p];
        if (stencil) {
            Nb o = nb_of(d, i, j, k);
            acc = fmaf(h.aw[i], e[p + o.w], acc);
            acc = fmaf(h.ae[i], e[p + o.e], acc);
            acc = fmaf(h.as[j], e[p + o.s], acc);
            acc = fmaf(h.an[j], e[p + o.n], acc);
            acc = fmaf(h.ab[k], e[p + o.b], acc);
            acc = fmaf(h.af[k], e[p + o.f], acc);
        }
        en[p] = fmaf(r[p] - acc, inv, e[p]);
    }
}

__global__ void k_ib_jac32(IbDevF ib, const float *__restrict__ r, const float *__restrict__ e,
                           float *__restrict__ en, int first)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ib.n) {
        long long im = ib.im[t];
        float inv = __frcp_rn(ib.diag[t]);
        if (first) {
            en[im] = r[im] * inv;
        } else {
            float acc = ib.diag[t] * e[im];
            int c = ib.cnt[t];
            for (int g = 0; g < c; g++) acc += ib.val[t * 8 + g] * e[ib.col[t * 8 + g]];
            en[im] = fmaf(r[im] - acc, inv, e[im]);
        }
    }
    // launched as a programmatic dependent of the stencil sweep (which
    // writes the other points of en): end only after it has completed, so
    // that the kernels after this one see both
    pdl_wait();
}

inline dim3 hgrid(const Dims &d)
{
    return dim3((unsigned)((d.NX + HBX - 1) / HBX), (unsigned)((d.NY + HBY - 1) / HBY),
                (unsigned)((d.NZ + KC - 1) / KC));
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
    dim3 g = hgrid(d);
    return (long long)g.x * g.y * g.z;
}

long long norm_parts() { return NPART; }

void launch_helm_apply(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                       const double *x, double *y, const IbDev &ib)
{
    k_helm_apply<<<hgrid(d), dim3(HBX, HBY), 0, s>>>(d, h, st, a_dt, x, y);
    if (ib.n > 0) k_ib_apply<<<(ib.n + 255) / 256, 256, 0, s>>>(ib, x, y);
}

// part must hold helm_parts(d) + (ib.n+255)/256 entries
void launch_helm_jacobi(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                        const double *b, const double *x, double *xn, const IbDev &ib, double *part,
                        long long nparts)
{
    k_helm_jacobi<<<hgrid(d), dim3(HBX, HBY), 0, s>>>(d, h, st, a_dt, b, x, xn, part);
    if (ib.n > 0) k_ib_jacobi<<<(ib.n + 255) / 256, 256, 0, s>>>(ib, b, x, xn, part + nparts);
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

void launch_add_corr(cudaStream_t s, long long n, const double *x, const float *e, double *xn)
{
    k_add_corr<<<1216, 256, 0, s>>>(n, x, e, xn);
}

// a launch with the programmatic stream serialisation attribute: the kernel
// may start while the one before it on the stream runs (the immersed rows'
// kernels are written for that: they read nothing the stencil kernel writes,
// write only immersed points, and end with pdl_wait)
template <typename... P, typename... A>
static void launch_pdl(void (*k)(P...), dim3 g, dim3 b, cudaStream_t s, A... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}

void launch_helm_resid64(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                         const double *b, const double *x, float *rf, const IbDev &ib, double *part,
                         long long nparts)
{
    k_helm_resid64<<<hgrid(d), dim3(HBX, HBY), 0, s>>>(d, h, st, a_dt, b, x, rf, part);
    if (ib.n > 0) launch_pdl(k_ib_resid64, dim3((ib.n + 255) / 256), dim3(256), s, ib, b, x, rf, part + nparts);
}

// marching 1: the FP32 Jacobi sweeps after the first march along k through
// shared-memory plane tiles (k_helm_jac32z); 0: k_helm_jac32v throughout
void launch_helm_jac32(cudaStream_t s, const Dims &d, const HelmTabF &h, const uint8_t *st, float a_dt,
                       const float *r, const float *e, float *en, const IbDevF &ib, int first, int marching)
{
    dim3 g((unsigned)((d.NX + 4 * HBX - 1) / (4 * HBX)), (unsigned)((d.NY + HBY - 1) / HBY),
           (unsigned)((d.NZ + KCJ - 1) / KCJ));
    if (!first && marching) {
        dim3 gz((unsigned)((d.NX + 4 * HBX - 1) / (4 * HBX)), (unsigned)((d.NY + HBY - 1) / HBY),
                (unsigned)((d.NZ + JZ - 1) / JZ));
        k_helm_jac32z<<<gz, dim3(HBX, HBY), 0, s>>>(d, h, st, a_dt, r, e, en);
        // k_helm_jac32z writes placeholders at immersed points: the immersed
        // rows go after it in plain stream order
        if (ib.n > 0) k_ib_jac32<<<(ib.n + 255) / 256, 256, 0, s>>>(ib, r, e, en, first);
        return;
    }
    k_helm_jac32v<<<g, dim3(HBX, HBY), 0, s>>>(d, h, st, a_dt, r, e, en, first);
    if (ib.n > 0) launch_pdl(k_ib_jac32, dim3((ib.n + 255) / 256), dim3(256), s, ib, r, e, en, first);
}
