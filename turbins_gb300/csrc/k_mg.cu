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
    int split;
    long long half;
    // storage index of cell c = (i, j, k)
    __device__ __forceinline__ long long at(long long c, int i, int j, int k) const
    {
        return split ? ((long long)((i + j + k) & 1) * half + (c >> 1)) : c;
    }
};

__device__ __forceinline__ long long lev_at(const MgDevLevel &L, long long c, int i, int j, int k)
{
    return L.split ? ((long long)((i + j + k) & 1) * (((long long)L.nx * L.ny * L.nz) >> 1) + (c >> 1)) : c;
}

template <typename T>
__device__ __forceinline__ LevelT<T> lev_of(const MgDevLevel &L);

template <>
__device__ __forceinline__ LevelT<double> lev_of<double>(const MgDevLevel &L)
{
    LevelT<double> o{L.nx, L.ny, L.nz, L.dxd, L.dyd, L.dzd, L.rfxd, L.rfyd, L.rfzd, L.pin, L.split,
                     ((long long)L.nx * L.ny * L.nz) >> 1};
    return o;
}
template <>
__device__ __forceinline__ LevelT<float> lev_of<float>(const MgDevLevel &L)
{
    LevelT<float> o{L.nx, L.ny, L.nz, L.dxf, L.dyf, L.dzf, L.rfxf, L.rfyf, L.rfzf, (float)L.pin, L.split,
                    ((long long)L.nx * L.ny * L.nz) >> 1};
    return o;
}

// explicitly rounded arithmetic, so that every smoother variant (natural,
// colour-split, vectorised) evaluates a row with the same operations
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }

// S x - evaluated as  diag*x_p - sum f*x_nb ; returns (offsum, diag)
template <typename T>
__device__ __forceinline__ void s_row(const LevelT<T> &L, const T *__restrict__ x, int i, int j, int k,
                                      T &off, T &dg)
{
    long long nx = L.nx, nxy = (long long)L.nx * L.ny;
    long long c = ((long long)k * L.ny + j) * nx + i;
    T dyz = rmul(L.dy[j], L.dz[k]), dxz = rmul(L.dx[i], L.dz[k]), dxy = rmul(L.dx[i], L.dy[j]);
    T o = 0, d = 0, f;
    if (i > 0) { f = rmul(dyz, L.rfx[i]); d = radd(d, f); o = rfma(f, x[L.at(c - 1, i - 1, j, k)], o); }
    if (i < L.nx - 1) { f = rmul(dyz, L.rfx[i + 1]); d = radd(d, f); o = rfma(f, x[L.at(c + 1, i + 1, j, k)], o); }
    if (j > 0) { f = rmul(dxz, L.rfy[j]); d = radd(d, f); o = rfma(f, x[L.at(c - nx, i, j - 1, k)], o); }
    if (j < L.ny - 1) { f = rmul(dxz, L.rfy[j + 1]); d = radd(d, f); o = rfma(f, x[L.at(c + nx, i, j + 1, k)], o); }
    if (k > 0) { f = rmul(dxy, L.rfz[k]); d = radd(d, f); o = rfma(f, x[L.at(c - nxy, i, j, k - 1)], o); }
    if (k < L.nz - 1) { f = rmul(dxy, L.rfz[k + 1]); d = radd(d, f); o = rfma(f, x[L.at(c + nxy, i, j, k + 1)], o); }
    if (i == L.nx - 1 && j == L.ny - 1 && k == L.nz - 1) d = radd(d, L.pin);
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
        invd[L.at(c, i, j, k)] = T(1) / d;
    }
}

// one cell of a red-black Gauss-Seidel half sweep; zero_init: x taken as 0
// on entry (first sweep of a cycle, colour 0 only)
template <typename T>
__device__ __forceinline__ void rb_cell(const LevelT<T> &L, int zero_init, const T *__restrict__ b,
                                        const T *__restrict__ invd, T *__restrict__ x, int i, int j, int k)
{
    long long c = ((long long)k * L.ny + j) * L.nx + i;
    long long o = L.at(c, i, j, k);
    if (zero_init) { x[o] = rmul(b[o], invd[o]); return; }
    T off, dg;
    s_row<T>(L, x, i, j, k, off, dg);
    x[o] = rmul(radd(b[o], off), invd[o]);
}

template <typename T>
__global__ void k_rbgs(MgDevLevel Ld, int color, int zero_init, const T *__restrict__ b, const T *__restrict__ invd,
                       T *__restrict__ x)
{
    pdl_trigger();
    pdl_wait();
    LevelT<T> L = lev_of<T>(Ld);
    int i2 = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (j >= L.ny) return;
    int i = 2 * i2 + ((j + k + color) & 1);
    if (i >= L.nx) return;
    rb_cell<T>(L, zero_init, b, invd, x, i, j, k);
}

// The same half sweep on colour-split FP32 storage, four cells of one row per
// thread (nx a multiple of 8) in each of `planes` planes (2 on the large
// levels, 1 on the small ones, whose launches are latency-bound and need
// every thread they can get): the cells' own
// b and invd, their x-neighbours (other colour, indices m-1+p .. m+p for row
// parity p) and the j+-1 / k+-1 neighbours are float4 loads, the x metric
// tables come as float4 from their parity-split copies (dxp / rlp / rrp),
// indices are 32-bit, and the row constants are loaded once.  The arithmetic
// per cell is s_row's, operation for operation.
constexpr int RB4_PLANES = 2;                    // planes per thread on the large levels
constexpr long long RB4_PLANES_CELLS = 1ll << 22;   // levels of at least this many cells
__global__ void k_rbgs4(MgDevLevel Ld, int color, int zero_init, int planes, const float *__restrict__ b,
                        const float *__restrict__ invd, float *__restrict__ x)
{
    pdl_trigger();
    pdl_wait();
    const int nx = Ld.nx, ny = Ld.ny, nz = Ld.nz, hx = nx >> 1;
    const int q4 = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= ny || 4 * q4 >= hx) return;
    const int half = (int)(((long long)nx * ny * nz) >> 1), hxy = hx * ny;
    const float dyj = Ld.dyf[j], ryj = Ld.rfyf[j], ryj1 = Ld.rfyf[j + 1];
#pragma unroll
    for (int g = 0; g < RB4_PLANES; g++) {
        const int k = blockIdx.z * planes + g;
        if (g >= planes || k >= nz) break;
        const int p = (color + j + k) & 1;
        const int m0 = (k * ny + j) * hx + 4 * q4;
        const float4 bb = *reinterpret_cast<const float4 *>(b + (size_t)color * half + m0);
        const float4 dd = *reinterpret_cast<const float4 *>(invd + (size_t)color * half + m0);
        if (zero_init) {
            *reinterpret_cast<float4 *>(x + (size_t)color * half + m0) =
                make_float4(rmul(bb.x, dd.x), rmul(bb.y, dd.y), rmul(bb.z, dd.z), rmul(bb.w, dd.w));
            continue;
        }
        const float *oth = x + (size_t)(1 - color) * half;
        const float4 c4 = *reinterpret_cast<const float4 *>(oth + m0);
        float ex = 0.0f;   // the fifth x-neighbour: left of the group (p = 0) or right of it (p = 1)
        if (p == 0) { if (q4 > 0) ex = oth[m0 - 1]; }
        else { if (4 * q4 + 4 < hx) ex = oth[m0 + 4]; }
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 jm = j > 0 ? *reinterpret_cast<const float4 *>(oth + m0 - hx) : zero4;
        const float4 jp = j < ny - 1 ? *reinterpret_cast<const float4 *>(oth + m0 + hx) : zero4;
        const float4 km = k > 0 ? *reinterpret_cast<const float4 *>(oth + m0 - hxy) : zero4;
        const float4 kp = k < nz - 1 ? *reinterpret_cast<const float4 *>(oth + m0 + hxy) : zero4;
        const float4 dx4 = *reinterpret_cast<const float4 *>(Ld.dxpf + p * hx + 4 * q4);
        const float4 rl4 = *reinterpret_cast<const float4 *>(Ld.rlpf + p * hx + 4 * q4);
        const float4 rr4 = *reinterpret_cast<const float4 *>(Ld.rrpf + p * hx + 4 * q4);
        const float dzk = Ld.dzf[k];
        const float dyz = rmul(dyj, dzk);
        const float rzk = Ld.rfzf[k], rzk1 = Ld.rfzf[k + 1];
        const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
        const float bv[4] = {bb.x, bb.y, bb.z, bb.w}, dv[4] = {dd.x, dd.y, dd.z, dd.w};
        const float jmv[4] = {jm.x, jm.y, jm.z, jm.w}, jpv[4] = {jp.x, jp.y, jp.z, jp.w};
        const float kmv[4] = {km.x, km.y, km.z, km.w}, kpv[4] = {kp.x, kp.y, kp.z, kp.w};
        const float dxv[4] = {dx4.x, dx4.y, dx4.z, dx4.w};
        const float rlv[4] = {rl4.x, rl4.y, rl4.z, rl4.w}, rrv[4] = {rr4.x, rr4.y, rr4.z, rr4.w};
        float out[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int i = 2 * (4 * q4 + e) + p;
            const float xl = p == 0 ? (e == 0 ? ex : cv[e - 1]) : cv[e];
            const float xr = p == 0 ? cv[e] : (e == 3 ? ex : cv[e + 1]);
            const float dxi = dxv[e];
            const float dxz = rmul(dxi, dzk), dxy = rmul(dxi, dyj);
            float o = 0.0f, f;
            if (i > 0) { f = rmul(dyz, rlv[e]); o = rfma(f, xl, o); }
            if (i < nx - 1) { f = rmul(dyz, rrv[e]); o = rfma(f, xr, o); }
            if (j > 0) { f = rmul(dxz, ryj); o = rfma(f, jmv[e], o); }
            if (j < ny - 1) { f = rmul(dxz, ryj1); o = rfma(f, jpv[e], o); }
            if (k > 0) { f = rmul(dxy, rzk); o = rfma(f, kmv[e], o); }
            if (k < nz - 1) { f = rmul(dxy, rzk1); o = rfma(f, kpv[e], o); }
            out[e] = rmul(radd(bv[e], o), dv[e]);
        }
        *reinterpret_cast<float4 *>(x + (size_t)color * half + m0) = make_float4(out[0], out[1], out[2], out[3]);
    }
}

// The half sweep of k_rbgs4 marching along k (not the first, zero-initial
// one): a block of 32 x 8 threads owns 128 cells of its colour in each of 8
// rows of every plane of a chunk of jz planes.  The other colour's plane k
// (with a halo row above and below and a halo column either side) is a
// shared-memory tile; its planes k-1 and k+1 at the thread's own cells stay
// in registers, loaded one plane ahead.  Each cell's arithmetic is k_rbgs4's,
// operation for operation, so the results are the same bits.
constexpr int RTX = 4 * 32 + 2;
__global__ void __launch_bounds__(256, 3) k_rbgs4z(MgDevLevel Ld, int color, int jz, const float *__restrict__ b,
                                                   const float *__restrict__ invd, float *__restrict__ x)
{
    pdl_trigger();
    pdl_wait();
    __shared__ float tile[8 + 2][RTX];
    const int nx = Ld.nx, ny = Ld.ny, nz = Ld.nz, hx = nx >> 1;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int q4 = blockIdx.x * 32 + tx, j = blockIdx.y * 8 + ty;
    const int k0 = blockIdx.z * jz, k1 = min(k0 + jz, nz);
    const bool act = j < ny && 4 * q4 < hx;
    const int half = (int)(((long long)nx * ny * nz) >> 1), hxy = hx * ny;
    const float *oth = x + (size_t)(1 - color) * half;
    const float *bc = b + (size_t)color * half, *dc = invd + (size_t)color * half;
    float *xc = x + (size_t)color * half;
    const int mj = j * hx + 4 * q4;                    // plane offset of the thread's cells
    const int jh = ty == 0 ? j - 1 : (ty == 7 ? j + 1 : -1);
    const bool hrow = act && jh >= 0 && jh < ny;       // edge rows also load a halo row
    const int mh = jh * hx + 4 * q4;
    const bool hl = act && tx == 0 && q4 > 0, hr = act && tx == 31 && 4 * q4 + 4 < hx;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    auto ld = [&](const float *a, int off, int k) -> float4 {
        return (act && k >= 0 && k < nz) ? *reinterpret_cast<const float4 *>(a + k * hxy + off) : z4;
    };
    const float dyj = act ? Ld.dyf[j] : 0.f;
    const float ryj = act ? Ld.rfyf[j] : 0.f, ryj1 = act ? Ld.rfyf[j + 1] : 0.f;
    float4 ob = ld(oth, mj, k0 - 1), oc = ld(oth, mj, k0), of = ld(oth, mj, k0 + 1);
    float4 bb = ld(bc, mj, k0), dd = ld(dc, mj, k0);
    float4 hc = (hrow && k0 < nz) ? ld(oth, mh, k0) : z4;
    float xl = (hl && k0 < nz) ? oth[k0 * hxy + mj - 1] : 0.f, xr = (hr && k0 < nz) ? oth[k0 * hxy + mj + 4] : 0.f;
    for (int k = k0; k < k1; k++) {
        float *row = &tile[ty + 1][1 + 4 * tx];
        row[0] = oc.x; row[1] = oc.y; row[2] = oc.z; row[3] = oc.w;
        if (hrow) {
            float *h = &tile[ty == 0 ? 0 : 9][1 + 4 * tx];
            h[0] = hc.x; h[1] = hc.y; h[2] = hc.z; h[3] = hc.w;
        }
        if (hl) tile[ty + 1][0] = xl;
        if (hr) tile[ty + 1][RTX - 1] = xr;
        __syncthreads();
        const int kn = k + 1;
        const float4 of2 = ld(oth, mj, kn + 1), bn = ld(bc, mj, kn), dn = ld(dc, mj, kn);
        const float4 hn = (hrow && kn < nz) ? ld(oth, mh, kn) : z4;
        const float xln = (hl && kn < nz) ? oth[kn * hxy + mj - 1] : 0.f;
        const float xrn = (hr && kn < nz) ? oth[kn * hxy + mj + 4] : 0.f;
        if (act) {
            const int p = (color + j + k) & 1;
            const float cv[4] = {oc.x, oc.y, oc.z, oc.w};
            // the fifth x-neighbour: left of the group (p = 0) or right of it (p = 1)
            float ex = 0.0f;
            if (p == 0) { if (q4 > 0) ex = tile[ty + 1][4 * tx]; }
            else { if (4 * q4 + 4 < hx) ex = tile[ty + 1][4 * tx + 5]; }
            float jmv[4], jpv[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                jmv[e] = j > 0 ? tile[ty][1 + 4 * tx + e] : 0.f;
                jpv[e] = j < ny - 1 ? tile[ty + 2][1 + 4 * tx + e] : 0.f;
            }
            const float4 km = k > 0 ? ob : z4, kp = k < nz - 1 ? of : z4;
            const float kmv[4] = {km.x, km.y, km.z, km.w}, kpv[4] = {kp.x, kp.y, kp.z, kp.w};
            const float bv[4] = {bb.x, bb.y, bb.z, bb.w}, dv[4] = {dd.x, dd.y, dd.z, dd.w};
            const float dzk = Ld.dzf[k];
            const float dyz = rmul(dyj, dzk);
            const float rzk = Ld.rfzf[k], rzk1 = Ld.rfzf[k + 1];
            float out[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int i = 2 * (4 * q4 + e) + p;
                const float xlv = p == 0 ? (e == 0 ? ex : cv[e - 1]) : cv[e];
                const float xrv = p == 0 ? cv[e] : (e == 3 ? ex : cv[e + 1]);
                const float dxi = Ld.dxf[i];
                const float dxz = rmul(dxi, dzk), dxy = rmul(dxi, dyj);
                float o = 0.0f, f;
                if (i > 0) { f = rmul(dyz, Ld.rfxf[i]); o = rfma(f, xlv, o); }
                if (i < nx - 1) { f = rmul(dyz, Ld.rfxf[i + 1]); o = rfma(f, xrv, o); }
                if (j > 0) { f = rmul(dxz, ryj); o = rfma(f, jmv[e], o); }
                if (j < ny - 1) { f = rmul(dxz, ryj1); o = rfma(f, jpv[e], o); }
                if (k > 0) { f = rmul(dxy, rzk); o = rfma(f, kmv[e], o); }
                if (k < nz - 1) { f = rmul(dxy, rzk1); o = rfma(f, kpv[e], o); }
                out[e] = rmul(radd(bv[e], o), dv[e]);
            }
            *reinterpret_cast<float4 *>(xc + k * hxy + mj) = make_float4(out[0], out[1], out[2], out[3]);
        }
        __syncthreads();
        ob = oc;
        oc = of;
        of = of2;
        bb = bn;
        dd = dn;
        hc = hn;
        xl = xln;
        xr = xrn;
    }
}

template <typename T>
__device__ __forceinline__ void resid_cell(const LevelT<T> &L, const T *__restrict__ b, const T *__restrict__ x,
                                           T *__restrict__ r, int i, int j, int k)
{
    long long c = ((long long)k * L.ny + j) * L.nx + i;
    T off, dg;
    s_row<T>(L, x, i, j, k, off, dg);
    long long o = L.at(c, i, j, k);
    r[c] = radd(b[o], -rfma(dg, x[o], -off));
}

template <typename T>
__global__ void k_resid(MgDevLevel Ld, const T *__restrict__ b, const T *__restrict__ x, T *__restrict__ r)
{
    pdl_trigger();
    pdl_wait();
    LevelT<T> L = lev_of<T>(Ld);
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= L.nx || j >= L.ny) return;
    resid_cell<T>(L, b, x, r, i, j, k);
}

// residual r = b - S x of a colour-split FP32 level (nx a multiple of 8),
// eight cells of one row per thread: cells 2(m0+e) and 2(m0+e)+1 of the row
// live at index m0+e of colour halves c0 = (j+k)&1 and c0^1, so every x and
// b access is a float4 (two scalars for the row ends); r is written in the
// natural order the restriction reads.  Per cell the arithmetic is s_row's.
__global__ void __launch_bounds__(256, 4) k_resid8(MgDevLevel Ld, const float *__restrict__ b, const float *__restrict__ x,
                                                   float *__restrict__ r)
{
    pdl_trigger();
    pdl_wait();
    const int nx = Ld.nx, ny = Ld.ny, nz = Ld.nz, hx = nx >> 1;
    int q = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (j >= ny || 4 * q >= hx) return;
    const int half = (int)(((long long)nx * ny * nz) >> 1), hxy = hx * ny;
    const int c0 = (j + k) & 1;
    const int m0 = (k * ny + j) * hx + 4 * q;
    const float *h0 = x + (size_t)c0 * half, *h1 = x + (size_t)(c0 ^ 1) * half;
    auto ld4 = [](const float *p) { return *reinterpret_cast<const float4 *>(p); };
    auto inter = [](float4 a, float4 b, float (&v)[8]) {   // cells 2e from a, 2e+1 from b
        v[0] = a.x; v[1] = b.x; v[2] = a.y; v[3] = b.y; v[4] = a.z; v[5] = b.z; v[6] = a.w; v[7] = b.w;
    };
    auto inter4 = [](float4 a, float4 b, float *v) {   // a then b
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    };
    float xc[8], bc[8], xjm[8], xjp[8], xkm[8], xkp[8];
    inter(ld4(h0 + m0), ld4(h1 + m0), xc);
    inter(ld4(b + (size_t)c0 * half + m0), ld4(b + (size_t)(c0 ^ 1) * half + m0), bc);
    // rows j+-1 and planes k+-1 have the opposite colour at the same i
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    inter(j > 0 ? ld4(h1 + m0 - hx) : z4, j > 0 ? ld4(h0 + m0 - hx) : z4, xjm);
    inter(j < ny - 1 ? ld4(h1 + m0 + hx) : z4, j < ny - 1 ? ld4(h0 + m0 + hx) : z4, xjp);
    inter(k > 0 ? ld4(h1 + m0 - hxy) : z4, k > 0 ? ld4(h0 + m0 - hxy) : z4, xkm);
    inter(k < nz - 1 ? ld4(h1 + m0 + hxy) : z4, k < nz - 1 ? ld4(h0 + m0 + hxy) : z4, xkp);
    const int i0 = 8 * q;
    const float xl = i0 > 0 ? h1[m0 - 1] : 0.0f;             // cell i0-1: colour c0^1, pair m0-1
    const float xr = i0 + 8 < nx ? h0[m0 + 4] : 0.0f;        // cell i0+8: colour c0, pair m0+4
    const float dyj = Ld.dyf[j], dzk = Ld.dzf[k];
    const float dyz = rmul(dyj, dzk);
    const float ryj = Ld.rfyf[j], ryj1 = Ld.rfyf[j + 1], rzk = Ld.rfzf[k], rzk1 = Ld.rfzf[k + 1];
    // the x tables of cells i0 .. i0+7 (and face i0+8) as float4 loads
    float dxv[8], rxv[9];
    inter4(ld4(Ld.dxf + i0), ld4(Ld.dxf + i0 + 4), dxv);
    inter4(ld4(Ld.rfxf + i0), ld4(Ld.rfxf + i0 + 4), rxv);
    rxv[8] = Ld.rfxf[i0 + 8];
    float out[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
        const int i = i0 + e;
        const float dxi = dxv[e];
        const float dxz = rmul(dxi, dzk), dxy = rmul(dxi, dyj);
        const float xw = e == 0 ? xl : xc[e - 1], xe = e == 7 ? xr : xc[e + 1];
        float o = 0.0f, d = 0.0f, f;
        if (i > 0) { f = rmul(dyz, rxv[e]); d = radd(d, f); o = rfma(f, xw, o); }
        if (i < nx - 1) { f = rmul(dyz, rxv[e + 1]); d = radd(d, f); o = rfma(f, xe, o); }
        if (j > 0) { f = rmul(dxz, ryj); d = radd(d, f); o = rfma(f, xjm[e], o); }
        if (j < ny - 1) { f = rmul(dxz, ryj1); d = radd(d, f); o = rfma(f, xjp[e], o); }
        if (k > 0) { f = rmul(dxy, rzk); d = radd(d, f); o = rfma(f, xkm[e], o); }
        if (k < nz - 1) { f = rmul(dxy, rzk1); d = radd(d, f); o = rfma(f, xkp[e], o); }
        if (i == nx - 1 && j == ny - 1 && k == nz - 1) d = radd(d, (float)Ld.pin);
        out[e] = radd(bc[e], -rfma(d, xc[e], -o));
    }
    float *rr = r + ((size_t)(k * ny + j) * nx + i0);
    *reinterpret_cast<float4 *>(rr) = make_float4(out[0], out[1], out[2], out[3]);
    *reinterpret_cast<float4 *>(rr + 4) = make_float4(out[4], out[5], out[6], out[7]);
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
// full-weighting restriction to coarse cell (I, J, K) and linear
// prolongation (stretching-aware weights) added to fine cell (i, j, k);
// explicitly rounded, so the kernels and the fused tail agree bit for bit
template <typename T>
__device__ __forceinline__ void restrict_cell(const MgDevLevel &Lf, const MgDevLevel &Lc, const T *__restrict__ rf,
                                              T *__restrict__ bc, int I, int J, int K)
{
    long long c = ((long long)K * Lc.ny + J) * Lc.nx + I;
    const T *rwx = rw_of<T>(Lf.tx), *rwy = rw_of<T>(Lf.ty), *rwz = rw_of<T>(Lf.tz);
    int nxx = Lf.tx.rcnt[I], nyy = Lf.ty.rcnt[J], nzz = Lf.tz.rcnt[K];
    T s = 0;
    for (int c3 = 0; c3 < nzz; c3++) {
        int k = Lf.tz.rf[4 * K + c3];
        T wz = rwz[4 * K + c3];
        for (int b = 0; b < nyy; b++) {
            int j = Lf.ty.rf[4 * J + b];
            T wyz = rmul(wz, rwy[4 * J + b]);
            const T *row = rf + ((long long)k * Lf.ny + j) * Lf.nx;
            for (int a = 0; a < nxx; a++) s = rfma(rmul(wyz, rwx[4 * I + a]), row[Lf.tx.rf[4 * I + a]], s);
        }
    }
    bc[lev_at(Lc, c, I, J, K)] = s;
}

template <typename T>
__device__ __forceinline__ void prolong_cell(const MgDevLevel &Lf, const MgDevLevel &Lc, const T *__restrict__ xc,
                                             T *__restrict__ xf, int i, int j, int k)
{
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
            long long row = ((long long)Iz[d] * Lc.ny + Iy[b]) * Lc.nx;
            T wyz = rmul(wz[d], wy[b]);
#pragma unroll
            for (int a = 0; a < 2; a++)
                if (wx[a] != T(0)) acc = rfma(rmul(wyz, wx[a]), xc[lev_at(Lc, row + Ix[a], Ix[a], Iy[b], Iz[d])], acc);
        }
    }
    long long o = lev_at(Lf, c, i, j, k);
    xf[o] = radd(xf[o], acc);
}

template <typename T>
__global__ void k_restrict(MgDevLevel Lf, MgDevLevel Lc, const T *__restrict__ rf, T *__restrict__ bc)
{
    pdl_trigger();
    pdl_wait();
    int I = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y * blockDim.y + threadIdx.y, K = blockIdx.z;
    if (I >= Lc.nx || J >= Lc.ny) return;
    restrict_cell<T>(Lf, Lc, rf, bc, I, J, K);
}

template <typename T>
__global__ void k_prolong(MgDevLevel Lf, MgDevLevel Lc, const T *__restrict__ xc, T *__restrict__ xf)
{
    pdl_trigger();
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= Lf.nx || j >= Lf.ny) return;
    prolong_cell<T>(Lf, Lc, xc, xf, i, j, k);
}

// eight consecutive values (cells i0..i0+7 of row (j, k)) of a level's FP32
// storage; nx a multiple of 8, i0 a multiple of 8
__device__ __forceinline__ void ld8(const MgDevLevel &L, const float *a, int i0, int j, int k, float (&v)[8])
{
    const int hx = L.nx >> 1;
    if (L.split) {
        const int half = (int)(((long long)L.nx * L.ny * L.nz) >> 1), c0 = (j + k) & 1;
        const int m0 = (k * L.ny + j) * hx + (i0 >> 1);
        const float4 a0 = *reinterpret_cast<const float4 *>(a + (size_t)c0 * half + m0);
        const float4 a1 = *reinterpret_cast<const float4 *>(a + (size_t)(c0 ^ 1) * half + m0);
        v[0] = a0.x; v[1] = a1.x; v[2] = a0.y; v[3] = a1.y; v[4] = a0.z; v[5] = a1.z; v[6] = a0.w; v[7] = a1.w;
    } else {
        const float *p = a + ((size_t)(k * L.ny + j) * L.nx + i0);
        const float4 a0 = *reinterpret_cast<const float4 *>(p), a1 = *reinterpret_cast<const float4 *>(p + 4);
        v[0] = a0.x; v[1] = a0.y; v[2] = a0.z; v[3] = a0.w; v[4] = a1.x; v[5] = a1.y; v[6] = a1.z; v[7] = a1.w;
    }
}
__device__ __forceinline__ void st8(const MgDevLevel &L, float *a, int i0, int j, int k, const float (&v)[8])
{
    const int hx = L.nx >> 1;
    if (L.split) {
        const int half = (int)(((long long)L.nx * L.ny * L.nz) >> 1), c0 = (j + k) & 1;
        const int m0 = (k * L.ny + j) * hx + (i0 >> 1);
        *reinterpret_cast<float4 *>(a + (size_t)c0 * half + m0) = make_float4(v[0], v[2], v[4], v[6]);
        *reinterpret_cast<float4 *>(a + (size_t)(c0 ^ 1) * half + m0) = make_float4(v[1], v[3], v[5], v[7]);
    } else {
        float *p = a + ((size_t)(k * L.ny + j) * L.nx + i0);
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<float4 *>(p + 4) = make_float4(v[4], v[5], v[6], v[7]);
    }
}

// restriction where x is not coarsened (cx = 0: identity in x), eight cells
// of a coarse row per thread; r is natural, b of the coarse level in its
// storage order
__global__ void k_restrict_yz8(MgDevLevel Lf, MgDevLevel Lc, const float *__restrict__ rf, float *__restrict__ bc)
{
    pdl_trigger();
    pdl_wait();
    const int q = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y * blockDim.y + threadIdx.y, K = blockIdx.z;
    if (8 * q >= Lc.nx || J >= Lc.ny) return;
    const int i0 = 8 * q;
    const int nyy = Lf.ty.rcnt[J], nzz = Lf.tz.rcnt[K];
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int c3 = 0; c3 < nzz; c3++) {
        const int k = Lf.tz.rf[4 * K + c3];
        const float wz = Lf.tz.rwf[4 * K + c3];
        for (int b = 0; b < nyy; b++) {
            const int j = Lf.ty.rf[4 * J + b];
            const float wyz = __fmul_rn(wz, Lf.ty.rwf[4 * J + b]);
            const float *row = rf + ((size_t)(k * Lf.ny + j) * Lf.nx + i0);
            const float4 a0 = *reinterpret_cast<const float4 *>(row), a1 = *reinterpret_cast<const float4 *>(row + 4);
            const float v[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
            for (int e = 0; e < 8; e++) s[e] = __fmaf_rn(wyz, v[e], s[e]);
        }
    }
    st8(Lc, bc, i0, J, K, s);
}

// prolongation where x is not coarsened, eight cells of a fine row per thread
__global__ void k_prolong_yz8(MgDevLevel Lf, MgDevLevel Lc, const float *__restrict__ xc, float *__restrict__ xf)
{
    pdl_trigger();
    pdl_wait();
    const int q = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (8 * q >= Lf.nx || j >= Lf.ny) return;
    const int i0 = 8 * q;
    const int Iy[2] = {Lf.ty.I0[j], Lf.ty.I1[j]}, Iz[2] = {Lf.tz.I0[k], Lf.tz.I1[k]};
    const float wy[2] = {Lf.ty.w0f[j], Lf.ty.w1f[j]}, wz[2] = {Lf.tz.w0f[k], Lf.tz.w1f[k]};
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < 2; d++) {
        if (wz[d] == 0.0f) continue;
#pragma unroll
        for (int b = 0; b < 2; b++) {
            if (wy[b] == 0.0f) continue;
            const float wyz = __fmul_rn(wz[d], wy[b]);
            float v[8];
            ld8(Lc, xc, i0, Iy[b], Iz[d], v);
#pragma unroll
            for (int e = 0; e < 8; e++) acc[e] = __fmaf_rn(wyz, v[e], acc[e]);
        }
    }
    float x8[8];
    ld8(Lf, xf, i0, j, k, x8);
#pragma unroll
    for (int e = 0; e < 8; e++) x8[e] = __fadd_rn(x8[e], acc[e]);
    st8(Lf, xf, i0, j, k, x8);
}

template <typename T>
__device__ __forceinline__ void coarse_row(int n, const double *__restrict__ ainv, const T *__restrict__ b,
                                           T *__restrict__ x, int r)
{
    double s = 0.0;
    for (int c = 0; c < n; c++) s = __fma_rn(ainv[r * n + c], (double)b[c], s);
    x[r] = (T)s;
}

template <typename T>
__global__ void k_coarse(int n, const double *__restrict__ ainv, const T *__restrict__ b, T *__restrict__ x)
{
    pdl_trigger();
    pdl_wait();
    int r = threadIdx.x;
    if (r >= n) return;
    coarse_row<T>(n, ainv, b, x, r);
}

// The V-cycle from level l0 down to the coarsest and back in one block of
// TAIL_THREADS threads (levels small enough that a launch per half sweep
// costs more than the sweep): the same per-cell operations as the kernels,
// phases separated by block barriers.
constexpr int TAIL_THREADS = 1024;

template <typename T>
struct TailArgs {
    int nlev;                                         // levels l0 .. coarsest
    MgDevLevel L[MG_TAIL_MAXLEV];
    T *x[MG_TAIL_MAXLEV], *b[MG_TAIL_MAXLEV], *r[MG_TAIL_MAXLEV];
    const T *invd[MG_TAIL_MAXLEV];
    int pre[MG_TAIL_MAXLEV], post[MG_TAIL_MAXLEV];
    const double *coarse_inv;
};

template <typename T>
__device__ void tail_half(const MgDevLevel &Ld, int color, int zero_init, const T *b, const T *invd, T *x)
{
    LevelT<T> L = lev_of<T>(Ld);
    int hx = (L.nx + 1) >> 1;
    long long n2 = (long long)hx * L.ny * L.nz;
    for (long long t = threadIdx.x; t < n2; t += TAIL_THREADS) {
        int i2 = (int)(t % hx);
        long long q = t / hx;
        int j = (int)(q % L.ny), k = (int)(q / L.ny);
        int i = 2 * i2 + ((j + k + color) & 1);
        if (i < L.nx) rb_cell<T>(L, zero_init, b, invd, x, i, j, k);
    }
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(TAIL_THREADS) k_vcycle_tail(const TailArgs<T> a)
{
    pdl_trigger();
    pdl_wait();
    const int last = a.nlev - 1;
    for (int l = 0; l < last; l++) {
        const MgDevLevel &Ld = a.L[l];
        for (int it = 0; it < a.pre[l]; it++) {
            tail_half<T>(Ld, 0, it == 0, a.b[l], a.invd[l], a.x[l]);
            tail_half<T>(Ld, 1, 0, a.b[l], a.invd[l], a.x[l]);
        }
        LevelT<T> L = lev_of<T>(Ld);
        long long n = (long long)L.nx * L.ny * L.nz;
        for (long long c = threadIdx.x; c < n; c += TAIL_THREADS)
            resid_cell<T>(L, a.b[l], a.x[l], a.r[l], (int)(c % L.nx), (int)((c / L.nx) % L.ny),
                          (int)(c / ((long long)L.nx * L.ny)));
        __syncthreads();
        const MgDevLevel &C = a.L[l + 1];
        long long nc = (long long)C.nx * C.ny * C.nz;
        for (long long c = threadIdx.x; c < nc; c += TAIL_THREADS)
            restrict_cell<T>(Ld, C, a.r[l], a.b[l + 1], (int)(c % C.nx), (int)((c / C.nx) % C.ny),
                             (int)(c / ((long long)C.nx * C.ny)));
        __syncthreads();
    }
    {
        const MgDevLevel &C = a.L[last];
        int n = C.nx * C.ny * C.nz;
        for (int r = threadIdx.x; r < n; r += TAIL_THREADS) coarse_row<T>(n, a.coarse_inv, a.b[last], a.x[last], r);
        __syncthreads();
    }
    for (int l = last - 1; l >= 0; l--) {
        const MgDevLevel &Ld = a.L[l], &C = a.L[l + 1];
        long long n = (long long)Ld.nx * Ld.ny * Ld.nz;
        for (long long c = threadIdx.x; c < n; c += TAIL_THREADS)
            prolong_cell<T>(Ld, C, a.x[l + 1], a.x[l], (int)(c % Ld.nx), (int)((c / Ld.nx) % Ld.ny),
                            (int)(c / ((long long)Ld.nx * Ld.ny)));
        __syncthreads();
        for (int it = 0; it < a.post[l]; it++) {
            tail_half<T>(Ld, 1, 0, a.b[l], a.invd[l], a.x[l]);
            tail_half<T>(Ld, 0, 0, a.b[l], a.invd[l], a.x[l]);
        }
    }
}

// The V-cycle from level l0 down and back in one launch of one thread-block
// cluster (CLUSTER_CTAS blocks on as many SMs): the first ncl levels are
// swept by every block of the cluster, phases separated by the hardware
// cluster barrier (release / acquire at cluster scope, so the global-memory
// writes of one phase are seen by every block in the next); the levels below
// by block 0 alone with block barriers (the single-block tail above) while
// the other blocks wait at the next cluster barrier.  Every cell's
// operations are those of the per-launch kernels (rb_cell, resid_cell,
// restrict_cell, prolong_cell), so the iterates are the same bits.  Every
// block passes the same sequence of cluster barriers.
constexpr int CLUSTER_THREADS = TAIL_THREADS;

template <typename T>
struct ClusterArgs {
    int nlev, ncl;
    MgDevLevel L[MG_CLUSTER_MAXLEV];
    T *x[MG_CLUSTER_MAXLEV], *b[MG_CLUSTER_MAXLEV], *r[MG_CLUSTER_MAXLEV];
    const T *invd[MG_CLUSTER_MAXLEV];
    int pre[MG_CLUSTER_MAXLEV], post[MG_CLUSTER_MAXLEV];
    const double *coarse_inv;
};

__device__ __forceinline__ void cluster_barrier()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <typename T>
__device__ void cluster_half(const MgDevLevel &Ld, int color, int zero_init, const T *b, const T *invd, T *x)
{
    LevelT<T> L = lev_of<T>(Ld);
    const int hx = (L.nx + 1) >> 1;
    const int n2 = hx * L.ny * L.nz;
    for (int t = blockIdx.x * CLUSTER_THREADS + threadIdx.x; t < n2; t += gridDim.x * CLUSTER_THREADS) {
        const int i2 = t % hx, q = t / hx;
        const int j = q % L.ny, k = q / L.ny;
        const int i = 2 * i2 + ((j + k + color) & 1);
        if (i < L.nx) rb_cell<T>(L, zero_init, b, invd, x, i, j, k);
    }
    cluster_barrier();
}

template <typename T>
__global__ void __launch_bounds__(CLUSTER_THREADS) k_vcycle_cluster(const ClusterArgs<T> a)
{
    pdl_trigger();
    pdl_wait();
    const int last = a.nlev - 1, ncl = min(a.ncl, last);
    const int gstride = gridDim.x * CLUSTER_THREADS, g0 = blockIdx.x * CLUSTER_THREADS + threadIdx.x;
    for (int l = 0; l < ncl; l++) {
        const MgDevLevel &Ld = a.L[l];
        for (int it = 0; it < a.pre[l]; it++) {
            cluster_half<T>(Ld, 0, it == 0, a.b[l], a.invd[l], a.x[l]);
            cluster_half<T>(Ld, 1, 0, a.b[l], a.invd[l], a.x[l]);
        }
        LevelT<T> L = lev_of<T>(Ld);
        const int n = L.nx * L.ny * L.nz;
        for (int c = g0; c < n; c += gstride)
            resid_cell<T>(L, a.b[l], a.x[l], a.r[l], c % L.nx, (c / L.nx) % L.ny, c / (L.nx * L.ny));
        cluster_barrier();
        const MgDevLevel &C = a.L[l + 1];
        const int nc = C.nx * C.ny * C.nz;
        for (int c = g0; c < nc; c += gstride)
            restrict_cell<T>(Ld, C, a.r[l], a.b[l + 1], c % C.nx, (c / C.nx) % C.ny, c / (C.nx * C.ny));
        cluster_barrier();
    }
    if (blockIdx.x == 0) {   // the small levels: block 0 alone
        for (int l = ncl; l < last; l++) {
            const MgDevLevel &Ld = a.L[l];
            for (int it = 0; it < a.pre[l]; it++) {
                tail_half<T>(Ld, 0, it == 0, a.b[l], a.invd[l], a.x[l]);
                tail_half<T>(Ld, 1, 0, a.b[l], a.invd[l], a.x[l]);
            }
            LevelT<T> L = lev_of<T>(Ld);
            const int n = L.nx * L.ny * L.nz;
            for (int c = threadIdx.x; c < n; c += CLUSTER_THREADS)
                resid_cell<T>(L, a.b[l], a.x[l], a.r[l], c % L.nx, (c / L.nx) % L.ny, c / (L.nx * L.ny));
            __syncthreads();
            const MgDevLevel &C = a.L[l + 1];
            const int nc = C.nx * C.ny * C.nz;
            for (int c = threadIdx.x; c < nc; c += CLUSTER_THREADS)
                restrict_cell<T>(Ld, C, a.r[l], a.b[l + 1], c % C.nx, (c / C.nx) % C.ny, c / (C.nx * C.ny));
            __syncthreads();
        }
        {
            const MgDevLevel &C = a.L[last];
            const int n = C.nx * C.ny * C.nz;
            for (int r = threadIdx.x; r < n; r += CLUSTER_THREADS) coarse_row<T>(n, a.coarse_inv, a.b[last], a.x[last], r);
            __syncthreads();
        }
        for (int l = last - 1; l >= ncl; l--) {
            const MgDevLevel &Ld = a.L[l], &C = a.L[l + 1];
            const int n = Ld.nx * Ld.ny * Ld.nz;
            for (int c = threadIdx.x; c < n; c += CLUSTER_THREADS)
                prolong_cell<T>(Ld, C, a.x[l + 1], a.x[l], c % Ld.nx, (c / Ld.nx) % Ld.ny, c / (Ld.nx * Ld.ny));
            __syncthreads();
            for (int it = 0; it < a.post[l]; it++) {
                tail_half<T>(Ld, 1, 0, a.b[l], a.invd[l], a.x[l]);
                tail_half<T>(Ld, 0, 0, a.b[l], a.invd[l], a.x[l]);
            }
        }
    }
    cluster_barrier();
    for (int l = ncl - 1; l >= 0; l--) {
        const MgDevLevel &Ld = a.L[l], &C = a.L[l + 1];
        const int n = Ld.nx * Ld.ny * Ld.nz;
        for (int c = g0; c < n; c += gstride)
            prolong_cell<T>(Ld, C, a.x[l + 1], a.x[l], c % Ld.nx, (c / Ld.nx) % Ld.ny, c / (Ld.nx * Ld.ny));
        cluster_barrier();
        for (int it = 0; it < a.post[l]; it++) {
            cluster_half<T>(Ld, 1, 0, a.b[l], a.invd[l], a.x[l]);
            cluster_half<T>(Ld, 0, 0, a.b[l], a.invd[l], a.x[l]);
        }
    }
}

// FP64 <-> FP32 between the natural order and a level's storage order
__global__ void k_to_float_lev(MgDevLevel L, const double *__restrict__ a, float *__restrict__ b)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= L.nx || j >= L.ny) return;
    long long c = ((long long)k * L.ny + j) * L.nx + i;
    b[lev_at(L, c, i, j, k)] = (float)a[c];
}
__global__ void k_to_double_lev(MgDevLevel L, const float *__restrict__ a, double *__restrict__ b)
{
    pdl_trigger();
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= L.nx || j >= L.ny) return;
    long long c = ((long long)k * L.ny + j) * L.nx + i;
    b[c] = (double)a[lev_at(L, c, i, j, k)];
}

// the same, eight cells of a row per thread (nx a multiple of 8): FP64 as
// double2, FP32 as one float4 per colour (colour-split) or two (natural)
__global__ void k_to_float_lev8(MgDevLevel L, const double *__restrict__ a, float *__restrict__ b)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (8 * q >= L.nx || j >= L.ny) return;
    const long long c0 = ((long long)k * L.ny + j) * L.nx + 8 * q;
    float v[8];
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const double2 d2 = *reinterpret_cast<const double2 *>(a + c0 + 2 * t);
        v[2 * t] = (float)d2.x;
        v[2 * t + 1] = (float)d2.y;
    }
    if (L.split) {
        const long long half = ((long long)L.nx * L.ny * L.nz) >> 1;
        const int ce = (j + k) & 1;   // colour of the even cells
        *reinterpret_cast<float4 *>(b + ce * half + (c0 >> 1)) = make_float4(v[0], v[2], v[4], v[6]);
        *reinterpret_cast<float4 *>(b + (1 - ce) * half + (c0 >> 1)) = make_float4(v[1], v[3], v[5], v[7]);
    } else {
        *reinterpret_cast<float4 *>(b + c0) = make_float4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<float4 *>(b + c0 + 4) = make_float4(v[4], v[5], v[6], v[7]);
    }
}
__global__ void k_to_double_lev8(MgDevLevel L, const float *__restrict__ a, double *__restrict__ b)
{
    pdl_trigger();
    pdl_wait();
    const int q = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (8 * q >= L.nx || j >= L.ny) return;
    const long long c0 = ((long long)k * L.ny + j) * L.nx + 8 * q;
    float v[8];
    if (L.split) {
        const long long half = ((long long)L.nx * L.ny * L.nz) >> 1;
        const int ce = (j + k) & 1;
        const float4 e4 = *reinterpret_cast<const float4 *>(a + ce * half + (c0 >> 1));
        const float4 o4 = *reinterpret_cast<const float4 *>(a + (1 - ce) * half + (c0 >> 1));
        v[0] = e4.x; v[1] = o4.x; v[2] = e4.y; v[3] = o4.y; v[4] = e4.z; v[5] = o4.z; v[6] = e4.w; v[7] = o4.w;
    } else {
        const float4 l4 = *reinterpret_cast<const float4 *>(a + c0), h4 = *reinterpret_cast<const float4 *>(a + c0 + 4);
        v[0] = l4.x; v[1] = l4.y; v[2] = l4.z; v[3] = l4.w; v[4] = h4.x; v[5] = h4.y; v[6] = h4.z; v[7] = h4.w;
    }
#pragma unroll
    for (int t = 0; t < 4; t++)
        *reinterpret_cast<double2 *>(b + c0 + 2 * t) = make_double2((double)v[2 * t], (double)v[2 * t + 1]);
}

inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// a V-cycle kernel launch; pdl: with the programmatic stream serialisation
// attribute (the kernels start with pdl_trigger / pdl_wait), so that a small
// level's launches overlap the drain of the kernel before them
template <typename... P, typename... A>
void launch_k(int pdl, void (*k)(P...), dim3 g, dim3 b, cudaStream_t s, A... args)
{
    if (!pdl) {
        k<<<g, b, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}
inline dim3 g3(int nx, int ny, int nz) { return dim3((unsigned)((nx + 31) / 32), (unsigned)((ny + 7) / 8), (unsigned)nz); }
const dim3 B38(32, 8, 1);

}  // namespace

template <typename T>
void mg_setup_invdiag(cudaStream_t s, const MgDevLevel &L, T *invd)
{
    k_invdiag<T><<<1024, 256, 0, s>>>(L, invd);
}

// One V-cycle from level l: input b[l], output x[l] (x starts at zero).
// one red-black half sweep of level L: the vectorised kernel where the
// level is colour-split FP32 with nx a multiple of 8
// marching: half sweeps after the first of a cycle march along k (k_rbgs4z)
// on the levels large enough to fill the GPU with them
template <typename T>
void rb_half(cudaStream_t s, const MgDevLevel &L, int color, int zero_init, const T *b, const T *invd, T *x,
             int marching, int pdl)
{
    if constexpr (sizeof(T) == 4) {
        if (L.split && L.nx % 8 == 0) {
            dim3 g4((unsigned)((L.nx / 8 + 31) / 32), (unsigned)((L.ny + 7) / 8), (unsigned)L.nz);
            if (marching && !zero_init) {
                // planes per block: the most (up to 16) that still gives two
                // waves of three blocks on every SM
                long long bxy = (long long)g4.x * g4.y;
                int jz = 16;
                while (jz > 2 && bxy * ((L.nz + jz - 1) / jz) < 2 * 3 * 152) jz >>= 1;
                if (bxy * ((L.nz + jz - 1) / jz) >= 152) {
                    dim3 gz(g4.x, g4.y, (unsigned)((L.nz + jz - 1) / jz));
                    launch_k(pdl, k_rbgs4z, gz, B38, s, L, color, jz, b, invd, x);
                    return;
                }
            }
            const int planes = (long long)L.nx * L.ny * L.nz >= RB4_PLANES_CELLS ? RB4_PLANES : 1;
            dim3 g4p(g4.x, g4.y, (unsigned)((L.nz + planes - 1) / planes));
            launch_k(pdl, k_rbgs4, g4p, B38, s, L, color, zero_init, planes, b, invd, x);
            return;
        }
    }
    launch_k(pdl, k_rbgs<T>, g3((L.nx + 1) >> 1, L.ny, L.nz), B38, s, L, color, zero_init, b, invd, x);
}

template <typename T>
void resid_lev(cudaStream_t s, const MgDevLevel &L, const T *b, const T *x, T *r, int pdl)
{
    if constexpr (sizeof(T) == 4) {
        if (L.split && L.nx % 8 == 0) {
            dim3 g8((unsigned)((L.nx / 8 + 31) / 32), (unsigned)((L.ny + 7) / 8), (unsigned)L.nz);
            launch_k(pdl, k_resid8, g8, B38, s, L, b, x, r);
            return;
        }
    }
    launch_k(pdl, k_resid<T>, g3(L.nx, L.ny, L.nz), B38, s, L, b, x, r);
}

template <typename T>
void mg_vcycle(cudaStream_t s, const MgHier<T> &H, int l, const int *pre, const int *post)
{
    const MgDevLevel &L = H.lev[l];
    const int npre = pre[l], npost = post[l];
    long long n = (long long)L.nx * L.ny * L.nz;
    if (H.tail_from >= 0 && l == H.tail_from && H.nl - l <= MG_TAIL_MAXLEV && l < H.nl - 1) {
        TailArgs<T> a;
        a.nlev = H.nl - l;
        for (int t = 0; t < a.nlev; t++) {
            a.L[t] = H.lev[l + t];
            a.x[t] = H.x[l + t];
            a.b[t] = H.b[l + t];
            a.r[t] = H.r[l + t];
            a.invd[t] = H.invd[l + t];
            a.pre[t] = pre[l + t];
            a.post[t] = post[l + t];
        }
        a.coarse_inv = H.coarse_inv;
        launch_k(H.pdl, k_vcycle_tail<T>, dim3(1), dim3(TAIL_THREADS), s, a);
        return;
    }
    if (H.cluster_from >= 0 && l == H.cluster_from && H.nl - l <= MG_CLUSTER_MAXLEV && l < H.nl - 1 &&
        H.cluster_ctas > 0) {
        ClusterArgs<T> a;
        a.nlev = H.nl - l;
        // the levels above the single-block tail (or all but the coarsest)
        a.ncl = (H.tail_from > l) ? H.tail_from - l : a.nlev - 1;
        for (int t = 0; t < a.nlev; t++) {
            a.L[t] = H.lev[l + t];
            a.x[t] = H.x[l + t];
            a.b[t] = H.b[l + t];
            a.r[t] = H.r[l + t];
            a.invd[t] = H.invd[l + t];
            a.pre[t] = pre[l + t];
            a.post[t] = post[l + t];
        }
        a.coarse_inv = H.coarse_inv;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)H.cluster_ctas);
        cfg.blockDim = dim3(CLUSTER_THREADS);
        cfg.stream = s;
        cudaLaunchAttribute at[2];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)H.cluster_ctas;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = H.pdl ? 2 : 1;
        cudaLaunchKernelEx(&cfg, k_vcycle_cluster<T>, a);
        return;
    }
    if (l == H.nl - 1) {
        launch_k(H.pdl, k_coarse<T>, dim3(1), dim3(64), s, (int)n, H.coarse_inv, H.b[l], H.x[l]);
        return;
    }
    // level 0 in FP32: sweeps in pairs, one pass each (an even number of
    // passes, so that x ends in its own array), the rest one half sweep each
    int pre_done = 0, post_done = 0;
    if constexpr (sizeof(T) == 4) {
        if (l == 0 && H.tb) {
            const int np = (npre / 4) * 2, nq = (npost / 4) * 2;
            for (int f = 0; f < np; f++) mg_tb_sweeps(s, *H.tb, f & 1, 0, f == 0, H.pdl);
            pre_done = 2 * np;
            post_done = 2 * nq;
        }
    }
    for (int it = pre_done; it < npre; it++) {
        // the first colour-0 half sweep takes x = 0 (it reads no neighbours);
        // every colour-1 point is then rewritten from colour-0 values only
        rb_half<T>(s, L, 0, it == 0, H.b[l], H.invd[l], H.x[l], H.marching, H.pdl);
        rb_half<T>(s, L, 1, 0, H.b[l], H.invd[l], H.x[l], H.marching, H.pdl);
    }
    resid_lev<T>(s, L, H.b[l], H.x[l], H.r[l], H.pdl);
    const MgDevLevel &C = H.lev[l + 1];
    bool yz8 = false;
    if constexpr (sizeof(T) == 4) yz8 = L.cx == 0 && L.nx % 8 == 0 && C.nx == L.nx;
    if (yz8) {
        if constexpr (sizeof(T) == 4) {
            launch_k(H.pdl, k_restrict_yz8, g3((C.nx / 8 + 31) / 32 * 32, C.ny, C.nz), B38, s, L, C, H.r[l], H.b[l + 1]);
            mg_vcycle<T>(s, H, l + 1, pre, post);
            launch_k(H.pdl, k_prolong_yz8, g3((L.nx / 8 + 31) / 32 * 32, L.ny, L.nz), B38, s, L, C, H.x[l + 1], H.x[l]);
        }
    } else {
        launch_k(H.pdl, k_restrict<T>, g3(C.nx, C.ny, C.nz), B38, s, L, C, H.r[l], H.b[l + 1]);
        mg_vcycle<T>(s, H, l + 1, pre, post);
        launch_k(H.pdl, k_prolong<T>, g3(L.nx, L.ny, L.nz), B38, s, L, C, H.x[l + 1], H.x[l]);
    }
    if constexpr (sizeof(T) == 4) {
        for (int f = 0; f < post_done / 2; f++) mg_tb_sweeps(s, *H.tb, f & 1, 1, 0, H.pdl);
    }
    for (int it = post_done; it < npost; it++) {
        rb_half<T>(s, L, 1, 0, H.b[l], H.invd[l], H.x[l], H.marching, H.pdl);
        rb_half<T>(s, L, 0, 0, H.b[l], H.invd[l], H.x[l], H.marching, H.pdl);
    }
}

void mg_to_float(cudaStream_t s, const MgDevLevel &L, const double *a, float *b)
{
    if (L.nx % 8 == 0)
        k_to_float_lev8<<<g3(L.nx / 8, L.ny, L.nz), B38, 0, s>>>(L, a, b);
    else
        k_to_float_lev<<<g3(L.nx, L.ny, L.nz), B38, 0, s>>>(L, a, b);
}
void mg_to_double(cudaStream_t s, const MgDevLevel &L, const float *a, double *b, int pdl)
{
    if (L.nx % 8 == 0)
        launch_k(pdl, k_to_double_lev8, g3(L.nx / 8, L.ny, L.nz), B38, s, L, a, b);
    else
        launch_k(pdl, k_to_double_lev, g3(L.nx, L.ny, L.nz), B38, s, L, a, b);
}

// Algorithmic bytes of one V-cycle from level l (each array a kernel reads
// or writes counted once per launch): a half sweep of a colour reads b, invd
// and the other colour's x and writes its own x (the first one of a cycle
// reads b and invd only); the residual reads b, x and writes r; restriction
// reads r and writes the coarse b; prolongation reads the coarse x and
// reads and writes the fine x; the coarsest solve and the single-block tail
// read b and write x of their levels (their sweeps stay in L1/L2).
template <typename T>
double mg_vcycle_bytes(const MgHier<T> &H, int l, const int *pre, const int *post)
{
    const double e = (double)sizeof(T);
    double total = 0.0;
    for (; l < H.nl; l++) {
        const MgDevLevel &L = H.lev[l];
        double n = (double)L.nx * L.ny * L.nz;
        bool tail = H.tail_from >= 0 && l == H.tail_from && H.nl - l <= MG_TAIL_MAXLEV && l < H.nl - 1;
        if (tail || l == H.nl - 1) {
            for (int t = l; t < H.nl; t++) {
                const MgDevLevel &M = H.lev[t];
                total += 2.0 * e * (double)M.nx * M.ny * M.nz;
            }
            break;
        }
        const MgDevLevel &C = H.lev[l + 1];
        double nc = (double)C.nx * C.ny * C.nz;
        int halves = 2 * pre[l] + 2 * post[l];
        if (l == 0 && H.tb && sizeof(T) == 4) {
            // a pass of two sweeps reads b, 1/diag and one colour of x and
            // writes x (the first of a cycle reads no x)
            const int np = (pre[l] / 4) * 2, nq = (post[l] / 4) * 2;
            total += np > 0 ? 3.0 * e * n + (np - 1) * 3.5 * e * n : 0.0;
            total += nq * 3.5 * e * n;
            halves -= 4 * (np + nq);
            total += halves * 2.0 * e * n;   // the remaining half sweeps (none of them the first)
        } else {
            total += (halves > 0 ? 1.5 * e * n : 0.0) + (halves > 1 ? (halves - 1) * 2.0 * e * n : 0.0);
        }
        total += 3.0 * e * n;                 // residual
        total += e * n + e * nc;              // restriction
        total += e * nc + 2.0 * e * n;        // prolongation
    }
    return total;
}

template double mg_vcycle_bytes<double>(const MgHier<double> &, int, const int *, const int *);
template double mg_vcycle_bytes<float>(const MgHier<float> &, int, const int *, const int *);

int mg_vcycle_launches(int nl, const int *pre, const int *post, int tail_from, int cluster_from, int tb0)
{
    // per non-coarsest level: 2*pre + resid + restrict + prolong + 2*post;
    // coarsest: 1; the fused tail from tail_from on: 1; the one-cluster
    // V-cycle from cluster_from on: 1; level 0 with sweep pairs (tb0): one
    // launch per pair of sweeps in place of four
    int n = 1;
    for (int l = 0; l < nl - 1; l++) {
        if (cluster_from >= 0 && l == cluster_from && nl - l <= MG_CLUSTER_MAXLEV) return n;
        if (tail_from >= 0 && l == tail_from && nl - l <= MG_TAIL_MAXLEV) return n;
        n += 2 * pre[l] + 3 + 2 * post[l];
        if (l == 0 && tb0) n -= 3 * ((pre[l] / 4) * 2 + (post[l] / 4) * 2);
    }
    return n;
}

// blocks of the one-cluster V-cycle: 16 if a cluster of 16 such blocks can
// be resident (a non-portable cluster size), else 8, else 0 (not used)
template <typename T>
int mg_cluster_ctas()
{
    if (cudaFuncSetAttribute(k_vcycle_cluster<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
    }
    for (int ctas = 16; ctas >= 8; ctas /= 2) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)ctas);
        cfg.blockDim = dim3(CLUSTER_THREADS);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)ctas;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, k_vcycle_cluster<T>, &cfg) == cudaSuccess && nc >= 1) return ctas;
        cudaGetLastError();
    }
    return 0;
}
template int mg_cluster_ctas<float>();
template int mg_cluster_ctas<double>();

template void mg_setup_invdiag<double>(cudaStream_t, const MgDevLevel &, double *);
template void mg_setup_invdiag<float>(cudaStream_t, const MgDevLevel &, float *);
template void mg_vcycle<double>(cudaStream_t, const MgHier<double> &, int, const int *, const int *);
template void mg_vcycle<float>(cudaStream_t, const MgHier<float> &, int, const int *, const int *);
