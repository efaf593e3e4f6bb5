// k_rbtb.cu -- two red-black Gauss-Seidel sweeps of the finest FP32
// multigrid level in one pass over memory.
//
// A launch applies four half sweeps (colours c0, 1-c0, c0, 1-c0) to the
// colour-split FP32 level: the arithmetic of every cell update is that of
// k_rbgs4 (the same products, the same neighbour order, the same explicit
// rounding), and every update sees the neighbour values the four separate
// half sweeps would give it, so the result is bit-identical to them.
//
// Blocking.  The level is cut into x-y tiles of 64 x 32 cells; a block
// marches through a range of z-planes of a tile as a wavefront: at step t it
// updates colour c0 on plane t, 1-c0 on plane t-1, c0 (second sweep) on plane
// t-2 and 1-c0 (second sweep) on plane t-3, then writes plane t-3.  The
// in-plane dependencies are met by overlapped tiles: the four stages update
// the tile grown by 3, 2, 1 and 0 cells on every side, reading a halo of 4.
// Planes of the old x (only colour 1-c0: the first stage reads nothing else)
// are staged in a shared-memory ring by TMA tensor loads, three planes ahead
// of the step that needs them; the updates happen in place in the ring; the
// result goes to a second x array (x_out != x_in), because neighbouring
// tiles still read the old x of this tile's halo.  b and 1/diag go straight
// from global memory into registers, each thread loading its cells' values
// for the step's stages before the stages run (the first stage's one step
// earlier).  A thread updates four consecutive cells of one colour in a row
// (float4 shared-memory reads, as k_rbgs4 does from global memory).  A
// launch therefore moves b, 1/diag, half of x in and all of x out once (14
// bytes per cell) where the four half sweeps move 32.
//
// Persistent blocks: one per SM, each taking a contiguous range of the
// (tile, plane) units; a range that crosses tiles is walked as one segment
// per tile.  Every mbarrier wait gives up after a second, sets *err, drains
// the copies still in flight (again bounded) and ends the block.
#include <cstdint>
#include <cuda.h>
#include <cudaTypedefs.h>

#include "tc_ptx.cuh"
#include "turb_internal.cuh"
#include "turb_mg.cuh"

namespace {

constexpr int TB_W2 = 32;                    // interior columns per colour (64 cells)
constexpr int TB_H = 32;                     // interior rows
constexpr int TB_HX = 4;                     // halo columns per colour (8 cells; TMA x alignment)
constexpr int TB_HY = 4;                     // halo rows
constexpr int TB_C = TB_W2 + 2 * TB_HX;      // 40 columns
constexpr int TB_R = TB_H + 2 * TB_HY;       // 40 rows
constexpr int TB_PL = TB_R * TB_C;           // floats per colour plane
constexpr int TB_SLOT = 2 * TB_PL;           // floats per plane slot (both colours)
constexpr int TB_PF = 3;                     // planes loaded ahead of the step that needs them
constexpr int TB_NX = 6 + TB_PF;             // x ring: planes t+1+PF .. t-4
constexpr int TB_THREADS = 512;
constexpr int TB_TX = TB_C + 4;              // x tables per parity (40 columns, padded)
constexpr uint32_t TB_XBYTES = TB_PL * 4;    // one colour plane of x

struct TbSmem {
    float x[TB_NX][TB_SLOT];
    // x tables split by parity: [par][m] is cell i0-8+2m+par; rfxs[m] is
    // rfx of cell i0-8+2m+2 (the right face of an odd cell), so that every
    // 4-cell group reads its tables as float4
    float dx[2][TB_TX], rfx[2][TB_TX], rfxs[TB_TX];
    float dy[TB_R + 4], rfy[TB_R + 4];
    unsigned long long xbar[TB_NX];
    int abort;
};

struct TbArgs {
    MgDevLevel L;
    const float *b, *invd;   // colour-split
    float *xo;               // x out (colour-split)
    int c0;                  // colour of the first and third half sweeps
    int zero_init;           // the first half sweep takes x = 0 (reads no x)
    int tiles_x, ntiles;
    int *err;
};

__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// The item of a thread in the stage that grows the tile by E: a group of four
// consecutive columns (4g .. 4g+3) of row rr of the slot.
template <int E>
struct TbItem {
    static constexpr int NG = E == 0 ? 8 : 10, G0 = E == 0 ? 1 : 0, NR = TB_H + 2 * E, R0 = TB_HY - E;
    static constexpr int N = NR * NG;
    int rr, cb;
    bool active;
    __device__ __forceinline__ TbItem(int tid)
    {
        active = tid < N;
        rr = R0 + tid / NG;
        cb = 4 * (G0 + tid % NG);
    }
};

struct Bd {
    float4 b, d;
};

// b and 1/diag of the item's four cells (colour c, plane k), zero outside the level
template <int E>
__device__ __forceinline__ Bd tb_load_bd(const TbArgs &a, const TbItem<E> &it, int c, int k, int jb, int i2b,
                                         long long half)
{
    Bd r;
    r.b = r.d = make_float4(0.f, 0.f, 0.f, 0.f);
    const int j = jb + it.rr, i2 = i2b + it.cb, hx = a.L.nx >> 1;
    if (it.active && k >= 0 && k < a.L.nz && j >= 0 && j < a.L.ny && i2 >= 0 && i2 < hx) {
        const long long g = c * half + ((long long)k * a.L.ny + j) * hx + i2;
        r.b = __ldg(reinterpret_cast<const float4 *>(a.b + g));
        r.d = __ldg(reinterpret_cast<const float4 *>(a.invd + g));
    }
    return r;
}

// One half sweep of colour c on plane k for the thread's item (tile grown by
// E).  xk / xm / xp: the ring slots of planes k, k-1, k+1.  Cells outside the
// grown tile or the level keep their values; each update is k_rbgs4's:
// o = sum of f * neighbour in the order x-, x+, y-, y+, z-, z+ (absent
// neighbours skipped), x = (b + o) * (1/diag).
template <int E>
__device__ __forceinline__ void tb_stage(const TbSmem &S, const TbItem<E> &it, float *__restrict__ xk,
                                         const float *__restrict__ xm, const float *__restrict__ xp, const Bd &bd,
                                         int c, int k, int zero, const MgDevLevel &L, int i0, int jb, int i2b)
{
    if (!it.active) return;
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    const int rr = it.rr, cb = it.cb;
    const int j = jb + rr;
    if (j < 0 || j >= ny) return;
    const int p = (j + k + c) & 1;
    const int ib = 2 * (i2b + cb) + p;   // cell of column cb
    bool v[4];
    bool any = false;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int i = ib + 2 * e;
        v[e] = i >= i0 - E && i < i0 + 2 * TB_W2 + E && i >= 0 && i < nx;
        any |= v[e];
    }
    if (!any) return;
    const int idx = rr * TB_C + cb;
    float *own = xk + c * TB_PL;
    const float4 cur = *reinterpret_cast<const float4 *>(own + idx);
    const float bv[4] = {bd.b.x, bd.b.y, bd.b.z, bd.b.w}, dv[4] = {bd.d.x, bd.d.y, bd.d.z, bd.d.w};
    float out[4] = {cur.x, cur.y, cur.z, cur.w};
    if (zero) {
#pragma unroll
        for (int e = 0; e < 4; e++)
            if (v[e]) out[e] = rmul(bv[e], dv[e]);
    } else {
        const float *oth = xk + (1 - c) * TB_PL;
        const float4 c4 = *reinterpret_cast<const float4 *>(oth + idx);
        float ex = 0.0f;   // the fifth x-neighbour: left of the group (p = 0) or right of it (p = 1)
        if (p == 0) { if (cb > 0) ex = oth[idx - 1]; }
        else { if (cb + 4 < TB_C) ex = oth[idx + 4]; }
        const float4 jm = *reinterpret_cast<const float4 *>(oth + idx - TB_C);
        const float4 jp = *reinterpret_cast<const float4 *>(oth + idx + TB_C);
        const float4 km = *reinterpret_cast<const float4 *>(xm + (1 - c) * TB_PL + idx);
        const float4 kp = *reinterpret_cast<const float4 *>(xp + (1 - c) * TB_PL + idx);
        const float4 dx4 = *reinterpret_cast<const float4 *>(&S.dx[p][cb]);
        const float4 rl4 = *reinterpret_cast<const float4 *>(&S.rfx[p][cb]);
        const float4 rr4 = *reinterpret_cast<const float4 *>(p == 0 ? &S.rfx[1][cb] : &S.rfxs[cb]);
        const float dyj = S.dy[rr], ryj = S.rfy[rr], ryj1 = S.rfy[rr + 1];
        const float dzk = L.dzf[k], rzk = L.rfzf[k], rzk1 = L.rfzf[k + 1];
        const float dyz = rmul(dyj, dzk);
        const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
        const float jmv[4] = {jm.x, jm.y, jm.z, jm.w}, jpv[4] = {jp.x, jp.y, jp.z, jp.w};
        const float kmv[4] = {km.x, km.y, km.z, km.w}, kpv[4] = {kp.x, kp.y, kp.z, kp.w};
        const float dxv[4] = {dx4.x, dx4.y, dx4.z, dx4.w};
        const float rlv[4] = {rl4.x, rl4.y, rl4.z, rl4.w}, rrv[4] = {rr4.x, rr4.y, rr4.z, rr4.w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int i = ib + 2 * e;
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
            if (v[e]) out[e] = rmul(radd(bv[e], o), dv[e]);
        }
    }
    *reinterpret_cast<float4 *>(own + idx) = make_float4(out[0], out[1], out[2], out[3]);
}

__global__ void __launch_bounds__(TB_THREADS, 1) k_rbgs_tb(const __grid_constant__ CUtensorMap mapx, const TbArgs a)
{
    extern __shared__ __align__(128) unsigned char tb_raw[];
    // the TMA destinations want 128-byte alignment: round the base up
    const uint32_t pad = (128u - (tc::smem_u32(tb_raw) & 127u)) & 127u;
    TbSmem &S = *reinterpret_cast<TbSmem *>(tb_raw + pad);
    const MgDevLevel &L = a.L;
    const int nx = L.nx, ny = L.ny, nz = L.nz, hx = nx >> 1;
    const long long half = ((long long)nx * ny * nz) >> 1;
    const int c0 = a.c0, c1 = 1 - c0;
    const int tid = threadIdx.x;
    const TbItem<3> it3(tid);
    const TbItem<2> it2(tid);
    const TbItem<1> it1(tid);
    const TbItem<0> it0(tid);

    if (tid == 0) {
        for (int q = 0; q < TB_NX; q++) tc::mbar_init(tc::smem_u32(&S.xbar[q]), 1);
        tc::mbar_fence_init();
        S.abort = 0;
        tc::prefetch_map(&mapx);
    }
    pdl_trigger();
    pdl_wait();
    __syncthreads();

    const long long units = (long long)a.ntiles * nz;
    const long long u0 = units * blockIdx.x / gridDim.x, u1 = units * (blockIdx.x + 1) / gridDim.x;
    // sequence numbers of the x loads: load n uses slot n % TB_NX and
    // completes phase n / TB_NX of that slot's barrier
    unsigned xseq = 0, xwaited = 0;
    bool ok = true;

    for (long long u = u0; u < u1 && ok;) {
        const int tile = (int)(u / nz);
        const int ka = (int)(u - (long long)tile * nz);
        const int kb = (int)((long long)tile * nz + nz < u1 ? nz : u1 - (long long)tile * nz);
        u = (long long)tile * nz + kb;
        const int tx = tile % a.tiles_x, ty = tile / a.tiles_x;
        const int i0 = tx * 2 * TB_W2, j0 = ty * TB_H;
        const int i2b = tx * TB_W2 - TB_HX, jb = j0 - TB_HY;

        // the tile's 1-D metric tables (entries outside the level: 0, never used)
        for (int q = tid; q < 2 * TB_TX; q += TB_THREADS) {
            const int i = i0 - 2 * TB_HX + q;
            const bool in = i >= 0 && i < nx;
            S.dx[q & 1][q >> 1] = in ? L.dxf[i] : 0.0f;
            S.rfx[q & 1][q >> 1] = in ? L.rfxf[i] : 0.0f;
        }
        for (int q = tid; q < TB_TX; q += TB_THREADS) {
            const int i = i0 - 2 * TB_HX + 2 * q + 2;
            S.rfxs[q] = (i >= 0 && i < nx) ? L.rfxf[i] : 0.0f;
        }
        for (int q = tid; q < TB_R + 4; q += TB_THREADS) {
            const int j = jb + q;
            const bool in = j >= 0 && j < ny;
            S.dy[q] = in ? L.dyf[j] : 0.0f;
            S.rfy[q] = in ? L.rfyf[j] : 0.0f;
        }

        const int t0 = ka - 3, t1 = kb + 2;   // steps
        const unsigned xs0 = xseq - (unsigned)(t0 - 1);   // plane p: x load xs0 + p
        auto xslot = [&](int p) -> float * { return S.x[(xs0 + (unsigned)p) % TB_NX]; };
        auto issue_x = [&](int p) {   // thread 0: old x, colour c1, plane p
            const int sl = (int)(xseq % TB_NX);
            if (!a.zero_init) {
                const uint32_t bar = tc::smem_u32(&S.xbar[sl]);
                tc::mbar_expect_tx(bar, TB_XBYTES);
                tc::tma_load4(tc::smem_u32(&S.x[sl][c1 * TB_PL]), &mapx, i2b, jb, p, c1, bar);
            }
            xseq++;
        };
        __syncthreads();   // tables written; every slot's previous contents consumed
        // x planes t0-1 .. t0+PF ahead of the first step
        const int xpro = min(t0 + TB_PF, kb + 3) - (t0 - 1) + 1;
        if (tid == 0) {
            tc::fence_proxy_async();
            for (int q = 0; q < xpro; q++) issue_x(t0 - 1 + q);
        } else {
            xseq += xpro;
        }
        Bd bd3n = tb_load_bd<3>(a, it3, c0, t0, jb, i2b, half);   // the first stage's b, 1/diag one step ahead
        for (int t = t0; t <= t1; t++) {
            if (t + 1 + TB_PF <= kb + 3) {   // old x up to plane kb+3 (read by the first stage on plane kb+2)
                if (tid == 0) { tc::fence_proxy_async(); issue_x(t + 1 + TB_PF); } else xseq++;
            }
            const Bd bd3 = bd3n;
            const bool s2 = t - 1 >= ka - 2, s1 = t - 2 >= ka - 1 && t - 2 < kb + 1, s0 = t - 3 >= ka && t - 3 < kb;
            const Bd bd2 = s2 ? tb_load_bd<2>(a, it2, c1, t - 1, jb, i2b, half) : Bd{};
            const Bd bd1 = s1 ? tb_load_bd<1>(a, it1, c0, t - 2, jb, i2b, half) : Bd{};
            const Bd bd0 = s0 ? tb_load_bd<0>(a, it0, c1, t - 3, jb, i2b, half) : Bd{};
            if (t + 1 <= t1) bd3n = tb_load_bd<3>(a, it3, c0, t + 1, jb, i2b, half);
            // wait for x planes up to t+1
            while (ok && xwaited != xs0 + (unsigned)(t + 2)) {
                if (!a.zero_init) {
                    const int sl = (int)(xwaited % TB_NX);
                    if (!tc::mbar_wait(tc::smem_u32(&S.xbar[sl]), (xwaited / TB_NX) & 1u, &S.abort)) {
                        S.abort = 1;
                        ok = false;
                        break;
                    }
                }
                xwaited++;
            }
            __syncthreads();
            if (S.abort) { ok = false; break; }
            // the four stages of the wavefront
            if (t >= 0 && t < nz)
                tb_stage<3>(S, it3, xslot(t), xslot(t - 1), xslot(t + 1), bd3, c0, t, a.zero_init, L, i0, jb, i2b);
            __syncthreads();
            if (s2 && t - 1 >= 0 && t - 1 < nz)
                tb_stage<2>(S, it2, xslot(t - 1), xslot(t - 2), xslot(t), bd2, c1, t - 1, 0, L, i0, jb, i2b);
            __syncthreads();
            if (s1 && t - 2 >= 0 && t - 2 < nz)
                tb_stage<1>(S, it1, xslot(t - 2), xslot(t - 3), xslot(t - 1), bd1, c0, t - 2, 0, L, i0, jb, i2b);
            __syncthreads();
            const int kw = t - 3;
            if (s0) tb_stage<0>(S, it0, xslot(kw), xslot(kw - 1), xslot(kw + 1), bd0, c1, kw, 0, L, i0, jb, i2b);
            __syncthreads();
            if (s0) {   // plane kw is final: both colours of the interior, one float4 per thread
                const float *src = xslot(kw);
                const int c = tid / (TB_H * (TB_W2 / 4)), r = (tid / (TB_W2 / 4)) % TB_H, v = tid % (TB_W2 / 4);
                const float4 val =
                    *reinterpret_cast<const float4 *>(src + c * TB_PL + (r + TB_HY) * TB_C + TB_HX + 4 * v);
                *reinterpret_cast<float4 *>(a.xo + c * half + ((long long)kw * ny + j0 + r) * hx +
                                            (long long)tx * TB_W2 + 4 * v) = val;
            }
        }
    }
    if (!ok) {
        if (tid == 0) {
            atomicExch(a.err, 1);
            // let the copies still in flight land before the block ends
            volatile int never = 0;
            if (!a.zero_init)
                for (; xwaited != xseq; xwaited++)
                    tc::mbar_wait(tc::smem_u32(&S.xbar[(int)(xwaited % TB_NX)]), (xwaited / TB_NX) & 1u, &never);
        }
        __syncthreads();
    }
}

static_assert(2 * TB_H * (TB_W2 / 4) == TB_THREADS, "one float4 of the written plane per thread");
static_assert(TbItem<3>::N <= TB_THREADS && TbItem<0>::N <= TB_THREADS, "one item per thread and stage");

}  // namespace

size_t mg_tb_smem() { return sizeof(TbSmem) + 128; }

// 4-D map of a colour-split FP32 level array: (x / 2, y, z, colour), box
// (40, 40, 1, ncol)
static int tb_map(CUtensorMap *m, const float *ptr, const MgDevLevel &L, int ncol)
{
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return 1;
    auto enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    const cuuint64_t hx = (cuuint64_t)(L.nx / 2);
    cuuint64_t dims[4] = {hx, (cuuint64_t)L.ny, (cuuint64_t)L.nz, 2};
    cuuint64_t str[3] = {hx * 4, hx * L.ny * 4, hx * L.ny * L.nz * 4};
    cuuint32_t box[4] = {(cuuint32_t)TB_C, (cuuint32_t)TB_R, 1, (cuuint32_t)ncol};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float *>(ptr), dims, str, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : 1;
}

int mg_tb_plan(RbTbPlan *p, const MgDevLevel &L0, float *x0, float *x1, const float *b0, const float *invd0, int *err)
{
    p->ok = 0;
    if (!L0.split || L0.nx % (2 * TB_W2) != 0 || L0.ny % TB_H != 0 || L0.nz < 1) return 1;
    if (((uintptr_t)x0 | (uintptr_t)x1 | (uintptr_t)b0 | (uintptr_t)invd0) & 15) return 1;
    if (tb_map(&p->mx[0], x0, L0, 1) || tb_map(&p->mx[1], x1, L0, 1)) return 1;
    if (cudaFuncSetAttribute(k_rbgs_tb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mg_tb_smem()) !=
        cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    int dev = 0, nsm = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rbgs_tb, TB_THREADS, mg_tb_smem()) != cudaSuccess ||
        per < 1) {
        cudaGetLastError();
        return 1;
    }
    p->lev = L0;
    p->b = b0;
    p->invd = invd0;
    p->xo[0] = x0;
    p->xo[1] = x1;
    p->tiles_x = L0.nx / (2 * TB_W2);
    p->ntiles = p->tiles_x * (L0.ny / TB_H);
    long long units = (long long)p->ntiles * L0.nz;
    p->grid = (int)(units < (long long)nsm * per ? units : (long long)nsm * per);
    p->err = err;
    p->ok = 1;
    return 0;
}

// two sweeps (colours c0, 1-c0, c0, 1-c0) from xo[in] into xo[1-in]
void mg_tb_sweeps(cudaStream_t s, const RbTbPlan &p, int in, int c0, int zero_init, int pdl)
{
    TbArgs a;
    a.L = p.lev;
    a.b = p.b;
    a.invd = p.invd;
    a.xo = p.xo[1 - in];
    a.c0 = c0;
    a.zero_init = zero_init;
    a.tiles_x = p.tiles_x;
    a.ntiles = p.ntiles;
    a.err = p.err;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)p.grid);
    cfg.blockDim = dim3(TB_THREADS);
    cfg.dynamicSmemBytes = mg_tb_smem();
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k_rbgs_tb, p.mx[in], a);
}
