// k_conv.cu -- 3x3x3 convolutions (stride 1, zero padding 1) as implicit
// GEMMs on the tcgen05 tensor cores: BF16 operands, FP32 accumulators in
// TMEM, operands staged by TMA, one producer warp, one MMA warp and four
// epilogue warps per CTA, persistent CTAs with a double-buffered accumulator.
//
// Forward (and data gradient, the same kernel on mirrored weights):
//   out[v][co] = sum_tap sum_ci W[tap][co][ci] * in[v + off(tap)][ci]
// GEMM view per output tile: M = 128 voxels, N = cout, K = 27 taps x cin.
// On grids at least 128 voxels wide a tile is one x row and, per channel
// chunk, ONE TMA box (130 x 3 x 3 voxels) feeds all 27 taps: the A operand of
// tap (dx, dy, dz) is the same shared-memory slab at a 16-byte-granular offset.
// Narrower grids load one 128-voxel box per tap (TMA fills the padding with
// zeros either way).
//
// Weight gradient: dW[tap][co][ci] = sum_v dy[v][co] * in[v + off(tap)][ci];
// M = (taps of a group) x cin = 128 rows, N = cout, K = voxels, both operands
// MN-major straight from the channel-blocked layout.  Each CTA accumulates a
// range of voxel tiles in TMEM and adds its partial sums to FP32 dW.
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "tc_ptx.cuh"
#include "turb_conv.cuh"

namespace {

char g_conv_err[256] = "";

// barrier slots
constexpr int FA = 0, EA = 4, FB = 8, EB = 16, AF = 24, AE = 26, WB = 28, FIN = 29, NBAR = 30;

struct ConvArgs {
    int X, Y, Z, cin, cout, kc, nkc;
    int slab, bx, by, bz, ntx, nty, ntz, ntiles;
    int wres, sa, sb;
    uint32_t abytes, bbytes, astride, bstride, wbytes, a_lbo;
    const bf16 *wpk;
    const float *bias;
    int relu;
    const bf16 *skip, *mask;
    bf16 *out;
    const float *headw, *headb;
    float *hout;
    int *err;
};

__device__ __forceinline__ void fail(volatile int *abort_, int *err, int code)
{
    *abort_ = 1;
    atomicExch(err, code);
}

// last fill of stage s among `n` fills of an S-stage ring, waited for so that
// no copy is still landing when the CTA exits
__device__ __forceinline__ void drain(uint32_t bars, int base, uint32_t n, int S, volatile int *abort_)
{
    for (int s = 0; s < S; s++) {
        if ((uint32_t)s >= n) break;
        uint32_t last = (uint32_t)s + (uint32_t)S * ((n - 1 - (uint32_t)s) / (uint32_t)S);
        tc::mbar_wait(bars + 8 * (base + s), (last / S) & 1, abort_);
    }
}

// epilogue of one 128-voxel tile: this thread's accumulator row (all cout
// columns from TMEM, loaded by the whole warp) -> bias, skip, ReLU, mask,
// BF16 store, optional 1x1x1 head
struct EpiP {
    const float *bias;
    int relu;
    const bf16 *skip, *mask;
    bf16 *out;
    const float *headw, *headb;
    float *hout;
    int cout;
    size_t plane;
};

__device__ __forceinline__ void epilogue(const EpiP &a, uint32_t taddr, size_t vox, bool valid)
{
    float hsum = 0.f;
    for (int ch = 0; ch < (a.cout >> 4); ch++) {
        uint32_t rr[16];
        tc::tmem_ld16(taddr + (uint32_t)ch * 16u, rr);
        tc::tmem_wait_ld();
        if (!valid) continue;
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = __uint_as_float(rr[j]);
        if (a.bias) {
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] += a.bias[ch * 16 + j];
        }
        size_t o0 = ((size_t)(2 * ch) * a.plane + vox) * 8, o1 = o0 + a.plane * 8;
        if (a.skip) {
            uint4 s0 = *reinterpret_cast<const uint4 *>(a.skip + o0);
            uint4 s1 = *reinterpret_cast<const uint4 *>(a.skip + o1);
            const bf16 *p0 = reinterpret_cast<const bf16 *>(&s0), *p1 = reinterpret_cast<const bf16 *>(&s1);
#pragma unroll
            for (int j = 0; j < 8; j++) { v[j] += __bfloat162float(p0[j]); v[8 + j] += __bfloat162float(p1[j]); }
        }
        if (a.relu) {
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = fmaxf(v[j], 0.f);
        }
        if (a.mask) {
            uint4 m0 = *reinterpret_cast<const uint4 *>(a.mask + o0);
            uint4 m1 = *reinterpret_cast<const uint4 *>(a.mask + o1);
            const bf16 *p0 = reinterpret_cast<const bf16 *>(&m0), *p1 = reinterpret_cast<const bf16 *>(&m1);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                if (!(__bfloat162float(p0[j]) > 0.f)) v[j] = 0.f;
                if (!(__bfloat162float(p1[j]) > 0.f)) v[8 + j] = 0.f;
            }
        }
        uint4 w0, w1;
        bf16 *q0 = reinterpret_cast<bf16 *>(&w0), *q1 = reinterpret_cast<bf16 *>(&w1);
#pragma unroll
        for (int j = 0; j < 8; j++) { q0[j] = __float2bfloat16_rn(v[j]); q1[j] = __float2bfloat16_rn(v[8 + j]); }
        if (a.out) {
            *reinterpret_cast<uint4 *>(a.out + o0) = w0;
            *reinterpret_cast<uint4 *>(a.out + o1) = w1;
        }
        if (a.headw) {
#pragma unroll
            for (int j = 0; j < 8; j++) {
                hsum = fmaf(a.headw[ch * 16 + j], __bfloat162float(q0[j]), hsum);
                hsum = fmaf(a.headw[ch * 16 + 8 + j], __bfloat162float(q1[j]), hsum);
            }
        }
    }
    if (valid && a.hout) a.hout[vox] = hsum + *a.headb;
}

__global__ void __launch_bounds__(192) k_conv(const __grid_constant__ CUtensorMap mapA, ConvArgs a)
{
    extern __shared__ uint8_t dsm[];
    __shared__ __align__(8) uint64_t bar[NBAR];
    __shared__ uint32_t tslot;
    __shared__ int abort_s;
    volatile int *abort_ = &abort_s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t sraw = tc::smem_u32(dsm);
    const uint32_t sA = (sraw + 1023u) & ~1023u;
    const uint32_t nA = a.slab ? 2u : (uint32_t)a.sa;
    const uint32_t sB = sA + nA * a.astride;
    const uint32_t bars = tc::smem_u32(bar);
    const uint32_t ncols = a.cout * 2 < 32 ? 32u : (uint32_t)(a.cout * 2);

    if (threadIdx.x == 0) {
        abort_s = 0;
        for (int i = 0; i < NBAR; i++) tc::mbar_init(bars + 8 * i, (i == AE || i == AE + 1) ? 4u : 1u);
        tc::mbar_fence_init();
        tc::prefetch_map(&mapA);
    }
    if (warp == 1) {
        tc::tmem_alloc(tc::smem_u32(&tslot), ncols);
        tc::tmem_relinquish();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tbase = tslot;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t ua = 0, ub = 0;
            bool ok = true;
            if (a.wres) {
                tc::mbar_expect_tx(bars + 8 * WB, a.wbytes);
                tc::bulk_load(sB, a.wpk, a.wbytes, bars + 8 * WB);
            }
            for (int t = blockIdx.x; ok && t < a.ntiles; t += gridDim.x) {
                int tx = t % a.ntx, r = t / a.ntx, ty = r % a.nty, tz = r / a.nty;
                int x0 = tx * a.bx, y0 = ty * a.by, z0 = tz * a.bz;
                for (int kci = 0; ok && kci < a.nkc; kci++) {
                    int cb = kci * (a.kc >> 3);
                    if (a.slab) {
                        uint32_t s = ua & 1u;
                        if (!tc::mbar_wait(bars + 8 * (EA + s), ((ua >> 1) & 1u) ^ 1u, abort_)) { ok = false; break; }
                        tc::mbar_expect_tx(bars + 8 * (FA + s), a.abytes);
                        tc::tma_load5(sA + s * a.astride, &mapA, 0, x0 - 1, y0 - 1, z0 - 1, cb, bars + 8 * (FA + s));
                        ua++;
                    }
                    for (int tap = 0; tap < 27; tap++) {
                        if (!a.slab) {
                            uint32_t s = ua % (uint32_t)a.sa;
                            if (!tc::mbar_wait(bars + 8 * (EA + s), ((ua / a.sa) & 1u) ^ 1u, abort_)) { ok = false; break; }
                            int dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;
                            tc::mbar_expect_tx(bars + 8 * (FA + s), a.abytes);
                            tc::tma_load5(sA + s * a.astride, &mapA, 0, x0 + dx - 1, y0 + dy - 1, z0 + dz - 1, cb,
                                          bars + 8 * (FA + s));
                            ua++;
                        }
                        if (!a.wres) {
                            uint32_t s = ub % (uint32_t)a.sb;
                            if (!tc::mbar_wait(bars + 8 * (EB + s), ((ub / a.sb) & 1u) ^ 1u, abort_)) { ok = false; break; }
                            tc::mbar_expect_tx(bars + 8 * (FB + s), a.bbytes);
                            tc::bulk_load(sB + s * a.bstride, a.wpk + (size_t)(kci * 27 + tap) * a.kc * a.cout, a.bbytes,
                                          bars + 8 * (FB + s));
                            ub++;
                        }
                    }
                }
            }
            if (!ok) fail(abort_, a.err, 1);
            drain(bars, FA, ua, (int)nA, abort_);
            if (!a.wres) drain(bars, FB, ub, a.sb, abort_);
            if (a.wres) tc::mbar_wait(bars + 8 * WB, 0, abort_);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, a.cout, 0, 0);
            const uint32_t b_lbo = (uint32_t)a.cout * 16u;
            uint32_t ua = 0, ub = 0, it = 0;
            bool ok = true;
            if (a.wres && !tc::mbar_wait(bars + 8 * WB, 0, abort_)) ok = false;
            for (int t = blockIdx.x; ok && t < a.ntiles; t += gridDim.x, it++) {
                uint32_t ab = it & 1u;
                if (!tc::mbar_wait(bars + 8 * (AE + ab), ((it >> 1) & 1u) ^ 1u, abort_)) { ok = false; break; }
                tc::fence_after();
                uint32_t dt = tbase + ab * (uint32_t)a.cout;
                for (int kci = 0; ok && kci < a.nkc; kci++) {
                    uint32_t abuf = 0, sa_slab = 0;
                    if (a.slab) {
                        sa_slab = ua & 1u;
                        if (!tc::mbar_wait(bars + 8 * (FA + sa_slab), (ua >> 1) & 1u, abort_)) { ok = false; break; }
                        abuf = sA + sa_slab * a.astride;
                    }
                    for (int tap = 0; tap < 27; tap++) {
                        uint32_t s_a = 0, s_b = 0, bbuf, aoff = 0;
                        if (!a.slab) {
                            s_a = ua % (uint32_t)a.sa;
                            if (!tc::mbar_wait(bars + 8 * (FA + s_a), (ua / a.sa) & 1u, abort_)) { ok = false; break; }
                            abuf = sA + s_a * a.astride;
                        } else {
                            int dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;
                            aoff = (uint32_t)(((dz * 3 + dy) * (a.bx + 2) + dx) * 16);
                        }
                        if (!a.wres) {
                            s_b = ub % (uint32_t)a.sb;
                            if (!tc::mbar_wait(bars + 8 * (FB + s_b), (ub / a.sb) & 1u, abort_)) { ok = false; break; }
                            bbuf = sB + s_b * a.bstride;
                        } else {
                            bbuf = sB + (uint32_t)((kci * 27 + tap) * a.kc * a.cout * 2);
                        }
                        tc::fence_after();
                        for (int ks = 0; ks < (a.kc >> 4); ks++) {
                            uint64_t ad = tc::sdesc(abuf + aoff + (uint32_t)ks * 2u * a.a_lbo, a.a_lbo, 128);
                            uint64_t bd = tc::sdesc(bbuf + (uint32_t)ks * 2u * b_lbo, b_lbo, 128);
                            tc::mma_bf16(dt, ad, bd, idesc, (kci | tap | ks) != 0);
                        }
                        if (!a.wres) { tc::mma_commit(bars + 8 * (EB + s_b)); ub++; }
                        if (!a.slab) { tc::mma_commit(bars + 8 * (EA + s_a)); ua++; }
                    }
                    if (ok && a.slab) { tc::mma_commit(bars + 8 * (EA + sa_slab)); ua++; }
                }
                if (ok) tc::mma_commit(bars + 8 * (AF + ab));
            }
            if (!ok) fail(abort_, a.err, 1);
            tc::mma_commit(bars + 8 * FIN);
            tc::mbar_wait(bars + 8 * FIN, 0, abort_);
        }
    } else if (warp >= 2) {
        const int q = warp & 3, row = q * 32 + lane;
        const int xx = row % a.bx, yy = (row / a.bx) % a.by, zz = row / (a.bx * a.by);
        const size_t plane = (size_t)a.X * a.Y * a.Z;
        uint32_t it = 0;
        for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x, it++) {
            uint32_t ab = it & 1u;
            if (!tc::mbar_wait(bars + 8 * (AF + ab), (it >> 1) & 1u, abort_)) { fail(abort_, a.err, 1); break; }
            tc::fence_after();
            int tx = t % a.ntx, r = t / a.ntx, ty = r % a.nty, tz = r / a.nty;
            int gx = tx * a.bx + xx, gy = ty * a.by + yy, gz = tz * a.bz + zz;
            bool valid = zz < a.bz && gx < a.X && gy < a.Y && gz < a.Z;
            size_t vox = ((size_t)gz * a.Y + gy) * a.X + gx;
            uint32_t taddr = tbase + ((uint32_t)(q * 32) << 16) + ab * (uint32_t)a.cout;
            epilogue(EpiP{a.bias, a.relu, a.skip, a.mask, a.out, a.headw, a.headb, a.hout, a.cout, plane}, taddr, vox,
                     valid);
            tc::fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(bars + 8 * (AE + ab));
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 1) tc::tmem_dealloc(tbase, ncols);
}


// ---- row-ring convolution (grids at least 128 voxels wide, cin <= 32) ------------
// A CTA takes items of (x tile of 128 voxels, z, a run of consecutive y rows).
// Operands use the 128-byte-swizzle K-major layout, the one the tensor core
// fetches fastest: every shared-memory row is one voxel holding 64 K elements,
// here the channels of its three z planes (K = dz * cin + ci, zero padded),
// 16-byte chunk c of row p stored at chunk c ^ (p % 8).  One input y row of
// the tile (136 voxel rows, x0 - 1 ...) is a ring slot, filled by 16-byte
// cp.async (producer warp L % 4 loads row L).  The A operand of tap dx is the
// slot shifted by dx rows; dz and the channels are the K steps.  Every input row r feeds the output rows r+1, r, r-1
// (dy = 0, 1, 2): the weights of the three dy taps are stacked along N, so
// one MMA (M = 128 voxels, N = 3 cout, K = 16) per dx and K step covers all
// of them; the three targets are consecutive blocks of a TMEM ring of NBLK
// accumulator blocks (block of virtual row v = NBLK-1 - v mod NBLK, so rows
// r+1, r, r-1 are ascending; a wrap splits the MMA).  Accumulation is always
// on: the epilogue zeroes a block after draining it.  Weights are resident.
constexpr int RING = 4, RW = 130, RROWS = 136;   // ring slots, voxels used / stored per slot
constexpr int NBLK = 8;                          // TMEM accumulator blocks

struct RowArgs {
    int X, Y, Z, cin, cout;
    int ntx, ych, nyc, nitems;
    int nkb;                      // 128-byte K blocks per voxel row: ceil(3 cin / 64)
    uint32_t slot_bytes, slab_bytes, wbytes;
    const bf16 *in, *wpk;
    EpiP epi;
    int *err;
};

__host__ __device__ inline int rows_nkb(int cin) { return (3 * cin + 63) / 64; }
// resident weights of the row kernel: per dx and K block, 3 cout rows of 128 bytes
__host__ __device__ inline uint32_t rows_wbytes(int cin, int cout) { return 3u * (uint32_t)rows_nkb(cin) * 3u * cout * 128u; }
// 128-byte-swizzle K-major operand at saddr (8-row groups 1024 bytes apart);
// the swizzle follows the absolute address, so shifted starts need no offset
__host__ __device__ inline uint64_t sw128_desc(uint32_t saddr)
{
    return tc::sdesc(saddr, 16, 1024) | (2ull << 61);
}

// barrier slots of k_conv_rows
constexpr int RF = 0, RE = RING, BRDY = 2 * RING, BFREE = 2 * RING + NBLK, RWB = 2 * RING + 2 * NBLK,
              RFIN = RWB + 1, RNBAR = RWB + 2;

__host__ __device__ inline uint32_t rows_ncols(int cout)
{
    uint32_t n = 32;
    while (n < (uint32_t)(NBLK * cout)) n <<= 1;
    return n;
}
__device__ __forceinline__ int blk_of(uint32_t v) { return NBLK - 1 - (int)(v % NBLK); }

__device__ __forceinline__ void tmem_st16_zero(uint32_t taddr)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
        "%1};" ::"r"(taddr),
        "r"(0u)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void row_item(const RowArgs &a, int it, int &x0, int &z, int &yb, int &ny)
{
    int tx = it % a.ntx, r = it / a.ntx;
    z = r % a.Z;
    int yc = r / a.Z;
    x0 = tx * 128;
    yb = yc * a.ych;
    ny = min(a.ych, a.Y - yb);
}

__global__ void __launch_bounds__(288) k_conv_rows(RowArgs a)
{
    extern __shared__ uint8_t dsm[];
    __shared__ __align__(8) uint64_t bar[RNBAR];
    __shared__ uint32_t tslot;
    __shared__ int abort_s;
    volatile int *abort_ = &abort_s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t sS = (tc::smem_u32(dsm) + 1023u) & ~1023u;   // slab ring
    const uint32_t sW = sS + ((a.slab_bytes + 1023u) & ~1023u);  // resident stacked weights
    const uint32_t bars = tc::smem_u32(bar);
    const uint32_t ncols = rows_ncols(a.cout);
    const int nkg = a.cin >> 3;           // channel blocks of 8
    const int nreal = 3 * nkg;            // real 16-byte chunks per voxel row (3 z planes)

    if (threadIdx.x == 0) {
        abort_s = 0;
        for (int i = 0; i < RNBAR; i++) {
            uint32_t cnt = 1;
            if (i >= RF && i < RF + RING) cnt = 32;             // the producer warp of the row
            if (i >= BFREE && i < BFREE + NBLK) cnt = 4;       // epilogue warps
            tc::mbar_init(bars + 8 * i, cnt);
        }
        tc::mbar_fence_init();
    }
    if (warp == 8) {
        tc::tmem_alloc(tc::smem_u32(&tslot), ncols);
        tc::tmem_relinquish();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tbase = tslot;
    if (warp < 4) {   // accumulators start at zero
        for (int b = 0; b < NBLK; b++)
            for (int ch = 0; ch < (a.cout >> 4); ch++)
                tmem_st16_zero(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * a.cout + ch * 16));
        tmem_wait_st();
    } else if (warp < 8) {   // K padding chunks of the slab are never loaded: zero them once
        uint8_t *g = dsm + (sS - tc::smem_u32(dsm));
        int npad = 8 * a.nkb - nreal;
        for (int i = threadIdx.x - 128; i < RING * RROWS * npad; i += 128) {
            int c = nreal + i % npad, r = i / npad, p = r % RROWS, slot = r / RROWS;
            int kb = c >> 3, cc = c & 7;
            uint32_t off = (uint32_t)slot * a.slot_bytes + (uint32_t)kb * (RROWS * 128) + (uint32_t)p * 128u +
                           (uint32_t)((cc ^ (p & 7)) << 4);
            *reinterpret_cast<uint4 *>(g + off) = make_uint4(0, 0, 0, 0);
        }
        tc::fence_proxy_async();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();

    if (warp >= 4 && warp < 8) {
        // ---- producers
        const int pw = warp - 4;
        if (pw == 0 && lane == 0) {
            tc::mbar_expect_tx(bars + 8 * RWB, a.wbytes);
            tc::bulk_load(sW, a.wpk, a.wbytes, bars + 8 * RWB);
        }
        uint32_t L = 0;
        bool ok = true;
        for (int it = blockIdx.x; ok && it < a.nitems; it += gridDim.x) {
            int x0, z, yb, ny;
            row_item(a, it, x0, z, yb, ny);
            for (int j = 0; j < ny + 2; j++, L++) {
                if ((int)(L & 3u) != pw) continue;
                uint32_t slot = L % RING;
                if (L >= RING && !tc::mbar_wait(bars + 8 * (RE + slot), ((L / RING) & 1u) ^ 1u, abort_)) {
                    ok = false;
                    break;
                }
                // chunk c = dz * nkg + cb of voxel row p (x = x0 - 1 + p) comes from
                // channel block cb of plane z + dz - 1; zero outside the grid
                int yy = yb - 1 + j;
                bool yok = yy >= 0 && yy < a.Y;
                uint32_t fullb = bars + 8 * (RF + slot);
                uint32_t sbase = sS + slot * a.slot_bytes;
                for (int c = 0; c < nreal; c++) {
                    int dz = c / nkg, cb = c - dz * nkg, zz = z + dz - 1, kb = c >> 3, cc = c & 7;
                    bool rok = yok && zz >= 0 && zz < a.Z;
                    const bf16 *rsrc = a.in + ((((size_t)cb * a.Z + (rok ? zz : 0)) * a.Y + (rok ? yy : 0)) * a.X) * 8;
                    uint32_t rdst = sbase + (uint32_t)kb * (RROWS * 128);
                    for (int p = lane; p < RW; p += 32) {
                        int xg = x0 - 1 + p;
                        bool v = rok && xg >= 0 && xg < a.X;
                        cp_async16(rdst + (uint32_t)p * 128u + (uint32_t)((cc ^ (p & 7)) << 4),
                                   v ? rsrc + (size_t)xg * 8 : a.in, v ? 16u : 0u);
                    }
                }
                cp_async_commit();
                cp_async_wait0();
                tc::fence_proxy_async();
                tc::mbar_arrive(fullb);
            }
        }
        cp_async_wait0();
        if (!ok) fail(abort_, a.err, 3);
        if (pw == 0 && lane == 0) tc::mbar_wait(bars + 8 * RWB, 0, abort_);
    } else if (warp == 8) {
        if (lane == 0) {
            const uint32_t N3 = 3u * (uint32_t)a.cout;
            const uint32_t wreg = N3 * 128u;                        // weights of one (dx, K block)
            const int nks = (3 * a.cin) / 16;                       // K steps of 16 per dx
            uint32_t L = 0, V = 0;
            bool ok = tc::mbar_wait(bars + 8 * RWB, 0, abort_);
            for (int it = blockIdx.x; ok && it < a.nitems; it += gridDim.x) {
                int x0, z, yb, ny;
                row_item(a, it, x0, z, yb, ny);
                const int nv = ny + 2;   // virtual output rows yb-1 .. yb+ny of this item
                for (int j = 0; ok && j < nv; j++) {
                    // blocks touched for the first time: rows j+1 (and j at the start)
                    for (int v = (j == 0 ? 0 : j + 1); v <= j + 1 && v < nv; v++) {
                        uint32_t g = V + (uint32_t)v;
                        if (!tc::mbar_wait(bars + 8 * (BFREE + blk_of(g)), ((g / NBLK) & 1u) ^ 1u, abort_)) { ok = false; break; }
                    }
                    uint32_t Lr = L + (uint32_t)j, slot = Lr % RING;
                    if (!ok || !tc::mbar_wait(bars + 8 * (RF + slot), (Lr / RING) & 1u, abort_)) { ok = false; break; }
                    tc::fence_after();
                    // runs of consecutive valid target blocks among rows j+1, j, j-1 (k = dy)
                    int kb[3], kv[3];
                    for (int k = 0; k < 3; k++) {
                        int row = j + 1 - k;
                        kv[k] = row >= 0 && row < nv;
                        kb[k] = kv[k] ? blk_of(V + (uint32_t)row) : -1;
                    }
                    const uint32_t sbase = sS + slot * a.slot_bytes;
                    for (int dx = 0; dx < 3; dx++) {
                        int k = 0;
                        while (k < 3) {
                            if (!kv[k]) { k++; continue; }
                            int k1 = k + 1;
                            while (k1 < 3 && kv[k1] && kb[k1] == kb[k1 - 1] + 1) k1++;
                            uint32_t n = (uint32_t)(k1 - k) * (uint32_t)a.cout;
                            uint32_t idesc = tc::idesc_bf16(128, (int)n, 0, 0);
                            uint32_t dt = tbase + (uint32_t)(kb[k] * a.cout);
                            for (int ks = 0; ks < nks; ks++) {
                                uint32_t kbk = (uint32_t)(ks >> 2), kk = (uint32_t)(ks & 3);
                                uint64_t ad = sw128_desc(sbase + kbk * (RROWS * 128) + (uint32_t)dx * 128u + kk * 32u);
                                uint64_t bd = sw128_desc(sW + ((uint32_t)dx * (uint32_t)a.nkb + kbk) * wreg +
                                                         (uint32_t)(k * a.cout) * 128u + kk * 32u);
                                tc::mma_bf16(dt, ad, bd, idesc, 1u);
                            }
                            k = k1;
                        }
                    }
                    tc::mma_commit(bars + 8 * (RE + slot));                           // input row done
                    if (j >= 1) tc::mma_commit(bars + 8 * (BRDY + kb[2]));            // output row j-1 done
                }
                if (!ok) break;
                tc::mma_commit(bars + 8 * (BRDY + blk_of(V + (uint32_t)(nv - 1))));   // partial last row
                L += (uint32_t)nv;
                V += (uint32_t)nv;
            }
            if (!ok) fail(abort_, a.err, 3);
            tc::mma_commit(bars + 8 * RFIN);
            tc::mbar_wait(bars + 8 * RFIN, 0, abort_);
        }
    } else if (warp < 4) {
        // ---- epilogue: drain each virtual row's block, store the real rows, zero it
        const int row = warp * 32 + lane;
        uint32_t V = 0;
        bool ok = true;
        for (int it = blockIdx.x; ok && it < a.nitems; it += gridDim.x) {
            int x0, z, yb, ny;
            row_item(a, it, x0, z, yb, ny);
            for (int j = 0; j < ny + 2; j++) {
                uint32_t g = V + (uint32_t)j;
                int b = blk_of(g);
                if (!tc::mbar_wait(bars + 8 * (BRDY + b), (g / NBLK) & 1u, abort_)) { fail(abort_, a.err, 3); ok = false; break; }
                tc::fence_after();
                uint32_t taddr = tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * a.cout);
                if (j >= 1 && j <= ny) {
                    int gx = x0 + row;
                    size_t vox = ((size_t)z * a.Y + (yb + j - 1)) * a.X + gx;
                    epilogue(a.epi, taddr, vox, gx < a.X);
                }
                for (int ch = 0; ch < (a.cout >> 4); ch++) tmem_st16_zero(taddr + (uint32_t)ch * 16u);
                tmem_wait_st();
                tc::fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(bars + 8 * (BFREE + b));
            }
            V += (uint32_t)(ny + 2);
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 8) tc::tmem_dealloc(tbase, ncols);
}

// ---- weight gradient --------------------------------------------------------------
struct WgArgs {
    int X, Y, Z, cin, cout, G, ngroups, nsplit;
    int bx, by, bz, nb, ntx, nty, ntz, ntiles;
    uint32_t tapbytes, bbytes, stride;
    float *dw;
    int *err;
};

constexpr int WG_STAGES = 3;

__global__ void __launch_bounds__(192) k_wgrad(const __grid_constant__ CUtensorMap mapX,
                                               const __grid_constant__ CUtensorMap mapD, WgArgs a)
{
    extern __shared__ uint8_t dsm[];
    __shared__ __align__(8) uint64_t bar[2 * WG_STAGES + 2];
    __shared__ uint32_t tslot;
    __shared__ int abort_s;
    volatile int *abort_ = &abort_s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t s0 = (tc::smem_u32(dsm) + 1023u) & ~1023u;
    const uint32_t bars = tc::smem_u32(bar);
    const int F = 0, E = WG_STAGES, DONE = 2 * WG_STAGES, FINB = 2 * WG_STAGES + 1;
    const uint32_t ncols = a.cout < 32 ? 32u : (uint32_t)a.cout;
    const int g = blockIdx.x % a.ngroups, sp = blockIdx.x / a.ngroups;
    const int ntaps = min(a.G, 27 - g * a.G);

    if (threadIdx.x == 0) {
        abort_s = 0;
        for (int i = 0; i < 2 * WG_STAGES + 2; i++) tc::mbar_init(bars + 8 * i, 1);
        tc::mbar_fence_init();
        tc::prefetch_map(&mapX);
        tc::prefetch_map(&mapD);
    }
    if (warp == 1) {
        tc::tmem_alloc(tc::smem_u32(&tslot), ncols);
        tc::tmem_relinquish();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tbase = tslot;
    const uint32_t sbo = (uint32_t)a.nb * 16u;   // next 8 channels
    const int nks = a.nb >> 4;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t u = 0;
            bool ok = true;
            for (int t = sp; t < a.ntiles; t += a.nsplit) {
                int tx = t % a.ntx, r = t / a.ntx, ty = r % a.nty, tz = r / a.nty;
                int x0 = tx * a.bx, y0 = ty * a.by, z0 = tz * a.bz;
                uint32_t s = u % WG_STAGES;
                if (!tc::mbar_wait(bars + 8 * (E + s), ((u / WG_STAGES) & 1u) ^ 1u, abort_)) { ok = false; break; }
                uint32_t buf = s0 + s * a.stride;
                tc::mbar_expect_tx(bars + 8 * (F + s), (uint32_t)ntaps * a.tapbytes + a.bbytes);
                for (int tl = 0; tl < ntaps; tl++) {
                    int tap = g * a.G + tl, dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;
                    tc::tma_load5(buf + (uint32_t)tl * a.tapbytes, &mapX, 0, x0 + dx - 1, y0 + dy - 1, z0 + dz - 1, 0,
                                  bars + 8 * (F + s));
                }
                tc::tma_load5(buf + (uint32_t)a.G * a.tapbytes, &mapD, 0, x0, y0, z0, 0, bars + 8 * (F + s));
                u++;
            }
            if (!ok) fail(abort_, a.err, 2);
            drain(bars, F, u, WG_STAGES, abort_);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, a.cout, 1, 1);
            uint32_t u = 0;
            bool ok = true;
            for (int t = sp; t < a.ntiles; t += a.nsplit) {
                uint32_t s = u % WG_STAGES;
                if (!tc::mbar_wait(bars + 8 * (F + s), (u / WG_STAGES) & 1u, abort_)) { ok = false; break; }
                tc::fence_after();
                uint32_t abuf = s0 + s * a.stride, bbuf = abuf + (uint32_t)a.G * a.tapbytes;
                for (int ks = 0; ks < nks; ks++) {
                    uint64_t ad = tc::sdesc(abuf + (uint32_t)ks * 256u, 128, sbo);
                    uint64_t bd = tc::sdesc(bbuf + (uint32_t)ks * 256u, 128, sbo);
                    tc::mma_bf16(tbase, ad, bd, idesc, (u | (uint32_t)ks) != 0);
                }
                tc::mma_commit(bars + 8 * (E + s));
                u++;
            }
            if (!ok) fail(abort_, a.err, 2);
            tc::mma_commit(bars + 8 * DONE);
            tc::mma_commit(bars + 8 * FINB);
            tc::mbar_wait(bars + 8 * FINB, 0, abort_);
        }
    } else if (warp >= 2) {
        const int q = warp & 3, row = q * 32 + lane;
        const bool have = sp < a.ntiles;
        if (have) {
            if (!tc::mbar_wait(bars + 8 * DONE, 0, abort_)) {
                fail(abort_, a.err, 2);
            } else {
                tc::fence_after();
                const int tl = row / a.cin, ci = row % a.cin, tap = g * a.G + tl;
                const bool valid = tl < ntaps && !*abort_;
                uint32_t taddr = tbase + ((uint32_t)(q * 32) << 16);
                for (int ch = 0; ch < (a.cout >> 4); ch++) {
                    uint32_t rr[16];
                    tc::tmem_ld16(taddr + (uint32_t)ch * 16u, rr);
                    tc::tmem_wait_ld();
                    if (!valid) continue;
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        atomicAdd(a.dw + ((size_t)tap * a.cout + ch * 16 + j) * a.cin + ci, __uint_as_float(rr[j]));
                }
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 1) tc::tmem_dealloc(tbase, ncols);
}

// ---- descriptor self-test ------------------------------------------------------------
// One CTA: A (128 x 32) and B (64 x 32) written by the threads into shared
// memory in a K-major or MN-major core-matrix layout, two MMAs (K = 16 each)
// into TMEM, the result compared with an exact FP32 product (all values are
// small multiples of 1/4, so every sum is exact).  Shared memory is sized so
// that every read stays inside it even if the LBO and SBO fields are swapped.
// swap = 2 issues no MMA: the completion wait then runs out after its time
// limit, which is how the bounded waits are tested (result: 1000000 + the
// wrong values of the untouched accumulator).
constexpr int ST_M = 128, ST_N = 64, ST_K = 32, ST_SMEM = 128 * 1024;

__device__ __forceinline__ float st_a(int m, int k) { return (float)(((m * 3 + k * 7) % 9) - 4) * 0.25f; }
__device__ __forceinline__ float st_b(int n, int k) { return (float)(((n * 5 + k * 3) % 7) - 3) * 0.5f; }

// mn = 2: both operands in the 128-byte-swizzle K-major layout (rows of 64
// elements, 16-byte chunk c of row r stored at chunk c ^ (r % 8)), K = 64 in
// four MMAs advancing 32 bytes; A starts `swap` (0..7) rows into a 136-row
// tile.  The swizzle is applied to absolute shared-memory address bits, so a
// start that is not 1024-byte aligned needs no base offset (field left 0).
constexpr int SW_K = 64;
__device__ __forceinline__ float sw_a(int p, int k) { return (float)(((p * 5 + k * 3) % 11) - 5) * 0.25f; }

__global__ void __launch_bounds__(128) k_umma_selftest(int mn, int swap, unsigned long long *bad)
{
    extern __shared__ uint8_t dsm[];
    __shared__ __align__(8) uint64_t bar[1];
    __shared__ uint32_t tslot;
    __shared__ int abort_s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t s0 = (tc::smem_u32(dsm) + 1023u) & ~1023u;
    uint8_t *g0 = dsm + (s0 - tc::smem_u32(dsm));
    const uint32_t offB = 32 * 1024;
    if (threadIdx.x == 0) {
        abort_s = 0;
        tc::mbar_init(tc::smem_u32(bar), 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_u32(&tslot), 64);
        tc::tmem_relinquish();
    }
    for (int i = threadIdx.x; i < (ST_SMEM - 1024) / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(g0)[i] = 0u;
    __syncthreads();
    if (mn == 2) {
        for (int i = threadIdx.x; i < 136 * SW_K; i += blockDim.x) {
            int p = i / SW_K, k = i % SW_K;
            uint32_t off = (uint32_t)(p * 128 + (((k >> 3) ^ (p & 7)) << 4) + (k & 7) * 2);
            *reinterpret_cast<bf16 *>(g0 + off) = __float2bfloat16_rn(sw_a(p, k));
        }
        for (int i = threadIdx.x; i < ST_N * SW_K; i += blockDim.x) {
            int n = i / SW_K, k = i % SW_K;
            uint32_t off = (uint32_t)(n * 128 + (((k >> 3) ^ (n & 7)) << 4) + (k & 7) * 2);
            *reinterpret_cast<bf16 *>(g0 + offB + off) = __float2bfloat16_rn(st_b(n, k));
        }
    }
    for (int i = threadIdx.x; mn != 2 && i < ST_M * ST_K; i += blockDim.x) {
        int m = i / ST_K, k = i % ST_K;
        uint32_t off = mn ? (uint32_t)((m / 8) * (ST_K * 16) + (k / 8) * 128 + (k % 8) * 16 + (m % 8) * 2)
                          : (uint32_t)((k / 8) * (ST_M * 16) + (m / 8) * 128 + (m % 8) * 16 + (k % 8) * 2);
        *reinterpret_cast<bf16 *>(g0 + off) = __float2bfloat16_rn(st_a(m, k));
    }
    for (int i = threadIdx.x; mn != 2 && i < ST_N * ST_K; i += blockDim.x) {
        int n = i / ST_K, k = i % ST_K;
        uint32_t off = mn ? (uint32_t)((n / 8) * (ST_K * 16) + (k / 8) * 128 + (k % 8) * 16 + (n % 8) * 2)
                          : (uint32_t)((k / 8) * (ST_N * 16) + (n / 8) * 128 + (n % 8) * 16 + (k % 8) * 2);
        *reinterpret_cast<bf16 *>(g0 + offB + off) = __float2bfloat16_rn(st_b(n, k));
    }
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tbase = tslot;
    if (threadIdx.x == 0 && mn == 2) {
        uint32_t idesc = tc::idesc_bf16(ST_M, ST_N, 0, 0);
        uint32_t sh = (uint32_t)swap & 7u;
        for (int ks = 0; ks < SW_K / 16; ks++) {
            uint32_t aa = s0 + sh * 128u + (uint32_t)ks * 32u, bb = s0 + offB + (uint32_t)ks * 32u;
            uint64_t ad = tc::sdesc(aa, 16, 1024) | (2ull << 61);
            uint64_t bd = tc::sdesc(bb, 16, 1024) | (2ull << 61);
            tc::mma_bf16(tbase, ad, bd, idesc, ks > 0);
        }
        tc::mma_commit(tc::smem_u32(bar));
    } else if (threadIdx.x == 0 && swap != 2) {
        // (K-group stride, M/N-group stride) of the layouts written above
        uint32_t a_k = mn ? 128u : ST_M * 16u, a_m = mn ? ST_K * 16u : 128u;
        uint32_t b_k = mn ? 128u : ST_N * 16u, b_n = mn ? ST_K * 16u : 128u;
        uint32_t idesc = tc::idesc_bf16(ST_M, ST_N, mn, mn);
        for (int ks = 0; ks < ST_K / 16; ks++) {
            uint32_t aa = s0 + (uint32_t)ks * 2u * a_k, bb = s0 + offB + (uint32_t)ks * 2u * b_k;
            uint64_t ad = swap ? tc::sdesc(aa, a_m, a_k) : tc::sdesc(aa, a_k, a_m);
            uint64_t bd = swap ? tc::sdesc(bb, b_n, b_k) : tc::sdesc(bb, b_k, b_n);
            tc::mma_bf16(tbase, ad, bd, idesc, ks > 0);
        }
        tc::mma_commit(tc::smem_u32(bar));
    }
    bool ok = tc::mbar_wait(tc::smem_u32(bar), 0, &abort_s);
    tc::fence_after();
    unsigned long long nbad = ok ? 0ull : 1000000ull;
    int row = (warp & 3) * 32 + lane;
    for (int ch = 0; ch < ST_N / 16; ch++) {
        uint32_t rr[16];
        tc::tmem_ld16(tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)ch * 16u, rr);
        tc::tmem_wait_ld();
        for (int j = 0; j < 16; j++) {
            int n = ch * 16 + j;
            float ref = 0.f;
            if (mn == 2) {
                for (int k = 0; k < SW_K; k++) ref += sw_a(row + (swap & 7), k) * st_b(n, k);
            } else {
                for (int k = 0; k < ST_K; k++) ref += st_a(row, k) * st_b(n, k);
            }
            if (__uint_as_float(rr[j]) != ref) nbad++;
        }
    }
    atomicAdd(bad, nbad);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::tmem_dealloc(tbase, 64);
}

// ---- weight packing ------------------------------------------------------------------
// Standard layout (TMA kernel), per (channel chunk, tap) the B operand
// [kc/8][N][8]:
//   fwd: wf[((kci*27 + tap)*(kc/8) + kg)*cout + n][e] = W[tap][n][kci*kc + kg*8 + e]
//   bwd: wd[((kci*27 + tap)*(kcb/8) + kg)*cin + n][e] = W[26 - tap][kci*kcb + kg*8 + e][n]
// Row-kernel layout (kc = cin): per (dx, 128-byte K block) the rows
// n' = dy * N + n (three dy taps stacked along N) of 64 K elements
// K = dz * cin + k, 128-byte swizzled: byte
//   ((dx * nkb + K / 64) * 3N + n') * 128 + (((K % 64) / 8) ^ (n' % 8)) * 16 + (K % 8) * 2
__device__ __forceinline__ long long pack_index(int stacked, int kc, int nout, int tap, int n, int k)
{
    int kci = k / kc, r = k % kc, kg = r >> 3, e = r & 7;
    if (!stacked) return ((((long long)kci * 27 + tap) * (kc >> 3) + kg) * nout + n) * 8 + e;
    int dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;
    int K = dz * kc + k, kb = K >> 6, k64 = K & 63, np = dy * nout + n, nkb = rows_nkb(kc);
    long long byte = ((long long)(dx * nkb + kb) * (3 * nout) + np) * 128 + (((k64 >> 3) ^ (np & 7)) << 4) + (k64 & 7) * 2;
    return byte >> 1;
}

__global__ void k_pack(const float *__restrict__ W, int cin, int cout, int kcf, int kcb, int stf, int stb,
                       bf16 *__restrict__ wf, bf16 *__restrict__ wd)
{
    long long n = 27LL * cin * cout;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        int ci = (int)(idx % cin);
        long long t = idx / cin;
        int co = (int)(t % cout), tap = (int)(t / cout);
        bf16 w = __float2bfloat16_rn(W[idx]);
        wf[pack_index(stf, kcf, cout, tap, co, ci)] = w;
        wd[pack_index(stb, kcb, cin, 26 - tap, ci, co)] = w;
    }
}

// ---- host -----------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

int get_encode()
{
    std::call_once(g_encode_once, []() {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    return g_encode ? 0 : 1;
}

// channel-blocked tensor [C/8][Z][Y][X][8] as a 5-D map (8, X, Y, Z, C/8)
int make_map(CUtensorMap *m, const void *ptr, int X, int Y, int Z, int C, int b1, int b2, int b3, int b4)
{
    if (get_encode()) { snprintf(g_conv_err, sizeof(g_conv_err), "cuTensorMapEncodeTiled unavailable"); return 1; }
    cuuint64_t dims[5] = {8, (cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)(C / 8)};
    cuuint64_t str[4] = {16, (cuuint64_t)X * 16, (cuuint64_t)X * Y * 16, (cuuint64_t)X * Y * Z * 16};
    cuuint32_t box[5] = {8, (cuuint32_t)b1, (cuuint32_t)b2, (cuuint32_t)b3, (cuuint32_t)b4};
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(ptr), dims, str, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        snprintf(g_conv_err, sizeof(g_conv_err), "cuTensorMapEncodeTiled failed (%d) for %dx%dx%dx%d box %d,%d,%d,%d",
                 (int)r, X, Y, Z, C, b1, b2, b3, b4);
        return 1;
    }
    return 0;
}

inline uint32_t r1024(uint32_t v) { return (v + 1023u) & ~1023u; }

void tile_dims(int X, int Y, int Z, int &bx, int &by, int &bz)
{
    bx = X < 128 ? X : 128;
    by = Y < 128 / bx ? Y : 128 / bx;
    bz = Z < 128 / (bx * by) ? Z : 128 / (bx * by);
}

// largest dynamic shared memory a launch of fn may request (opt-in limit
// minus the kernel's static shared memory); set as fn's attribute once
int dyn_smem_limit(const void *fn)
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) return 0;
    int lim = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess) return 0;
    return lim;
}

int launch_error(const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return 0;
    snprintf(g_conv_err, sizeof(g_conv_err), "%s launch: %s", what, cudaGetErrorString(e));
    return 1;
}

// resident CTAs per SM allowed by shared memory (228 KB per SM, 1 KB reserved
// per CTA) and TMEM (512 columns), at most 4
int ctas_per_sm(uint32_t smem, int ncols)
{
    int n = (int)((228u * 1024u) / (smem + 1024u + 512u));
    int t = 512 / ncols;
    if (n > t) n = t;
    if (n > 4) n = 4;
    return n < 1 ? 1 : n;
}


}  // namespace

const char *conv_last_error() { return g_conv_err; }

ConvPlan conv_plan(int X, int Y, int Z, int cin, int cout)
{
    ConvPlan p{};
    p.slab = X >= 128;
    p.rows = X >= 128 && cin <= 32 && cout <= 32;
    p.kc = cin < (p.slab ? 32 : 64) ? cin : (p.slab ? 32 : 64);
    p.nkc = cin / p.kc;
    if (p.slab) { p.bx = 128; p.by = 1; p.bz = 1; }
    else tile_dims(X, Y, Z, p.bx, p.by, p.bz);
    p.nb = p.bx * p.by * p.bz;
    p.ntx = (X + p.bx - 1) / p.bx; p.nty = (Y + p.by - 1) / p.by; p.ntz = (Z + p.bz - 1) / p.bz;
    p.ntiles = p.ntx * p.nty * p.ntz;
    p.wbytes = 27u * cin * cout * 2u;
    p.wres = p.wbytes <= 65536u;
    p.sa = 4; p.sb = 4;
    if (p.slab) {
        p.abytes = 8u * (p.bx + 2) * 3u * 3u * (p.kc / 8) * 2u;
        p.a_lbo = (uint32_t)(p.bx + 2) * 9u * 16u;
    } else {
        p.abytes = (uint32_t)p.nb * p.kc * 2u;
        p.a_lbo = (uint32_t)p.nb * 16u;
    }
    // a stage always spans 128 rows per 8 channels so that the MMA reads stay in it
    p.astride = r1024(p.abytes > 256u * p.kc ? p.abytes : 256u * p.kc);
    p.bbytes = (uint32_t)p.kc * cout * 2u;
    p.bstride = r1024(p.bbytes);
    uint32_t na = p.slab ? 2u : (uint32_t)p.sa;
    p.smem = na * p.astride + (p.wres ? r1024(p.wbytes) : (uint32_t)p.sb * p.bstride) + 1024u;
    p.ncols = cout * 2 < 32 ? 32 : cout * 2;
    return p;
}

void conv_pack_weights(cudaStream_t s, const float *W, int cin, int cout, const ConvPlan &pf, const ConvPlan &pb,
                       bf16 *wf, bf16 *wd)
{
    long long n = 27LL * cin * cout;
    int nb = (int)((n + 255) / 256);
    k_pack<<<nb < 2048 ? nb : 2048, 256, 0, s>>>(W, cin, cout, pf.kc, pb.kc, pf.rows, pb.rows, wf, wd);
}

int conv3_fwd(cudaStream_t s, const bf16 *in, int X, int Y, int Z, int cin, int cout, const bf16 *wpk,
              const ConvEpi &e, int *err, int nsm)
{
    if (cin % 16 || cout % 16 || cout > 128 || cin > 128) { snprintf(g_conv_err, sizeof(g_conv_err), "conv channels"); return 1; }
    ConvPlan p = conv_plan(X, Y, Z, cin, cout);
    CUtensorMap map;
    int rc = p.slab ? make_map(&map, in, X, Y, Z, cin, p.bx + 2, 3, 3, p.kc / 8)
                    : make_map(&map, in, X, Y, Z, cin, p.bx, p.by, p.bz, p.kc / 8);
    if (rc) return 1;
    ConvArgs a{};
    a.X = X; a.Y = Y; a.Z = Z; a.cin = cin; a.cout = cout; a.kc = p.kc; a.nkc = p.nkc;
    a.slab = p.slab; a.bx = p.bx; a.by = p.by; a.bz = p.bz; a.ntx = p.ntx; a.nty = p.nty; a.ntz = p.ntz;
    a.ntiles = p.ntiles; a.wres = p.wres; a.sa = p.sa; a.sb = p.sb;
    a.abytes = p.abytes; a.bbytes = p.bbytes; a.astride = p.astride; a.bstride = p.bstride; a.wbytes = p.wbytes;
    a.a_lbo = p.a_lbo; a.wpk = wpk;
    a.bias = e.bias; a.relu = e.relu; a.skip = e.skip; a.mask = e.mask; a.out = e.out;
    a.headw = e.headw; a.headb = e.headb; a.hout = e.hout; a.err = err;
    if (p.rows) {
        RowArgs r{};
        r.X = X; r.Y = Y; r.Z = Z; r.cin = cin; r.cout = cout;
        r.ntx = (X + 127) / 128;
        r.nkb = rows_nkb(cin);
        r.slot_bytes = (uint32_t)r.nkb * RROWS * 128u;
        r.slab_bytes = RING * r.slot_bytes;
        r.wbytes = rows_wbytes(cin, cout);
        r.in = in; r.wpk = wpk;
        r.epi = EpiP{e.bias, e.relu, e.skip, e.mask, e.out, e.headw, e.headb, e.hout, cout, (size_t)X * Y * Z};
        r.err = err;
        uint32_t smem = ((r.slab_bytes + 1023u) & ~1023u) + ((r.wbytes + 1023u) & ~1023u) + 1024u;
        static int rlim = dyn_smem_limit((const void *)k_conv_rows);
        if ((int)smem > rlim) { snprintf(g_conv_err, sizeof(g_conv_err), "conv rows needs %u B of shared memory", smem); return 1; }
        int bps = ctas_per_sm(smem, (int)rows_ncols(cout));
        int grid = nsm * bps;
        // rows per item: up to 32, fewer when that leaves CTAs without two items
        long long rows = (long long)r.ntx * Z * Y;
        r.ych = 32;
        while (r.ych > 4 && rows / r.ych < 2LL * grid) r.ych >>= 1;
        r.nyc = (Y + r.ych - 1) / r.ych;
        r.nitems = r.ntx * Z * r.nyc;
        if (grid > r.nitems) grid = r.nitems;
        k_conv_rows<<<grid, 288, smem, s>>>(r);
        return launch_error("k_conv_rows");
    }
    static int lim = dyn_smem_limit((const void *)k_conv);
    if ((int)p.smem > lim) { snprintf(g_conv_err, sizeof(g_conv_err), "conv needs %u B of shared memory", p.smem); return 1; }
    int bps = ctas_per_sm(p.smem, p.ncols);
    int grid = nsm * bps;
    if (grid > p.ntiles) grid = p.ntiles;
    k_conv<<<grid, 192, p.smem, s>>>(map, a);
    return launch_error("k_conv");
}

int conv3_wgrad(cudaStream_t s, const bf16 *x, const bf16 *dy, int X, int Y, int Z, int cin, int cout, float *dw,
                int *err, int nsm)
{
    if (cin % 16 || cout % 16 || cout > 128 || cin > 128) { snprintf(g_conv_err, sizeof(g_conv_err), "wgrad channels"); return 1; }
    WgArgs a{};
    tile_dims(X, Y, Z, a.bx, a.by, a.bz);
    a.nb = a.bx * a.by * a.bz;
    if (a.nb % 16) { snprintf(g_conv_err, sizeof(g_conv_err), "wgrad grid below 16 voxels"); return 1; }
    a.X = X; a.Y = Y; a.Z = Z; a.cin = cin; a.cout = cout;
    a.G = 128 / cin; a.ngroups = (27 + a.G - 1) / a.G;
    a.ntx = (X + a.bx - 1) / a.bx; a.nty = (Y + a.by - 1) / a.by; a.ntz = (Z + a.bz - 1) / a.bz;
    a.ntiles = a.ntx * a.nty * a.ntz;
    a.tapbytes = (uint32_t)a.nb * cin * 2u;
    a.bbytes = (uint32_t)a.nb * cout * 2u;
    // operand reads span 128 rows per 8 channels: keep that much room per stage
    uint32_t abig = 128u * 16u * (uint32_t)(a.G * cin / 8), bbig = 128u * 16u * (uint32_t)(cout / 8);
    uint32_t aroom = (uint32_t)a.G * a.tapbytes;
    a.stride = r1024((aroom > abig ? aroom : abig) + (a.bbytes > bbig ? a.bbytes : bbig));
    uint32_t smem = WG_STAGES * a.stride + 1024u;
    CUtensorMap mx, md;
    if (make_map(&mx, x, X, Y, Z, cin, a.bx, a.by, a.bz, cin / 8)) return 1;
    if (make_map(&md, dy, X, Y, Z, cout, a.bx, a.by, a.bz, cout / 8)) return 1;
    static int lim = dyn_smem_limit((const void *)k_wgrad);
    if ((int)smem > lim) { snprintf(g_conv_err, sizeof(g_conv_err), "wgrad needs %u B of shared memory", smem); return 1; }
    int want = 2 * nsm / a.ngroups;
    a.nsplit = want < 1 ? 1 : want;
    if (a.nsplit > a.ntiles) a.nsplit = a.ntiles;
    a.dw = dw; a.err = err;
    k_wgrad<<<a.ngroups * a.nsplit, 192, smem, s>>>(mx, md, a);
    return launch_error("k_wgrad");
}

int conv_selftest_umma(int mn_major, int swap, unsigned long long *mismatches)
{
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return 1;
    cudaMemset(d, 0, sizeof(*d));
    cudaFuncSetAttribute(k_umma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, ST_SMEM);
    k_umma_selftest<<<1, 128, ST_SMEM>>>(mn_major, swap, d);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, d, sizeof(*d), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) { snprintf(g_conv_err, sizeof(g_conv_err), "%s", cudaGetErrorString(e)); return 1; }
    return 0;
}
