// k_net.cu -- the learned initial guess of the pressure solve: a 4-level 3-D
// U-Net (channels 16-32-64-128, 3x3x3 kernels, BF16 weights and activations,
// FP32 accumulation) whose convolutions, data and weight gradients run on the
// tcgen05 tensor cores (k_conv.cu); pooling, upsampling, gradient masks, the
// loss and Adam are the SIMT kernels below.
//
//   a0 = relu(conv_in(x0))                      level 0, 16 ch (3 used inputs)
//   a1 = relu(conv1(pool a0))  a2 = relu(conv2(pool a1))  a3 = relu(conv3(pool a2))
//   b3 = relu(conv3b(a3))
//   s2 = relu(up(conv_up2 b3) + a2)   b2 = relu(conv2b(s2))
//   s1 = relu(up(conv_up1 b2) + a1)   b1 = relu(conv1b(s1))
//   s0 = relu(up(conv_up0 b1) + a0)   b0 = relu(conv0b(s0))
//   out = head . b0 + hb                        (1x1x1, FP32)
// pool = 2x2x2 average, up = nearest (each coarse cell to its 8 children).
//
// Inputs (per cell of the compact pressure layout): the divergence residual
// that the previous pressure leaves, r1 = W b - S p1, scaled by its rms s;
// the last pressure increment p1 - p2 and the divergence W b, each scaled by
// its own rms.  Output: the correction
// delta = s * diag(S)^-1 * out added to the previous pressure.  Training
// minimises |r1 - S delta|^2 / |r1|^2, the squared relative initial residual
// of the corrected guess, i.e. exactly what the solver's guard compares.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/turbins_gb300.h"
#include "turb_conv.cuh"
#include "turb_net.cuh"

namespace {

constexpr int NL = 11;
struct LayerDef {
    int cin, cout, lev;
};
constexpr LayerDef DEFS[NL] = {{16, 16, 0}, {16, 32, 1},  {32, 64, 2},  {64, 128, 3}, {128, 128, 3}, {128, 64, 3},
                               {64, 64, 2}, {64, 32, 2},  {32, 32, 1},  {32, 16, 1},  {16, 16, 0}};

__device__ __forceinline__ void ld8(const bf16 *p, float (&v)[8])
{
    uint4 u = *reinterpret_cast<const uint4 *>(p);
    const bf16 *b = reinterpret_cast<const bf16 *>(&u);
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = __bfloat162float(b[j]);
}
__device__ __forceinline__ void st8(bf16 *p, const float (&v)[8])
{
    uint4 u;
    bf16 *b = reinterpret_cast<bf16 *>(&u);
#pragma unroll
    for (int j = 0; j < 8; j++) b[j] = __float2bfloat16_rn(v[j]);
    *reinterpret_cast<uint4 *>(p) = u;
}

struct G3 {
    int X, Y, Z;
    __device__ __forceinline__ long long n() const { return (long long)X * Y * Z; }
};

#define GRID_STRIDE(i, n) \
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

// x0 channel block 0 = (in3[0], in3[1], in3[2], 0, ..., 0); block 1 stays zero
__global__ void k_pack_input(long long n, const float *__restrict__ in3, bf16 *__restrict__ x0)
{
    GRID_STRIDE(v, n)
    {
        float a[8] = {in3[v], in3[n + v], in3[2 * n + v], 0.f, 0.f, 0.f, 0.f, 0.f};
        st8(x0 + v * 8, a);
    }
}

// 2x2x2 average; g = coarse grid, C/8 channel blocks
__global__ void k_pool(G3 g, int ncb, const bf16 *__restrict__ in, bf16 *__restrict__ out)
{
    long long nc = g.n(), nf = nc * 8;
    GRID_STRIDE(idx, nc * ncb)
    {
        long long cb = idx / nc, v = idx % nc;
        int x = (int)(v % g.X), y = (int)((v / g.X) % g.Y), z = (int)(v / ((long long)g.X * g.Y));
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int c = 0; c < 8; c++) {
            long long f = ((long long)(2 * z + (c >> 2)) * (2 * g.Y) + (2 * y + ((c >> 1) & 1))) * (2 * g.X) + 2 * x + (c & 1);
            float t[8];
            ld8(in + (cb * nf + f) * 8, t);
#pragma unroll
            for (int j = 0; j < 8; j++) acc[j] += t[j];
        }
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j] *= 0.125f;
        st8(out + idx * 8, acc);
    }
}

__device__ __forceinline__ long long parent(long long v, const G3 &f)
{
    int x = (int)(v % f.X), y = (int)((v / f.X) % f.Y), z = (int)(v / ((long long)f.X * f.Y));
    return ((long long)(z >> 1) * (f.Y >> 1) + (y >> 1)) * (f.X >> 1) + (x >> 1);
}

// s = relu(up(c) + a) on the fine grid f
__global__ void k_up_add_relu(G3 f, int ncb, const bf16 *__restrict__ c, const bf16 *__restrict__ a,
                              bf16 *__restrict__ s)
{
    long long nf = f.n(), nc = nf / 8;
    GRID_STRIDE(idx, nf * ncb)
    {
        long long cb = idx / nf, v = idx % nf;
        float x[8], y[8];
        ld8(c + (cb * nc + parent(v, f)) * 8, x);
        ld8(a + idx * 8, y);
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = fmaxf(x[j] + y[j], 0.f);
        st8(s + idx * 8, x);
    }
}

// adjoint of the nearest upsampling: sum over the 8 children; g = coarse grid
__global__ void k_down_sum(G3 g, int ncb, const bf16 *__restrict__ d, bf16 *__restrict__ out)
{
    long long nc = g.n(), nf = nc * 8;
    GRID_STRIDE(idx, nc * ncb)
    {
        long long cb = idx / nc, v = idx % nc;
        int x = (int)(v % g.X), y = (int)((v / g.X) % g.Y), z = (int)(v / ((long long)g.X * g.Y));
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int c = 0; c < 8; c++) {
            long long f = ((long long)(2 * z + (c >> 2)) * (2 * g.Y) + (2 * y + ((c >> 1) & 1))) * (2 * g.X) + 2 * x + (c & 1);
            float t[8];
            ld8(d + (cb * nf + f) * 8, t);
#pragma unroll
            for (int j = 0; j < 8; j++) acc[j] += t[j];
        }
        st8(out + idx * 8, acc);
    }
}

// dz = (dzs + up(dp) / 8) * (a > 0) on the fine grid f
__global__ void k_combine(G3 f, int ncb, const bf16 *__restrict__ dzs, const bf16 *__restrict__ dp,
                          const bf16 *__restrict__ a, bf16 *__restrict__ dz)
{
    long long nf = f.n(), nc = nf / 8;
    GRID_STRIDE(idx, nf * ncb)
    {
        long long cb = idx / nf, v = idx % nf;
        float s[8], p[8], m[8];
        ld8(dzs + idx * 8, s);
        ld8(dp + (cb * nc + parent(v, f)) * 8, p);
        ld8(a + idx * 8, m);
#pragma unroll
        for (int j = 0; j < 8; j++) s[j] = m[j] > 0.f ? s[j] + 0.125f * p[j] : 0.f;
        st8(dz + idx * 8, s);
    }
}

__device__ __forceinline__ float wsum(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// per-channel sums over voxels (bias gradients): grid (blocks, ncb)
__global__ void k_chan_sum(long long n, const bf16 *__restrict__ d, float *__restrict__ g)
{
    int cb = blockIdx.y;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        float t[8];
        ld8(d + ((long long)cb * n + v) * 8, t);
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j] += t[j];
    }
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float s = wsum(acc[j]);
        if ((threadIdx.x & 31) == 0) atomicAdd(g + cb * 8 + j, s);
    }
}

// head backward: dz0b = hw * g * (b0 > 0); dhw += b0 * g; dhb += g
__global__ void k_head_bwd(long long n, const float *__restrict__ gout, const bf16 *__restrict__ b0,
                           const float *__restrict__ hw, bf16 *__restrict__ dz, float *__restrict__ ghw,
                           float *__restrict__ ghb)
{
    float acc[17];
#pragma unroll
    for (int j = 0; j < 17; j++) acc[j] = 0.f;
    GRID_STRIDE(v, n)
    {
        float g = gout[v];
        acc[16] += g;
#pragma unroll
        for (int cb = 0; cb < 2; cb++) {
            float b[8], o[8];
            ld8(b0 + ((long long)cb * n + v) * 8, b);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                acc[cb * 8 + j] += b[j] * g;
                o[j] = b[j] > 0.f ? hw[cb * 8 + j] * g : 0.f;
            }
            st8(dz + ((long long)cb * n + v) * 8, o);
        }
    }
#pragma unroll
    for (int j = 0; j < 17; j++) {
        float s = wsum(acc[j]);
        if ((threadIdx.x & 31) == 0) atomicAdd(j < 16 ? ghw + j : ghb, s);
    }
}

__global__ void k_adam(long long n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2)
{
    GRID_STRIDE(i, n)
    {
        float gi = g[i];
        float mi = b1 * m[i] + (1.f - b1) * gi;
        float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// partial sums of r1^2, b^2 and (p1 - p2)^2: part[k * NSUM + block]
constexpr int NSUM = 512;
__global__ void k_sumsq3(long long n, const double *__restrict__ r1, const double *__restrict__ bw,
                         const double *__restrict__ p1, const double *__restrict__ p2, double *__restrict__ part)
{
    double a = 0.0, b = 0.0, c = 0.0;
    GRID_STRIDE(v, n)
    {
        double d = p1[v] - p2[v];
        a = fma(r1[v], r1[v], a);
        b = fma(bw[v], bw[v], b);
        c = fma(d, d, c);
    }
    __shared__ double sm[3][8];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { sm[0][w] = a; sm[1][w] = b; sm[2][w] = c; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += sm[threadIdx.x][i];
        part[threadIdx.x * NSUM + blockIdx.x] = t;
    }
}

// network inputs from the solver state (compact layout), each channel scaled
// by its rms: sc[0] = |r1|^2, sc[1] = |b|^2, sc[2] = |p1 - p2|^2
__global__ void k_prep(long long n, const double *__restrict__ r1, const double *__restrict__ bw,
                       const double *__restrict__ p1, const double *__restrict__ p2, const double *__restrict__ sc,
                       float *__restrict__ in3)
{
    double rs = sqrt(sc[0] / (double)n), bs = sqrt(sc[1] / (double)n), ds = sqrt(sc[2] / (double)n);
    double ir = rs > 0.0 ? 1.0 / rs : 0.0, ib = bs > 0.0 ? 1.0 / bs : 0.0, id = ds > 0.0 ? 1.0 / ds : 0.0;
    GRID_STRIDE(v, n)
    {
        in3[v] = (float)(r1[v] * ir);
        in3[n + v] = (float)((p1[v] - p2[v]) * id);
        in3[2 * n + v] = (float)(bw[v] * ib);
    }
}

// snapshot target: out* = (p - base) / (invd * s), s = |r1|_rms
__global__ void k_target(long long n, const double *__restrict__ p, const double *__restrict__ base,
                         const double *__restrict__ invd, const double *__restrict__ sc, float *__restrict__ t)
{
    double rs = sqrt(sc[0] / (double)n), ir = rs > 0.0 ? 1.0 / rs : 0.0;
    GRID_STRIDE(v, n) t[v] = (float)((p[v] - base[v]) / invd[v] * ir);
}

// energy-norm loss: x = invd * (t - h); the S-products come from k_apply
__global__ void k_energy_in(long long n, const float *__restrict__ h, const float *__restrict__ t,
                            const double *__restrict__ invd, double *__restrict__ x)
{
    GRID_STRIDE(v, n) x[v] = invd[v] * ((double)t[v] - (double)h[v]);
}
// gout += -2 w / e0 * invd * q
__global__ void k_grad_add(long long n, double w, const double *__restrict__ e0, const double *__restrict__ q,
                           const double *__restrict__ invd, float *__restrict__ gout)
{
    double f = *e0 > 0.0 ? -2.0 * w / *e0 : 0.0;
    GRID_STRIDE(v, n) gout[v] += (float)(f * invd[v] * q[v]);
}
__global__ void k_t64(long long n, const float *__restrict__ t, const double *__restrict__ invd, double *__restrict__ x)
{
    GRID_STRIDE(v, n) x[v] = invd[v] * (double)t[v];
}

// out = base + s * invd * h
__global__ void k_post(long long n, const double *__restrict__ base, const double *__restrict__ invd,
                       const float *__restrict__ h, const double *__restrict__ sc, double *__restrict__ out)
{
    double rs = sqrt(sc[0] / (double)n);
    GRID_STRIDE(v, n) out[v] = base[v] + rs * invd[v] * (double)h[v];
}

// training loss: x = h * invd, r1n = in3[0] (FP64)
__global__ void k_loss_in(long long n, const float *__restrict__ h, const double *__restrict__ invd,
                          const float *__restrict__ in3, double *__restrict__ x, double *__restrict__ r)
{
    GRID_STRIDE(v, n)
    {
        x[v] = (double)h[v] * invd[v];
        r[v] = (double)in3[v];
    }
}
__global__ void k_scale_f(long long n, float f, float *__restrict__ a)
{
    GRID_STRIDE(v, n) a[v] *= f;
}
__global__ void k_loss_grad(long long n, const double *__restrict__ q, const double *__restrict__ invd,
                            float *__restrict__ gout)
{
    double f = -2.0 / (double)n;
    GRID_STRIDE(v, n) gout[v] = (float)(f * invd[v] * q[v]);
}

inline int nblk(long long n, int bs = 256)
{
    long long b = (n + bs - 1) / bs;
    return (int)(b < 4096 ? (b < 1 ? 1 : b) : 4096);
}

// splitmix64 + Box-Muller for the initial weights
struct Rng {
    unsigned long long s;
    unsigned long long next()
    {
        unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() { return std::sqrt(-2.0 * std::log(uni())) * std::cos(6.283185307179586 * uni()); }
};

}  // namespace

struct TurbNet {
    int nx, ny, nz, train, nsm;
    int X[4], Y[4], Z[4];
    long long V[4];
    long long nparam = 0, woff[NL], boff[NL], hw_off, hb_off;
    bf16 *wf[NL], *wd[NL];
    float *P = nullptr, *G = nullptr, *M = nullptr, *Vv = nullptr;
    long long adam_t = 0;
    double wr = 1.0, we = 0.0;   // training loss weights: residual form, energy form
    bf16 *x0, *a0, *p0, *a1, *p1, *a2, *p2, *a3, *b3, *c2, *s2, *b2, *c1, *s1, *b1, *c0, *s0, *b0;
    bf16 *dz0b, *dzs0, *dc0, *dz1b, *dzs1, *dc1, *dz2b, *dzs2, *dc2, *dz3b, *dz3, *dp2, *dz2, *dp1, *dz1, *dp0, *dz0;
    float *in3 = nullptr, *hout = nullptr, *gout = nullptr;
    double *x64 = nullptr, *r64 = nullptr, *rr = nullptr, *q64 = nullptr, *part = nullptr, *sc = nullptr;
    long long nparts = 0;
    int *err = nullptr;
    std::vector<void *> allocs;
    cudaError_t aerr = cudaSuccess;
    template <typename T>
    T *alloc(long long n)
    {
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, (size_t)(n > 0 ? n : 1) * sizeof(T));
        if (e != cudaSuccess) { aerr = e; return nullptr; }
        cudaMemset(p, 0, (size_t)(n > 0 ? n : 1) * sizeof(T));
        allocs.push_back(p);
        return (T *)p;
    }
    ~TurbNet()
    {
        for (void *p : allocs) cudaFree(p);
    }
};

// snapshot k: data[k][c][cell], channels 0-2 the network inputs, channel 3
// the target out* = (p_converged - p_previous) diag(S) / s of that solve
constexpr int SNAP_CH = 4;
struct TurbSnaps {
    int nx, ny, nz, cap, n = 0;
    int pending = -1;              // snapshot waiting for its solve's converged pressure
    long long V;
    float *data = nullptr;
    double *sc = nullptr, *part = nullptr, *base = nullptr, *x64 = nullptr, *q64 = nullptr;
    double *e0 = nullptr;          // per snapshot: energy norm of its target, t^T invd S invd t
    long long nparts = 0;
};

namespace {

bf16 *act(TurbNet *n, int lev, int c) { return n->alloc<bf16>(n->V[lev] * c); }

int conv(TurbNet *n, cudaStream_t s, int l, const bf16 *in, const ConvEpi &e)
{
    const LayerDef &d = DEFS[l];
    int lv = d.lev;
    int rc = conv3_fwd(s, in, n->X[lv], n->Y[lv], n->Z[lv], d.cin, d.cout, n->wf[l], e, n->err, n->nsm);
    return rc ? turb_set_error_text(conv_last_error()) : TURB_OK;
}
// data gradient of layer l: dy (cout ch) -> dx (cin ch), masked by `mask`
int dgrad(TurbNet *n, cudaStream_t s, int l, const bf16 *dy, const bf16 *mask, bf16 *dx)
{
    const LayerDef &d = DEFS[l];
    int lv = d.lev;
    ConvEpi e;
    e.mask = mask;
    e.out = dx;
    int rc = conv3_fwd(s, dy, n->X[lv], n->Y[lv], n->Z[lv], d.cout, d.cin, n->wd[l], e, n->err, n->nsm);
    return rc ? turb_set_error_text(conv_last_error()) : TURB_OK;
}
int wgrad(TurbNet *n, cudaStream_t s, int l, const bf16 *x, const bf16 *dy)
{
    const LayerDef &d = DEFS[l];
    int lv = d.lev;
    int rc = conv3_wgrad(s, x, dy, n->X[lv], n->Y[lv], n->Z[lv], d.cin, d.cout, n->G + n->woff[l], n->err, n->nsm);
    if (rc) return turb_set_error_text(conv_last_error());
    k_chan_sum<<<dim3(nblk(n->V[lv]) < 256 ? nblk(n->V[lv]) : 256, d.cout / 8), 256, 0, s>>>(n->V[lv], dy,
                                                                                              n->G + n->boff[l]);
    return TURB_OK;
}
G3 g3(const TurbNet *n, int l) { return G3{n->X[l], n->Y[l], n->Z[l]}; }

void pack_all(TurbNet *n, cudaStream_t s)
{
    for (int l = 0; l < NL; l++) {
        const LayerDef &d = DEFS[l];
        int lv = d.lev;
        ConvPlan pf = conv_plan(n->X[lv], n->Y[lv], n->Z[lv], d.cin, d.cout);
        ConvPlan pb = conv_plan(n->X[lv], n->Y[lv], n->Z[lv], d.cout, d.cin);
        conv_pack_weights(s, n->P + n->woff[l], d.cin, d.cout, pf, pb, n->wf[l], n->wd[l]);
    }
}

#define NCHK(x)                          \
    do {                                 \
        int rc_ = (x);                   \
        if (rc_ != TURB_OK) return rc_;  \
    } while (0)

int forward(TurbNet *n, cudaStream_t s, const float *in3, float *hout)
{
    k_pack_input<<<nblk(n->V[0]), 256, 0, s>>>(n->V[0], in3, n->x0);
    const float *P = n->P;
    ConvEpi e;
    e.relu = 1;
    e.bias = P + n->boff[0]; e.out = n->a0;
    NCHK(conv(n, s, 0, n->x0, e));
    k_pool<<<nblk(n->V[1] * 2), 256, 0, s>>>(g3(n, 1), 2, n->a0, n->p0);
    e.bias = P + n->boff[1]; e.out = n->a1;
    NCHK(conv(n, s, 1, n->p0, e));
    k_pool<<<nblk(n->V[2] * 4), 256, 0, s>>>(g3(n, 2), 4, n->a1, n->p1);
    e.bias = P + n->boff[2]; e.out = n->a2;
    NCHK(conv(n, s, 2, n->p1, e));
    k_pool<<<nblk(n->V[3] * 8), 256, 0, s>>>(g3(n, 3), 8, n->a2, n->p2);
    e.bias = P + n->boff[3]; e.out = n->a3;
    NCHK(conv(n, s, 3, n->p2, e));
    e.bias = P + n->boff[4]; e.out = n->b3;
    NCHK(conv(n, s, 4, n->a3, e));
    ConvEpi u;
    u.bias = P + n->boff[5]; u.out = n->c2;
    NCHK(conv(n, s, 5, n->b3, u));
    k_up_add_relu<<<nblk(n->V[2] * 8), 256, 0, s>>>(g3(n, 2), 8, n->c2, n->a2, n->s2);
    e.bias = P + n->boff[6]; e.out = n->b2;
    NCHK(conv(n, s, 6, n->s2, e));
    u.bias = P + n->boff[7]; u.out = n->c1;
    NCHK(conv(n, s, 7, n->b2, u));
    k_up_add_relu<<<nblk(n->V[1] * 4), 256, 0, s>>>(g3(n, 1), 4, n->c1, n->a1, n->s1);
    e.bias = P + n->boff[8]; e.out = n->b1;
    NCHK(conv(n, s, 8, n->s1, e));
    u.bias = P + n->boff[9]; u.out = n->c0;
    NCHK(conv(n, s, 9, n->b1, u));
    k_up_add_relu<<<nblk(n->V[0] * 2), 256, 0, s>>>(g3(n, 0), 2, n->c0, n->a0, n->s0);
    ConvEpi h;
    h.relu = 1;
    h.bias = P + n->boff[10];
    h.out = n->train ? n->b0 : nullptr;
    h.headw = P + n->hw_off;
    h.headb = P + n->hb_off;
    h.hout = hout;
    NCHK(conv(n, s, 10, n->s0, h));
    return cudaGetLastError() == cudaSuccess ? TURB_OK : TURB_ERR_CUDA;
}

int backward(TurbNet *n, cudaStream_t s, const float *gout)
{
    cudaMemsetAsync(n->G, 0, (size_t)n->nparam * sizeof(float), s);
    k_head_bwd<<<nblk(n->V[0]) < 1024 ? nblk(n->V[0]) : 1024, 256, 0, s>>>(n->V[0], gout, n->b0, n->P + n->hw_off,
                                                                           n->dz0b, n->G + n->hw_off, n->G + n->hb_off);
    NCHK(wgrad(n, s, 10, n->s0, n->dz0b));
    NCHK(dgrad(n, s, 10, n->dz0b, n->s0, n->dzs0));
    k_down_sum<<<nblk(n->V[1] * 2), 256, 0, s>>>(g3(n, 1), 2, n->dzs0, n->dc0);
    NCHK(wgrad(n, s, 9, n->b1, n->dc0));
    NCHK(dgrad(n, s, 9, n->dc0, n->b1, n->dz1b));
    NCHK(wgrad(n, s, 8, n->s1, n->dz1b));
    NCHK(dgrad(n, s, 8, n->dz1b, n->s1, n->dzs1));
    k_down_sum<<<nblk(n->V[2] * 4), 256, 0, s>>>(g3(n, 2), 4, n->dzs1, n->dc1);
    NCHK(wgrad(n, s, 7, n->b2, n->dc1));
    NCHK(dgrad(n, s, 7, n->dc1, n->b2, n->dz2b));
    NCHK(wgrad(n, s, 6, n->s2, n->dz2b));
    NCHK(dgrad(n, s, 6, n->dz2b, n->s2, n->dzs2));
    k_down_sum<<<nblk(n->V[3] * 8), 256, 0, s>>>(g3(n, 3), 8, n->dzs2, n->dc2);
    NCHK(wgrad(n, s, 5, n->b3, n->dc2));
    NCHK(dgrad(n, s, 5, n->dc2, n->b3, n->dz3b));
    NCHK(wgrad(n, s, 4, n->a3, n->dz3b));
    NCHK(dgrad(n, s, 4, n->dz3b, n->a3, n->dz3));
    NCHK(wgrad(n, s, 3, n->p2, n->dz3));
    NCHK(dgrad(n, s, 3, n->dz3, nullptr, n->dp2));
    k_combine<<<nblk(n->V[2] * 8), 256, 0, s>>>(g3(n, 2), 8, n->dzs2, n->dp2, n->a2, n->dz2);
    NCHK(wgrad(n, s, 2, n->p1, n->dz2));
    NCHK(dgrad(n, s, 2, n->dz2, nullptr, n->dp1));
    k_combine<<<nblk(n->V[1] * 4), 256, 0, s>>>(g3(n, 1), 4, n->dzs1, n->dp1, n->a1, n->dz1);
    NCHK(wgrad(n, s, 1, n->p0, n->dz1));
    NCHK(dgrad(n, s, 1, n->dz1, nullptr, n->dp0));
    k_combine<<<nblk(n->V[0] * 2), 256, 0, s>>>(g3(n, 0), 2, n->dzs0, n->dp0, n->a0, n->dz0);
    NCHK(wgrad(n, s, 0, n->x0, n->dz0));
    return cudaGetLastError() == cudaSuccess ? TURB_OK : TURB_ERR_CUDA;
}

void adam(TurbNet *n, cudaStream_t s, float lr)
{
    n->adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.f - std::pow(b1, (float)n->adam_t), c2 = 1.f - std::pow(b2, (float)n->adam_t);
    k_adam<<<nblk(n->nparam), 256, 0, s>>>(n->nparam, n->P, n->G, n->M, n->Vv, lr, b1, b2, 1e-8f, c1, c2);
    pack_all(n, s);
}

int read_err(TurbNet *n, cudaStream_t s)
{
    int h = 0;
    if (cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return TURB_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return TURB_ERR_CUDA;
    if (h) {
        cudaMemsetAsync(n->err, 0, sizeof(int), s);
        return turb_set_error_text(h == 2 ? "weight-gradient kernel: barrier wait timed out"
                                          : "convolution kernel: barrier wait timed out");
    }
    return TURB_OK;
}

int ensure_parts(double **part, long long *have, const MgDevLevel &L0)
{
    long long need = pcg_stencil_parts(L0);
    if (need < 2LL * pcg_nparts()) need = 2LL * pcg_nparts();
    if (need < 3LL * NSUM) need = 3LL * NSUM;
    if (*have >= need) return TURB_OK;
    if (*part) cudaFree(*part);
    *part = nullptr;
    if (cudaMalloc(part, (size_t)need * sizeof(double)) != cudaSuccess) { *have = 0; return TURB_ERR_ALLOC; }
    *have = need;
    return TURB_OK;
}

// |r1|^2, |b|^2 and |p1 - p2|^2 into sc[0..2]
void input_norms(cudaStream_t s, long long n, const double *r1, const double *bw, const double *p1, const double *p2,
                 double *part, double *sc)
{
    k_sumsq3<<<NSUM, 256, 0, s>>>(n, r1, bw, p1, p2, part);
    for (int k = 0; k < 3; k++) pcg_reduce(s, part + k * NSUM, 1, sc + k, NSUM);
}

// losses of the current forward output against snapshot `snap` (inputs and
// target): sc[2] = |r1n - S invd h|^2 (residual form), sc[3] = e^T S e with
// e = invd (t - h) (energy form, CG's own error norm); both are divided by
// the cell count on the host.  gout = d(wr * L_R + we * L_E) / dh.
int loss(TurbNet *n, cudaStream_t s, const MgDevLevel &L0, const double *invd, const float *snap, const double *e0,
         int want_grad)
{
    long long V = n->V[0];
    int np = pcg_stencil_parts(L0);
    k_loss_in<<<nblk(V), 256, 0, s>>>(V, n->hout, invd, snap, n->x64, n->r64);
    pcg_resid(s, L0, n->r64, n->x64, n->rr, n->part);
    pcg_reduce(s, n->part, 1, n->sc + 2, np);
    if (want_grad) {
        pcg_apply(s, L0, n->rr, n->q64, n->part);
        k_loss_grad<<<nblk(V), 256, 0, s>>>(V, n->q64, invd, n->gout);
        if (n->wr != 1.0) k_scale_f<<<nblk(V), 256, 0, s>>>(V, (float)n->wr, n->gout);
    }
    k_energy_in<<<nblk(V), 256, 0, s>>>(V, n->hout, snap + 3 * V, invd, n->x64);
    pcg_apply(s, L0, n->x64, n->q64, n->part);
    pcg_reduce(s, n->part, 1, n->sc + 3, np);
    if (want_grad && n->we != 0.0) k_grad_add<<<nblk(V), 256, 0, s>>>(V, n->we, e0, n->q64, invd, n->gout);
    return cudaGetLastError() == cudaSuccess ? TURB_OK : TURB_ERR_CUDA;
}

bool same_grid(const TurbNet *n, const MgDevLevel &L0)
{
    return L0.nx == n->nx && L0.ny == n->ny && L0.nz == n->nz;
}

}  // namespace

int net_dims(const TurbNet *n, int *nx, int *ny, int *nz)
{
    *nx = n->nx; *ny = n->ny; *nz = n->nz;
    return TURB_OK;
}
int snaps_dims(const TurbSnaps *s, int *nx, int *ny, int *nz)
{
    *nx = s->nx; *ny = s->ny; *nz = s->nz;
    return TURB_OK;
}

int net_guess(TurbNet *n, cudaStream_t st, const MgDevLevel &L0, const double *invd, const double *r1,
              const double *bw, const double *p1, const double *p2, const double *base, double *out)
{
    if (!n || !same_grid(n, L0)) return TURB_ERR_ARG;
    if (ensure_parts(&n->part, &n->nparts, L0)) return TURB_ERR_ALLOC;
    long long V = n->V[0];
    input_norms(st, V, r1, bw, p1, p2, n->part, n->sc);
    k_prep<<<nblk(V), 256, 0, st>>>(V, r1, bw, p1, p2, n->sc, n->in3);
    NCHK(forward(n, st, n->in3, n->hout));
    k_post<<<nblk(V), 256, 0, st>>>(V, base, invd, n->hout, n->sc, out);
    if (cudaGetLastError() != cudaSuccess) return TURB_ERR_CUDA;
    return read_err(n, st);
}

int net_snapshot(TurbSnaps *sn, cudaStream_t st, const MgDevLevel &L0, const double *invd, const double *r1,
                 const double *bw, const double *p1, const double *p2, const double *base)
{
    if (!sn || L0.nx != sn->nx || L0.ny != sn->ny || L0.nz != sn->nz) return TURB_ERR_ARG;
    if (sn->n >= sn->cap) return TURB_OK;   // store full: later solves are not recorded
    if (ensure_parts(&sn->part, &sn->nparts, L0)) return TURB_ERR_ALLOC;
    long long V = sn->V;
    input_norms(st, V, r1, bw, p1, p2, sn->part, sn->sc);
    k_prep<<<nblk(V), 256, 0, st>>>(V, r1, bw, p1, p2, sn->sc, sn->data + (long long)sn->n * SNAP_CH * V);
    cudaMemcpyAsync(sn->base, base, (size_t)V * sizeof(double), cudaMemcpyDeviceToDevice, st);
    sn->pending = sn->n;
    sn->n++;
    return cudaGetLastError() == cudaSuccess ? TURB_OK : TURB_ERR_CUDA;
}

int net_snapshot_finish(TurbSnaps *sn, cudaStream_t st, const MgDevLevel &L0, const double *invd, const double *p,
                        int converged)
{
    if (!sn || sn->pending < 0) return TURB_OK;
    int k = sn->pending;
    sn->pending = -1;
    if (!converged) {   // keep only snapshots whose solve reached the tolerance
        if (k == sn->n - 1) sn->n--;
        return TURB_OK;
    }
    long long V = sn->V;
    if (!sn->x64 && (cudaMalloc(&sn->x64, (size_t)V * 8) != cudaSuccess || cudaMalloc(&sn->q64, (size_t)V * 8) != cudaSuccess))
        return TURB_ERR_ALLOC;
    float *t = sn->data + (long long)k * SNAP_CH * V + 3 * V;
    k_target<<<nblk(V), 256, 0, st>>>(V, p, sn->base, invd, sn->sc, t);
    k_t64<<<nblk(V), 256, 0, st>>>(V, t, invd, sn->x64);
    pcg_apply(st, L0, sn->x64, sn->q64, sn->part);
    pcg_reduce(st, sn->part, 1, sn->e0 + k, pcg_stencil_parts(L0));
    return cudaGetLastError() == cudaSuccess ? TURB_OK : TURB_ERR_CUDA;
}

int net_train(TurbNet *n, cudaStream_t st, const MgDevLevel &L0, const double *invd, TurbSnaps *sn, int steps,
              float lr, unsigned long long seed, double *mean_loss)
{
    if (!n || !sn || !n->train || !same_grid(n, L0) || sn->n < 1 || steps < 1) return TURB_ERR_ARG;
    if (ensure_parts(&n->part, &n->nparts, L0)) return TURB_ERR_ALLOC;
    Rng rng{seed};
    double *hbuf = nullptr;
    if (cudaMallocHost(&hbuf, (size_t)steps * 3 * sizeof(double)) != cudaSuccess) return TURB_ERR_ALLOC;
    long long V = n->V[0];
    int rc = TURB_OK;
    for (int k = 0; k < steps && rc == TURB_OK; k++) {
        int idx = (int)(rng.next() % (unsigned long long)sn->n);
        const float *snap = sn->data + (long long)idx * SNAP_CH * V;
        rc = forward(n, st, snap, n->hout);
        if (rc == TURB_OK) rc = loss(n, st, L0, invd, snap, sn->e0 + idx, 1);
        if (rc == TURB_OK) rc = backward(n, st, n->gout);
        if (rc == TURB_OK) adam(n, st, lr);
        if (rc == TURB_OK && (cudaMemcpyAsync(hbuf + 3 * k, n->sc + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) !=
                                  cudaSuccess ||
                              cudaMemcpyAsync(hbuf + 3 * k + 2, sn->e0 + idx, sizeof(double), cudaMemcpyDeviceToHost,
                                              st) != cudaSuccess))
            rc = TURB_ERR_CUDA;
    }
    if (rc == TURB_OK) rc = read_err(n, st);
    if (rc == TURB_OK && mean_loss) {
        double acc = 0.0;
        for (int k = 0; k < steps; k++) {
            double lr_ = hbuf[3 * k] / (double)V, le = hbuf[3 * k + 2] > 0.0 ? hbuf[3 * k + 1] / hbuf[3 * k + 2] : 0.0;
            acc += n->wr * lr_ + n->we * le;
        }
        *mean_loss = acc / steps;
    }
    cudaFreeHost(hbuf);
    return rc;
}

int net_eval(TurbNet *n, cudaStream_t st, const MgDevLevel &L0, const double *invd, TurbSnaps *sn, int first,
             int count, double *mean_res, double *mean_energy)
{
    if (!n || !sn || !same_grid(n, L0) || first < 0 || count < 1 || first + count > sn->n) return TURB_ERR_ARG;
    if (ensure_parts(&n->part, &n->nparts, L0)) return TURB_ERR_ALLOC;
    if (!n->x64) {   // inference nets get the loss buffers on first use
        n->x64 = n->alloc<double>(n->V[0]); n->r64 = n->alloc<double>(n->V[0]);
        n->rr = n->alloc<double>(n->V[0]); n->q64 = n->alloc<double>(n->V[0]);
        if (n->aerr != cudaSuccess) return TURB_ERR_ALLOC;
    }
    double *hbuf = nullptr;
    if (cudaMallocHost(&hbuf, (size_t)count * 3 * sizeof(double)) != cudaSuccess) return TURB_ERR_ALLOC;
    long long V = n->V[0];
    int rc = TURB_OK;
    for (int k = 0; k < count && rc == TURB_OK; k++) {
        int idx = first + k;
        const float *snap = sn->data + (long long)idx * SNAP_CH * V;
        rc = forward(n, st, snap, n->hout);
        if (rc == TURB_OK) rc = loss(n, st, L0, invd, snap, sn->e0 + idx, 0);
        if (rc == TURB_OK && (cudaMemcpyAsync(hbuf + 3 * k, n->sc + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) !=
                                  cudaSuccess ||
                              cudaMemcpyAsync(hbuf + 3 * k + 2, sn->e0 + idx, sizeof(double), cudaMemcpyDeviceToHost,
                                              st) != cudaSuccess))
            rc = TURB_ERR_CUDA;
    }
    if (rc == TURB_OK) rc = read_err(n, st);
    if (rc == TURB_OK) {
        double ar = 0.0, ae = 0.0;
        for (int k = 0; k < count; k++) {
            ar += hbuf[3 * k] / (double)V;
            ae += hbuf[3 * k + 2] > 0.0 ? hbuf[3 * k + 1] / hbuf[3 * k + 2] : 0.0;
        }
        if (mean_res) *mean_res = ar / count;
        if (mean_energy) *mean_energy = ae / count;
    }
    cudaFreeHost(hbuf);
    return rc;
}

// ---- C ABI ------------------------------------------------------------------------------
extern "C" {

int turb_net_create(int nx, int ny, int nz, int train, turb_net **out)
{
    if (!out) return TURB_ERR_ARG;
    *out = nullptr;
    if (nx < 16 || ny < 16 || nz < 16 || nx % 8 || ny % 8 || nz % 8) return TURB_ERR_ARG;
    if ((long long)(nx / 8) * (ny / 8) * (nz / 8) < 16) return TURB_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TURB_ERR_CUDA;
    TurbNet *n = new TurbNet();
    n->nx = nx; n->ny = ny; n->nz = nz; n->train = train ? 1 : 0;
    cudaDeviceGetAttribute(&n->nsm, cudaDevAttrMultiProcessorCount, dev);
    for (int l = 0; l < 4; l++) {
        n->X[l] = nx >> l; n->Y[l] = ny >> l; n->Z[l] = nz >> l;
        n->V[l] = (long long)n->X[l] * n->Y[l] * n->Z[l];
    }
    long long off = 0;
    for (int l = 0; l < NL; l++) {
        const LayerDef &d = DEFS[l];
        n->woff[l] = off; off += 27LL * d.cin * d.cout;
        n->boff[l] = off; off += d.cout;
        int lv = d.lev;
        n->wf[l] = n->alloc<bf16>(conv_pack_elems(d.cin, d.cout));
        n->wd[l] = n->alloc<bf16>(conv_pack_elems(d.cout, d.cin));
    }
    n->hw_off = off; off += 16;
    n->hb_off = off; off += 1;
    n->nparam = off;
    n->P = n->alloc<float>(off);
    n->x0 = act(n, 0, 16); n->a0 = act(n, 0, 16); n->p0 = act(n, 1, 16); n->a1 = act(n, 1, 32);
    n->p1 = act(n, 2, 32); n->a2 = act(n, 2, 64); n->p2 = act(n, 3, 64); n->a3 = act(n, 3, 128);
    n->b3 = act(n, 3, 128); n->c2 = act(n, 3, 64); n->s2 = act(n, 2, 64); n->b2 = act(n, 2, 64);
    n->c1 = act(n, 2, 32); n->s1 = act(n, 1, 32); n->b1 = act(n, 1, 32); n->c0 = act(n, 1, 16);
    n->s0 = act(n, 0, 16);
    n->in3 = n->alloc<float>(3 * n->V[0]);
    n->hout = n->alloc<float>(n->V[0]);
    n->sc = n->alloc<double>(8);
    n->err = n->alloc<int>(1);
    if (n->train) {
        n->G = n->alloc<float>(off); n->M = n->alloc<float>(off); n->Vv = n->alloc<float>(off);
        n->b0 = act(n, 0, 16);
        n->dz0b = act(n, 0, 16); n->dzs0 = act(n, 0, 16); n->dc0 = act(n, 1, 16); n->dz1b = act(n, 1, 32);
        n->dzs1 = act(n, 1, 32); n->dc1 = act(n, 2, 32); n->dz2b = act(n, 2, 64); n->dzs2 = act(n, 2, 64);
        n->dc2 = act(n, 3, 64); n->dz3b = act(n, 3, 128); n->dz3 = act(n, 3, 128); n->dp2 = act(n, 3, 64);
        n->dz2 = act(n, 2, 64); n->dp1 = act(n, 2, 32); n->dz1 = act(n, 1, 32); n->dp0 = act(n, 1, 16);
        n->dz0 = act(n, 0, 16);
        n->gout = n->alloc<float>(n->V[0]);
        n->x64 = n->alloc<double>(n->V[0]); n->r64 = n->alloc<double>(n->V[0]);
        n->rr = n->alloc<double>(n->V[0]); n->q64 = n->alloc<double>(n->V[0]);
    }
    if (n->aerr != cudaSuccess) { delete n; return TURB_ERR_ALLOC; }
    pack_all(n, 0);
    if (cudaDeviceSynchronize() != cudaSuccess) { delete n; return TURB_ERR_CUDA; }
    *out = reinterpret_cast<turb_net *>(n);
    return TURB_OK;
}

int turb_net_destroy(turb_net *h)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n) return TURB_ERR_ARG;
    cudaDeviceSynchronize();
    if (n->part) cudaFree(n->part);
    delete n;
    return TURB_OK;
}

long long turb_net_num_params(const turb_net *h)
{
    const TurbNet *n = reinterpret_cast<const TurbNet *>(h);
    return n ? n->nparam : -1;
}

int turb_net_init_params(turb_net *h, unsigned long long seed)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n) return TURB_ERR_ARG;
    std::vector<float> p((size_t)n->nparam, 0.f);
    Rng rng{seed};
    for (int l = 0; l < NL; l++) {
        double sd = std::sqrt(2.0 / (27.0 * DEFS[l].cin));
        for (long long i = 0; i < 27LL * DEFS[l].cin * DEFS[l].cout; i++) p[(size_t)(n->woff[l] + i)] = (float)(sd * rng.normal());
    }
    for (int j = 0; j < 16; j++) p[(size_t)(n->hw_off + j)] = (float)(0.05 * rng.normal());
    return turb_net_set_params(h, p.data(), n->nparam);
}

int turb_net_set_params(turb_net *h, const float *host, long long count)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n || !host || count != n->nparam) return TURB_ERR_ARG;
    if (cudaMemcpy(n->P, host, (size_t)count * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return TURB_ERR_CUDA;
    if (n->train) {
        cudaMemset(n->M, 0, (size_t)count * sizeof(float));
        cudaMemset(n->Vv, 0, (size_t)count * sizeof(float));
        n->adam_t = 0;
    }
    pack_all(n, 0);
    return cudaDeviceSynchronize() == cudaSuccess ? TURB_OK : TURB_ERR_CUDA;
}

int turb_net_get_params(turb_net *h, float *host, long long count)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n || !host || count != n->nparam) return TURB_ERR_ARG;
    return cudaMemcpy(host, n->P, (size_t)count * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? TURB_OK
                                                                                                       : TURB_ERR_CUDA;
}

int turb_net_get_grads(turb_net *h, float *host, long long count)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n || !n->train || !host || count != n->nparam) return TURB_ERR_ARG;
    return cudaMemcpy(host, n->G, (size_t)count * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? TURB_OK
                                                                                                       : TURB_ERR_CUDA;
}

int turb_net_forward(turb_net *h, const float *in3, float *out, void *stream)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n || !in3 || !out) return TURB_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    NCHK(forward(n, s, in3, out));
    return read_err(n, s);
}

int turb_net_backward(turb_net *h, const float *gout, void *stream)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n || !n->train || !gout) return TURB_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    NCHK(backward(n, s, gout));
    return read_err(n, s);
}

int turb_net_set_loss(turb_net *h, double w_residual, double w_energy)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n || !(w_residual >= 0.0) || !(w_energy >= 0.0) || w_residual + w_energy <= 0.0) return TURB_ERR_ARG;
    n->wr = w_residual;
    n->we = w_energy;
    return TURB_OK;
}

int turb_net_adam(turb_net *h, float lr, void *stream)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n || !n->train || !(lr > 0.f)) return TURB_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    adam(n, s, lr);
    return cudaStreamSynchronize(s) == cudaSuccess ? TURB_OK : TURB_ERR_CUDA;
}

// forward activations in order x0 a0 p0 a1 p1 a2 p2 a3 b3 c2 s2 b2 c1 s1 b1 c0 s0 b0,
// copied as raw BF16 bits in the channel-blocked layout
int turb_net_get_activation(turb_net *h, int which, uint16_t *host, long long count)
{
    TurbNet *n = reinterpret_cast<TurbNet *>(h);
    if (!n || !host || which < 0 || which > 17) return TURB_ERR_ARG;
    struct A { bf16 *p; int lev, c; };
    const A t[18] = {{n->x0, 0, 16}, {n->a0, 0, 16}, {n->p0, 1, 16}, {n->a1, 1, 32}, {n->p1, 2, 32}, {n->a2, 2, 64},
                     {n->p2, 3, 64}, {n->a3, 3, 128}, {n->b3, 3, 128}, {n->c2, 3, 64}, {n->s2, 2, 64}, {n->b2, 2, 64},
                     {n->c1, 2, 32}, {n->s1, 1, 32}, {n->b1, 1, 32}, {n->c0, 1, 16}, {n->s0, 0, 16}, {n->b0, 0, 16}};
    const A &a = t[which];
    if (!a.p || count != n->V[a.lev] * a.c) return TURB_ERR_ARG;
    return cudaMemcpy(host, a.p, (size_t)count * 2, cudaMemcpyDeviceToHost) == cudaSuccess ? TURB_OK : TURB_ERR_CUDA;
}

int turb_snaps_create(int nx, int ny, int nz, int capacity, turb_snaps **out)
{
    if (!out || nx < 1 || ny < 1 || nz < 1 || capacity < 1) return TURB_ERR_ARG;
    *out = nullptr;
    TurbSnaps *s = new TurbSnaps();
    s->nx = nx; s->ny = ny; s->nz = nz; s->cap = capacity;
    s->V = (long long)nx * ny * nz;
    if (cudaMalloc(&s->data, (size_t)capacity * SNAP_CH * s->V * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&s->sc, 8 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&s->base, (size_t)s->V * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&s->e0, (size_t)capacity * sizeof(double)) != cudaSuccess) {
        if (s->data) cudaFree(s->data);
        delete s;
        return TURB_ERR_ALLOC;
    }
    *out = reinterpret_cast<turb_snaps *>(s);
    return TURB_OK;
}

int turb_snaps_destroy(turb_snaps *h)
{
    TurbSnaps *s = reinterpret_cast<TurbSnaps *>(h);
    if (!s) return TURB_ERR_ARG;
    cudaDeviceSynchronize();
    cudaFree(s->data);
    cudaFree(s->sc);
    cudaFree(s->base);
    cudaFree(s->e0);
    if (s->x64) cudaFree(s->x64);
    if (s->q64) cudaFree(s->q64);
    if (s->part) cudaFree(s->part);
    delete s;
    return TURB_OK;
}

int turb_snaps_count(const turb_snaps *h)
{
    const TurbSnaps *s = reinterpret_cast<const TurbSnaps *>(h);
    return s ? s->n : -1;
}

int turb_snaps_data(turb_snaps *h, int index, const float **dev_ptr)
{
    TurbSnaps *s = reinterpret_cast<TurbSnaps *>(h);
    if (!s || !dev_ptr || index < 0 || index >= s->n) return TURB_ERR_ARG;
    *dev_ptr = s->data + (long long)index * SNAP_CH * s->V;
    return TURB_OK;
}

int turb_conv3_test(int X, int Y, int Z, int cin, int cout, const void *in, const float *W, const float *bias,
                    int relu, int dgrad_mode, void *out, void *stream)
{
    if (!in || !W || !out || X < 1 || Y < 1 || Z < 1 || cin % 16 || cout % 16 || cin > 128 || cout > 128)
        return TURB_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    ConvPlan pf = conv_plan(X, Y, Z, cin, cout), pb = conv_plan(X, Y, Z, cout, cin);
    bf16 *wf = nullptr, *wd = nullptr;
    int *err = nullptr;
    size_t nwf = (size_t)conv_pack_elems(cin, cout), nwd = (size_t)conv_pack_elems(cout, cin);
    if (cudaMalloc(&wf, nwf * 2) != cudaSuccess || cudaMalloc(&wd, nwd * 2) != cudaSuccess ||
        cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
        cudaFree(wf); cudaFree(wd);
        return TURB_ERR_ALLOC;
    }
    cudaMemsetAsync(wf, 0, nwf * 2, s);
    cudaMemsetAsync(wd, 0, nwd * 2, s);
    cudaMemsetAsync(err, 0, sizeof(int), s);
    conv_pack_weights(s, W, cin, cout, pf, pb, wf, wd);
    ConvEpi e;
    e.bias = dgrad_mode ? nullptr : bias;
    e.relu = relu;
    e.out = reinterpret_cast<bf16 *>(out);
    int rc = dgrad_mode ? conv3_fwd(s, reinterpret_cast<const bf16 *>(in), X, Y, Z, cout, cin, wd, e, err, nsm)
                        : conv3_fwd(s, reinterpret_cast<const bf16 *>(in), X, Y, Z, cin, cout, wf, e, err, nsm);
    int h = 0;
    cudaError_t ce = cudaStreamSynchronize(s);
    if (ce == cudaSuccess) ce = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(wf); cudaFree(wd); cudaFree(err);
    if (rc) return turb_set_error_text(conv_last_error());
    return (ce != cudaSuccess || h) ? TURB_ERR_CUDA : TURB_OK;
}

int turb_conv3_wgrad_test(int X, int Y, int Z, int cin, int cout, const void *x, const void *dy, float *dw,
                          void *stream)
{
    if (!x || !dy || !dw || cin % 16 || cout % 16 || cin > 128 || cout > 128) return TURB_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int *err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return TURB_ERR_ALLOC;
    cudaMemsetAsync(err, 0, sizeof(int), s);
    cudaMemsetAsync(dw, 0, 27ull * cin * cout * sizeof(float), s);
    int rc = conv3_wgrad(s, reinterpret_cast<const bf16 *>(x), reinterpret_cast<const bf16 *>(dy), X, Y, Z, cin, cout,
                         dw, err, nsm);
    int h = 0;
    cudaError_t ce = cudaStreamSynchronize(s);
    if (ce == cudaSuccess) ce = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(err);
    if (rc) return turb_set_error_text(conv_last_error());
    return (ce != cudaSuccess || h) ? TURB_ERR_CUDA : TURB_OK;
}

int turb_selftest_umma(int mn_major, int swap, unsigned long long *mismatches)
{
    if (!mismatches) return TURB_ERR_ARG;
    return conv_selftest_umma(mn_major, swap, mismatches) ? TURB_ERR_CUDA : TURB_OK;
}

}  // extern "C"
