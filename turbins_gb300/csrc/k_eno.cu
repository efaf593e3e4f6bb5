// k_eno.cu -- ENO convection: the line driver restated around
// ENO_compute_convective_terms (ENO.c:103-245) and the ghost-cell rules of
// Velocity_{u,v,w}_ENO_ghost_cells / Conc_ENO_ghost_cells.
//
// Work per (quantity, direction) pass, conv = Vx dq/dx (+ Vy dq/dy) (+ Vz dq/dz):
//  * x: one block per x-line; the line buffer (interior + ghosts) is staged in
//       shared memory and each divided difference is formed once;
//  * y, z: one thread per line walking along it with a sliding register
//       window (loads coalesced across i); each step forms one new D1, D2, D3.
// Every divided difference is an IEEE division on the same operands as the
// reference, and all sums/products are rounded one by one (no FMA), so the
// stencil choices and fluxes are bit-identical to the reference's C.
#include <algorithm>

#include "turb_internal.cuh"
#include "turb_kernels.cuh"
#include "turb_div.cuh"

namespace {

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }

// a / h[b] rounded to nearest: IEEE division or the reciprocal-based form;
// for a power-of-two spacing (flag bit `bit` of T.p2[b]) one exact scaling,
// for a spacing whose two-term quotient is exact (bit `bit` << 3) that
// quotient without the correction
__device__ __forceinline__ double dd(const EnoTab &T, double a, const double *__restrict__ h,
                                     const double *__restrict__ rh, const double *__restrict__ rl, int b, int bit)
{
    if (!T.fastdiv) return dv(a, h[b]);
    const int f = T.p2[b];
    if (f & bit) return __dmul_rn(a, rh[b]);
    if (f & (bit << 3)) return div_by_spacing_2t(a, h[b], rh[b], rl[b]);
    return div_by_spacing(a, h[b], rh[b], rl[b]);
}

__device__ __forceinline__ double interp4(double q0, double q1, double q2, double q3, double wx0,
                                          double wx1, double wy0, double wy1)
{
    double qt = ad(ml(wx0, q2), ml(wx1, q3));
    double qb = ad(ml(wx0, q0), ml(wx1, q1));
    return ad(ml(wy0, qb), ml(wy1, qt));
}

struct Vel3 {
    const double *u, *v, *w;
};

__device__ __forceinline__ double adv_vel(const AdvSrc &a, const Dims &d, long long p, int i, int j, int k)
{
    const double *f = a.a;
    long long X = 1, Y = d.PX, Z = d.plane;
    switch (a.kind) {
    case 0: return f[p];
    case 1: return ad(f[p], a.shift);
    case 2: return interp4(f[p - X], f[p], f[p - X + Y], f[p + Y], a.wx.w0[i], a.wx.w1[i], a.wy.w0[j], a.wy.w1[j]);
    case 3: return interp4(f[p - X], f[p], f[p - X + Z], f[p + Z], a.wx.w0[i], a.wx.w1[i], a.wy.w0[k], a.wy.w1[k]);
    case 4: {
        double q0 = f[p - Y], q1 = f[p - Y + X], q2 = f[p], q3 = f[p + X];
        if (a.pin && i == 0 && j > 0) { q0 = a.pin[(long long)k * a.pNY + j - 1]; q2 = a.pin[(long long)k * a.pNY + j]; }
        if (a.pout && i == a.nx - 1 && j > 0) {
            q1 = a.pout[(long long)k * a.pNY + j - 1];
            q3 = a.pout[(long long)k * a.pNY + j];
        }
        return interp4(q0, q1, q2, q3, a.wx.w0[i], a.wx.w1[i], a.wy.w0[j], a.wy.w1[j]);
    }
    case 5: return interp4(f[p - Y], f[p - Y + Z], f[p], f[p + Z], a.wx.w0[k], a.wx.w1[k], a.wy.w0[j], a.wy.w1[j]);
    case 6: {
        double q0 = f[p - Z], q1 = f[p - Z + X], q2 = f[p], q3 = f[p + X];
        if (a.pin && i == 0 && k > 0) { q0 = a.pin[(long long)(k - 1) * a.pNY + j]; q2 = a.pin[(long long)k * a.pNY + j]; }
        if (a.pout && i == a.nx - 1 && k > 0) {
            q1 = a.pout[(long long)(k - 1) * a.pNY + j];
            q3 = a.pout[(long long)k * a.pNY + j];
        }
        return interp4(q0, q1, q2, q3, a.wx.w0[i], a.wx.w1[i], a.wy.w0[k], a.wy.w1[k]);
    }
    default: return interp4(f[p - Z], f[p], f[p - Z + Y], f[p + Y], a.wx.w0[k], a.wx.w1[k], a.wy.w0[j], a.wy.w1[j]);
    }
}

// D0 of buffer index b (ghost rules precomputed in the table; line = k*NY + j
// of an x line, for the open-face planes)
__device__ __forceinline__ double d0_at(const EnoTab &T, const double *__restrict__ q, long long base,
                                        long long stride, int b, double qf, double ql, long long line = 0)
{
    int r = T.r;
    if (b >= r && b < T.nb - r) return q[base + (long long)(b - r + T.s0) * stride];
    int gi = (b < r) ? b : 3 + (T.nb - 1 - b);
    int src = T.gsrc[gi];
    if (src == 0) return 0.0;
    if (src == 3) return T.glo[line];
    if (src == 4) return T.ghi[line];
    return ml(T.gm[gi], src == 1 ? qf : ql);
}

// ENO_compute_convective_terms body for node c (ENO.c:184-244)
template <int R>
__device__ __forceinline__ double eno_eval(double vel, double d1m1, double d1c, double d2m1, double d2c,
                                          double d2p1, double d3m2, double d3m1, double d3c, double d3p1,
                                          const double *__restrict__ g2, const double *__restrict__ g3)
{
    bool up = vel > 0.0;
    double dQ = up ? d1m1 : d1c;
    if (R > 1) {
        double a = up ? d2m1 : d2c, b = up ? d2c : d2p1;
        bool left = fabs(a) <= fabs(b);
        double cc = left ? a : b;
        dQ = ad(dQ, ml(cc, up ? g2[0] : g2[1]));
        if (R > 2) {
            int kso = (up ? -1 : 0) + (left ? -1 : 0);
            double e = kso == -2 ? d3m2 : (kso == -1 ? d3m1 : d3c);
            double f = kso == -2 ? d3m1 : (kso == -1 ? d3c : d3p1);
            double cs = fabs(e) <= fabs(f) ? e : f;
            dQ = ad(dQ, ml(cs, g3[kso + 2]));
        }
    }
    return ml(vel, dQ);
}

// x pass: one block per line (j = t1, k = t2)
template <int R>
__global__ void k_eno_x(Dims d, EnoTab T, const double *__restrict__ q, AdvSrc adv, int t1a, int t2a,
                        int first, double *__restrict__ conv)
{
    extern __shared__ double sm[];
    int nb = T.nb;
    double *s0 = sm, *s1 = sm + nb, *s2 = sm + 2 * nb, *s3 = sm + 3 * nb;
    int j = t1a + blockIdx.x, k = t2a + blockIdx.y;
    long long base = d.at(0, j, k);
    double qf = q[base + T.s0], ql = q[base + T.e0];
    const long long line = (long long)k * T.gNY + j;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s0[b] = d0_at(T, q, base, 1, b, qf, ql, line);
    __syncthreads();
    for (int b = threadIdx.x; b < nb - 1; b += blockDim.x) s1[b] = dd(T, sb(s0[b + 1], s0[b]), T.h1, T.rh1, T.rl1, b, 1);
    __syncthreads();
    if (R > 1) {
        for (int b = 1 + threadIdx.x; b < nb - 1; b += blockDim.x) s2[b] = dd(T, sb(s1[b], s1[b - 1]), T.h2, T.rh2, T.rl2, b, 2);
        __syncthreads();
    }
    if (R > 2) {
        for (int b = 1 + threadIdx.x; b < nb - 2; b += blockDim.x) s3[b] = dd(T, sb(s2[b + 1], s2[b]), T.h3, T.rh3, T.rl3, b, 4);
        __syncthreads();
    }
    for (int c = R + threadIdx.x; c < nb - R; c += blockDim.x) {
        int i = c - R + T.s0;
        long long p = base + i;
        double vel = adv_vel(adv, d, p, i, j, k);
        double o = eno_eval<R>(vel, s1[c - 1], s1[c], R > 1 ? s2[c - 1] : 0.0, R > 1 ? s2[c] : 0.0,
                               R > 1 ? s2[c + 1] : 0.0, R > 2 ? s3[c - 2] : 0.0, R > 2 ? s3[c - 1] : 0.0,
                               R > 2 ? s3[c] : 0.0, R > 2 ? s3[c + 1] : 0.0, T.g2 + 2 * c, T.g3 + 3 * c);
        conv[p] = first ? o : ad(conv[p], o);
    }
}

// y / z pass: one thread per segment of a line (blockIdx.z of nseg), a
// sliding window along it.  A segment starts its window afresh from the
// buffer entries before it, so every divided difference is formed from the
// same operands as in one walk of the whole line and the results are the same
// bits; the segments multiply the threads in flight, which hide the latency
// of the line walk.
// 16 blocks of 64 per SM (64 registers, a few spilled to L1): measured 3.7 %
// faster at 512x256x256 than the 10 blocks that 96 registers allow, and
// faster than 12, 20 or 24 blocks
template <int R>
__global__ void __launch_bounds__(64, 16) k_eno_yz(Dims d, int dir, EnoTab T, const double *__restrict__ q, AdvSrc adv, int t1a,
                         int t1b, int t2a, int first, int seglen, double *__restrict__ conv)
{
    int i = t1a + blockIdx.x * blockDim.x + threadIdx.x;
    if (i > t1b) return;
    int o2 = t2a + blockIdx.y;   // k for the y pass, j for the z pass
    const int cs = R + blockIdx.z * seglen, ce = min(cs + seglen, T.nb - R);
    if (cs >= ce) return;
    long long stride = dir == 1 ? d.PX : d.plane;
    long long base = dir == 1 ? d.at(i, 0, o2) : d.at(i, o2, 0);
    double qf = q[base + (long long)T.s0 * stride], ql = q[base + (long long)T.e0 * stride];
    const int W = 2 * R + 1;
    const int b0 = cs - R;       // buffer index of the window's first entry
    double w0[7], w1[6], w2[5], w3[4];
    // window for c = cs
#pragma unroll
    for (int t = 0; t < W; t++) w0[t] = d0_at(T, q, base, stride, b0 + t, qf, ql);
#pragma unroll
    for (int t = 0; t < 2 * R; t++) w1[t] = dd(T, sb(w0[t + 1], w0[t]), T.h1, T.rh1, T.rl1, b0 + t, 1);
    if (R > 1) {
#pragma unroll
        for (int t = 0; t < 2 * R - 1; t++) w2[t] = dd(T, sb(w1[t + 1], w1[t]), T.h2, T.rh2, T.rl2, b0 + t + 1, 2);
    }
    if (R > 2) {
#pragma unroll
        for (int t = 0; t < 2 * R - 2; t++) w3[t] = dd(T, sb(w2[t + 1], w2[t]), T.h3, T.rh3, T.rl3, b0 + t + 1, 4);
    }
    for (int c = cs; c < ce; c++) {
        int m = c - R + T.s0;
        long long p = base + (long long)m * stride;
        int jj = dir == 1 ? m : o2, kk = dir == 1 ? o2 : m;
        double vel = adv_vel(adv, d, p, i, jj, kk);
        constexpr int R2 = R > 1 ? R - 2 : 0;
        double o = eno_eval<R>(vel, w1[R - 1], w1[R], R > 1 ? w2[R2] : 0.0, R > 1 ? w2[R2 + 1] : 0.0,
                               R > 1 ? w2[R2 + 2] : 0.0, R > 2 ? w3[0] : 0.0, R > 2 ? w3[1] : 0.0,
                               R > 2 ? w3[2] : 0.0, R > 2 ? w3[3] : 0.0, T.g2 + 2 * c, T.g3 + 3 * c);
        conv[p] = first ? o : ad(conv[p], o);
        if (c + 1 < ce) {
            // slide: new D0[c+1+R], D1[c+R], D2[c+R], D3[c+R-1]
#pragma unroll
            for (int t = 0; t < W - 1; t++) w0[t] = w0[t + 1];
            w0[W - 1] = d0_at(T, q, base, stride, c + 1 + R, qf, ql);
#pragma unroll
            for (int t = 0; t < 2 * R - 1; t++) w1[t] = w1[t + 1];
            w1[2 * R - 1] = dd(T, sb(w0[W - 1], w0[W - 2]), T.h1, T.rh1, T.rl1, c + R, 1);
            if (R > 1) {
#pragma unroll
                for (int t = 0; t < 2 * R - 2; t++) w2[t] = w2[t + 1];
                w2[2 * R - 2] = dd(T, sb(w1[2 * R - 1], w1[2 * R - 2]), T.h2, T.rh2, T.rl2, c + R, 2);
            }
            if (R > 2) {
#pragma unroll
                for (int t = 0; t < 2 * R - 3; t++) w3[t] = w3[t + 1];
                w3[2 * R - 3] = dd(T, sb(w2[2 * R - 2], w2[2 * R - 3]), T.h3, T.rh3, T.rl3, c + R - 1, 4);
            }
        }
    }
}

// one full line exactly as ENO.c (host line API)
__global__ void k_eno_line(int order, int n, const double *__restrict__ D0, const double *__restrict__ P,
                           const double *__restrict__ V, double *__restrict__ out)
{
    extern __shared__ double sm[];
    double *D1 = sm, *D2 = sm + n, *D3 = sm + 2 * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) { D1[i] = 0.0; D2[i] = 0.0; D3[i] = 0.0; }
    __syncthreads();
    for (int i = threadIdx.x; i < n - 1; i += blockDim.x) D1[i] = dv(sb(D0[i + 1], D0[i]), sb(P[i + 1], P[i]));
    __syncthreads();
    if (order > 1)
        for (int i = 1 + threadIdx.x; i < n - 1; i += blockDim.x) D2[i] = dv(sb(D1[i], D1[i - 1]), sb(P[i + 1], P[i - 1]));
    __syncthreads();
    if (order > 2)
        for (int i = 1 + threadIdx.x; i < n - 2; i += blockDim.x) D3[i] = dv(sb(D2[i + 1], D2[i]), sb(P[i + 2], P[i - 1]));
    __syncthreads();
    for (int i = order + threadIdx.x; i < n - order; i += blockDim.x) {
        int k = V[i] > 0.0 ? i - 1 : i, ks = 0;
        double dQ = D1[k];
        if (order > 1) {
            double c;
            if (fabs(D2[k]) <= fabs(D2[k + 1])) { c = D2[k]; ks = k - 1; }
            else { c = D2[k + 1]; ks = k; }
            dQ = ad(dQ, ml(c, ad(sb(P[i], P[k]), sb(P[i], P[k + 1]))));
        }
        if (order > 2) {
            double cs = fabs(D3[ks]) <= fabs(D3[ks + 1]) ? D3[ks] : D3[ks + 1];
            double xi = P[i], a = P[ks], b = P[ks + 1], e = P[ks + 2];
            double g = ad(ad(ml(sb(xi, a), sb(xi, b)), ml(sb(xi, b), sb(xi, e))), ml(sb(xi, a), sb(xi, e)));
            dQ = ad(dQ, ml(cs, g));
        }
        out[i] = ml(V[i], dQ);
    }
}

}  // namespace

// segments: per y / z line, 0 = about 64 nodes per segment, 1 = each line
// walked by one thread
void launch_eno_pass(cudaStream_t s, const Dims &d, int dir, const EnoTab &tab, const double *q, AdvSrc adv,
                     int t1a, int t1b, int t2a, int t2b, int first, double *conv, int segments)
{
    int n1 = t1b - t1a + 1, n2 = t2b - t2a + 1;
    if (n1 <= 0 || n2 <= 0) return;
    if (dir == 0) {
        dim3 g(n1, n2);
        size_t sh = sizeof(double) * 4 * (size_t)tab.nb;
        if (tab.r == 1) k_eno_x<1><<<g, 128, sh, s>>>(d, tab, q, adv, t1a, t2a, first, conv);
        else if (tab.r == 2) k_eno_x<2><<<g, 128, sh, s>>>(d, tab, q, adv, t1a, t2a, first, conv);
        else k_eno_x<3><<<g, 128, sh, s>>>(d, tab, q, adv, t1a, t2a, first, conv);
    } else {
        // segments of about 64 nodes per line (at least one)
        const int ncen = tab.nb - 2 * tab.r;
        const int nseg = segments > 0 ? segments : std::max(1, (ncen + 32) / 64);
        const int seglen = (ncen + nseg - 1) / nseg;
        dim3 g((n1 + 63) / 64, n2, nseg);
        if (tab.r == 1) k_eno_yz<1><<<g, 64, 0, s>>>(d, dir, tab, q, adv, t1a, t1b, t2a, first, seglen, conv);
        else if (tab.r == 2) k_eno_yz<2><<<g, 64, 0, s>>>(d, dir, tab, q, adv, t1a, t1b, t2a, first, seglen, conv);
        else k_eno_yz<3><<<g, 64, 0, s>>>(d, dir, tab, q, adv, t1a, t1b, t2a, first, seglen, conv);
    }
}

int launch_eno_line(int order, int n, const double *D0, const double *P, const double *V, double *out,
                    cudaStream_t s)
{
    size_t sh = sizeof(double) * 3 * (size_t)n;
    if (sh > 200 * 1024) return 1;
    if (sh > 48 * 1024) cudaFuncSetAttribute(k_eno_line, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    k_eno_line<<<1, 256, sh, s>>>(order, n, D0, P, V, out);
    return 0;
}
