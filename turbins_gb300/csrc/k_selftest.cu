// k_selftest.cu -- on-device self-tests of arithmetic building blocks.
// turb_selftest_division compares div_by_spacing (turb_div.cuh) with the IEEE
// division __ddiv_rn bit for bit on random and adversarial operands;
// turb_selftest_division_pairs returns the two-term quotient
// (div_by_spacing_2t) and the IEEE quotient of caller-chosen pairs, and
// turb_division_two_term_exact is the set-up's per-spacing check.
#include <algorithm>
#include <cstdint>
#include "../../include/turbins_gb300.h"
#include "turb_div.cuh"
#include "turb_internal.cuh"

namespace {

__device__ __forceinline__ unsigned long long mix(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// double with random mantissa and exponent in [emin, emax]
__device__ __forceinline__ double rnd(unsigned long long r, int emin, int emax, bool sign)
{
    unsigned long long m = r & 0xFFFFFFFFFFFFFULL;
    int e = emin + (int)((r >> 52) % (unsigned)(emax - emin + 1));
    unsigned long long bits = ((unsigned long long)(e + 1023) << 52) | m;
    if (sign && ((r >> 63) & 1)) bits |= 0x8000000000000000ULL;
    return __longlong_as_double((long long)bits);
}

__global__ void k_selftest(long long n, unsigned long long seed, unsigned long long *bad, double *ex)
{
    unsigned long long nbad = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        unsigned long long r1 = mix(seed ^ (2 * t)), r2 = mix(seed ^ (2 * t + 1)), r3 = mix(r1 ^ r2);
        double h = rnd(r2, -14, 3, false);               // spacings 6e-5 .. 16
        double y = __ddiv_rn(1.0, h);
        double a;
        switch ((r3 >> 60) == 0 ? 4 + (int)((r3 >> 56) & 3) : (int)(r3 & 3)) {
        case 4: a = ((r3 >> 1) & 1) ? -0.0 : 0.0; break;  // zero numerators keep their sign
        case 5: a = rnd(r1, -1022, -880, true); break;    // tiny: IEEE branch and its edge
        case 6: a = rnd(r1, 880, 1000, true); break;      // huge: IEEE branch and its edge
        case 7: a = __longlong_as_double((long long)(r1 & 0x800FFFFFFFFFFFFFULL)); break;   // subnormal
        case 0: a = rnd(r1, -80, 80, true); break;        // generic
        case 1: a = __dmul_rn(rnd(r1, -40, 40, true), h); break;   // a/h near a double
        case 2: {                                         // a/h near a midpoint
            double q = rnd(r1, -40, 40, true);
            double qm = __dadd_rn(q, __dmul_rn(0.5, __dadd_rn(__longlong_as_double(__double_as_longlong(q) + 1), -q)));
            a = __dmul_rn(qm, h);
            break;
        }
        default: {                                        // difference of nearby values
            double b0 = rnd(r1, -20, 20, true);
            a = __dadd_rn(__longlong_as_double(__double_as_longlong(b0) + (long long)(r3 >> 40) % 9), -b0);
            break;
        }
        }
        double q1 = div_by_spacing(a, h, y, recip_low(h, y)), q2 = __ddiv_rn(a, h);
        if (__double_as_longlong(q1) != __double_as_longlong(q2)) {
            nbad++;
            ex[0] = a; ex[1] = h;
        }
    }
    if (nbad) atomicAdd(bad, nbad);
}

// FP64 pipe throughput: eight independent FMA chains per thread (the chains
// hide the FMA latency), values kept near 1 so no operand turns subnormal
__global__ void k_dfma_rate(int iters, double b, double c, double *out)
{
    double a[8];
#pragma unroll
    for (int t = 0; t < 8; t++) a[t] = 1.0 + 1e-3 * (threadIdx.x + t);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int t = 0; t < 8; t++) a[t] = fma(a[t], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < 8; t++) s += a[t];
    if (s == 12345.678) out[0] = s;   // never true: keeps the chains live
}

// per pair: the kernels' two-term quotient (div_by_spacing_2t, with the
// reciprocal and its correction formed here as the set-up forms them) and the
// IEEE quotient
__global__ void k_div_pairs(long long n, const double *__restrict__ a, const double *__restrict__ h,
                            double *__restrict__ q2t, double *__restrict__ qd)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double y = __ddiv_rn(1.0, h[t]);
        q2t[t] = div_by_spacing_2t(a[t], h[t], y, recip_low(h[t], y));
        qd[t] = __ddiv_rn(a[t], h[t]);
    }
}

}  // namespace

extern "C" int turb_division_two_term_exact(double h)
{
    const double y = 1.0 / h;
    return div_two_term_exact(h, y, recip_low(h, y)) ? 1 : 0;
}

extern "C" int turb_selftest_division_pairs(long long n, const double *a, const double *h, double *q_two_term,
                                            double *q_ieee)
{
    if (n <= 0 || !a || !h || !q_two_term || !q_ieee) return TURB_ERR_ARG;
    const size_t b = sizeof(double) * (size_t)n;
    double *buf = nullptr;
    TURB_CHECK(cudaMalloc(&buf, 4 * b));
    double *da = buf, *dh = buf + n, *d2 = buf + 2 * n, *dd = buf + 3 * n;
    cudaError_t e = cudaMemcpy(da, a, b, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dh, h, b, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const long long blocks = std::min<long long>((n + 255) / 256, 4096);
        k_div_pairs<<<(unsigned)blocks, 256>>>(n, da, dh, d2, dd);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(q_two_term, d2, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(q_ieee, dd, b, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    return TURB_OK;
}

// FP64 FMA instructions per second of this GPU (thread-level, so one DFMA of
// one thread counts once; FLOP/s is twice this): a fixed number of DFMAs on
// every SM, timed with CUDA events on the legacy stream after one untimed
// launch.  Reports the larger of two timed launches' rates.
extern "C" int turb_measure_fp64_rate(double *dfma_per_s)
{
    if (!dfma_per_s) return TURB_ERR_ARG;
    int dev = 0, nsm = 0;
    TURB_CHECK(cudaGetDevice(&dev));
    TURB_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    double *dout = nullptr;
    TURB_CHECK(cudaMalloc(&dout, sizeof(double)));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = nsm * 8, threads = 256, iters = 4096;
    double best = 0.0;
    cudaError_t e = cudaSuccess;
    for (int rep = 0; rep < 3 && e == cudaSuccess; rep++) {
        cudaEventRecord(e0, 0);
        k_dfma_rate<<<blocks, threads>>>(iters, 1.0000000001, 1e-12, dout);
        cudaEventRecord(e1, 0);
        e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        double ops = (double)blocks * threads * iters * 8.0;
        if (rep > 0 && ms > 0.0f) best = std::max(best, ops / (ms * 1e-3));
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(dout);
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    *dfma_per_s = best;
    return TURB_OK;
}

extern "C" int turb_selftest_division(long long nsamples, unsigned long long seed, unsigned long long *mismatches,
                                      double *example)
{
    if (nsamples <= 0 || !mismatches) return TURB_ERR_ARG;
    unsigned long long *dbad = nullptr;
    double *dex = nullptr;
    TURB_CHECK(cudaMalloc(&dbad, sizeof(unsigned long long)));
    TURB_CHECK(cudaMalloc(&dex, 2 * sizeof(double)));
    cudaMemset(dbad, 0, sizeof(unsigned long long));
    cudaMemset(dex, 0, 2 * sizeof(double));
    k_selftest<<<1216, 256>>>(nsamples, seed, dbad, dex);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, dbad, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && example) e = cudaMemcpy(example, dex, 2 * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dbad);
    cudaFree(dex);
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    return TURB_OK;
}
