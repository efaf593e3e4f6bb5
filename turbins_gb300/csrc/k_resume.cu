// k_resume.cu -- staging kernels of the restart files: a pitched FP64 field
// (or the uint8 c status as FP64 codes, the reference's G_c_status) to the
// compact, big-endian words of a PETSc binary vector, and back.  One thread
// per point along x, one block row per (j, k): every access is coalesced.
#include <cstdint>
#include "turb_internal.cuh"

namespace {

__device__ __forceinline__ unsigned long long bswap64(unsigned long long x)
{
    unsigned lo = (unsigned)x, hi = (unsigned)(x >> 32);
    return ((unsigned long long)__byte_perm(lo, 0, 0x0123) << 32) | __byte_perm(hi, 0, 0x0123);
}

__global__ void k_pack_be(Dims d, const double *__restrict__ src, unsigned long long *__restrict__ dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= d.NX) return;
    long long t = ((long long)k * d.NY + j) * d.NX + i;
    dst[t] = bswap64((unsigned long long)__double_as_longlong(src[d.at(i, j, k)]));
}

__global__ void k_pack_status_be(Dims d, const uint8_t *__restrict__ st, unsigned long long *__restrict__ dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= d.NX) return;
    long long t = ((long long)k * d.NY + j) * d.NX + i;
    dst[t] = bswap64((unsigned long long)__double_as_longlong((double)st[d.at(i, j, k)]));
}

__global__ void k_unpack_be(Dims d, const unsigned long long *__restrict__ src, double *__restrict__ dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= d.NX) return;
    long long t = ((long long)k * d.NY + j) * d.NX + i;
    dst[d.at(i, j, k)] = __longlong_as_double((long long)bswap64(src[t]));
}

inline dim3 grid_of(const Dims &d) { return dim3((d.NX + 127) / 128, d.NY, d.NZ); }

}  // namespace

void launch_pack_be(cudaStream_t s, const Dims &d, const double *src, unsigned long long *dst)
{
    k_pack_be<<<grid_of(d), 128, 0, s>>>(d, src, dst);
}
void launch_pack_status_be(cudaStream_t s, const Dims &d, const uint8_t *st, unsigned long long *dst)
{
    k_pack_status_be<<<grid_of(d), 128, 0, s>>>(d, st, dst);
}
void launch_unpack_be(cudaStream_t s, const Dims &d, const unsigned long long *src, double *dst)
{
    k_unpack_be<<<grid_of(d), 128, 0, s>>>(d, src, dst);
}
