// k_noalloc.cu -- the velocity-divergence check (Pressure_compute_velocity_divergence,
// Pressure.c:462-586, closed box) for callers that cannot allocate GPU memory.
//
// Some callers cannot call cudaMalloc: a host that runs under a fixed device
// memory budget, or a plugin that gets its device buffers from a host
// application and may not create its own.  turb_velocity_divergence_noalloc
// takes every input and output as caller-owned device memory and keeps the
// only scratch it needs -- one partial maximum per thread block -- in a
// file-scope __device__ array of fixed size, so no call allocates.  The array
// is part of the library image: every GPU that loads the library holds it
// (TURB_NOALLOC_MAX_BLOCKS doubles, 512 KB) until the process exits.
//
// The call copies the maximum to the host and synchronizes its stream, so it
// is made outside any stream capture.  Its first call on a device resolves
// the array's device address; cudaDeviceReset after that call is not
// supported (the cached address would belong to the old context).
//
// The arithmetic is that of k_divergence (k_stencil.cu) without the open-face
// branches, so on a closed box both entry points return the same bits.
#include <mutex>

#include "../../include/turbins_gb300.h"
#include "turb_internal.cuh"

namespace {

constexpr int KCN = 8;   // planes per thread: keeps the block count small

// shared by every call on a device; the last slot holds the final maximum
__device__ __align__(256) double g_noalloc_scratch[TURB_NOALLOC_MAX_BLOCKS + 1];

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }

__device__ __forceinline__ double block_max(double m)
{
    __shared__ double sm[32];
    int lt = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    m = turb_warp_maxbits(m);
    if ((lt & 31) == 0) sm[lt >> 5] = m;
    __syncthreads();
    if (lt < 32) {
        m = (lt < (nt >> 5)) ? sm[lt] : 0.0;
        m = turb_warp_maxbits(m);
    }
    return m;
}

__global__ void k_div_noalloc(int NX, int NY, int NZ, long long PX, const double *__restrict__ u,
                              const double *__restrict__ v, const double *__restrict__ w,
                              const uint8_t *__restrict__ st, const double *__restrict__ mxc,
                              const double *__restrict__ myc, const double *__restrict__ mzc, double a_dEta,
                              double a_dXi, double a_dPhi, double *__restrict__ div, double *__restrict__ part)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    long long plane = PX * NY;
    double m = 0.0;
    if (i < NX && j < NY)
        for (int kk = 0; kk < KCN; kk++) {
            int k = blockIdx.z * KCN + kk;
            if (k >= NZ) break;
            long long p = ((long long)k * NY + j) * PX + i;
            double dc = 0.0;
            // the last layer i = nx, j = ny, k = nz is BOUNDARY in a valid
            // status array; the index test keeps every neighbour read inside
            // the caller's buffers even when it is not
            if (st[p] != T_BOUNDARY && i < NX - 1 && j < NY - 1 && k < NZ - 1) {
                double dudx = ml(ml(sb(u[p + 1], u[p]), a_dEta), mxc[i]);
                double dvdy = ml(ml(sb(v[p + PX], v[p]), a_dXi), myc[j]);
                double dwdz = ml(ml(sb(w[p + plane], w[p]), a_dPhi), mzc[k]);
                dc = fabs(ad(ad(dudx, dvdy), dwdz));
            }
            div[p] = dc;
            m = turb_maxbits(m, dc);
        }
    m = block_max(m);
    if (threadIdx.x == 0 && threadIdx.y == 0)
        part[((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = m;
}

__global__ void k_max_noalloc(int nparts, double *__restrict__ part)
{
    double m = 0.0;
    for (int t = threadIdx.x; t < nparts; t += blockDim.x) m = turb_maxbits(m, part[t]);
    m = block_max(m);
    if (threadIdx.x == 0) part[TURB_NOALLOC_MAX_BLOCKS] = m;
}

// device address of the scratch array, resolved once per device with that
// device current (a host-side reference to the array is not a device address)
std::mutex g_lock;
double *g_scratch[256] = {nullptr};

int scratch_of_current_device(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    if (dev < 0 || dev >= 256) return TURB_ERR_ARG;
    std::lock_guard<std::mutex> g(g_lock);
    if (!g_scratch[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
        g_scratch[dev] = (double *)p;
    }
    *out = g_scratch[dev];
    return TURB_OK;
}

}  // namespace

extern "C" int turb_velocity_divergence_noalloc(int nx, int ny, int nz, long long pitch, const double *u,
                                                const double *v, const double *w, const uint8_t *c_status,
                                                const double *mxc, const double *myc, const double *mzc,
                                                double *div, double *div_max, void *stream)
{
    if (nx < 2 || ny < 2 || nz < 2 || pitch < nx + 1 || !u || !v || !w || !c_status || !mxc || !myc || !mzc ||
        !div || !div_max)
        return TURB_ERR_ARG;
    int NX = nx + 1, NY = ny + 1, NZ = nz + 1;
    dim3 g((unsigned)((NX + 31) / 32), (unsigned)((NY + 7) / 8), (unsigned)((NZ + KCN - 1) / KCN));
    long long nparts = (long long)g.x * g.y * g.z;
    if (nparts > TURB_NOALLOC_MAX_BLOCKS) return TURB_ERR_SCRATCH_LIMIT;
    double *part = nullptr;
    int rc = scratch_of_current_device(&part);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    k_div_noalloc<<<g, dim3(32, 8), 0, s>>>(NX, NY, NZ, pitch, u, v, w, c_status, mxc, myc, mzc, 1.0 / (1.0 / nx),
                                            1.0 / (1.0 / ny), 1.0 / (1.0 / nz), div, part);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_max_noalloc<<<1, 1024, 0, s>>>((int)nparts, part);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(div_max, part + TURB_NOALLOC_MAX_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    return (*div_max != *div_max) ? TURB_ERR_NAN : TURB_OK;
}
