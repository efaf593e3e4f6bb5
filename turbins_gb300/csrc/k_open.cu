// k_open.cu -- open boundaries on the device: the inflow profiles of
// Inflow.c and the convective outflow condition, mass correction, storage
// and plane copies of Outflow.c / Velocity.c / Conc.c.  Planes are [NZ][NY]
// arrays (j fastest), one thread per (j, k).
#include "turb_internal.cuh"

namespace {

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }

constexpr int OB = 256;

__device__ double block_sum(double v)
{
    __shared__ double sm[OB / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int t = 0; t < OB / 32; t++) r += sm[t];
    return r;
}

// Inflow_u_velocity_profile, Inflow.c:13-160: u_inflow = 1 (times the
// transient factor) where u at i = 1 is FLUID, and its partial influx
__global__ void k_inflow_u(Dims d, const uint8_t *__restrict__ st_u, const double *__restrict__ yv,
                           const double *__restrict__ zw, double tf, double *__restrict__ in, double *__restrict__ part)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double f = 0.0;
    if (t < d.NY * d.NZ) {
        int k = t / d.NY, j = t - k * d.NY;
        if (st_u[d.at(1, j, k)] == T_FLUID) {
            double val = ml(1.0, tf);
            in[t] = val;
            double dA = ml(sb(yv[j + 1], yv[j]), sb(zw[k + 1], zw[k]));
            f = ml(val, dA);
        }
    }
    double s = block_sum(f);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Inflow_conc_profile, Inflow.c:162-260: c_inflow = 1 (times the transient
// factor) where c at i = 0 is not SOLID
__global__ void k_inflow_c(Dims d, const uint8_t *__restrict__ st_c, double tf, double *__restrict__ in)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.NY * d.NZ) return;
    int k = t / d.NY, j = t - k * d.NY;
    if (st_c[d.at(0, j, k)] != T_SOLID) in[t] = ml(1.0, tf);
}

// Outflow_{vel,conc}_impose_convective_boundary, Outflow.c:30-160:
// out = (1 - coef) out + coef q(nx-1) where q's node at i = nx-1 is FLUID or
// IMMERSED, coef = dt U / (xu[nx] - xu[nx-1])
__global__ void k_outflow_conv(Dims d, const uint8_t *__restrict__ st, double coef, const double *__restrict__ q,
                               double *__restrict__ out)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.NY * d.NZ) return;
    int k = t / d.NY, j = t - k * d.NY;
    long long p = d.at(d.nx - 1, j, k);
    int s = st[p];
    if (s == T_FLUID || s == T_IMMERSED) out[t] = ad(ml(sb(1.0, coef), out[t]), ml(coef, q[p]));
}

// Outflow_update_u_velocity_to_conserve_mass, Outflow.c:163-303: partial
// outflux (dA * out) and area over the u nodes at i = nx-1 that are FLUID or
// IMMERSED
__global__ void k_outflux(Dims d, const uint8_t *__restrict__ st_u, const double *__restrict__ yv,
                          const double *__restrict__ zw, const double *__restrict__ out, double *__restrict__ part)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double f = 0.0, a = 0.0;
    if (t < d.NY * d.NZ) {
        int k = t / d.NY, j = t - k * d.NY;
        int s = st_u[d.at(d.nx - 1, j, k)];
        if (s == T_FLUID || s == T_IMMERSED) {
            double dA = ml(sb(yv[j + 1], yv[j]), sb(zw[k + 1], zw[k]));
            a = dA;
            f = ml(dA, out[t]);
        }
    }
    double sf = block_sum(f);
    __syncthreads();
    double sa = block_sum(a);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = sf; part[2 * blockIdx.x + 1] = sa; }
}

// sums the partials in block order; res = {outflux, area, correction}
__global__ void k_outflux_final(int nb, const double *__restrict__ part, const double *__restrict__ influx,
                                double *__restrict__ res)
{
    if (threadIdx.x != 0) return;
    double f = 0.0, a = 0.0;
    for (int b = 0; b < nb; b++) { f += part[2 * b]; a += part[2 * b + 1]; }
    res[0] = f;
    res[1] = a;
    res[2] = __ddiv_rn(sb(*influx, f), a);
}

__global__ void k_outflow_correct(Dims d, const uint8_t *__restrict__ st_u, const double *__restrict__ res,
                                  double *__restrict__ out)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.NY * d.NZ) return;
    int k = t / d.NY, j = t - k * d.NY;
    int s = st_u[d.at(d.nx - 1, j, k)];
    if (s == T_FLUID || s == T_IMMERSED) out[t] = ad(out[t], res[2]);
}

__global__ void k_sum_parts(int nb, const double *__restrict__ part, double *__restrict__ out)
{
    if (threadIdx.x != 0) return;
    double f = 0.0;
    for (int b = 0; b < nb; b++) f += part[b];
    *out = f;
}

// *_rk_average_outflow: out = a out_old + b out
__global__ void k_plane_axpby(int n, double a, const double *__restrict__ old, double b, double *__restrict__ out)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = ad(ml(a, old[t]), ml(b, out[t]));
}

// Outflow_*_copy_data_into_last_plane / _2D_array: the plane i = nx of q
__global__ void k_plane_to_field(Dims d, const double *__restrict__ pl, int set, double *__restrict__ q)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.NY * d.NZ) return;
    int k = t / d.NY, j = t - k * d.NY;
    q[d.at(d.nx, j, k)] = set ? pl[t] : 0.0;
}
__global__ void k_field_to_plane(Dims d, const double *__restrict__ q, double *__restrict__ pl)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.NY * d.NZ) return;
    int k = t / d.NY, j = t - k * d.NY;
    pl[t] = q[d.at(d.nx, j, k)];
}

inline int nblk(const Dims &d) { return (d.NY * d.NZ + OB - 1) / OB; }

}  // namespace

int open_parts(const Dims &d) { return 2 * nblk(d) + 4; }

// influx is left in part[2 nblk] on the device
void launch_inflow_u(cudaStream_t s, const Dims &d, const uint8_t *st_u, const double *yv, const double *zw,
                     double tf, double *in, double *part, double *influx)
{
    k_inflow_u<<<nblk(d), OB, 0, s>>>(d, st_u, yv, zw, tf, in, part);
    k_sum_parts<<<1, 32, 0, s>>>(nblk(d), part, influx);
}
void launch_inflow_c(cudaStream_t s, const Dims &d, const uint8_t *st_c, double tf, double *in)
{
    k_inflow_c<<<nblk(d), OB, 0, s>>>(d, st_c, tf, in);
}
void launch_outflow_conv(cudaStream_t s, const Dims &d, const uint8_t *st, double coef, const double *q, double *out)
{
    k_outflow_conv<<<nblk(d), OB, 0, s>>>(d, st, coef, q, out);
}
void launch_outflow_mass(cudaStream_t s, const Dims &d, const uint8_t *st_u, const double *yv, const double *zw,
                         const double *influx, double *out, double *part, double *res)
{
    k_outflux<<<nblk(d), OB, 0, s>>>(d, st_u, yv, zw, out, part);
    k_outflux_final<<<1, 32, 0, s>>>(nblk(d), part, influx, res);
    k_outflow_correct<<<nblk(d), OB, 0, s>>>(d, st_u, res, out);
}
void launch_plane_axpby(cudaStream_t s, int n, double a, const double *old, double b, double *out)
{
    k_plane_axpby<<<(n + OB - 1) / OB, OB, 0, s>>>(n, a, old, b, out);
}
void launch_plane_to_field(cudaStream_t s, const Dims &d, const double *pl, int set, double *q)
{
    k_plane_to_field<<<nblk(d), OB, 0, s>>>(d, pl, set, q);
}
void launch_field_to_plane(cudaStream_t s, const Dims &d, const double *q, double *pl)
{
    k_field_to_plane<<<nblk(d), OB, 0, s>>>(d, q, pl);
}
