// k_diag.cu -- flow diagnostics of the current state, on the device:
//   Extract_total_kinetic_energy (Extract.c:803-882),
//   Extract_kinetic_potential_conversion_rate (Extract.c:727-801),
//   Conc_compute_total_suspended_mass (Conc.c:1471-1522),
//   Conc_compute_potential_energies (Conc.c:1934-2055; suspended part),
//   Conc_compute_ave_height_x (Conc.c:1524-1608).
// Every term follows the reference's own expression (e.g. dV = dx*dy*dz for
// the energies but dz*dy*dx for the suspended mass); the sums run in a fixed
// block order, so results are run-to-run deterministic and differ from the
// reference's serial loops only by summation order.
#include "../../include/turbins_gb300.h"
#include "turb_internal.cuh"

namespace {

constexpr int DBX = 32, DBY = 8, DKC = 4;
constexpr int NQ = 2 + 4 * TURB_MAXCONC;

struct DiagArgs {
    Dims d;
    const uint8_t *cst;
    const double *dxc, *dyc, *dzc, *yc;
    const double *ubc, *vbc, *wbc, *ct;
    const double *c[TURB_MAXCONC];
    int nconc;
    double y_ref;
};

// per block: the 2 + 4 nconc sums, partial[q * nblocks + block]
__global__ void k_diag_sums(DiagArgs a, double *__restrict__ part)
{
    int i = blockIdx.x * DBX + threadIdx.x, j = blockIdx.y * DBY + threadIdx.y;
    double acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) acc[q] = 0.0;
    if (i < a.d.NX && j < a.d.NY) {
        double dx = a.dxc[i], dy = a.dyc[j], yj = a.yc[j] - a.y_ref;
        for (int kk = 0; kk < DKC; kk++) {
            int k = blockIdx.z * DKC + kk;
            if (k >= a.d.NZ) break;
            long long p = a.d.at(i, j, k);
            if (a.cst[p] != T_FLUID) continue;
            double dz = a.dzc[k];
            double dV = __dmul_rn(__dmul_rn(dx, dy), dz);
            double dVm = __dmul_rn(__dmul_rn(dz, dy), dx);
            double u = a.ubc[p], v = a.vbc[p], w = a.wbc[p];
            double e = __dadd_rn(__dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)), __dmul_rn(w, w));
            acc[0] = __dadd_rn(acc[0], __dmul_rn(e, dV));
            acc[1] = __dadd_rn(acc[1], __dmul_rn(__dmul_rn(-v, a.ct[p]), dV));
#pragma unroll
            for (int ic = 0; ic < TURB_MAXCONC; ic++) {
                if (ic >= a.nconc) break;
                double cc = a.c[ic][p], cdv = __dmul_rn(cc, dV);
                acc[2 + 4 * ic] = __dadd_rn(acc[2 + 4 * ic], __dmul_rn(cc, dVm));
                acc[3 + 4 * ic] = __dadd_rn(acc[3 + 4 * ic], __dmul_rn(cdv, yj));
                acc[4 + 4 * ic] = __dadd_rn(acc[4 + 4 * ic], cdv);
                acc[5 + 4 * ic] = __dadd_rn(acc[5 + 4 * ic], __dmul_rn(__dmul_rn(v, cc), dV));
            }
        }
    }
    __shared__ double sm[NQ][DBX * DBY / 32];
    int lt = threadIdx.y * DBX + threadIdx.x, w = lt >> 5;
    long long nb = (long long)gridDim.x * gridDim.y * gridDim.z;
    long long b = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        double s = acc[q];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((lt & 31) == 0) sm[q][w] = s;
    }
    __syncthreads();
    if (lt < NQ) {
        double s = 0.0;
        for (int t = 0; t < DBX * DBY / 32; t++) s += sm[lt][t];
        part[(long long)lt * nb + b] = s;
    }
}

// out[q] = sum over blocks of part[q * nb + .], in a fixed order
__global__ void k_diag_final(long long nb, int nq, const double *__restrict__ part, double *__restrict__ out)
{
    int q = blockIdx.x;
    if (q >= nq) return;
    double s = 0.0;
    for (long long t = threadIdx.x; t < nb; t += blockDim.x) s += part[q * nb + t];
    __shared__ double sm[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int t = 0; t < (int)(blockDim.x >> 5); t++) r += sm[t];
        out[q] = r;
    }
}

// spanwise heights: hpart[(ic * HG + g) * NX + i] = sum over the (j, k) rows of
// group g of c dy dz at FLUID nodes (Conc.c:1575-1584 term order); threads
// run along i, so every load is coalesced
constexpr int HG = 64;
__global__ void k_diag_height(DiagArgs a, double *__restrict__ hpart)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y;
    if (i >= a.d.NX) return;
    int nrow = a.d.NY * a.d.NZ;
    int r0 = (int)((long long)nrow * g / HG), r1 = (int)((long long)nrow * (g + 1) / HG);
    for (int ic = 0; ic < a.nconc; ic++) {
        double s = 0.0;
        for (int r = r0; r < r1; r++) {
            int k = r / a.d.NY, j = r - k * a.d.NY;
            long long p = a.d.at(i, j, k);
            if (a.cst[p] == T_FLUID) s = __dadd_rn(s, __dmul_rn(__dmul_rn(a.c[ic][p], a.dyc[j]), a.dzc[k]));
        }
        hpart[((long long)ic * HG + g) * a.d.NX + i] = s;
    }
}

__global__ void k_diag_height_final(int NX, int nconc, double coef, const double *__restrict__ hpart,
                                    double *__restrict__ h)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, ic = blockIdx.y;
    if (i >= NX || ic >= nconc) return;
    double s = 0.0;
    for (int g = 0; g < HG; g++) s += hpart[((long long)ic * HG + g) * NX + i];
    h[(long long)ic * NX + i] = __dmul_rn(s, coef);
}

}  // namespace

long long diag_scratch_doubles(const Dims &d)
{
    long long nb = (long long)((d.NX + DBX - 1) / DBX) * ((d.NY + DBY - 1) / DBY) * ((d.NZ + DKC - 1) / DKC);
    long long hp = (long long)TURB_MAXCONC * HG * d.NX;
    return NQ * nb + NQ + hp + (long long)TURB_MAXCONC * d.NX;
}

// sums (NQ doubles) and heights (nconc x NX) end up in `scratch`
void launch_diagnostics(cudaStream_t s, const Dims &d, const uint8_t *cst, const double *dxc, const double *dyc,
                        const double *dzc, const double *yc, double y_ref, double coef, const double *ubc,
                        const double *vbc, const double *wbc, const double *ct, const double *const *c, int nconc,
                        double *scratch, double **sums, double **heights)
{
    DiagArgs a;
    a.d = d; a.cst = cst; a.dxc = dxc; a.dyc = dyc; a.dzc = dzc; a.yc = yc;
    a.ubc = ubc; a.vbc = vbc; a.wbc = wbc; a.ct = ct; a.nconc = nconc; a.y_ref = y_ref;
    for (int ic = 0; ic < TURB_MAXCONC; ic++) a.c[ic] = ic < nconc ? c[ic] : nullptr;
    dim3 g((d.NX + DBX - 1) / DBX, (d.NY + DBY - 1) / DBY, (d.NZ + DKC - 1) / DKC);
    long long nb = (long long)g.x * g.y * g.z;
    double *part = scratch, *out = scratch + NQ * nb, *hp = out + NQ, *h = hp + (long long)TURB_MAXCONC * HG * d.NX;
    k_diag_sums<<<g, dim3(DBX, DBY), 0, s>>>(a, part);
    k_diag_final<<<NQ, 256, 0, s>>>(nb, NQ, part, out);
    k_diag_height<<<dim3((d.NX + 127) / 128, HG), 128, 0, s>>>(a, hp);
    k_diag_height_final<<<dim3((d.NX + 127) / 128, nconc), 128, 0, s>>>(d.NX, nconc, coef, hp, h);
    *sums = out;
    *heights = h;
}
