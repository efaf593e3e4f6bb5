// k_diag.cu -- flow diagnostics of the current state and the deposited
// sediment, on the device:
//   Extract_total_kinetic_energy (Extract.c:803-882),
//   Extract_kinetic_potential_conversion_rate (Extract.c:727-801),
//   Extract_viscous_dissipation_rate (Extract.c:453-725),
//   Conc_compute_total_suspended_mass (Conc.c:1471-1522),
//   Conc_compute_potential_energies (Conc.c:1934-2055),
//   Conc_compute_ave_height_x (Conc.c:1524-1608),
//   Conc_compute_sedimentation_rate / Conc_bottom_sed_rate (Conc.c:2098-2230),
//   Grid_set_interface_y_index (Grid.c:1972-2012) and
//   Conc_integrate_deposited_height (Conc.c:1675-1749).
// Every per-node term follows the reference's own expression order with
// explicitly rounded products and sums (e.g. dV = dx*dy*dz for the energies
// but dz*dy*dx for the suspended mass), so terms are bit-identical; the sums
// run in a fixed block order, so results are run-to-run deterministic and
// differ from the reference's serial loops only by summation order.
#include "../../include/turbins_gb300.h"
#include "turb_diag.cuh"

namespace {

constexpr int DBX = 32, DBY = 8, DKC = 4;
constexpr int NQ = DIAG_NQ;                  // ke, rate, visc, 4 per fraction
constexpr int NQB = 2 * TURB_MAXCONC;        // bed sums: ep_passive, sed_rate per fraction

#define MUL __dmul_rn
#define ADD __dadd_rn

// u lap(u) dV_u + v lap(v) dV_v + w lap(w) dV_w of Extract.c:531-703 at the
// FLUID c node (i, j, k)
__device__ double visc_term(const DiagIn &a, int i, int j, int k, long long p)
{
    const Geo &g = a.geo;
    const Dims &d = a.d;
    int NI = d.nx, NJ = d.ny, NK = d.nz;
    double Cx = a.Cx, Cy = a.Cy, Cz = a.Cz;
    double U_ae = MUL(MUL(Cx, g.mxu[i]), g.mxc[i]), U_aw = MUL(Cx, g.mxu[i]);
    double U_an = MUL(MUL(Cy, g.myc[j]), g.myv[j + 1]), U_as = MUL(MUL(Cy, g.myc[j]), g.myv[j]);
    double U_af = MUL(MUL(Cz, g.mzc[k]), g.mzw[k + 1]), U_ab = MUL(MUL(Cz, g.mzc[k]), g.mzw[k]);
    double V_ae = MUL(MUL(Cx, g.mxc[i]), g.mxu[i + 1]), V_aw = MUL(MUL(Cx, g.mxc[i]), g.mxu[i]);
    double V_an = MUL(MUL(Cy, g.myv[j]), g.myc[j]), V_as = MUL(Cy, g.myv[j]);
    double V_af = MUL(MUL(Cz, g.mzc[k]), g.mzw[k + 1]), V_ab = MUL(MUL(Cz, g.mzc[k]), g.mzw[k]);
    double W_ae = MUL(MUL(Cx, g.mxc[i]), g.mxu[i + 1]), W_aw = MUL(MUL(Cx, g.mxc[i]), g.mxu[i]);
    double W_an = MUL(MUL(Cy, g.myc[j]), g.myv[j + 1]), W_as = MUL(MUL(Cy, g.myc[j]), g.myv[j]);
    double W_af = MUL(MUL(Cz, g.mzw[k]), g.mzc[k]), W_ab = MUL(Cz, g.mzw[k]);
    const double *u = a.u, *v = a.v, *w = a.w;
    double u_ = u[p], v_ = v[p], w_ = w[p];
    double U_w, U_e, U_n, U_s, U_f, U_b, V_w, V_e, V_n, V_s, V_f, V_b, W_w, W_e, W_n, W_s, W_f, W_b;
    if (i == 0) {
        U_aw = MUL(U_aw, g.mxc[i]);
        U_w = a.ob.in ? a.ob.pl(a.ob.u_in, j, k) : 0.0;   // Extract.c:582-592
        V_w = MUL(a.kw[0], v_); W_w = MUL(a.kw[0], w_);
    } else {
        U_aw = MUL(U_aw, g.mxc[i - 1]);
        U_w = u[p - 1]; V_w = v[p - 1]; W_w = w[p - 1];
    }
    if (j == 0) {
        V_as = MUL(V_as, g.myc[j]);
        U_s = MUL(a.kw[2], u_); V_s = 0.0; W_s = MUL(a.kw[2], w_);
    } else {
        V_as = MUL(V_as, g.myc[j - 1]);
        U_s = u[p - d.PX]; V_s = v[p - d.PX]; W_s = w[p - d.PX];
    }
    if (k == 0) {
        W_ab = MUL(W_ab, g.mzc[k]);
        U_b = MUL(a.kw[4], u_); V_b = MUL(a.kw[4], v_); W_b = 0.0;
    } else {
        W_ab = MUL(W_ab, g.mzc[k - 1]);
        U_b = u[p - d.plane]; V_b = v[p - d.plane]; W_b = w[p - d.plane];
    }
    if (i == NI - 1) {
        if (a.ob.out) {   // Extract.c:634-639
            U_e = a.ob.pl(a.ob.out_f[0], j, k); V_e = a.ob.pl(a.ob.out_f[1], j, k); W_e = a.ob.pl(a.ob.out_f[2], j, k);
        } else {
            U_e = 0.0; V_e = MUL(a.kw[1], v_); W_e = MUL(a.kw[1], w_);
        }
    } else {
        U_e = u[p + 1]; V_e = v[p + 1]; W_e = w[p + 1];
    }
    if (j == NJ - 1) {
        U_n = MUL(a.kw[3], u_); V_n = 0.0; W_n = MUL(a.kw[3], w_);
    } else {
        U_n = u[p + d.PX]; V_n = v[p + d.PX]; W_n = w[p + d.PX];
    }
    if (k == NK - 1) {
        U_f = MUL(a.kw[5], u_); V_f = MUL(a.kw[5], v_); W_f = 0.0;
    } else {
        U_f = u[p + d.plane]; V_f = v[p + d.plane]; W_f = w[p + d.plane];
    }
    double U_ap = -ADD(ADD(ADD(ADD(ADD(U_ae, U_aw), U_ab), U_af), U_as), U_an);
    double V_ap = -ADD(ADD(ADD(ADD(ADD(V_ae, V_aw), V_ab), V_af), V_as), V_an);
    double W_ap = -ADD(ADD(ADD(ADD(ADD(W_ae, W_aw), W_ab), W_af), W_as), W_an);
    double lu = ADD(ADD(ADD(ADD(MUL(U_ae, U_e), MUL(U_aw, U_w)), ADD(MUL(U_an, U_n), MUL(U_as, U_s))),
                        ADD(MUL(U_af, U_f), MUL(U_ab, U_b))), MUL(U_ap, u_));
    double lv = ADD(ADD(ADD(ADD(MUL(V_ae, V_e), MUL(V_aw, V_w)), ADD(MUL(V_an, V_n), MUL(V_as, V_s))),
                        ADD(MUL(V_af, V_f), MUL(V_ab, V_b))), MUL(V_ap, v_));
    double lw = ADD(ADD(ADD(ADD(MUL(W_ae, W_e), MUL(W_aw, W_w)), ADD(MUL(W_an, W_n), MUL(W_as, W_s))),
                        ADD(MUL(W_af, W_f), MUL(W_ab, W_b))), MUL(W_ap, w_));
    double dVu = MUL(MUL(ADD(g.xc[i + 1], -g.xc[i]), a.dyc[j]), a.dzc[k]);
    double dVv = MUL(MUL(ADD(g.yc[j + 1], -g.yc[j]), a.dxc[i]), a.dzc[k]);
    double dVw = MUL(MUL(ADD(g.zc[k + 1], -g.zc[k]), a.dxc[i]), a.dyc[j]);
    return ADD(ADD(MUL(MUL(u_, lu), dVu), MUL(MUL(v_, lv), dVv)), MUL(MUL(w_, lw), dVw));
}

template <int NQT>
__device__ void block_partials(double (&acc)[NQT], double *__restrict__ part)
{
    __shared__ double sm[NQT][DBX * DBY / 32];
    int lt = threadIdx.y * DBX + threadIdx.x, w = lt >> 5;
    long long nb = (long long)gridDim.x * gridDim.y * gridDim.z;
    long long b = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
#pragma unroll
    for (int q = 0; q < NQT; q++) {
        double s = acc[q];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((lt & 31) == 0) sm[q][w] = s;
    }
    __syncthreads();
    if (lt < NQT) {
        double s = 0.0;
        for (int t = 0; t < DBX * DBY / 32; t++) s += sm[lt][t];
        part[(long long)lt * nb + b] = s;
    }
}

// volume sums over FLUID c nodes, one partial per block
__global__ void __launch_bounds__(DBX *DBY) k_diag_sums(DiagIn a, double *__restrict__ part)
{
    int i = blockIdx.x * DBX + threadIdx.x, j = blockIdx.y * DBY + threadIdx.y;
    double acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) acc[q] = 0.0;
    if (i < a.d.NX && j < a.d.NY) {
        double dx = a.dxc[i], dy = a.dyc[j], yj = ADD(a.geo.yc[j], -a.y_ref);
        for (int kk = 0; kk < DKC; kk++) {
            int k = blockIdx.z * DKC + kk;
            if (k >= a.d.NZ) break;
            long long p = a.d.at(i, j, k);
            if (a.cst[p] != T_FLUID) continue;
            double dz = a.dzc[k];
            double dV = MUL(MUL(dx, dy), dz);
            double dVm = MUL(MUL(dz, dy), dx);
            double u = a.ubc[p], v = a.vbc[p], w = a.wbc[p];
            double e = ADD(ADD(MUL(u, u), MUL(v, v)), MUL(w, w));
            acc[0] = ADD(acc[0], MUL(e, dV));
            acc[1] = ADD(acc[1], MUL(MUL(-v, a.ct[p]), dV));
            acc[2] = ADD(acc[2], visc_term(a, i, j, k, p));
#pragma unroll
            for (int ic = 0; ic < TURB_MAXCONC; ic++) {
                if (ic >= a.nconc) break;
                double cc = a.c[ic][p], cdv = MUL(cc, dV);
                acc[3 + 4 * ic] = ADD(acc[3 + 4 * ic], MUL(cc, dVm));
                acc[4 + 4 * ic] = ADD(acc[4 + 4 * ic], MUL(cdv, yj));
                acc[5 + 4 * ic] = ADD(acc[5 + 4 * ic], cdv);
                acc[6 + 4 * ic] = ADD(acc[6 + 4 * ic], MUL(MUL(v, cc), dV));
            }
        }
    }
    block_partials<NQ>(acc, part);
}

// bed sums over (i, k): deposited potential energy and sedimentation rate of
// each particle fraction at its bed node; sed_bottom gets the per-node rates
__global__ void __launch_bounds__(DBX *DBY) k_diag_bed(DiagIn a, double *__restrict__ part,
                                                       double *__restrict__ sed_bottom)
{
    int i = blockIdx.x * DBX + threadIdx.x, k = blockIdx.y * DBY + threadIdx.y;
    double acc[NQB];
#pragma unroll
    for (int q = 0; q < NQB; q++) acc[q] = 0.0;
    if (i < a.d.NX && k < a.d.NZ) {
        long long b2 = (long long)k * a.d.NX + i;
        int jb = a.iy[b2];
        double dx = a.dxc[i], dz = a.dzc[k];
#pragma unroll
        for (int ic = 0; ic < TURB_MAXCONC; ic++) {
            if (ic >= a.nconc) break;
            double r = 0.0;
            if (a.particle[ic] && jb >= 0 && jb < a.d.NY) {
                if (a.dep) {
                    double h = a.dep[(long long)ic * a.d.NZ * a.d.NX + b2];
                    acc[2 * ic] = MUL(MUL(MUL(h, dx), dz), ADD(a.geo.yc[jb], -a.y_ref));
                }
                r = MUL(MUL(MUL(a.us[ic], a.c[ic][a.d.at(i, jb, k)]), dx), dz);
                acc[2 * ic + 1] = r;
            }
            sed_bottom[(long long)ic * a.d.NZ * a.d.NX + b2] = r;
        }
    }
    block_partials<NQB>(acc, part);
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
__global__ void k_diag_height(DiagIn a, double *__restrict__ hpart)
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
            if (a.cst[p] == T_FLUID) s = ADD(s, MUL(MUL(a.c[ic][p], a.dyc[j]), a.dzc[k]));
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
    h[(long long)ic * NX + i] = MUL(s, coef);
}

// Grid_set_interface_y_index: first IMMERSED c node of the column, or j = 0
// when the bottom node is FLUID, else -1
__global__ void k_bed_index(Dims d, const uint8_t *__restrict__ cst, int32_t *__restrict__ iy)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i >= d.NX || k >= d.NZ) return;
    int r = -1;
    for (int j = 0; j < d.NY; j++) {
        uint8_t s = cst[d.at(i, j, k)];
        if (s == T_IMMERSED || (j == 0 && s == T_FLUID)) {
            r = j;
            break;
        }
    }
    iy[(long long)k * d.NX + i] = r;
}

// Conc_integrate_deposited_height with weight_factor = alpha:
// dep += dt |Vs0| alpha 0.5 (c + c_old) at the bed node of each column
__global__ void k_deposit(Dims d, const int32_t *__restrict__ iy, DepIn a, double *__restrict__ dep)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y, ic = blockIdx.z;
    if (i >= d.NX || k >= d.NZ || ic >= a.nconc) return;
    long long b2 = (long long)k * d.NX + i;
    int jb = iy[b2];
    if (jb < 0 || jb >= d.NY) return;
    long long p = d.at(i, jb, k);
    double f = MUL(MUL(MUL(a.dt, a.us[ic]), a.alpha[ic]), 0.5);
    double *h = dep + (long long)ic * d.NZ * d.NX + b2;
    *h = ADD(*h, MUL(f, ADD(a.c[ic][p], a.c_old[ic][p])));
}

inline long long sums_blocks(const Dims &d)
{
    return (long long)((d.NX + DBX - 1) / DBX) * ((d.NY + DBY - 1) / DBY) * ((d.NZ + DKC - 1) / DKC);
}
inline long long bed_blocks(const Dims &d)
{
    return (long long)((d.NX + DBX - 1) / DBX) * ((d.NZ + DBY - 1) / DBY);
}

}  // namespace

long long diag_scratch_doubles(const Dims &d)
{
    long long bed = (long long)TURB_MAXCONC * d.NZ * d.NX;
    return NQ * sums_blocks(d) + NQ + (long long)TURB_MAXCONC * HG * d.NX + (long long)TURB_MAXCONC * d.NX +
           NQB * bed_blocks(d) + NQB + bed;
}

void launch_diagnostics(cudaStream_t s, const DiagIn &a, double *scratch, DiagOut *o)
{
    const Dims &d = a.d;
    long long nb = sums_blocks(d), nb2 = bed_blocks(d);
    double *part = scratch;
    o->sums = part + NQ * nb;
    double *hp = o->sums + NQ;
    o->heights = hp + (long long)TURB_MAXCONC * HG * d.NX;
    double *part2 = o->heights + (long long)TURB_MAXCONC * d.NX;
    o->bed_sums = part2 + NQB * nb2;
    o->sed_bottom = o->bed_sums + NQB;
    dim3 g((d.NX + DBX - 1) / DBX, (d.NY + DBY - 1) / DBY, (d.NZ + DKC - 1) / DKC);
    k_diag_sums<<<g, dim3(DBX, DBY), 0, s>>>(a, part);
    k_diag_final<<<NQ, 256, 0, s>>>(nb, NQ, part, o->sums);
    k_diag_height<<<dim3((d.NX + 127) / 128, HG), 128, 0, s>>>(a, hp);
    k_diag_height_final<<<dim3((d.NX + 127) / 128, a.nconc), 128, 0, s>>>(d.NX, a.nconc, a.hcoef, hp, o->heights);
    dim3 g2((d.NX + DBX - 1) / DBX, (d.NZ + DBY - 1) / DBY);
    k_diag_bed<<<g2, dim3(DBX, DBY), 0, s>>>(a, part2, o->sed_bottom);
    k_diag_final<<<NQB, 256, 0, s>>>(nb2, NQB, part2, o->bed_sums);
}

void launch_bed_index(cudaStream_t s, const Dims &d, const uint8_t *cst, int32_t *iy)
{
    k_bed_index<<<dim3((d.NX + 127) / 128, d.NZ), 128, 0, s>>>(d, cst, iy);
}

void launch_deposit(cudaStream_t s, const Dims &d, const int32_t *iy, const DepIn &a, double *dep)
{
    k_deposit<<<dim3((d.NX + 127) / 128, d.NZ, a.nconc), 128, 0, s>>>(d, iy, a, dep);
}
