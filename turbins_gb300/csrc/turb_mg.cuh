// turb_mg.cuh -- multigrid hierarchy descriptors (device pointers).
#pragma once
#include <cuda.h>

#include "turb_internal.cuh"

#define TURB_MG_MAXLEV 24
#define MG_TAIL_MAXLEV 6   // levels a fused single-block V-cycle tail may hold
#define MG_CLUSTER_MAXLEV 8   // levels a one-cluster V-cycle launch may hold

// 1-D transfer tables between a level and the next coarser one along one
// direction: prolongation weights per fine index (two coarse cells) and the
// transposed (restriction) lists per coarse index (up to four fine cells).
struct Xfer1D {
    const int *I0, *I1;
    const double *w0d, *w1d;
    const float *w0f, *w1f;
    const int *rcnt, *rf;
    const double *rwd;
    const float *rwf;
};

struct MgDevLevel {
    int nx, ny, nz;
    int cx, cy, cz;                                   // coarsened into next level
    Xfer1D tx, ty, tz;                                // transfer to the next level
    const double *dxd, *dyd, *dzd, *rfxd, *rfyd, *rfzd;
    const float *dxf, *dyf, *dzf, *rfxf, *rfyf, *rfzf;
    // the x tables split by parity for 4-cell float4 reads (nx even): entry
    // par * nx/2 + m is cell i = 2m + par: dx[i], 1/f of its left face
    // (rfx[i]) and of its right face (rfx[i+1])
    const float *dxpf = nullptr, *rlpf = nullptr, *rrpf = nullptr;
    double pin;
    // colour-split storage (x, b, invd; not r): with nx even, cell c of colour
    // (i+j+k)&1 lives at colour*(n/2) + c/2, so a red-black half sweep reads
    // and writes dense half arrays
    int split = 0;
};

// the finest FP32 level's two-sweeps-per-pass smoother (k_rbtb.cu): TMA
// maps of x (both ping-pong arrays), b and 1/diag, and the launch shape
struct RbTbPlan {
    CUtensorMap mx[2];
    MgDevLevel lev;
    const float *b = nullptr, *invd = nullptr;
    float *xo[2];
    int tiles_x = 0, ntiles = 0, grid = 0;
    int *err = nullptr;
    int ok = 0;
};
int mg_tb_plan(RbTbPlan *p, const MgDevLevel &L0, float *x0, float *x1, const float *b0, const float *invd0, int *err);
void mg_tb_sweeps(cudaStream_t s, const RbTbPlan &p, int in, int c0, int zero_init, int pdl);
size_t mg_tb_smem();

template <typename T>
struct MgHier {
    int nl;
    MgDevLevel lev[TURB_MG_MAXLEV];
    T *x[TURB_MG_MAXLEV], *b[TURB_MG_MAXLEV], *r[TURB_MG_MAXLEV], *invd[TURB_MG_MAXLEV];
    const double *coarse_inv;
    // from this level on (-1: never) the V-cycle runs as one single-block
    // kernel (k_vcycle_tail); it must leave at most MG_TAIL_MAXLEV levels
    int tail_from = -1;
    // 1: FP32 half sweeps after the first of a cycle march along k (k_rbgs4z)
    int marching = 0;
    // 1: the V-cycle's kernels use programmatic dependent launch
    int pdl = 1;
    // from this level on (-1: never) the V-cycle runs as one launch of one
    // thread-block cluster of cluster_ctas blocks (k_vcycle_cluster)
    int cluster_from = -1;
    int cluster_ctas = 0;
    // level 0 (FP32 only): pairs of sweeps in one pass each (k_rbgs_tb), when set
    const RbTbPlan *tb = nullptr;
};

template <typename T>
void mg_setup_invdiag(cudaStream_t s, const MgDevLevel &L, T *invd);
template <typename T>
// level l smooths with pre[l] / post[l] red-black sweeps
void mg_vcycle(cudaStream_t s, const MgHier<T> &H, int l, const int *pre, const int *post);
int mg_vcycle_launches(int nl, const int *pre, const int *post, int tail_from, int cluster_from = -1, int tb0 = 0);
template <typename T>
int mg_cluster_ctas();
template <typename T>
double mg_vcycle_bytes(const MgHier<T> &H, int l, const int *pre, const int *post);

// FP64 CG vector kernels on the compact level-0 layout (k_pcg.cu)
struct PcgScal {
    double bb, rr, rz, zr_old, rz_old, pq, alpha, beta;   // slot order is used by the reductions
};
void pcg_gather(cudaStream_t s, const Dims &d, const MgDevLevel &L0, const double *phi_da, const double *pb_da,
                double *x, double *bw);
void pcg_scatter(cudaStream_t s, const Dims &d, const MgDevLevel &L0, const double *x, double *phi_da);
void pcg_resid(cudaStream_t s, const MgDevLevel &L0, const double *bw, const double *x, double *r, double *part);
void pcg_apply(cudaStream_t s, const MgDevLevel &L0, const double *p, double *q, double *part);
void pcg_dot(cudaStream_t s, long long n, const double *a, const double *b, double *part);
void pcg_dot2(cudaStream_t s, long long n, const double *r, const double *z, const double *rold, double *part);
void pcg_reduce(cudaStream_t s, const double *part, int nvals, double *dst, int nper = 0);
int pcg_stencil_parts(const MgDevLevel &L);
void pcg_pupdate(cudaStream_t s, long long n, const double *z, double *p, const PcgScal *sc, int first);
void pcg_xrupdate(cudaStream_t s, long long n, double *x, double *r, double *rold, const double *p,
                  const double *q, const PcgScal *sc, double *part);
void pcg_scalars(cudaStream_t s, PcgScal *sc, int what);
void pcg_to_float(cudaStream_t s, long long n, const double *a, float *b);
void pcg_to_double(cudaStream_t s, long long n, const float *a, double *b);
// the same into / out of a level's storage order (colour-split or not)
void mg_to_float(cudaStream_t s, const MgDevLevel &L, const double *a, float *b);
void mg_to_double(cudaStream_t s, const MgDevLevel &L, const float *a, double *b, int pdl = 0);
void pcg_copy(cudaStream_t s, long long n, const double *a, double *b);
int pcg_nparts();
void pcg_lincomb(cudaStream_t s, long long n, double a, const double *x, double b, const double *y, double *out);

// Galerkin fit of the initial guess (k_pcg.cu): up to GAL_MAX candidate
// solutions y_m, each with w_m = the right-hand side it solved (resid 0) or
// its computed residual (resid 1)
#define GAL_MAX 3
struct GalDirs {
    const double *y[GAL_MAX];
    const double *w[GAL_MAX];
    int resid[GAL_MAX];
    int nd;
};
struct GalCoef {
    double a[GAL_MAX];
};
// dst[a * GAL_MAX + b] = d_a . s_b, dst[GAL_MAX^2 + a] = d_a . r1 (part: >= 12 * 512 doubles)
void pcg_gal_dots(cudaStream_t s, long long n, const GalDirs &dd, const double *x0, const double *r1,
                  const double *bw, double *part, double *dst);
void pcg_gal_update(cudaStream_t s, long long n, const GalDirs &dd, const GalCoef &al, const double *x0, double *x);
// *dst = max_c |r_c| / (dx dy dz)_c on level 0 (part: >= pcg_stencil_parts(L0) doubles)
void pcg_rmax(cudaStream_t s, const MgDevLevel &L0, const double *r, double *part, double *dst);
