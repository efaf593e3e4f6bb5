// turb_kernels.cuh -- launcher declarations shared by the host API.
#pragma once
#include "turb_internal.cuh"

struct TransW {       // bilinear weight tables of the transposed velocities
    W2 xu, xc, yc, yv, zc, zw;
};
struct ConcPtrs {
    const double *p[4];
};
struct ConcW {
    double v[4];
};
struct ProjArgs {
    const uint8_t *su, *sv, *sw;
    const double *mxu, *cyv, *czw;
    double a_dEta, dt, coef;
};

// element-wise / stencil kernels (k_stencil.cu)
void launch_cell_center(cudaStream_t s, const Dims &d, Interp2 ix, Interp2 iy, Interp2 iz, const OpenBC &ob,
                        const double *u, const double *v, const double *w, double *ubc, double *vbc, double *wbc);
void launch_transpose(cudaStream_t s, const Dims &d, int which, const uint8_t *st, TransW tw, const OpenBC &ob,
                      const double *u, const double *v, const double *w, double *A, double *B);
void launch_total_conc(cudaStream_t s, long long n, int nc, ConcPtrs c, ConcW a, double *ct);
void launch_shift(cudaStream_t s, long long n, const double *x, double sh, double *y);
void launch_rhs_vel(cudaStream_t s, const Dims &d, int q, const uint8_t *st, double a_dt, const double *x,
                    const double *conv, const double *dp, const double *ct, int buoy, Interp2 iyv,
                    const OpenBC &ob, double *b);
void launch_rhs_conc(cudaStream_t s, const Dims &d, int ic, const uint8_t *st, double a_dt, const double *c,
                     const double *conv, const OpenBC &ob, double *b);
void launch_pressure_rhs(cudaStream_t s, const Dims &d, const uint8_t *st, const double *cx, const double *cy,
                         const double *cz, double a_dt, const OpenBC &ob, const double *u, const double *v,
                         const double *w, double *b);
void launch_project(cudaStream_t s, const Dims &d, ProjArgs a, const double *phi, const double *pb, double *u,
                    double *v, double *w, double *dpx, double *dpy, double *dpz);
long long divergence_parts(const Dims &d);
void launch_divergence(cudaStream_t s, const Dims &d, const uint8_t *st, const double *mxc, const double *myc,
                       const double *mzc, double a_dEta, double a_dXi, double a_dPhi, const OpenBC &ob,
                       const double *u, const double *v, const double *w, double *div, double *part, double *out);
void launch_axpby(cudaStream_t s, long long n, double a, const double *x, double b, double *y);

// ENO convection (k_eno.cu)
// Advecting-velocity source of one (quantity, direction) pass.
struct AdvSrc {
    int kind;               // 0: a[p]; 1: a[p]+shift; 2..7: bilinear transposes
    const double *a;        // primary array
    double shift;
    W2 wx, wy;              // weights of the bilinear transposes
    // u at v (kind 4) / w (kind 6) nodes next to open faces: the inflow and
    // outflow planes replace u at i = 0 / i = nx ([NZ][NY], null when closed)
    const double *pin = nullptr, *pout = nullptr;
    int pNY = 0, nx = 0;
};
void launch_eno_pass(cudaStream_t s, const Dims &d, int dir, const EnoTab &tab, const double *q, AdvSrc adv,
                     int t1a, int t1b, int t2a, int t2b, int first, double *conv, int segments = 0);
int launch_eno_line(int order, int n, const double *D0, const double *P, const double *V, double *out,
                    cudaStream_t s);

// solvers (k_solve.cu)
void launch_helm_apply(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                       const double *x, double *y, const IbDev &ib);
void launch_helm_jacobi(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                        const double *b, const double *x, double *xn, const IbDev &ib, double *part,
                        long long nparts);
long long helm_parts(const Dims &d);
void launch_add_corr(cudaStream_t s, long long n, const double *x, const float *e, double *xn);
void launch_helm_resid64(cudaStream_t s, const Dims &d, const HelmTab &h, const uint8_t *st, double a_dt,
                         const double *b, const double *x, float *rf, const IbDev &ib, double *part,
                         long long nparts);
void launch_helm_jac32(cudaStream_t s, const Dims &d, const HelmTabF &h, const uint8_t *st, float a_dt,
                       const float *r, const float *e, float *en, const IbDevF &ib, int first, int marching);
void launch_sum_final(cudaStream_t s, long long nparts, const double *part, double *out);
void launch_norm2(cudaStream_t s, long long n, const double *x, double *part, long long nparts, double *out);
long long norm_parts();
