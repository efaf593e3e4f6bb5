/*
 * turb_oracle.h -- CPU oracle for the TURBINS fractional-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file and turb_oracle.c are a plain-C,
 * single-threaded restatement of the reference's per-step arithmetic.  They
 * are the checker for the CUDA path (tests/, __graft_entry__.smoke()) and the
 * timed CPU baseline in bench.py.  Nothing in the product (turbins_gb300/)
 * links, loads or calls this code.
 *
 * Layout: every 3-D field is a flat double array in the reference's PETSc DA
 * order, a[(k*NY + j)*NX + i] with i fastest, where NX = nx+1, NY = ny+1,
 * NZ = nz+1 (one trailing half cell per direction, Grid.c:57-60).
 * Node status codes are those of Include/definitions.h:93-99.
 */
#ifndef TURB_ORACLE_H
#define TURB_ORACLE_H
#include <stdint.h>

#define TO_OUTSIDE 1
#define TO_SOLID 2
#define TO_FLUID 3
#define TO_IMMERSED 5
#define TO_BOUNDARY 7
#define TO_BUFFER_SOLID 11

#define TO_SALINITY 1
#define TO_PARTICLE 2

#define TO_MAXCONC 4

/* walls: 0 left(x=0) 1 right 2 bottom(y=0) 3 top 4 back(z=0) 5 front */
typedef struct {
    int nx, ny, nz;          /* physical cells (params->NX, NY, NZ)            */
    int eno_order;           /* 1..3 (Input.c:449 default 3)                    */
    double re;               /* Reynolds number                                 */
    int nconc;               /* number of concentration fractions (1..4)        */
    double pe[TO_MAXCONC];   /* Peclet number per fraction                      */
    double vs0[TO_MAXCONC];  /* settling speed after Input.c:481 sign flip      */
    double alpha[TO_MAXCONC];/* buoyancy weight after Input.c:454-483 rescale   */
    int ctype[TO_MAXCONC];   /* TO_SALINITY or TO_PARTICLE                      */
    int sedimentation;       /* params->sedimentation (Robin top ghost)         */
    int wall_noslip[6];      /* velocity walls: 1 no-slip, 0 free-slip          */
    int buoyancy;            /* 1: subtract c_term at v nodes                   */
    double vel_rtol;         /* Helmholtz relative residual (resmax)            */
    int vel_maxit;
    double p_rtol;           /* Poisson relative residual                       */
    int p_maxit;
} to_params;

typedef struct {
    int n;                   /* immersed nodes of this quantity                 */
    int32_t *im;             /* [n] linear DA index of the immersed node        */
    int32_t *nf;             /* [n] number of fluid nodes (1 or 8)              */
    int32_t *fidx;           /* [n*8] linear DA index of each fluid node        */
    double *fcoef;           /* [n*8] fluid_coef                                */
    double *bcoef;           /* [n] boundary_coef                               */
} to_ib;

typedef struct {
    int nx, ny, nz, NX, NY, NZ;
    double dEta, dXi, dPhi;
    double *xc, *yc, *zc, *xu, *yv, *zw;          /* [NX] / [NY] / [NZ]         */
    double *mxc, *myc, *mzc, *mxu, *myv, *mzw;    /* metrics, Grid.c:595-708    */
    uint8_t *st[4];                               /* u, v, w, c status [N]      */
    to_ib ib[4];                                  /* u, v, w, c                 */
} to_grid;

#ifdef __cplusplus
extern "C" {
#endif

void to_grid_metrics(to_grid *g);
void to_eno_line(int order, int n, const double *D0, const double *P,
                 const double *V, double *VdQdX);
void to_cell_center(const to_grid *g, const double *u, const double *v,
                    const double *w, double *ubc, double *vbc, double *wbc);
void to_transpose(const to_grid *g, char which, const double *u,
                  const double *v, const double *w, double *outA, double *outB);
void to_convection_vel(const to_grid *g, const to_params *p, char which,
                       const double *q, const double *velx, const double *vely,
                       const double *velz, double *conv);
void to_convection_conc(const to_grid *g, const to_params *p, int ic,
                        const double *c, const double *ubc, const double *vadv,
                        const double *wbc, double *conv);
void to_total_concentration(const to_grid *g, const to_params *p,
                            const double *const *c, double *ctot);
void to_set_rhs_vel(const to_grid *g, const to_params *p, char which, double dt,
                    const double *q, const double *conv, const double *dp,
                    const double *ctot, double *b);
void to_set_rhs_conc(const to_grid *g, double dt, const double *c,
                     const double *conv, double *b);
void to_helmholtz_apply(const to_grid *g, const to_params *p, char which,
                        int ic, double dt, const double *x, double *y);
int to_helmholtz_solve(const to_grid *g, const to_params *p, char which, int ic,
                       double dt, const double *b, double *x, int method,
                       double *relres);
void to_pressure_rhs(const to_grid *g, double dt, const double *u,
                     const double *v, const double *w, double *b);
void to_pressure_apply(const to_grid *g, const double *x, double *y);
int to_pressure_solve(const to_grid *g, const to_params *p, const double *b,
                      double *phi, double *relres);
void to_project(const to_grid *g, const to_params *p, double dt,
                const double *phi, const double *b, double *u, double *v,
                double *w, double *dpx, double *dpy, double *dpz);
double to_divergence(const to_grid *g, const double *u, const double *v,
                     const double *w, double *div);

typedef struct {
    double *u, *v, *w, *u_old, *v_old, *w_old;
    double *phi, *dpx, *dpy, *dpz, *pb;
    double *c[TO_MAXCONC], *c_old[TO_MAXCONC];
} to_state;

typedef struct {
    int vel_iters[3][2];
    int conc_iters[TO_MAXCONC][2];
    int p_iters[2];
    double p_relres[2];
    double div_max[2];
} to_step_stats;

void to_set_mg_options(int mode, int npre, int npost);
/* Flow diagnostics of one state (cell-centred velocities computed here, as
 * Velocity_cell_center does before the reference's output routines). */
typedef struct {
    double kinetic_energy;                 /* Extract_total_kinetic_energy           */
    double conversion_rate;                /* Extract_kinetic_potential_conversion_rate */
    double suspended_mass[TO_MAXCONC];     /* Conc_compute_total_suspended_mass      */
    double potential_energy[TO_MAXCONC];   /* Conc_compute_potential_energies: W_Ep  */
    double stokes_dissipation[TO_MAXCONC]; /*   ... W_Stokes_dissipation_rate        */
    double conversion_rate_c[TO_MAXCONC];  /*   ... W_kinetic_potential_conversion_rate */
    double front_location;                 /* Conc_find_front_location (-1: none)    */
    double viscous_dissipation;            /* Extract_viscous_dissipation_rate       */
    double ep_passive[TO_MAXCONC];         /* Conc_compute_potential_energies: W_Ep_passive */
    double ep_passive_rate[TO_MAXCONC];    /*   ... W_Ep_passive_rate                */
    double ep_rate[TO_MAXCONC];            /*   ... W_Ep_rate                        */
    double sed_rate[TO_MAXCONC];           /* Conc_compute_sedimentation_rate        */
} to_diag;
/* Grid_set_interface_y_index (Grid.c:1972-2012): per (i, k), iy[k*NX + i] =
 * the first j whose c node is IMMERSED, or 0 when the bottom c node is FLUID,
 * else -1 (NOT_FOUND). */
void to_interface_y_index(const to_grid *g, int32_t *iy);
/* Conc_integrate_deposited_height (Conc.c:1675-1749) for every fraction with
 * weight_factor = alpha_i: dep[ic][k][i] += dt |Vs0| alpha 0.5 (c + c_old)
 * at the bed node (i, iy, k).  dep: nconc x NZ x NX. */
void to_deposit_integrate(const to_grid *g, const to_params *p, const int32_t *iy,
                          const double *const *c, const double *const *c_old,
                          double dt, double *dep);
/* iy: bed index (to_interface_y_index); dep: nconc x NZ x NX deposited
 * heights, or NULL for none; h_ave: nconc x NX spanwise-averaged heights
 * (Conc_compute_ave_height_x) or NULL; sed_bottom: nconc x NZ x NX bed
 * sedimentation rates (Conc_bottom_sed_rate) or NULL. */
void to_diagnostics(const to_grid *g, const to_params *p, const double *u,
                    const double *v, const double *w, const double *const *c,
                    double front_limit, const int32_t *iy, const double *dep,
                    to_diag *out, double *h_ave, double *sed_bottom);

int to_step(const to_grid *g, const to_params *p, to_state *s, double dt,
            to_step_stats *stats);

/* threads of the parallel loops (OpenMP builds; results do not depend on it) */
void to_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
