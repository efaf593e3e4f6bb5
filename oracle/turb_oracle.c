/*
 * turb_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the TURBINS
 * fractional-step hot path: a plain-C restatement of the reference
 * arithmetic, cited routine by routine.  Used by tests/ as the checker of the
 * CUDA path and by bench.py as the timed CPU baseline ("kind": "port").  The
 * product never links or calls it.
 *
 * Build with -O2 -ffp-contract=off (no fused multiply-add, no fast-math) so
 * that every rounding matches the reference's own C compiled the same way.
 * With OpenMP, loops whose iterations write disjoint outputs run on
 * to_set_threads() threads (default 1); every sum stays serial, so results
 * are the same bits for any thread count.
 */
#include "turb_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif
#include <math.h>
#include <stdlib.h>
#include <string.h>

void to_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

#define IDX(g, i, j, k) (((size_t)(k) * (g)->NY + (size_t)(j)) * (g)->NX + (size_t)(i))
#define NPTS(g) ((size_t)(g)->NX * (g)->NY * (g)->NZ)

static int sti(const to_grid *g, int q, int i, int j, int k)
{
    /* Grid_get_{u,v,w,c}_status, Grid.c:1126-1224: OUTSIDE beyond the box */
    if (i < 0 || j < 0 || k < 0 || i > g->nx || j > g->ny || k > g->nz) return TO_OUTSIDE;
    return g->st[q][IDX(g, i, j, k)];
}

/* Grid_compute_metric_coefficients, Grid.c:595-708 (incl. the metric_zc quirk
 * at Grid.c:693 that divides by zc spacing, not zw spacing). */
void to_grid_metrics(to_grid *g)
{
    int NX = g->NX, NY = g->NY, NZ = g->NZ, i;
    g->dEta = 1.0 / (double)g->nx;
    g->dXi = 1.0 / (double)g->ny;
    g->dPhi = 1.0 / (double)g->nz;
    for (i = 1; i < NX - 1; i++) g->mxu[i] = g->dEta / (g->xc[i] - g->xc[i - 1]);
    g->mxu[0] = 0.5 * g->dEta / (g->xc[0] - g->xu[0]);
    g->mxu[NX - 1] = 0.5 * g->dEta / (g->xu[NX - 1] - g->xc[NX - 2]);
    for (i = 1; i < NY - 1; i++) g->myv[i] = g->dXi / (g->yc[i] - g->yc[i - 1]);
    g->myv[0] = 0.5 * g->dXi / (g->yc[0] - g->yv[0]);
    g->myv[NY - 1] = 0.5 * g->dXi / (g->yv[NY - 1] - g->yc[NY - 2]);
    for (i = 1; i < NZ - 1; i++) g->mzw[i] = g->dPhi / (g->zc[i] - g->zc[i - 1]);
    g->mzw[0] = 0.5 * g->dPhi / (g->zc[0] - g->zw[0]);
    g->mzw[NZ - 1] = 0.5 * g->dPhi / (g->zw[NZ - 1] - g->zc[NZ - 2]);
    for (i = 0; i < NX - 1; i++) g->mxc[i] = g->dEta / (g->xu[i + 1] - g->xu[i]);
    g->mxc[NX - 1] = g->dEta / (g->xc[NX - 1] - g->xc[NX - 2]);
    for (i = 0; i < NY - 1; i++) g->myc[i] = g->dXi / (g->yv[i + 1] - g->yv[i]);
    g->myc[NY - 1] = g->dXi / (g->yc[NY - 1] - g->yc[NY - 2]);
    for (i = 0; i < NZ - 1; i++) g->mzc[i] = g->dPhi / (g->zc[i + 1] - g->zc[i]);
    g->mzc[NZ - 1] = g->dPhi / (g->zc[NZ - 1] - g->zc[NZ - 2]);
}

/* ENO_compute_convective_terms, ENO.c:103-245.  Buffers of length n; the
 * first and last `order` entries are ghosts. */
void to_eno_line(int order, int n, const double *D0, const double *P,
                 const double *V, double *VdQdX)
{
    double *D1 = (double *)calloc((size_t)n, sizeof(double));
    double *D2 = (double *)calloc((size_t)n, sizeof(double));
    double *D3 = (double *)calloc((size_t)n, sizeof(double));
    int i, k, kstar = 0;
    for (i = 0; i < n - 1; i++) D1[i] = (D0[i + 1] - D0[i]) / (P[i + 1] - P[i]);
    if (order > 1)
        for (i = 1; i < n - 1; i++) D2[i] = (D1[i] - D1[i - 1]) / (P[i + 1] - P[i - 1]);
    if (order > 2)
        for (i = 1; i < n - 2; i++) D3[i] = (D2[i + 1] - D2[i]) / (P[i + 2] - P[i - 1]);
    for (i = order; i < n - order; i++) {
        double dQ, c, cs;
        k = (V[i] > 0.0) ? i - 1 : i;
        dQ = D1[k];
        if (order > 1) {
            if (fabs(D2[k]) <= fabs(D2[k + 1])) { c = D2[k]; kstar = k - 1; }
            else { c = D2[k + 1]; kstar = k; }
            dQ += c * ((P[i] - P[k]) + (P[i] - P[k + 1]));
        }
        if (order > 2) {
            double xi = P[i], a = P[kstar], b = P[kstar + 1], d = P[kstar + 2];
            cs = (fabs(D3[kstar]) <= fabs(D3[kstar + 1])) ? D3[kstar] : D3[kstar + 1];
            dQ += cs * ((xi - a) * (xi - b) + (xi - b) * (xi - d) + (xi - a) * (xi - d));
        }
        VdQdX[i] = V[i] * dQ;
    }
    free(D1); free(D2); free(D3);
}

/* MyMath_interpolate_quantity, MyMath.c:13-77, two-point branch */
static double interp2(double q0, double q1, double x0, double x1, double x)
{
    double m = (q1 - q0) / (x1 - x0);
    if (fabs(x1 - x0) < 1.0e-8) return q0;
    return m * (x - x0) + q0;
}

/* MyMath_interpolate_quantity, four-point branch (weights as written there) */
static double interp4(double q0, double q1, double q2, double q3, double X10,
                      double X11, double X20, double X22, double xq, double yq)
{
    double a_Dx = 1.0 / (X11 - X10);
    double Wp0 = fabs((xq - X10) * a_Dx);
    double Wp1 = 1.0 - Wp0;
    double qt = Wp0 * q2 + Wp1 * q3;
    double qb = Wp0 * q0 + Wp1 * q1;
    double a_Dy = 1.0 / (X22 - X20);
    double Wp2;
    Wp0 = fabs((yq - X20) * a_Dy);
    Wp2 = 1.0 - Wp0;
    return Wp0 * qb + Wp2 * qt;
}

/* Velocity_cell_center, Velocity.c:1476-1602 (inflow/outflow off) */
void to_cell_center(const to_grid *g, const double *u, const double *v,
                    const double *w, double *ubc, double *vbc, double *wbc)
{
    int i, j, k;
#pragma omp parallel for private(i, j) schedule(static)
    for (k = 0; k < g->nz; k++)
        for (j = 0; j < g->ny; j++)
            for (i = 0; i < g->nx; i++) {
                size_t p = IDX(g, i, j, k);
                ubc[p] = interp2(u[p], u[IDX(g, i + 1, j, k)], g->xu[i], g->xu[i + 1], g->xc[i]);
                vbc[p] = interp2(v[p], v[IDX(g, i, j + 1, k)], g->yv[j], g->yv[j + 1], g->yc[j]);
                wbc[p] = interp2(w[p], w[IDX(g, i, j, k + 1)], g->zw[k], g->zw[k + 1], g->zc[k]);
            }
}

/* Velocity_transpose_velocities, Velocity.c:3341-3663 (inflow/outflow off).
 * which='u': A=v@u, B=w@u; 'v': A=u@v, B=w@v; 'w': A=u@w, B=v@w.  The
 * coordinate aliases of Grid.c:1366-1378 apply: yu=yw=yc, zu=zv=zc, xv=xw=xc. */
void to_transpose(const to_grid *g, char which, const double *u,
                  const double *v, const double *w, double *A, double *B)
{
    int i, j, k, q = (which == 'u') ? 0 : (which == 'v') ? 1 : 2;
    const double *xc = g->xc, *yc = g->yc, *zc = g->zc, *xu = g->xu, *yv = g->yv, *zw = g->zw;
#pragma omp parallel for private(i, j) schedule(static)
    for (k = 0; k < g->NZ; k++)
        for (j = 0; j < g->NY; j++)
            for (i = 0; i < g->NX; i++) {
                size_t p = IDX(g, i, j, k);
                if (g->st[q][p] == TO_BOUNDARY) continue;
                if (which == 'u') {
                    A[p] = interp4(v[IDX(g, i - 1, j, k)], v[p], v[IDX(g, i - 1, j + 1, k)], v[IDX(g, i, j + 1, k)],
                                   xc[i - 1], xc[i], yv[j], yv[j + 1], xu[i], yc[j]);
                    B[p] = interp4(w[IDX(g, i - 1, j, k)], w[p], w[IDX(g, i - 1, j, k + 1)], w[IDX(g, i, j, k + 1)],
                                   xc[i - 1], xc[i], zw[k], zw[k + 1], xu[i], zc[k]);
                } else if (which == 'v') {
                    A[p] = interp4(u[IDX(g, i, j - 1, k)], u[IDX(g, i + 1, j - 1, k)], u[p], u[IDX(g, i + 1, j, k)],
                                   xu[i], xu[i + 1], yc[j - 1], yc[j], xc[i], yv[j]);
                    B[p] = interp4(w[IDX(g, i, j - 1, k)], w[IDX(g, i, j - 1, k + 1)], w[p], w[IDX(g, i, j, k + 1)],
                                   zw[k], zw[k + 1], yc[j - 1], yc[j], zc[k], yv[j]);
                } else {
                    A[p] = interp4(u[IDX(g, i, j, k - 1)], u[IDX(g, i + 1, j, k - 1)], u[p], u[IDX(g, i + 1, j, k)],
                                   xu[i], xu[i + 1], zc[k - 1], zc[k], xc[i], zw[k]);
                    B[p] = interp4(v[IDX(g, i, j, k - 1)], v[p], v[IDX(g, i, j + 1, k - 1)], v[IDX(g, i, j + 1, k)],
                                   zc[k - 1], zc[k], yv[j], yv[j + 1], zw[k], yc[j]);
                }
            }
}

/* ---------------------------------------------------------------------------
 * ENO line driver.  The reference ships no driver (the caller of
 * ENO_compute_convective_terms is absent); this is the restated one.  Each
 * full box line of non-BOUNDARY nodes is gathered into the buffer layout of
 * Velocity.c:2170/2243/2302 (interior node m at index m-start+order), its
 * ghosts are filled by the rules of Velocity_{u,v,w}_ENO_ghost_cells
 * (Velocity.c:2124-2801) and Conc_ENO_ghost_cells (Conc.c:1021-1220), and
 * conv = Vx dq/dx + Vy dq/dy + Vz dq/dz accumulates in x, y, z order.
 * ------------------------------------------------------------------------- */
enum { GH_WALL = 0, GH_MIRROR = 1 };

typedef struct {
    int kind;        /* GH_WALL: node on the wall (normal velocity), GH_MIRROR */
    double wall;     /* wall coordinate                                       */
    double mult;     /* WALL: value of mirrored ghosts = mult*first interior;  */
                     /* MIRROR: ghost = mult * first/last interior value      */
} ghost_rule;

static void fill_ghosts(int order, int n, double *D0, double *P,
                        const ghost_rule *lo, const ghost_rule *hi)
{
    int ex;
    for (ex = 0; ex < order; ex++) {
        int gi = ex;
        if (lo->kind == GH_WALL) {
            int ii = 2 * order - ex - 2;
            if (ex == order - 1) { P[gi] = lo->wall; D0[gi] = 0.0; }
            else { P[gi] = 2.0 * lo->wall - P[ii]; D0[gi] = lo->mult * D0[order]; }
        } else {
            int ii = 2 * order - ex - 1;
            P[gi] = 2.0 * lo->wall - P[ii];
            D0[gi] = lo->mult * D0[order];
        }
    }
    for (ex = 0; ex < order; ex++) {
        int gi = n - ex - 1;
        if (hi->kind == GH_WALL) {
            int ii = n - 2 * order + ex + 1;
            if (ex == order - 1) { P[gi] = hi->wall; D0[gi] = 0.0; }
            else { P[gi] = 2.0 * hi->wall - P[ii]; D0[gi] = hi->mult * D0[n - order - 1]; }
        } else {
            int ii = n - 2 * order + ex;
            P[gi] = 2.0 * hi->wall - P[ii];
            D0[gi] = hi->mult * D0[n - order - 1];
        }
    }
}

/* One direction of convection for a field on lines along `dir`. */
static void conv_dir(const to_grid *g, int order, int dir, const double *q,
                     const double *vel, const double *pos, int s0, int e0,
                     int r1a, int r1b, int r2a, int r2b, ghost_rule lo,
                     ghost_rule hi, double *conv, int first)
{
    int nint = e0 - s0 + 1, n = nint + 2 * order;
#pragma omp parallel
    {
    int a, b, m;
    double *D0 = (double *)malloc(sizeof(double) * n);
    double *P = (double *)malloc(sizeof(double) * n);
    double *V = (double *)calloc((size_t)n, sizeof(double));
    double *O = (double *)calloc((size_t)n, sizeof(double));
#pragma omp for schedule(static)
    for (b = r2a; b <= r2b; b++)
        for (a = r1a; a <= r1b; a++) {
            for (m = s0; m <= e0; m++) {
                size_t p = dir == 0 ? IDX(g, m, a, b) : dir == 1 ? IDX(g, a, m, b) : IDX(g, a, b, m);
                D0[m - s0 + order] = q[p];
                V[m - s0 + order] = vel[p];
                P[m - s0 + order] = pos[m];
            }
            fill_ghosts(order, n, D0, P, &lo, &hi);
            to_eno_line(order, n, D0, P, V, O);
            for (m = s0; m <= e0; m++) {
                size_t p = dir == 0 ? IDX(g, m, a, b) : dir == 1 ? IDX(g, a, m, b) : IDX(g, a, b, m);
                if (first) conv[p] = O[m - s0 + order];
                else conv[p] += O[m - s0 + order];
            }
        }
    free(D0); free(P); free(V); free(O);
    }
}

static double slip(int noslip) { return noslip ? -1.0 : 1.0; }

/* Convection of velocity component `which` with advecting velocities
 * velx/vely/velz given at its own nodes (itself along its own direction,
 * transposed components otherwise). */
void to_convection_vel(const to_grid *g, const to_params *p, char which,
                       const double *q, const double *velx, const double *vely,
                       const double *velz, double *conv)
{
    int nx = g->nx, ny = g->ny, nz = g->nz, o = p->eno_order;
    const int *ns = p->wall_noslip;
    ghost_rule lo, hi;
    memset(conv, 0, sizeof(double) * NPTS(g));
    if (which == 'u') {
        /* x: Velocity.c:2174-2236 (u normal to the x walls) */
        lo.kind = GH_WALL; lo.wall = g->xu[0]; lo.mult = -1.0;
        hi.kind = GH_WALL; hi.wall = g->xu[nx]; hi.mult = 0.0;
        conv_dir(g, o, 0, q, velx, g->xu, 1, nx - 1, 0, ny - 1, 0, nz - 1, lo, hi, conv, 1);
        lo.kind = hi.kind = GH_MIRROR;
        lo.wall = g->yv[0]; lo.mult = slip(ns[2]); hi.wall = g->yv[ny]; hi.mult = slip(ns[3]);
        conv_dir(g, o, 1, q, vely, g->yc, 0, ny - 1, 1, nx - 1, 0, nz - 1, lo, hi, conv, 0);
        lo.wall = g->zw[0]; lo.mult = slip(ns[4]); hi.wall = g->zw[nz]; hi.mult = slip(ns[5]);
        conv_dir(g, o, 2, q, velz, g->zc, 0, nz - 1, 1, nx - 1, 0, ny - 1, lo, hi, conv, 0);
    } else if (which == 'v') {
        lo.kind = hi.kind = GH_MIRROR;
        lo.wall = g->xu[0]; lo.mult = slip(ns[0]); hi.wall = g->xu[nx]; hi.mult = slip(ns[1]);
        conv_dir(g, o, 0, q, velx, g->xc, 0, nx - 1, 1, ny - 1, 0, nz - 1, lo, hi, conv, 1);
        /* y: Velocity.c:2448-2494 (v normal to the y walls, zero mirrored ghosts) */
        lo.kind = GH_WALL; lo.wall = g->yv[0]; lo.mult = 0.0;
        hi.kind = GH_WALL; hi.wall = g->yv[ny]; hi.mult = 0.0;
        conv_dir(g, o, 1, q, vely, g->yv, 1, ny - 1, 0, nx - 1, 0, nz - 1, lo, hi, conv, 0);
        lo.kind = hi.kind = GH_MIRROR;
        lo.wall = g->zw[0]; lo.mult = slip(ns[4]); hi.wall = g->zw[nz]; hi.mult = slip(ns[5]);
        conv_dir(g, o, 2, q, velz, g->zc, 0, nz - 1, 0, nx - 1, 1, ny - 1, lo, hi, conv, 0);
    } else {
        lo.kind = hi.kind = GH_MIRROR;
        lo.wall = g->xu[0]; lo.mult = slip(ns[0]); hi.wall = g->xu[nx]; hi.mult = slip(ns[1]);
        conv_dir(g, o, 0, q, velx, g->xc, 0, nx - 1, 0, ny - 1, 1, nz - 1, lo, hi, conv, 1);
        lo.wall = g->yv[0]; lo.mult = slip(ns[2]); hi.wall = g->yv[ny]; hi.mult = slip(ns[3]);
        conv_dir(g, o, 1, q, vely, g->yc, 0, ny - 1, 0, nx - 1, 1, nz - 1, lo, hi, conv, 0);
        /* z: Velocity.c:2745-2790 (w normal to the z walls) */
        lo.kind = GH_WALL; lo.wall = g->zw[0]; lo.mult = 0.0;
        hi.kind = GH_WALL; hi.wall = g->zw[nz]; hi.mult = 0.0;
        conv_dir(g, o, 2, q, velz, g->zw, 1, nz - 1, 0, nx - 1, 0, ny - 1, lo, hi, conv, 0);
    }
}

/* Robin factor of the particle no-flux top ghost, Conc.c:1164-1179 */
static double robin_top(const to_grid *g, const to_params *p, int ic)
{
    double coef = 2.0 / (p->pe[ic] * g->dXi) * g->myv[g->ny];
    double Vs = fabs(p->vs0[ic]);
    return (coef - Vs) / (coef + Vs);
}

/* Convection of concentration fraction ic: Conc_ENO_ghost_cells rules.  The
 * top ghosts of a SALINITY field (never written by the reference, Conc.c:1164)
 * take the Neumann value here. */
void to_convection_conc(const to_grid *g, const to_params *p, int ic,
                        const double *c, const double *ubc, const double *vadv,
                        const double *wbc, double *conv)
{
    int nx = g->nx, ny = g->ny, nz = g->nz, o = p->eno_order;
    ghost_rule lo, hi;
    memset(conv, 0, sizeof(double) * NPTS(g));
    lo.kind = hi.kind = GH_MIRROR; lo.mult = hi.mult = 1.0;
    lo.wall = g->xu[0]; hi.wall = g->xu[nx];
    conv_dir(g, o, 0, c, ubc, g->xc, 0, nx - 1, 0, ny - 1, 0, nz - 1, lo, hi, conv, 1);
    lo.wall = g->yv[0]; hi.wall = g->yv[ny];
    hi.mult = (p->ctype[ic] == TO_PARTICLE && p->sedimentation) ? robin_top(g, p, ic) : 1.0;
    conv_dir(g, o, 1, c, vadv, g->yc, 0, ny - 1, 0, nx - 1, 0, nz - 1, lo, hi, conv, 0);
    lo.wall = g->zw[0]; hi.wall = g->zw[nz]; hi.mult = 1.0;
    conv_dir(g, o, 2, c, wbc, g->zc, 0, nz - 1, 0, nx - 1, 0, ny - 1, lo, hi, conv, 0);
}

/* Conc_compute_total_concentration, Conc.c:1291-1314 (VecCopy, VecScale, VecAXPY) */
void to_total_concentration(const to_grid *g, const to_params *p,
                            const double *const *c, double *ctot)
{
    size_t n = NPTS(g), q;
    int ic;
    for (q = 0; q < n; q++) ctot[q] = c[0][q] * p->alpha[0];
    for (ic = 1; ic < p->nconc; ic++)
        for (q = 0; q < n; q++) ctot[q] = ctot[q] + p->alpha[ic] * c[ic][q];
}

/* Velocity_{u,v,w}_set_RHS, Velocity.c:1607-2043.  For v the buoyancy term
 * -c_term (Velocity.c:1861-1883, shipped as -0.0*c_term) is applied when
 * p->buoyancy is set; ctot is the total concentration (c[0] if one field). */
void to_set_rhs_vel(const to_grid *g, const to_params *p, char which, double dt,
                    const double *q, const double *conv, const double *dp,
                    const double *ctot, double *b)
{
    int qi = (which == 'u') ? 0 : (which == 'v') ? 1 : 2, i, j, k;
    double a_dt = 1.0 / dt;
    for (k = 0; k < g->NZ; k++)
        for (j = 0; j < g->NY; j++)
            for (i = 0; i < g->NX; i++) {
                size_t pp = IDX(g, i, j, k);
                int s = g->st[qi][pp];
                double r = 0.0;
                if (s == TO_FLUID || s == TO_BUFFER_SOLID) {
                    r = q[pp] * a_dt - conv[pp] - dp[pp];
                    if (qi == 1 && p->buoyancy) {
                        double ct = interp2(ctot[IDX(g, i, j - 1, k)], ctot[pp], g->yc[j - 1], g->yc[j], g->yv[j]);
                        r = r - ct;
                    }
                }
                b[pp] = r;
            }
}

/* Conc_set_RHS, Conc.c:864-992 (inflow/outflow off) */
void to_set_rhs_conc(const to_grid *g, double dt, const double *c,
                     const double *conv, double *b)
{
    size_t n = NPTS(g), q;
    double a_dt = 1.0 / dt;
    for (q = 0; q < n; q++)
        b[q] = (g->st[3][q] == TO_FLUID) ? c[q] * a_dt - conv[q] : 0.0;
}

/* ---------------------------------------------------------------------------
 * Helmholtz operators: rows of Velocity_{u,v,w}_form_LHS_matrix
 * (Velocity.c:449-1474) and Conc_form_LHS_matrix (Conc.c:390-730) with the
 * +1/dt of Velocity_modify_diagonal / Conc_modify_diagonal (Velocity.c:374-443,
 * Conc.c:293-354) on every non-IMMERSED row, applied matrix-free.
 * ------------------------------------------------------------------------- */
typedef struct {
    double ap, aw, ae, as, an, ab, af;  /* after wall adjustments          */
    int uw, ue, us, un, ub, uf;         /* neighbour present in the row     */
} row7;

static void vel_row(const to_grid *g, const to_params *p, int q, int i, int j,
                    int k, row7 *r)
{
    double Re = p->re;
    double Cx = -1.0 / (Re * g->dEta * g->dEta), Cy = -1.0 / (Re * g->dXi * g->dXi),
           Cz = -1.0 / (Re * g->dPhi * g->dPhi);
    double px, py, pz, ex, wx, ny_, sy, bz, fz;
    const int *ns = p->wall_noslip;
    if (q == 0) {
        px = g->mxu[i]; py = g->myc[j]; pz = g->mzc[k];
        ex = g->mxc[i]; wx = g->mxc[i - 1]; ny_ = g->myv[j + 1]; sy = g->myv[j];
        bz = g->mzw[k]; fz = g->mzw[k + 1];
    } else if (q == 1) {
        px = g->mxc[i]; py = g->myv[j]; pz = g->mzc[k];
        ex = g->mxu[i + 1]; wx = g->mxu[i]; ny_ = g->myc[j]; sy = g->myc[j - 1];
        bz = g->mzw[k]; fz = g->mzw[k + 1];
    } else {
        px = g->mxc[i]; py = g->myc[j]; pz = g->mzw[k];
        ex = g->mxu[i + 1]; wx = g->mxu[i]; ny_ = g->myv[j + 1]; sy = g->myv[j];
        bz = g->mzc[k - 1]; fz = g->mzc[k];
    }
    r->ap = -Cx * px * (ex + wx) - Cy * py * (ny_ + sy) - Cz * pz * (bz + fz);
    r->aw = Cx * px * wx; r->ae = Cx * px * ex;
    r->an = Cy * py * ny_; r->as = Cy * py * sy;
    r->ab = Cz * pz * bz; r->af = Cz * pz * fz;
    r->uw = r->ue = r->us = r->un = r->ub = r->uf = 1;
    /* x neighbours */
    if (q == 0) {
        r->uw = sti(g, 0, i - 1, j, k) != TO_BOUNDARY;
        r->ue = sti(g, 0, i + 1, j, k) != TO_BOUNDARY;
    } else {
        if (i == 0) { r->uw = 0; r->ap += ns[0] ? -r->aw : r->aw; }
        if (i == g->nx - 1) { r->ue = 0; r->ap += ns[1] ? -r->ae : r->ae; }
    }
    /* y neighbours */
    if (q == 1) {
        r->us = sti(g, 1, i, j - 1, k) != TO_BOUNDARY;
        r->un = sti(g, 1, i, j + 1, k) != TO_BOUNDARY;
    } else {
        if (j == 0) { r->us = 0; r->ap += ns[2] ? -r->as : r->as; }
        if (j == g->ny - 1) { r->un = 0; r->ap += ns[3] ? -r->an : r->an; }
    }
    /* z neighbours */
    if (q == 2) {
        r->ub = sti(g, 2, i, j, k - 1) != TO_BOUNDARY;
        r->uf = sti(g, 2, i, j, k + 1) != TO_BOUNDARY;
    } else {
        if (k == 0) { r->ub = 0; r->ap += ns[4] ? -r->ab : r->ab; }
        if (k == g->nz - 1) { r->uf = 0; r->ap += ns[5] ? -r->af : r->af; }
    }
}

static void conc_row(const to_grid *g, const to_params *p, int ic, int i, int j,
                     int k, row7 *r)
{
    double Pe = p->pe[ic];
    double Cx = -1.0 / (Pe * g->dEta * g->dEta), Cy = -1.0 / (Pe * g->dXi * g->dXi),
           Cz = -1.0 / (Pe * g->dPhi * g->dPhi);
    double px = g->mxc[i], py = g->myc[j], pz = g->mzc[k];
    double ex = g->mxu[i + 1], wx = g->mxu[i], ny_ = g->myv[j + 1], sy = g->myv[j];
    double bz = g->mzw[k], fz = g->mzw[k + 1];
    r->ap = -Cx * px * (ex + wx) - Cy * py * (ny_ + sy) - Cz * pz * (bz + fz);
    r->aw = Cx * px * wx; r->ae = Cx * px * ex;
    r->an = Cy * py * ny_; r->as = Cy * py * sy;
    r->ab = Cz * pz * bz; r->af = Cz * pz * fz;
    r->uw = r->ue = r->us = r->un = r->ub = r->uf = 1;
    if (k == 0) { r->ub = 0; r->ap += r->ab; }
    if (j == 0) { r->us = 0; r->ap += r->as; }
    if (i == 0) { r->uw = 0; r->ap += r->aw; }
    if (i == g->nx - 1) { r->ue = 0; r->ap += r->ae; }
    if (j == g->ny - 1) {
        double coef = r->an;
        r->un = 0;
        if (p->ctype[ic] == TO_PARTICLE) {
            /* Conc.c:623-628 */
            double b = 2.0 / (Pe * g->dXi) * ny_;
            coef = r->an * (b - fabs(p->vs0[ic])) / (b + fabs(p->vs0[ic]));
        }
        r->ap += coef;
    }
    if (k == g->nz - 1) { r->uf = 0; r->ap += r->af; }
}

static double ap_solid_of(const to_grid *g, double coefRe)
{
    double Cx = -1.0 / (coefRe * g->dEta * g->dEta), Cy = -1.0 / (coefRe * g->dXi * g->dXi),
           Cz = -1.0 / (coefRe * g->dPhi * g->dPhi);
    return -Cx * g->mxc[0] - Cy * g->myc[0] - Cz * g->mzc[0];
}

/* Immersed rows: ap_solid * (x_im*(1+sum self coef) + sum_{|coef|>=1e-8} coef x_g),
 * Velocity.c:718-773, Conc.c:666-721 (LSYS_DROP_TOLERANCE definitions.h:152). */
static void ib_rows_apply(const to_grid *g, int q, double aps, const double *x, double *y)
{
    const to_ib *ib = &g->ib[q];
    int n, t;
    for (n = 0; n < ib->n; n++) {
        double dg = 1.0, acc;
        size_t im = (size_t)ib->im[n];
        for (t = 0; t < ib->nf[n]; t++)
            if ((size_t)ib->fidx[n * 8 + t] == im) dg += ib->fcoef[n * 8 + t];
        acc = aps * dg * x[im];
        for (t = 0; t < ib->nf[n]; t++) {
            size_t f = (size_t)ib->fidx[n * 8 + t];
            double cf = ib->fcoef[n * 8 + t];
            if (f != im && fabs(cf) >= 1.0e-8) acc += aps * cf * x[f];
        }
        y[im] = acc;
    }
}

static double ib_diag(const to_grid *g, int q, double aps, size_t im)
{
    const to_ib *ib = &g->ib[q];
    int n, t;
    for (n = 0; n < ib->n; n++)
        if ((size_t)ib->im[n] == im) {
            double dg = 1.0;
            for (t = 0; t < ib->nf[n]; t++)
                if ((size_t)ib->fidx[n * 8 + t] == im) dg += ib->fcoef[n * 8 + t];
            return aps * dg;
        }
    return aps;
}

static int is_stencil_row(int q, int s)
{
    return q == 3 ? (s == TO_FLUID) : (s == TO_FLUID || s == TO_BUFFER_SOLID);
}

void to_helmholtz_apply(const to_grid *g, const to_params *p, char which,
                        int ic, double dt, const double *x, double *y)
{
    int q = which == 'u' ? 0 : which == 'v' ? 1 : which == 'w' ? 2 : 3, i, j, k;
    double a_dt = 1.0 / dt;
    double aps = ap_solid_of(g, q == 3 ? p->pe[ic] : p->re);
    size_t NX = g->NX, NXY = (size_t)g->NX * g->NY;
#pragma omp parallel for private(i, j) schedule(static)
    for (k = 0; k < g->NZ; k++)
        for (j = 0; j < g->NY; j++)
            for (i = 0; i < g->NX; i++) {
                size_t pp = IDX(g, i, j, k);
                int s = g->st[q][pp];
                if (is_stencil_row(q, s)) {
                    row7 r;
                    double acc;
                    if (q == 3) conc_row(g, p, ic, i, j, k, &r);
                    else vel_row(g, p, q, i, j, k, &r);
                    acc = (r.ap + a_dt) * x[pp];
                    if (r.uw) acc += r.aw * x[pp - 1];
                    if (r.ue) acc += r.ae * x[pp + 1];
                    if (r.us) acc += r.as * x[pp - NX];
                    if (r.un) acc += r.an * x[pp + NX];
                    if (r.ub) acc += r.ab * x[pp - NXY];
                    if (r.uf) acc += r.af * x[pp + NXY];
                    y[pp] = acc;
                } else if (s != TO_IMMERSED) {
                    y[pp] = (aps + a_dt) * x[pp];
                }
            }
    ib_rows_apply(g, q, aps, x, y);
}

/* dot product summed in 64 fixed chunks (each serially, then the chunk sums
 * in order): the same bits for any thread count */
#define DOT_CHUNKS 64
static double dot(size_t n, const double *a, const double *b)
{
    double part[DOT_CHUNKS], s = 0.0;
    int c;
#pragma omp parallel for schedule(static)
    for (c = 0; c < DOT_CHUNKS; c++) {
        size_t i, lo = n * (size_t)c / DOT_CHUNKS, hi = n * (size_t)(c + 1) / DOT_CHUNKS;
        double t = 0.0;
        for (i = lo; i < hi; i++) t += a[i] * b[i];
        part[c] = t;
    }
    for (c = 0; c < DOT_CHUNKS; c++) s += part[c];
    return s;
}

/* KSPIBCGS with PCNONE (Solver.c:269-322, 39-86) is BiCGStab without a
 * preconditioner, nonzero initial guess, ||r|| <= rtol ||b|| (method 0).
 * method 1 is point-Jacobi iteration to the same test (the GPU algorithm). */
int to_helmholtz_solve(const to_grid *g, const to_params *p, char which, int ic,
                       double dt, const double *b, double *x, int method,
                       double *relres)
{
    size_t n = NPTS(g), t;
    int it = 0, q = which == 'u' ? 0 : which == 'v' ? 1 : which == 'w' ? 2 : 3;
    double *r = (double *)malloc(n * sizeof(double));
    double nb = sqrt(dot(n, b, b)), nr;
    to_helmholtz_apply(g, p, which, ic, dt, x, r);
    for (t = 0; t < n; t++) r[t] = b[t] - r[t];
    nr = sqrt(dot(n, r, r));
    if (method == 1) {
        double *dg = (double *)malloc(n * sizeof(double));
        double *e = (double *)calloc(n, sizeof(double));
        /* diagonal via unit probing of the row formula */
        {
            int i, j, k;
            double a_dt = 1.0 / dt, aps = ap_solid_of(g, q == 3 ? p->pe[ic] : p->re);
            for (k = 0; k < g->NZ; k++)
                for (j = 0; j < g->NY; j++)
                    for (i = 0; i < g->NX; i++) {
                        size_t pp = IDX(g, i, j, k);
                        int s = g->st[q][pp];
                        row7 rr;
                        if (is_stencil_row(q, s)) {
                            if (q == 3) conc_row(g, p, ic, i, j, k, &rr);
                            else vel_row(g, p, q, i, j, k, &rr);
                            dg[pp] = rr.ap + a_dt;
                        } else if (s == TO_IMMERSED) dg[pp] = ib_diag(g, q, aps, pp);
                        else dg[pp] = aps + a_dt;
                    }
        }
        while (nr > p->vel_rtol * nb && it < p->vel_maxit) {
            for (t = 0; t < n; t++) x[t] += r[t] / dg[t];
            it++;
            to_helmholtz_apply(g, p, which, ic, dt, x, r);
            for (t = 0; t < n; t++) r[t] = b[t] - r[t];
            nr = sqrt(dot(n, r, r));
        }
        free(dg); free(e);
    } else {
        double *rh = (double *)malloc(n * sizeof(double)), *pv = (double *)calloc(n, sizeof(double));
        double *v = (double *)calloc(n, sizeof(double)), *s = (double *)malloc(n * sizeof(double));
        double *tv = (double *)malloc(n * sizeof(double));
        double rho = 1.0, alpha = 1.0, omega = 1.0;
        memcpy(rh, r, n * sizeof(double));
        while (nr > p->vel_rtol * nb && it < p->vel_maxit) {
            double rho1 = dot(n, rh, r), beta;
            if (rho1 == 0.0) break;
            beta = (rho1 / rho) * (alpha / omega);
#pragma omp parallel for schedule(static)
            for (t = 0; t < n; t++) pv[t] = r[t] + beta * (pv[t] - omega * v[t]);
            to_helmholtz_apply(g, p, which, ic, dt, pv, v);
            alpha = rho1 / dot(n, rh, v);
#pragma omp parallel for schedule(static)
            for (t = 0; t < n; t++) s[t] = r[t] - alpha * v[t];
            to_helmholtz_apply(g, p, which, ic, dt, s, tv);
            {
                double tt = dot(n, tv, tv);
                omega = tt > 0.0 ? dot(n, tv, s) / tt : 0.0;
            }
#pragma omp parallel for schedule(static)
            for (t = 0; t < n; t++) {
                x[t] += alpha * pv[t] + omega * s[t];
                r[t] = s[t] - omega * tv[t];
            }
            rho = rho1;
            nr = sqrt(dot(n, r, r));
            it++;
            if (omega == 0.0) break;
        }
        free(rh); free(pv); free(v); free(s); free(tv);
    }
    if (relres) *relres = nb > 0.0 ? nr / nb : 0.0;
    free(r);
    return it;
}

/* Pressure_set_RHS, Pressure.c:171-276 (inflow/outflow off) */
void to_pressure_rhs(const to_grid *g, double dt, const double *u,
                     const double *v, const double *w, double *b)
{
    int i, j, k;
    double a_dEta = 1.0 / g->dEta, a_dXi = 1.0 / g->dXi, a_dPhi = 1.0 / g->dPhi, a_dt = 1.0 / dt;
    for (k = 0; k < g->NZ; k++) {
        double Cz = g->mzc[k] * a_dPhi;
        for (j = 0; j < g->NY; j++) {
            double Cy = g->myc[j] * a_dXi;
            for (i = 0; i < g->NX; i++) {
                size_t p = IDX(g, i, j, k);
                double r = 0.0;
                if (g->st[3][p] != TO_BOUNDARY) {
                    double Cx = g->mxc[i] * a_dEta;
                    double dudx = (u[IDX(g, i + 1, j, k)] - u[p]) * Cx;
                    double dvdy = (v[IDX(g, i, j + 1, k)] - v[p]) * Cy;
                    double dwdz = (w[IDX(g, i, j, k + 1)] - w[p]) * Cz;
                    r = -(dudx + dvdy + dwdz) * a_dt;
                }
                b[p] = r;
            }
        }
    }
}

/* Pressure_form_LHS_matrix, Pressure.c:691-936, applied matrix-free: metric
 * 7-point -Laplacian, Neumann walls folded into ap, east term of the corner
 * cell (NI-1,NJ-1,NK-1) kept (the pin, Pressure.c:864-868), BOUNDARY rows
 * ap_solid.  The pressure system ignores the immersed body (Pressure.c:768). */
void to_pressure_apply(const to_grid *g, const double *x, double *y)
{
    int i, j, k, NI = g->nx, NJ = g->ny, NK = g->nz;
    double Cx = -1.0 / (g->dEta * g->dEta), Cy = -1.0 / (g->dXi * g->dXi), Cz = -1.0 / (g->dPhi * g->dPhi);
    double aps = -Cx * g->mxc[0] - Cy * g->myc[0] - Cz * g->mzc[0];
    size_t NX = g->NX, NXY = (size_t)g->NX * g->NY;
    for (k = 0; k < g->NZ; k++)
        for (j = 0; j < g->NY; j++)
            for (i = 0; i < g->NX; i++) {
                size_t p = IDX(g, i, j, k);
                if (g->st[3][p] != TO_BOUNDARY) {
                    double px = g->mxc[i], py = g->myc[j], pz = g->mzc[k];
                    double ex = g->mxu[i + 1], wx = g->mxu[i], ny_ = g->myv[j + 1], sy = g->myv[j];
                    double fz = g->mzw[k + 1], bz = g->mzw[k];
                    double ap = -Cx * px * (ex + wx) - Cy * py * (ny_ + sy) - Cz * pz * (bz + fz);
                    double aw = Cx * px * wx, ae = Cx * px * ex, an = Cy * py * ny_, as = Cy * py * sy;
                    double ab = Cz * pz * bz, af = Cz * pz * fz, acc = 0.0;
                    if (k > 0) acc += ab * x[p - NXY]; else ap += ab;
                    if (j > 0) acc += as * x[p - NX]; else ap += as;
                    if (i > 0) acc += aw * x[p - 1]; else ap += aw;
                    if (i < NI - 1) acc += ae * x[p + 1];
                    else if (!(i == NI - 1 && j == NJ - 1 && k == NK - 1)) ap += ae;
                    if (j < NJ - 1) acc += an * x[p + NX]; else ap += an;
                    if (k < NK - 1) acc += af * x[p + NXY]; else ap += af;
                    y[p] = acc + ap * x[p];
                } else {
                    y[p] = aps * x[p];
                }
            }
}

/* ---------------------------------------------------------------------------
 * Poisson solve.  hypre BoomerAMG + GMRES(20) (Solver.c:90-265) is not
 * available; the exact discrete solution of the same system is found with
 * geometric-multigrid-preconditioned CG on the volume-weighted (symmetric)
 * form S = W A, W = cell volume, over the physical cells.  BOUNDARY cells
 * solve to 0 (their rows are ap_solid * x = 0).
 * ------------------------------------------------------------------------- */
typedef struct {
    int nx, ny, nz;
    double *DX, *DY, *DZ, *FX, *FY, *FZ;  /* widths [n], face distances [n+1] */
    double pin;
    double *x, *b, *r;
    int cx, cy, cz;                        /* coarsened from this level?      */
    double *chol;                          /* coarsest dense factor           */
} mg_lev;

#define MGMAX 24
typedef struct { int nl; mg_lev L[MGMAX]; } mg_hier;

static size_t LI(const mg_lev *l, int i, int j, int k)
{
    return ((size_t)k * l->ny + j) * l->nx + i;
}

static double fcx(const mg_lev *l, int i, int j, int k) { return l->DY[j] * l->DZ[k] / l->FX[i]; }
static double fcy(const mg_lev *l, int i, int j, int k) { return l->DX[i] * l->DZ[k] / l->FY[j]; }
static double fcz(const mg_lev *l, int i, int j, int k) { return l->DX[i] * l->DY[j] / l->FZ[k]; }

static double mg_diag(const mg_lev *l, int i, int j, int k)
{
    double d = 0.0;
    if (i > 0) d += fcx(l, i, j, k);
    if (i < l->nx - 1) d += fcx(l, i + 1, j, k);
    if (j > 0) d += fcy(l, i, j, k);
    if (j < l->ny - 1) d += fcy(l, i, j + 1, k);
    if (k > 0) d += fcz(l, i, j, k);
    if (k < l->nz - 1) d += fcz(l, i, j, k + 1);
    if (i == l->nx - 1 && j == l->ny - 1 && k == l->nz - 1) d += l->pin;
    return d;
}

static double mg_offsum(const mg_lev *l, const double *x, int i, int j, int k)
{
    double s = 0.0;
    size_t p = LI(l, i, j, k), NX = l->nx, NXY = (size_t)l->nx * l->ny;
    if (i > 0) s += fcx(l, i, j, k) * x[p - 1];
    if (i < l->nx - 1) s += fcx(l, i + 1, j, k) * x[p + 1];
    if (j > 0) s += fcy(l, i, j, k) * x[p - NX];
    if (j < l->ny - 1) s += fcy(l, i, j + 1, k) * x[p + NX];
    if (k > 0) s += fcz(l, i, j, k) * x[p - NXY];
    if (k < l->nz - 1) s += fcz(l, i, j, k + 1) * x[p + NXY];
    return s;
}

static void mg_apply(const mg_lev *l, const double *x, double *y)
{
    int i, j, k;
#pragma omp parallel for private(i, j) schedule(static)
    for (k = 0; k < l->nz; k++)
        for (j = 0; j < l->ny; j++)
            for (i = 0; i < l->nx; i++) {
                size_t p = LI(l, i, j, k);
                y[p] = mg_diag(l, i, j, k) * x[p] - mg_offsum(l, x, i, j, k);
            }
}

static void mg_rbgs(const mg_lev *l, double *x, const double *b, int color)
{
    int i, j, k;
    /* the cells of one colour have no neighbour of that colour: updated in
     * any order (or in parallel) they give the same bits */
#pragma omp parallel for private(i, j) schedule(static)
    for (k = 0; k < l->nz; k++)
        for (j = 0; j < l->ny; j++)
            for (i = ((j + k + color) & 1); i < l->nx; i += 2) {
                size_t p = LI(l, i, j, k);
                x[p] = (b[p] + mg_offsum(l, x, i, j, k)) / mg_diag(l, i, j, k);
            }
}

static double avgw(const double *d, int n)
{
    double s = 0.0;
    int i;
    for (i = 0; i < n; i++) s += d[i];
    return s / n;
}

static void faces_from_widths(const double *D, int n, double *F)
{
    int i;
    F[0] = 0.5 * D[0];
    for (i = 1; i < n; i++) F[i] = 0.5 * (D[i - 1] + D[i]);
    F[n] = 0.5 * D[n - 1];
}

static void mg_build(const to_grid *g, mg_hier *H)
{
    mg_lev *l = &H->L[0];
    int i, lev;
    l->nx = g->nx; l->ny = g->ny; l->nz = g->nz;
    l->DX = malloc(sizeof(double) * l->nx); l->FX = malloc(sizeof(double) * (l->nx + 1));
    l->DY = malloc(sizeof(double) * l->ny); l->FY = malloc(sizeof(double) * (l->ny + 1));
    l->DZ = malloc(sizeof(double) * l->nz); l->FZ = malloc(sizeof(double) * (l->nz + 1));
    for (i = 0; i < l->nx; i++) l->DX[i] = g->dEta / g->mxc[i];
    for (i = 0; i <= l->nx; i++) l->FX[i] = g->dEta / g->mxu[i];
    for (i = 0; i < l->ny; i++) l->DY[i] = g->dXi / g->myc[i];
    for (i = 0; i <= l->ny; i++) l->FY[i] = g->dXi / g->myv[i];
    for (i = 0; i < l->nz; i++) l->DZ[i] = g->dPhi / g->mzc[i];
    for (i = 0; i <= l->nz; i++) l->FZ[i] = g->dPhi / g->mzw[i];
    l->pin = l->DY[l->ny - 1] * l->DZ[l->nz - 1] / l->FX[l->nx];
    for (lev = 0; lev < MGMAX - 1; lev++) {
        mg_lev *f = &H->L[lev], *c = &H->L[lev + 1];
        double hx = avgw(f->DX, f->nx), hy = avgw(f->DY, f->ny), hz = avgw(f->DZ, f->nz);
        double hmin = hx < hy ? (hx < hz ? hx : hz) : (hy < hz ? hy : hz);
        size_t ncell = (size_t)f->nx * f->ny * f->nz;
        f->cx = (f->nx % 2 == 0) && f->nx >= 2 && hx <= 2.0 * hmin;
        f->cy = (f->ny % 2 == 0) && f->ny >= 2 && hy <= 2.0 * hmin;
        f->cz = (f->nz % 2 == 0) && f->nz >= 2 && hz <= 2.0 * hmin;
        if (ncell <= 64 || !(f->cx || f->cy || f->cz)) { f->cx = f->cy = f->cz = 0; break; }
        c->nx = f->cx ? f->nx / 2 : f->nx;
        c->ny = f->cy ? f->ny / 2 : f->ny;
        c->nz = f->cz ? f->nz / 2 : f->nz;
        c->DX = malloc(sizeof(double) * c->nx); c->FX = malloc(sizeof(double) * (c->nx + 1));
        c->DY = malloc(sizeof(double) * c->ny); c->FY = malloc(sizeof(double) * (c->ny + 1));
        c->DZ = malloc(sizeof(double) * c->nz); c->FZ = malloc(sizeof(double) * (c->nz + 1));
        for (i = 0; i < c->nx; i++) c->DX[i] = f->cx ? f->DX[2 * i] + f->DX[2 * i + 1] : f->DX[i];
        for (i = 0; i < c->ny; i++) c->DY[i] = f->cy ? f->DY[2 * i] + f->DY[2 * i + 1] : f->DY[i];
        for (i = 0; i < c->nz; i++) c->DZ[i] = f->cz ? f->DZ[2 * i] + f->DZ[2 * i + 1] : f->DZ[i];
        if (f->cx) faces_from_widths(c->DX, c->nx, c->FX); else memcpy(c->FX, f->FX, sizeof(double) * (c->nx + 1));
        if (f->cy) faces_from_widths(c->DY, c->ny, c->FY); else memcpy(c->FY, f->FY, sizeof(double) * (c->ny + 1));
        if (f->cz) faces_from_widths(c->DZ, c->nz, c->FZ); else memcpy(c->FZ, f->FZ, sizeof(double) * (c->nz + 1));
        c->pin = f->pin;
        H->nl = lev + 2;
    }
    if (H->nl < 1) H->nl = 1;
    for (lev = 0; lev < H->nl; lev++) {
        mg_lev *L = &H->L[lev];
        size_t nc = (size_t)L->nx * L->ny * L->nz;
        L->x = calloc(nc, sizeof(double));
        L->b = calloc(nc, sizeof(double));
        L->r = calloc(nc, sizeof(double));
        L->chol = NULL;
    }
    {   /* dense Cholesky of the coarsest operator */
        mg_lev *L = &H->L[H->nl - 1];
        int n = L->nx * L->ny * L->nz, a, b2, c2;
        double *M = calloc((size_t)n * n, sizeof(double)), *e = calloc((size_t)n, sizeof(double)), *y = calloc((size_t)n, sizeof(double));
        for (a = 0; a < n; a++) {
            e[a] = 1.0;
            mg_apply(L, e, y);
            for (b2 = 0; b2 < n; b2++) M[(size_t)b2 * n + a] = y[b2];
            e[a] = 0.0;
        }
        for (a = 0; a < n; a++) {
            double s = M[(size_t)a * n + a];
            for (c2 = 0; c2 < a; c2++) s -= M[(size_t)a * n + c2] * M[(size_t)a * n + c2];
            M[(size_t)a * n + a] = sqrt(s);
            for (b2 = a + 1; b2 < n; b2++) {
                double t = M[(size_t)b2 * n + a];
                for (c2 = 0; c2 < a; c2++) t -= M[(size_t)b2 * n + c2] * M[(size_t)a * n + c2];
                M[(size_t)b2 * n + a] = t / M[(size_t)a * n + a];
            }
        }
        L->chol = M;
        free(e); free(y);
    }
}

static void mg_free(mg_hier *H)
{
    int l;
    for (l = 0; l < H->nl; l++) {
        mg_lev *L = &H->L[l];
        free(L->DX); free(L->DY); free(L->DZ); free(L->FX); free(L->FY); free(L->FZ);
        free(L->x); free(L->b); free(L->r); free(L->chol);
    }
}

static void mg_coarse_solve(mg_lev *L)
{
    int n = L->nx * L->ny * L->nz, a, c2;
    double *M = L->chol;
    for (a = 0; a < n; a++) {
        double s = L->b[a];
        for (c2 = 0; c2 < a; c2++) s -= M[(size_t)a * n + c2] * L->x[c2];
        L->x[a] = s / M[(size_t)a * n + a];
    }
    for (a = n - 1; a >= 0; a--) {
        double s = L->x[a];
        for (c2 = a + 1; c2 < n; c2++) s -= M[(size_t)c2 * n + a] * L->x[c2];
        L->x[a] = s / M[(size_t)a * n + a];
    }
}

/* restriction and prolongation.  mode 0: sum of the (up to 8) children and
 * its transpose (piecewise constant); mode 1: linear interpolation between
 * coarse cell centres along each coarsened direction (positions from the
 * cell widths, so it follows the stretching) and its transpose. */
static int g_mg_mode = 1;
static int g_npre = 2, g_npost = 2;
void to_set_mg_options(int mode, int npre, int npost) { g_mg_mode = mode; g_npre = npre; g_npost = npost; }

static void centres(const double *D, int n, double *X)
{
    int i;
    X[0] = 0.5 * D[0];
    for (i = 1; i < n; i++) X[i] = X[i - 1] + 0.5 * (D[i - 1] + D[i]);
}

/* 1-D prolongation weights of fine index i: coarse (I0, I1), weights (w0, w1) */
static void pw(const double *xf, const double *xc, int nc, int coarsened, int i, int *I0, int *I1,
               double *w0, double *w1)
{
    int I;
    if (!coarsened) { *I0 = *I1 = i; *w0 = 1.0; *w1 = 0.0; return; }
    I = i / 2;
    if (g_mg_mode == 0) { *I0 = *I1 = I; *w0 = 1.0; *w1 = 0.0; return; }
    if (xf[i] < xc[I]) {
        if (I == 0) { *I0 = *I1 = 0; *w0 = 1.0; *w1 = 0.0; return; }
        *I0 = I - 1; *I1 = I;
    } else {
        if (I == nc - 1) { *I0 = *I1 = I; *w0 = 1.0; *w1 = 0.0; return; }
        *I0 = I; *I1 = I + 1;
    }
    *w1 = (xf[i] - xc[*I0]) / (xc[*I1] - xc[*I0]);
    *w0 = 1.0 - *w1;
}

typedef struct { int *I0, *I1; double *w0, *w1; } pw_tab;

static void pw_build(const double *Df, int nf, const double *Dc, int nc, int coarsened, pw_tab *t)
{
    double *xf = malloc(sizeof(double) * nf), *xc = malloc(sizeof(double) * nc);
    int i;
    centres(Df, nf, xf);
    centres(Dc, nc, xc);
    t->I0 = malloc(sizeof(int) * nf); t->I1 = malloc(sizeof(int) * nf);
    t->w0 = malloc(sizeof(double) * nf); t->w1 = malloc(sizeof(double) * nf);
    for (i = 0; i < nf; i++) pw(xf, xc, nc, coarsened, i, &t->I0[i], &t->I1[i], &t->w0[i], &t->w1[i]);
    free(xf); free(xc);
}

static void pw_free(pw_tab *t) { free(t->I0); free(t->I1); free(t->w0); free(t->w1); }

static void mg_transfer(const mg_lev *f, const mg_lev *c, double *xf, double *xc, int restrict_)
{
    pw_tab tx, ty, tz;
    int i, j, k, a, b, d;
    pw_build(f->DX, f->nx, c->DX, c->nx, f->cx, &tx);
    pw_build(f->DY, f->ny, c->DY, c->ny, f->cy, &ty);
    pw_build(f->DZ, f->nz, c->DZ, c->nz, f->cz, &tz);
    if (restrict_) memset(xc, 0, sizeof(double) * (size_t)c->nx * c->ny * c->nz);
    /* prolongation writes each fine cell once (parallel); restriction
     * scatters into shared coarse cells and stays serial */
#pragma omp parallel for private(i, j, a, b, d) schedule(static) if (!restrict_)
    for (k = 0; k < f->nz; k++)
        for (j = 0; j < f->ny; j++)
            for (i = 0; i < f->nx; i++) {
                size_t pf = LI(f, i, j, k);
                double acc = 0.0;
                for (d = 0; d < 2; d++) {
                    int K = d ? tz.I1[k] : tz.I0[k];
                    double wz = d ? tz.w1[k] : tz.w0[k];
                    if (wz == 0.0) continue;
                    for (b = 0; b < 2; b++) {
                        int J = b ? ty.I1[j] : ty.I0[j];
                        double wy = b ? ty.w1[j] : ty.w0[j];
                        if (wy == 0.0) continue;
                        for (a = 0; a < 2; a++) {
                            int I = a ? tx.I1[i] : tx.I0[i];
                            double wx = a ? tx.w1[i] : tx.w0[i], w = wx * wy * wz;
                            if (wx == 0.0) continue;
                            if (restrict_) xc[LI(c, I, J, K)] += w * xf[pf];
                            else acc += w * xc[LI(c, I, J, K)];
                        }
                    }
                }
                if (!restrict_) xf[pf] += acc;
            }
    pw_free(&tx); pw_free(&ty); pw_free(&tz);
}

static void mg_restrict(const mg_lev *f, const double *rf, const mg_lev *c, double *bc)
{
    mg_transfer(f, c, (double *)rf, bc, 1);
}

static void mg_prolong_add(const mg_lev *f, double *xf, const mg_lev *c, const double *xc)
{
    mg_transfer(f, c, xf, (double *)xc, 0);
}


static void mg_vcycle(mg_hier *H, int lev)
{
    mg_lev *L = &H->L[lev];
    size_t nc = (size_t)L->nx * L->ny * L->nz, t;
    int s;
    if (lev == H->nl - 1) { mg_coarse_solve(L); return; }
    memset(L->x, 0, nc * sizeof(double));
    for (s = 0; s < g_npre; s++) { mg_rbgs(L, L->x, L->b, 0); mg_rbgs(L, L->x, L->b, 1); }
    mg_apply(L, L->x, L->r);
#pragma omp parallel for schedule(static)
    for (t = 0; t < nc; t++) L->r[t] = L->b[t] - L->r[t];
    mg_restrict(L, L->r, &H->L[lev + 1], H->L[lev + 1].b);
    mg_vcycle(H, lev + 1);
    mg_prolong_add(L, L->x, &H->L[lev + 1], H->L[lev + 1].x);
    for (s = 0; s < g_npost; s++) { mg_rbgs(L, L->x, L->b, 1); mg_rbgs(L, L->x, L->b, 0); }
}

int to_pressure_solve(const to_grid *g, const to_params *p, const double *b,
                      double *phi, double *relres)
{
    mg_hier H;
    mg_lev *L0;
    size_t nc, t;
    int i, j, k, it = 0;
    double *bw, *x, *r, *z, *pv, *q, rz, nbw, nr;
    memset(&H, 0, sizeof(H));
    mg_build(g, &H);
    L0 = &H.L[0];
    nc = (size_t)L0->nx * L0->ny * L0->nz;
    bw = malloc(nc * sizeof(double)); x = malloc(nc * sizeof(double));
    r = malloc(nc * sizeof(double)); z = malloc(nc * sizeof(double));
    pv = malloc(nc * sizeof(double)); q = malloc(nc * sizeof(double));
    for (k = 0; k < L0->nz; k++)
        for (j = 0; j < L0->ny; j++)
            for (i = 0; i < L0->nx; i++) {
                size_t c = LI(L0, i, j, k), d = IDX(g, i, j, k);
                bw[c] = L0->DX[i] * L0->DY[j] * L0->DZ[k] * b[d];
                x[c] = phi[d];
            }
    mg_apply(L0, x, r);
    for (t = 0; t < nc; t++) r[t] = bw[t] - r[t];
    nbw = sqrt(dot(nc, bw, bw));
    nr = sqrt(dot(nc, r, r));
    rz = 0.0;
    {
        int restart = 1;
        for (;;) {
            double rz1, alpha;
            if (nr <= p->p_rtol * nbw || it >= p->p_maxit) {
                /* the recursive residual drifts from b - S x; confirm with the
                   true residual and restart from it if the test fails */
                mg_apply(L0, x, r);
                for (t = 0; t < nc; t++) r[t] = bw[t] - r[t];
                nr = sqrt(dot(nc, r, r));
                if (nr <= p->p_rtol * nbw || it >= p->p_maxit) break;
                restart = 1;
            }
            memcpy(L0->b, r, nc * sizeof(double));
            mg_vcycle(&H, 0);
            memcpy(z, L0->x, nc * sizeof(double));
            rz1 = dot(nc, r, z);
            if (restart) memcpy(pv, z, nc * sizeof(double));
            else {
                double beta = rz1 / rz;
#pragma omp parallel for schedule(static)
                for (t = 0; t < nc; t++) pv[t] = z[t] + beta * pv[t];
            }
            restart = 0;
            rz = rz1;
            mg_apply(L0, pv, q);
            alpha = rz / dot(nc, pv, q);
#pragma omp parallel for schedule(static)
            for (t = 0; t < nc; t++) { x[t] += alpha * pv[t]; r[t] -= alpha * q[t]; }
            nr = sqrt(dot(nc, r, r));
            it++;
        }
    }
    for (k = 0; k < g->NZ; k++)
        for (j = 0; j < g->NY; j++)
            for (i = 0; i < g->NX; i++)
                phi[IDX(g, i, j, k)] = (i < g->nx && j < g->ny && k < g->nz) ? x[LI(L0, i, j, k)] : 0.0;
    if (relres) {
        size_t n = NPTS(g);
        double *ax = malloc(n * sizeof(double)), s = 0.0, sb = 0.0;
        to_pressure_apply(g, phi, ax);
        for (t = 0; t < n; t++) { double d = b[t] - ax[t]; s += d * d; sb += b[t] * b[t]; }
        *relres = sb > 0.0 ? sqrt(s / sb) : 0.0;
        free(ax);
    }
    free(bw); free(x); free(r); free(z); free(pv); free(q);
    mg_free(&H);
    return it;
}

/* Pressure_project_velocity, Pressure.c:280-439 (rotational dp update) */
void to_project(const to_grid *g, const to_params *p, double dt,
                const double *phi, const double *b, double *u, double *v,
                double *w, double *dpx, double *dpy, double *dpz)
{
    int i, j, k;
    double coef = dt / p->re, a_dEta = 1.0 / g->dEta, a_dXi = 1.0 / g->dXi, a_dPhi = 1.0 / g->dPhi;
    size_t NX = g->NX, NXY = (size_t)g->NX * g->NY;
    for (k = 0; k < g->NZ; k++)
        for (j = 0; j < g->NY; j++)
            for (i = 0; i < g->NX; i++) {
                size_t q = IDX(g, i, j, k);
                if (g->st[0][q] != TO_BOUNDARY) {
                    double me = g->mxu[i];
                    double d = (phi[q] - phi[q - 1]) * a_dEta * me;
                    double lap;
                    u[q] -= dt * d;
                    lap = -(b[q] - b[q - 1]) * me * a_dEta;
                    dpx[q] += d - coef * lap;
                }
            }
    for (k = 0; k < g->NZ; k++)
        for (j = 0; j < g->NY; j++) {
            double Cy = a_dXi * g->myv[j];
            for (i = 0; i < g->NX; i++) {
                size_t q = IDX(g, i, j, k);
                if (g->st[1][q] != TO_BOUNDARY) {
                    double d = (phi[q] - phi[q - NX]) * Cy, lap;
                    v[q] -= dt * d;
                    lap = -(b[q] - b[q - NX]) * Cy;
                    dpy[q] += d - coef * lap;
                }
            }
        }
    for (k = 0; k < g->NZ; k++) {
        double Cz = g->mzw[k] * a_dPhi;
        for (j = 0; j < g->NY; j++)
            for (i = 0; i < g->NX; i++) {
                size_t q = IDX(g, i, j, k);
                if (g->st[2][q] != TO_BOUNDARY) {
                    double d = (phi[q] - phi[q - NXY]) * Cz, lap;
                    w[q] -= dt * d;
                    lap = -(b[q] - b[q - NXY]) * Cz;
                    dpz[q] += d - coef * lap;
                }
            }
    }
}

/* Pressure_compute_velocity_divergence, Pressure.c:462-586 */
double to_divergence(const to_grid *g, const double *u, const double *v,
                     const double *w, double *div)
{
    int i, j, k;
    double a_dEta = 1.0 / g->dEta, a_dXi = 1.0 / g->dXi, a_dPhi = 1.0 / g->dPhi, mx = 0.0;
    for (k = 0; k < g->NZ; k++)
        for (j = 0; j < g->NY; j++)
            for (i = 0; i < g->NX; i++) {
                size_t p = IDX(g, i, j, k);
                double dc = 0.0;
                if (g->st[3][p] != TO_BOUNDARY) {
                    double dudx = (u[IDX(g, i + 1, j, k)] - u[p]) * a_dEta * g->mxc[i];
                    double dvdy = (v[IDX(g, i, j + 1, k)] - v[p]) * a_dXi * g->myc[j];
                    double dwdz = (w[IDX(g, i, j, k + 1)] - w[p]) * a_dPhi * g->mzc[k];
                    dc = fabs(dudx + dvdy + dwdz);
                }
                if (div) div[p] = dc;
                if (dc >= mx) mx = dc;
            }
    return mx;
}

/* One TVD-RK2 step (definitions.h:148-149) in the restated stage order:
 * store_old (Velocity.c:297, Conc.c:997); per stage: cell_center, total
 * concentration, particle velocity (Conc.c:734-761), transposes + convection,
 * set_RHS, Helmholtz solves, pressure RHS, Poisson solve, projection,
 * divergence; then rk_average(0.5, 0.5) (Velocity.c:2047, Conc.c:1007). */
int to_step(const to_grid *g, const to_params *p, to_state *s, double dt,
            to_step_stats *st)
{
    size_t n = NPTS(g), t;
    int stage, ic, nc = p->nconc;
    double *ubc = calloc(n, 8), *vbc = calloc(n, 8), *wbc = calloc(n, 8);
    double *A = calloc(n, 8), *B = calloc(n, 8), *ctot = calloc(n, 8);
    double *cu = calloc(n, 8), *cv = calloc(n, 8), *cw = calloc(n, 8);
    double *bu = calloc(n, 8), *bv = calloc(n, 8), *bw = calloc(n, 8);
    double *cc[TO_MAXCONC], *bc = calloc(n, 8), *vp = calloc(n, 8);
    for (ic = 0; ic < nc; ic++) cc[ic] = calloc(n, 8);
    memcpy(s->u_old, s->u, n * 8); memcpy(s->v_old, s->v, n * 8); memcpy(s->w_old, s->w, n * 8);
    for (ic = 0; ic < nc; ic++) memcpy(s->c_old[ic], s->c[ic], n * 8);
    for (stage = 0; stage < 2; stage++) {
        double rr;
        to_cell_center(g, s->u, s->v, s->w, ubc, vbc, wbc);
        if (nc > 1) to_total_concentration(g, p, (const double *const *)s->c, ctot);
        else memcpy(ctot, s->c[0], n * 8);
        to_transpose(g, 'u', s->u, s->v, s->w, A, B);
        to_convection_vel(g, p, 'u', s->u, s->u, A, B, cu);
        to_transpose(g, 'v', s->u, s->v, s->w, A, B);
        to_convection_vel(g, p, 'v', s->v, A, s->v, B, cv);
        to_transpose(g, 'w', s->u, s->v, s->w, A, B);
        to_convection_vel(g, p, 'w', s->w, A, B, s->w, cw);
        for (ic = 0; ic < nc; ic++) {
            const double *va = vbc;
            if (p->ctype[ic] == TO_PARTICLE) {
                for (t = 0; t < n; t++) vp[t] = vbc[t] + p->vs0[ic];
                va = vp;
            }
            to_convection_conc(g, p, ic, s->c[ic], ubc, va, wbc, cc[ic]);
        }
        to_set_rhs_vel(g, p, 'u', dt, s->u, cu, s->dpx, ctot, bu);
        to_set_rhs_vel(g, p, 'v', dt, s->v, cv, s->dpy, ctot, bv);
        to_set_rhs_vel(g, p, 'w', dt, s->w, cw, s->dpz, ctot, bw);
        st->vel_iters[0][stage] = to_helmholtz_solve(g, p, 'u', 0, dt, bu, s->u, 0, &rr);
        st->vel_iters[1][stage] = to_helmholtz_solve(g, p, 'v', 0, dt, bv, s->v, 0, &rr);
        st->vel_iters[2][stage] = to_helmholtz_solve(g, p, 'w', 0, dt, bw, s->w, 0, &rr);
        for (ic = 0; ic < nc; ic++) {
            to_set_rhs_conc(g, dt, s->c[ic], cc[ic], bc);
            st->conc_iters[ic][stage] = to_helmholtz_solve(g, p, 'c', ic, dt, bc, s->c[ic], 0, &rr);
        }
        to_pressure_rhs(g, dt, s->u, s->v, s->w, s->pb);
        st->p_iters[stage] = to_pressure_solve(g, p, s->pb, s->phi, &st->p_relres[stage]);
        to_project(g, p, dt, s->phi, s->pb, s->u, s->v, s->w, s->dpx, s->dpy, s->dpz);
        st->div_max[stage] = to_divergence(g, s->u, s->v, s->w, NULL);
    }
    for (t = 0; t < n; t++) {
        s->u[t] = 0.5 * s->u_old[t] + 0.5 * s->u[t];
        s->v[t] = 0.5 * s->v_old[t] + 0.5 * s->v[t];
        s->w[t] = 0.5 * s->w_old[t] + 0.5 * s->w[t];
    }
    for (ic = 0; ic < nc; ic++)
        for (t = 0; t < n; t++) s->c[ic][t] = 0.5 * s->c_old[ic][t] + 0.5 * s->c[ic][t];
    free(ubc); free(vbc); free(wbc); free(A); free(B); free(ctot);
    free(cu); free(cv); free(cw); free(bu); free(bv); free(bw); free(bc); free(vp);
    for (ic = 0; ic < nc; ic++) free(cc[ic]);
    return 0;
}

/* ---- diagnostics ---------------------------------------------------------
 * Cell widths dx_c, dy_c, dz_c of Grid_compute_metric_coefficients
 * (Grid.c:633-637, 650-654, 667-671): x_{i+1} - x_i of the face coordinates,
 * the last one repeating its neighbour. */
static void cell_widths(const double *f, int n, double *d)
{
    int i;
    for (i = 1; i < n - 1; i++) d[i] = f[i + 1] - f[i];
    d[0] = f[1] - f[0];
    d[n - 1] = f[n - 1] - f[n - 2];
}

void to_interface_y_index(const to_grid *g, int32_t *iy)
{
    int i, j, k;
    for (k = 0; k < g->NZ; k++)
        for (i = 0; i < g->NX; i++) {
            int32_t r = -1;
            for (j = 0; j < g->NY; j++) {
                uint8_t s = g->st[3][IDX(g, i, j, k)];
                if (s == TO_IMMERSED || (j == 0 && s == TO_FLUID)) {
                    r = j;
                    break;
                }
            }
            iy[(size_t)k * g->NX + i] = r;
        }
}

void to_deposit_integrate(const to_grid *g, const to_params *p, const int32_t *iy,
                          const double *const *c, const double *const *c_old,
                          double dt, double *dep)
{
    int i, k, ic;
    for (ic = 0; ic < p->nconc; ic++) {
        double *h = dep + (size_t)ic * g->NZ * g->NX;
        for (k = 0; k < g->NZ; k++)
            for (i = 0; i < g->NX; i++) {
                int j = iy[(size_t)k * g->NX + i];
                if (j >= 0 && j < g->NY) {
                    size_t q = IDX(g, i, j, k);
                    double dh = dt * fabs(p->vs0[ic]) * p->alpha[ic] * 0.5 * (c[ic][q] + c_old[ic][q]);
                    h[(size_t)k * g->NX + i] += dh;
                }
            }
    }
}

/* Extract_viscous_dissipation_rate, Extract.c:453-725: sum over FLUID c
 * nodes of u lap(u) dV_u + v lap(v) dV_v + w lap(w) dV_w (each velocity at
 * its own face node, the c node's index), over Re; box-wall ghosts are
 * k * (own value) with k = -1 no-slip, +1 free-slip, the normal component
 * 0; no inflow / outflow. */
static double viscous_dissipation(const to_grid *g, const to_params *p, const double *u,
                                  const double *v, const double *w, const double *dxc,
                                  const double *dyc, const double *dzc)
{
    int NX = g->NX, NY = g->NY, NZ = g->NZ, NI = NX - 1, NJ = NY - 1, NK = NZ - 1, i, j, k;
    double kw[6], G = 0.0;
    double Cx = 1.0 / (g->dEta * g->dEta), Cy = 1.0 / (g->dXi * g->dXi), Cz = 1.0 / (g->dPhi * g->dPhi);
    const double *mxc = g->mxc, *myc = g->myc, *mzc = g->mzc, *mxu = g->mxu, *myv = g->myv, *mzw = g->mzw;
    for (i = 0; i < 6; i++) kw[i] = p->wall_noslip[i] ? -1.0 : 1.0;
    for (k = 0; k < NZ; k++)
        for (j = 0; j < NY; j++)
            for (i = 0; i < NX; i++) {
                size_t q = IDX(g, i, j, k);
                double U_w, U_e, U_n, U_s, U_f, U_b, V_w, V_e, V_n, V_s, V_f, V_b, W_w, W_e, W_n, W_s, W_f, W_b;
                if (g->st[3][q] != TO_FLUID) continue;
                double U_ae = Cx * mxu[i] * mxc[i], U_aw = Cx * mxu[i];
                double U_an = Cy * myc[j] * myv[j + 1], U_as = Cy * myc[j] * myv[j];
                double U_af = Cz * mzc[k] * mzw[k + 1], U_ab = Cz * mzc[k] * mzw[k];
                double V_ae = Cx * mxc[i] * mxu[i + 1], V_aw = Cx * mxc[i] * mxu[i];
                double V_an = Cy * myv[j] * myc[j], V_as = Cy * myv[j];
                double V_af = Cz * mzc[k] * mzw[k + 1], V_ab = Cz * mzc[k] * mzw[k];
                double W_ae = Cx * mxc[i] * mxu[i + 1], W_aw = Cx * mxc[i] * mxu[i];
                double W_an = Cy * myc[j] * myv[j + 1], W_as = Cy * myc[j] * myv[j];
                double W_af = Cz * mzw[k] * mzc[k], W_ab = Cz * mzw[k];
                double u_ = u[q], v_ = v[q], w_ = w[q];
                if (i == 0) {
                    U_aw *= mxc[i];
                    U_w = 0.0; V_w = kw[0] * v_; W_w = kw[0] * w_;
                } else {
                    U_aw *= mxc[i - 1];
                    U_w = u[q - 1]; V_w = v[q - 1]; W_w = w[q - 1];
                }
                if (j == 0) {
                    V_as *= myc[j];
                    U_s = kw[2] * u_; V_s = 0.0; W_s = kw[2] * w_;
                } else {
                    V_as *= myc[j - 1];
                    U_s = u[IDX(g, i, j - 1, k)]; V_s = v[IDX(g, i, j - 1, k)]; W_s = w[IDX(g, i, j - 1, k)];
                }
                if (k == 0) {
                    W_ab *= mzc[k];
                    U_b = kw[4] * u_; V_b = kw[4] * v_; W_b = 0.0;
                } else {
                    W_ab *= mzc[k - 1];
                    U_b = u[IDX(g, i, j, k - 1)]; V_b = v[IDX(g, i, j, k - 1)]; W_b = w[IDX(g, i, j, k - 1)];
                }
                if (i == NI - 1) {
                    U_e = 0.0; V_e = kw[1] * v_; W_e = kw[1] * w_;
                } else {
                    U_e = u[q + 1]; V_e = v[q + 1]; W_e = w[q + 1];
                }
                if (j == NJ - 1) {
                    U_n = kw[3] * u_; V_n = 0.0; W_n = kw[3] * w_;
                } else {
                    U_n = u[IDX(g, i, j + 1, k)]; V_n = v[IDX(g, i, j + 1, k)]; W_n = w[IDX(g, i, j + 1, k)];
                }
                if (k == NK - 1) {
                    U_f = kw[5] * u_; V_f = kw[5] * v_; W_f = 0.0;
                } else {
                    U_f = u[IDX(g, i, j, k + 1)]; V_f = v[IDX(g, i, j, k + 1)]; W_f = w[IDX(g, i, j, k + 1)];
                }
                {
                    double U_ap = -(U_ae + U_aw + U_ab + U_af + U_as + U_an);
                    double V_ap = -(V_ae + V_aw + V_ab + V_af + V_as + V_an);
                    double W_ap = -(W_ae + W_aw + W_ab + W_af + W_as + W_an);
                    double lu = (U_ae * U_e + U_aw * U_w) + (U_an * U_n + U_as * U_s) + (U_af * U_f + U_ab * U_b) + U_ap * u_;
                    double lv = (V_ae * V_e + V_aw * V_w) + (V_an * V_n + V_as * V_s) + (V_af * V_f + V_ab * V_b) + V_ap * v_;
                    double lw = (W_ae * W_e + W_aw * W_w) + (W_an * W_n + W_as * W_s) + (W_af * W_f + W_ab * W_b) + W_ap * w_;
                    double dVu = (g->xc[i + 1] - g->xc[i]) * dyc[j] * dzc[k];
                    double dVv = (g->yc[j + 1] - g->yc[j]) * dxc[i] * dzc[k];
                    double dVw = (g->zc[k + 1] - g->zc[k]) * dxc[i] * dyc[j];
                    G += u_ * lu * dVu + v_ * lv * dVv + w_ * lw * dVw;
                }
            }
    return G * (1.0 / p->re);
}

void to_diagnostics(const to_grid *g, const to_params *p, const double *u,
                    const double *v, const double *w, const double *const *c,
                    double front_limit, const int32_t *iy, const double *dep,
                    to_diag *out, double *h_ave, double *sed_bottom)
{
    size_t n = NPTS(g);
    int NX = g->NX, NY = g->NY, NZ = g->NZ, i, j, k, ic, nc = p->nconc;
    double *ubc = (double *)calloc(n, sizeof(double)), *vbc = (double *)calloc(n, sizeof(double));
    double *wbc = (double *)calloc(n, sizeof(double)), *ctot = NULL;
    double *dxc = (double *)malloc(NX * sizeof(double)), *dyc = (double *)malloc(NY * sizeof(double));
    double *dzc = (double *)malloc(NZ * sizeof(double)), *h = (double *)calloc((size_t)nc * NX, sizeof(double));
    const double *ct;
    const uint8_t *cs = g->st[3];
    double ke = 0.0, rate = 0.0, y_ref = g->yv[0];
    to_cell_center(g, u, v, w, ubc, vbc, wbc);
    cell_widths(g->xu, NX, dxc);
    cell_widths(g->yv, NY, dyc);
    cell_widths(g->zw, NZ, dzc);
    if (nc > 1) {
        ctot = (double *)calloc(n, sizeof(double));
        to_total_concentration(g, p, c, ctot);
        ct = ctot;
    } else {
        ct = c[0];
    }
    /* Extract_total_kinetic_energy, Extract.c:803-882 */
    for (k = 0; k < NZ; k++) {
        double dz = dzc[k];
        for (j = 0; j < NY; j++) {
            double dy = dyc[j];
            for (i = 0; i < NX; i++) {
                size_t q = IDX(g, i, j, k);
                if (cs[q] == TO_FLUID) {
                    double dx = dxc[i], dV = dx * dy * dz;
                    ke += (ubc[q] * ubc[q] + vbc[q] * vbc[q] + wbc[q] * wbc[q]) * dV;
                }
            }
        }
    }
    out->kinetic_energy = ke * 0.5;
    out->viscous_dissipation = viscous_dissipation(g, p, u, v, w, dxc, dyc, dzc);
    /* Extract_kinetic_potential_conversion_rate, Extract.c:727-801 */
    for (k = 0; k < NZ; k++) {
        double dz = dzc[k];
        for (j = 0; j < NY; j++) {
            double dy = dyc[j];
            for (i = 0; i < NX; i++) {
                size_t q = IDX(g, i, j, k);
                if (cs[q] == TO_FLUID) {
                    double dx = dxc[i];
                    rate += -vbc[q] * ct[q] * (dx * dy * dz);
                }
            }
        }
    }
    out->conversion_rate = rate;
    for (ic = 0; ic < TO_MAXCONC; ic++) {
        out->suspended_mass[ic] = out->potential_energy[ic] = 0.0;
        out->stokes_dissipation[ic] = out->conversion_rate_c[ic] = 0.0;
        out->ep_passive[ic] = out->ep_passive_rate[ic] = out->ep_rate[ic] = out->sed_rate[ic] = 0.0;
    }
    for (ic = 0; ic < nc; ic++) {
        const double *cc = c[ic];
        double m = 0.0, ep = 0.0, st = 0.0, cr = 0.0;
        /* Conc_compute_total_suspended_mass, Conc.c:1471-1522 */
        for (k = 0; k < NZ; k++) {
            double dz = dzc[k];
            for (j = 0; j < NY; j++) {
                double dy = dyc[j];
                for (i = 0; i < NX; i++) {
                    size_t q = IDX(g, i, j, k);
                    if (cs[q] == TO_FLUID) {
                        double dV = dz * dy * dxc[i];
                        m += cc[q] * dV;
                    }
                }
            }
        }
        out->suspended_mass[ic] = m;
        /* Conc_compute_potential_energies, Conc.c:1934-2055 (suspended part) */
        for (k = 0; k < NZ; k++) {
            double dz = dzc[k];
            for (j = 0; j < NY; j++) {
                double dy = dyc[j];
                for (i = 0; i < NX; i++) {
                    size_t q = IDX(g, i, j, k);
                    if (cs[q] == TO_FLUID) {
                        double dx = dxc[i], dV = dx * dy * dz;
                        ep += cc[q] * dV * (g->yc[j] - y_ref);
                        st += cc[q] * dV;
                        cr += vbc[q] * cc[q] * (dx * dy * dz);
                    }
                }
            }
        }
        out->potential_energy[ic] = ep * p->alpha[ic];
        out->stokes_dissipation[ic] = st * (fabs(p->vs0[ic]) * p->alpha[ic]);
        out->conversion_rate_c[ic] = cr * p->alpha[ic];
        /* the deposited part of Conc_compute_potential_energies (Conc.c:1955-1985),
         * Conc_compute_sedimentation_rate (Conc.c:2098-2156) and
         * Conc_bottom_sed_rate (Conc.c:2158-2230): bed nodes of particle fractions */
        {
            double epp = 0.0, sr = 0.0, us = fabs(p->vs0[ic]);
            const double *dh = dep ? dep + (size_t)ic * NZ * NX : NULL;
            double *sb = sed_bottom ? sed_bottom + (size_t)ic * NZ * NX : NULL;
            for (k = 0; k < NZ; k++) {
                double dz = dzc[k];
                for (i = 0; i < NX; i++) {
                    double dx = dxc[i], r = 0.0;
                    int jb = iy[(size_t)k * NX + i];
                    if (p->ctype[ic] == TO_PARTICLE && jb >= 0 && jb < NY) {
                        if (dh) epp += dh[(size_t)k * NX + i] * dx * dz * (g->yc[jb] - y_ref);
                        r = us * cc[IDX(g, i, jb, k)] * dx * dz;
                        sr += r;
                    }
                    if (sb) sb[(size_t)k * NX + i] = r;
                }
            }
            out->ep_passive[ic] = epp;
            out->ep_passive_rate[ic] = epp * us;
            out->ep_rate[ic] = out->conversion_rate_c[ic] + out->ep_passive_rate[ic] - out->stokes_dissipation[ic];
            out->sed_rate[ic] = sr;
        }
        /* Conc_compute_ave_height_x, Conc.c:1524-1608 */
        {
            double Ly = g->yv[NY - 1] - g->yv[0], Lz = g->zw[NZ - 1] - g->zw[0], coef = 1.0 / (Ly * Lz);
            for (i = 0; i < NX; i++) {
                double ht = 0.0;
                for (k = 0; k < NZ; k++) {
                    double dz = dzc[k];
                    for (j = 0; j < NY; j++) {
                        size_t q = IDX(g, i, j, k);
                        if (cs[q] == TO_FLUID) {
                            double dy = dyc[j];
                            ht += cc[q] * dy * dz;
                        }
                    }
                }
                h[(size_t)ic * NX + i] = ht * coef;
            }
        }
    }
    /* Conc_find_front_location, Conc.c:1610-1672 */
    out->front_location = -1.0;
    for (i = NX - 2; i > 0; i--) {
        double h0 = 0.0, h1 = 0.0;
        for (ic = 0; ic < nc; ic++) {
            h0 += h[(size_t)ic * NX + i - 1] * p->alpha[ic];
            h1 += h[(size_t)ic * NX + i] * p->alpha[ic];
        }
        if (h1 <= front_limit && h0 >= front_limit) {
            /* x at the limit: MyMath_interpolate_quantity with the heights as
             * coordinates and the cell-centre x as values (Conc.c:1652-1662) */
            out->front_location = interp2(g->xc[i - 1], g->xc[i], h0, h1, front_limit);
            break;
        }
    }
    if (h_ave) memcpy(h_ave, h, (size_t)nc * NX * sizeof(double));
    free(ubc); free(vbc); free(wbc); free(ctot); free(dxc); free(dyc); free(dzc); free(h);
}
