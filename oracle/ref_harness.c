/*
 * ref_harness.c -- drives the reference's own routines, compiled unmodified
 * against the single-rank PETSc shim, on caller-supplied arrays (TEST
 * INFRASTRUCTURE ONLY).  Linked with the reference sources into
 * oracle/_ref/libturbins_ref.so by oracle/refbuild.py; used to pin the CPU
 * oracle (turb_oracle.c) and to generate tests/golden fixtures.
 *
 * Arrays are DA-ordered doubles of (nx+1)(ny+1)(nz+1) points.  The harness
 * builds the MAC_grid by hand (coordinates + the reference's
 * Grid_compute_metric_coefficients), fills the status vectors and the
 * ImmersedNode stencils, and creates the Velocity / Pressure / Concentration
 * objects with the reference's *_create routines.
 */
#include "definitions.h"
#include "DataTypes.h"
#include "ENO.h"
#include "Grid.h"
#include "Immersed.h"
#include "Velocity.h"
#include "Conc.h"
#include "Pressure.h"
#include "Extract.h"
#include "Memory.h"
#include "Resume.h"
#include "Solver.h"
#include <string.h>
#include <unistd.h>

typedef struct {
    MAC_grid *g;
    Parameters *p;
    Velocity *u, *v, *w;
    Pressure *pr;
    Concentration *c[4];
    ENO_Scheme *eno;
    long n;
    double *hbuf[8];   /* G_ / W_ave_height_x of each fraction (ref_diagnostics) */
} ref_case;

static void vset(Vec v, const double *a, long n) { memcpy(shim_vec_data(v), a, sizeof(double) * n); }
static void vget(Vec v, double *a, long n) { memcpy(a, shim_vec_data(v), sizeof(double) * n); }

ref_case *ref_create(int nx, int ny, int nz, const double *xc, const double *yc, const double *zc,
                     const double *xu, const double *yv, const double *zw, const unsigned char *st_u,
                     const unsigned char *st_v, const unsigned char *st_w, const unsigned char *st_c,
                     int eno_order, double re, int nconc, const double *pe, const double *vs0,
                     const double *alpha, const int *ctype, int sedimentation)
{
    ref_case *r = (ref_case *)calloc(1, sizeof(ref_case));
    Parameters *p = (Parameters *)calloc(1, sizeof(Parameters));
    MAC_grid *g = (MAC_grid *)calloc(1, sizeof(MAC_grid));
    /* the reference pauses on getchar() after some warnings (e.g.
     * Immersed_is_valid, Immersed.c:1422-1425); with stdin at end of file
     * those pauses return at once instead of waiting on the caller's stdin */
    if (!freopen("/dev/null", "r", stdin)) clearerr(stdin);
    int NX = nx + 1, NY = ny + 1, NZ = nz + 1, i;
    long n = (long)NX * NY * NZ, t;
    const unsigned char *st[4] = {st_u, st_v, st_w, st_c};
    Vec *gs[4], *ls[4];
    double ***sp[4];
    r->g = g; r->p = p; r->n = n;
    p->NX = nx; p->NY = ny; p->NZ = nz;
    p->Re = re; p->NConc = nconc; p->ENO_scheme_order = eno_order;
    p->Pe = (double *)calloc(4, sizeof(double)); p->Phi = (double *)calloc(4, sizeof(double));
    p->Conc_alpha = (double *)calloc(4, sizeof(double)); p->V_s0 = (double *)calloc(4, sizeof(double));
    p->conc_type = (int *)calloc(4, sizeof(int));
    for (i = 0; i < nconc; i++) {
        p->Pe[i] = pe[i]; p->V_s0[i] = vs0[i]; p->Conc_alpha[i] = alpha[i]; p->conc_type[i] = ctype[i];
    }
    p->sedimentation = (short)sedimentation;
    p->viscosity_type = CONSTANT_VISCOSITY;
    p->resmax = 1e-12;
    p->xmin = xu[0]; p->ymin = yv[0]; p->zmin = zw[0];
    /* grid */
    g->NX = NX; g->NY = NY; g->NZ = NZ; g->NT = NX * NY * NZ;
    g->NI = NX - 1; g->NJ = NY - 1; g->NK = NZ - 1;
    g->dEta = 1.0 / (double)nx; g->dXi = 1.0 / (double)ny; g->dPhi = 1.0 / (double)nz;
    g->G_Is = g->G_Js = g->G_Ks = 0; g->G_Ie = NX; g->G_Je = NY; g->G_Ke = NZ;
    g->L_Is = g->L_Js = g->L_Ks = 0; g->L_Ie = NX; g->L_Je = NY; g->L_Ke = NZ;
    DACreate3d(PCW, DA_NONPERIODIC, DA_STENCIL_STAR, NX, NY, NZ, 1, 1, 1, 1, eno_order, 0, 0, 0, &g->DA_3D);
    DACreate3d(PCW, DA_NONPERIODIC, DA_STENCIL_BOX, NX, NY, NZ, 1, 1, 1, 1, 3, 0, 0, 0, &g->DA_3D_BOX);
    DACreate3d(PCW, DA_NONPERIODIC, DA_STENCIL_STAR, NX, NY, NZ, 1, 1, 1, 1, 1, 0, 0, 0, &g->DA_3D_Lsys);
#define A1(name, len) g->name = (double *)calloc((size_t)(len), sizeof(double))
    A1(xc, NX); A1(yc, NY); A1(zc, NZ); A1(xu, NX); A1(yu, NY); A1(zu, NZ); A1(xv, NX); A1(yv, NY); A1(zv, NZ);
    A1(xw, NX); A1(yw, NY); A1(zw, NZ); A1(metric_xc, NX); A1(metric_yc, NY); A1(metric_zc, NZ);
    A1(metric_xu, NX); A1(metric_yv, NY); A1(metric_zw, NZ); A1(dx_c, NX); A1(dy_c, NY); A1(dz_c, NZ);
#undef A1
    memcpy(g->xc, xc, 8 * NX); memcpy(g->yc, yc, 8 * NY); memcpy(g->zc, zc, 8 * NZ);
    memcpy(g->xu, xu, 8 * NX); memcpy(g->yv, yv, 8 * NY); memcpy(g->zw, zw, 8 * NZ);
    /* aliases of Grid_import_grid_from_file, Grid.c:1366-1378 */
    memcpy(g->xv, xc, 8 * NX); memcpy(g->xw, xc, 8 * NX); memcpy(g->yu, yc, 8 * NY);
    memcpy(g->yw, yc, 8 * NY); memcpy(g->zu, zc, 8 * NZ); memcpy(g->zv, zc, 8 * NZ);
    Grid_compute_metric_coefficients(g, 'u');
    Grid_compute_metric_coefficients(g, 'v');
    Grid_compute_metric_coefficients(g, 'w');
    Grid_compute_metric_coefficients(g, 'c');
    gs[0] = &g->G_u_status; gs[1] = &g->G_v_status; gs[2] = &g->G_w_status; gs[3] = &g->G_c_status;
    ls[0] = &g->L_u_status; ls[1] = &g->L_v_status; ls[2] = &g->L_w_status; ls[3] = &g->L_c_status;
    for (i = 0; i < 4; i++) {
        double *a;
        DACreateGlobalVector(g->DA_3D_BOX, gs[i]);
        *ls[i] = *gs[i];
        a = shim_vec_data(*gs[i]);
        for (t = 0; t < n; t++) a[t] = (double)st[i][t];
    }
    DAVecGetArray(g->DA_3D_BOX, g->L_u_status, (void ***)&g->u_status);
    DAVecGetArray(g->DA_3D_BOX, g->L_v_status, (void ***)&g->v_status);
    DAVecGetArray(g->DA_3D_BOX, g->L_w_status, (void ***)&g->w_status);
    DAVecGetArray(g->DA_3D_BOX, g->L_c_status, (void ***)&g->c_status);
    (void)sp;
    DACreateGlobalVector(g->DA_3D, &g->lsys_diagonal);
    DACreateGlobalVector(g->DA_3D, &g->G_dummy1); g->L_dummy1 = g->G_dummy1;
    DACreateGlobalVector(g->DA_3D, &g->G_dummy2); g->L_dummy2 = g->G_dummy2;
    r->u = Velocity_create(g, p, 'u');
    r->v = Velocity_create(g, p, 'v');
    r->w = Velocity_create(g, p, 'w');
    r->pr = Pressure_create(g, p);
    for (i = 0; i < nconc; i++) r->c[i] = Conc_create(g, p, i);
    r->eno = ENO_create(p);
    return r;
}

/* immersed stencils of quantity q: im/fidx are DA linear indices */
void ref_set_immersed(ref_case *r, char q, int n, const int *im, const int *nf, const int *fidx,
                      const double *fcoef, const double *bcoef)
{
    MAC_grid *g = r->g;
    Immersed *I;
    int NX = g->NX, NY = g->NY, t, k;
    I = Immersed_create(g, q);
    if (q == 'u') g->u_immersed = I;
    else if (q == 'v') g->v_immersed = I;
    else if (q == 'w') g->w_immersed = I;
    else g->c_immersed = I;
    Immersed_set_q_immersed_indices(g, q);
    Immersed_set_q_immersed_boundary_condition(g, q);
    for (t = 0; t < n; t++) {
        int ii = im[t] % NX, jj = (im[t] / NX) % NY, kk = im[t] / (NX * NY);
        int gi = Immersed_get_ib_global_index(I, ii, jj, kk);
        ImmersedNode *nd = Immersed_get_ib_node(I, gi);
        nd->n_fluid = nf[t];
        nd->boundary_coef = bcoef[t];
        for (k = 0; k < nf[t]; k++) {
            int f = fidx[t * 8 + k];
            nd->fluid_index[k].x_index = f % NX;
            nd->fluid_index[k].y_index = (f / NX) % NY;
            nd->fluid_index[k].z_index = f / (NX * NY);
            nd->fluid_coef[k] = fcoef[t * 8 + k];
        }
    }
}

void ref_eno_line(ref_case *r, int order, int n, const double *D0, const double *P, const double *V, double *out)
{
    /* a scheme sized for this line (ENO_create sizes its buffers from NX/NY/NZ) */
    Parameters tmp = *r->p;
    ENO_Scheme *e;
    tmp.NX = n; tmp.NY = 1; tmp.NZ = 1; tmp.ENO_scheme_order = order;
    e = ENO_create(&tmp);
    memcpy(e->D0, D0, 8 * n); memcpy(e->Position, P, 8 * n); memcpy(e->Velocity, V, 8 * n);
    memset(e->VdQdX, 0, 8 * n);
    ENO_compute_convective_terms(e, n);
    memcpy(out, e->VdQdX, 8 * n);
    ENO_destroy(e);
}

static Velocity *vel_of(ref_case *r, char q) { return q == 'u' ? r->u : q == 'v' ? r->v : r->w; }

void ref_cell_center(ref_case *r, const double *u, const double *v, const double *w, double *ub, double *vb, double *wb)
{
    long n = r->n;
    vset(r->u->G_data, u, n); vset(r->v->G_data, v, n); vset(r->w->G_data, w, n);
    VecSet(r->u->G_data_bc, 0.0); VecSet(r->v->G_data_bc, 0.0); VecSet(r->w->G_data_bc, 0.0);
    Velocity_cell_center(r->u, r->v, r->w, r->g, r->p);
    vget(r->u->G_data_bc, ub, n); vget(r->v->G_data_bc, vb, n); vget(r->w->G_data_bc, wb, n);
}

void ref_transpose(ref_case *r, char q, const double *u, const double *v, const double *w, double *A, double *B)
{
    long n = r->n;
    vset(r->u->L_data, u, n); vset(r->v->L_data, v, n); vset(r->w->L_data, w, n);
    VecSet(r->g->G_dummy1, 0.0); VecSet(r->g->G_dummy2, 0.0);
    Velocity_transpose_velocities(r->u, r->v, r->w, r->g, r->p, q);
    vget(r->g->G_dummy1, A, n); vget(r->g->G_dummy2, B, n);
}

/* ghost cells of one line: buffer D0/P (length nbuf) holds the interior at
 * [order, nbuf-order); the routine fills the ghosts in place */
void ref_ghost_cells(ref_case *r, char q, int ic, char dir, int i0, int j0, int k0, int i1, int j1, int k1,
                     int nbuf, double *D0, double *P)
{
    ENO_Scheme *e = r->eno;
    Indices s, t;
    s.x_index = i0; s.y_index = j0; s.z_index = k0;
    t.x_index = i1; t.y_index = j1; t.z_index = k1;
    memcpy(e->D0, D0, 8 * nbuf); memcpy(e->Position, P, 8 * nbuf);
    if (q == 'u') Velocity_u_ENO_ghost_cells(e, r->u, r->g, r->p, s, t, dir);
    else if (q == 'v') Velocity_v_ENO_ghost_cells(e, r->v, r->g, r->p, s, t, dir);
    else if (q == 'w') Velocity_w_ENO_ghost_cells(e, r->w, r->g, r->p, s, t, dir);
    else Conc_ENO_ghost_cells(e, r->c[ic], r->g, r->p, s, t, dir);
    memcpy(D0, e->D0, 8 * nbuf); memcpy(P, e->Position, 8 * nbuf);
}

void ref_set_rhs_vel(ref_case *r, char q, double dt, const double *x, const double *conv, const double *dp,
                     const double *ctot, double *b)
{
    long n = r->n;
    Velocity *V = vel_of(r, q);
    vset(V->G_data, x, n);
    vset(V->G_conv, conv, n);
    if (q == 'u') { vset(r->pr->G_dp_dx, dp, n); Velocity_u_set_RHS(V, r->pr, r->g, r->p, dt); }
    else if (q == 'w') { vset(r->pr->G_dp_dz, dp, n); Velocity_w_set_RHS(V, r->pr, r->g, r->p, dt); }
    else {
        vset(r->pr->G_dp_dy, dp, n);
        if (r->p->NConc > 1) vset(r->c[0]->G_c_total, ctot, n);
        else vset(r->c[0]->G_data, ctot, n);
        Velocity_v_set_RHS(V, r->pr, r->c, r->g, r->p, dt);
    }
    vget(V->G_b, b, n);
}

void ref_set_rhs_conc(ref_case *r, int ic, double dt, const double *c, const double *conv, double *b)
{
    long n = r->n;
    vset(r->c[ic]->G_data, c, n);
    vset(r->c[ic]->G_conv, conv, n);
    Conc_set_RHS(r->c[ic], r->g, r->p, dt);
    vget(r->c[ic]->G_b, b, n);
}

void ref_total_concentration(ref_case *r, const double *const *c, double *ct)
{
    long n = r->n;
    int i;
    for (i = 0; i < r->p->NConc; i++) vset(r->c[i]->G_data, c[i], n);
    Conc_compute_total_concentration(r->c, r->p);
    vget(r->c[0]->G_c_total, ct, n);
}

/* y = (LHS + 1/dt on non-immersed rows) x, assembled by the reference */
void ref_lhs_apply(ref_case *r, char q, int ic, double dt, const double *x, double *y)
{
    Mat A;
    if (q == 'c') {
        Concentration *c = r->c[ic];
        MatDestroy(c->A);
        DAGetMatrix(r->g->DA_3D_Lsys, MATMPIAIJ, &c->A);
        Conc_form_LHS_matrix(c, r->g, r->p);
        Conc_modify_diagonal(c, r->g, dt, 0.0);
        A = c->A;
    } else {
        Velocity *V = vel_of(r, q);
        MatDestroy(V->A);
        DAGetMatrix(r->g->DA_3D_Lsys, MATMPIAIJ, &V->A);
        if (q == 'u') Velocity_u_form_LHS_matrix(V, r->g, r->p);
        else if (q == 'v') Velocity_v_form_LHS_matrix(V, r->g, r->p);
        else Velocity_w_form_LHS_matrix(V, r->g, r->p);
        Velocity_modify_diagonal(V, r->g, r->p, dt, 0.0);
        A = V->A;
    }
    shim_mat_mult(A, x, y);
}

/* y = A x with A assembled once and its diagonal updated by the reference's
 * modify_diagonal routine for each time step of dts in turn (dt_old = 0 for
 * the first, then the previous entry), as a run whose dt changes does: the
 * diagonal accumulates 1/dt0 + (1/dt1 - 1/dt0) + ..., a change of 1/dt of at
 * most 1e-10 is skipped, and IMMERSED rows never get the term
 * (Velocity.c:374-443, Conc.c:293-354) */
void ref_lhs_apply_dts(ref_case *r, char q, int ic, int ndt, const double *dts, const double *x, double *y)
{
    Mat A;
    int t;
    if (q == 'c') {
        Concentration *c = r->c[ic];
        MatDestroy(c->A);
        DAGetMatrix(r->g->DA_3D_Lsys, MATMPIAIJ, &c->A);
        Conc_form_LHS_matrix(c, r->g, r->p);
        for (t = 0; t < ndt; t++) Conc_modify_diagonal(c, r->g, dts[t], t ? dts[t - 1] : 0.0);
        A = c->A;
    } else {
        Velocity *V = vel_of(r, q);
        MatDestroy(V->A);
        DAGetMatrix(r->g->DA_3D_Lsys, MATMPIAIJ, &V->A);
        if (q == 'u') Velocity_u_form_LHS_matrix(V, r->g, r->p);
        else if (q == 'v') Velocity_v_form_LHS_matrix(V, r->g, r->p);
        else Velocity_w_form_LHS_matrix(V, r->g, r->p);
        for (t = 0; t < ndt; t++) Velocity_modify_diagonal(V, r->g, r->p, dts[t], t ? dts[t - 1] : 0.0);
        A = V->A;
    }
    shim_mat_mult(A, x, y);
}

/* the reference's linear solves (the shim's KSPSolve is BiCGStab without a
 * preconditioner, Solver.c's KSPIBCGS; for the pressure it stands in for
 * GMRES(20) + BoomerAMG): LHS formed and diagonal modified as ref_lhs_apply,
 * the KSP from Solver_get_*_solver (rtol = resmax), initial guess x.
 * Returns the iteration count. */
int ref_solve(ref_case *r, char q, int ic, double dt, const double *b, double *x)
{
    long n = r->n;
    int its;
    if (q == 'p') {
        Pressure *P = r->pr;
        MatDestroy(P->A);
        DAGetMatrix(r->g->DA_3D_Lsys, MATMPIAIJ, &P->A);
        Pressure_form_LHS_matrix(P, r->g);
        P->solver = Solver_get_pressure_solver(P->A, r->p);
        vset(P->G_b, b, n); vset(P->G_data, x, n);
        its = Pressure_solve(P);
        vget(P->G_data, x, n);
        KSPDestroy(P->solver);
        return its;
    }
    if (q == 'c') {
        Concentration *c = r->c[ic];
        MatDestroy(c->A);
        DAGetMatrix(r->g->DA_3D_Lsys, MATMPIAIJ, &c->A);
        Conc_form_LHS_matrix(c, r->g, r->p);
        Conc_modify_diagonal(c, r->g, dt, 0.0);
        c->solver = Solver_get_concentration_solver(c->A, r->p);
        vset(c->G_b, b, n); vset(c->G_data, x, n);
        its = Conc_solve(c);
        vget(c->G_data, x, n);
        KSPDestroy(c->solver);
        return its;
    } else {
        Velocity *V = vel_of(r, q);
        MatDestroy(V->A);
        DAGetMatrix(r->g->DA_3D_Lsys, MATMPIAIJ, &V->A);
        if (q == 'u') Velocity_u_form_LHS_matrix(V, r->g, r->p);
        else if (q == 'v') Velocity_v_form_LHS_matrix(V, r->g, r->p);
        else Velocity_w_form_LHS_matrix(V, r->g, r->p);
        Velocity_modify_diagonal(V, r->g, r->p, dt, 0.0);
        V->solver = Solver_get_velocity_solver(V->A, r->p);
        vset(V->G_b, b, n); vset(V->G_data, x, n);
        its = Velocity_solve(V);
        vget(V->G_data, x, n);
        KSPDestroy(V->solver);
        return its;
    }
}

void ref_pressure_apply(ref_case *r, const double *x, double *y)
{
    MatDestroy(r->pr->A);
    DAGetMatrix(r->g->DA_3D_Lsys, MATMPIAIJ, &r->pr->A);
    Pressure_form_LHS_matrix(r->pr, r->g);
    shim_mat_mult(r->pr->A, x, y);
}

void ref_pressure_rhs(ref_case *r, double dt, const double *u, const double *v, const double *w, double *b)
{
    long n = r->n;
    vset(r->u->L_data, u, n); vset(r->v->L_data, v, n); vset(r->w->L_data, w, n);
    Pressure_set_RHS(r->pr, r->u, r->v, r->w, r->g, r->p, dt);
    vget(r->pr->G_b, b, n);
}

void ref_project(ref_case *r, double dt, const double *phi, const double *pb, double *u, double *v, double *w,
                 double *dpx, double *dpy, double *dpz)
{
    long n = r->n;
    vset(r->pr->G_data, phi, n); vset(r->pr->G_b, pb, n);
    vset(r->u->G_data, u, n); vset(r->v->G_data, v, n); vset(r->w->G_data, w, n);
    vset(r->pr->G_dp_dx, dpx, n); vset(r->pr->G_dp_dy, dpy, n); vset(r->pr->G_dp_dz, dpz, n);
    Pressure_project_velocity(r->pr, r->u, r->v, r->w, r->g, r->p, dt);
    vget(r->u->G_data, u, n); vget(r->v->G_data, v, n); vget(r->w->G_data, w, n);
    vget(r->pr->G_dp_dx, dpx, n); vget(r->pr->G_dp_dy, dpy, n); vget(r->pr->G_dp_dz, dpz, n);
}

double ref_divergence(ref_case *r, const double *u, const double *v, const double *w, double *div)
{
    long n = r->n;
    double m;
    vset(r->u->G_data, u, n); vset(r->v->G_data, v, n); vset(r->w->G_data, w, n);
    m = Pressure_compute_velocity_divergence(r->pr, r->u, r->v, r->w, r->g, r->p);
    vget(r->pr->G_divergence, div, n);
    return m;
}

void ref_metrics(ref_case *r, double *mxc, double *myc, double *mzc, double *mxu, double *myv, double *mzw)
{
    MAC_grid *g = r->g;
    memcpy(mxc, g->metric_xc, 8 * g->NX); memcpy(myc, g->metric_yc, 8 * g->NY); memcpy(mzc, g->metric_zc, 8 * g->NZ);
    memcpy(mxu, g->metric_xu, 8 * g->NX); memcpy(myv, g->metric_yv, 8 * g->NY); memcpy(mzw, g->metric_zw, 8 * g->NZ);
}

static void bed_index(MAC_grid *g)
{
    if (!g->interface_y_index) g->interface_y_index = Memory_allocate_2D_int(g->NX, g->NZ);
    Grid_set_interface_y_index(g);
}

/* Grid_set_interface_y_index, copied out as iy[k * NX + i] */
void ref_interface_y_index(ref_case *r, int *iy)
{
    MAC_grid *g = r->g;
    int i, k;
    bed_index(g);
    for (k = 0; k < g->NZ; k++)
        for (i = 0; i < g->NX; i++) iy[(long)k * g->NX + i] = g->interface_y_index[k][i];
}

/* G_deposit_height of fraction ic <- dep (nconc x NZ x NX), or zeros */
static void set_deposit(ref_case *r, int ic, const double *dep)
{
    MAC_grid *g = r->g;
    Concentration *cc = r->c[ic];
    int i, k;
    if (!cc->G_deposit_height) cc->G_deposit_height = Memory_allocate_2D_double(g->NX, g->NZ);
    for (k = 0; k < g->NZ; k++)
        for (i = 0; i < g->NX; i++)
            cc->G_deposit_height[k][i] = dep ? dep[((long)ic * g->NZ + k) * g->NX + i] : 0.0;
}

/* Conc_integrate_deposited_height of every fraction (weight_factor =
 * Conc_alpha, as Conc_dump_particles weighs the deposit) on dep in place */
void ref_deposit_integrate(ref_case *r, const double *const *c, const double *const *c_old, double dt, double *dep)
{
    MAC_grid *g = r->g;
    int i, k, ic;
    bed_index(g);
    for (ic = 0; ic < r->p->NConc; ic++) {
        Concentration *cc = r->c[ic];
        set_deposit(r, ic, dep);
        vset(cc->G_data, c[ic], r->n);
        vset(cc->G_data_old, c_old[ic], r->n);
        Conc_integrate_deposited_height(cc, g, r->p->Conc_alpha[ic], dt);
        for (k = 0; k < g->NZ; k++)
            for (i = 0; i < g->NX; i++) dep[((long)ic * g->NZ + k) * g->NX + i] = cc->G_deposit_height[k][i];
    }
}

/* flow diagnostics through the reference's own routines:
 * out[0] = Extract_total_kinetic_energy, out[1] = Extract_kinetic_potential_conversion_rate,
 * per fraction i (base 2 + 4 i): Conc_compute_total_suspended_mass, and
 * Conc_compute_potential_energies' W_Ep, W_Stokes_dissipation_rate,
 * W_kinetic_potential_conversion_rate;
 * out[2 + 4 nconc] = Conc_find_front_location(front_limit);
 * out[3 + 4 nconc] = Extract_viscous_dissipation_rate;
 * per fraction i (base 4 + 4 nconc + 4 i): W_Ep_passive, W_Ep_passive_rate,
 * W_Ep_rate, Conc_compute_sedimentation_rate's W_sed_rate.
 * dep: deposited heights (nconc x NZ x NX) or NULL; h_ave (nconc x NX) =
 * Conc_compute_ave_height_x; sed_bottom (nconc x NZ x NX) = Conc_bottom_sed_rate. */
void ref_diagnostics(ref_case *r, const double *u, const double *v, const double *w, const double *const *c,
                     double front_limit, const double *dep, double *out, double *h_ave, double *sed_bottom)
{
    long n = r->n;
    int i, k, x, nc = r->p->NConc, NX = r->g->NX, NZ = r->g->NZ;
    MAC_grid *g = r->g;
    Parameters *p = r->p;
    double *ext = out + 3 + 4 * nc;
    bed_index(g);
    p->Ly = g->yv[g->NY - 1] - g->yv[0];
    p->Lz = g->zw[g->NZ - 1] - g->zw[0];
    vset(r->u->G_data, u, n); vset(r->v->G_data, v, n); vset(r->w->G_data, w, n);
    vset(r->u->L_data, u, n); vset(r->v->L_data, v, n); vset(r->w->L_data, w, n);
    Velocity_cell_center(r->u, r->v, r->w, g, p);
    for (i = 0; i < nc; i++) vset(r->c[i]->G_data, c[i], n);
    if (nc > 1) Conc_compute_total_concentration(r->c, p);
    Extract_total_kinetic_energy(r->u, r->v, r->w, g);
    Extract_kinetic_potential_conversion_rate(r->v, r->c, g, p);
    Extract_viscous_dissipation_rate(r->u, r->v, r->w, g, p);
    out[0] = r->u->W_kinetic_energy;
    out[1] = r->v->W_kinetic_potential_conversion_rate;
    ext[0] = r->u->W_dissipation_rate;
    for (i = 0; i < nc; i++) {
        Concentration *cc = r->c[i];
        set_deposit(r, i, dep);
        if (!cc->G_sed_rate_bottom) {
            cc->G_sed_rate_bottom = Memory_allocate_2D_double(NX, NZ);
            cc->W_sed_rate_bottom = Memory_allocate_2D_double(NX, NZ);
        }
        Conc_compute_total_suspended_mass(cc, g);
        Conc_compute_potential_energies(cc, r->v, g, p);
        Conc_compute_sedimentation_rate(cc, g, p);
        Conc_bottom_sed_rate(cc, g, p);
        out[2 + 4 * i] = cc->W_total_susp_mass;
        out[3 + 4 * i] = cc->W_Ep;
        out[4 + 4 * i] = cc->W_Stokes_dissipation_rate;
        out[5 + 4 * i] = cc->W_kinetic_potential_conversion_rate;
        ext[1 + 4 * i] = cc->W_Ep_passive;
        ext[2 + 4 * i] = cc->W_Ep_passive_rate;
        ext[3 + 4 * i] = cc->W_Ep_rate;
        ext[4 + 4 * i] = cc->W_sed_rate;
        if (sed_bottom)
            for (k = 0; k < NZ; k++)
                for (x = 0; x < NX; x++)
                    sed_bottom[((long)i * NZ + k) * NX + x] =
                        cc->Type == PARTICLE ? cc->W_sed_rate_bottom[k][x] : 0.0;
    }
    for (i = 0; i < nc; i++) {   /* Conc_create leaves them unset without ave_height_output */
        if (!r->hbuf[i]) {
            r->hbuf[i] = Memory_allocate_1D_double(g->NX);
            r->hbuf[4 + i] = Memory_allocate_1D_double(g->NX);
        }
        r->c[i]->G_ave_height_x = r->hbuf[i];
        r->c[i]->W_ave_height_x = r->hbuf[4 + i];
    }
    Conc_compute_ave_height_x(r->c, g, p);
    out[2 + 4 * nc] = Conc_find_front_location(r->c, g, p, front_limit);
    if (h_ave)
        for (i = 0; i < nc; i++) memcpy(h_ave + (long)i * NX, r->c[i]->W_ave_height_x, sizeof(double) * NX);
}

/* ---- restart files through Resume.c --------------------------------------
 * Resume_set_data / Resume_write_data / Resume_write_primary_data in the
 * directory dir (the reference writes to the working directory), and
 * Resume_write_2D_data of each fraction's deposited height to
 * "Resume_deposit_height<i>.bin" (the reference ships no caller of it; the
 * name is this harness's).  fields: u, v, w, dp_dx, dp_dy, dp_dz, c_0.. */
static Resume *resume_of(ref_case *r, int grid_flag, GVG_bag *bag)
{
    Resume *rs = Resume_create(6 + r->p->NConc + (grid_flag ? 1 : 0));
    Resume_reset_read_flag(rs);
    Resume_reset_write_flag(rs);
    if (grid_flag) Resume_set_IO_grid_flag(rs); else Resume_reset_IO_grid_flag(rs);
    memset(bag, 0, sizeof(*bag));
    bag->u = r->u; bag->v = r->v; bag->w = r->w; bag->p = r->pr; bag->c = r->c;
    bag->grid = r->g; bag->params = r->p;
    Resume_set_data(rs, bag);
    return rs;
}

static void dep_name(char *s, int ic) { sprintf(s, "Resume_deposit_height%d.bin", ic); }

int ref_resume_write(ref_case *r, const char *dir, const double *const *fields, int grid_flag, double time,
                     double dt, double dt_old, int iter, int output_iter, const double *dep)
{
    char cwd[4096], name[64];
    GVG_bag bag;
    Resume *rs;
    int i, k, ic, nc = r->p->NConc;
    MAC_grid *g = r->g;
    Vec *v[6];
    if (!getcwd(cwd, sizeof(cwd)) || chdir(dir)) return 1;
    v[0] = &r->u->G_data; v[1] = &r->v->G_data; v[2] = &r->w->G_data;
    v[3] = &r->pr->G_dp_dx; v[4] = &r->pr->G_dp_dy; v[5] = &r->pr->G_dp_dz;
    for (i = 0; i < 6; i++) vset(*v[i], fields[i], r->n);
    for (i = 0; i < nc; i++) vset(r->c[i]->G_data, fields[6 + i], r->n);
    rs = resume_of(r, grid_flag, &bag);
    bag.time = time; bag.dt = dt; bag.dt_old = dt_old; bag.iter = iter; bag.output_iter = output_iter;
    Resume_write_data(rs);
    Resume_write_primary_data(rs, &bag);
    if (dep)   /* G_deposit_height exists for particle fractions only (Conc.c:188-199) */
        for (ic = 0; ic < nc; ic++) {
            Concentration *cc = r->c[ic];
            if (cc->Type != PARTICLE) continue;
            set_deposit(r, ic, dep);
            dep_name(name, ic);
            Resume_write_2D_data(rs, cc->G_deposit_height, name, g->NX, g->NZ);
        }
    (void)k;
    Resume_destroy(rs);
    return chdir(cwd) ? 1 : 0;
}

/* the reverse: Resume_read_data, Resume_read_primary_data and
 * Resume_read_2D_data; prim = {time, dt, dt_old, iter, output_iter} */
int ref_resume_read(ref_case *r, const char *dir, double *const *fields, int grid_flag, double *prim, double *dep)
{
    char cwd[4096], name[64];
    GVG_bag bag;
    Resume *rs;
    int i, k, x, ic, nc = r->p->NConc;
    MAC_grid *g = r->g;
    if (!getcwd(cwd, sizeof(cwd)) || chdir(dir)) return 1;
    rs = resume_of(r, grid_flag, &bag);
    Resume_read_data(rs);
    Resume_read_primary_data(rs, &bag);
    vget(r->u->G_data, fields[0], r->n); vget(r->v->G_data, fields[1], r->n); vget(r->w->G_data, fields[2], r->n);
    vget(r->pr->G_dp_dx, fields[3], r->n); vget(r->pr->G_dp_dy, fields[4], r->n);
    vget(r->pr->G_dp_dz, fields[5], r->n);
    for (i = 0; i < nc; i++) vget(r->c[i]->G_data, fields[6 + i], r->n);
    prim[0] = bag.time; prim[1] = bag.dt; prim[2] = bag.dt_old; prim[3] = bag.iter; prim[4] = bag.output_iter;
    if (dep)
        for (ic = 0; ic < nc; ic++) {
            Concentration *cc = r->c[ic];
            set_deposit(r, ic, NULL);
            if (cc->Type != PARTICLE) continue;
            dep_name(name, ic);
            Resume_read_2D_data(rs, cc->G_deposit_height, name, g->NX, g->NZ);
            for (k = 0; k < g->NZ; k++)
                for (x = 0; x < g->NX; x++) dep[((long)ic * g->NZ + k) * g->NX + x] = cc->G_deposit_height[k][x];
        }
    Resume_destroy(rs);
    return chdir(cwd) ? 1 : 0;
}

/* ---- open boundaries (Inflow.c, Outflow.c and the inflow / outflow
 * branches of the step routines) ----------------------------------------
 * ref_set_open turns params->inflow / outflow on and allocates the 2-D
 * [NZ][NY] arrays Velocity_create / Conc_create would have made
 * (Velocity.c:128-158, Conc.c:67-98).  Arrays are exchanged flat, j fastest. */
#include "Inflow.h"
#include "Outflow.h"

void ref_set_open(ref_case *r, int inflow, int outflow, double U, int transient, double time_c, double Ly,
                  double Lz)
{
    MAC_grid *g = r->g;
    Parameters *p = r->p;
    int i;
    Velocity *V[3] = {r->u, r->v, r->w};
    p->inflow = (short)inflow;
    p->outflow = (short)outflow;
    p->U = U;
    p->transient_inflow = (short)transient;
    p->time_c = time_c;
    p->Ly = Ly;
    p->Lz = Lz;
    for (i = 0; i < 3; i++) {
        if (outflow && !V[i]->G_outflow) {
            V[i]->G_outflow = Memory_allocate_2D_double(g->NY, g->NZ);
            V[i]->G_outflow_old = Memory_allocate_2D_double(g->NY, g->NZ);
        }
    }
    if (inflow && !r->u->G_inflow) r->u->G_inflow = Memory_allocate_2D_double(g->NY, g->NZ);
    for (i = 0; i < p->NConc; i++) {
        Concentration *c = r->c[i];
        if (outflow && !c->G_outflow) {
            c->G_outflow = Memory_allocate_2D_double(g->NY, g->NZ);
            c->G_outflow_old = Memory_allocate_2D_double(g->NY, g->NZ);
        }
        if (inflow && !c->G_inflow) c->G_inflow = Memory_allocate_2D_double(g->NY, g->NZ);
    }
}

/* which: 0 inflow, 1 outflow, 2 outflow_old; q: 'u', 'v', 'w', 'c' (ic) */
static double **open_arr(ref_case *r, int which, char q, int ic)
{
    if (q == 'c') {
        Concentration *c = r->c[ic];
        return which == 0 ? c->G_inflow : which == 1 ? c->G_outflow : c->G_outflow_old;
    } else {
        Velocity *V = vel_of(r, q);
        return which == 0 ? V->G_inflow : which == 1 ? V->G_outflow : V->G_outflow_old;
    }
}

void ref_open_set(ref_case *r, int which, char q, int ic, const double *a)
{
    double **d = open_arr(r, which, q, ic);
    int j, k;
    for (k = 0; k < r->g->NZ; k++)
        for (j = 0; j < r->g->NY; j++) d[k][j] = a[(long)k * r->g->NY + j];
}

void ref_open_get(ref_case *r, int which, char q, int ic, double *a)
{
    double **d = open_arr(r, which, q, ic);
    int j, k;
    for (k = 0; k < r->g->NZ; k++)
        for (j = 0; j < r->g->NY; j++) a[(long)k * r->g->NY + j] = d[k][j];
}

/* Inflow_u_velocity_profile (returns W_influx) and Inflow_conc_profile */
double ref_inflow_u(ref_case *r, double time)
{
    Inflow_u_velocity_profile(r->u, r->g, r->p, time);
    return r->u->W_influx;
}

void ref_inflow_c(ref_case *r, int ic, double time) { Inflow_conc_profile(r->c[ic], r->g, r->p, time); }

/* Outflow_vel_impose_convective_boundary (with the mass correction for u,
 * from the influx `influx`) / Outflow_conc_impose_convective_boundary on the
 * field x */
void ref_outflow_impose(ref_case *r, char q, int ic, double dt, const double *x, double influx)
{
    if (q == 'c') {
        vset(r->c[ic]->G_data, x, r->n);
        Outflow_conc_impose_convective_boundary(r->c[ic], r->g, r->p, dt);
    } else {
        Velocity *V = vel_of(r, q);
        vset(V->G_data, x, r->n);
        r->u->W_influx = influx;
        Outflow_vel_impose_convective_boundary(V, r->g, r->p, dt);
    }
}

/* *_store_old_outflow and *_rk_average_outflow of one quantity */
void ref_outflow_store_old(ref_case *r, char q, int ic)
{
    if (q == 'c') Conc_store_old_outflow(r->c[ic]);
    else Velocity_store_old_outflow(vel_of(r, q));
}

void ref_outflow_rk_average(ref_case *r, char q, int ic, double old_frac, double new_frac)
{
    if (q == 'c') Conc_rk_average_outflow(r->c[ic], old_frac, new_frac);
    else Velocity_rk_average_outflow(vel_of(r, q), old_frac, new_frac);
}

/* Outflow_*_copy_data_into_last_plane (field x in / out) and
 * Outflow_*_copy_data_into_2D_array */
void ref_outflow_to_plane(ref_case *r, char q, int ic, int should_set, double *x)
{
    if (q == 'c') {
        vset(r->c[ic]->G_data, x, r->n);
        Outflow_concentration_copy_data_into_last_plane(r->c[ic], r->g, should_set);
        vget(r->c[ic]->G_data, x, r->n);
    } else {
        Velocity *V = vel_of(r, q);
        vset(V->G_data, x, r->n);
        Outflow_vel_copy_data_into_last_plane(V, r->g, should_set);
        vget(V->G_data, x, r->n);
    }
}

void ref_outflow_from_plane(ref_case *r, char q, int ic, const double *x)
{
    if (q == 'c') {
        vset(r->c[ic]->G_data, x, r->n);
        Outflow_concentration_copy_data_into_2D_array(r->c[ic], r->g);
    } else {
        Velocity *V = vel_of(r, q);
        vset(V->G_data, x, r->n);
        Outflow_vel_copy_data_into_2D_array(V, r->g);
    }
}

/* ---- immersed-boundary geometry ------------------------------------------
 * The reference's set-up of a bottom topography y = h(x, z): the sdf guess
 * yc - interface_position (Surface_initialize, Surface.c:96-195), level-set
 * reinitialisation (Surface_find_exact_sdf -> Levelset_reinitialize,
 * Levelset.c:85-160), sdf at the u, v, w nodes (Surface_find_q_sdf,
 * Surface.c:216-336) and the node status (Grid_identify_geometry,
 * Grid.c:1825-1871: box boundaries, surface tagging, BUFFER_SOLID layers,
 * interface index).  ipos: [NZ][NX] interface heights at the cell centres.
 * Outputs: sdf of c, u, v, w (DA arrays) and the four status arrays as codes. */
#include "Surface.h"
#include "Levelset.h"

void ref_geometry(ref_case *r, const double *ipos, double *c_sdf, double *u_sdf, double *v_sdf, double *w_sdf,
                  unsigned char *st_out)
{
    MAC_grid *g = r->g;
    Parameters *p = r->p;
    int i, k, q;
    long t;
    Vec *gs[4];
    if (!g->interface_position) g->interface_position = Memory_allocate_2D_double(g->NX, g->NZ);
    for (k = 0; k < g->NZ; k++)
        for (i = 0; i < g->NX; i++) g->interface_position[k][i] = ipos[(long)k * g->NX + i];
    p->Lx = g->xu[g->NX - 1] - g->xu[0];
    p->Ly = g->yv[g->NY - 1] - g->yv[0];
    p->Lz = g->zw[g->NZ - 1] - g->zw[0];
    if (!g->interface_y_index) g->interface_y_index = Memory_allocate_2D_int(g->NX, g->NZ);
    g->surf = Surface_create(g);
    Surface_initialize(g->surf, g, p);
    Surface_find_exact_sdf(g->surf, g);
    Surface_find_q_sdf(g->surf, g);
    Grid_identify_geometry(g);
    vget(g->surf->G_c_sdf, c_sdf, r->n);
    vget(g->surf->G_u_sdf, u_sdf, r->n);
    vget(g->surf->G_v_sdf, v_sdf, r->n);
    vget(g->surf->G_w_sdf, w_sdf, r->n);
    gs[0] = &g->G_u_status; gs[1] = &g->G_v_status; gs[2] = &g->G_w_status; gs[3] = &g->G_c_status;
    for (q = 0; q < 4; q++) {
        const double *a = shim_vec_data(*gs[q]);
        for (t = 0; t < r->n; t++) st_out[(long)q * r->n + t] = (unsigned char)a[t];
    }
}

/* The reference's ghost-cell stencils of quantity q built from the current
 * geometry (call ref_geometry first): Immersed_setup_q_immersed_nodes
 * (Immersed.c:546-616: indices in DA order, coordinates, normals, control and
 * image points, boundary condition, 8-node box or nearest fluid node,
 * Dirichlet / Neumann coefficients).  Returns N; with cap >= N the arrays get
 * im (DA linear index), nf, fidx[8] (DA linear), fcoef[8], bcoef and pts[12]
 * (normal, control, image point, im_point). */
int ref_immersed(ref_case *r, char q, int cap, int *im, int *nf, int *fidx, double *fcoef, double *bcoef,
                 double *pts)
{
    MAC_grid *g = r->g;
    Immersed *I;
    int t, m;
    long NX = g->NX, NY = g->NY;
    Immersed_setup_q_immersed_nodes(g, q);
    I = q == 'u' ? g->u_immersed : q == 'v' ? g->v_immersed : q == 'w' ? g->w_immersed : g->c_immersed;
    if (I->N > cap) return I->N;
    for (t = 0; t < I->N; t++) {
        ImmersedNode *nd = &I->ib_nodes[t];
        im[t] = (int)((nd->im_index.z_index * NY + nd->im_index.y_index) * NX + nd->im_index.x_index);
        nf[t] = nd->n_fluid;
        for (m = 0; m < 8; m++) {
            if (m < nd->n_fluid) {
                fidx[t * 8 + m] = (int)((nd->fluid_index[m].z_index * NY + nd->fluid_index[m].y_index) * NX +
                                        nd->fluid_index[m].x_index);
                fcoef[t * 8 + m] = nd->fluid_coef[m];
            } else {
                fidx[t * 8 + m] = 0;
                fcoef[t * 8 + m] = 0.0;
            }
        }
        bcoef[t] = nd->boundary_coef;
        pts[t * 12 + 0] = nd->n.vx; pts[t * 12 + 1] = nd->n.vy; pts[t * 12 + 2] = nd->n.vz;
        pts[t * 12 + 3] = nd->control_point.x; pts[t * 12 + 4] = nd->control_point.y;
        pts[t * 12 + 5] = nd->control_point.z;
        pts[t * 12 + 6] = nd->image_point.x; pts[t * 12 + 7] = nd->image_point.y; pts[t * 12 + 8] = nd->image_point.z;
        pts[t * 12 + 9] = nd->im_point.x; pts[t * 12 + 10] = nd->im_point.y; pts[t * 12 + 11] = nd->im_point.z;
    }
    return I->N;
}
