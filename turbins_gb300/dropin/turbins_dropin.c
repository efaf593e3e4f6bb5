/*
 * turbins_dropin.c -- the reference's hot-path routines under their own
 * names and signatures (Include/Velocity.h, Conc.h, Pressure.h, ENO.h),
 * each forwarding to the GPU implementation in libturbgpu.so.
 *
 * Every struct pointer is a key: turb_dropin_bind_* records which device
 * state (context, field) it stands for, and the routines look the key up.
 * Nothing here reads a reference struct, so the file builds against the
 * opaque declarations of include/turbins_dropin.h alone; built with
 * -DTURB_DROPIN_REFERENCE_HEADERS and the reference's Include directory (and
 * PETSc's) on the include path, it also includes the reference's headers so
 * that the compiler checks each definition against the reference prototype.
 * Host data moves only in turb_dropin_upload / turb_dropin_download, through
 * PETSc's VecGetArray / VecRestoreArray (a single-rank DA vector holds the
 * field contiguously in DA order).
 */
#ifdef TURB_DROPIN_REFERENCE_HEADERS
#include "definitions.h"
#include "DataTypes.h"
#include "Velocity.h"
#include "Conc.h"
#include "Pressure.h"
#include "ENO.h"
#endif
#include "../../include/turbins_dropin.h"

#include <stdio.h>
#include <string.h>

#ifndef TURB_DROPIN_REFERENCE_HEADERS
/* PETSc 3.1 (petscvec.h) */
int VecGetArray(Vec v, double **a);
int VecRestoreArray(Vec v, double **a);
int VecGetSize(Vec v, int *n);
#endif

#define MAXGRID 16
#define MAXKEY 64

enum { K_VEL = 1, K_CONC, K_PRES, K_ENO, K_BAG };

typedef struct {
    const void *key;
    int kind;
    MAC_grid *grid;
    int field;        /* TURB_F_U.. / TURB_F_C0 + ic; the Pressure: TURB_F_PHI */
    int ic;           /* fraction, or the velocity component 0..2 */
    double dt;        /* set by *_modify_diagonal: the dt of the next solve */
    Vec vec[4];       /* bound host vectors (pressure: phi, dp_dx, dp_dy, dp_dz) */
    int nvec;
    int order;        /* ENO */
    double *buf[4];   /* ENO: D0, Position, Velocity, VdQdX */
} binding;

static struct { MAC_grid *grid; turb_ctx *ctx; } g_grids[MAXGRID];
static binding g_keys[MAXKEY];
static int g_status = 0;

static void note(int rc, const char *what)
{
    if (rc != TURB_OK && g_status == TURB_OK) {
        g_status = rc;
        fprintf(stderr, "turbins_dropin: %s: %s\n", what, turb_status_string(rc));
    }
}

static turb_ctx *ctx_of(MAC_grid *grid)
{
    int i;
    for (i = 0; i < MAXGRID; i++)
        if (g_grids[i].grid == grid && grid) return g_grids[i].ctx;
    return NULL;
}

static binding *find(const void *key, int kind)
{
    int i;
    for (i = 0; i < MAXKEY; i++)
        if (g_keys[i].key == key && key && g_keys[i].kind == kind) return &g_keys[i];
    return NULL;
}

static binding *slot(const void *key, int kind)
{
    binding *b = find(key, kind);
    int i;
    if (b) return b;
    for (i = 0; i < MAXKEY; i++)
        if (!g_keys[i].key) {
            memset(&g_keys[i], 0, sizeof(binding));
            g_keys[i].key = key;
            g_keys[i].kind = kind;
            return &g_keys[i];
        }
    return NULL;
}

/* context and binding of a struct key; records TURB_ERR_ARG when unbound */
static turb_ctx *lookup(const void *key, int kind, binding **out, const char *what)
{
    binding *b = find(key, kind);
    turb_ctx *c = b ? ctx_of(b->grid) : NULL;
    if (!c) note(TURB_ERR_ARG, what);
    if (out) *out = b;
    return c;
}

int turb_dropin_status(void)
{
    int s = g_status;
    g_status = TURB_OK;
    return s;
}

int turb_dropin_bind_grid(MAC_grid *grid, turb_ctx *ctx)
{
    int i;
    if (!grid || !ctx) return TURB_ERR_ARG;
    for (i = 0; i < MAXGRID; i++)
        if (g_grids[i].grid == grid) { g_grids[i].ctx = ctx; return TURB_OK; }
    for (i = 0; i < MAXGRID; i++)
        if (!g_grids[i].grid) { g_grids[i].grid = grid; g_grids[i].ctx = ctx; return TURB_OK; }
    return TURB_ERR_ARG;
}

int turb_dropin_unbind_grid(MAC_grid *grid)
{
    int i;
    if (!grid) return TURB_ERR_ARG;
    for (i = 0; i < MAXKEY; i++)
        if (g_keys[i].key && g_keys[i].grid == grid) memset(&g_keys[i], 0, sizeof(binding));
    for (i = 0; i < MAXGRID; i++)
        if (g_grids[i].grid == grid) { g_grids[i].grid = NULL; g_grids[i].ctx = NULL; }
    return TURB_OK;
}

int turb_dropin_bind_velocity(Velocity *vel, MAC_grid *grid, char component, Vec data)
{
    int q = component == 'u' ? 0 : component == 'v' ? 1 : component == 'w' ? 2 : -1;
    binding *b;
    if (!vel || q < 0 || !ctx_of(grid)) return TURB_ERR_ARG;
    if (!(b = slot(vel, K_VEL))) return TURB_ERR_ARG;
    b->grid = grid;
    b->field = TURB_F_U + q;
    b->ic = q;
    b->vec[0] = data;
    b->nvec = data ? 1 : 0;
    return TURB_OK;
}

int turb_dropin_bind_conc(Concentration *c, MAC_grid *grid, int ic, Vec data)
{
    binding *b;
    if (!c || ic < 0 || ic >= TURB_MAXCONC || !ctx_of(grid)) return TURB_ERR_ARG;
    if (!(b = slot(c, K_CONC))) return TURB_ERR_ARG;
    b->grid = grid;
    b->field = TURB_F_C0 + ic;
    b->ic = ic;
    b->vec[0] = data;
    b->nvec = data ? 1 : 0;
    return TURB_OK;
}

int turb_dropin_bind_pressure(Pressure *p, MAC_grid *grid, Vec phi, Vec dp_dx, Vec dp_dy, Vec dp_dz)
{
    binding *b;
    if (!p || !ctx_of(grid)) return TURB_ERR_ARG;
    if (!(b = slot(p, K_PRES))) return TURB_ERR_ARG;
    b->grid = grid;
    b->field = TURB_F_PHI;
    b->vec[0] = phi;
    b->vec[1] = dp_dx;
    b->vec[2] = dp_dy;
    b->vec[3] = dp_dz;
    b->nvec = 4;
    return TURB_OK;
}

int turb_dropin_bind_eno(ENO_Scheme *eno, int order, double *D0, double *Position, double *Velocity_,
                         double *VdQdX)
{
    binding *b;
    if (!eno || order < 1 || order > 3 || !D0 || !Position || !Velocity_ || !VdQdX) return TURB_ERR_ARG;
    if (!(b = slot(eno, K_ENO))) return TURB_ERR_ARG;
    b->order = order;
    b->buf[0] = D0;
    b->buf[1] = Position;
    b->buf[2] = Velocity_;
    b->buf[3] = VdQdX;
    return TURB_OK;
}

/* the device field of the v-th vector of binding b */
static int field_of(const binding *b, int v)
{
    if (b->kind == K_PRES) return v == 0 ? TURB_F_PHI : TURB_F_DPX + (v - 1);
    return b->field;
}

static int transfer(MAC_grid *grid, int up)
{
    turb_ctx *c = ctx_of(grid);
    int i, v, rc = TURB_OK;
    if (!c) return TURB_ERR_ARG;
    for (i = 0; i < MAXKEY && rc == TURB_OK; i++) {
        binding *b = &g_keys[i];
        if (!b->key || b->grid != grid) continue;
        for (v = 0; v < b->nvec && rc == TURB_OK; v++) {
            double *a = NULL;
            if (!b->vec[v]) continue;
            if (VecGetArray(b->vec[v], &a) != 0 || !a) return TURB_ERR_ARG;
            rc = up ? turb_field_upload(c, field_of(b, v), a) : turb_field_download(c, field_of(b, v), a);
            VecRestoreArray(b->vec[v], &a);
        }
    }
    if (rc == TURB_OK) rc = turb_synchronize(c);
    return rc;
}

int turb_dropin_upload(MAC_grid *grid) { return transfer(grid, 1); }
int turb_dropin_download(MAC_grid *grid) { return transfer(grid, 0); }

/* ---- the fused step ------------------------------------------------------ */

int turb_dropin_bind_bag(GVG_bag *bag, MAC_grid *grid)
{
    binding *b;
    if (!bag || !ctx_of(grid)) return TURB_ERR_ARG;
    if (!(b = slot(bag, K_BAG))) return TURB_ERR_ARG;
    b->grid = grid;
    return TURB_OK;
}

int turb_dropin_step(GVG_bag *bag, double dt, int *status)
{
    turb_ctx *c = lookup(bag, K_BAG, NULL, "turb_dropin_step");
    int rc = c ? turb_step(c, dt, NULL) : TURB_ERR_ARG;
    if (c) note(rc, "turb_dropin_step");
    if (status) *status = rc;
    return rc;
}

/* ---- Include/Velocity.h -------------------------------------------------- */

/* Velocity_store_old_data, Velocity.c:297 */
void Velocity_store_old_data(Velocity *vel)
{
    binding *b;
    turb_ctx *c = lookup(vel, K_VEL, &b, "Velocity_store_old_data");
    if (c) note(turb_store_old_field(c, b->field), "Velocity_store_old_data");
}

/* Velocity_cell_center, Velocity.c:1476-1602 */
void Velocity_cell_center(Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid, Parameters *params)
{
    turb_ctx *c = ctx_of(grid);
    (void)u; (void)v; (void)w; (void)params;
    if (!c) { note(TURB_ERR_ARG, "Velocity_cell_center"); return; }
    note(turb_Velocity_cell_center(c), "Velocity_cell_center");
}

static void set_rhs(Velocity *vel, MAC_grid *grid, double dt, const char *what)
{
    binding *b;
    turb_ctx *c = lookup(vel, K_VEL, &b, what);
    if (!c) return;
    if (b->grid != grid) { note(TURB_ERR_ARG, what); return; }
    note(turb_Velocity_set_RHS(c, "uvw"[b->ic], dt), what);
}

/* Velocity_u_set_RHS, Velocity.c:1607-1750 */
void Velocity_u_set_RHS(Velocity *u, Pressure *p, MAC_grid *grid, Parameters *params, double dt)
{
    (void)p; (void)params;
    set_rhs(u, grid, dt, "Velocity_u_set_RHS");
}

/* Velocity_v_set_RHS, Velocity.c:1755-1927 (buoyancy from the context's
 * parameters: on unless turb_params.buoyancy is 0; the shipped routine
 * multiplies it by 0.0, Velocity.c:1883) */
void Velocity_v_set_RHS(Velocity *v, Pressure *p, Concentration **cc, MAC_grid *grid, Parameters *params,
                        double dt)
{
    (void)p; (void)cc; (void)params;
    set_rhs(v, grid, dt, "Velocity_v_set_RHS");
}

/* Velocity_w_set_RHS, Velocity.c:1932-2043 */
void Velocity_w_set_RHS(Velocity *w, Pressure *p, MAC_grid *grid, Parameters *params, double dt)
{
    (void)p; (void)params;
    set_rhs(w, grid, dt, "Velocity_w_set_RHS");
}

/* Velocity_rk_average, Velocity.c:2047-2055 */
void Velocity_rk_average(Velocity *vel, double old_frac, double new_frac)
{
    binding *b;
    turb_ctx *c = lookup(vel, K_VEL, &b, "Velocity_rk_average");
    if (c) note(turb_rk_average_field(c, b->field, old_frac, new_frac), "Velocity_rk_average");
}

/* Velocity_modify_diagonal, Velocity.c:374-443: the library keeps the 1/dt
 * term of each system by the same rule when the solve runs; the dt is kept
 * for the next Velocity_solve */
void Velocity_modify_diagonal(Velocity *vel, MAC_grid *grid, Parameters *params, double dt, double dt_old)
{
    binding *b;
    turb_ctx *c = lookup(vel, K_VEL, &b, "Velocity_modify_diagonal");
    (void)grid; (void)params; (void)dt_old;
    if (c) b->dt = dt;
}

/* Velocity_solve, Velocity.c:306-324: returns the iteration count */
int Velocity_solve(Velocity *vel)
{
    binding *b;
    int it = 0, rc;
    turb_ctx *c = lookup(vel, K_VEL, &b, "Velocity_solve");
    if (!c) return -1;
    if (!(b->dt > 0.0)) { note(TURB_ERR_ARG, "Velocity_solve (no Velocity_modify_diagonal)"); return -1; }
    rc = turb_Velocity_solve(c, "uvw"[b->ic], b->dt, &it);
    note(rc, "Velocity_solve");
    return rc == TURB_OK ? it : -1;
}

/* Velocity_transpose_velocities, Velocity.c:3341-3663 */
void Velocity_transpose_velocities(Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid, Parameters *params,
                                   char which_quantity)
{
    turb_ctx *c = ctx_of(grid);
    (void)u; (void)v; (void)w; (void)params;
    if (!c) { note(TURB_ERR_ARG, "Velocity_transpose_velocities"); return; }
    note(turb_Velocity_transpose_velocities(c, which_quantity), "Velocity_transpose_velocities");
}

/* ---- Include/Conc.h ------------------------------------------------------ */

/* Conc_modify_diagonal, Conc.c:293-354 (see Velocity_modify_diagonal) */
void Conc_modify_diagonal(Concentration *cc, MAC_grid *grid, double dt, double dt_old)
{
    binding *b;
    turb_ctx *c = lookup(cc, K_CONC, &b, "Conc_modify_diagonal");
    (void)grid; (void)dt_old;
    if (c) b->dt = dt;
}

/* Conc_rk_average, Conc.c:1007-1017 */
void Conc_rk_average(Concentration *cc, double old_frac, double new_frac)
{
    binding *b;
    turb_ctx *c = lookup(cc, K_CONC, &b, "Conc_rk_average");
    if (c) note(turb_rk_average_field(c, b->field, old_frac, new_frac), "Conc_rk_average");
}

/* Conc_set_particle_v_velocity, Conc.c:734-761 */
void Conc_set_particle_v_velocity(Concentration *cc, Velocity *v, Parameters *params)
{
    binding *b;
    turb_ctx *c = lookup(cc, K_CONC, &b, "Conc_set_particle_v_velocity");
    (void)v; (void)params;
    if (c) note(turb_Conc_set_particle_v_velocity(c, b->ic), "Conc_set_particle_v_velocity");
}

/* Conc_solve, Conc.c:840-859: returns the iteration count */
int Conc_solve(Concentration *cc)
{
    binding *b;
    int it = 0, rc;
    turb_ctx *c = lookup(cc, K_CONC, &b, "Conc_solve");
    if (!c) return -1;
    if (!(b->dt > 0.0)) { note(TURB_ERR_ARG, "Conc_solve (no Conc_modify_diagonal)"); return -1; }
    rc = turb_Conc_solve(c, b->ic, b->dt, &it);
    note(rc, "Conc_solve");
    return rc == TURB_OK ? it : -1;
}

/* Conc_set_RHS, Conc.c:864-992 */
void Conc_set_RHS(Concentration *cc, MAC_grid *grid, Parameters *params, double dt)
{
    binding *b;
    turb_ctx *c = lookup(cc, K_CONC, &b, "Conc_set_RHS");
    (void)grid; (void)params;
    if (c) note(turb_Conc_set_RHS(c, b->ic, dt), "Conc_set_RHS");
}

/* Conc_store_old_data, Conc.c:997 */
void Conc_store_old_data(Concentration *cc)
{
    binding *b;
    turb_ctx *c = lookup(cc, K_CONC, &b, "Conc_store_old_data");
    if (c) note(turb_store_old_field(c, b->field), "Conc_store_old_data");
}

/* Conc_compute_total_concentration, Conc.c:1291-1314 (c: the NConc fractions) */
void Conc_compute_total_concentration(Concentration **cc, Parameters *params)
{
    binding *b;
    turb_ctx *c = lookup(cc ? cc[0] : NULL, K_CONC, &b, "Conc_compute_total_concentration");
    (void)params;
    if (c) note(turb_Conc_compute_total_concentration(c), "Conc_compute_total_concentration");
}

/* ---- Include/Pressure.h -------------------------------------------------- */

/* Pressure_set_RHS, Pressure.c:171-276 */
void Pressure_set_RHS(Pressure *p, Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid, Parameters *params,
                      double dt)
{
    turb_ctx *c = lookup(p, K_PRES, NULL, "Pressure_set_RHS");
    (void)u; (void)v; (void)w; (void)grid; (void)params;
    if (c) note(turb_Pressure_set_RHS(c, dt), "Pressure_set_RHS");
}

/* Pressure_project_velocity, Pressure.c:280-439 */
void Pressure_project_velocity(Pressure *p, Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid,
                               Parameters *params, double dt)
{
    turb_ctx *c = lookup(p, K_PRES, NULL, "Pressure_project_velocity");
    (void)u; (void)v; (void)w; (void)grid; (void)params;
    if (c) note(turb_Pressure_project_velocity(c, dt), "Pressure_project_velocity");
}

/* Pressure_solve, Pressure.c:443-458 (GMRES + BoomerAMG replaced by MG-CG):
 * returns the iteration count */
int Pressure_solve(Pressure *p)
{
    int it = 0, rc;
    double rr = 0.0;
    turb_ctx *c = lookup(p, K_PRES, NULL, "Pressure_solve");
    if (!c) return -1;
    rc = turb_Pressure_solve(c, &it, &rr);
    note(rc, "Pressure_solve");
    return rc == TURB_OK ? it : -1;
}

/* Pressure_compute_velocity_divergence, Pressure.c:462-586: max |div u| */
double Pressure_compute_velocity_divergence(Pressure *p, Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid,
                                            Parameters *params)
{
    double m = -1.0;
    int rc;
    turb_ctx *c = lookup(p, K_PRES, NULL, "Pressure_compute_velocity_divergence");
    (void)u; (void)v; (void)w; (void)grid; (void)params;
    if (!c) return -1.0;
    rc = turb_Pressure_compute_velocity_divergence(c, &m);
    note(rc, "Pressure_compute_velocity_divergence");
    return rc == TURB_OK ? m : (rc == TURB_ERR_NAN ? m : -1.0);
}

/* ---- Include/ENO.h ------------------------------------------------------- */

/* ENO_compute_convective_terms, ENO.c:103-245: the bound line buffers */
void ENO_compute_convective_terms(ENO_Scheme *ENO, int Nmax_local)
{
    binding *b = find(ENO, K_ENO);
    if (!b) { note(TURB_ERR_ARG, "ENO_compute_convective_terms"); return; }
    note(turb_ENO_compute_convective_terms(b->order, Nmax_local, b->buf[0], b->buf[1], b->buf[2], b->buf[3]),
         "ENO_compute_convective_terms");
}
