/*
 * dropin_step.c -- a host step written with the reference's own routine
 * names (include/turbins_dropin.h), as the reference's missing main loop
 * would call them, running on the GPU through libturbdropin.so.
 *
 * Built by tests/test_dropin.py into a shared library together with the
 * PETSc stand-in (oracle/shim) that provides the DA vectors.  The struct
 * pointers are the driver's own keys: the layer never looks inside them.
 */
#include <string.h>

#include "petsc.h"
#include "turbins_dropin.h"

static char k_grid, k_params, k_u, k_v, k_w, k_p, k_c[TURB_MAXCONC];

/* fields: u v w phi dp_dx dp_dy dp_dz c_0 .. c_{nconc-1}, DA order, updated
 * in place by one TVD-RK2 step; div_max: the two stages' max |div u|.
 * Returns the layer's status (0: every call succeeded). */
int dropin_step(turb_ctx *ctx, int nx, int ny, int nz, int nconc, double dt, double *const *fields,
                double *div_max, int *iters)
{
    MAC_grid *grid = (MAC_grid *)&k_grid;
    Parameters *params = (Parameters *)&k_params;
    Velocity *u = (Velocity *)&k_u, *v = (Velocity *)&k_v, *w = (Velocity *)&k_w;
    Pressure *p = (Pressure *)&k_p;
    Concentration *c[TURB_MAXCONC];
    DA da;
    Vec vec[7 + TURB_MAXCONC];
    long n = (long)(nx + 1) * (ny + 1) * (nz + 1);
    int f, i, stage, nf = 7 + nconc, rc;

    if (nconc < 1 || nconc > TURB_MAXCONC) return TURB_ERR_ARG;
    DACreate3d(0, DA_NONPERIODIC, DA_STENCIL_STAR, nx + 1, ny + 1, nz + 1, 1, 1, 1, 1, 1, 0, 0, 0, &da);
    for (f = 0; f < nf; f++) {
        double *a;
        DACreateGlobalVector(da, &vec[f]);
        VecGetArray(vec[f], &a);
        memcpy(a, fields[f], (size_t)n * sizeof(double));
        VecRestoreArray(vec[f], &a);
    }
    for (i = 0; i < nconc; i++) c[i] = (Concentration *)&k_c[i];

    rc = turb_dropin_bind_grid(grid, ctx);
    if (!rc) rc = turb_dropin_bind_velocity(u, grid, 'u', vec[0]);
    if (!rc) rc = turb_dropin_bind_velocity(v, grid, 'v', vec[1]);
    if (!rc) rc = turb_dropin_bind_velocity(w, grid, 'w', vec[2]);
    if (!rc) rc = turb_dropin_bind_pressure(p, grid, vec[3], vec[4], vec[5], vec[6]);
    for (i = 0; i < nconc && !rc; i++) rc = turb_dropin_bind_conc(c[i], grid, i, vec[7 + i]);
    if (!rc) rc = turb_dropin_upload(grid);

    if (!rc) {
        Velocity_store_old_data(u);
        Velocity_store_old_data(v);
        Velocity_store_old_data(w);
        for (i = 0; i < nconc; i++) Conc_store_old_data(c[i]);
        for (stage = 0; stage < 2; stage++) {
            Velocity_cell_center(u, v, w, grid, params);
            if (nconc > 1) Conc_compute_total_concentration(c, params);
            /* the convection driver the reference does not ship */
            turb_Velocity_convective_terms(ctx, 'u');
            turb_Velocity_convective_terms(ctx, 'v');
            turb_Velocity_convective_terms(ctx, 'w');
            for (i = 0; i < nconc; i++) turb_Conc_convective_terms(ctx, i);
            Velocity_u_set_RHS(u, p, grid, params, dt);
            Velocity_v_set_RHS(v, p, c, grid, params, dt);
            Velocity_w_set_RHS(w, p, grid, params, dt);
            Velocity_modify_diagonal(u, grid, params, dt, dt);
            Velocity_modify_diagonal(v, grid, params, dt, dt);
            Velocity_modify_diagonal(w, grid, params, dt, dt);
            iters[0] += Velocity_solve(u);
            iters[1] += Velocity_solve(v);
            iters[2] += Velocity_solve(w);
            for (i = 0; i < nconc; i++) {
                Conc_set_RHS(c[i], grid, params, dt);
                Conc_modify_diagonal(c[i], grid, dt, dt);
                iters[3] += Conc_solve(c[i]);
            }
            Pressure_set_RHS(p, u, v, w, grid, params, dt);
            iters[4] += Pressure_solve(p);
            Pressure_project_velocity(p, u, v, w, grid, params, dt);
            div_max[stage] = Pressure_compute_velocity_divergence(p, u, v, w, grid, params);
        }
        Velocity_rk_average(u, 0.5, 0.5);
        Velocity_rk_average(v, 0.5, 0.5);
        Velocity_rk_average(w, 0.5, 0.5);
        for (i = 0; i < nconc; i++) Conc_rk_average(c[i], 0.5, 0.5);
        rc = turb_dropin_status();
        if (!rc) rc = turb_dropin_download(grid);
    }
    for (f = 0; f < nf; f++) {
        double *a;
        VecGetArray(vec[f], &a);
        if (!rc) memcpy(fields[f], a, (size_t)n * sizeof(double));
        VecRestoreArray(vec[f], &a);
        VecDestroy(vec[f]);
    }
    DADestroy(da);
    turb_dropin_unbind_grid(grid);
    return rc;
}
