/*
 * turbins_dropin.h -- the reference's own hot-path routines, same names and
 * signatures, running on the GPU through libturbgpu.so (libturbdropin.so).
 *
 * A TURBINS host program (its missing main loop) calls Velocity_u_set_RHS,
 * Velocity_solve, Pressure_solve, ... exactly as it calls the reference's
 * Velocity.c / Conc.c / Pressure.c / ENO.c routines.  Linked (or
 * LD_PRELOADed) ahead of those files, this layer takes the calls: each
 * struct pointer the routines receive is a key to the device state it was
 * bound to, and the state's PETSc Vecs are copied between host and device
 * only by turb_dropin_upload / turb_dropin_download.  Between those calls the
 * device copy is the current one (the host Vecs are stale).
 *
 * The struct types are the reference's (Include/DataTypes.h: struct velocity,
 * struct pressure, ...); this layer never looks inside them, so it builds
 * with or without the reference's headers.  With them on the include path
 * (TURB_DROPIN_REFERENCE_HEADERS) the compiler checks every definition here
 * against the reference's own prototype.
 *
 * Errors: the routines the reference declares void record the first
 * non-zero library status, which turb_dropin_status() returns and clears;
 * the int / double routines also return -1 on error.  Like the reference
 * (single-threaded per MPI rank) the layer is not thread-safe.
 */
#ifndef TURBINS_DROPIN_H
#define TURBINS_DROPIN_H

#include "turbins_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct velocity Velocity;           /* Include/DataTypes.h:349 */
typedef struct pressure Pressure;           /* Include/DataTypes.h:174 */
typedef struct concentration Concentration; /* Include/DataTypes.h:101 */
typedef struct parameters Parameters;       /* Include/DataTypes.h:249 */
typedef struct eno_scheme ENO_Scheme;       /* Include/DataTypes.h:369 */
typedef struct mac_grid MAC_grid;           /* Include/DataTypes.h:628 */
typedef struct gvg_bag GVG_bag;             /* Include/DataTypes.h:645 */
typedef struct _p_Vec *Vec;                 /* PETSc vector handle */

/* ---- binding (no reference counterpart) -----------------------------------
 * grid: the MAC_grid whose fields ctx holds (turb_create from its
 * coordinates, statuses and immersed stencils).  Each Velocity (component
 * 'u' / 'v' / 'w'), Concentration (fraction ic) and the Pressure is bound to
 * the grid with the Vecs of its state: Velocity.G_data, Concentration.G_data,
 * Pressure.G_data (phi) and G_dp_dx / G_dp_dy / G_dp_dz.  An ENO_Scheme is
 * bound with its order and line buffers (D0, Position, Velocity, VdQdX).  At
 * most 16 grids, 64 structs. */
int turb_dropin_bind_grid(MAC_grid *grid, turb_ctx *ctx);
int turb_dropin_bind_velocity(Velocity *vel, MAC_grid *grid, char component, Vec data);
int turb_dropin_bind_conc(Concentration *c, MAC_grid *grid, int ic, Vec data);
int turb_dropin_bind_pressure(Pressure *p, MAC_grid *grid, Vec phi, Vec dp_dx, Vec dp_dy, Vec dp_dz);
int turb_dropin_bind_eno(ENO_Scheme *eno, int order, double *D0, double *Position, double *Velocity_,
                         double *VdQdX);
/* copy every bound Vec of grid host -> device / device -> host (DA order) */
int turb_dropin_upload(MAC_grid *grid);
int turb_dropin_download(MAC_grid *grid);
/* first non-zero status recorded since the last call (0: none); clears it */
int turb_dropin_status(void);
/* forget every binding of grid (the context is the caller's) */
int turb_dropin_unbind_grid(MAC_grid *grid);

/* ---- the fused step (no reference routine: the reference ships no time-step
 * driver) -------------------------------------------------------------------
 * bag: the GVG_bag holding the grid's structs, bound to the grid.  One
 * TVD-RK2 step of dt on the bound device state (turb_step: both stages of
 * convection, Helmholtz solves, Poisson solve and projection, then the RK
 * average); *status (if given) receives the library status, which is also
 * returned (0: ok).  The layer never writes the bag: its time and iteration
 * counters stay the host's. */
int turb_dropin_bind_bag(GVG_bag *bag, MAC_grid *grid);
int turb_dropin_step(GVG_bag *bag, double dt, int *status);

/* ---- the reference's routines ---------------------------------------------
 * Include/Velocity.h */
void Velocity_store_old_data(Velocity *vel);
void Velocity_cell_center(Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid, Parameters *params);
void Velocity_u_set_RHS(Velocity *u, Pressure *p, MAC_grid *grid, Parameters *params, double dt);
void Velocity_v_set_RHS(Velocity *v, Pressure *p, Concentration **c, MAC_grid *grid, Parameters *params, double dt);
void Velocity_w_set_RHS(Velocity *w, Pressure *p, MAC_grid *grid, Parameters *params, double dt);
void Velocity_rk_average(Velocity *vel, double old_frac, double new_frac);
void Velocity_modify_diagonal(Velocity *vel, MAC_grid *grid, Parameters *params, double dt, double dt_old);
int Velocity_solve(Velocity *vel);
void Velocity_transpose_velocities(Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid, Parameters *params,
                                   char which_quantity);
/* Include/Conc.h */
void Conc_modify_diagonal(Concentration *c, MAC_grid *grid, double dt, double dt_old);
void Conc_rk_average(Concentration *c, double old_frac, double new_frac);
void Conc_set_particle_v_velocity(Concentration *c, Velocity *v, Parameters *params);
int Conc_solve(Concentration *c);
void Conc_set_RHS(Concentration *c, MAC_grid *grid, Parameters *params, double dt);
void Conc_store_old_data(Concentration *c);
void Conc_compute_total_concentration(Concentration **c, Parameters *params);
/* Include/Pressure.h */
void Pressure_set_RHS(Pressure *p, Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid, Parameters *params,
                      double dt);
void Pressure_project_velocity(Pressure *p, Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid,
                               Parameters *params, double dt);
int Pressure_solve(Pressure *p);
double Pressure_compute_velocity_divergence(Pressure *p, Velocity *u, Velocity *v, Velocity *w, MAC_grid *grid,
                                            Parameters *params);
/* Include/ENO.h */
void ENO_compute_convective_terms(ENO_Scheme *ENO, int Nmax_local);

#ifdef __cplusplus
}
#endif
#endif
