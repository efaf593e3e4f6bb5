/*
 * turbins_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * TURBINS fractional-step hot path.
 *
 * One context (turb_ctx) is the device-side counterpart of the reference's
 * GVG_bag (Include/DataTypes.h:632-645): the MAC grid (MAC_grid, :573-628),
 * the velocity, pressure and concentration vectors, and one CUDA stream.  All
 * fields stay resident in HBM across calls; host memory is touched only by
 * turb_field_upload / turb_field_download, which take the reference's PETSc DA
 * layout a[(k*NY + j)*NX + i], NX = nx+1, NY = ny+1, NZ = nz+1, FP64.
 *
 * Every entry point returns a turb_status (0 = success).  Entry points named
 * turb_<RefName> replace the reference routine <RefName> with the same
 * argument meaning; the reference's struct arguments (Velocity*, Pressure*,
 * Concentration*, MAC_grid*, Parameters*) are folded into the context.
 * Nothing here allocates host memory that the caller must free, and no call
 * falls back to the CPU: without a usable GB300 every call returns
 * TURB_ERR_CUDA.
 */
#ifndef TURBINS_GB300_H
#define TURBINS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TURB_OK = 0,
    TURB_ERR_ARG = 1,            /* bad argument (size, id, NULL)           */
    TURB_ERR_CUDA = 2,           /* CUDA runtime error / no device          */
    TURB_ERR_NOT_CONVERGED = 3,  /* solver reached max_iter (cf. Solver.c:326-348) */
    TURB_ERR_NAN = 4,            /* non-finite residual                     */
    TURB_ERR_ALLOC = 5,          /* device allocation failed                */
    TURB_ERR_SCRATCH_LIMIT = 6,  /* grid larger than the fixed scratch of turb_velocity_divergence_noalloc */
    TURB_ERR_IO = 7,             /* a restart file could not be opened, written or read in full */
    TURB_ERR_FORMAT = 8          /* a restart file does not hold what the context expects */
} turb_status;

/* node status codes, Include/definitions.h:93-99 */
#define TURB_SOLID 2
#define TURB_FLUID 3
#define TURB_IMMERSED 5
#define TURB_BOUNDARY 7
#define TURB_BUFFER_SOLID 11

#define TURB_SALINITY 1
#define TURB_PARTICLE 2
#define TURB_MAXCONC 4

/* Parameters (Include/DataTypes.h:177-248), after the Input.c:405-509 rules */
typedef struct {
    int nx, ny, nz;              /* physical cells                            */
    int eno_order;               /* 1..3                                       */
    double re;                   /* Reynolds number                            */
    int nconc;                   /* 1..TURB_MAXCONC                             */
    double pe[TURB_MAXCONC];     /* Peclet number                               */
    double vs0[TURB_MAXCONC];    /* settling speed after the sign flip           */
    double alpha[TURB_MAXCONC];  /* buoyancy weights after the rescale           */
    int ctype[TURB_MAXCONC];     /* TURB_SALINITY / TURB_PARTICLE               */
    int sedimentation;           /* Robin top ghost for particle fractions       */
    int wall_noslip[6];          /* velocity walls x-,x+,y-,y+,z-,z+: 1 no-slip */
    int buoyancy;                /* subtract c at v nodes                        */
    double vel_rtol;             /* Helmholtz relative residual (resmax)        */
    int vel_maxit;
    double p_rtol;               /* Poisson relative residual                    */
    int p_maxit;
} turb_params;

/* Ghost-cell immersed-boundary stencils of one quantity (ImmersedNode,
 * Include/DataTypes.h:520-546), linear DA indices. */
typedef struct {
    int n;
    const int32_t *im;           /* [n]   immersed node                         */
    const int32_t *nf;           /* [n]   1 or 8 fluid nodes                    */
    const int32_t *fidx;         /* [n*8] fluid nodes                           */
    const double *fcoef;         /* [n*8] fluid_coef                            */
    const double *bcoef;         /* [n]   boundary_coef                         */
} turb_ib_desc;

typedef struct {
    int nx, ny, nz;
    const double *xc, *yc, *zc;  /* cell centres, nx+1 / ny+1 / nz+1 entries   */
    const double *xu, *yv, *zw;  /* faces, nx+1 / ny+1 / nz+1 entries           */
    const uint8_t *status[4];    /* u, v, w, c node status, DA layout           */
    turb_ib_desc ib[4];          /* u, v, w, c                                  */
} turb_grid_desc;

typedef struct turb_ctx turb_ctx;

/* Field identifiers for upload/download (the reference Vec each mirrors). */
enum {
    TURB_F_U = 0, TURB_F_V, TURB_F_W,               /* Velocity.G_data          */
    TURB_F_PHI, TURB_F_DPX, TURB_F_DPY, TURB_F_DPZ, /* Pressure.G_data, G_dp_d* */
    TURB_F_PB, TURB_F_DIV,                          /* Pressure.G_b, G_divergence */
    TURB_F_UBC, TURB_F_VBC, TURB_F_WBC,             /* Velocity.G_data_bc       */
    TURB_F_CONV_U, TURB_F_CONV_V, TURB_F_CONV_W,    /* Velocity.G_conv          */
    TURB_F_B_U, TURB_F_B_V, TURB_F_B_W,             /* Velocity.G_b             */
    TURB_F_CTOT,                                    /* Concentration.G_c_total  */
    TURB_F_SCRATCH0, TURB_F_SCRATCH1,               /* MAC_grid.G_dummy1/2      */
    TURB_F_C0 = 32,                                 /* + ic: Concentration.G_data */
    TURB_F_CCONV0 = 40,                             /* + ic: Concentration.G_conv */
    TURB_F_CB0 = 48,                                /* + ic: Concentration.G_b   */
    TURB_F_VP0 = 56                                 /* + ic: G_v_particle        */
};

typedef struct {
    int vel_iters[3][2];
    int conc_iters[TURB_MAXCONC][2];
    int p_iters[2];
    double p_relres[2];
    double div_max[2];
    int kernel_launches;         /* launches of this library's kernels         */
} turb_step_stats;

/* Pressure solver modes for turb_set_pressure_mode */
#define TURB_PMODE_FP64 0        /* plain FP64 MG-preconditioned CG             */
#define TURB_PMODE_MIXED 1       /* FP32 V-cycles inside FP64 flexible CG       */

/* Helmholtz (implicit viscous / diffusive) solver modes */
#define TURB_HMODE_FP64 0        /* FP64 point-Jacobi iteration                 */
#define TURB_HMODE_MIXED 1       /* FP64 defect correction, FP32 inner sweeps   */

/* ---- context -------------------------------------------------------------
 * Replaces Grid_create + Velocity_create + Pressure_create + Conc_create +
 * *_setup_lsys_accounting_geometry (Grid.c:21, Velocity.c:19, Pressure.c:15,
 * Conc.c:22, Velocity.c:329, Pressure.c:129, Conc.c:358): allocates every
 * field (zeroed) and the solver hierarchies on the current CUDA device. */
int turb_create(const turb_grid_desc *grid, const turb_params *params, turb_ctx **out);
int turb_destroy(turb_ctx *ctx);
int turb_field_upload(turb_ctx *ctx, int field, const double *host_da);
int turb_field_download(turb_ctx *ctx, int field, double *host_da);
/* n fields in one call (host[t] <-> fields[t]); the call returns when every
 * copy has completed.  A field moves either as one contiguous copy through a
 * device staging buffer, the copy of one field overlapping the layout
 * conversion of the one before (from page-locked arrays -- turb_host_alloc
 * or turb_host_register, whole array -- on the copy engines), or, for a
 * page-locked array, by the layout kernel reading / writing it in place
 * across the host link.  TURB_HOST_COPY_KERNEL (default): page-locked
 * arrays by the kernel; TURB_HOST_COPY_DMA: through staging on the copy
 * engines.  Pageable arrays always go through staging. */
int turb_fields_upload(turb_ctx *ctx, int n, const int *fields, const double *const *host_da);
int turb_fields_download(turb_ctx *ctx, int n, const int *fields, double *const *host_da);
#define TURB_HOST_COPY_DMA 1
#define TURB_HOST_COPY_KERNEL 2
int turb_set_host_copy(turb_ctx *ctx, int mode);
int turb_set_pressure_mode(turb_ctx *ctx, int mode);
/* Initial guess of the Poisson solve.  PREVIOUS: the last solution (the
 * reference's nonzero initial guess, Solver.c:84).  EXTRAPOLATE: 2 p1 - p2 from
 * the last two solutions of the same RK stage.  LEARNED: p1 + net(b, p1, p2)
 * from the warm-start network (turb_net_*).  A candidate is used only if its
 * initial residual is below the PREVIOUS guess's; the solve always iterates
 * to the same FP64 tolerance. */
#define TURB_GUESS_PREVIOUS 0
#define TURB_GUESS_EXTRAPOLATE 1
#define TURB_GUESS_LEARNED 2
/* no reference counterpart: the energy-norm best guess in the span of the
 * previous guess and this RK stage's last two solutions (a Galerkin fit over
 * earlier solutions, after Fischer's projection method for successive
 * right-hand sides) */
#define TURB_GUESS_PROJECT 3
int turb_set_pressure_guess(turb_ctx *ctx, int mode);
/* forget the earlier solutions the extrapolated, projected and learned
 * guesses start from (after fields were replaced from elsewhere, e.g. a
 * state loaded again); the next solves of each stage rebuild it */
int turb_reset_pressure_history(turb_ctx *ctx);
/* RK stages whose pressure solve tries the extrapolated / learned candidate:
 * bit 0 the first stage, bit 1 the second (default 3, both).  With the
 * Galerkin fit on (turb_set_guess_galerkin), the learned mode's other stages
 * take the fit over their earlier solutions alone (no network). */
/* kernel variants, all giving the same bits: TURB_KV_MARCHING, the FP32
 * Helmholtz Jacobi sweeps and FP32 red-black half sweeps march along k
 * through shared-memory plane tiles (else one point, four cells, per thread);
 * TURB_KV_ENO_SEGMENTS, every y / z ENO line is walked in segments of about
 * 64 nodes by separate threads (else one thread per line); TURB_KV_PDL,
 * the V-cycle's kernels are launched with programmatic dependent launch, so
 * that each may be scheduled while the one before it drains (else plain
 * stream order); TURB_KV_CLUSTER_VCYCLE, the V-cycle from the first level
 * of at most turb_set_mg_cluster cells down runs as one launch of one
 * thread-block cluster (16 blocks of 1024 threads, or 8 where 16 do not fit),
 * its phases separated by the hardware cluster barrier; TURB_KV_SWEEP_PAIRS,
 * the finest FP32 level (colour-split, nx a multiple of 64, ny of 32)
 * applies its red-black sweeps two at a time in one pass over memory: z
 * planes staged in shared memory by TMA, a wavefront of four half sweeps
 * along z over overlapped 64 x 32 tiles, the result in a second x array.
 * Default:
 * TURB_KV_ENO_SEGMENTS | TURB_KV_PDL (measured fastest on GB300 at
 * 512x256x256). */
#define TURB_KV_MARCHING 1
#define TURB_KV_ENO_SEGMENTS 2
#define TURB_KV_PDL 4   /* V-cycle kernels with programmatic dependent launch */
#define TURB_KV_CLUSTER_VCYCLE 8   /* coarse V-cycle levels in one thread-block cluster */
#define TURB_KV_SWEEP_PAIRS 16    /* finest FP32 level: two sweeps per pass */
int turb_set_sweep_kernels(turb_ctx *ctx, int variants);
/* max_div > 0: every Poisson solve, after reaching its relative residual,
 * also iterates until dt * max|b - A phi| (the largest divergence the
 * projection with phi leaves, dt of the last turb_Pressure_set_RHS) is at
 * most max_div, or until the residual's 2-norm is at its round-off floor
 * (64 DBL_EPSILON |b|: there the estimate sees the rounding of b - A phi
 * divided by the smallest cell volumes, which no iteration removes); 0
 * (default) turns the gate off.  The counts are how often a solve had to go
 * on, and how often the gate let a solve go at the floor. */
int turb_set_divergence_gate(turb_ctx *ctx, double max_div);
int turb_divergence_gate_count(turb_ctx *ctx, long long *tightened);
int turb_divergence_gate_floor_count(turb_ctx *ctx, long long *at_floor);
/* 1: the learned candidate also goes through the Galerkin fit with this
 * stage's last two solutions (TURB_GUESS_PROJECT's span plus the network's
 * direction).  A fit is kept when it lowers the residual in the S^-1 norm
 * (equivalently the S-norm of the error, the norm CG minimises); a network
 * candidate alone when it lowers the residual's 2-norm. */
int turb_set_guess_galerkin(turb_ctx *ctx, int on);
int turb_set_guess_stages(turb_ctx *ctx, int mask);
int turb_pressure_guess_stats(turb_ctx *ctx, int *tried, int *taken);
/* geometric mean over the tried candidates of |r(candidate)| / |r(previous)|
 * (initial residuals; 1 when nothing was tried) */
int turb_pressure_guess_ratio(turb_ctx *ctx, double *geo_mean);
/* red-black Gauss-Seidel sweeps of the pressure V-cycle before / after the
 * coarse-grid correction on every level, for the current pressure mode
 * (1..16; defaults: 4 / 4 with FP64 V-cycles; with FP32 V-cycles 4 / 4 on the
 * finest level, 5 / 5 on the next and 12 / 12 on the coarser ones) */
int turb_set_mg_sweeps(turb_ctx *ctx, int npre, int npost);
/* levels from_level and coarser (0 = the finest, >= 1) of the current
 * pressure mode's V-cycle smooth with npre / npost sweeps (1..16) instead */
int turb_set_mg_coarse_sweeps(turb_ctx *ctx, int from_level, int npre, int npost);
/* the V-cycle from the first level of at most max_cells cells (default
 * 4096; 0: never) down to the coarsest and back runs as one single-block
 * kernel instead of a launch per half sweep; results are bit-identical */
int turb_set_mg_tail(turb_ctx *ctx, long long max_cells);
/* with TURB_KV_CLUSTER_VCYCLE, the V-cycle from the first level of at most
 * max_cells cells (default 131072; 0: never) runs as one thread-block
 * cluster launch, the levels from the single-block tail's on in block 0 of
 * it; results are bit-identical */
int turb_set_mg_cluster(turb_ctx *ctx, long long max_cells);
/* storage order of the FP32 multigrid levels: 1 (default) colour-split (red
 * and black cells in separate halves, dense half sweeps), 0 natural.  The
 * arithmetic is the same, so results are bit-identical either way. */
int turb_set_mg_split(turb_ctx *ctx, int on);
/* both modes stop on the FP64 residual ||b - A x|| <= vel_rtol ||b||;
 * inner_sweeps: FP32 Jacobi sweeps per defect-correction step of the mixed
 * mode (1..64, default 5) */
int turb_set_helmholtz_mode(turb_ctx *ctx, int mode, int inner_sweeps);
/* ENO divided differences: 1 (default) divides by a grid spacing through its
 * precomputed two-term reciprocal and one correction step (FP64: 1 multiply +
 * 3 FMA, range tests on the integer pipe), without the correction (1
 * multiply + 1 FMA) for the spacings the set-up proves it unneeded for
 * (turb_division_two_term_exact), and by one exact multiply for
 * power-of-two spacings; 0 uses IEEE division; all round to nearest, so the
 * results are the same bits */
int turb_set_eno_division(turb_ctx *ctx, int fast);
int turb_synchronize(turb_ctx *ctx);
const char *turb_status_string(int status);

/* ---- hot-path routines (same-named reference routine in the comment) ----- */
/* ENO_compute_convective_terms, ENO.c:103-245: one host line, run on the GPU */
int turb_ENO_compute_convective_terms(int order, int n, const double *D0,
                                      const double *position,
                                      const double *velocity, double *VdQdX);
/* Velocity_cell_center, Velocity.c:1476-1602 */
int turb_Velocity_cell_center(turb_ctx *ctx);
/* Velocity_transpose_velocities, Velocity.c:3341-3663; results in SCRATCH0/1 */
int turb_Velocity_transpose_velocities(turb_ctx *ctx, char which);
/* Conc_compute_total_concentration, Conc.c:1291-1314 */
int turb_Conc_compute_total_concentration(turb_ctx *ctx);
/* Conc_set_particle_v_velocity, Conc.c:734-761 */
int turb_Conc_set_particle_v_velocity(turb_ctx *ctx, int ic);
/* the convection driver (absent from the reference) around
 * ENO_compute_convective_terms and Velocity_{u,v,w}_ENO_ghost_cells
 * (Velocity.c:2124-2801): fills TURB_F_CONV_{U,V,W} */
int turb_Velocity_convective_terms(turb_ctx *ctx, char which);
/* the same around Conc_ENO_ghost_cells (Conc.c:1021-1220): TURB_F_CCONV0+ic */
int turb_Conc_convective_terms(turb_ctx *ctx, int ic);
/* Velocity_{u,v,w}_set_RHS, Velocity.c:1607-2043 (with buoyancy on v) */
int turb_Velocity_set_RHS(turb_ctx *ctx, char which, double dt);
/* Conc_set_RHS, Conc.c:864-992 */
int turb_Conc_set_RHS(turb_ctx *ctx, int ic, double dt);
/* Velocity_modify_diagonal + Velocity_solve, Velocity.c:374-443, 306-324 */
int turb_Velocity_solve(turb_ctx *ctx, char which, double dt, int *iters);
/* Conc_modify_diagonal + Conc_solve, Conc.c:293-354, 840-859 */
int turb_Conc_solve(turb_ctx *ctx, int ic, double dt, int *iters);
/* Pressure_set_RHS, Pressure.c:171-276 */
int turb_Pressure_set_RHS(turb_ctx *ctx, double dt);
/* Pressure_solve, Pressure.c:443-458 (GMRES+BoomerAMG replaced by MG-CG) */
int turb_Pressure_solve(turb_ctx *ctx, int *iters, double *relres);
/* Pressure_project_velocity, Pressure.c:280-439 */
int turb_Pressure_project_velocity(turb_ctx *ctx, double dt);
/* Pressure_compute_velocity_divergence, Pressure.c:462-586 */
int turb_Pressure_compute_velocity_divergence(turb_ctx *ctx, double *div_max);
/* Velocity_store_old_data / Conc_store_old_data, Velocity.c:297, Conc.c:997 */
int turb_store_old_data(turb_ctx *ctx);
/* Velocity_rk_average / Conc_rk_average, Velocity.c:2047, Conc.c:1007 */
int turb_rk_average(turb_ctx *ctx, double old_frac, double new_frac);
/* the same for one state field (TURB_F_U..TURB_F_W or TURB_F_C0 + ic):
 * Velocity_store_old_data / Conc_store_old_data and Velocity_rk_average /
 * Conc_rk_average of a single Velocity or Concentration */
int turb_store_old_field(turb_ctx *ctx, int field);
int turb_rk_average_field(turb_ctx *ctx, int field, double old_frac, double new_frac);
/* No reference counterpart: the divergence check of
 * Pressure_compute_velocity_divergence on a closed box (no inflow / outflow
 * faces) for callers that cannot allocate GPU memory (a host under a fixed
 * device memory budget, a plugin that only receives device buffers from its
 * host application).  Every argument is caller-owned: u, v, w (FP64, DA order
 * with rows of `pitch` doubles, pitch >= nx+1), c_status (uint8, same pitch),
 * the metrics mxc/myc/mzc (nx+1/ny+1/nz+1 doubles) and the output div on the
 * device, div_max on the host.  c_status must mark the last layers i = nx,
 * j = ny and k = nz BOUNDARY (7), as the reference's DA does; those
 * layers are never evaluated, so no read leaves the buffers whatever the
 * status holds.  A NaN in the fields gives a NaN div_max and TURB_ERR_NAN.
 * The only scratch is a file-scope __device__ array of
 * TURB_NOALLOC_MAX_BLOCKS doubles (512 KB) that every GPU loading this
 * library holds until exit; grids needing more than TURB_NOALLOC_MAX_BLOCKS
 * blocks of 32 x 8 x 8 points return TURB_ERR_SCRATCH_LIMIT.  Nothing is
 * allocated: the first call on a device resolves the array's device address
 * (cudaGetSymbolAddress); cudaDeviceReset after it is not supported.  All
 * calls share the array, so calls that overlap on the GPU (different
 * streams, no ordering) race.  The call copies div_max to the host and
 * synchronizes `stream` (a cudaStream_t, 0 = legacy default stream), so it
 * is made outside any stream capture. */
#define TURB_NOALLOC_MAX_BLOCKS 65536
int turb_velocity_divergence_noalloc(int nx, int ny, int nz, long long pitch, const double *u,
                                     const double *v, const double *w, const uint8_t *c_status,
                                     const double *mxc, const double *myc, const double *mzc,
                                     double *div, double *div_max, void *stream);

/* one TVD-RK2 step of the restated driver (the absent main loop) */
int turb_step(turb_ctx *ctx, double dt, turb_step_stats *stats);
/* turb_fields_upload, turb_step, turb_fields_download of the same n fields
 * and host arrays in one call, for a driver that moves the state every step:
 * the same results, with the copies of the fields the step reads late
 * (the concentrations after the velocity convective terms when no open face
 * sets them, dpx, dpy, dpz at the velocity RHS, phi at the Poisson solve)
 * overlapping the step's first kernels, and the downloads of the
 * concentrations (final after the second stage's concentration solve) and
 * of dpx, dpy, dpz, phi its last ones (page-locked arrays with
 * TURB_HOST_COPY_KERNEL; otherwise the three calls in turn).
 * Returns when every copy has landed. */
int turb_step_host(turb_ctx *ctx, double dt, int n, const int *fields, double *const *host_da,
                   turb_step_stats *stats);

/* ---- measurement ---------------------------------------------------------
 * CUDA-event timing per kernel group on the context stream (enable resets the
 * accumulators; read synchronizes and returns ms and launches per group). */
#define TURB_PROF_ENO_X 0      /* x-direction ENO passes                        */
#define TURB_PROF_ENO_YZ 1     /* y/z-direction ENO passes                      */
#define TURB_PROF_JACOBI 2     /* Helmholtz FP64 sweeps / FP64 residuals        */
#define TURB_PROF_MG 3         /* multigrid V-cycles (all levels)               */
#define TURB_PROF_PCG 4        /* FP64 CG vector kernels and reductions         */
#define TURB_PROF_INNER32 5    /* FP32 inner sweeps of the Helmholtz correction */
#define TURB_PROF_NET 6        /* warm-start network: inputs, forward, guard     */
#define TURB_PROF_NGROUPS 7
int turb_profile_enable(turb_ctx *ctx, int on);
int turb_profile_read(turb_ctx *ctx, double *ms, long long *launches);
/* algorithmic bytes of the timed launches per group since profiling was
 * enabled (each array a kernel reads or writes counted once per launch;
 * TURB_PROF_NGROUPS values, 0 for the network) */
int turb_profile_bytes(turb_ctx *ctx, double *bytes);
/* events 0..7 on the context stream; elapsed waits for event b */
int turb_event_record(turb_ctx *ctx, int slot);
int turb_event_elapsed(turb_ctx *ctx, int a, int b, double *ms);
/* number of this library's kernel launches issued by ctx so far */
int turb_kernel_launches(turb_ctx *ctx, long long *n);
/* page-lock caller memory for the host-buffer transfers */
int turb_host_register(void *ptr, size_t bytes);
int turb_host_unregister(void *ptr);
/* page-locked host memory from the driver: transfers from and to it keep
 * the host link's full rate however fragmented the process's own heap is
 * (memory registered after the fact may sit on small pages) */
int turb_host_alloc(size_t bytes, void **ptr);
int turb_host_free(void *ptr);

/* FP64 FMA instructions per second of the current GPU (thread-level;
 * FLOP/s = 2x), measured with CUDA events on a DFMA-only kernel over every SM;
 * the denominator of the FP64-pipe fractions */
int turb_measure_fp64_rate(double *dfma_per_s);
/* self-test: the ENO kernels' division by a grid spacing (two-term
 * reciprocal, one Markstein correction) against IEEE division on nsamples
 * operand pairs;
 * returns the number of bitwise mismatches (and one offending (a, h)) */
int turb_selftest_division(long long nsamples, unsigned long long seed,
                           unsigned long long *mismatches, double *example);
/* 1 when the two-term quotient RN(a y + RN(a yl)) (y = RN(1/h), yl its
 * correction) rounds as a/h for every numerator a, so the ENO kernels divide
 * by h with one multiply and one fused multiply-add; decided at set-up by
 * trying the form on the few numerators whose quotient lies within its error
 * of a midpoint between doubles.  Host only, needs no GPU. */
int turb_division_two_term_exact(double h);
/* self-test: for n caller-chosen pairs, the kernels' two-term quotient of
 * a[t] / h[t] and the IEEE quotient, computed on the GPU */
int turb_selftest_division_pairs(long long n, const double *a, const double *h,
                                 double *q_two_term, double *q_ieee);

/* ---- learned initial guess of the pressure solve ---------------------------
 * No reference counterpart: the reference starts each Poisson solve from the
 * previous pressure (Solver.c:84).  A 4-level 3-D U-Net (channels
 * 16-32-64-128, 3x3x3 kernels, BF16 weights and activations, FP32
 * accumulation on the tcgen05 tensor cores) on the nx x ny x nz physical
 * cells (each a multiple of 8, at least 16) maps three channels -- the
 * residual r1 = b - A p1 of the previous pressure p1, the last increment
 * p1 - p2 of the same RK stage and b, each scaled by its rms (s for r1) --
 * to a correction delta = s diag(A)^-1 out; the candidate p1 + delta is
 * guarded like every other guess.  Parameters are FP32 masters (Adam); the
 * convolutions use BF16 copies.  train = 1 allocates the backward buffers. */
typedef struct turb_net turb_net;
typedef struct turb_snaps turb_snaps;
int turb_net_create(int nx, int ny, int nz, int train, turb_net **out);
int turb_net_destroy(turb_net *net);
long long turb_net_num_params(const turb_net *net);
int turb_net_init_params(turb_net *net, unsigned long long seed);
int turb_net_set_params(turb_net *net, const float *host, long long count);
int turb_net_get_params(turb_net *net, float *host, long long count);
/* gradients of the last turb_net_backward (train nets) */
int turb_net_get_grads(turb_net *net, float *host, long long count);
/* forward activations of the last forward (0..17: x0 a0 p0 a1 p1 a2 p2 a3 b3
 * c2 s2 b2 c1 s1 b1 c0 s0 b0), raw BF16 bits, channel-blocked layout; b0
 * exists on train nets only */
int turb_net_get_activation(turb_net *net, int which, uint16_t *host, long long count);
/* in3: 3 x ncell FP32 device array (channel-major, cells x fastest);
 * out: ncell FP32 device array; stream NULL = default stream */
int turb_net_forward(turb_net *net, const float *in3, float *out, void *stream);
/* gradients for d loss / d out = gout (ncell FP32 device) of the last forward */
int turb_net_backward(turb_net *net, const float *gout, void *stream);
int turb_net_adam(turb_net *net, float lr, void *stream);
/* snapshot store: per pressure solve the network inputs (3 channels, in3
 * layout) and the target channel out* = (p - p_previous) diag(A) / s of the
 * converged pressure p; a solve that does not converge leaves no snapshot */
int turb_snaps_create(int nx, int ny, int nz, int capacity, turb_snaps **out);
int turb_snaps_destroy(turb_snaps *snaps);
int turb_snaps_count(const turb_snaps *snaps);
int turb_snaps_data(turb_snaps *snaps, int index, const float **dev_ptr);
/* record one snapshot at every pressure solve that has a two-deep history of
 * its RK stage (NULL stops recording) */
int turb_set_snapshot_store(turb_ctx *ctx, turb_snaps *snaps);
/* use net for TURB_GUESS_LEARNED (grid of net = physical cells of ctx) */
int turb_set_learned_net(turb_ctx *ctx, turb_net *net);
/* training loss = w_residual L_R + w_energy L_E with ctx's pressure operator A:
 * L_R = |r1 - A delta|^2 / |r1|^2 (the squared relative initial residual of
 * the candidate, what the guard compares) and L_E = e^T A e / e0^T A e0 with
 * e = dp* - delta, e0 = dp* (the A-norm error left, relative to the previous
 * pressure's; dp* = the converged increment of that solve, recorded with the
 * snapshot).  Default (1, 0). */
int turb_net_set_loss(turb_net *net, double w_residual, double w_energy);
/* steps of Adam on randomly drawn snapshots; mean training loss */
int turb_net_train(turb_net *net, turb_ctx *ctx, turb_snaps *snaps, int steps, float lr,
                   unsigned long long seed, double *mean_loss);
/* forward only: mean L_R and L_E over snapshots first .. first+count-1 */
int turb_net_eval(turb_net *net, turb_ctx *ctx, turb_snaps *snaps, int first, int count,
                  double *mean_residual, double *mean_energy);
/* self-test of the tcgen05 operand descriptors: one 128 x 64 x 32 BF16 MMA
 * from K-major (mn_major = 0) or MN-major (1) shared-memory layouts; swap = 1
 * exchanges the LBO and SBO fields.  mn_major = 2: K-major 128-byte-swizzle
 * operands (K = 64), A starting `swap` (0..7) rows into its tile (the
 * swizzle follows absolute addresses: no descriptor base offset).  mn_major < 2, swap = 2 issues no MMA so that the
 * kernel's bounded completion wait runs out (>= 1000000 reported, the
 * context stays usable).  Returns the number of wrong results. */
int turb_selftest_umma(int mn_major, int swap, unsigned long long *mismatches);
/* one convolution of the network's kernels on caller device buffers
 * (channel-blocked BF16 [C/8][Z][Y][X][8]; W FP32 [27][cout][cin]):
 * dgrad_mode 0: out (cout ch) = relu?(conv(in) + bias); 1: out (cin ch) =
 * data gradient of in (cout ch).  wgrad: dw (FP32 [27][cout][cin]) = weight
 * gradient of dy (cout ch) against x (cin ch). */
int turb_conv3_test(int X, int Y, int Z, int cin, int cout, const void *in, const float *W,
                    const float *bias, int relu, int dgrad_mode, void *out, void *stream);
int turb_conv3_wgrad_test(int X, int Y, int Z, int cin, int cout, const void *x, const void *dy,
                          float *dw, void *stream);

/* ---- flow diagnostics of the current state --------------------------------
 * Replaces the reference's output-time reductions (Output_flow_properties,
 * Output.c:2062-2215): Extract_total_kinetic_energy (Extract.c:803-882),
 * Extract_kinetic_potential_conversion_rate (Extract.c:727-801),
 * Extract_viscous_dissipation_rate (Extract.c:453-725),
 * Conc_compute_total_suspended_mass (Conc.c:1471-1522),
 * Conc_compute_potential_energies (Conc.c:1934-2055),
 * Conc_compute_ave_height_x (Conc.c:1524-1608), Conc_find_front_location
 * (Conc.c:1610-1672), Conc_compute_sedimentation_rate and
 * Conc_bottom_sed_rate (Conc.c:2098-2230).  Refreshes the cell-centre
 * velocities (and the total concentration) first, as the reference's output
 * path does.  ave_height: host array of nconc x (nx+1) spanwise-averaged
 * heights, or NULL; sed_bottom: host array of nconc x (nz+1) x (nx+1) bed
 * sedimentation rates, or NULL.  The passive potential energy uses the
 * context's deposited heights (turb_deposit_*). */
typedef struct {
    double kinetic_energy;                    /* W_kinetic_energy                       */
    double conversion_rate;                   /* -int v c_total dV                      */
    double suspended_mass[TURB_MAXCONC];      /* W_total_susp_mass                      */
    double potential_energy[TURB_MAXCONC];    /* W_Ep                                   */
    double stokes_dissipation[TURB_MAXCONC];  /* W_Stokes_dissipation_rate              */
    double conversion_rate_c[TURB_MAXCONC];   /* W_kinetic_potential_conversion_rate    */
    double front_location;                    /* -1 when no crossing                    */
    double viscous_dissipation;               /* W_dissipation_rate                     */
    double ep_passive[TURB_MAXCONC];          /* W_Ep_passive (deposited sediment)      */
    double ep_passive_rate[TURB_MAXCONC];     /* W_Ep_passive_rate                      */
    double ep_rate[TURB_MAXCONC];             /* W_Ep_rate                              */
    double sed_rate[TURB_MAXCONC];            /* W_sed_rate                             */
} turb_diag;
int turb_diagnostics(turb_ctx *ctx, double front_limit, turb_diag *out, double *ave_height, double *sed_bottom);

/* ---- deposited sediment ---------------------------------------------------
 * turb_bed_index: Grid_set_interface_y_index (Grid.c:1972-2012) copied out,
 * iy[k*(nx+1) + i] = first IMMERSED c node of the column, 0 over a FLUID
 * bottom, -1 none.  turb_deposit_integrate: Conc_integrate_deposited_height
 * (Conc.c:1675-1749) of every fraction with weight_factor = alpha_i, from the
 * current concentrations and those saved by turb_store_old_data.
 * turb_deposit_enable(1) runs it at the end of every turb_step.
 * turb_deposit_get / _set: the heights, nconc x (nz+1) x (nx+1) doubles
 * (G_deposit_height of each fraction; restart state). */
int turb_bed_index(turb_ctx *ctx, int32_t *iy);
int turb_deposit_integrate(turb_ctx *ctx, double dt);
int turb_deposit_enable(turb_ctx *ctx, int on);
int turb_deposit_get(turb_ctx *ctx, double *host);
int turb_deposit_set(turb_ctx *ctx, const double *host);

/* ---- immersed-boundary geometry ------------------------------------------
 * turb_geometry: the set-up of a bottom surface on the device, replacing
 * Surface_create + Surface_initialize + Surface_find_exact_sdf +
 * Surface_find_q_sdf (Surface.c:16-336) and Grid_identify_geometry
 * (Grid.c:1825-1870, with the BUFFER_SOLID pass of SOLVE_INSIDE_SOLID).
 * ipos: interface heights [nz+1][nx+1] (MAC_grid.interface_position).  The
 * cell-centre guess yc - ipos is reinitialised to a signed distance by the
 * Godunov level-set iteration of Levelset.c:85-578 (up to 503 steps, stop at
 * an L2 change below 1e-5), copied to the last planes, interpolated to the
 * u/v/w nodes and tagged.  Outputs, host, DA layout [nz+1][ny+1][nx+1], each
 * array or pointer may be null: sdf c, u, v, w (doubles); status u, v, w, c
 * (TURB_* codes); iterations = Godunov steps taken.  The context's own
 * statuses and stencils are left as they are. */
int turb_geometry(turb_ctx *ctx, const double *ipos, double *const *sdf, uint8_t *const *status, int *iterations);

/* The ghost-cell stencils that the last turb_geometry built from its statuses
 * and sdf, quantity q = 0..3 (u, v, w, c), as Immersed_setup_q_immersed_nodes
 * (Immersed.c:546-616) builds them: IMMERSED nodes in DA order, normal from
 * the sdf gradient, control point on the surface, image point twice as far
 * into the fluid, the 8-node box around it (or the nearest fluid node), and
 * Dirichlet (u, v, w) / Neumann (c) coefficients.  *n = node count; each
 * array may be null, else holds n (im, nf, bcoef), 8n (fidx, fcoef) or 12n
 * (pts: normal, control point, image point, node point) entries; im / fidx
 * are DA linear indices (the turb_ib_desc layout). */
int turb_geometry_stencils(turb_ctx *ctx, int q, int *n, int32_t *im, int32_t *nf, int32_t *fidx, double *fcoef,
                           double *bcoef, double *pts);

/* ---- open boundaries -------------------------------------------------------
 * params->inflow / outflow of the reference: an inflow face at x = xmin and a
 * convective outflow face at x = xmax.  turb_set_open_boundaries turns them
 * on (U: convective velocity params->U; transient_inflow, time_c: the
 * 1 - exp(-(t + 0.01)/time_c) ramp of Inflow.c) and makes every routine of
 * the step take the faces into account: cell centres (Velocity.c:1544-1558),
 * transposes (Velocity.c:3491-3605), RHS of u, v, w, c (Velocity.c:1691-1721,
 * 1885-1896, 2011-2022; Conc.c:938-962), Helmholtz rows (Velocity.c:989,
 * 1336; Conc.c:583-606), ENO ghosts of x lines (Velocity.c:2194-2235,
 * 2442-2449, 2669-2676; Conc.c:1099-1124), pressure RHS and divergence
 * (Pressure.c:242-248, 541-547), viscous dissipation (Extract.c:582-639).
 * Planes are [nz+1][ny+1] doubles (j fastest): which 0 = inflow (u: q 0; c:
 * q 3, ic), 1 = outflow, 2 = outflow_old (q 0..2 = u, v, w, 3 = c_ic).
 * The routines replace Inflow_u_velocity_profile / Inflow_conc_profile
 * (Inflow.c:13-260), Outflow_{vel,conc}_impose_convective_boundary with the
 * mass correction of u (Outflow.c:30-303), *_store_old_outflow /
 * *_rk_average_outflow (Velocity.c:2059-2118, Conc.c:1224-1290) and
 * Outflow_*_copy_data_into_{last_plane,2D_array} (Outflow.c:306-503).
 * turb_set_influx sets u's W_influx that the mass correction uses (normally
 * left by turb_Inflow_u_velocity_profile). */
int turb_set_open_boundaries(turb_ctx *ctx, int inflow, int outflow, double U, int transient_inflow,
                             double time_c);
int turb_open_plane_get(turb_ctx *ctx, int which, int q, int ic, double *host);
int turb_open_plane_set(turb_ctx *ctx, int which, int q, int ic, const double *host);
int turb_Inflow_u_velocity_profile(turb_ctx *ctx, double time, double *influx);
int turb_Inflow_conc_profile(turb_ctx *ctx, int ic, double time);
int turb_set_influx(turb_ctx *ctx, double influx);
/* simulated time (GVG_bag.time): advanced by dt in every turb_step; the
 * inflow ramp is evaluated at the step's starting time.  With open faces a
 * step first sets the inflow planes (u, then each c) and stores the outflow
 * planes, imposes the convective outflow (with u's mass correction) at the
 * start of each RK stage, and RK-averages the outflow planes at the end. */
int turb_set_time(turb_ctx *ctx, double time);
int turb_get_time(turb_ctx *ctx, double *time);
int turb_Outflow_vel_impose_convective_boundary(turb_ctx *ctx, char which, double dt);
int turb_Outflow_conc_impose_convective_boundary(turb_ctx *ctx, int ic, double dt);
int turb_Outflow_impose_convective_boundary(turb_ctx *ctx, double dt);
int turb_store_old_outflow(turb_ctx *ctx);
int turb_rk_average_outflow(turb_ctx *ctx, double old_frac, double new_frac);
int turb_Outflow_copy_data_into_last_plane(turb_ctx *ctx, char which, int ic, int should_set);
int turb_Outflow_copy_data_into_2D_array(turb_ctx *ctx, char which, int ic);

/* ---- checkpoint / resume ---------------------------------------------------
 * The reference's restart set (Resume_set_data, Resume.c:208-244) in its
 * formats, written to / read from directory dir:
 *   Resume_u.bin, Resume_v.bin, Resume_w.bin, Resume_dpdx.bin, Resume_dpdy.bin,
 *   Resume_dpdz.bin, [Resume_gridc.bin], Resume_conc<i>.bin: PETSc binary
 *   vectors (VecView / VecLoadIntoVector: int32 {1211214, N}, N doubles, all
 *   big-endian) in the DA order [k][j][i];
 *   Resume_primary.dat: Resume_write_primary_data's text (time, dt, dt_old,
 *   iteration, output_iter);
 * and, with flags:
 *   TURB_RESUME_GRID: Resume_gridc.bin, the c node status as FP64 codes (on
 *     read it must equal the context's geometry, else TURB_ERR_FORMAT);
 *   TURB_RESUME_DEPOSIT: Resume_deposit_height<i>.bin per particle fraction,
 *     Resume_write_2D_data's raw [NZ][NX] doubles (the reference ships no
 *     caller of it; the name is this library's);
 *   TURB_RESUME_PHI: Resume_phi.bin, the last pressure (not in the
 *     reference's set; with it a resumed run repeats the uninterrupted one
 *     bit for bit).  Without it, reading sets the pressure to 0 as a fresh
 *     reference process has it.
 * Reading resets the pressure-guess history.  The host helpers work without a
 * GPU. */
#define TURB_RESUME_GRID 1
#define TURB_RESUME_DEPOSIT 2
#define TURB_RESUME_PHI 4
typedef struct {
    double time, dt, dt_old;
    int iter, output_iter;
} turb_primary;
int turb_resume_write(turb_ctx *ctx, const char *dir, const turb_primary *prim, int flags);
int turb_resume_read(turb_ctx *ctx, const char *dir, turb_primary *prim, int flags);
int turb_petsc_vec_write(const char *path, const double *data, long long n);
int turb_petsc_vec_read(const char *path, double *data, long long n);
int turb_resume_primary_write(const char *dir, const turb_primary *prim);
int turb_resume_primary_read(const char *dir, turb_primary *prim);
int turb_resume_2d_write(const char *path, const double *data, int nx, int nz);
int turb_resume_2d_read(const char *path, double *data, int nx, int nz);

/* operator hooks used by the parity tests: y = A x on device fields */
int turb_helmholtz_apply(turb_ctx *ctx, char which, int ic, double dt, int field_x, int field_y);
int turb_pressure_apply(turb_ctx *ctx, int field_x, int field_y);

#ifdef __cplusplus
}
#endif
#endif
