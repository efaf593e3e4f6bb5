// turb_diag.cuh -- inputs and outputs of the diagnostics and deposit kernels
// (k_diag.cu).
#pragma once
#include "../../include/turbins_gb300.h"
#include "turb_internal.cuh"

constexpr int DIAG_NQ = 3 + 4 * TURB_MAXCONC;   // ke, rate, visc, 4 per fraction

struct DiagIn {
    Dims d;
    Geo geo;
    const uint8_t *cst;
    const double *dxc, *dyc, *dzc;            // cell widths (Grid.c:633-671)
    const double *u, *v, *w;                  // face velocities
    const double *ubc, *vbc, *wbc, *ct;       // cell-centre velocities, total concentration
    const double *c[TURB_MAXCONC];
    int nconc;
    int particle[TURB_MAXCONC];
    double us[TURB_MAXCONC];                  // |Vs0|
    double y_ref;                             // yv[0]
    double hcoef;                             // 1 / (Ly Lz)
    double Cx, Cy, Cz;                        // 1/dEta^2, 1/dXi^2, 1/dPhi^2
    double kw[6];                             // wall ghost factors: -1 no-slip, +1 free-slip
    OpenBC ob;                                // open faces (viscous dissipation)
    const int32_t *iy;                        // bed index [NZ][NX]
    const double *dep;                        // deposited heights [nconc][NZ][NX] or null
};

struct DiagOut {
    double *sums;         // DIAG_NQ volume sums
    double *heights;      // [nconc][NX]
    double *bed_sums;     // per fraction: ep_passive, sed_rate
    double *sed_bottom;   // [nconc][NZ][NX]
};

struct DepIn {
    int nconc;
    double dt;
    double us[TURB_MAXCONC], alpha[TURB_MAXCONC];
    const double *c[TURB_MAXCONC], *c_old[TURB_MAXCONC];
};

long long diag_scratch_doubles(const Dims &d);
void launch_diagnostics(cudaStream_t s, const DiagIn &a, double *scratch, DiagOut *o);
void launch_bed_index(cudaStream_t s, const Dims &d, const uint8_t *cst, int32_t *iy);
void launch_deposit(cudaStream_t s, const Dims &d, const int32_t *iy, const DepIn &a, double *dep);
