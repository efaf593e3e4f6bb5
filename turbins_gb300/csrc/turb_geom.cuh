// turb_geom.cuh -- the immersed-boundary geometry set-up on the device
// (k_geom.cu): signed distance to a bottom surface by level-set
// reinitialisation, sdf at the u/v/w nodes, node status tagging.
#pragma once
#include "turb_internal.cuh"

struct GeomArgs {
    Dims d;
    // device arrays, NX / NY / NZ entries
    const double *xc, *yc, *zc, *xu, *yv, *zw;
    const double *mxu, *myv, *mzw;        // face metrics metric_xu/yv/zw
    const double *dxc, *dyc, *dzc;        // cell widths dx_c/dy_c/dz_c
    double a_dEta, a_dXi, a_dPhi;         // 1/dEta, 1/dXi, 1/dPhi
    double dt;                            // fictitious time step
    int max_iterations;                   // Surface_find_exact_sdf passes 500
};

struct GeomOut {
    double *sdf[4];        // c, u, v, w (G_c_sdf, G_u_sdf, G_v_sdf, G_w_sdf)
    uint8_t *st[4];        // u, v, w, c status
    int iterations;        // Godunov steps taken
    double last_error;     // the last NORM2 change
};

// scratch: geom_scratch_doubles(d) doubles and d.n bytes
long long geom_scratch_doubles(const Dims &d);
cudaError_t geom_setup(cudaStream_t s, const GeomArgs &a, const double *ipos, double *scratch, uint8_t *tmp,
                       GeomOut *o);

// ghost-cell stencils of one quantity, device arrays of n (im, nf, bcoef),
// 8n (fidx, fcoef) and 12n (pts: normal, control point, image point, node
// point; may be null) entries; im / fidx are DA linear indices
struct GeomIb {
    int n = 0;
    int32_t *im = nullptr, *nf = nullptr, *fidx = nullptr;
    double *fcoef = nullptr, *bcoef = nullptr, *pts = nullptr;
};

cudaError_t geom_ib_count(cudaStream_t s, const Dims &d, const uint8_t *st, int *rows, int *n);
cudaError_t geom_ib_build(cudaStream_t s, const GeomArgs &a, int q, const double *sdf, const uint8_t *st,
                          const int *rows, int *node, const GeomIb &o);
