// turb_internal.cuh -- device-side data layout shared by the kernels.
//
// Field layout in HBM: the DA order of the reference, [k][j][i] with i
// fastest, with the i-row padded to a pitch PX = round_up(NX, 8) doubles so
// that every row starts on a 64-byte boundary (TMA/vector friendly).  A field
// holds PX*NY*NZ doubles; the pad columns stay zero.  The pressure multigrid
// works on compact per-level arrays of the physical cells (nx*ny*nz).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define T_SOLID 2
#define T_FLUID 3
#define T_IMMERSED 5
#define T_BOUNDARY 7
#define T_BUFFER_SOLID 11

struct Dims {
    int nx, ny, nz;      // physical cells
    int NX, NY, NZ;      // DA points (cells + 1)
    int PX;              // padded row pitch (doubles)
    long long plane;     // PX*NY
    long long n;         // PX*NY*NZ
    __host__ __device__ long long at(int i, int j, int k) const
    {
        return ((long long)k * NY + j) * PX + i;
    }
};

// Open boundaries (params->inflow / outflow): the inflow and outflow planes
// of Inflow.c / Outflow.c as [NZ][NY] arrays (j fastest) and the RHS
// coefficients of the boundary-adjacent rows.  in = out = 0 is the closed box.
struct OpenBC {
    int in = 0, out = 0;
    int NY = 0;
    const double *u_in = nullptr;            // Velocity.G_inflow of u
    const double *c_in[4] = {};              // Concentration.G_inflow
    const double *out_f[7] = {};             // G_outflow of u, v, w, c_0..c_3
    // RHS terms: u at i = 1 (aw u_in), u at i = nx-2+1... see k_stencil.cu
    double u_aw = 0.0, u_ae = 0.0, vw_ae[2] = {0.0, 0.0};
    double c_aw[4] = {}, c_ae[4] = {};
    __host__ __device__ double pl(const double *a, int j, int k) const { return a[(long long)k * NY + j]; }
};

// 1-D grid arrays on the device (coordinates and metrics of Grid.c:595-708)
struct Geo {
    const double *xc, *yc, *zc, *xu, *yv, *zw;
    const double *mxc, *myc, *mzc, *mxu, *myv, *mzw;
};

// Two-point interpolation table (MyMath.c:13-43): node value at xq from
// (x0, x1): dx = x1 - x0, dq = xq - x0, flat = |dx| < 1e-8; the division by
// dx as div = 0: IEEE division, 1: one exact multiply by rdx = 1/dx (a power
// of two), 2: the reciprocal-based correctly rounded division (turb_div.cuh,
// rdxl its correction term), 3: its two-term quotient alone, for spacings
// that pass div_two_term_exact.
struct Interp2 {
    const double *dx, *dq, *rdx, *rdxl;
    const uint8_t *flat, *div;
};

// Four-point bilinear weights of MyMath.c:54-74 along one direction:
// W0 = |(xq - X0) / (X1 - X0)| (as a_D * (xq - X0)), W1 = 1 - W0.
struct W2 {
    const double *w0, *w1;
};

// ENO line tables of one (quantity, direction): buffer index b in [0, nb),
// interior node m = b - r + s0 for b in [r, nb - r).  Denominators and the
// stencil-position factors depend only on the grid and are built on the host
// with the reference's own expressions (ENO.c:159-244, ghost positions of the
// *_ENO_ghost_cells routines), so device results round identically.
struct EnoTab {
    int r, s0, e0, nb;
    const double *h1;    // P[b+1]-P[b]
    const double *h2;    // P[b+1]-P[b-1]
    const double *h3;    // P[b+2]-P[b-1]
    const double *g2;    // [nb*2]: k=b-1, k=b  -> (x_i-x_k)+(x_i-x_k1)
    const double *g3;    // [nb*3]: kstar=b-2,b-1,b -> three-product sum
    const double *rh1, *rh2, *rh3;   // RN(1/h*) for the reciprocal-based division
    const double *rl1, *rl2, *rl3;   // and its correction RN((1 - RN(1/h) h)/h)
    int fastdiv;         // 1: div_by_spacing (turb_div.cuh), 0: IEEE division
    const uint8_t *p2;   // per b: bit 0/1/2 set when h1/h2/h3 is a power of two, so that
                         // a/h = a*RN(1/h) exactly; bit 3/4/5 when the two-term
                         // quotient alone is exact (div_two_term_exact; fastdiv only)
    int gsrc[6];         // ghost b<r: [0..r), ghost b>=nb-r: [3..3+r) by ex
    double gm[6];        // 0: zero, 1: m*q[s0], 2: m*q[e0], 3: glo[line], 4: ghi[line]
    const double *glo = nullptr, *ghi = nullptr;   // x lines at open faces: [NZ][NY] planes
    int gNY = 0;
};

struct IbDev {
    int n;
    const int32_t *im;   // linear index in the pitched layout
    const int32_t *cnt;  // number of off-diagonal entries kept
    const int32_t *col;  // [n*8] pitched indices of kept off-diagonal entries
    const double *val;   // [n*8] ap_solid * fluid_coef
    const double *diag;  // [n]   ap_solid * (1 + sum of self coefficients)
};

// 1-D coefficient tables of one Helmholtz operator (separable rows of the
// *_form_LHS_matrix routines, wall folding included)
struct HelmTab {
    const double *apx, *apy, *apz;   // ap = apx[i] + apy[j] + apz[k]
    const double *aw, *ae, *as, *an, *ab, *af;   // 0 where the entry is absent
    double ap_solid;
    int q;                           // 0 u, 1 v, 2 w, 3 c
};

// FP32 copies for the inner solves of the mixed-precision defect correction
struct IbDevF {
    int n;
    const int32_t *im, *cnt, *col;
    const float *val, *diag;
};
struct HelmTabF {
    const float *apx, *apy, *apz, *aw, *ae, *as, *an, *ab, *af;
    float ap_solid;
    int q;
};

// Multigrid level (compact nx*ny*nz layout)
struct MgLevel {
    int nx, ny, nz;
    long long n;
    int cx, cy, cz;          // coarsened into the next level along x/y/z
    const double *rfx, *rfy, *rfz;  // 1/face distance [n+1]
    const double *dx, *dy, *dz;     // widths
    double pin;                     // corner east-face coefficient
};

// Maximum of two values whose magnitude is all that can appear (fabs results
// and products of non-negative factors: non-negative numbers, +inf, NaN) that
// keeps a NaN -- fmax drops a NaN operand, which would let a non-finite field
// pass a divergence gate.  It compares the bit patterns on the integer pipe,
// which leaves the FP64 pipe to the stencil arithmetic: for such values the
// order of the patterns as unsigned integers is the numeric order, and every
// NaN pattern (either sign) lies above +inf.
__device__ __forceinline__ double turb_maxbits(double a, double b)
{
    const unsigned long long x = (unsigned long long)__double_as_longlong(a);
    const unsigned long long y = (unsigned long long)__double_as_longlong(b);
    return __longlong_as_double((long long)(x > y ? x : y));
}
// turb_maxbits over the 32 lanes of a warp (every lane gets the result)
__device__ __forceinline__ double turb_warp_maxbits(double v)
{
    unsigned long long m = (unsigned long long)__double_as_longlong(v);
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    return __longlong_as_double((long long)m);
}

// Programmatic dependent launch.  A kernel launched with the programmatic
// stream serialisation attribute may be scheduled while the kernel before it
// on the stream drains; pdl_wait (before its first global-memory access)
// holds it until that kernel has completed and its writes are visible, and
// pdl_trigger lets the kernel after it be scheduled early.  In a kernel
// launched without the attribute both return at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

#define TURB_CHECK(x)                                                          \
    do {                                                                       \
        cudaError_t e_ = (x);                                                  \
        if (e_ != cudaSuccess) return turb_set_cuda_error(e_, __FILE__, __LINE__); \
    } while (0)

int turb_set_cuda_error(cudaError_t e, const char *file, int line);
