// turb_api.cu -- the C ABI (include/turbins_gb300.h): context set-up, host
// tables, field transfer and the per-step driver.  All arithmetic of the hot
// path runs in the kernels of k_*.cu; the host only builds the 1-D tables of
// grid-only quantities (with the reference's own expressions, so device
// roundings match) and sequences launches on the context's stream.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/turbins_gb300.h"
#include "turb_internal.cuh"
#include "turb_diag.cuh"
#include "turb_geom.cuh"
#include "turb_div.cuh"

// open boundaries (k_open.cu)
int open_parts(const Dims &d);
void launch_inflow_u(cudaStream_t s, const Dims &d, const uint8_t *st_u, const double *yv, const double *zw,
                     double tf, double *in, double *part, double *influx);
void launch_inflow_c(cudaStream_t s, const Dims &d, const uint8_t *st_c, double tf, double *in);
void launch_outflow_conv(cudaStream_t s, const Dims &d, const uint8_t *st, double coef, const double *q, double *out);
void launch_outflow_mass(cudaStream_t s, const Dims &d, const uint8_t *st_u, const double *yv, const double *zw,
                         const double *influx, double *out, double *part, double *res);
void launch_plane_axpby(cudaStream_t s, int n, double a, const double *old, double b, double *out);
void launch_plane_to_field(cudaStream_t s, const Dims &d, const double *pl, int set, double *q);
void launch_field_to_plane(cudaStream_t s, const Dims &d, const double *q, double *pl);

// restart files (k_resume.cu, turb_resume.cu)
void launch_pack_be(cudaStream_t s, const Dims &d, const double *src, unsigned long long *dst);
void launch_pack_status_be(cudaStream_t s, const Dims &d, const uint8_t *st, unsigned long long *dst);
void launch_unpack_be(cudaStream_t s, const Dims &d, const unsigned long long *src, double *dst);
int petsc_vec_write_be(const char *path, const void *be_words, long long n);
int petsc_vec_read_be(const char *path, void *be_words, long long n);
std::string resume_path(const char *dir, const char *name);
#include "turb_kernels.cuh"
#include "turb_mg.cuh"
#include "turb_net.cuh"

static char g_errmsg[512] = "";

int turb_set_error_text(const char *msg)
{
    snprintf(g_errmsg, sizeof(g_errmsg), "%s", msg);
    return TURB_ERR_CUDA;
}

int turb_set_cuda_error(cudaError_t e, const char *file, int line)
{
    snprintf(g_errmsg, sizeof(g_errmsg), "%s (%s:%d)", cudaGetErrorString(e), file, line);
    return TURB_ERR_CUDA;
}


// extra launchers defined at the end of this file
void launch_pressure_apply(cudaStream_t s, const Dims &d, const uint8_t *st, const Geo &g, double dEta, double dXi,
                           double dPhi, const double *x, double *y);

namespace {

struct DevBuf {
    std::vector<void *> ptrs;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T *alloc(size_t n)
    {
        void *p = nullptr;
        if (n == 0) n = 1;
        cudaError_t e = cudaMalloc(&p, n * sizeof(T));
        if (e != cudaSuccess) { err = e; return nullptr; }
        cudaMemset(p, 0, n * sizeof(T));
        ptrs.push_back(p);
        return (T *)p;
    }
    template <typename T>
    T *upload(const std::vector<T> &h)
    {
        T *p = alloc<T>(h.size());
        if (p && !h.empty()) cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
        return p;
    }
    void release()
    {
        for (void *p : ptrs) cudaFree(p);
        ptrs.clear();
    }
};

}  // namespace

// Algorithmic bytes per DA point of one launch of the step's kernels (each
// array a kernel reads or writes counted once, status masks at 1 byte):
// ENO x pass: q, advecting velocity read, conv written; y / z passes also
// read conv.  FP64 Jacobi sweep: x, b, status read, x' written; FP64
// Helmholtz residual: x, b, status read, FP32 r written; FP32 Jacobi sweep:
// r, e, status read, e' written (the first sweep starts from e = 0).  An
// immersed row: its diagonal, count, eight columns, values and x entries, b
// and the row's result.
constexpr double ENO_X_BYTES = 24.0, ENO_YZ_BYTES = 32.0;
constexpr double HELM_JACOBI_BYTES = 25.0, HELM_RESID64_BYTES = 21.0;
constexpr double HELM_JAC32_FIRST_BYTES = 9.0, HELM_JAC32_BYTES = 13.0;
constexpr double IB_ROW_BYTES = 8.0 + 4.0 + 8.0 * (4.0 + 8.0 + 8.0) + 8.0 + 8.0;

struct turb_ctx {
    Dims d;
    turb_params prm;
    cudaStream_t s = nullptr;
    DevBuf mem;
    std::vector<double> xc, yc, zc, xu, yv, zw, mxc, myc, mzc, mxu, myv, mzw;
    double dEta, dXi, dPhi;
    Geo geo;
    double *fld[64] = {nullptr};
    double *old[3 + TURB_MAXCONC] = {nullptr};
    double *jtmp = nullptr;
    uint8_t *st[4] = {nullptr};
    IbDev ib[4];
    Interp2 icx, icy, icz, iyv;
    TransW tw;
    EnoTab eno[4][3];
    EnoTab eno_cy[TURB_MAXCONC];
    HelmTab helm[3], helm_c[TURB_MAXCONC];
    HelmTabF helmf[3], helmf_c[TURB_MAXCONC];
    IbDevF ibf[4];
    float *hrf = nullptr, *he0 = nullptr, *he1 = nullptr;   // defect-correction buffers
    int hmode = TURB_HMODE_MIXED;
    // the 1/dt term of each Helmholtz diagonal (u, v, w, c_0..) and the dt it
    // was last updated for (0: not yet)
    double adt[3 + TURB_MAXCONC] = {};
    double adt_dt[3 + TURB_MAXCONC] = {};
    int hinner = 5;   // FP32 Jacobi sweeps per defect-correction step (5: the fewest that keep 2 outer steps at 512x256x256)
    const double *pcx, *pcy, *pcz;
    ProjArgs proj;
    // pressure
    int pmode = TURB_PMODE_MIXED;
    MgHier<double> H64;
    MgHier<float> H32;
    double *px, *pbw, *pr, *pz, *pp, *pq, *pro;
    PcgScal *sc;
    double *part, *dscal;
    double *hscal = nullptr;   // pinned host scalars
    long long nparts = 0;
    long long launches = 0;
    // per-group CUDA-event timing (turb_profile_*)
    int prof = 0;
    struct Rec { int g, nl; double bytes; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    double prof_ms[TURB_PROF_NGROUPS] = {0};
    long long prof_nl[TURB_PROF_NGROUPS] = {0};
    double prof_bytes[TURB_PROF_NGROUPS] = {0};   // algorithmic bytes of the timed launches
    cudaEvent_t user_ev[8] = {nullptr};
    // CUDA graphs: V-cycle per pressure mode, CG vector step (restart / not),
    // FP32 inner sweeps of each Helmholtz field
    cudaGraphExec_t g_mg[2] = {nullptr, nullptr};
    cudaGraphExec_t g_pcg[2] = {nullptr, nullptr};
    cudaGraphExec_t g_inner[3 + TURB_MAXCONC] = {nullptr};
    int g_inner_n[3 + TURB_MAXCONC] = {0};
    int use_graphs = 1;
    // red-black Gauss-Seidel sweeps before / after the coarse correction per
    // level (0 = the finest) and pressure mode, set in turb_create
    int mg_pre[2][TURB_MG_MAXLEV], mg_post[2][TURB_MG_MAXLEV];
    int mg_split = 1;   // colour-split storage of the FP32 levels
    // pressure initial guess: history of the last two solutions per RK stage
    int guess_mode = TURB_GUESS_PREVIOUS;
    int guess_stages = 3;   // RK stages (bit 0: first, bit 1: second) that try the candidate guess
    int stage = 0;
    double *ph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    double *pw[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};   // the right-hand sides W b of ph
    int galerkin = 0;   // the learned candidate goes through the Galerkin fit with the history
    // kernel variants (TURB_KV_*): FP32 sweeps marching along k through
    // shared-memory plane tiles, ENO y / z lines walked in segments
    int kvariant = TURB_KV_ENO_SEGMENTS | TURB_KV_PDL;
    long long mg_cluster_cells = 1 << 17;   // TURB_KV_CLUSTER_VCYCLE from the first level of at most this many cells
    // TURB_KV_SWEEP_PAIRS: the finest FP32 level's two-sweeps-per-pass smoother
    RbTbPlan tbplan;
    int host_copy = TURB_HOST_COPY_KERNEL;   // how page-locked host arrays move (turb_set_host_copy)
    float *tb_x1 = nullptr;   // its second x array (ping-pong)
    int *tb_err = nullptr;    // set by a block whose copy wait timed out
    double div_gate = 0.0;       // > 0: Poisson solves also reach dt * max|b - A phi| <= div_gate
    double p_dt = 0.0;           // dt of the last Pressure_set_RHS
    long long gate_tightened = 0;
    long long gate_floor = 0;   // solves the gate let go at the residual's round-off floor
    int nh[2] = {0, 0};
    int guess_taken = 0, guess_tried = 0;
    double guess_logsum = 0.0;   // sum of log(|r candidate| / |r previous|)
    // learned guess (k_net.cu) and the snapshot store that training reads
    TurbNet *net = nullptr;
    TurbSnaps *snaps = nullptr;
    // diagnostics: cell widths dx_c, dy_c, dz_c (Grid.c:633-671) and scratch
    double *diag_dxc = nullptr, *diag_dyc = nullptr, *diag_dzc = nullptr, *diag_scr = nullptr;
    // bed index [NZ][NX] and deposited heights [nconc][NZ][NX]
    int32_t *bed_iy = nullptr;
    double *dep = nullptr;
    int deposit_on = 0;
    // open boundaries: the planes of Inflow.c / Outflow.c ([NZ][NY]) and the
    // device view the kernels take; conc x-pass ENO tables per fraction
    OpenBC ob;
    double *pl_in_u = nullptr, *pl_in_c[TURB_MAXCONC] = {}, *pl_out[3 + TURB_MAXCONC] = {},
           *pl_out_old[3 + TURB_MAXCONC] = {};
    double open_U = 0.0, open_time_c = 1.0;
    double time = 0.0;            // simulated time, advanced by turb_step (GVG_bag.time)
    int open_transient = 0;
    double *open_scr = nullptr;   // partials; influx at [open_parts], mass results after it
    EnoTab eno_cx[TURB_MAXCONC];
    // restart staging: one field as big-endian words, on the device and pinned
    unsigned long long *rs_dev = nullptr;
    void *rs_host = nullptr;
    // host transfers: two contiguous device staging buffers of one DA field,
    // a copy stream and the events that hand a buffer between the streams
    double *xfer[2] = {nullptr, nullptr};
    cudaStream_t cs = nullptr, cs2 = nullptr;   // copy streams of the staged host copies (even / odd fields)
    // turb_step_host: the stream that moves the late fields, its events and
    // the step's hooks (set only during that call)
    cudaStream_t ios = nullptr;
    // start, dp in, phi in, dp / phi out, c in, c out
    cudaEvent_t io_ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    struct StepIo *io = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_freed[2] = {nullptr, nullptr};
    // ghost-cell stencils made by turb_geometry (one allocation per quantity)
    GeomIb gib[4];
    void *gib_buf[4] = {nullptr, nullptr, nullptr, nullptr};
};

namespace {

inline long long da_to_pitched(const Dims &d, long long L)
{
    long long i = L % d.NX, t = L / d.NX, j = t % d.NY, k = t / d.NY;
    return d.at((int)i, (int)j, (int)k);
}

// Grid_compute_metric_coefficients, Grid.c:595-708
void metrics(turb_ctx *c)
{
    int NX = c->d.NX, NY = c->d.NY, NZ = c->d.NZ;
    c->dEta = 1.0 / (double)c->d.nx;
    c->dXi = 1.0 / (double)c->d.ny;
    c->dPhi = 1.0 / (double)c->d.nz;
    auto &xc = c->xc, &yc = c->yc, &zc = c->zc, &xu = c->xu, &yv = c->yv, &zw = c->zw;
    c->mxc.assign(NX, 0.0); c->myc.assign(NY, 0.0); c->mzc.assign(NZ, 0.0);
    c->mxu.assign(NX, 0.0); c->myv.assign(NY, 0.0); c->mzw.assign(NZ, 0.0);
    for (int i = 1; i < NX - 1; i++) c->mxu[i] = c->dEta / (xc[i] - xc[i - 1]);
    c->mxu[0] = 0.5 * c->dEta / (xc[0] - xu[0]);
    c->mxu[NX - 1] = 0.5 * c->dEta / (xu[NX - 1] - xc[NX - 2]);
    for (int i = 1; i < NY - 1; i++) c->myv[i] = c->dXi / (yc[i] - yc[i - 1]);
    c->myv[0] = 0.5 * c->dXi / (yc[0] - yv[0]);
    c->myv[NY - 1] = 0.5 * c->dXi / (yv[NY - 1] - yc[NY - 2]);
    for (int i = 1; i < NZ - 1; i++) c->mzw[i] = c->dPhi / (zc[i] - zc[i - 1]);
    c->mzw[0] = 0.5 * c->dPhi / (zc[0] - zw[0]);
    c->mzw[NZ - 1] = 0.5 * c->dPhi / (zw[NZ - 1] - zc[NZ - 2]);
    for (int i = 0; i < NX - 1; i++) c->mxc[i] = c->dEta / (xu[i + 1] - xu[i]);
    c->mxc[NX - 1] = c->dEta / (xc[NX - 1] - xc[NX - 2]);
    for (int i = 0; i < NY - 1; i++) c->myc[i] = c->dXi / (yv[i + 1] - yv[i]);
    c->myc[NY - 1] = c->dXi / (yc[NY - 1] - yc[NY - 2]);
    for (int i = 0; i < NZ - 1; i++) c->mzc[i] = c->dPhi / (zc[i + 1] - zc[i]);
    c->mzc[NZ - 1] = c->dPhi / (zc[NZ - 1] - zc[NZ - 2]);
}

Interp2 mk_interp2(DevBuf &m, int n, const std::vector<double> &X0, const std::vector<double> &X1,
                   const std::vector<double> &XQ, int first)
{
    std::vector<double> dx(n, 1.0), dq(n, 0.0), rdx(n, 1.0), rdxl(n, 0.0);
    std::vector<uint8_t> fl(n, 0), dm(n, 0);
    for (int t = first; t < n; t++) {
        dx[t] = X1[t] - X0[t];
        dq[t] = XQ[t] - X0[t];
        fl[t] = std::fabs(X1[t] - X0[t]) < 1.0e-8;
        // the slope's division: positive spacings in a safe exponent range
        // take the reciprocal forms, which round exactly as the division
        double h = dx[t];
        int e = 0;
        if (h > 0.0 && std::isfinite(h) && std::frexp(h, &e) && e > -500 && e < 500) {
            rdx[t] = 1.0 / h;
            rdxl[t] = recip_low(h, rdx[t]);
            dm[t] = std::frexp(h, &e) == 0.5 ? 1 : (div_two_term_exact(h, rdx[t], rdxl[t]) ? 3 : 2);
        }
    }
    Interp2 o;
    o.dx = m.upload(dx);
    o.dq = m.upload(dq);
    o.rdx = m.upload(rdx);
    o.rdxl = m.upload(rdxl);
    o.flat = m.upload(fl);
    o.div = m.upload(dm);
    return o;
}

// W0 = |(xq - X0) * (1/(X1 - X0))|, W1 = 1 - W0 (MyMath.c:63-72)
W2 mk_w2(DevBuf &m, int n, int first, int last, const std::vector<double> &X0, const std::vector<double> &X1,
         const std::vector<double> &XQ)
{
    std::vector<double> w0(n, 0.0), w1(n, 0.0);
    for (int t = first; t <= last; t++) {
        double a = 1.0 / (X1[t] - X0[t]);
        w0[t] = std::fabs((XQ[t] - X0[t]) * a);
        w1[t] = 1.0 - w0[t];
    }
    W2 o;
    o.w0 = m.upload(w0);
    o.w1 = m.upload(w1);
    return o;
}

struct GhostRule {
    int wall;      // 1: node on the wall (normal component), 0: mirror
    double pos;    // wall coordinate
    double mult;
};

// ENO line tables (positions and ghost rules of the *_ENO_ghost_cells routines)
EnoTab mk_eno(DevBuf &m, int r, const std::vector<double> &pos, int s0, int e0, GhostRule lo, GhostRule hi)
{
    int nb = e0 - s0 + 1 + 2 * r;
    std::vector<double> P(nb, 0.0);
    for (int b = r; b < nb - r; b++) P[b] = pos[b - r + s0];
    EnoTab T;
    T.r = r; T.s0 = s0; T.e0 = e0; T.nb = nb;
    for (int t = 0; t < 6; t++) { T.gsrc[t] = 0; T.gm[t] = 0.0; }
    for (int ex = 0; ex < r; ex++) {
        int gi = ex;
        if (lo.wall) {
            int ii = 2 * r - ex - 2;
            if (ex == r - 1) { P[gi] = lo.pos; T.gsrc[ex] = 0; }
            else { P[gi] = 2.0 * lo.pos - P[ii]; T.gsrc[ex] = lo.mult == 0.0 ? 0 : 1; T.gm[ex] = lo.mult; }
        } else {
            int ii = 2 * r - ex - 1;
            P[gi] = 2.0 * lo.pos - P[ii];
            T.gsrc[ex] = 1; T.gm[ex] = lo.mult;
        }
    }
    for (int ex = 0; ex < r; ex++) {
        int gi = nb - ex - 1;
        if (hi.wall) {
            int ii = nb - 2 * r + ex + 1;
            if (ex == r - 1) { P[gi] = hi.pos; T.gsrc[3 + ex] = 0; }
            else { P[gi] = 2.0 * hi.pos - P[ii]; T.gsrc[3 + ex] = hi.mult == 0.0 ? 0 : 2; T.gm[3 + ex] = hi.mult; }
        } else {
            int ii = nb - 2 * r + ex;
            P[gi] = 2.0 * hi.pos - P[ii];
            T.gsrc[3 + ex] = 2; T.gm[3 + ex] = hi.mult;
        }
    }
    std::vector<double> h1(nb, 1.0), h2(nb, 1.0), h3(nb, 1.0), g2(2 * nb, 0.0), g3(3 * nb, 0.0);
    for (int b = 0; b < nb - 1; b++) h1[b] = P[b + 1] - P[b];
    for (int b = 1; b < nb - 1; b++) h2[b] = P[b + 1] - P[b - 1];
    for (int b = 1; b < nb - 2; b++) h3[b] = P[b + 2] - P[b - 1];
    for (int c = 1; c < nb - 1; c++) {
        double xi = P[c];
        g2[2 * c + 0] = (xi - P[c - 1]) + (xi - P[c]);
        g2[2 * c + 1] = (xi - P[c]) + (xi - P[c + 1]);
        for (int t = 0; t < 3; t++) {
            int ks = c - 2 + t;
            if (ks < 0 || ks + 2 >= nb) continue;
            double a = P[ks], bb = P[ks + 1], e = P[ks + 2];
            g3[3 * c + t] = (xi - a) * (xi - bb) + (xi - bb) * (xi - e) + (xi - a) * (xi - e);
        }
    }
    T.h1 = m.upload(h1);
    T.h2 = m.upload(h2);
    T.h3 = m.upload(h3);
    std::vector<double> r1(nb), r2(nb), r3(nb), l1(nb), l2(nb), l3(nb);
    for (int b = 0; b < nb; b++) {
        r1[b] = 1.0 / h1[b]; r2[b] = 1.0 / h2[b]; r3[b] = 1.0 / h3[b];
        l1[b] = recip_low(h1[b], r1[b]); l2[b] = recip_low(h2[b], r2[b]); l3[b] = recip_low(h3[b], r3[b]);
    }
    T.rh1 = m.upload(r1);
    T.rh2 = m.upload(r2);
    T.rh3 = m.upload(r3);
    T.rl1 = m.upload(l1);
    T.rl2 = m.upload(l2);
    T.rl3 = m.upload(l3);
    T.fastdiv = 1;   // reciprocal-based, correctly rounded (turb_div.cuh); 0 = IEEE division
    // power-of-two spacings (uniform grids with 2^k cells per unit length):
    // the reciprocal is exact and a/h = a*(1/h) is the same real number, so
    // one multiplication rounds exactly as the division does
    auto pow2 = [](double h) {
        int e;
        return h > 0.0 && std::isfinite(h) && std::frexp(h, &e) == 0.5;
    };
    // other spacings whose two-term quotient alone rounds as the division
    // for every numerator (div_two_term_exact, turb_div.cuh): bits 3-5
    std::vector<uint8_t> p2(nb, 0);
    for (int b = 0; b < nb; b++) {
        int f = (pow2(h1[b]) ? 1 : 0) | (pow2(h2[b]) ? 2 : 0) | (pow2(h3[b]) ? 4 : 0);
        if (!(f & 1) && div_two_term_exact(h1[b], r1[b], l1[b])) f |= 8;
        if (!(f & 2) && div_two_term_exact(h2[b], r2[b], l2[b])) f |= 16;
        if (!(f & 4) && div_two_term_exact(h3[b], r3[b], l3[b])) f |= 32;
        p2[b] = (uint8_t)f;
    }
    T.p2 = m.upload(p2);
    T.g2 = m.upload(g2);
    T.g3 = m.upload(g3);
    return T;
}

double slip(int noslip) { return noslip ? -1.0 : 1.0; }

void build_eno(turb_ctx *c)
{
    int r = c->prm.eno_order, nx = c->d.nx, ny = c->d.ny, nz = c->d.nz;
    const int *ns = c->prm.wall_noslip;
    auto M = [](double p, double mult) { return GhostRule{0, p, mult}; };
    auto Wl = [](double p, double mult) { return GhostRule{1, p, mult}; };
    double x0 = c->xu[0], x1 = c->xu[nx], y0 = c->yv[0], y1 = c->yv[ny], z0 = c->zw[0], z1 = c->zw[nz];
    // u: Velocity.c:2124-2352
    c->eno[0][0] = mk_eno(c->mem, r, c->xu, 1, nx - 1, Wl(x0, -1.0), Wl(x1, 0.0));
    c->eno[0][1] = mk_eno(c->mem, r, c->yc, 0, ny - 1, M(y0, slip(ns[2])), M(y1, slip(ns[3])));
    c->eno[0][2] = mk_eno(c->mem, r, c->zc, 0, nz - 1, M(z0, slip(ns[4])), M(z1, slip(ns[5])));
    // v: Velocity.c:2356-2575
    c->eno[1][0] = mk_eno(c->mem, r, c->xc, 0, nx - 1, M(x0, slip(ns[0])), M(x1, slip(ns[1])));
    c->eno[1][1] = mk_eno(c->mem, r, c->yv, 1, ny - 1, Wl(y0, 0.0), Wl(y1, 0.0));
    c->eno[1][2] = mk_eno(c->mem, r, c->zc, 0, nz - 1, M(z0, slip(ns[4])), M(z1, slip(ns[5])));
    // w: Velocity.c:2579-2801
    c->eno[2][0] = mk_eno(c->mem, r, c->xc, 0, nx - 1, M(x0, slip(ns[0])), M(x1, slip(ns[1])));
    c->eno[2][1] = mk_eno(c->mem, r, c->yc, 0, ny - 1, M(y0, slip(ns[2])), M(y1, slip(ns[3])));
    c->eno[2][2] = mk_eno(c->mem, r, c->zw, 1, nz - 1, Wl(z0, 0.0), Wl(z1, 0.0));
    // c: Conc.c:1021-1220 (Neumann; Robin top for particles with sedimentation;
    // salinity top ghosts take the Neumann value, the reference leaves them unset)
    c->eno[3][0] = mk_eno(c->mem, r, c->xc, 0, nx - 1, M(x0, 1.0), M(x1, 1.0));
    c->eno[3][1] = mk_eno(c->mem, r, c->yc, 0, ny - 1, M(y0, 1.0), M(y1, 1.0));
    c->eno[3][2] = mk_eno(c->mem, r, c->zc, 0, nz - 1, M(z0, 1.0), M(z1, 1.0));
    for (int ic = 0; ic < c->prm.nconc; ic++) {
        EnoTab T = c->eno[3][1];
        if (c->prm.ctype[ic] == TURB_PARTICLE && c->prm.sedimentation) {
            double coef = 2.0 / (c->prm.pe[ic] * c->dXi) * c->myv[ny];
            double Vs = std::fabs(c->prm.vs0[ic]);
            double f = (coef - Vs) / (coef + Vs);
            for (int ex = 0; ex < r; ex++) T.gm[3 + ex] = f;
        }
        c->eno_cy[ic] = T;
    }
}

// separable 1-D tables of the Helmholtz rows (Velocity.c:449-1474, Conc.c:390-730)
HelmTab mk_helm(turb_ctx *c, int q, int ic)
{
    int nx = c->d.nx, ny = c->d.ny, nz = c->d.nz, NX = c->d.NX, NY = c->d.NY, NZ = c->d.NZ;
    const int *ns = c->prm.wall_noslip;
    double coefRe = q == 3 ? c->prm.pe[ic] : c->prm.re;
    double Cx = -1.0 / (coefRe * c->dEta * c->dEta), Cy = -1.0 / (coefRe * c->dXi * c->dXi),
           Cz = -1.0 / (coefRe * c->dPhi * c->dPhi);
    std::vector<double> apx(NX, 0.0), apy(NY, 0.0), apz(NZ, 0.0), aw(NX, 0.0), ae(NX, 0.0), as(NY, 0.0),
        an(NY, 0.0), ab(NZ, 0.0), af(NZ, 0.0);
    auto wallfold = [](double a, int noslip) { return noslip ? -a : a; };
    // x
    for (int i = 0; i < NX; i++) {
        double px, ex, wx;
        if (q == 0) {
            if (i < 1 || i > nx - 1) continue;
            px = c->mxu[i]; ex = c->mxc[i]; wx = c->mxc[i - 1];
        } else {
            if (i > nx - 1) continue;
            px = c->mxc[i]; ex = c->mxu[i + 1]; wx = c->mxu[i];
        }
        double a_w = Cx * px * wx, a_e = Cx * px * ex;
        apx[i] = -Cx * px * (ex + wx);
        if (q == 0) {
            aw[i] = (i - 1 >= 1) ? a_w : 0.0;
            ae[i] = (i + 1 <= nx - 1) ? a_e : 0.0;
        } else {
            aw[i] = i > 0 ? a_w : 0.0;
            ae[i] = i < nx - 1 ? a_e : 0.0;
            // open faces drop the wall fold, the face value goes to the RHS:
            // concentration at both faces (Conc.c:583-606), v and w at the
            // outflow face, where the east column is not inserted either
            // (Velocity.c:989-1011, 1336-1358)
            if (i == 0 && !(q == 3 && c->ob.in)) apx[i] += q == 3 ? a_w : wallfold(a_w, ns[0]);
            if (i == nx - 1 && !c->ob.out) apx[i] += q == 3 ? a_e : wallfold(a_e, ns[1]);
        }
    }
    // y
    for (int j = 0; j < NY; j++) {
        double py, ny_, sy;
        if (q == 1) {
            if (j < 1 || j > ny - 1) continue;
            py = c->myv[j]; ny_ = c->myc[j]; sy = c->myc[j - 1];
        } else {
            if (j > ny - 1) continue;
            py = c->myc[j]; ny_ = c->myv[j + 1]; sy = c->myv[j];
        }
        double a_s = Cy * py * sy, a_n = Cy * py * ny_;
        apy[j] = -Cy * py * (ny_ + sy);
        if (q == 1) {
            as[j] = (j - 1 >= 1) ? a_s : 0.0;
            an[j] = (j + 1 <= ny - 1) ? a_n : 0.0;
        } else {
            as[j] = j > 0 ? a_s : 0.0;
            an[j] = j < ny - 1 ? a_n : 0.0;
            if (j == 0) apy[j] += q == 3 ? a_s : wallfold(a_s, ns[2]);
            if (j == ny - 1) {
                if (q == 3) {
                    double cf = a_n;
                    if (c->prm.ctype[ic] == TURB_PARTICLE) {
                        double b = 2.0 / (coefRe * c->dXi) * ny_;
                        cf = a_n * (b - std::fabs(c->prm.vs0[ic])) / (b + std::fabs(c->prm.vs0[ic]));
                    }
                    apy[j] += cf;
                } else {
                    apy[j] += wallfold(a_n, ns[3]);
                }
            }
        }
    }
    // z
    for (int k = 0; k < NZ; k++) {
        double pz, fz, bz;
        if (q == 2) {
            if (k < 1 || k > nz - 1) continue;
            pz = c->mzw[k]; bz = c->mzc[k - 1]; fz = c->mzc[k];
        } else {
            if (k > nz - 1) continue;
            pz = c->mzc[k]; bz = c->mzw[k]; fz = c->mzw[k + 1];
        }
        double a_b = Cz * pz * bz, a_f = Cz * pz * fz;
        apz[k] = -Cz * pz * (bz + fz);
        if (q == 2) {
            ab[k] = (k - 1 >= 1) ? a_b : 0.0;
            af[k] = (k + 1 <= nz - 1) ? a_f : 0.0;
        } else {
            ab[k] = k > 0 ? a_b : 0.0;
            af[k] = k < nz - 1 ? a_f : 0.0;
            if (k == 0) apz[k] += q == 3 ? a_b : wallfold(a_b, ns[4]);
            if (k == nz - 1) apz[k] += q == 3 ? a_f : wallfold(a_f, ns[5]);
        }
    }
    HelmTab h;
    h.apx = c->mem.upload(apx); h.apy = c->mem.upload(apy); h.apz = c->mem.upload(apz);
    h.aw = c->mem.upload(aw); h.ae = c->mem.upload(ae); h.as = c->mem.upload(as); h.an = c->mem.upload(an);
    h.ab = c->mem.upload(ab); h.af = c->mem.upload(af);
    h.ap_solid = -Cx * c->mxc[0] - Cy * c->myc[0] - Cz * c->mzc[0];
    h.q = q;
    return h;
}

IbDev mk_ib(turb_ctx *c, int q, const turb_ib_desc &ib, double aps)
{
    IbDev o;
    o.n = ib.n;
    std::vector<int32_t> im(ib.n), cnt(ib.n), col((size_t)ib.n * 8, 0);
    std::vector<double> val((size_t)ib.n * 8, 0.0), dg(ib.n);
    for (int t = 0; t < ib.n; t++) {
        long long L = ib.im[t];
        double self = 1.0;
        int n = 0;
        for (int g = 0; g < ib.nf[t]; g++)
            if (ib.fidx[t * 8 + g] == ib.im[t]) self += ib.fcoef[t * 8 + g];
        for (int g = 0; g < ib.nf[t]; g++) {
            double cf = ib.fcoef[t * 8 + g];
            if (ib.fidx[t * 8 + g] != ib.im[t] && std::fabs(cf) >= 1.0e-8) {
                col[(size_t)t * 8 + n] = (int32_t)da_to_pitched(c->d, ib.fidx[t * 8 + g]);
                val[(size_t)t * 8 + n] = aps * cf;
                n++;
            }
        }
        im[t] = (int32_t)da_to_pitched(c->d, L);
        cnt[t] = n;
        dg[t] = aps * self;
    }
    (void)q;
    o.im = c->mem.upload(im);
    o.cnt = c->mem.upload(cnt);
    o.col = c->mem.upload(col);
    o.val = c->mem.upload(val);
    o.diag = c->mem.upload(dg);
    return o;
}

HelmTabF mk_helmf(turb_ctx *c, const HelmTab &h)
{
    // x tables padded with zeros to the row pitch, for the four-point loads
    // of the vectorised sweep
    auto cp = [&](const double *dp, int n, int npad) {
        std::vector<double> tmp(n);
        cudaMemcpy(tmp.data(), dp, sizeof(double) * n, cudaMemcpyDeviceToHost);
        std::vector<float> f(tmp.begin(), tmp.end());
        f.resize(std::max(n, npad), 0.0f);
        return (const float *)c->mem.upload(f);
    };
    HelmTabF o;
    int NX = c->d.NX, NY = c->d.NY, NZ = c->d.NZ, PX = c->d.PX;
    o.apx = cp(h.apx, NX, PX); o.aw = cp(h.aw, NX, PX); o.ae = cp(h.ae, NX, PX);
    o.apy = cp(h.apy, NY, 0); o.as = cp(h.as, NY, 0); o.an = cp(h.an, NY, 0);
    o.apz = cp(h.apz, NZ, 0); o.ab = cp(h.ab, NZ, 0); o.af = cp(h.af, NZ, 0);
    o.ap_solid = (float)h.ap_solid;
    o.q = h.q;
    return o;
}

IbDevF mk_ibf(turb_ctx *c, const IbDev &ib)
{
    IbDevF o;
    o.n = ib.n;
    o.im = ib.im; o.cnt = ib.cnt; o.col = ib.col;
    std::vector<double> v((size_t)std::max(ib.n, 1) * 8, 0.0), dg(std::max(ib.n, 1), 1.0);
    if (ib.n > 0) {
        cudaMemcpy(v.data(), ib.val, sizeof(double) * 8 * ib.n, cudaMemcpyDeviceToHost);
        cudaMemcpy(dg.data(), ib.diag, sizeof(double) * ib.n, cudaMemcpyDeviceToHost);
    }
    std::vector<float> vf(v.begin(), v.end()), df(dg.begin(), dg.end());
    o.val = c->mem.upload(vf);
    o.diag = c->mem.upload(df);
    return o;
}

// multigrid hierarchy (same coarsening rule as the CPU oracle)
struct HostLev {
    int nx, ny, nz, cx = 0, cy = 0, cz = 0;
    std::vector<double> D[3], F[3];
    double pin;
};

std::vector<HostLev> mg_host(turb_ctx *c)
{
    std::vector<HostLev> L(1);
    HostLev &l0 = L[0];
    l0.nx = c->d.nx; l0.ny = c->d.ny; l0.nz = c->d.nz;
    const std::vector<double> *mc[3] = {&c->mxc, &c->myc, &c->mzc}, *mf[3] = {&c->mxu, &c->myv, &c->mzw};
    double de[3] = {c->dEta, c->dXi, c->dPhi};
    int n0[3] = {l0.nx, l0.ny, l0.nz};
    for (int a = 0; a < 3; a++) {
        l0.D[a].resize(n0[a]);
        l0.F[a].resize(n0[a] + 1);
        for (int i = 0; i < n0[a]; i++) l0.D[a][i] = de[a] / (*mc[a])[i];
        for (int i = 0; i <= n0[a]; i++) l0.F[a][i] = de[a] / (*mf[a])[i];
    }
    l0.pin = l0.D[1][l0.ny - 1] * l0.D[2][l0.nz - 1] / l0.F[0][l0.nx];
    for (int lev = 0; lev < TURB_MG_MAXLEV - 1; lev++) {
        HostLev f = L[lev];
        int nn[3] = {f.nx, f.ny, f.nz};
        double h[3];
        for (int a = 0; a < 3; a++) {
            double s = 0.0;
            for (double v : f.D[a]) s += v;
            h[a] = s / nn[a];
        }
        double hmin = std::min(h[0], std::min(h[1], h[2]));
        long long ncell = (long long)f.nx * f.ny * f.nz;
        int cc[3];
        for (int a = 0; a < 3; a++) cc[a] = (nn[a] % 2 == 0) && nn[a] >= 2 && h[a] <= 2.0 * hmin;
        if (ncell <= 64 || !(cc[0] || cc[1] || cc[2])) break;
        L[lev].cx = cc[0]; L[lev].cy = cc[1]; L[lev].cz = cc[2];
        HostLev g;
        int gn[3];
        for (int a = 0; a < 3; a++) {
            gn[a] = cc[a] ? nn[a] / 2 : nn[a];
            g.D[a].resize(gn[a]);
            g.F[a].resize(gn[a] + 1);
            for (int i = 0; i < gn[a]; i++) g.D[a][i] = cc[a] ? f.D[a][2 * i] + f.D[a][2 * i + 1] : f.D[a][i];
            if (cc[a]) {
                g.F[a][0] = 0.5 * g.D[a][0];
                for (int i = 1; i < gn[a]; i++) g.F[a][i] = 0.5 * (g.D[a][i - 1] + g.D[a][i]);
                g.F[a][gn[a]] = 0.5 * g.D[a][gn[a] - 1];
            } else {
                g.F[a] = f.F[a];
            }
        }
        g.nx = gn[0]; g.ny = gn[1]; g.nz = gn[2];
        g.pin = f.pin;
        L.push_back(g);
    }
    return L;
}

// linear prolongation along one direction between cell centres (positions
// accumulated from the widths) and its transpose
Xfer1D mk_xfer(DevBuf &m, const std::vector<double> &Df, const std::vector<double> &Dc, int coarsened)
{
    int nf = (int)Df.size(), nc = (int)Dc.size();
    std::vector<double> xf(nf), xc(nc);
    xf[0] = 0.5 * Df[0];
    for (int i = 1; i < nf; i++) xf[i] = xf[i - 1] + 0.5 * (Df[i - 1] + Df[i]);
    xc[0] = 0.5 * Dc[0];
    for (int i = 1; i < nc; i++) xc[i] = xc[i - 1] + 0.5 * (Dc[i - 1] + Dc[i]);
    std::vector<int> I0(nf), I1(nf), rcnt(nc, 0), rf(4 * (size_t)nc, 0);
    std::vector<double> w0(nf), w1(nf), rw(4 * (size_t)nc, 0.0);
    for (int i = 0; i < nf; i++) {
        if (!coarsened) { I0[i] = I1[i] = i; w0[i] = 1.0; w1[i] = 0.0; continue; }
        int I = i / 2, a, b;
        if (xf[i] < xc[I]) {
            if (I == 0) { I0[i] = I1[i] = 0; w0[i] = 1.0; w1[i] = 0.0; continue; }
            a = I - 1; b = I;
        } else {
            if (I == nc - 1) { I0[i] = I1[i] = I; w0[i] = 1.0; w1[i] = 0.0; continue; }
            a = I; b = I + 1;
        }
        I0[i] = a; I1[i] = b;
        w1[i] = (xf[i] - xc[a]) / (xc[b] - xc[a]);
        w0[i] = 1.0 - w1[i];
    }
    for (int i = 0; i < nf; i++) {
        int Is[2] = {I0[i], I1[i]};
        double ws[2] = {w0[i], w1[i]};
        for (int t = 0; t < 2; t++) {
            if (ws[t] == 0.0 || (t == 1 && Is[1] == Is[0])) continue;
            int C = Is[t], q = rcnt[C];
            if (q < 4) { rf[4 * (size_t)C + q] = i; rw[4 * (size_t)C + q] = ws[t]; rcnt[C] = q + 1; }
        }
    }
    std::vector<float> w0f(w0.begin(), w0.end()), w1f(w1.begin(), w1.end()), rwf(rw.begin(), rw.end());
    Xfer1D t;
    t.I0 = m.upload(I0); t.I1 = m.upload(I1);
    t.w0d = m.upload(w0); t.w1d = m.upload(w1); t.w0f = m.upload(w0f); t.w1f = m.upload(w1f);
    t.rcnt = m.upload(rcnt); t.rf = m.upload(rf); t.rwd = m.upload(rw); t.rwf = m.upload(rwf);
    return t;
}


// With TURB_KV_CLUSTER_VCYCLE, the first level of at most mg_cluster_cells
// cells (and at most MG_CLUSTER_MAXLEV levels from it to the coarsest) runs
// the rest of the V-cycle as one launch of one thread-block cluster, if the
// device can hold such a cluster.
static void set_cluster_from(turb_ctx *c)
{
    int from = -1;
    if ((c->kvariant & TURB_KV_CLUSTER_VCYCLE) && c->H32.cluster_ctas > 0 && c->H64.cluster_ctas > 0)
        for (int l = 0; l + 1 < c->H32.nl && c->mg_cluster_cells > 0; l++) {
            const MgDevLevel &m = c->H32.lev[l];
            if ((long long)m.nx * m.ny * m.nz <= c->mg_cluster_cells && c->H32.nl - l <= MG_CLUSTER_MAXLEV) {
                from = l;
                break;
            }
        }
    c->H32.cluster_from = c->H64.cluster_from = from;
}

// With TURB_KV_SWEEP_PAIRS, the finest FP32 level smooths two sweeps per
// pass (k_rbgs_tb) where its shape allows (colour-split, nx a multiple of 64,
// ny of 32); the second x array is allocated on first use.
static void set_tb(turb_ctx *c)
{
    c->H32.tb = nullptr;
    if (!(c->kvariant & TURB_KV_SWEEP_PAIRS) || c->H32.nl < 2) return;
    const MgDevLevel &L0 = c->H32.lev[0];
    if (!L0.split || L0.nx % 64 != 0 || L0.ny % 32 != 0) return;
    if (!c->tb_x1) {
        c->tb_x1 = c->mem.alloc<float>((size_t)L0.nx * L0.ny * L0.nz);
        c->tb_err = c->mem.alloc<int>(1);
        if (c->mem.err != cudaSuccess) {
            c->mem.err = cudaSuccess;
            cudaGetLastError();
            return;
        }
    }
    if (!c->tbplan.ok && mg_tb_plan(&c->tbplan, L0, c->H32.x[0], c->tb_x1, c->H32.b[0], c->H32.invd[0], c->tb_err))
        return;
    c->tbplan.lev = L0;
    c->H32.tb = &c->tbplan;
}
int build_mg(turb_ctx *c)
{
    std::vector<HostLev> L = mg_host(c);
    int nl = (int)L.size();
    c->H64.nl = c->H32.nl = nl;
    for (int l = 0; l < nl; l++) {
        HostLev &h = L[l];
        MgDevLevel m;
        m.nx = h.nx; m.ny = h.ny; m.nz = h.nz;
        m.cx = h.cx; m.cy = h.cy; m.cz = h.cz;
        m.pin = h.pin;
        if (l + 1 < nl) {
            m.tx = mk_xfer(c->mem, h.D[0], L[l + 1].D[0], h.cx);
            m.ty = mk_xfer(c->mem, h.D[1], L[l + 1].D[1], h.cy);
            m.tz = mk_xfer(c->mem, h.D[2], L[l + 1].D[2], h.cz);
        }
        std::vector<double> rf[3];
        std::vector<float> Df[3], rff[3];
        for (int a = 0; a < 3; a++) {
            rf[a].resize(h.F[a].size());
            rff[a].resize(h.F[a].size());
            for (size_t i = 0; i < h.F[a].size(); i++) { rf[a][i] = 1.0 / h.F[a][i]; rff[a][i] = (float)rf[a][i]; }
            Df[a].resize(h.D[a].size());
            for (size_t i = 0; i < h.D[a].size(); i++) Df[a][i] = (float)h.D[a][i];
        }
        m.dxd = c->mem.upload(h.D[0]); m.dyd = c->mem.upload(h.D[1]); m.dzd = c->mem.upload(h.D[2]);
        m.rfxd = c->mem.upload(rf[0]); m.rfyd = c->mem.upload(rf[1]); m.rfzd = c->mem.upload(rf[2]);
        m.dxf = c->mem.upload(Df[0]); m.dyf = c->mem.upload(Df[1]); m.dzf = c->mem.upload(Df[2]);
        m.rfxf = c->mem.upload(rff[0]); m.rfyf = c->mem.upload(rff[1]); m.rfzf = c->mem.upload(rff[2]);
        if (h.nx % 2 == 0) {   // parity-split copies of the x tables (k_rbgs4)
            const int hx = h.nx / 2;
            std::vector<float> dxp(h.nx), rlp(h.nx), rrp(h.nx);
            for (int par = 0; par < 2; par++)
                for (int q = 0; q < hx; q++) {
                    const int i = 2 * q + par;
                    dxp[par * hx + q] = Df[0][i];
                    rlp[par * hx + q] = rff[0][i];
                    rrp[par * hx + q] = i + 1 < (int)rff[0].size() ? rff[0][i + 1] : 0.0f;
                }
            m.dxpf = c->mem.upload(dxp); m.rlpf = c->mem.upload(rlp); m.rrpf = c->mem.upload(rrp);
        }
        c->H64.lev[l] = m;
        // FP32 levels store x, b, invd colour-split where nx is even (not on
        // the coarsest level, which the dense inverse reads in natural order)
        m.split = c->mg_split && (h.nx % 2 == 0) && l + 1 < nl;
        c->H32.lev[l] = m;
        long long n = (long long)h.nx * h.ny * h.nz;
        if (l > 0) {
            c->H64.x[l] = c->mem.alloc<double>(n);
            c->H64.b[l] = c->mem.alloc<double>(n);
        }
        c->H64.r[l] = c->mem.alloc<double>(n);
        c->H64.invd[l] = c->mem.alloc<double>(n);
        c->H32.x[l] = c->mem.alloc<float>(n);
        c->H32.b[l] = c->mem.alloc<float>(n);
        c->H32.r[l] = c->mem.alloc<float>(n);
        c->H32.invd[l] = c->mem.alloc<float>(n);
        if (c->mem.err != cudaSuccess) return TURB_ERR_ALLOC;
        mg_setup_invdiag<double>(c->s, c->H64.lev[l], c->H64.invd[l]);
        mg_setup_invdiag<float>(c->s, c->H32.lev[l], c->H32.invd[l]);
    }
    // dense inverse of the coarsest operator (Gauss-Jordan, partial pivoting)
    HostLev &h = L[nl - 1];
    int n = h.nx * h.ny * h.nz;
    if (n > 256) return TURB_ERR_ARG;
    std::vector<double> A((size_t)n * n, 0.0), I((size_t)n * n, 0.0);
    auto id = [&](int i, int j, int k) { return (k * h.ny + j) * h.nx + i; };
    for (int k = 0; k < h.nz; k++)
        for (int j = 0; j < h.ny; j++)
            for (int i = 0; i < h.nx; i++) {
                int r = id(i, j, k);
                double dyz = h.D[1][j] * h.D[2][k], dxz = h.D[0][i] * h.D[2][k], dxy = h.D[0][i] * h.D[1][j];
                double d = 0.0, f;
                if (i > 0) { f = dyz / h.F[0][i]; d += f; A[(size_t)r * n + id(i - 1, j, k)] = -f; }
                if (i < h.nx - 1) { f = dyz / h.F[0][i + 1]; d += f; A[(size_t)r * n + id(i + 1, j, k)] = -f; }
                if (j > 0) { f = dxz / h.F[1][j]; d += f; A[(size_t)r * n + id(i, j - 1, k)] = -f; }
                if (j < h.ny - 1) { f = dxz / h.F[1][j + 1]; d += f; A[(size_t)r * n + id(i, j + 1, k)] = -f; }
                if (k > 0) { f = dxy / h.F[2][k]; d += f; A[(size_t)r * n + id(i, j, k - 1)] = -f; }
                if (k < h.nz - 1) { f = dxy / h.F[2][k + 1]; d += f; A[(size_t)r * n + id(i, j, k + 1)] = -f; }
                if (i == h.nx - 1 && j == h.ny - 1 && k == h.nz - 1) d += h.pin;
                A[(size_t)r * n + r] = d;
            }
    for (int i = 0; i < n; i++) I[(size_t)i * n + i] = 1.0;
    for (int col = 0; col < n; col++) {
        int piv = col;
        for (int r = col + 1; r < n; r++)
            if (std::fabs(A[(size_t)r * n + col]) > std::fabs(A[(size_t)piv * n + col])) piv = r;
        if (piv != col)
            for (int t = 0; t < n; t++) {
                std::swap(A[(size_t)piv * n + t], A[(size_t)col * n + t]);
                std::swap(I[(size_t)piv * n + t], I[(size_t)col * n + t]);
            }
        double dv = A[(size_t)col * n + col];
        for (int t = 0; t < n; t++) { A[(size_t)col * n + t] /= dv; I[(size_t)col * n + t] /= dv; }
        for (int r = 0; r < n; r++) {
            if (r == col) continue;
            double f = A[(size_t)r * n + col];
            if (f == 0.0) continue;
            for (int t = 0; t < n; t++) {
                A[(size_t)r * n + t] -= f * A[(size_t)col * n + t];
                I[(size_t)r * n + t] -= f * I[(size_t)col * n + t];
            }
        }
    }
    c->H64.coarse_inv = c->H32.coarse_inv = c->mem.upload(I);
    long long n0 = (long long)c->d.nx * c->d.ny * c->d.nz;
    c->px = c->mem.alloc<double>(n0);
    c->pbw = c->mem.alloc<double>(n0);
    c->pr = c->mem.alloc<double>(n0);
    c->pz = c->mem.alloc<double>(n0);
    c->pp = c->mem.alloc<double>(n0);
    c->pq = c->mem.alloc<double>(n0);
    c->pro = c->mem.alloc<double>(n0);
    c->H64.x[0] = c->pz;   // FP64 V-cycle writes z directly
    c->H64.b[0] = c->pr;   // and reads r directly
    c->sc = c->mem.alloc<PcgScal>(1);
    // levels of at most 4096 cells finish the V-cycle in one block
    // (turb_set_mg_tail; at 512x256x256 larger tails ran slower than a
    // launch per half sweep, one SM having too little memory parallelism)
    c->H64.tail_from = c->H32.tail_from = -1;
    for (int l = 0; l + 1 < nl; l++) {
        const MgDevLevel &m = c->H32.lev[l];
        if ((long long)m.nx * m.ny * m.nz <= 4096 && nl - l <= MG_TAIL_MAXLEV) {
            c->H64.tail_from = c->H32.tail_from = l;
            break;
        }
    }
    c->H64.cluster_ctas = mg_cluster_ctas<double>();
    c->H32.cluster_ctas = mg_cluster_ctas<float>();
    set_cluster_from(c);
    set_tb(c);
    return c->mem.err == cudaSuccess ? TURB_OK : TURB_ERR_ALLOC;
}

int qidx(char which)
{
    switch (which) {
    case 'u': return 0;
    case 'v': return 1;
    case 'w': return 2;
    case 'c': return 3;
    default: return -1;
    }
}

int check_launch(turb_ctx *c)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    (void)c;
    return TURB_OK;
}

int fetch_scalars(turb_ctx *c, int n)
{
    TURB_CHECK(cudaMemcpyAsync(c->hscal, c->dscal, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

cudaEvent_t prof_event(turb_ctx *c)
{
    if (!c->pool.empty()) {
        cudaEvent_t e = c->pool.back();
        c->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// open a timed group on the context stream; returns a handle for prof_end
int prof_begin(turb_ctx *c, int g)
{
    if (!c->prof) return -1;
    turb_ctx::Rec r;
    r.g = g;
    r.nl = 0;
    r.bytes = 0.0;
    r.a = prof_event(c);
    r.b = prof_event(c);
    cudaEventRecord(r.a, c->s);
    c->recs.push_back(r);
    return (int)c->recs.size() - 1;
}

// bytes: the algorithmic bytes of the launches in the group (each array a
// kernel reads or writes counted once per launch)
void prof_end(turb_ctx *c, int h, int nlaunch, double bytes = 0.0)
{
    if (h < 0) return;
    cudaEventRecord(c->recs[h].b, c->s);
    c->recs[h].nl = nlaunch;
    c->recs[h].bytes = bytes;
}

void prof_collect(turb_ctx *c)
{
    cudaStreamSynchronize(c->s);
    for (auto &r : c->recs) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        c->prof_ms[r.g] += ms;
        c->prof_nl[r.g] += r.nl;
        c->prof_bytes[r.g] += r.bytes;
        c->pool.push_back(r.a);
        c->pool.push_back(r.b);
    }
    c->recs.clear();
}

template <typename F>
int capture(turb_ctx *c, cudaGraphExec_t *out, F body)
{
    cudaGraph_t g = nullptr;
    TURB_CHECK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    body();
    cudaError_t e = cudaStreamEndCapture(c->s, &g);
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    return TURB_OK;
}

void free_graphs(turb_ctx *c)
{
    for (auto &g : c->g_mg) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    for (auto &g : c->g_pcg) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    for (auto &g : c->g_inner) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *turb_status_string(int status)
{
    switch (status) {
    case TURB_OK: return "ok";
    case TURB_ERR_ARG: return "bad argument";
    case TURB_ERR_CUDA: return g_errmsg[0] ? g_errmsg : "CUDA error";
    case TURB_ERR_NOT_CONVERGED: return "solver did not converge";
    case TURB_ERR_NAN: return "non-finite residual";
    case TURB_ERR_ALLOC: return "device allocation failed";
    case TURB_ERR_SCRATCH_LIMIT: return "grid larger than the static scratch of the no-allocation entry point";
    case TURB_ERR_IO: return "restart file could not be opened, written or read";
    case TURB_ERR_FORMAT: return "restart file does not match the context";
    default: return "unknown status";
    }
}

int turb_create(const turb_grid_desc *g, const turb_params *p, turb_ctx **out)
{
    if (!g || !p || !out) return TURB_ERR_ARG;
    *out = nullptr;
    if (g->nx < 4 || g->ny < 4 || g->nz < 4 || p->nconc < 1 || p->nconc > TURB_MAXCONC || p->eno_order < 1 ||
        p->eno_order > 3 || g->nx != p->nx || g->ny != p->ny || g->nz != p->nz)
        return TURB_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        snprintf(g_errmsg, sizeof(g_errmsg), "no CUDA device");
        return TURB_ERR_CUDA;
    }
    turb_ctx *c = new turb_ctx();
    c->prm = *p;
    // V-cycle sweeps (turb_set_mg_sweeps / turb_set_mg_coarse_sweeps):
    // FP64 levels 4 + 4; FP32 levels 4 + 4 on the finest, 5 + 5 on the next,
    // 12 + 12 below, where a sweep costs little and the stretched,
    // anisotropic coarse problems need many (at 512x256x256: 6-7 CG
    // iterations instead of 8 with 6 + 6 everywhere, 9 % less step time)
    for (int l = 0; l < TURB_MG_MAXLEV; l++) {
        c->mg_pre[0][l] = c->mg_post[0][l] = 4;
        c->mg_pre[1][l] = c->mg_post[1][l] = l == 0 ? 4 : (l == 1 ? 5 : 12);
    }
    Dims &d = c->d;
    d.nx = g->nx; d.ny = g->ny; d.nz = g->nz;
    d.NX = d.nx + 1; d.NY = d.ny + 1; d.NZ = d.nz + 1;
    d.PX = (d.NX + 7) / 8 * 8;
    d.plane = (long long)d.PX * d.NY;
    d.n = d.plane * d.NZ;
    c->xc.assign(g->xc, g->xc + d.NX); c->yc.assign(g->yc, g->yc + d.NY); c->zc.assign(g->zc, g->zc + d.NZ);
    c->xu.assign(g->xu, g->xu + d.NX); c->yv.assign(g->yv, g->yv + d.NY); c->zw.assign(g->zw, g->zw + d.NZ);
    metrics(c);
    if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess) { delete c; return TURB_ERR_CUDA; }
    DevBuf &m = c->mem;
    c->geo.xc = m.upload(c->xc); c->geo.yc = m.upload(c->yc); c->geo.zc = m.upload(c->zc);
    c->geo.xu = m.upload(c->xu); c->geo.yv = m.upload(c->yv); c->geo.zw = m.upload(c->zw);
    c->geo.mxc = m.upload(c->mxc); c->geo.myc = m.upload(c->myc); c->geo.mzc = m.upload(c->mzc);
    c->geo.mxu = m.upload(c->mxu); c->geo.myv = m.upload(c->myv); c->geo.mzw = m.upload(c->mzw);
    // fields
    int ids[] = {TURB_F_U, TURB_F_V, TURB_F_W, TURB_F_PHI, TURB_F_DPX, TURB_F_DPY, TURB_F_DPZ, TURB_F_PB,
                 TURB_F_DIV, TURB_F_UBC, TURB_F_VBC, TURB_F_WBC, TURB_F_CONV_U, TURB_F_CONV_V, TURB_F_CONV_W,
                 TURB_F_B_U, TURB_F_B_V, TURB_F_B_W, TURB_F_CTOT, TURB_F_SCRATCH0, TURB_F_SCRATCH1};
    for (int id : ids) c->fld[id] = m.alloc<double>(d.n);
    for (int ic = 0; ic < p->nconc; ic++) {
        c->fld[TURB_F_C0 + ic] = m.alloc<double>(d.n);
        c->fld[TURB_F_CCONV0 + ic] = m.alloc<double>(d.n);
        c->fld[TURB_F_CB0 + ic] = m.alloc<double>(d.n);
        c->fld[TURB_F_VP0 + ic] = m.alloc<double>(d.n);
        c->old[3 + ic] = m.alloc<double>(d.n);
    }
    for (int q = 0; q < 3; q++) c->old[q] = m.alloc<double>(d.n);
    c->jtmp = m.alloc<double>(d.n);
    // status (DA layout in, pitched on the device)
    for (int q = 0; q < 4; q++) {
        std::vector<uint8_t> h((size_t)d.n, (uint8_t)T_BOUNDARY);
        for (int k = 0; k < d.NZ; k++)
            for (int j = 0; j < d.NY; j++)
                for (int i = 0; i < d.NX; i++) h[(size_t)d.at(i, j, k)] = g->status[q][((size_t)k * d.NY + j) * d.NX + i];
        c->st[q] = m.upload(h);
    }
    // tables
    int nx = d.nx, ny = d.ny, nz = d.nz;
    {
        std::vector<double> x0(d.NX), x1(d.NX), xq(d.NX);
        for (int i = 0; i < nx; i++) { x0[i] = c->xu[i]; x1[i] = c->xu[i + 1]; xq[i] = c->xc[i]; }
        c->icx = mk_interp2(m, d.NX, x0, x1, xq, 0);
        std::vector<double> y0(d.NY), y1(d.NY), yq(d.NY);
        for (int j = 0; j < ny; j++) { y0[j] = c->yv[j]; y1[j] = c->yv[j + 1]; yq[j] = c->yc[j]; }
        c->icy = mk_interp2(m, d.NY, y0, y1, yq, 0);
        std::vector<double> z0(d.NZ), z1(d.NZ), zq(d.NZ);
        for (int k = 0; k < nz; k++) { z0[k] = c->zw[k]; z1[k] = c->zw[k + 1]; zq[k] = c->zc[k]; }
        c->icz = mk_interp2(m, d.NZ, z0, z1, zq, 0);
        std::vector<double> v0(d.NY, 0.0), v1(d.NY, 1.0), vq(d.NY, 0.0);
        for (int j = 1; j < d.NY; j++) { v0[j] = c->yc[j - 1]; v1[j] = c->yc[j]; vq[j] = c->yv[j]; }
        c->iyv = mk_interp2(m, d.NY, v0, v1, vq, 1);
    }
    {
        std::vector<double> a0(d.NX + 1, 0.0), a1(d.NX + 1, 1.0), aq(d.NX + 1, 0.0);
        for (int i = 1; i <= nx - 1; i++) { a0[i] = c->xc[i - 1]; a1[i] = c->xc[i]; aq[i] = c->xu[i]; }
        c->tw.xu = mk_w2(m, d.NX, 1, nx - 1, a0, a1, aq);
        for (int i = 0; i <= nx - 1; i++) { a0[i] = c->xu[i]; a1[i] = c->xu[i + 1]; aq[i] = c->xc[i]; }
        c->tw.xc = mk_w2(m, d.NX, 0, nx - 1, a0, a1, aq);
        std::vector<double> b0(d.NY + 1, 0.0), b1(d.NY + 1, 1.0), bq(d.NY + 1, 0.0);
        for (int j = 0; j <= ny - 1; j++) { b0[j] = c->yv[j]; b1[j] = c->yv[j + 1]; bq[j] = c->yc[j]; }
        c->tw.yc = mk_w2(m, d.NY, 0, ny - 1, b0, b1, bq);
        for (int j = 1; j <= ny - 1; j++) { b0[j] = c->yc[j - 1]; b1[j] = c->yc[j]; bq[j] = c->yv[j]; }
        c->tw.yv = mk_w2(m, d.NY, 1, ny - 1, b0, b1, bq);
        std::vector<double> e0(d.NZ + 1, 0.0), e1(d.NZ + 1, 1.0), eq(d.NZ + 1, 0.0);
        for (int k = 0; k <= nz - 1; k++) { e0[k] = c->zw[k]; e1[k] = c->zw[k + 1]; eq[k] = c->zc[k]; }
        c->tw.zc = mk_w2(m, d.NZ, 0, nz - 1, e0, e1, eq);
        for (int k = 1; k <= nz - 1; k++) { e0[k] = c->zc[k - 1]; e1[k] = c->zc[k]; eq[k] = c->zw[k]; }
        c->tw.zw = mk_w2(m, d.NZ, 1, nz - 1, e0, e1, eq);
    }
    build_eno(c);
    for (int q = 0; q < 3; q++) c->helm[q] = mk_helm(c, q, 0);
    for (int ic = 0; ic < p->nconc; ic++) c->helm_c[ic] = mk_helm(c, 3, ic);
    for (int q = 0; q < 4; q++) {
        double aps = q < 3 ? c->helm[q].ap_solid : c->helm_c[0].ap_solid;
        turb_ib_desc e = g->ib[q];
        if (e.n < 0 || (e.n > 0 && (!e.im || !e.nf || !e.fidx || !e.fcoef))) { m.release(); delete c; return TURB_ERR_ARG; }
        c->ib[q] = mk_ib(c, q, e, aps);
        c->ibf[q] = mk_ibf(c, c->ib[q]);
    }
    for (int q = 0; q < 3; q++) c->helmf[q] = mk_helmf(c, c->helm[q]);
    for (int ic = 0; ic < p->nconc; ic++) c->helmf_c[ic] = mk_helmf(c, c->helm_c[ic]);
    c->hrf = m.alloc<float>(d.n);
    c->he0 = m.alloc<float>(d.n);
    c->he1 = m.alloc<float>(d.n);
    {
        double a_dEta = 1.0 / c->dEta, a_dXi = 1.0 / c->dXi, a_dPhi = 1.0 / c->dPhi;
        std::vector<double> cx(d.NX), cy(d.NY), cz(d.NZ), cyv(d.NY), czw(d.NZ);
        for (int i = 0; i < d.NX; i++) cx[i] = c->mxc[i] * a_dEta;
        for (int j = 0; j < d.NY; j++) { cy[j] = c->myc[j] * a_dXi; cyv[j] = a_dXi * c->myv[j]; }
        for (int k = 0; k < d.NZ; k++) { cz[k] = c->mzc[k] * a_dPhi; czw[k] = c->mzw[k] * a_dPhi; }
        c->pcx = m.upload(cx); c->pcy = m.upload(cy); c->pcz = m.upload(cz);
        c->proj.su = c->st[0]; c->proj.sv = c->st[1]; c->proj.sw = c->st[2];
        c->proj.mxu = c->geo.mxu; c->proj.cyv = m.upload(cyv); c->proj.czw = m.upload(czw);
        c->proj.a_dEta = a_dEta;
    }
    c->nparts = std::max<long long>(std::max(helm_parts(d), divergence_parts(d)), (long long)pcg_nparts() * 2);
    c->nparts = std::max<long long>(c->nparts, (long long)((d.nx + 31) / 32) * ((d.ny + 7) / 8) * d.nz);
    c->part = m.alloc<double>(c->nparts + 4096);
    c->dscal = m.alloc<double>(16);
    if (m.err != cudaSuccess) { m.release(); cudaStreamDestroy(c->s); delete c; return TURB_ERR_ALLOC; }
    int rc = build_mg(c);
    if (rc != TURB_OK) { m.release(); cudaStreamDestroy(c->s); delete c; return rc; }
    if (cudaMallocHost(&c->hscal, 16 * sizeof(double)) != cudaSuccess) { m.release(); delete c; return TURB_ERR_ALLOC; }
    if (cudaStreamSynchronize(c->s) != cudaSuccess) { m.release(); delete c; return TURB_ERR_CUDA; }
    *out = c;
    return TURB_OK;
}

int turb_destroy(turb_ctx *c)
{
    if (!c) return TURB_ERR_ARG;
    cudaStreamSynchronize(c->s);
    prof_collect(c);
    free_graphs(c);
    for (cudaEvent_t e : c->pool) cudaEventDestroy(e);
    for (cudaEvent_t e : c->user_ev)
        if (e) cudaEventDestroy(e);
    c->mem.release();
    if (c->hscal) cudaFreeHost(c->hscal);
    if (c->rs_host) cudaFreeHost(c->rs_host);
    for (void *b : c->gib_buf)
        if (b) cudaFree(b);
    for (int t = 0; t < 2; t++) {
        if (c->xfer[t]) cudaFree(c->xfer[t]);
        if (c->ev_copied[t]) cudaEventDestroy(c->ev_copied[t]);
        if (c->ev_freed[t]) cudaEventDestroy(c->ev_freed[t]);
    }
    if (c->cs) cudaStreamDestroy(c->cs);
    if (c->ios) cudaStreamDestroy(c->ios);
    for (auto &e : c->io_ev)
        if (e) cudaEventDestroy(e);
    if (c->cs2) cudaStreamDestroy(c->cs2);
    cudaStreamDestroy(c->s);
    delete c;
    return TURB_OK;
}

static double *field_ptr(turb_ctx *c, int f)
{
    if (f < 0 || f >= 64) return nullptr;
    return c->fld[f];
}

void launch_da_pitch(cudaStream_t s, const Dims &d, const double *src, double *dst, int to_pitched);
void launch_da_pitch_lean(cudaStream_t s, const Dims &d, const double *src, double *dst, int to_pitched);

// transfer staging, made on first use
static int stage_setup(turb_ctx *c)
{
    if (c->xfer[0]) return TURB_OK;
    size_t b = sizeof(double) * (size_t)c->d.NX * c->d.NY * c->d.NZ;
    TURB_CHECK(cudaStreamCreateWithFlags(&c->cs, cudaStreamNonBlocking));
    TURB_CHECK(cudaStreamCreateWithFlags(&c->cs2, cudaStreamNonBlocking));
    for (int t = 0; t < 2; t++) {
        TURB_CHECK(cudaEventCreateWithFlags(&c->ev_copied[t], cudaEventDisableTiming));
        TURB_CHECK(cudaEventCreateWithFlags(&c->ev_freed[t], cudaEventDisableTiming));
        TURB_CHECK(cudaMalloc(&c->xfer[t], b));
    }
    return TURB_OK;
}

// Host <-> device for several fields.  A field moves as one contiguous copy
// on a copy stream into / out of one of two staging buffers, and the kernel
// on the context's stream converts between the contiguous and the pitched
// layout, so the copy of one field overlaps the conversion of the one before
// (for page-locked arrays the copies run on the copy engines at the host
// link's rate); or, for page-locked arrays, the layout kernel reads or
// writes the host array in place (its loads / stores cross the host link).
// TURB_HOST_COPY_KERNEL (default) takes the second way for page-locked
// arrays: on GB300 the copy engines' transfers issued after a long step ran
// at 190-210 GB/s in some runs and at a quarter of that in others, in either
// direction, while the kernel's loads and stores held a steady 170-200 GB/s.
// Returns when everything has landed.
// the device address of page-locked host memory (cudaMallocHost or
// registered), or null for pageable memory
static const void *host_device_ptr(const void *h)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int turb_fields_upload(turb_ctx *c, int n, const int *fields, const double *const *host)
{
    if (!c || n < 0 || (n > 0 && (!fields || !host))) return TURB_ERR_ARG;
    for (int t = 0; t < n; t++)
        if (!field_ptr(c, fields[t]) || !host[t]) return TURB_ERR_ARG;
    // page-locked arrays with TURB_HOST_COPY_KERNEL (default): the layout
    // kernel reads them over the host link
    bool direct = c->host_copy == TURB_HOST_COPY_KERNEL;
    for (int t = 0; t < n && direct; t++) direct = host_device_ptr(host[t]) != nullptr;
    if (direct) {
        for (int t = 0; t < n; t++)
            launch_da_pitch(c->s, c->d, (const double *)host_device_ptr(host[t]), field_ptr(c, fields[t]), 1);
        TURB_CHECK(cudaStreamSynchronize(c->s));
        return TURB_OK;
    }
    int rc = stage_setup(c);
    if (rc) return rc;
    const Dims &d = c->d;
    size_t b = sizeof(double) * (size_t)d.NX * d.NY * d.NZ;
    // the previous work on the context's stream may still read the fields
    TURB_CHECK(cudaEventRecord(c->ev_freed[0], c->s));
    TURB_CHECK(cudaEventRecord(c->ev_freed[1], c->s));
    for (int t = 0; t < n; t++) {
        int u = t & 1;
        cudaStream_t cp = u ? c->cs2 : c->cs;   // two copies in flight, on two copy engines
        TURB_CHECK(cudaStreamWaitEvent(cp, c->ev_freed[u], 0));
        TURB_CHECK(cudaMemcpyAsync(c->xfer[u], host[t], b, cudaMemcpyHostToDevice, cp));
        TURB_CHECK(cudaEventRecord(c->ev_copied[u], cp));
        TURB_CHECK(cudaStreamWaitEvent(c->s, c->ev_copied[u], 0));
        launch_da_pitch(c->s, d, c->xfer[u], field_ptr(c, fields[t]), 1);
        TURB_CHECK(cudaEventRecord(c->ev_freed[u], c->s));
    }
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

int turb_fields_download(turb_ctx *c, int n, const int *fields, double *const *host)
{
    if (!c || n < 0 || (n > 0 && (!fields || !host))) return TURB_ERR_ARG;
    for (int t = 0; t < n; t++)
        if (!field_ptr(c, fields[t]) || !host[t]) return TURB_ERR_ARG;
    // page-locked arrays with TURB_HOST_COPY_KERNEL (default): the layout
    // kernel writes them over the host link
    bool direct = c->host_copy == TURB_HOST_COPY_KERNEL;
    for (int t = 0; t < n && direct; t++) direct = host_device_ptr(host[t]) != nullptr;
    if (direct) {
        for (int t = 0; t < n; t++)
            launch_da_pitch(c->s, c->d, field_ptr(c, fields[t]), (double *)host_device_ptr(host[t]), 0);
        TURB_CHECK(cudaStreamSynchronize(c->s));
        return TURB_OK;
    }
    int rc = stage_setup(c);
    if (rc) return rc;
    const Dims &d = c->d;
    size_t b = sizeof(double) * (size_t)d.NX * d.NY * d.NZ;
    TURB_CHECK(cudaEventRecord(c->ev_freed[0], c->cs));
    TURB_CHECK(cudaEventRecord(c->ev_freed[1], c->cs2));
    for (int t = 0; t < n; t++) {
        int u = t & 1;
        TURB_CHECK(cudaStreamWaitEvent(c->s, c->ev_freed[u], 0));
        launch_da_pitch(c->s, d, field_ptr(c, fields[t]), c->xfer[u], 0);
        TURB_CHECK(cudaEventRecord(c->ev_copied[u], c->s));
        cudaStream_t cp = u ? c->cs2 : c->cs;
        TURB_CHECK(cudaStreamWaitEvent(cp, c->ev_copied[u], 0));
        TURB_CHECK(cudaMemcpyAsync(host[t], c->xfer[u], b, cudaMemcpyDeviceToHost, cp));
        TURB_CHECK(cudaEventRecord(c->ev_freed[u], cp));
    }
    TURB_CHECK(cudaStreamSynchronize(c->cs));
    TURB_CHECK(cudaStreamSynchronize(c->cs2));
    return TURB_OK;
}

int turb_set_host_copy(turb_ctx *c, int mode)
{
    if (!c || (mode != TURB_HOST_COPY_DMA && mode != TURB_HOST_COPY_KERNEL)) return TURB_ERR_ARG;
    c->host_copy = mode;
    return TURB_OK;
}

int turb_field_upload(turb_ctx *c, int field, const double *h)
{
    return turb_fields_upload(c, 1, &field, &h);
}

int turb_field_download(turb_ctx *c, int field, double *h)
{
    return turb_fields_download(c, 1, &field, &h);
}

int turb_set_pressure_guess(turb_ctx *c, int mode)
{
    if (!c || mode < TURB_GUESS_PREVIOUS || mode > TURB_GUESS_PROJECT) return TURB_ERR_ARG;
    if (mode == TURB_GUESS_LEARNED && !c->net) return TURB_ERR_ARG;
    c->guess_mode = mode;
    return TURB_OK;
}

int turb_set_sweep_kernels(turb_ctx *c, int variants)
{
    const int all = TURB_KV_MARCHING | TURB_KV_ENO_SEGMENTS | TURB_KV_PDL | TURB_KV_CLUSTER_VCYCLE | TURB_KV_SWEEP_PAIRS;
    if (!c || variants < 0 || variants > all) return TURB_ERR_ARG;
    if ((c->kvariant ^ variants) & (all & ~TURB_KV_ENO_SEGMENTS)) {   // captured graphs hold the old launches
        for (auto &g : c->g_inner)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
        for (auto &g : c->g_mg)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    }
    c->kvariant = variants;
    c->H64.marching = (variants & TURB_KV_MARCHING) ? 1 : 0;
    c->H32.marching = c->H64.marching;
    c->H64.pdl = (variants & TURB_KV_PDL) ? 1 : 0;
    c->H32.pdl = c->H64.pdl;
    set_cluster_from(c);
    set_tb(c);
    return TURB_OK;
}

int turb_set_divergence_gate(turb_ctx *c, double max_div)
{
    if (!c || !(max_div >= 0.0)) return TURB_ERR_ARG;
    c->div_gate = max_div;
    return TURB_OK;
}

int turb_divergence_gate_count(turb_ctx *c, long long *tightened)
{
    if (!c || !tightened) return TURB_ERR_ARG;
    *tightened = c->gate_tightened;
    return TURB_OK;
}

int turb_reset_pressure_history(turb_ctx *c)
{
    if (!c) return TURB_ERR_ARG;
    c->nh[0] = c->nh[1] = 0;
    return TURB_OK;
}

int turb_divergence_gate_floor_count(turb_ctx *c, long long *at_floor)
{
    if (!c || !at_floor) return TURB_ERR_ARG;
    *at_floor = c->gate_floor;
    return TURB_OK;
}

int turb_set_guess_galerkin(turb_ctx *c, int on)
{
    if (!c || (on != 0 && on != 1)) return TURB_ERR_ARG;
    c->galerkin = on;
    return TURB_OK;
}

int turb_set_guess_stages(turb_ctx *c, int mask)
{
    if (!c || mask < 0 || mask > 3) return TURB_ERR_ARG;
    c->guess_stages = mask;
    return TURB_OK;
}

int turb_set_snapshot_store(turb_ctx *c, turb_snaps *snaps)
{
    if (!c) return TURB_ERR_ARG;
    TurbSnaps *sn = reinterpret_cast<TurbSnaps *>(snaps);
    if (sn) {
        int nx, ny, nz;
        snaps_dims(sn, &nx, &ny, &nz);
        const MgDevLevel &L0 = c->H64.lev[0];
        if (nx != L0.nx || ny != L0.ny || nz != L0.nz) return TURB_ERR_ARG;
    }
    c->snaps = sn;
    return TURB_OK;
}

int turb_set_learned_net(turb_ctx *c, turb_net *net)
{
    if (!c) return TURB_ERR_ARG;
    TurbNet *n = reinterpret_cast<TurbNet *>(net);
    if (n) {
        int nx, ny, nz;
        net_dims(n, &nx, &ny, &nz);
        const MgDevLevel &L0 = c->H64.lev[0];
        if (nx != L0.nx || ny != L0.ny || nz != L0.nz) return TURB_ERR_ARG;
    } else if (c->guess_mode == TURB_GUESS_LEARNED) {
        c->guess_mode = TURB_GUESS_PREVIOUS;
    }
    c->net = n;
    return TURB_OK;
}

int turb_net_train(turb_net *net, turb_ctx *c, turb_snaps *snaps, int steps, float lr, unsigned long long seed,
                   double *mean_loss)
{
    if (!c || !net || !snaps) return TURB_ERR_ARG;
    return net_train(reinterpret_cast<TurbNet *>(net), c->s, c->H64.lev[0], c->H64.invd[0],
                     reinterpret_cast<TurbSnaps *>(snaps), steps, lr, seed, mean_loss);
}

int turb_net_eval(turb_net *net, turb_ctx *c, turb_snaps *snaps, int first, int count, double *mean_residual,
                  double *mean_energy)
{
    if (!c || !net || !snaps) return TURB_ERR_ARG;
    return net_eval(reinterpret_cast<TurbNet *>(net), c->s, c->H64.lev[0], c->H64.invd[0],
                    reinterpret_cast<TurbSnaps *>(snaps), first, count, mean_residual, mean_energy);
}

int turb_pressure_guess_ratio(turb_ctx *c, double *geo_mean)
{
    if (!c || !geo_mean) return TURB_ERR_ARG;
    *geo_mean = c->guess_tried > 0 ? std::exp(c->guess_logsum / c->guess_tried) : 1.0;
    return TURB_OK;
}

int turb_pressure_guess_stats(turb_ctx *c, int *tried, int *taken)
{
    if (!c || !tried || !taken) return TURB_ERR_ARG;
    *tried = c->guess_tried;
    *taken = c->guess_taken;
    return TURB_OK;
}

int turb_set_pressure_mode(turb_ctx *c, int mode)
{
    if (!c || (mode != TURB_PMODE_FP64 && mode != TURB_PMODE_MIXED)) return TURB_ERR_ARG;
    c->pmode = mode;
    return TURB_OK;
}

// sweeps of levels [from, TURB_MG_MAXLEV) of the current pressure mode; a change
// drops the captured V-cycle
static int set_sweeps(turb_ctx *c, int from, int npre, int npost)
{
    if (!c || from < 0 || npre < 1 || npost < 1 || npre > 16 || npost > 16) return TURB_ERR_ARG;
    int m = c->pmode == TURB_PMODE_FP64 ? 0 : 1;
    bool changed = false;
    for (int l = from; l < TURB_MG_MAXLEV; l++) {
        changed |= c->mg_pre[m][l] != npre || c->mg_post[m][l] != npost;
        c->mg_pre[m][l] = npre;
        c->mg_post[m][l] = npost;
    }
    if (changed && c->g_mg[m]) { cudaGraphExecDestroy(c->g_mg[m]); c->g_mg[m] = nullptr; }
    return TURB_OK;
}

int turb_set_mg_sweeps(turb_ctx *c, int npre, int npost) { return set_sweeps(c, 0, npre, npost); }

int turb_set_mg_coarse_sweeps(turb_ctx *c, int from_level, int npre, int npost)
{
    if (from_level < 1) return TURB_ERR_ARG;
    return set_sweeps(c, from_level, npre, npost);
}

// ---- open boundaries ------------------------------------------------------
int turb_set_open_boundaries(turb_ctx *c, int inflow, int outflow, double U, int transient_inflow, double time_c)
{
    if (!c || !(time_c > 0.0)) return TURB_ERR_ARG;
    const Dims &d = c->d;
    int np = d.NY * d.NZ, nc = c->prm.nconc;
    if (!c->open_scr) {
        c->pl_in_u = c->mem.alloc<double>(np);
        for (int q = 0; q < 3 + TURB_MAXCONC; q++) {
            c->pl_out[q] = c->mem.alloc<double>(np);
            c->pl_out_old[q] = c->mem.alloc<double>(np);
        }
        for (int ic = 0; ic < TURB_MAXCONC; ic++) c->pl_in_c[ic] = c->mem.alloc<double>(np);
        c->open_scr = c->mem.alloc<double>(open_parts(d) + 8);
        if (c->mem.err != cudaSuccess) return TURB_ERR_ALLOC;
    }
    c->open_U = U;
    c->open_transient = transient_inflow ? 1 : 0;
    c->open_time_c = time_c;
    OpenBC &o = c->ob;
    o = OpenBC();
    o.in = inflow ? 1 : 0;
    o.out = outflow ? 1 : 0;
    o.NY = d.NY;
    o.u_in = c->pl_in_u;
    for (int ic = 0; ic < TURB_MAXCONC; ic++) o.c_in[ic] = c->pl_in_c[ic];
    for (int q = 0; q < 3 + TURB_MAXCONC; q++) o.out_f[q] = c->pl_out[q];
    // RHS coefficients of the rows next to the open faces, in the reference's
    // expression order: u Velocity.c:1691-1717, v / w Velocity.c:1885-1893 and
    // 2011-2019, c Conc.c:938-960
    int nx = d.nx;
    double Cx = -1.0 / (c->prm.re * c->dEta * c->dEta);
    o.u_aw = -Cx * c->mxu[1] * c->mxc[0];
    o.u_ae = -Cx * c->mxu[nx - 1] * c->mxc[nx - 1];
    o.vw_ae[0] = o.vw_ae[1] = -Cx * c->mxc[nx - 1] * c->mxu[nx];
    for (int ic = 0; ic < nc; ic++) {
        double Cc = -1.0 / (c->prm.pe[ic] * c->dEta * c->dEta);
        o.c_aw[ic] = -Cc * c->mxc[0] * c->mxu[0];
        o.c_ae[ic] = -Cc * c->mxc[nx - 1] * c->mxu[nx - 1];
    }
    // operators and ENO x tables follow the faces
    for (int q = 0; q < 3; q++) c->helm[q] = mk_helm(c, q, 0);
    for (int ic = 0; ic < nc; ic++) c->helm_c[ic] = mk_helm(c, 3, ic);
    for (int q = 0; q < 3; q++) c->helmf[q] = mk_helmf(c, c->helm[q]);
    for (int ic = 0; ic < nc; ic++) c->helmf_c[ic] = mk_helmf(c, c->helm_c[ic]);
    build_eno(c);
    int r = c->prm.eno_order;
    auto open_lo = [&](EnoTab &T, const double *pl) {
        for (int ex = 0; ex < r; ex++) T.gsrc[ex] = 3;
        T.glo = pl;
        T.gNY = d.NY;
    };
    auto open_hi = [&](EnoTab &T, const double *pl) {
        for (int ex = 0; ex < r; ex++) T.gsrc[3 + ex] = 4;
        T.ghi = pl;
        T.gNY = d.NY;
    };
    // ghosts of x lines at the open faces (Velocity.c:2194-2235, 2442-2449,
    // 2669-2676; Conc.c:1099-1124)
    if (o.in) open_lo(c->eno[0][0], c->pl_in_u);
    if (o.out) {
        open_hi(c->eno[0][0], c->pl_out[0]);
        open_hi(c->eno[1][0], c->pl_out[1]);
        open_hi(c->eno[2][0], c->pl_out[2]);
    }
    for (int ic = 0; ic < nc; ic++) {
        c->eno_cx[ic] = c->eno[3][0];
        if (o.in) open_lo(c->eno_cx[ic], c->pl_in_c[ic]);
        if (o.out) open_hi(c->eno_cx[ic], c->pl_out[3 + ic]);
    }
    free_graphs(c);
    return check_launch(c);
}

static double *open_plane(turb_ctx *c, int which, int q, int ic)
{
    if (q < 0 || q > 3 || (q == 3 && (ic < 0 || ic >= c->prm.nconc))) return nullptr;
    int f = q < 3 ? q : 3 + ic;
    if (which == 0) return q == 0 ? c->pl_in_u : q == 3 ? c->pl_in_c[ic] : nullptr;
    if (which == 1) return c->pl_out[f];
    if (which == 2) return c->pl_out_old[f];
    return nullptr;
}

int turb_open_plane_get(turb_ctx *c, int which, int q, int ic, double *host)
{
    if (!c || !host || !c->open_scr) return TURB_ERR_ARG;
    double *p = open_plane(c, which, q, ic);
    if (!p) return TURB_ERR_ARG;
    TURB_CHECK(cudaMemcpyAsync(host, p, sizeof(double) * c->d.NY * c->d.NZ, cudaMemcpyDeviceToHost, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

int turb_open_plane_set(turb_ctx *c, int which, int q, int ic, const double *host)
{
    if (!c || !host || !c->open_scr) return TURB_ERR_ARG;
    double *p = open_plane(c, which, q, ic);
    if (!p) return TURB_ERR_ARG;
    TURB_CHECK(cudaMemcpyAsync(p, host, sizeof(double) * c->d.NY * c->d.NZ, cudaMemcpyHostToDevice, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

static double open_time_factor(const turb_ctx *c, double time)
{
    return c->open_transient ? (1.0 - std::exp(-(time + 0.01) / c->open_time_c)) : 1.0;
}

int turb_Inflow_u_velocity_profile(turb_ctx *c, double time, double *influx)
{
    if (!c || !c->ob.in) return TURB_ERR_ARG;
    double *inf = c->open_scr + open_parts(c->d);
    launch_inflow_u(c->s, c->d, c->st[0], c->geo.yv, c->geo.zw, open_time_factor(c, time), c->pl_in_u,
                    c->open_scr, inf);
    c->launches += 2;
    if (influx) {
        TURB_CHECK(cudaMemcpyAsync(influx, inf, sizeof(double), cudaMemcpyDeviceToHost, c->s));
        TURB_CHECK(cudaStreamSynchronize(c->s));
    }
    return check_launch(c);
}

int turb_set_time(turb_ctx *c, double time)
{
    if (!c) return TURB_ERR_ARG;
    c->time = time;
    return TURB_OK;
}

int turb_get_time(turb_ctx *c, double *time)
{
    if (!c || !time) return TURB_ERR_ARG;
    *time = c->time;
    return TURB_OK;
}

int turb_set_influx(turb_ctx *c, double influx)
{
    if (!c || !c->open_scr) return TURB_ERR_ARG;
    TURB_CHECK(cudaMemcpyAsync(c->open_scr + open_parts(c->d), &influx, sizeof(double), cudaMemcpyHostToDevice, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

int turb_Inflow_conc_profile(turb_ctx *c, int ic, double time)
{
    if (!c || !c->ob.in || ic < 0 || ic >= c->prm.nconc) return TURB_ERR_ARG;
    launch_inflow_c(c->s, c->d, c->st[3], open_time_factor(c, time), c->pl_in_c[ic]);
    c->launches += 1;
    return check_launch(c);
}

static double open_coef(const turb_ctx *c, double dt)
{
    int NI = c->d.nx;
    double dx = c->xu[NI] - c->xu[NI - 1];
    return dt * c->open_U / dx;
}

int turb_Outflow_vel_impose_convective_boundary(turb_ctx *c, char which, double dt)
{
    int q = qidx(which);
    if (!c || !c->ob.out || q < 0 || q > 2 || !(dt > 0.0)) return TURB_ERR_ARG;
    launch_outflow_conv(c->s, c->d, c->st[q], open_coef(c, dt), c->fld[TURB_F_U + q], c->pl_out[q]);
    c->launches += 1;
    if (q == 0) {
        double *inf = c->open_scr + open_parts(c->d);
        launch_outflow_mass(c->s, c->d, c->st[0], c->geo.yv, c->geo.zw, inf, c->pl_out[0], c->open_scr, inf + 1);
        c->launches += 3;
    }
    return check_launch(c);
}

int turb_Outflow_conc_impose_convective_boundary(turb_ctx *c, int ic, double dt)
{
    if (!c || !c->ob.out || ic < 0 || ic >= c->prm.nconc || !(dt > 0.0)) return TURB_ERR_ARG;
    launch_outflow_conv(c->s, c->d, c->st[3], open_coef(c, dt), c->fld[TURB_F_C0 + ic], c->pl_out[3 + ic]);
    c->launches += 1;
    return check_launch(c);
}

int turb_Outflow_impose_convective_boundary(turb_ctx *c, double dt)
{
    int rc;
    for (char q : {'u', 'v', 'w'})
        if ((rc = turb_Outflow_vel_impose_convective_boundary(c, q, dt))) return rc;
    for (int ic = 0; ic < c->prm.nconc; ic++)
        if ((rc = turb_Outflow_conc_impose_convective_boundary(c, ic, dt))) return rc;
    return TURB_OK;
}

int turb_store_old_outflow(turb_ctx *c)
{
    if (!c || !c->ob.out) return TURB_ERR_ARG;
    size_t b = sizeof(double) * c->d.NY * c->d.NZ;
    for (int q = 0; q < 3 + c->prm.nconc; q++)
        TURB_CHECK(cudaMemcpyAsync(c->pl_out_old[q], c->pl_out[q], b, cudaMemcpyDeviceToDevice, c->s));
    return TURB_OK;
}

int turb_rk_average_outflow(turb_ctx *c, double old_frac, double new_frac)
{
    if (!c || !c->ob.out) return TURB_ERR_ARG;
    for (int q = 0; q < 3 + c->prm.nconc; q++)
        launch_plane_axpby(c->s, c->d.NY * c->d.NZ, old_frac, c->pl_out_old[q], new_frac, c->pl_out[q]);
    c->launches += 3 + c->prm.nconc;
    return check_launch(c);
}

static int open_field(turb_ctx *c, char which, int ic)
{
    int q = which == 'c' ? 3 : qidx(which);
    if (q < 0 || q > 3 || (q == 3 && (ic < 0 || ic >= c->prm.nconc))) return -1;
    return q < 3 ? q : 3 + ic;
}

int turb_Outflow_copy_data_into_last_plane(turb_ctx *c, char which, int ic, int should_set)
{
    if (!c || !c->open_scr) return TURB_ERR_ARG;
    int f = open_field(c, which, ic);
    if (f < 0) return TURB_ERR_ARG;
    double *q = f < 3 ? c->fld[TURB_F_U + f] : c->fld[TURB_F_C0 + f - 3];
    launch_plane_to_field(c->s, c->d, c->pl_out[f], should_set, q);
    c->launches += 1;
    return check_launch(c);
}

int turb_Outflow_copy_data_into_2D_array(turb_ctx *c, char which, int ic)
{
    if (!c || !c->open_scr) return TURB_ERR_ARG;
    int f = open_field(c, which, ic);
    if (f < 0) return TURB_ERR_ARG;
    const double *q = f < 3 ? c->fld[TURB_F_U + f] : c->fld[TURB_F_C0 + f - 3];
    launch_field_to_plane(c->s, c->d, q, c->pl_out[f]);
    c->launches += 1;
    return check_launch(c);
}

// the first level with at most max_cells cells (and at most MG_TAIL_MAXLEV
// levels from it to the coarsest) runs the rest of the V-cycle in one block
static void set_tail(turb_ctx *c, long long max_cells)
{
    int from = -1;
    for (int l = 0; l + 1 < c->H32.nl && max_cells > 0; l++) {
        const MgDevLevel &m = c->H32.lev[l];
        if ((long long)m.nx * m.ny * m.nz <= max_cells && c->H32.nl - l <= MG_TAIL_MAXLEV) { from = l; break; }
    }
    c->H32.tail_from = c->H64.tail_from = from;
    for (int m = 0; m < 2; m++)
        if (c->g_mg[m]) { cudaGraphExecDestroy(c->g_mg[m]); c->g_mg[m] = nullptr; }
}

int turb_set_mg_cluster(turb_ctx *c, long long max_cells)
{
    if (!c || max_cells < 0) return TURB_ERR_ARG;
    c->mg_cluster_cells = max_cells;
    set_cluster_from(c);
    for (int m = 0; m < 2; m++)
        if (c->g_mg[m]) { cudaGraphExecDestroy(c->g_mg[m]); c->g_mg[m] = nullptr; }
    return TURB_OK;
}

int turb_set_mg_tail(turb_ctx *c, long long max_cells)
{
    if (!c || max_cells < 0) return TURB_ERR_ARG;
    set_tail(c, max_cells);
    return TURB_OK;
}

int turb_set_mg_split(turb_ctx *c, int on)
{
    if (!c) return TURB_ERR_ARG;
    c->mg_split = on ? 1 : 0;
    for (int l = 0; l < c->H32.nl; l++) {
        MgDevLevel &m = c->H32.lev[l];
        m.split = c->mg_split && (m.nx % 2 == 0) && l + 1 < c->H32.nl;
        mg_setup_invdiag<float>(c->s, m, c->H32.invd[l]);
    }
    set_tb(c);
    if (c->g_mg[1]) { cudaGraphExecDestroy(c->g_mg[1]); c->g_mg[1] = nullptr; }
    return check_launch(c);
}

int turb_synchronize(turb_ctx *c)
{
    if (!c) return TURB_ERR_ARG;
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

int turb_ENO_compute_convective_terms(int order, int n, const double *D0, const double *P, const double *V,
                                      double *out)
{
    if (order < 1 || order > 3 || n < 2 * order + 2 || !D0 || !P || !V || !out) return TURB_ERR_ARG;
    double *buf = nullptr;
    TURB_CHECK(cudaMalloc(&buf, sizeof(double) * 4 * (size_t)n));
    cudaMemcpy(buf, D0, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(buf + n, P, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(buf + 2 * n, V, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(buf + 3 * n, out, sizeof(double) * n, cudaMemcpyHostToDevice);
    int rc = launch_eno_line(order, n, buf, buf + n, buf + 2 * n, buf + 3 * n, 0);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, buf + 3 * n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (rc) return TURB_ERR_ARG;
    if (e != cudaSuccess) return turb_set_cuda_error(e, __FILE__, __LINE__);
    return TURB_OK;
}

int turb_Velocity_cell_center(turb_ctx *c)
{
    if (!c) return TURB_ERR_ARG;
    launch_cell_center(c->s, c->d, c->icx, c->icy, c->icz, c->ob, c->fld[TURB_F_U], c->fld[TURB_F_V],
                       c->fld[TURB_F_W], c->fld[TURB_F_UBC], c->fld[TURB_F_VBC], c->fld[TURB_F_WBC]);
    c->launches += 1;
    return check_launch(c);
}

int turb_Velocity_transpose_velocities(turb_ctx *c, char which)
{
    int q = qidx(which);
    if (!c || q < 0 || q > 2) return TURB_ERR_ARG;
    launch_transpose(c->s, c->d, q, c->st[q], c->tw, c->ob, c->fld[TURB_F_U], c->fld[TURB_F_V], c->fld[TURB_F_W],
                     c->fld[TURB_F_SCRATCH0], c->fld[TURB_F_SCRATCH1]);
    c->launches += 1;
    return check_launch(c);
}

// Grid_compute_metric_coefficients' cell widths: f[i+1] - f[i], the last
// repeating its neighbour (Grid.c:633-637)
static std::vector<double> cell_widths(const std::vector<double> &f)
{
    size_t n = f.size();
    std::vector<double> d(n, 0.0);
    for (size_t i = 1; i + 1 < n; i++) d[i] = f[i + 1] - f[i];
    d[0] = f[1] - f[0];
    d[n - 1] = f[n - 1] - f[n - 2];
    return d;
}

// bed index and deposit buffer, made on first use
static int bed_setup(turb_ctx *c)
{
    if (c->bed_iy) return TURB_OK;
    const Dims &d = c->d;
    c->bed_iy = c->mem.alloc<int32_t>((long long)d.NZ * d.NX);
    c->dep = c->mem.alloc<double>((long long)TURB_MAXCONC * d.NZ * d.NX);
    if (c->mem.err != cudaSuccess) return TURB_ERR_ALLOC;
    TURB_CHECK(cudaMemsetAsync(c->dep, 0, sizeof(double) * TURB_MAXCONC * d.NZ * d.NX, c->s));
    launch_bed_index(c->s, d, c->st[3], c->bed_iy);
    c->launches++;
    return check_launch(c);
}

int turb_diagnostics(turb_ctx *c, double front_limit, turb_diag *out, double *ave_height, double *sed_bottom)
{
    if (!c || !out) return TURB_ERR_ARG;
    const Dims &d = c->d;
    int nc = c->prm.nconc;
    int rc = bed_setup(c);
    if (rc) return rc;
    if (!c->diag_scr) {
        c->diag_dxc = c->mem.upload(cell_widths(c->xu));
        c->diag_dyc = c->mem.upload(cell_widths(c->yv));
        c->diag_dzc = c->mem.upload(cell_widths(c->zw));
        c->diag_scr = c->mem.alloc<double>(diag_scratch_doubles(d));
        if (c->mem.err != cudaSuccess) return TURB_ERR_ALLOC;
    }
    // the reference's output routines read the cell-centre velocities and the
    // total concentration of the current state (Velocity_cell_center, Conc.c:1291)
    rc = turb_Velocity_cell_center(c);
    if (rc) return rc;
    const double *ct = c->fld[TURB_F_C0];
    if (nc > 1) {
        rc = turb_Conc_compute_total_concentration(c);
        if (rc) return rc;
        ct = c->fld[TURB_F_CTOT];
    }
    DiagIn a;
    memset(&a, 0, sizeof(a));
    a.d = d;
    a.geo = c->geo;
    a.cst = c->st[3];
    a.dxc = c->diag_dxc; a.dyc = c->diag_dyc; a.dzc = c->diag_dzc;
    a.u = c->fld[TURB_F_U]; a.v = c->fld[TURB_F_V]; a.w = c->fld[TURB_F_W];
    a.ubc = c->fld[TURB_F_UBC]; a.vbc = c->fld[TURB_F_VBC]; a.wbc = c->fld[TURB_F_WBC]; a.ct = ct;
    a.nconc = nc;
    for (int i = 0; i < nc; i++) {
        a.c[i] = c->fld[TURB_F_C0 + i];
        a.particle[i] = c->prm.ctype[i] == TURB_PARTICLE;
        a.us[i] = std::fabs(c->prm.vs0[i]);
    }
    a.y_ref = c->yv[0];
    double Ly = c->yv[d.NY - 1] - c->yv[0], Lz = c->zw[d.NZ - 1] - c->zw[0];
    a.hcoef = 1.0 / (Ly * Lz);
    a.Cx = 1.0 / (c->dEta * c->dEta); a.Cy = 1.0 / (c->dXi * c->dXi); a.Cz = 1.0 / (c->dPhi * c->dPhi);
    for (int q = 0; q < 6; q++) a.kw[q] = c->prm.wall_noslip[q] ? -1.0 : 1.0;
    a.ob = c->ob;
    a.iy = c->bed_iy;
    a.dep = c->dep;
    DiagOut o;
    launch_diagnostics(c->s, a, c->diag_scr, &o);
    c->launches += 6;
    std::vector<double> sh(DIAG_NQ), bs(2 * TURB_MAXCONC), hh((size_t)nc * d.NX);
    TURB_CHECK(cudaMemcpyAsync(sh.data(), o.sums, sh.size() * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    TURB_CHECK(cudaMemcpyAsync(bs.data(), o.bed_sums, bs.size() * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    TURB_CHECK(cudaMemcpyAsync(hh.data(), o.heights, hh.size() * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    if (sed_bottom)
        TURB_CHECK(cudaMemcpyAsync(sed_bottom, o.sed_bottom, sizeof(double) * nc * d.NZ * d.NX,
                                   cudaMemcpyDeviceToHost, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    memset(out, 0, sizeof(*out));
    out->kinetic_energy = sh[0] * 0.5;
    out->conversion_rate = sh[1];
    out->viscous_dissipation = sh[2] * (1.0 / c->prm.re);
    for (int i = 0; i < nc; i++) {
        double al = c->prm.alpha[i], us = std::fabs(c->prm.vs0[i]);
        out->suspended_mass[i] = sh[3 + 4 * i];
        out->potential_energy[i] = sh[4 + 4 * i] * al;
        out->stokes_dissipation[i] = sh[5 + 4 * i] * (us * al);
        out->conversion_rate_c[i] = sh[6 + 4 * i] * al;
        out->ep_passive[i] = bs[2 * i];
        out->ep_passive_rate[i] = bs[2 * i] * us;
        out->ep_rate[i] = out->conversion_rate_c[i] + out->ep_passive_rate[i] - out->stokes_dissipation[i];
        out->sed_rate[i] = bs[2 * i + 1];
    }
    // Conc_find_front_location, Conc.c:1610-1672: first x from the right where
    // the alpha-weighted height crosses the limit, interpolated linearly in the
    // height (MyMath_interpolate_quantity, two-point branch)
    out->front_location = -1.0;
    for (int i = d.NX - 2; i > 0; i--) {
        double h0 = 0.0, h1 = 0.0;
        for (int ic = 0; ic < nc; ic++) {
            h0 += hh[(size_t)ic * d.NX + i - 1] * c->prm.alpha[ic];
            h1 += hh[(size_t)ic * d.NX + i] * c->prm.alpha[ic];
        }
        if (h1 <= front_limit && h0 >= front_limit) {
            double m = (c->xc[i] - c->xc[i - 1]) / (h1 - h0);
            out->front_location = std::fabs(h1 - h0) < 1.0e-8 ? c->xc[i - 1] : m * (front_limit - h0) + c->xc[i - 1];
            break;
        }
    }
    if (ave_height) memcpy(ave_height, hh.data(), hh.size() * sizeof(double));
    return check_launch(c);
}

int turb_bed_index(turb_ctx *c, int32_t *iy)
{
    if (!c || !iy) return TURB_ERR_ARG;
    int rc = bed_setup(c);
    if (rc) return rc;
    TURB_CHECK(cudaMemcpyAsync(iy, c->bed_iy, sizeof(int32_t) * c->d.NZ * c->d.NX, cudaMemcpyDeviceToHost, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

int turb_deposit_integrate(turb_ctx *c, double dt)
{
    if (!c || !(dt > 0.0)) return TURB_ERR_ARG;
    int rc = bed_setup(c);
    if (rc) return rc;
    DepIn a;
    memset(&a, 0, sizeof(a));
    a.nconc = c->prm.nconc;
    a.dt = dt;
    for (int i = 0; i < a.nconc; i++) {
        a.us[i] = std::fabs(c->prm.vs0[i]);
        a.alpha[i] = c->prm.alpha[i];
        a.c[i] = c->fld[TURB_F_C0 + i];
        a.c_old[i] = c->old[3 + i];
    }
    launch_deposit(c->s, c->d, c->bed_iy, a, c->dep);
    c->launches++;
    return check_launch(c);
}

int turb_deposit_enable(turb_ctx *c, int on)
{
    if (!c) return TURB_ERR_ARG;
    int rc = bed_setup(c);
    if (rc) return rc;
    c->deposit_on = on ? 1 : 0;
    return TURB_OK;
}

int turb_deposit_get(turb_ctx *c, double *host)
{
    if (!c || !host) return TURB_ERR_ARG;
    int rc = bed_setup(c);
    if (rc) return rc;
    size_t b = sizeof(double) * c->prm.nconc * c->d.NZ * c->d.NX;
    TURB_CHECK(cudaMemcpyAsync(host, c->dep, b, cudaMemcpyDeviceToHost, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

int turb_deposit_set(turb_ctx *c, const double *host)
{
    if (!c || !host) return TURB_ERR_ARG;
    int rc = bed_setup(c);
    if (rc) return rc;
    size_t b = sizeof(double) * c->prm.nconc * c->d.NZ * c->d.NX;
    TURB_CHECK(cudaMemcpyAsync(c->dep, host, b, cudaMemcpyHostToDevice, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

// immersed-boundary geometry set-up for a bottom surface (k_geom.cu)
int turb_geometry(turb_ctx *c, const double *ipos, double *const *sdf, uint8_t *const *status, int *iterations)
{
    if (!c || !ipos) return TURB_ERR_ARG;
    const Dims &d = c->d;
    std::vector<double> wx = cell_widths(c->xu), wy = cell_widths(c->yv), wz = cell_widths(c->zw);
    if (!c->diag_dxc) {
        c->diag_dxc = c->mem.upload(wx);
        c->diag_dyc = c->mem.upload(wy);
        c->diag_dzc = c->mem.upload(wz);
        if (c->mem.err != cudaSuccess) return TURB_ERR_ALLOC;
    }
    // Levelset_compute_fictitious_time (Levelset.c:590-640): half the
    // smallest cell width of the physical cells
    double mxw = 1000.0, myw = 1000.0, mzw = 1000.0;
    for (int i = 0; i < d.nx; i++) if (wx[i] < mxw) mxw = wx[i];
    for (int j = 0; j < d.ny; j++) if (wy[j] < myw) myw = wy[j];
    for (int k = 0; k < d.nz; k++) if (wz[k] < mzw) mzw = wz[k];
    double dmin = myw < mxw ? myw : mxw;
    dmin = mzw < dmin ? mzw : dmin;
    GeomArgs a;
    a.d = d;
    a.xc = c->geo.xc; a.yc = c->geo.yc; a.zc = c->geo.zc;
    a.xu = c->geo.xu; a.yv = c->geo.yv; a.zw = c->geo.zw;
    a.mxu = c->geo.mxu; a.myv = c->geo.myv; a.mzw = c->geo.mzw;
    a.dxc = c->diag_dxc; a.dyc = c->diag_dyc; a.dzc = c->diag_dzc;
    a.a_dEta = 1.0 / c->dEta; a.a_dXi = 1.0 / c->dXi; a.a_dPhi = 1.0 / c->dPhi;
    a.dt = 0.5 * dmin;
    a.max_iterations = 500;
    // results and scratch live only for the call
    size_t fb = sizeof(double) * d.n;
    size_t need = 4 * fb + 4 * (size_t)d.n + (size_t)d.n + sizeof(double) * geom_scratch_doubles(d) +
                  sizeof(double) * d.NX * d.NZ;
    char *buf = nullptr;
    TURB_CHECK(cudaMalloc(&buf, need));
    GeomOut o;
    char *q = buf;
    for (int f = 0; f < 4; f++, q += fb) o.sdf[f] = (double *)q;
    double *scr = (double *)q;
    q += sizeof(double) * geom_scratch_doubles(d);
    double *dip = (double *)q;
    q += sizeof(double) * d.NX * d.NZ;
    for (int f = 0; f < 4; f++, q += d.n) o.st[f] = (uint8_t *)q;
    uint8_t *tmp = (uint8_t *)q;
    cudaError_t e = cudaMemcpyAsync(dip, ipos, sizeof(double) * d.NX * d.NZ, cudaMemcpyHostToDevice, c->s);
    if (e == cudaSuccess) e = geom_setup(c->s, a, dip, scr, tmp, &o);
    // ghost-cell stencils of u, v, w, c from the statuses and sdf just made
    // (Immersed_setup_q_immersed_nodes for each quantity)
    int *rows = nullptr, *node = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&rows, sizeof(int) * ((size_t)d.NY * d.NZ + 1));
    const int sq[4] = {1, 2, 3, 0};   // sdf index of u, v, w, c
    for (int q = 0; q < 4 && e == cudaSuccess; q++) {
        if (c->gib_buf[q]) cudaFree(c->gib_buf[q]);
        c->gib_buf[q] = nullptr;
        c->gib[q] = GeomIb();
        int n = 0;
        e = geom_ib_count(c->s, d, o.st[q], rows, &n);
        if (e != cudaSuccess || n == 0) continue;
        size_t bi = sizeof(int32_t) * (size_t)n, bd = sizeof(double) * (size_t)n;
        char *b = nullptr;
        e = cudaMalloc(&b, 10 * bi + 21 * bd);
        if (e != cudaSuccess) break;
        c->gib_buf[q] = b;
        GeomIb &g = c->gib[q];
        g.n = n;
        g.fcoef = (double *)b; b += 8 * bd;
        g.bcoef = (double *)b; b += bd;
        g.pts = (double *)b; b += 12 * bd;
        g.im = (int32_t *)b; b += bi;
        g.nf = (int32_t *)b; b += bi;
        g.fidx = (int32_t *)b; b += 8 * bi;
        if (node) cudaFree(node);
        node = nullptr;
        e = cudaMalloc(&node, bi);
        if (e == cudaSuccess) e = geom_ib_build(c->s, a, q, o.sdf[sq[q]], o.st[q], rows, node, g);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
    }
    if (rows) cudaFree(rows);
    if (node) cudaFree(node);
    for (int f = 0; f < 4 && e == cudaSuccess; f++) {
        if (sdf && sdf[f])
            e = cudaMemcpy2DAsync(sdf[f], (size_t)d.NX * 8, o.sdf[f], (size_t)d.PX * 8, (size_t)d.NX * 8,
                                  (size_t)d.NY * d.NZ, cudaMemcpyDeviceToHost, c->s);
        if (e == cudaSuccess && status && status[f])
            e = cudaMemcpy2DAsync(status[f], (size_t)d.NX, o.st[f], (size_t)d.PX, (size_t)d.NX,
                                  (size_t)d.NY * d.NZ, cudaMemcpyDeviceToHost, c->s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
    cudaFree(buf);
    if (e != cudaSuccess) return TURB_ERR_CUDA;
    if (iterations) *iterations = o.iterations;
    return TURB_OK;
}

int turb_geometry_stencils(turb_ctx *c, int q, int *n, int32_t *im, int32_t *nf, int32_t *fidx, double *fcoef,
                           double *bcoef, double *pts)
{
    if (!c || q < 0 || q > 3 || !n) return TURB_ERR_ARG;
    const GeomIb &g = c->gib[q];
    *n = g.n;
    if (g.n == 0) return TURB_OK;
    size_t N = (size_t)g.n;
    if (im) TURB_CHECK(cudaMemcpyAsync(im, g.im, 4 * N, cudaMemcpyDeviceToHost, c->s));
    if (nf) TURB_CHECK(cudaMemcpyAsync(nf, g.nf, 4 * N, cudaMemcpyDeviceToHost, c->s));
    if (fidx) TURB_CHECK(cudaMemcpyAsync(fidx, g.fidx, 32 * N, cudaMemcpyDeviceToHost, c->s));
    if (fcoef) TURB_CHECK(cudaMemcpyAsync(fcoef, g.fcoef, 64 * N, cudaMemcpyDeviceToHost, c->s));
    if (bcoef) TURB_CHECK(cudaMemcpyAsync(bcoef, g.bcoef, 8 * N, cudaMemcpyDeviceToHost, c->s));
    if (pts) TURB_CHECK(cudaMemcpyAsync(pts, g.pts, 96 * N, cudaMemcpyDeviceToHost, c->s));
    TURB_CHECK(cudaStreamSynchronize(c->s));
    return TURB_OK;
}

// the restart set of Resume_set_data (Resume.c:208-244): file name, field
static std::vector<std::pair<std::string, int>> resume_set(const turb_ctx *c)
{
    std::vector<std::pair<std::string, int>> v = {
        {"Resume_u.bin", TURB_F_U},       {"Resume_v.bin", TURB_F_V},       {"Resume_w.bin", TURB_F_W},
        {"Resume_dpdx.bin", TURB_F_DPX}, {"Resume_dpdy.bin", TURB_F_DPY}, {"Resume_dpdz.bin", TURB_F_DPZ}};
    for (int ic = 0; ic < c->prm.nconc; ic++) v.push_back({"Resume_conc" + std::to_string(ic) + ".bin", TURB_F_C0 + ic});
    return v;
}

static int resume_staging(turb_ctx *c)
{
    const Dims &d = c->d;
    long long n = (long long)d.NX * d.NY * d.NZ;
    if (!c->rs_dev) {
        c->rs_dev = c->mem.alloc<unsigned long long>(n);
        if (c->mem.err != cudaSuccess) return TURB_ERR_ALLOC;
    }
    if (!c->rs_host) TURB_CHECK(cudaMallocHost(&c->rs_host, (size_t)n * 8));
    return TURB_OK;
}

static std::string dep_name(int ic) { return "Resume_deposit_height" + std::to_string(ic) + ".bin"; }

int turb_resume_write(turb_ctx *c, const char *dir, const turb_primary *prim, int flags)
{
    if (!c || !prim) return TURB_ERR_ARG;
    const Dims &d = c->d;
    long long n = (long long)d.NX * d.NY * d.NZ;
    int rc = resume_staging(c);
    if (rc) return rc;
    auto put = [&](const std::string &name, const double *f, const uint8_t *st) -> int {
        if (f) launch_pack_be(c->s, d, f, c->rs_dev);
        else launch_pack_status_be(c->s, d, st, c->rs_dev);
        c->launches++;
        TURB_CHECK(cudaMemcpyAsync(c->rs_host, c->rs_dev, (size_t)n * 8, cudaMemcpyDeviceToHost, c->s));
        TURB_CHECK(cudaStreamSynchronize(c->s));
        return petsc_vec_write_be(resume_path(dir, name.c_str()).c_str(), c->rs_host, n);
    };
    for (auto &e : resume_set(c))
        if ((rc = put(e.first, c->fld[e.second], nullptr))) return rc;
    if ((flags & TURB_RESUME_GRID) && (rc = put("Resume_gridc.bin", nullptr, c->st[3]))) return rc;
    if ((flags & TURB_RESUME_PHI) && (rc = put("Resume_phi.bin", c->fld[TURB_F_PHI], nullptr))) return rc;
    if ((rc = turb_resume_primary_write(dir, prim))) return rc;
    if (flags & TURB_RESUME_DEPOSIT) {
        std::vector<double> h((size_t)c->prm.nconc * d.NZ * d.NX);
        if ((rc = turb_deposit_get(c, h.data()))) return rc;
        for (int ic = 0; ic < c->prm.nconc; ic++)
            if (c->prm.ctype[ic] == TURB_PARTICLE &&
                (rc = turb_resume_2d_write(resume_path(dir, dep_name(ic).c_str()).c_str(),
                                           h.data() + (size_t)ic * d.NZ * d.NX, d.NX, d.NZ)))
                return rc;
    }
    return check_launch(c);
}

int turb_resume_read(turb_ctx *c, const char *dir, turb_primary *prim, int flags)
{
    if (!c || !prim) return TURB_ERR_ARG;
    const Dims &d = c->d;
    long long n = (long long)d.NX * d.NY * d.NZ;
    int rc = resume_staging(c);
    if (rc) return rc;
    auto get = [&](const std::string &name, double *f) -> int {
        int r = petsc_vec_read_be(resume_path(dir, name.c_str()).c_str(), c->rs_host, n);
        if (r) return r;
        TURB_CHECK(cudaMemcpyAsync(c->rs_dev, c->rs_host, (size_t)n * 8, cudaMemcpyHostToDevice, c->s));
        launch_unpack_be(c->s, d, c->rs_dev, f);
        c->launches++;
        TURB_CHECK(cudaStreamSynchronize(c->s));   // the staging buffers are reused by the next file
        return TURB_OK;
    };
    turb_primary q;
    if ((rc = turb_resume_primary_read(dir, &q))) return rc;
    if (flags & TURB_RESUME_GRID) {
        std::vector<unsigned long long> file((size_t)n);
        if ((rc = petsc_vec_read_be(resume_path(dir, "Resume_gridc.bin").c_str(), file.data(), n))) return rc;
        launch_pack_status_be(c->s, d, c->st[3], c->rs_dev);
        c->launches++;
        TURB_CHECK(cudaMemcpyAsync(c->rs_host, c->rs_dev, (size_t)n * 8, cudaMemcpyDeviceToHost, c->s));
        TURB_CHECK(cudaStreamSynchronize(c->s));
        if (memcmp(file.data(), c->rs_host, (size_t)n * 8) != 0) return TURB_ERR_FORMAT;
    }
    for (auto &e : resume_set(c))
        if ((rc = get(e.first, c->fld[e.second]))) return rc;
    if (flags & TURB_RESUME_PHI) {
        if ((rc = get("Resume_phi.bin", c->fld[TURB_F_PHI]))) return rc;
    } else {
        TURB_CHECK(cudaMemsetAsync(c->fld[TURB_F_PHI], 0, sizeof(double) * d.n, c->s));
    }
    if (flags & TURB_RESUME_DEPOSIT) {
        std::vector<double> h((size_t)c->prm.nconc * d.NZ * d.NX, 0.0);
        for (int ic = 0; ic < c->prm.nconc; ic++)
            if (c->prm.ctype[ic] == TURB_PARTICLE &&
                (rc = turb_resume_2d_read(resume_path(dir, dep_name(ic).c_str()).c_str(),
                                          h.data() + (size_t)ic * d.NZ * d.NX, d.NX, d.NZ)))
                return rc;
        if ((rc = turb_deposit_set(c, h.data()))) return rc;
    }
    c->nh[0] = c->nh[1] = 0;
    *prim = q;
    return check_launch(c);
}

int turb_Conc_compute_total_concentration(turb_ctx *c)
{
    if (!c) return TURB_ERR_ARG;
    ConcPtrs cp;
    ConcW cw;
    for (int i = 0; i < 4; i++) { cp.p[i] = i < c->prm.nconc ? c->fld[TURB_F_C0 + i] : nullptr; cw.v[i] = c->prm.alpha[i]; }
    launch_total_conc(c->s, c->d.n, c->prm.nconc, cp, cw, c->fld[TURB_F_CTOT]);
    c->launches += 1;
    return check_launch(c);
}

int turb_Conc_set_particle_v_velocity(turb_ctx *c, int ic)
{
    if (!c || ic < 0 || ic >= c->prm.nconc) return TURB_ERR_ARG;
    double sh = c->prm.ctype[ic] == TURB_PARTICLE ? c->prm.vs0[ic] : 0.0;
    if (c->prm.ctype[ic] == TURB_PARTICLE)
        launch_shift(c->s, c->d.n, c->fld[TURB_F_VBC], sh, c->fld[TURB_F_VP0 + ic]);
    else
        cudaMemcpyAsync(c->fld[TURB_F_VP0 + ic], c->fld[TURB_F_VBC], c->d.n * 8, cudaMemcpyDeviceToDevice, c->s);
    c->launches += 1;
    return check_launch(c);
}

static AdvSrc adv_of(int kind, const double *a, W2 wx, W2 wy, double shift = 0.0)
{
    AdvSrc s;
    s.kind = kind;
    s.a = a;
    s.wx = wx;
    s.wy = wy;
    s.shift = shift;
    return s;
}

// u next to the open faces for the transposes inside the ENO x pass
static void open_adv(const turb_ctx *c, AdvSrc &a)
{
    a.pin = c->ob.in ? c->pl_in_u : nullptr;
    a.pout = c->ob.out ? c->pl_out[0] : nullptr;
    a.pNY = c->d.NY;
    a.nx = c->d.nx;
}

int turb_Velocity_convective_terms(turb_ctx *c, char which)
{
    int q = qidx(which);
    if (!c || q < 0 || q > 2) return TURB_ERR_ARG;
    const Dims &d = c->d;
    int nx = d.nx, ny = d.ny, nz = d.nz;
    int i0 = q == 0 ? 1 : 0, j0 = q == 1 ? 1 : 0, k0 = q == 2 ? 1 : 0;
    const double *u = c->fld[TURB_F_U], *v = c->fld[TURB_F_V], *w = c->fld[TURB_F_W];
    const double *self = q == 0 ? u : q == 1 ? v : w;
    double *conv = c->fld[TURB_F_CONV_U + q];
    W2 z{nullptr, nullptr};
    AdvSrc ax, ay, az;
    if (q == 0) {
        ax = adv_of(0, u, z, z);
        ay = adv_of(2, v, c->tw.xu, c->tw.yc);
        az = adv_of(3, w, c->tw.xu, c->tw.zc);
    } else if (q == 1) {
        ax = adv_of(4, u, c->tw.xc, c->tw.yv);
        open_adv(c, ax);
        ay = adv_of(0, v, z, z);
        az = adv_of(5, w, c->tw.zc, c->tw.yv);
    } else {
        ax = adv_of(6, u, c->tw.xc, c->tw.zw);
        open_adv(c, ax);
        ay = adv_of(7, v, c->tw.zw, c->tw.yc);
        az = adv_of(0, w, z, z);
    }
    cudaMemsetAsync(conv, 0, d.n * 8, c->s);
    const double npts = (double)d.NX * d.NY * d.NZ;
    int h = prof_begin(c, TURB_PROF_ENO_X);
    launch_eno_pass(c->s, d, 0, c->eno[q][0], self, ax, j0, ny - 1, k0, nz - 1, 1, conv, (c->kvariant & TURB_KV_ENO_SEGMENTS) ? 0 : 1);
    prof_end(c, h, 1, ENO_X_BYTES * npts);
    h = prof_begin(c, TURB_PROF_ENO_YZ);
    launch_eno_pass(c->s, d, 1, c->eno[q][1], self, ay, i0, nx - 1, k0, nz - 1, 0, conv, (c->kvariant & TURB_KV_ENO_SEGMENTS) ? 0 : 1);
    launch_eno_pass(c->s, d, 2, c->eno[q][2], self, az, i0, nx - 1, j0, ny - 1, 0, conv, (c->kvariant & TURB_KV_ENO_SEGMENTS) ? 0 : 1);
    prof_end(c, h, 2, 2.0 * ENO_YZ_BYTES * npts);
    c->launches += 3;
    return check_launch(c);
}

int turb_Conc_convective_terms(turb_ctx *c, int ic)
{
    if (!c || ic < 0 || ic >= c->prm.nconc) return TURB_ERR_ARG;
    const Dims &d = c->d;
    W2 z{nullptr, nullptr};
    double *conv = c->fld[TURB_F_CCONV0 + ic];
    const double *cf = c->fld[TURB_F_C0 + ic];
    AdvSrc ax = adv_of(0, c->fld[TURB_F_UBC], z, z);
    AdvSrc ay = c->prm.ctype[ic] == TURB_PARTICLE ? adv_of(1, c->fld[TURB_F_VBC], z, z, c->prm.vs0[ic])
                                                  : adv_of(0, c->fld[TURB_F_VBC], z, z);
    AdvSrc az = adv_of(0, c->fld[TURB_F_WBC], z, z);
    cudaMemsetAsync(conv, 0, d.n * 8, c->s);
    const double npts = (double)d.NX * d.NY * d.NZ;
    int h = prof_begin(c, TURB_PROF_ENO_X);
    launch_eno_pass(c->s, d, 0, c->ob.in || c->ob.out ? c->eno_cx[ic] : c->eno[3][0], cf, ax, 0, d.ny - 1, 0,
                    d.nz - 1, 1, conv, (c->kvariant & TURB_KV_ENO_SEGMENTS) ? 0 : 1);
    prof_end(c, h, 1, ENO_X_BYTES * npts);
    h = prof_begin(c, TURB_PROF_ENO_YZ);
    launch_eno_pass(c->s, d, 1, c->eno_cy[ic], cf, ay, 0, d.nx - 1, 0, d.nz - 1, 0, conv, (c->kvariant & TURB_KV_ENO_SEGMENTS) ? 0 : 1);
    launch_eno_pass(c->s, d, 2, c->eno[3][2], cf, az, 0, d.nx - 1, 0, d.ny - 1, 0, conv, (c->kvariant & TURB_KV_ENO_SEGMENTS) ? 0 : 1);
    prof_end(c, h, 2, 2.0 * ENO_YZ_BYTES * npts);
    c->launches += 3;
    return check_launch(c);
}

int turb_Velocity_set_RHS(turb_ctx *c, char which, double dt)
{
    int q = qidx(which);
    if (!c || q < 0 || q > 2 || !(dt > 0.0)) return TURB_ERR_ARG;
    const double *ct = c->prm.nconc > 1 ? c->fld[TURB_F_CTOT] : c->fld[TURB_F_C0];
    launch_rhs_vel(c->s, c->d, q, c->st[q], 1.0 / dt, c->fld[TURB_F_U + q], c->fld[TURB_F_CONV_U + q],
                   c->fld[TURB_F_DPX + q], ct, c->prm.buoyancy, c->iyv, c->ob, c->fld[TURB_F_B_U + q]);
    c->launches += 1;
    return check_launch(c);
}

int turb_Conc_set_RHS(turb_ctx *c, int ic, double dt)
{
    if (!c || ic < 0 || ic >= c->prm.nconc || !(dt > 0.0)) return TURB_ERR_ARG;
    launch_rhs_conc(c->s, c->d, ic, c->st[3], 1.0 / dt, c->fld[TURB_F_C0 + ic], c->fld[TURB_F_CCONV0 + ic], c->ob,
                    c->fld[TURB_F_CB0 + ic]);
    c->launches += 1;
    return check_launch(c);
}

// The 1/dt term of the diagonal of Helmholtz system sys (0..2 u, v, w;
// 3 + ic the fractions), kept as Velocity_modify_diagonal /
// Conc_modify_diagonal keep it (Velocity.c:384-396, Conc.c:304-314): the
// first call sets 1/dt; a later call with a new dt adds 1/dt - 1/dt_old
// (dt_old = the dt of the previous call) only when that exceeds 1e-10 in
// magnitude.  IMMERSED rows never carry it (the kernels skip them).
static double diag_term(turb_ctx *c, int sys, double dt)
{
    double &a = c->adt[sys], &last = c->adt_dt[sys];
    if (!(last > 0.0)) {
        a = 1.0 / dt;
    } else {
        double mod = 1.0 / dt - 1.0 / last;
        if (std::fabs(mod) > 1.0e-10) a = a + mod;
    }
    last = dt;
    return a;
}

static int helm_solve_fp64(turb_ctx *c, int q, int ic, int fx, int fb, double dt, int *iters)
{
    const Dims &d = c->d;
    const HelmTab &h = q < 3 ? c->helm[q] : c->helm_c[ic];
    const IbDev &ib = c->ib[q];
    double a_dt = diag_term(c, q < 3 ? q : 3 + ic, dt);
    double *b = c->fld[fb];
    launch_norm2(c->s, d.n, b, c->part, norm_parts(), c->dscal);
    int rc = fetch_scalars(c, 1);
    if (rc) return rc;
    double nb = std::sqrt(c->hscal[0]);
    long long hp = helm_parts(d);
    long long np = hp + (ib.n > 0 ? (ib.n + 255) / 256 : 0);
    int it = 0;
    c->launches += 2;
    for (;;) {
        double *x = c->fld[fx];
        int ph = prof_begin(c, TURB_PROF_JACOBI);
        launch_helm_jacobi(c->s, d, h, c->st[q], a_dt, b, x, c->jtmp, ib, c->part, hp);
        prof_end(c, ph, 1, HELM_JACOBI_BYTES * ((double)d.NX * d.NY * d.NZ) + IB_ROW_BYTES * ib.n);
        launch_sum_final(c->s, np, c->part, c->dscal);
        c->launches += 2 + (ib.n > 0);
        rc = fetch_scalars(c, 1);
        if (rc) return rc;
        double nr = std::sqrt(c->hscal[0]);
        if (!std::isfinite(nr)) { if (iters) *iters = it; return TURB_ERR_NAN; }
        if (nr <= c->prm.vel_rtol * nb) break;
        if (it >= c->prm.vel_maxit) { if (iters) *iters = it; return TURB_ERR_NOT_CONVERGED; }
        // the non-immersed and immersed rows of jtmp are all written: swap
        std::swap(c->fld[fx], c->jtmp);
        it++;
    }
    if (iters) *iters = it;
    return TURB_OK;
}

// FP64 defect correction with FP32 inner Jacobi sweeps: every outer step
// forms x <- x + e and r = b - A x in FP64 (the convergence test is on this
// FP64 residual), then approximately solves A e = r with hinner FP32 sweeps.
static int helm_solve_mixed(turb_ctx *c, int q, int ic, int fx, int fb, double dt, int *iters)
{
    const Dims &d = c->d;
    const HelmTab &h = q < 3 ? c->helm[q] : c->helm_c[ic];
    const HelmTabF &hf = q < 3 ? c->helmf[q] : c->helmf_c[ic];
    const IbDev &ib = c->ib[q];
    const IbDevF &ibf = c->ibf[q];
    double a_dt = diag_term(c, q < 3 ? q : 3 + ic, dt);
    double *b = c->fld[fb];
    launch_norm2(c->s, d.n, b, c->part, norm_parts(), c->dscal);
    int rc = fetch_scalars(c, 1);
    if (rc) return rc;
    double nb = std::sqrt(c->hscal[0]);
    long long hp = helm_parts(d);
    long long np = hp + (ib.n > 0 ? (ib.n + 255) / 256 : 0);
    int it = 0;
    c->launches += 2;
    float *e = c->he0, *en = c->he1;
    for (;;) {
        if (it > 0) {
            launch_add_corr(c->s, d.n, c->fld[fx], e, c->jtmp);   // x <- x + e
            std::swap(c->fld[fx], c->jtmp);
            c->launches += 1;
        }
        int ph = prof_begin(c, TURB_PROF_JACOBI);
        launch_helm_resid64(c->s, d, h, c->st[q], a_dt, b, c->fld[fx], c->hrf, ib, c->part, hp);
        prof_end(c, ph, 1, HELM_RESID64_BYTES * ((double)d.NX * d.NY * d.NZ) + IB_ROW_BYTES * ib.n);
        launch_sum_final(c->s, np, c->part, c->dscal);
        c->launches += 2 + (ib.n > 0);
        rc = fetch_scalars(c, 1);
        if (rc) return rc;
        double nr = std::sqrt(c->hscal[0]);
        if (!std::isfinite(nr)) { if (iters) *iters = it; return TURB_ERR_NAN; }
        if (nr <= c->prm.vel_rtol * nb) break;
        if (it >= c->prm.vel_maxit) { if (iters) *iters = it; return TURB_ERR_NOT_CONVERGED; }
        ph = prof_begin(c, TURB_PROF_INNER32);
        int gi = q < 3 ? q : 3 + ic;
        auto sweeps = [&]() {
            float *ea = c->he0, *eb = c->he1;
            for (int t = 0; t < c->hinner; t++) {
                launch_helm_jac32(c->s, d, hf, c->st[q], (float)a_dt, c->hrf, ea, eb, ibf, t == 0,
                                  c->kvariant & TURB_KV_MARCHING);
                std::swap(ea, eb);
            }
        };
        if (c->use_graphs) {
            if (c->g_inner[gi] && c->g_inner_n[gi] != c->hinner) { cudaGraphExecDestroy(c->g_inner[gi]); c->g_inner[gi] = nullptr; }
            if (!c->g_inner[gi]) { int rc2 = capture(c, &c->g_inner[gi], sweeps); if (rc2) return rc2; c->g_inner_n[gi] = c->hinner; }
            TURB_CHECK(cudaGraphLaunch(c->g_inner[gi], c->s));
        } else {
            sweeps();
        }
        // the sweeps start from he0 and alternate; the result is in he0 after
        // an even number of sweeps
        e = (c->hinner % 2 == 0) ? c->he0 : c->he1;
        en = (e == c->he0) ? c->he1 : c->he0;
        prof_end(c, ph, c->hinner,
                 (HELM_JAC32_FIRST_BYTES + HELM_JAC32_BYTES * (c->hinner - 1)) * ((double)d.NX * d.NY * d.NZ) +
                     IB_ROW_BYTES * 0.5 * ibf.n * c->hinner);
        c->launches += c->hinner * (1 + (ib.n > 0));
        it++;
    }
    if (iters) *iters = it;
    return TURB_OK;
}

static int helm_solve(turb_ctx *c, int q, int ic, int fx, int fb, double dt, int *iters)
{
    return c->hmode == TURB_HMODE_MIXED ? helm_solve_mixed(c, q, ic, fx, fb, dt, iters)
                                        : helm_solve_fp64(c, q, ic, fx, fb, dt, iters);
}

int turb_set_eno_division(turb_ctx *c, int fast)
{
    if (!c || (fast != 0 && fast != 1)) return TURB_ERR_ARG;
    for (int q = 0; q < 4; q++)
        for (int dd = 0; dd < 3; dd++) c->eno[q][dd].fastdiv = fast;
    for (int ic = 0; ic < TURB_MAXCONC; ic++) c->eno_cy[ic].fastdiv = fast;
    return TURB_OK;
}

int turb_set_helmholtz_mode(turb_ctx *c, int mode, int inner_sweeps)
{
    if (!c || (mode != TURB_HMODE_FP64 && mode != TURB_HMODE_MIXED) || inner_sweeps < 1 || inner_sweeps > 64)
        return TURB_ERR_ARG;
    c->hmode = mode;
    c->hinner = inner_sweeps;
    return TURB_OK;
}

int turb_Velocity_solve(turb_ctx *c, char which, double dt, int *iters)
{
    int q = qidx(which);
    if (!c || q < 0 || q > 2 || !(dt > 0.0)) return TURB_ERR_ARG;
    return helm_solve(c, q, 0, TURB_F_U + q, TURB_F_B_U + q, dt, iters);
}

int turb_Conc_solve(turb_ctx *c, int ic, double dt, int *iters)
{
    if (!c || ic < 0 || ic >= c->prm.nconc || !(dt > 0.0)) return TURB_ERR_ARG;
    return helm_solve(c, 3, ic, TURB_F_C0 + ic, TURB_F_CB0 + ic, dt, iters);
}

int turb_helmholtz_apply(turb_ctx *c, char which, int ic, double dt, int fx, int fy)
{
    int q = qidx(which);
    if (!c || q < 0 || !(dt > 0.0) || !field_ptr(c, fx) || !field_ptr(c, fy)) return TURB_ERR_ARG;
    if (q == 3 && (ic < 0 || ic >= c->prm.nconc)) return TURB_ERR_ARG;
    launch_helm_apply(c->s, c->d, q < 3 ? c->helm[q] : c->helm_c[ic], c->st[q], diag_term(c, q < 3 ? q : 3 + ic, dt),
                      c->fld[fx], c->fld[fy], c->ib[q]);
    c->launches += 2;
    return check_launch(c);
}

int turb_Pressure_set_RHS(turb_ctx *c, double dt)
{
    if (!c || !(dt > 0.0)) return TURB_ERR_ARG;
    c->p_dt = dt;
    launch_pressure_rhs(c->s, c->d, c->st[3], c->pcx, c->pcy, c->pcz, 1.0 / dt, c->ob, c->fld[TURB_F_U],
                        c->fld[TURB_F_V], c->fld[TURB_F_W], c->fld[TURB_F_PB]);
    c->launches += 1;
    return check_launch(c);
}

// Galerkin fit of the initial guess of stage st (projection onto earlier
// solutions, after Fischer's method for successive right-hand sides): over
// x0 + span{p1 - x0, p2 - x0 [, candidate - x0]}, with x0 the current guess
// (px, residual pr), p1 / p2 this stage's last two solutions (S p_m = W b_m
// to their tolerance) and the network candidate (pz, computed residual pq),
// the coefficients minimise the S-norm of the error: (D^T S D) a = D^T r.
// Directions whose pivot is negligible are dropped.  The fit goes to pp,
// its true residual to pro; *nr_out = |pro| (0 when no fit was made) and
// *de_out = -a^T g / 2, the change of the energy 1/2 x^T S x - x^T W b from
// x0 to the fit (< 0: a smaller S-norm of the error, equivalently a smaller
// S^-1-norm of the residual, the norm CG minimises).
static int galerkin_guess(turb_ctx *c, int st, int with_net, double *nr_out, double *de_out)
{
    const MgDevLevel &L0 = c->H64.lev[0];
    long long n0 = (long long)L0.nx * L0.ny * L0.nz;
    cudaStream_t s = c->s;
    GalDirs dd;
    dd.nd = 0;
    for (int m = 0; m < 2; m++) {
        dd.y[dd.nd] = c->ph[st][m];
        dd.w[dd.nd] = c->pw[st][m];
        dd.resid[dd.nd] = 0;
        dd.nd++;
    }
    if (with_net) {
        dd.y[dd.nd] = c->pz;
        dd.w[dd.nd] = c->pq;
        dd.resid[dd.nd] = 1;
        dd.nd++;
    }
    *nr_out = 0.0;
    *de_out = 0.0;
    pcg_gal_dots(s, n0, dd, c->px, c->pr, c->pbw, c->part, c->dscal);
    const int nv = GAL_MAX * GAL_MAX + GAL_MAX;
    TURB_CHECK(cudaMemcpyAsync(c->hscal, c->dscal, nv * sizeof(double), cudaMemcpyDeviceToHost, s));
    TURB_CHECK(cudaStreamSynchronize(s));
    c->launches += 2;
    double G[GAL_MAX][GAL_MAX], g[GAL_MAX];
    int n = dd.nd;
    for (int a = 0; a < n; a++) {
        g[a] = c->hscal[GAL_MAX * GAL_MAX + a];
        for (int b = 0; b < n; b++)
            G[a][b] = 0.5 * (c->hscal[a * GAL_MAX + b] + c->hscal[b * GAL_MAX + a]);   // S is symmetric
    }
    // Cholesky with pivots below 1e-12 of the largest diagonal dropped
    double dmax = 0.0;
    for (int a = 0; a < n; a++) dmax = std::max(dmax, G[a][a]);
    if (!(dmax > 0.0) || !std::isfinite(dmax)) return TURB_OK;
    double L[GAL_MAX][GAL_MAX] = {}, y[GAL_MAX] = {}, al[GAL_MAX] = {};
    int keep[GAL_MAX] = {};
    for (int a = 0; a < n; a++) {
        double d = G[a][a];
        for (int k = 0; k < a; k++) if (keep[k]) d -= L[a][k] * L[a][k];
        if (!(d > 1e-12 * dmax)) continue;
        keep[a] = 1;
        L[a][a] = std::sqrt(d);
        for (int b = a + 1; b < n; b++) {
            double t = G[b][a];
            for (int k = 0; k < a; k++) if (keep[k]) t -= L[b][k] * L[a][k];
            L[b][a] = t / L[a][a];
        }
    }
    for (int a = 0; a < n; a++) {
        if (!keep[a]) continue;
        double t = g[a];
        for (int k = 0; k < a; k++) if (keep[k]) t -= L[a][k] * y[k];
        y[a] = t / L[a][a];
    }
    for (int a = n - 1; a >= 0; a--) {
        if (!keep[a]) continue;
        double t = y[a];
        for (int k = a + 1; k < n; k++) if (keep[k]) t -= L[k][a] * al[k];
        al[a] = t / L[a][a];
    }
    GalCoef co;
    double de = 0.0;
    for (int a = 0; a < GAL_MAX; a++) {
        co.a[a] = a < n && keep[a] && std::isfinite(al[a]) ? al[a] : 0.0;
        if (a < n) de -= 0.5 * co.a[a] * g[a];
    }
    *de_out = de;
    pcg_gal_update(s, n0, dd, co, c->px, c->pp);
    pcg_resid(s, L0, c->pbw, c->pp, c->pro, c->part);
    pcg_reduce(s, c->part, 1, c->dscal, pcg_stencil_parts(L0));
    TURB_CHECK(cudaMemcpyAsync(c->hscal, c->dscal, sizeof(double), cudaMemcpyDeviceToHost, s));
    TURB_CHECK(cudaStreamSynchronize(s));
    c->launches += 3;
    double nr = std::sqrt(c->hscal[0]);
    *nr_out = std::isfinite(nr) ? nr : 0.0;
    return TURB_OK;
}

int turb_Pressure_solve(turb_ctx *c, int *iters, double *relres)
{
    if (!c) return TURB_ERR_ARG;
    const Dims &d = c->d;
    const MgDevLevel &L0 = c->H64.lev[0];
    long long n0 = (long long)L0.nx * L0.ny * L0.nz;
    cudaStream_t s = c->s;
    PcgScal *sc = c->sc;
    double *dsc = reinterpret_cast<double *>(sc);   // bb rr rz zr_old rz_old pq alpha beta
    pcg_gather(s, d, L0, c->fld[TURB_F_PHI], c->fld[TURB_F_PB], c->px, c->pbw);
    pcg_dot(s, n0, c->pbw, c->pbw, c->part);
    pcg_reduce(s, c->part, 1, dsc + 0);
    int nsp = pcg_stencil_parts(L0);
    pcg_resid(s, L0, c->pbw, c->px, c->pr, c->part);
    pcg_reduce(s, c->part, 1, dsc + 1, nsp);
    c->launches += 5;
    TURB_CHECK(cudaMemcpyAsync(c->hscal, dsc, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    TURB_CHECK(cudaStreamSynchronize(s));
    double nb = std::sqrt(c->hscal[0]), nr = std::sqrt(c->hscal[1]);
    // candidate initial guess from this stage's history; kept only if it
    // lowers the initial residual below the previous-solution guess
    int st = c->stage & 1;
    if (c->snaps && c->nh[st] >= 2) {
        int rc = net_snapshot(c->snaps, s, L0, c->H64.invd[0], c->pr, c->pbw, c->ph[st][0], c->ph[st][1], c->px);
        if (rc) return rc;
        c->launches += 5;
    }
    // the stages that evaluate the candidate (guess_stages); with the
    // Galerkin fit on, the learned mode fits the earlier solutions alone in
    // the other stages
    const bool cand_stage = (c->guess_stages >> st) & 1;
    const bool fit_only = !cand_stage && c->guess_mode == TURB_GUESS_LEARNED && c->galerkin;
    if (c->guess_mode != TURB_GUESS_PREVIOUS && c->nh[st] >= 2 && (cand_stage || fit_only)) {
        int ok = 0, ph = -1, fitted = 0;
        double nrc = 0.0;
        if (fit_only) {
            // no candidate: the fit below over this stage's earlier solutions
        } else if (c->guess_mode == TURB_GUESS_EXTRAPOLATE) {
            pcg_lincomb(s, n0, 2.0, c->ph[st][0], -1.0, c->ph[st][1], c->pz);
            c->launches += 1;
            ok = 1;
        } else if (c->guess_mode == TURB_GUESS_LEARNED && c->net) {
            // candidate = previous pressure + network correction of its residual
            ph = prof_begin(c, TURB_PROF_NET);
            int rc = net_guess(c->net, s, L0, c->H64.invd[0], c->pr, c->pbw, c->ph[st][0], c->ph[st][1], c->px,
                               c->pz);
            if (rc) return rc;
            c->launches += NET_GUESS_LAUNCHES;
            ok = 1;
        }
        if (ok) {
            pcg_resid(s, L0, c->pbw, c->pz, c->pq, c->part);
            pcg_reduce(s, c->part, 1, dsc + 1, nsp);
            c->launches += 2;
            TURB_CHECK(cudaMemcpyAsync(c->hscal + 2, dsc + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
            TURB_CHECK(cudaStreamSynchronize(s));
            nrc = std::sqrt(c->hscal[2]);
            if (ph >= 0) prof_end(c, ph, NET_GUESS_LAUNCHES + 2);
        }
        // Galerkin fit over the earlier solutions of this stage (and the
        // network candidate): the energy-norm best guess in their span
        if ((c->guess_mode == TURB_GUESS_PROJECT || (c->guess_mode == TURB_GUESS_LEARNED && c->galerkin && (ok || fit_only))) &&
            c->pw[st][1]) {
            double ng = 0.0, de = 0.0;
            int rc = galerkin_guess(c, st, ok && c->guess_mode == TURB_GUESS_LEARNED, &ng, &de);
            if (rc) return rc;
            // the fit minimises the S-norm of the error over a span that holds
            // x0 and the network candidate: it is kept whenever it lowers the
            // residual in the S^-1 norm (de < 0), the norm CG reduces
            fitted = ng > 0.0 && de < 0.0;
            if (fitted) {   // the fit is in pp / pro
                std::swap(c->pz, c->pp);
                std::swap(c->pq, c->pro);
                nrc = ng;
                ok = 1;
            }
        }
        if (ok) {
            c->guess_tried++;
            if (nr > 0.0 && nrc > 0.0 && std::isfinite(nrc)) c->guess_logsum += std::log(nrc / nr);
            if (fitted || nrc < nr) {
                pcg_copy(s, n0, c->pz, c->px);
                pcg_copy(s, n0, c->pq, c->pr);
                c->launches += 2;
                nr = nrc;
                c->guess_taken++;
            }
        }
    }
    double tol = c->prm.p_rtol * nb;
    int it = 0, restart = 1, status = TURB_OK;
    const int pmi = c->pmode == TURB_PMODE_FP64 ? 0 : 1;
    const int *npre = c->mg_pre[pmi], *npost = c->mg_post[pmi];
    int vl = pmi == 0 ? mg_vcycle_launches(c->H64.nl, npre, npost, c->H64.tail_from, c->H64.cluster_from, 0)
                      : mg_vcycle_launches(c->H32.nl, npre, npost, c->H32.tail_from, c->H32.cluster_from, c->H32.tb ? 1 : 0);
    for (;;) {
        if (!std::isfinite(nr)) { status = TURB_ERR_NAN; break; }
        if (nr <= tol || it >= c->prm.p_maxit) {
            pcg_resid(s, L0, c->pbw, c->px, c->pr, c->part);
            pcg_reduce(s, c->part, 1, dsc + 1, nsp);
            c->launches += 2;
            TURB_CHECK(cudaMemcpyAsync(c->hscal + 1, dsc + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
            TURB_CHECK(cudaStreamSynchronize(s));
            nr = std::sqrt(c->hscal[1]);
            if (nr <= tol) {
                if (!(c->div_gate > 0.0)) break;
                // the divergence the projection with this phi leaves is dt
                // times the unweighted residual b - A phi = r / (dx dy dz)
                pcg_rmax(s, L0, c->pr, c->part, c->dscal);
                TURB_CHECK(cudaMemcpyAsync(c->hscal + 3, c->dscal, sizeof(double), cudaMemcpyDeviceToHost, s));
                TURB_CHECK(cudaStreamSynchronize(s));
                c->launches += 2;
                double dmax = c->p_dt * c->hscal[3];
                if (dmax <= c->div_gate) break;
                if (!std::isfinite(dmax)) { status = TURB_ERR_NAN; break; }
                // relative residual met, divergence not: tighten in
                // proportion, down to the residual's round-off floor.  At the
                // floor more iterations cannot lower r; what the estimate
                // still sees is the rounding of b - A phi divided by the
                // smallest cell volumes of a stretched grid, not divergence
                // the projection would leave
                const double floor = 64.0 * DBL_EPSILON * nb;
                if (nr <= floor) {
                    c->gate_floor++;
                    break;
                }
                tol = std::max(floor, nr * std::min(0.5, 0.5 * c->div_gate / dmax));
                c->gate_tightened++;
            }
            if (it >= c->prm.p_maxit) { status = TURB_ERR_NOT_CONVERGED; break; }
            restart = 1;
        }
        int pm = c->pmode == TURB_PMODE_FP64 ? 0 : 1;
        auto vcycle = [&]() {
            if (pm == 0) {
                mg_vcycle<double>(s, c->H64, 0, npre, npost);
            } else {
                mg_to_float(s, c->H32.lev[0], c->pr, c->H32.b[0]);
                mg_vcycle<float>(s, c->H32, 0, npre, npost);
                mg_to_double(s, c->H32.lev[0], c->H32.x[0], c->pz, c->H32.pdl);
            }
        };
        auto cgstep = [&](int rs) {
            pcg_dot2(s, n0, c->pr, c->pz, c->pro, c->part);
            pcg_reduce(s, c->part, 2, dsc + 2);   // rz and z.r_old
            if (!rs) pcg_scalars(s, sc, 0);
            pcg_pupdate(s, n0, c->pz, c->pp, sc, rs);
            pcg_apply(s, L0, c->pp, c->pq, c->part);
            pcg_reduce(s, c->part, 1, dsc + 5, nsp);
            pcg_scalars(s, sc, 1);
            pcg_xrupdate(s, n0, c->px, c->pr, c->pro, c->pp, c->pq, sc, c->part);
            pcg_reduce(s, c->part, 1, dsc + 1);
        };
        int nmg = vl + (pm ? 2 : 0), ncg = 8 + (restart ? 0 : 1);
        int ph = prof_begin(c, TURB_PROF_MG);
        if (c->use_graphs) {
            if (!c->g_mg[pm]) { int rc = capture(c, &c->g_mg[pm], vcycle); if (rc) return rc; }
            TURB_CHECK(cudaGraphLaunch(c->g_mg[pm], s));
        } else {
            vcycle();
        }
        prof_end(c, ph, nmg,
                 pm == 0 ? mg_vcycle_bytes<double>(c->H64, 0, npre, npost)
                         : mg_vcycle_bytes<float>(c->H32, 0, npre, npost) + 24.0 * n0);
        ph = prof_begin(c, TURB_PROF_PCG);
        if (c->use_graphs) {
            if (!c->g_pcg[restart]) {
                int rs = restart;
                int rc = capture(c, &c->g_pcg[restart], [&]() { cgstep(rs); });
                if (rc) return rc;
            }
            TURB_CHECK(cudaGraphLaunch(c->g_pcg[restart], s));
        } else {
            cgstep(restart);
        }
        prof_end(c, ph, ncg, (restart ? 112.0 : 120.0) * n0);
        c->launches += nmg + ncg;
        TURB_CHECK(cudaMemcpyAsync(c->hscal + 1, dsc + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
        TURB_CHECK(cudaStreamSynchronize(s));
        nr = std::sqrt(c->hscal[1]);
        restart = 0;
        it++;
    }
    if (pmi == 1 && c->H32.tb) {   // a copy wait of the two-sweep smoother that timed out
        TURB_CHECK(cudaMemcpyAsync(c->hscal + 15, c->tb_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        TURB_CHECK(cudaStreamSynchronize(s));
        int bad = 0;
        std::memcpy(&bad, c->hscal + 15, sizeof(int));
        if (bad) {
            TURB_CHECK(cudaMemsetAsync(c->tb_err, 0, sizeof(int), s));
            return turb_set_cuda_error(cudaErrorLaunchTimeout, __FILE__, __LINE__);
        }
    }
    pcg_scatter(s, d, L0, c->px, c->fld[TURB_F_PHI]);
    c->launches += 1;
    if (c->snaps) {
        int rc = net_snapshot_finish(c->snaps, s, L0, c->H64.invd[0], c->px, status == TURB_OK);
        if (rc) return rc;
    }
    // the per-stage history of converged pressures (what the extrapolated and
    // learned guesses start from) is kept whenever a guess could use it
    if (status == TURB_OK && (c->guess_mode != TURB_GUESS_PREVIOUS || c->snaps || c->net)) {
        if (!c->ph[st][0]) {
            c->ph[st][0] = c->mem.alloc<double>(n0);
            c->ph[st][1] = c->mem.alloc<double>(n0);
            if (c->mem.err != cudaSuccess) return TURB_ERR_ALLOC;
        }
        std::swap(c->ph[st][0], c->ph[st][1]);
        pcg_copy(s, n0, c->px, c->ph[st][0]);
        {   // their right-hand sides, for the Galerkin fit
            if (!c->pw[st][0]) {
                c->pw[st][0] = c->mem.alloc<double>(n0);
                c->pw[st][1] = c->mem.alloc<double>(n0);
                if (c->mem.err != cudaSuccess) return TURB_ERR_ALLOC;
            }
            std::swap(c->pw[st][0], c->pw[st][1]);
            pcg_copy(s, n0, c->pbw, c->pw[st][0]);
            c->launches += 1;
        }
        c->launches += 1;
        c->nh[st] = std::min(c->nh[st] + 1, 2);
    }
    if (iters) *iters = it;
    if (relres) *relres = nb > 0.0 ? nr / nb : 0.0;
    int rc = check_launch(c);
    return rc ? rc : status;
}

int turb_pressure_apply(turb_ctx *c, int fx, int fy)
{
    if (!c || !field_ptr(c, fx) || !field_ptr(c, fy)) return TURB_ERR_ARG;
    launch_pressure_apply(c->s, c->d, c->st[3], c->geo, c->dEta, c->dXi, c->dPhi, c->fld[fx], c->fld[fy]);
    c->launches += 1;
    return check_launch(c);
}

int turb_Pressure_project_velocity(turb_ctx *c, double dt)
{
    if (!c || !(dt > 0.0)) return TURB_ERR_ARG;
    ProjArgs a = c->proj;
    a.dt = dt;
    a.coef = dt / c->prm.re;
    launch_project(c->s, c->d, a, c->fld[TURB_F_PHI], c->fld[TURB_F_PB], c->fld[TURB_F_U], c->fld[TURB_F_V],
                   c->fld[TURB_F_W], c->fld[TURB_F_DPX], c->fld[TURB_F_DPY], c->fld[TURB_F_DPZ]);
    c->launches += 1;
    return check_launch(c);
}

int turb_Pressure_compute_velocity_divergence(turb_ctx *c, double *div_max)
{
    if (!c) return TURB_ERR_ARG;
    launch_divergence(c->s, c->d, c->st[3], c->geo.mxc, c->geo.myc, c->geo.mzc, 1.0 / c->dEta, 1.0 / c->dXi,
                      1.0 / c->dPhi, c->ob, c->fld[TURB_F_U], c->fld[TURB_F_V], c->fld[TURB_F_W], c->fld[TURB_F_DIV],
                      c->part, c->dscal);
    c->launches += 2;
    int rc = check_launch(c);
    if (rc) return rc;
    if (div_max) {
        rc = fetch_scalars(c, 1);
        if (rc) return rc;
        *div_max = c->hscal[0];
        if (*div_max != *div_max) return TURB_ERR_NAN;   // the maximum keeps a NaN
    }
    return TURB_OK;
}

int turb_store_old_data(turb_ctx *c)
{
    if (!c) return TURB_ERR_ARG;
    size_t b = c->d.n * 8;
    for (int q = 0; q < 3; q++)
        TURB_CHECK(cudaMemcpyAsync(c->old[q], c->fld[TURB_F_U + q], b, cudaMemcpyDeviceToDevice, c->s));
    for (int ic = 0; ic < c->prm.nconc; ic++)
        TURB_CHECK(cudaMemcpyAsync(c->old[3 + ic], c->fld[TURB_F_C0 + ic], b, cudaMemcpyDeviceToDevice, c->s));
    return TURB_OK;
}

int turb_rk_average(turb_ctx *c, double old_frac, double new_frac)
{
    if (!c) return TURB_ERR_ARG;
    for (int q = 0; q < 3; q++) launch_axpby(c->s, c->d.n, old_frac, c->old[q], new_frac, c->fld[TURB_F_U + q]);
    for (int ic = 0; ic < c->prm.nconc; ic++)
        launch_axpby(c->s, c->d.n, old_frac, c->old[3 + ic], new_frac, c->fld[TURB_F_C0 + ic]);
    c->launches += 3 + c->prm.nconc;
    return check_launch(c);
}

// the old-data slot of a state field (u, v, w, c_i), -1 for others
static int old_slot(const turb_ctx *c, int field)
{
    if (field >= TURB_F_U && field <= TURB_F_W) return field - TURB_F_U;
    if (field >= TURB_F_C0 && field < TURB_F_C0 + c->prm.nconc) return 3 + field - TURB_F_C0;
    return -1;
}

int turb_store_old_field(turb_ctx *c, int field)
{
    if (!c) return TURB_ERR_ARG;
    int o = old_slot(c, field);
    if (o < 0) return TURB_ERR_ARG;
    TURB_CHECK(cudaMemcpyAsync(c->old[o], c->fld[field], c->d.n * 8, cudaMemcpyDeviceToDevice, c->s));
    return TURB_OK;
}

int turb_rk_average_field(turb_ctx *c, int field, double old_frac, double new_frac)
{
    if (!c) return TURB_ERR_ARG;
    int o = old_slot(c, field);
    if (o < 0) return TURB_ERR_ARG;
    launch_axpby(c->s, c->d.n, old_frac, c->old[o], new_frac, c->fld[field]);
    c->launches += 1;
    return check_launch(c);
}

int turb_profile_enable(turb_ctx *c, int on)
{
    if (!c) return TURB_ERR_ARG;
    prof_collect(c);
    for (int g = 0; g < TURB_PROF_NGROUPS; g++) { c->prof_ms[g] = 0.0; c->prof_nl[g] = 0; c->prof_bytes[g] = 0.0; }
    c->prof = on ? 1 : 0;
    return TURB_OK;
}

int turb_profile_read(turb_ctx *c, double *ms, long long *nlaunch)
{
    if (!c || !ms || !nlaunch) return TURB_ERR_ARG;
    prof_collect(c);
    for (int g = 0; g < TURB_PROF_NGROUPS; g++) { ms[g] = c->prof_ms[g]; nlaunch[g] = c->prof_nl[g]; }
    return TURB_OK;
}

int turb_profile_bytes(turb_ctx *c, double *bytes)
{
    if (!c || !bytes) return TURB_ERR_ARG;
    prof_collect(c);
    for (int g = 0; g < TURB_PROF_NGROUPS; g++) bytes[g] = c->prof_bytes[g];
    return TURB_OK;
}

int turb_event_record(turb_ctx *c, int slot)
{
    if (!c || slot < 0 || slot >= 8) return TURB_ERR_ARG;
    if (!c->user_ev[slot]) TURB_CHECK(cudaEventCreate(&c->user_ev[slot]));
    TURB_CHECK(cudaEventRecord(c->user_ev[slot], c->s));
    return TURB_OK;
}

int turb_event_elapsed(turb_ctx *c, int a, int b, double *ms)
{
    if (!c || !ms || a < 0 || b < 0 || a >= 8 || b >= 8 || !c->user_ev[a] || !c->user_ev[b]) return TURB_ERR_ARG;
    TURB_CHECK(cudaEventSynchronize(c->user_ev[b]));
    float f = 0.0f;
    TURB_CHECK(cudaEventElapsedTime(&f, c->user_ev[a], c->user_ev[b]));
    *ms = f;
    return TURB_OK;
}

int turb_kernel_launches(turb_ctx *c, long long *n)
{
    if (!c || !n) return TURB_ERR_ARG;
    *n = c->launches;
    return TURB_OK;
}

int turb_host_register(void *p, size_t bytes)
{
    if (!p || !bytes) return TURB_ERR_ARG;
    TURB_CHECK(cudaHostRegister(p, bytes, cudaHostRegisterDefault));
    return TURB_OK;
}

int turb_host_unregister(void *p)
{
    if (!p) return TURB_ERR_ARG;
    TURB_CHECK(cudaHostUnregister(p));
    return TURB_OK;
}

int turb_host_alloc(size_t bytes, void **out)
{
    if (!bytes || !out) return TURB_ERR_ARG;
    *out = nullptr;
    TURB_CHECK(cudaMallocHost(out, bytes));
    return TURB_OK;
}

int turb_host_free(void *p)
{
    if (!p) return TURB_ERR_ARG;
    TURB_CHECK(cudaFreeHost(p));
    return TURB_OK;
}

#define STEP_TRY(x)                      \
    do {                                 \
        int rc_ = (x);                   \
        if (rc_ != TURB_OK) return rc_;  \
    } while (0)

// turb_step_host: the fields the step reads late (the concentrations after
// the velocity convective terms, dpx, dpy, dpz at the velocity RHS, phi at
// the Poisson solve) are uploaded on a second stream while the step's first
// kernels run; the concentrations are downloaded on it once their RK average
// (right after the second stage's concentration solve) has written them,
// while the pressure solve runs, and dpx, dpy, dpz and phi once the second
// stage's projection has written them, while the last divergence check and
// the velocities' RK average run.  The step waits for them through these
// hooks; the copies beside the step use a kernel on a few SMs.
struct StepIo {
    std::vector<char> late;      // per field of the call: dpx, dpy, dpz, phi
    std::vector<char> conc;      // per field: c_i, moved with the late ones (no open boundaries)
    bool dp_wait = false, phi_wait = false, c_wait = false, out_started = false, c_out_started = false;
    int n = 0;
    const int *fields = nullptr;
    double *const *host = nullptr;
};

static bool late_field(int f)
{
    return f == TURB_F_DPX || f == TURB_F_DPY || f == TURB_F_DPZ || f == TURB_F_PHI;
}

static void step_io_before_rhs(turb_ctx *c)
{
    if (c->io->dp_wait) {
        cudaStreamWaitEvent(c->s, c->io_ev[1], 0);
        c->io->dp_wait = false;
    }
}

static void step_io_before_conc(turb_ctx *c)
{
    if (c->io->c_wait) {
        cudaStreamWaitEvent(c->s, c->io_ev[4], 0);
        c->io->c_wait = false;
    }
}

static void step_io_before_poisson(turb_ctx *c)
{
    if (c->io->phi_wait) {
        cudaStreamWaitEvent(c->s, c->io_ev[2], 0);
        c->io->phi_wait = false;
    }
}

static int step_io_after_conc_average(turb_ctx *c)
{
    StepIo &io = *c->io;
    bool any = false;
    for (int t = 0; t < io.n; t++) any = any || io.conc[t];
    if (!any) return TURB_OK;
    TURB_CHECK(cudaEventRecord(c->io_ev[0], c->s));   // the concentrations are final
    TURB_CHECK(cudaStreamWaitEvent(c->ios, c->io_ev[0], 0));
    for (int t = 0; t < io.n; t++)
        if (io.conc[t])
            launch_da_pitch_lean(c->ios, c->d, field_ptr(c, io.fields[t]), (double *)host_device_ptr(io.host[t]), 0);
    TURB_CHECK(cudaEventRecord(c->io_ev[5], c->ios));
    io.c_out_started = true;
    return check_launch(c);
}

static int step_io_after_projection(turb_ctx *c)
{
    StepIo &io = *c->io;
    TURB_CHECK(cudaEventRecord(c->io_ev[0], c->s));   // dpx, dpy, dpz, phi are final
    TURB_CHECK(cudaStreamWaitEvent(c->ios, c->io_ev[0], 0));
    for (int t = 0; t < io.n; t++)
        if (io.late[t])
            launch_da_pitch_lean(c->ios, c->d, field_ptr(c, io.fields[t]), (double *)host_device_ptr(io.host[t]), 0);
    TURB_CHECK(cudaEventRecord(c->io_ev[3], c->ios));
    io.out_started = true;
    return check_launch(c);
}

static int step_impl(turb_ctx *c, double dt, turb_step_stats *st);

int turb_step(turb_ctx *c, double dt, turb_step_stats *st)
{
    if (!c || !(dt > 0.0)) return TURB_ERR_ARG;
    return step_impl(c, dt, st);
}

static int step_impl(turb_ctx *c, double dt, turb_step_stats *st)
{
    if (!c || !(dt > 0.0)) return TURB_ERR_ARG;
    turb_step_stats local;
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    long long l0 = c->launches;
    // open faces (restated driver order): inflow planes at the step's time,
    // outflow planes stored, advanced by the convective condition at the
    // start of every stage and RK-averaged with the fields
    if (c->ob.in) {
        STEP_TRY(turb_Inflow_u_velocity_profile(c, c->time, nullptr));
        for (int ic = 0; ic < c->prm.nconc; ic++) STEP_TRY(turb_Inflow_conc_profile(c, ic, c->time));
    }
    if (c->ob.out) STEP_TRY(turb_store_old_outflow(c));
    // the old data of the velocities now, of the concentrations once the
    // velocity convective terms are queued (nothing reads the concentrations
    // before that, so a host copy of them can still be in flight)
    for (int q = 0; q < 3; q++) STEP_TRY(turb_store_old_field(c, TURB_F_U + q));
    for (int stage = 0; stage < 2; stage++) {
        c->stage = stage;
        if (c->ob.out) STEP_TRY(turb_Outflow_impose_convective_boundary(c, dt));
        STEP_TRY(turb_Velocity_cell_center(c));
        STEP_TRY(turb_Velocity_convective_terms(c, 'u'));
        STEP_TRY(turb_Velocity_convective_terms(c, 'v'));
        STEP_TRY(turb_Velocity_convective_terms(c, 'w'));
        if (stage == 0) {
            if (c->io) step_io_before_conc(c);
            for (int ic = 0; ic < c->prm.nconc; ic++) STEP_TRY(turb_store_old_field(c, TURB_F_C0 + ic));
        }
        if (c->prm.nconc > 1) STEP_TRY(turb_Conc_compute_total_concentration(c));
        for (int ic = 0; ic < c->prm.nconc; ic++) STEP_TRY(turb_Conc_convective_terms(c, ic));
        if (c->io) step_io_before_rhs(c);
        STEP_TRY(turb_Velocity_set_RHS(c, 'u', dt));
        STEP_TRY(turb_Velocity_set_RHS(c, 'v', dt));
        STEP_TRY(turb_Velocity_set_RHS(c, 'w', dt));
        STEP_TRY(turb_Velocity_solve(c, 'u', dt, &st->vel_iters[0][stage]));
        STEP_TRY(turb_Velocity_solve(c, 'v', dt, &st->vel_iters[1][stage]));
        STEP_TRY(turb_Velocity_solve(c, 'w', dt, &st->vel_iters[2][stage]));
        for (int ic = 0; ic < c->prm.nconc; ic++) {
            STEP_TRY(turb_Conc_set_RHS(c, ic, dt));
            STEP_TRY(turb_Conc_solve(c, ic, dt, &st->conc_iters[ic][stage]));
        }
        if (stage == 1) {   // the concentrations are final: their RK average now (nothing after reads them)
            for (int ic = 0; ic < c->prm.nconc; ic++) STEP_TRY(turb_rk_average_field(c, TURB_F_C0 + ic, 0.5, 0.5));
            if (c->io) STEP_TRY(step_io_after_conc_average(c));
        }
        STEP_TRY(turb_Pressure_set_RHS(c, dt));
        if (c->io) step_io_before_poisson(c);
        STEP_TRY(turb_Pressure_solve(c, &st->p_iters[stage], &st->p_relres[stage]));
        STEP_TRY(turb_Pressure_project_velocity(c, dt));
        if (c->io && stage == 1) STEP_TRY(step_io_after_projection(c));
        STEP_TRY(turb_Pressure_compute_velocity_divergence(c, &st->div_max[stage]));
    }
    for (int q = 0; q < 3; q++) STEP_TRY(turb_rk_average_field(c, TURB_F_U + q, 0.5, 0.5));
    if (c->ob.out) STEP_TRY(turb_rk_average_outflow(c, 0.5, 0.5));
    if (c->deposit_on) STEP_TRY(turb_deposit_integrate(c, dt));
    c->time += dt;
    st->kernel_launches = (int)(c->launches - l0);
    return TURB_OK;
}

int turb_step_host(turb_ctx *c, double dt, int n, const int *fields, double *const *host, turb_step_stats *st)
{
    if (!c || !(dt > 0.0) || n < 0 || (n > 0 && (!fields || !host))) return TURB_ERR_ARG;
    bool direct = c->host_copy == TURB_HOST_COPY_KERNEL;
    for (int t = 0; t < n; t++) {
        if (!field_ptr(c, fields[t]) || !host[t]) return TURB_ERR_ARG;
        direct = direct && host_device_ptr(host[t]) != nullptr;
    }
    if (!direct) {   // the calls it stands for, one after the other
        int rc = turb_fields_upload(c, n, fields, host);
        if (rc) return rc;
        rc = step_impl(c, dt, st);
        if (rc) return rc;
        return turb_fields_download(c, n, fields, host);
    }
    if (!c->ios) TURB_CHECK(cudaStreamCreateWithFlags(&c->ios, cudaStreamNonBlocking));
    for (auto &e : c->io_ev)
        if (!e) TURB_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    StepIo io;
    io.n = n;
    io.fields = fields;
    io.host = host;
    io.late.resize(n);
    io.conc.resize(n);
    // the open faces set concentrations at the step's start and average
    // the outflow planes at its end: then the concentrations move with u, v, w
    const bool open = c->ob.in || c->ob.out;
    for (int t = 0; t < n; t++) {
        io.late[t] = late_field(fields[t]) ? 1 : 0;
        io.conc[t] = (!open && fields[t] >= TURB_F_C0 && fields[t] < TURB_F_C0 + c->prm.nconc) ? 1 : 0;
    }
    for (int t = 0; t < n; t++)
        if (!io.late[t] && !io.conc[t])
            launch_da_pitch(c->s, c->d, (const double *)host_device_ptr(host[t]), field_ptr(c, fields[t]), 1);
    // the late copies start when the early ones have landed (they share the
    // host link, and the step waits for the early ones) and after the work
    // already on the context's stream, which may still use the fields
    TURB_CHECK(cudaEventRecord(c->io_ev[0], c->s));
    TURB_CHECK(cudaStreamWaitEvent(c->ios, c->io_ev[0], 0));
    // in the order the step reads them: c_i, then dpx, dpy, dpz, then phi
    for (int pass = 0; pass < 3; pass++) {
        bool any = false;
        for (int t = 0; t < n; t++) {
            if (!io.late[t] && !io.conc[t]) continue;
            const int kind = io.late[t] ? (fields[t] == TURB_F_PHI ? 2 : 1) : 0;
            if (kind != pass) continue;
            launch_da_pitch_lean(c->ios, c->d, (const double *)host_device_ptr(host[t]), field_ptr(c, fields[t]), 1);
            any = true;
        }
        if (any) {
            TURB_CHECK(cudaEventRecord(c->io_ev[pass == 0 ? 4 : pass], c->ios));
            (pass == 0 ? io.c_wait : pass == 1 ? io.dp_wait : io.phi_wait) = true;
        }
    }
    int rc = check_launch(c);
    if (rc) return rc;
    c->io = &io;
    rc = step_impl(c, dt, st);
    c->io = nullptr;
    if (rc) {
        cudaStreamSynchronize(c->ios);
        return rc;
    }
    // a stage that returned early never waited: the context's stream waits now
    if (io.c_wait) TURB_CHECK(cudaStreamWaitEvent(c->s, c->io_ev[4], 0));
    if (io.dp_wait) TURB_CHECK(cudaStreamWaitEvent(c->s, c->io_ev[1], 0));
    if (io.phi_wait) TURB_CHECK(cudaStreamWaitEvent(c->s, c->io_ev[2], 0));
    for (int t = 0; t < n; t++) {
        const bool done = (io.late[t] && io.out_started) || (io.conc[t] && io.c_out_started);
        if (!done) launch_da_pitch(c->s, c->d, field_ptr(c, fields[t]), (double *)host_device_ptr(host[t]), 0);
    }
    if (io.out_started) TURB_CHECK(cudaStreamWaitEvent(c->s, c->io_ev[3], 0));
    if (io.c_out_started) TURB_CHECK(cudaStreamWaitEvent(c->s, c->io_ev[5], 0));
    rc = check_launch(c);
    if (rc) return rc;
    TURB_CHECK(cudaStreamSynchronize(c->s));
    TURB_CHECK(cudaStreamSynchronize(c->ios));
    return TURB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// unweighted pressure operator (Pressure_form_LHS_matrix rows), for parity
// tests of the operator the MG-CG solves
// ---------------------------------------------------------------------------
namespace {
__global__ void k_pressure_apply(Dims d, const uint8_t *__restrict__ st, Geo g, double dEta, double dXi, double dPhi,
                                 const double *__restrict__ x, double *__restrict__ y)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    if (i >= d.NX || j >= d.NY) return;
    long long p = d.at(i, j, k);
    double Cx = -1.0 / (dEta * dEta), Cy = -1.0 / (dXi * dXi), Cz = -1.0 / (dPhi * dPhi);
    if (st[p] == T_BOUNDARY) {
        double aps = -Cx * g.mxc[0] - Cy * g.myc[0] - Cz * g.mzc[0];
        y[p] = aps * x[p];
        return;
    }
    int NI = d.nx, NJ = d.ny, NK = d.nz;
    double px = g.mxc[i], py = g.myc[j], pz = g.mzc[k];
    double ex = g.mxu[i + 1], wx = g.mxu[i], ny_ = g.myv[j + 1], sy = g.myv[j], fz = g.mzw[k + 1], bz = g.mzw[k];
    double ap = -Cx * px * (ex + wx) - Cy * py * (ny_ + sy) - Cz * pz * (bz + fz);
    double aw = Cx * px * wx, ae = Cx * px * ex, an = Cy * py * ny_, as = Cy * py * sy, ab = Cz * pz * bz,
           af = Cz * pz * fz, acc = 0.0;
    if (k > 0) acc += ab * x[p - d.plane]; else ap += ab;
    if (j > 0) acc += as * x[p - d.PX]; else ap += as;
    if (i > 0) acc += aw * x[p - 1]; else ap += aw;
    if (i < NI - 1) acc += ae * x[p + 1];
    else if (!(i == NI - 1 && j == NJ - 1 && k == NK - 1)) ap += ae;
    if (j < NJ - 1) acc += an * x[p + d.PX]; else ap += an;
    if (k < NK - 1) acc += af * x[p + d.plane]; else ap += af;
    y[p] = acc + ap * x[p];
}
}  // namespace

void launch_pressure_apply(cudaStream_t s, const Dims &d, const uint8_t *st, const Geo &g, double dEta, double dXi,
                           double dPhi, const double *x, double *y)
{
    k_pressure_apply<<<dim3((d.NX + 31) / 32, (d.NY + 7) / 8, d.NZ), dim3(32, 8), 0, s>>>(d, st, g, dEta, dXi, dPhi, x, y);
}

// contiguous DA array <-> pitched field (pad columns untouched)
__global__ void k_da_pitch(Dims d, const double *__restrict__ src, double *__restrict__ dst, int to_pitched)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= d.NX) return;
    long long c = ((long long)k * d.NY + j) * d.NX + i, p = d.at(i, j, k);
    if (to_pitched) dst[p] = src[c];
    else dst[c] = src[p];
}

// The same conversion from a few SMs only, for copies that run beside the
// step's kernels: a grid-stride loop over the DA array, four elements in
// flight per thread (the host link's latency wants many loads in flight, the
// step wants its SMs)
constexpr int DA_LEAN_BLOCKS = 16, DA_LEAN_THREADS = 1024;
__global__ void __launch_bounds__(DA_LEAN_THREADS) k_da_pitch_lean(Dims d, const double *__restrict__ src,
                                                                  double *__restrict__ dst, int to_pitched)
{
    const long long n = (long long)d.NX * d.NY * d.NZ;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; c0 < n; c0 += 4 * stride) {
        double v[4];
        long long at[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const long long c = c0 + u * stride;
            if (c < n) {
                const long long row = c / d.NX;
                const long long p = row * d.PX + (c - row * d.NX);
                at[u] = to_pitched ? p : c;
                v[u] = src[to_pitched ? c : p];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (c0 + u * stride < n) dst[at[u]] = v[u];
    }
}

void launch_da_pitch_lean(cudaStream_t s, const Dims &d, const double *src, double *dst, int to_pitched)
{
    k_da_pitch_lean<<<DA_LEAN_BLOCKS, DA_LEAN_THREADS, 0, s>>>(d, src, dst, to_pitched);
}

void launch_da_pitch(cudaStream_t s, const Dims &d, const double *src, double *dst, int to_pitched)
{
    k_da_pitch<<<dim3((unsigned)((d.NX + 127) / 128), (unsigned)d.NY, (unsigned)d.NZ), 128, 0, s>>>(d, src, dst,
                                                                                                   to_pitched);
}
