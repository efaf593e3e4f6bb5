/*
 * shim.c -- single-rank implementation of the PETSc/MPI subset declared in
 * petsc.h (TEST INFRASTRUCTURE ONLY; see petsc.h).
 */
#include "petsc.h"
#include <stdarg.h>
#include <stdint.h>
#include <string.h>

struct _p_DA { int M, N, P; };
struct _p_Vec { double *a; long n; double ***arr; int M, N, P; };
typedef struct { int col; double v; } shim_ent;
typedef struct { int n, cap; shim_ent *e; } shim_row;
struct _p_Mat { int M, N, P; long nr; shim_row *rows; };
struct _p_KSP { Mat A; double rtol; int maxit, its; KSPConvergedReason reason; int nonzero; int direct; };
struct _p_PC { int dummy; };
struct _p_Viewer { FILE *f; int mode; };
struct _p_NullSpace { int dummy; };

static int g_verbose = -1;

int PetscPrintf(MPI_Comm comm, const char *fmt, ...)
{
    va_list ap;
    (void)comm;
    if (g_verbose < 0) g_verbose = getenv("TURB_REF_VERBOSE") != NULL;
    if (!g_verbose) return 0;
    va_start(ap, fmt);
    vprintf(fmt, ap);
    va_end(ap);
    return 0;
}

int PetscError(int line, const char *func, const char *file, const char *dir, int n, int p, const char *mess, ...)
{
    (void)dir; (void)p; (void)mess;
    fprintf(stderr, "shim PetscError %d in %s (%s:%d)\n", n, func, file, line);
    return n;
}
int PetscFinalize(void) { return 0; }
int PetscGetTime(PetscLogDouble *t) { *t = 0.0; return 0; }
int PetscMallocGetCurrentUsage(PetscLogDouble *m) { *m = 0.0; return 0; }
int PetscOptionsSetValue(const char *a, const char *b) { (void)a; (void)b; return 0; }
int PetscMalloc(size_t n, void **p) { *p = malloc(n); return *p == NULL; }

static size_t dsize(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : sizeof(double); }
int MPI_Allreduce(void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
    (void)op; (void)c;
    memmove(r, s, (size_t)n * dsize(t));
    return 0;
}
int MPI_Reduce(void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{
    (void)root;
    return MPI_Allreduce(s, r, n, t, op, c);
}
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *r) { (void)c; *r = 1; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }

/* ---- DA ----------------------------------------------------------------- */
int DACreate3d(MPI_Comm c, DAPeriodicType p, DAStencilType st, int M, int N, int P, int m, int n, int pp,
               int dof, int s, const int *lx, const int *ly, const int *lz, DA *da)
{
    (void)c; (void)p; (void)st; (void)m; (void)n; (void)pp; (void)dof; (void)s; (void)lx; (void)ly; (void)lz;
    *da = (DA)calloc(1, sizeof(struct _p_DA));
    (*da)->M = M; (*da)->N = N; (*da)->P = P;
    return 0;
}
int DADestroy(DA da) { free(da); return 0; }
int DAView(DA da, PetscViewer v) { (void)da; (void)v; return 0; }

static Vec new_vec(int M, int N, int P)
{
    Vec v = (Vec)calloc(1, sizeof(struct _p_Vec));
    v->M = M; v->N = N; v->P = P;
    v->n = (long)M * N * P;
    v->a = (double *)calloc((size_t)v->n, sizeof(double));
    return v;
}
int DACreateGlobalVector(DA da, Vec *v) { *v = new_vec(da->M, da->N, da->P); return 0; }
int DACreateLocalVector(DA da, Vec *v) { *v = new_vec(da->M, da->N, da->P); return 0; }
int DAGetCorners(DA da, int *x, int *y, int *z, int *m, int *n, int *p)
{
    if (x) *x = 0;
    if (y) *y = 0;
    if (z) *z = 0;
    if (m) *m = da->M;
    if (n) *n = da->N;
    if (p) *p = da->P;
    return 0;
}
int DAGetGhostCorners(DA da, int *x, int *y, int *z, int *m, int *n, int *p) { return DAGetCorners(da, x, y, z, m, n, p); }
int DAGetGlobalIndices(DA da, int *n, int **idx)
{
    static int *ids = NULL;
    static long nids = 0;
    long t, nt = (long)da->M * da->N * da->P;
    if (nt > nids) {
        free(ids);
        ids = (int *)malloc(sizeof(int) * (size_t)nt);
        for (t = 0; t < nt; t++) ids[t] = (int)t;
        nids = nt;
    }
    *n = (int)nt;
    *idx = ids;
    return 0;
}
int DAGetInfo(DA da, int *dim, int *M, int *N, int *P, int *m, int *n, int *p, int *dof, int *s,
              DAPeriodicType *wrap, DAStencilType *st)
{
    if (dim) *dim = 3;
    if (M) *M = da->M;
    if (N) *N = da->N;
    if (P) *P = da->P;
    if (m) *m = 1;
    if (n) *n = 1;
    if (p) *p = 1;
    if (dof) *dof = 1;
    if (s) *s = 1;
    if (wrap) *wrap = DA_NONPERIODIC;
    if (st) *st = DA_STENCIL_STAR;
    return 0;
}
int DAGetOwnershipRanges(DA da, const int **lx, const int **ly, const int **lz)
{
    (void)da; (void)lx; (void)ly; (void)lz;
    return 0;
}
int DAGetMatrix(DA da, MatType t, Mat *A)
{
    Mat m = (Mat)calloc(1, sizeof(struct _p_Mat));
    (void)t;
    m->M = da->M; m->N = da->N; m->P = da->P;
    m->nr = (long)da->M * da->N * da->P;
    m->rows = (shim_row *)calloc((size_t)m->nr, sizeof(shim_row));
    *A = m;
    return 0;
}
int DAVecGetArray(DA da, Vec v, void *array)
{
    (void)da;
    if (!v->arr) {
        int k, j;
        v->arr = (double ***)malloc(sizeof(double **) * (size_t)v->P);
        for (k = 0; k < v->P; k++) {
            v->arr[k] = (double **)malloc(sizeof(double *) * (size_t)v->N);
            for (j = 0; j < v->N; j++) v->arr[k][j] = v->a + ((long)k * v->N + j) * v->M;
        }
    }
    *(double ****)array = v->arr;
    return 0;
}
int DAVecRestoreArray(DA da, Vec v, void *array) { (void)da; (void)v; (void)array; return 0; }
/* contiguous storage of a (single-rank) vector, DA order */
int VecGetArray(Vec v, PetscScalar **a) { *a = v->a; return 0; }
int VecRestoreArray(Vec v, PetscScalar **a) { (void)v; if (a) *a = NULL; return 0; }
int VecGetSize(Vec v, PetscInt *n) { *n = (PetscInt)v->n; return 0; }
int DAGlobalToLocalBegin(DA da, Vec g, InsertMode mode, Vec l)
{
    long t;
    (void)da;
    if (g == l) return 0;
    if (mode == ADD_VALUES) for (t = 0; t < g->n; t++) l->a[t] += g->a[t];
    else memcpy(l->a, g->a, sizeof(double) * (size_t)g->n);
    return 0;
}
int DAGlobalToLocalEnd(DA da, Vec g, InsertMode mode, Vec l) { (void)da; (void)g; (void)mode; (void)l; return 0; }

/* ---- Vec ---------------------------------------------------------------- */
int VecDuplicate(Vec v, Vec *n) { *n = new_vec(v->M, v->N, v->P); return 0; }
int VecDestroy(Vec v)
{
    if (!v) return 0;
    if (v->arr) {
        int k;
        for (k = 0; k < v->P; k++) free(v->arr[k]);
        free(v->arr);
    }
    free(v->a);
    free(v);
    return 0;
}
int VecCopy(Vec x, Vec y) { memcpy(y->a, x->a, sizeof(double) * (size_t)x->n); return 0; }
int VecAXPBY(Vec y, PetscScalar a, PetscScalar b, Vec x)
{
    long t;
    for (t = 0; t < y->n; t++) y->a[t] = a * x->a[t] + b * y->a[t];
    return 0;
}
int VecAXPY(Vec y, PetscScalar a, Vec x)
{
    long t;
    for (t = 0; t < y->n; t++) y->a[t] = y->a[t] + a * x->a[t];
    return 0;
}
int VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y)
{
    long t;
    for (t = 0; t < w->n; t++) w->a[t] = a * x->a[t] + y->a[t];
    return 0;
}
int VecScale(Vec x, PetscScalar a)
{
    long t;
    for (t = 0; t < x->n; t++) x->a[t] *= a;
    return 0;
}
int VecShift(Vec x, PetscScalar a)
{
    long t;
    for (t = 0; t < x->n; t++) x->a[t] += a;
    return 0;
}
int VecSet(Vec x, PetscScalar a)
{
    long t;
    for (t = 0; t < x->n; t++) x->a[t] = a;
    return 0;
}
int VecSum(Vec x, PetscScalar *s)
{
    long t;
    double acc = 0.0;
    for (t = 0; t < x->n; t++) acc += x->a[t];
    *s = acc;
    return 0;
}
/* PETSc binary vector files (PETSc 3.1, VecView_Seq_Binary and
 * VecLoadIntoVector_Binary): the int32 pair {VEC_FILE_COOKIE = 1211214, N}
 * followed by the N doubles, every word big-endian.  On one rank a DA
 * vector's natural order is its storage order. */
#define SHIM_VEC_COOKIE 1211214
static int put_be(FILE *f, const void *w, int size)
{
    unsigned char b[8];
    int i;
    uint64_t x = 0;
    if (size == 4) { uint32_t y; memcpy(&y, w, 4); x = y; } else memcpy(&x, w, 8);
    for (i = 0; i < size; i++) b[i] = (unsigned char)(x >> (8 * (size - 1 - i)));
    return fwrite(b, 1, (size_t)size, f) == (size_t)size ? 0 : 1;
}
static int get_be(FILE *f, void *w, int size)
{
    unsigned char b[8];
    int i;
    uint64_t x = 0;
    if (fread(b, 1, (size_t)size, f) != (size_t)size) return 1;
    for (i = 0; i < size; i++) x = (x << 8) | b[i];
    if (size == 4) { uint32_t y = (uint32_t)x; memcpy(w, &y, 4); } else memcpy(w, &x, 8);
    return 0;
}
int VecView(Vec x, PetscViewer v)
{
    int32_t hdr[2];
    long t;
    int bad = 0;
    if (!v || !v->f || v->mode != FILE_MODE_WRITE) return 0;
    hdr[0] = SHIM_VEC_COOKIE;
    hdr[1] = (int32_t)x->n;
    bad |= put_be(v->f, &hdr[0], 4) | put_be(v->f, &hdr[1], 4);
    for (t = 0; t < x->n; t++) bad |= put_be(v->f, &x->a[t], 8);
    return bad;
}
int VecLoadIntoVector(PetscViewer v, Vec x)
{
    int32_t hdr[2];
    long t;
    if (!v || !v->f || v->mode != FILE_MODE_READ) return 1;
    if (get_be(v->f, &hdr[0], 4) || get_be(v->f, &hdr[1], 4)) return 1;
    if (hdr[0] != SHIM_VEC_COOKIE || hdr[1] != x->n) return 1;
    for (t = 0; t < x->n; t++)
        if (get_be(v->f, &x->a[t], 8)) return 1;
    return 0;
}
int VecCreate(MPI_Comm c, Vec *v) { (void)c; *v = new_vec(0, 1, 1); return 0; }
int VecSetSizes(Vec v, int n, int N)
{
    long m = N > 0 ? N : n;
    free(v->a);
    v->M = (int)m; v->N = 1; v->P = 1; v->n = m;
    v->a = (double *)calloc((size_t)m, sizeof(double));
    return 0;
}
int VecSetFromOptions(Vec v) { (void)v; return 0; }

double *shim_vec_data(Vec v) { return v->a; }
long shim_vec_size(Vec v) { return v->n; }

/* ---- Mat ---------------------------------------------------------------- */
static void row_set(shim_row *r, int col, double v, InsertMode mode)
{
    int t;
    for (t = 0; t < r->n; t++)
        if (r->e[t].col == col) {
            if (mode == ADD_VALUES) r->e[t].v += v;
            else r->e[t].v = v;
            return;
        }
    if (r->n == r->cap) {
        r->cap = r->cap ? 2 * r->cap : 8;
        r->e = (shim_ent *)realloc(r->e, sizeof(shim_ent) * (size_t)r->cap);
    }
    r->e[r->n].col = col;
    r->e[r->n].v = v;
    r->n++;
}
static int sidx(Mat A, const MatStencil *s) { return (s->k * A->N + s->j) * A->M + s->i; }
int MatSetValuesStencil(Mat A, int m, const MatStencil *rows, int n, const MatStencil *cols,
                        const PetscScalar *v, InsertMode mode)
{
    int a, b;
    for (a = 0; a < m; a++) {
        shim_row *r = &A->rows[sidx(A, &rows[a])];
        for (b = 0; b < n; b++) row_set(r, sidx(A, &cols[b]), v[a * n + b], mode);
    }
    return 0;
}
int MatSetValues(Mat A, int m, const int *rows, int n, const int *cols, const PetscScalar *v, InsertMode mode)
{
    int a, b;
    for (a = 0; a < m; a++) {
        shim_row *r = &A->rows[rows[a]];
        for (b = 0; b < n; b++) row_set(r, cols[b], v[a * n + b], mode);
    }
    return 0;
}
int MatAssemblyBegin(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
int MatAssemblyEnd(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
int MatDiagonalSet(Mat A, Vec d, InsertMode mode)
{
    long t;
    for (t = 0; t < A->nr; t++) row_set(&A->rows[t], (int)t, d->a[t], mode);
    return 0;
}
int MatDestroy(Mat A)
{
    long t;
    if (!A) return 0;
    for (t = 0; t < A->nr; t++) free(A->rows[t].e);
    free(A->rows);
    free(A);
    return 0;
}
int MatCreate(MPI_Comm c, Mat *A) { (void)c; *A = NULL; return 0; }
int MatSetSizes(Mat A, int m, int n, int M, int N) { (void)A; (void)m; (void)n; (void)M; (void)N; return 0; }
int MatSetType(Mat A, MatType t) { (void)A; (void)t; return 0; }
int MatSetFromOptions(Mat A) { (void)A; return 0; }
int MatLoad(PetscViewer v, MatType t, Mat *A) { (void)v; (void)t; (void)A; return 1; }
int MatNullSpaceCreate(MPI_Comm c, PetscTruth has, int n, const Vec *v, MatNullSpace *sp)
{
    (void)c; (void)has; (void)n; (void)v;
    *sp = NULL;
    return 0;
}
int MatNullSpaceDestroy(MatNullSpace sp) { (void)sp; return 0; }

/* y = A x; row entries summed in column order (assembled CSR order) */
static int cmp_ent(const void *a, const void *b)
{
    int x = ((const shim_ent *)a)->col, y = ((const shim_ent *)b)->col;
    return (x > y) - (x < y);
}
int shim_mat_mult(Mat A, const double *x, double *y)
{
    long t;
    for (t = 0; t < A->nr; t++) {
        shim_row *r = &A->rows[t];
        double s = 0.0;
        int e;
        qsort(r->e, (size_t)r->n, sizeof(shim_ent), cmp_ent);
        for (e = 0; e < r->n; e++) s += r->e[e].v * x[r->e[e].col];
        y[t] = s;
    }
    return 0;
}

/* ---- KSP: unpreconditioned BiCGStab, ||r|| <= rtol ||b|| ---------------- */
int KSPCreate(MPI_Comm c, KSP *k)
{
    (void)c;
    *k = (KSP)calloc(1, sizeof(struct _p_KSP));
    (*k)->rtol = 1e-5;
    (*k)->maxit = 10000;
    return 0;
}
int KSPSetOperators(KSP k, Mat A, Mat P, MatStructure s) { (void)P; (void)s; k->A = A; return 0; }
/* KSPGMRES is the pressure solver's type (GMRES(20) + BoomerAMG in the
 * reference); the shim solves that system directly (banded LU), so the
 * harness returns the exact discrete solution.  Other types: BiCGStab. */
int KSPSetType(KSP k, KSPType t) { k->direct = strcmp(t, KSPGMRES) == 0; return 0; }
int KSPSetTolerances(KSP k, PetscReal rtol, PetscReal atol, PetscReal dtol, int maxits)
{
    (void)atol; (void)dtol;
    if (rtol != PETSC_DEFAULT) k->rtol = rtol;
    if (maxits != PETSC_DEFAULT) k->maxit = maxits;
    return 0;
}
int KSPGetPC(KSP k, PC *pc) { (void)k; static struct _p_PC p; *pc = &p; return 0; }
int KSPSetUp(KSP k) { (void)k; return 0; }
static double vdot(long n, const double *a, const double *b)
{
    long t;
    double s = 0.0;
    for (t = 0; t < n; t++) s += a[t] * b[t];
    return s;
}
/* banded LU without pivoting (the pressure matrix is an M-matrix with a
 * pinned corner), bandwidth from the assembled rows, followed by two steps
 * of iterative refinement */
static int shim_band_solve(Mat A, const double *b, double *x)
{
    long n = A->nr, t, c, r;
    long bw = 0;
    double *L, *res, *dx;
    for (t = 0; t < n; t++) {
        int e;
        for (e = 0; e < A->rows[t].n; e++) {
            long d = labs((long)A->rows[t].e[e].col - t);
            if (d > bw) bw = d;
        }
    }
    {
        long W = 2 * bw + 1;
        int pass;
        L = calloc((size_t)n * W, sizeof(double));
        if (!L) return 1;
#define BAND(i, j) L[(size_t)(i) * W + ((j) - (i) + bw)]
        for (t = 0; t < n; t++) {
            int e;
            for (e = 0; e < A->rows[t].n; e++) BAND(t, A->rows[t].e[e].col) += A->rows[t].e[e].v;
        }
        for (c = 0; c < n; c++) {
            double piv = BAND(c, c);
            long rmax = c + bw < n - 1 ? c + bw : n - 1;
            for (r = c + 1; r <= rmax; r++) {
                double f = BAND(r, c);
                long cm;
                if (f == 0.0) continue;
                f /= piv;
                BAND(r, c) = f;
                for (cm = c + 1; cm <= rmax; cm++) BAND(r, cm) -= f * BAND(c, cm);
            }
        }
        res = malloc(sizeof(double) * n);
        dx = malloc(sizeof(double) * n);
        memset(x, 0, sizeof(double) * n);
        for (pass = 0; pass < 3; pass++) {
            shim_mat_mult(A, x, res);
            for (t = 0; t < n; t++) res[t] = b[t] - res[t];
            for (t = 0; t < n; t++) {   /* forward: L y = res */
                double s = res[t];
                long c0 = t - bw > 0 ? t - bw : 0;
                for (c = c0; c < t; c++) s -= BAND(t, c) * dx[c];
                dx[t] = s;
            }
            for (t = n - 1; t >= 0; t--) {   /* backward: U dx = y */
                double s = dx[t];
                long c1 = t + bw < n - 1 ? t + bw : n - 1;
                for (c = t + 1; c <= c1; c++) s -= BAND(t, c) * dx[c];
                dx[t] = s / BAND(t, t);
            }
            for (t = 0; t < n; t++) x[t] += dx[t];
        }
#undef BAND
    }
    free(L); free(res); free(dx);
    return 0;
}

int KSPSolve(KSP k, Vec bv, Vec xv)
{
    if (k->direct) {
        int rc = shim_band_solve(k->A, bv->a, xv->a);
        k->its = 1;
        k->reason = rc ? KSP_DIVERGED_BREAKDOWN : KSP_CONVERGED_RTOL;
        return 0;
    }
    {
    long n = bv->n, t;
    double *b = bv->a, *x = xv->a;
    double *r = malloc(sizeof(double) * n), *rh = malloc(sizeof(double) * n), *p = calloc(n, sizeof(double));
    double *v = calloc(n, sizeof(double)), *s = malloc(sizeof(double) * n), *tt = malloc(sizeof(double) * n);
    double rho = 1.0, alpha = 1.0, omega = 1.0, nb, nr;
    int it = 0;
    if (!k->nonzero) memset(x, 0, sizeof(double) * n);
    shim_mat_mult(k->A, x, r);
    for (t = 0; t < n; t++) r[t] = b[t] - r[t];
    memcpy(rh, r, sizeof(double) * n);
    nb = sqrt(vdot(n, b, b));
    nr = sqrt(vdot(n, r, r));
    k->reason = KSP_CONVERGED_RTOL;
    while (nr > k->rtol * nb) {
        double rho1, beta, ts;
        if (it >= k->maxit) { k->reason = KSP_DIVERGED_ITS; break; }
        rho1 = vdot(n, rh, r);
        if (rho1 == 0.0) { k->reason = KSP_DIVERGED_BREAKDOWN; break; }
        beta = (rho1 / rho) * (alpha / omega);
        for (t = 0; t < n; t++) p[t] = r[t] + beta * (p[t] - omega * v[t]);
        shim_mat_mult(k->A, p, v);
        alpha = rho1 / vdot(n, rh, v);
        for (t = 0; t < n; t++) s[t] = r[t] - alpha * v[t];
        shim_mat_mult(k->A, s, tt);
        ts = vdot(n, tt, tt);
        omega = ts > 0.0 ? vdot(n, tt, s) / ts : 0.0;
        for (t = 0; t < n; t++) { x[t] += alpha * p[t] + omega * s[t]; r[t] = s[t] - omega * tt[t]; }
        rho = rho1;
        nr = sqrt(vdot(n, r, r));
        it++;
        if (omega == 0.0) { k->reason = KSP_DIVERGED_BREAKDOWN; break; }
    }
    k->its = it;
    free(r); free(rh); free(p); free(v); free(s); free(tt);
    return 0;
    }
}
int KSPGetIterationNumber(KSP k, int *its) { *its = k->its; return 0; }
int KSPGetConvergedReason(KSP k, KSPConvergedReason *r) { *r = k->reason; return 0; }
int KSPSetInitialGuessNonzero(KSP k, PetscTruth t) { k->nonzero = t; return 0; }
int KSPSetFromOptions(KSP k) { (void)k; return 0; }
int KSPDestroy(KSP k) { free(k); return 0; }
int KSPView(KSP k, PetscViewer v) { (void)k; (void)v; return 0; }
int KSPGMRESSetRestart(KSP k, int r) { (void)k; (void)r; return 0; }
int KSPSetNullSpace(KSP k, MatNullSpace sp) { (void)k; (void)sp; return 0; }
int PCSetType(PC pc, PCType t) { (void)pc; (void)t; return 0; }
int PCHYPRESetType(PC pc, const char *t) { (void)pc; (void)t; return 0; }
int PCFactorSetLevels(PC pc, int l) { (void)pc; (void)l; return 0; }
int PCFactorSetReuseOrdering(PC pc, PetscTruth t) { (void)pc; (void)t; return 0; }
int PCFactorSetReuseFill(PC pc, PetscTruth t) { (void)pc; (void)t; return 0; }
int PCFactorSetAllowDiagonalFill(PC pc) { (void)pc; return 0; }
int PCFactorSetUseInPlace(PC pc) { (void)pc; return 0; }
int PCFactorSetFill(PC pc, PetscReal f) { (void)pc; (void)f; return 0; }
int PCFactorSetUseDropTolerance(PC pc, PetscReal a, PetscReal b, int c) { (void)pc; (void)a; (void)b; (void)c; return 0; }
int PetscViewerBinaryOpen(MPI_Comm c, const char *name, PetscFileMode m, PetscViewer *v)
{
    FILE *f = fopen(name, m == FILE_MODE_WRITE ? "wb" : "rb");
    (void)c;
    *v = NULL;
    if (!f) return 1;
    *v = (PetscViewer)calloc(1, sizeof(struct _p_Viewer));
    (*v)->f = f;
    (*v)->mode = m;
    return 0;
}
int PetscViewerDestroy(PetscViewer v)
{
    if (v) {
        if (v->f) fclose(v->f);
        free(v);
    }
    return 0;
}
