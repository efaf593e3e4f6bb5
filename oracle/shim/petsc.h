/*
 * Single-rank stand-in for the PETSc 3.1 / MPI entry points that the
 * reference's hot-path C files call (TEST INFRASTRUCTURE ONLY).  It lets those
 * files compile unmodified into the checker library oracle/_ref; DA vectors
 * are contiguous [k][j][i] arrays, matrices are row lists, KSP is
 * unpreconditioned BiCGStab.  Nothing here is part of the product.
 */
#ifndef SHIM_PETSC_H
#define SHIM_PETSC_H
#include <stdio.h>
#include <stdlib.h>
#include <math.h>

typedef int PetscErrorCode;
typedef int PetscInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef int PetscTruth;
typedef double PetscLogDouble;
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct _p_Vec *Vec;
typedef struct _p_Mat *Mat;
typedef struct _p_KSP *KSP;
typedef struct _p_PC *PC;
typedef struct _p_DA *DA;
typedef struct _p_Viewer *PetscViewer;
typedef struct _p_NullSpace *MatNullSpace;
typedef const char *KSPType;
typedef const char *PCType;
typedef const char *MatType;
typedef struct { PetscInt k, j, i, c; } MatStencil;
typedef enum { INSERT_VALUES = 0, ADD_VALUES = 1 } InsertMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { SAME_NONZERO_PATTERN = 0, DIFFERENT_NONZERO_PATTERN = 1, SAME_PRECONDITIONER = 2 } MatStructure;
typedef enum { DA_NONPERIODIC = 0 } DAPeriodicType;
typedef enum { DA_STENCIL_STAR = 0, DA_STENCIL_BOX = 1 } DAStencilType;
typedef enum { FILE_MODE_READ = 0, FILE_MODE_WRITE = 1 } PetscFileMode;
typedef enum {
    KSP_CONVERGED_RTOL = 2, KSP_CONVERGED_ATOL = 3, KSP_CONVERGED_ITERATING = 0,
    KSP_DIVERGED_NULL = -2, KSP_DIVERGED_ITS = -3, KSP_DIVERGED_DTOL = -4, KSP_DIVERGED_BREAKDOWN = -5,
    KSP_DIVERGED_BREAKDOWN_BICG = -6, KSP_DIVERGED_NONSYMMETRIC = -7, KSP_DIVERGED_INDEFINITE_PC = -8,
    KSP_DIVERGED_NAN = -9, KSP_DIVERGED_INDEFINITE_MAT = -10
} KSPConvergedReason;

#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 1
#define PETSC_NULL 0
#define PETSC_DECIDE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_TRUE 1
#define PETSC_FALSE 0
#define MATMPIAIJ "mpiaij"
#define KSPIBCGS "ibcgs"
#define KSPBCGS "bcgs"
#define KSPGMRES "gmres"
#define KSPCG "cg"
#define PCNONE "none"
#define PCHYPRE "hypre"
#define PCILU "ilu"
#define PCJACOBI "jacobi"
#define PCBJACOBI "bjacobi"
#define PCSOR "sor"
#define PCLU "lu"
#define PCASM "asm"
#define PCEISENSTAT "eisenstat"
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#ifndef __SDIR__
#define __SDIR__ ""
#endif

int PetscPrintf(MPI_Comm comm, const char *fmt, ...);
int PetscError(int line, const char *func, const char *file, const char *dir, int n, int p, const char *mess, ...);
int PetscFinalize(void);
int PetscGetTime(PetscLogDouble *t);
int PetscMallocGetCurrentUsage(PetscLogDouble *m);
int PetscOptionsSetValue(const char *a, const char *b);
int PetscMalloc(size_t n, void **p);

int MPI_Allreduce(void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Reduce(void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Comm_rank(MPI_Comm c, int *r);
int MPI_Comm_size(MPI_Comm c, int *r);
int MPI_Barrier(MPI_Comm c);

int DACreate3d(MPI_Comm c, DAPeriodicType p, DAStencilType st, int M, int N, int P, int m, int n, int pp,
               int dof, int s, const int *lx, const int *ly, const int *lz, DA *da);
int DADestroy(DA da);
int DAView(DA da, PetscViewer v);
int DACreateGlobalVector(DA da, Vec *v);
int DACreateLocalVector(DA da, Vec *v);
int DAGetCorners(DA da, int *x, int *y, int *z, int *m, int *n, int *p);
int DAGetGhostCorners(DA da, int *x, int *y, int *z, int *m, int *n, int *p);
int DAGetGlobalIndices(DA da, int *n, int **idx);
int DAGetInfo(DA da, int *dim, int *M, int *N, int *P, int *m, int *n, int *p, int *dof, int *s,
              DAPeriodicType *wrap, DAStencilType *st);
int DAGetOwnershipRanges(DA da, const int **lx, const int **ly, const int **lz);
int DAGetMatrix(DA da, MatType t, Mat *A);
int VecGetArray(Vec v, PetscScalar **a);
int VecRestoreArray(Vec v, PetscScalar **a);
int VecGetSize(Vec v, PetscInt *n);
int DAVecGetArray(DA da, Vec v, void *array);
int DAVecRestoreArray(DA da, Vec v, void *array);
int DAGlobalToLocalBegin(DA da, Vec g, InsertMode mode, Vec l);
int DAGlobalToLocalEnd(DA da, Vec g, InsertMode mode, Vec l);

int VecDuplicate(Vec v, Vec *n);
int VecDestroy(Vec v);
int VecCopy(Vec x, Vec y);
int VecAXPBY(Vec y, PetscScalar a, PetscScalar b, Vec x);
int VecAXPY(Vec y, PetscScalar a, Vec x);
int VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y);
int VecScale(Vec x, PetscScalar a);
int VecShift(Vec x, PetscScalar a);
int VecSet(Vec x, PetscScalar a);
int VecSum(Vec x, PetscScalar *s);
int VecView(Vec x, PetscViewer v);
int VecCreate(MPI_Comm c, Vec *v);
int VecSetSizes(Vec v, int n, int N);
int VecSetFromOptions(Vec v);

int MatSetValuesStencil(Mat A, int m, const MatStencil *rows, int n, const MatStencil *cols,
                        const PetscScalar *v, InsertMode mode);
int MatSetValues(Mat A, int m, const int *rows, int n, const int *cols, const PetscScalar *v, InsertMode mode);
int MatAssemblyBegin(Mat A, MatAssemblyType t);
int MatAssemblyEnd(Mat A, MatAssemblyType t);
int MatDiagonalSet(Mat A, Vec d, InsertMode mode);
int MatDestroy(Mat A);
int MatCreate(MPI_Comm c, Mat *A);
int MatSetSizes(Mat A, int m, int n, int M, int N);
int MatSetType(Mat A, MatType t);
int MatSetFromOptions(Mat A);
int MatLoad(PetscViewer v, MatType t, Mat *A);
int MatNullSpaceCreate(MPI_Comm c, PetscTruth has, int n, const Vec *v, MatNullSpace *sp);
int MatNullSpaceDestroy(MatNullSpace sp);

int KSPCreate(MPI_Comm c, KSP *k);
int KSPSetOperators(KSP k, Mat A, Mat P, MatStructure s);
int KSPSetType(KSP k, KSPType t);
int KSPSetTolerances(KSP k, PetscReal rtol, PetscReal atol, PetscReal dtol, int maxits);
int KSPGetPC(KSP k, PC *pc);
int KSPSetUp(KSP k);
int KSPSolve(KSP k, Vec b, Vec x);
int KSPGetIterationNumber(KSP k, int *its);
int KSPGetConvergedReason(KSP k, KSPConvergedReason *r);
int KSPSetInitialGuessNonzero(KSP k, PetscTruth t);
int KSPSetFromOptions(KSP k);
int KSPDestroy(KSP k);
int KSPView(KSP k, PetscViewer v);
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)
int KSPGMRESSetRestart(KSP k, int r);
int KSPSetNullSpace(KSP k, MatNullSpace sp);
int PCSetType(PC pc, PCType t);
int PCHYPRESetType(PC pc, const char *t);
int PCFactorSetLevels(PC pc, int l);
int PCFactorSetReuseOrdering(PC pc, PetscTruth t);
int PCFactorSetReuseFill(PC pc, PetscTruth t);
int PCFactorSetAllowDiagonalFill(PC pc);
int PCFactorSetUseInPlace(PC pc);
int PCFactorSetFill(PC pc, PetscReal f);
int PCFactorSetUseDropTolerance(PC pc, PetscReal a, PetscReal b, int c);
int PetscViewerBinaryOpen(MPI_Comm c, const char *name, PetscFileMode m, PetscViewer *v);
int PetscViewerDestroy(PetscViewer v);
int VecLoadIntoVector(PetscViewer v, Vec x);

/* shim-only access used by the harness */
double *shim_vec_data(Vec v);
long shim_vec_size(Vec v);
int shim_mat_mult(Mat A, const double *x, double *y);
#endif
