/*
 * petsc.h - single-process stand-in for the PETSc interface the reference's hot-path
 * sources use (Vec, Mat, KSP, PC and the options database behind KSPSetFromOptions).
 *
 * TEST INFRASTRUCTURE ONLY (the parity library under oracle/_ref). Vectors own or borrow
 * (VecPlaceArray) a plain array; a matrix records MatSetValue into per-row entries that are
 * sorted by column at assembly, like an AIJ row, and MatMult sums them in that order; KSPSolve
 * is restarted GMRES with classical Gram-Schmidt and left Jacobi preconditioning (PETSc's
 * KSPGMRES + PCJACOBI defaults), stopping when the preconditioned residual norm falls below
 * max(rtol * ||B b||, abstol) or after max_it iterations. Tolerances come from
 * KSPSetTolerances and, through KSPSetFromOptions, from options "<prefix>ksp_rtol",
 * "<prefix>ksp_max_it" and "<prefix>ksp_gmres_restart" set with lsref_options_set.
 * Preconditioner types other than Jacobi are accepted and run as Jacobi.
 */
#ifndef LSREF_SHIM_PETSC_H_
#define LSREF_SHIM_PETSC_H_

#include "mpi.h"

typedef int PetscInt;
typedef int PetscErrorCode;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef enum { INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { MAT_NEW_NONZERO_ALLOCATION_ERR = 19, MAT_OTHER_OPTION = 100 } MatOption;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_INFINITY = 3 } NormType;
typedef enum {
    KSP_CONVERGED_RTOL = 2,
    KSP_CONVERGED_ATOL = 3,
    KSP_CONVERGED_ITERATING = 0,
    KSP_DIVERGED_ITS = -3,
    KSP_DIVERGED_DTOL = -4,
    KSP_DIVERGED_BREAKDOWN = -5,
    KSP_DIVERGED_NANORINF = -9
} KSPConvergedReason;
typedef const char* KSPType;
typedef const char* PCType;
typedef const char* MatType;

typedef struct _p_Vec* Vec;
typedef struct _p_Mat* Mat;
typedef struct _p_KSP* KSP;
typedef struct _p_PC* PC;
typedef struct _p_MatNullSpace* MatNullSpace;

#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE PETSC_DECIDE
#define PETSC_DEFAULT (-2)
#define PETSC_NULLPTR nullptr
#define PETSC_NULL nullptr
#define KSPGMRES "gmres"
#define PCJACOBI "jacobi"
#define PCSOR "sor"
#define PCILU "ilu"
#define PCBJACOBI "bjacobi"
#define MATMPIAIJ "mpiaij"

#ifdef __cplusplus
extern "C" {
#endif
PetscErrorCode PetscInitialize(int* argc, char*** argv, const char* file, const char* help);
PetscErrorCode PetscFinalize(void);

PetscErrorCode VecCreate(MPI_Comm comm, Vec* v);
PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt N);
PetscErrorCode VecSetFromOptions(Vec v);
PetscErrorCode VecDuplicate(Vec v, Vec* out);
PetscErrorCode VecDestroy(Vec* v);
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar value, InsertMode mode);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
PetscErrorCode VecZeroEntries(Vec v);
PetscErrorCode VecPlaceArray(Vec v, const PetscScalar* array);
PetscErrorCode VecResetArray(Vec v);
PetscErrorCode VecMin(Vec v, PetscInt* loc, PetscReal* value);
PetscErrorCode VecMax(Vec v, PetscInt* loc, PetscReal* value);
PetscErrorCode VecNorm(Vec v, NormType type, PetscReal* value);

PetscErrorCode MatCreate(MPI_Comm comm, Mat* A);
PetscErrorCode MatSetSizes(Mat A, PetscInt m, PetscInt n, PetscInt M, PetscInt N);
PetscErrorCode MatSetType(Mat A, MatType type);
PetscErrorCode MatMPIAIJSetPreallocation(Mat A, PetscInt d_nz, const PetscInt* d_nnz, PetscInt o_nz,
                                         const PetscInt* o_nnz);
PetscErrorCode MatSetOption(Mat A, MatOption op, PetscBool flag);
PetscErrorCode MatSetFromOptions(Mat A);
PetscErrorCode MatSetValue(Mat A, PetscInt i, PetscInt j, PetscScalar value, InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType type);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType type);
PetscErrorCode MatZeroEntries(Mat A);
PetscErrorCode MatDestroy(Mat* A);
PetscErrorCode MatAssembled(Mat A, PetscBool* flag);
PetscErrorCode MatCreateVecs(Mat A, Vec* right, Vec* left);
PetscErrorCode MatGetDiagonal(Mat A, Vec d);

PetscErrorCode KSPCreate(MPI_Comm comm, KSP* ksp);
PetscErrorCode KSPSetType(KSP ksp, KSPType type);
PetscErrorCode KSPSetOptionsPrefix(KSP ksp, const char* prefix);
PetscErrorCode KSPGetPC(KSP ksp, PC* pc);
PetscErrorCode PCSetType(PC pc, PCType type);
PetscErrorCode KSPSetTolerances(KSP ksp, PetscReal rtol, PetscReal abstol, PetscReal dtol, PetscInt maxits);
PetscErrorCode KSPSetInitialGuessNonzero(KSP ksp, PetscBool flag);
PetscErrorCode KSPSetFromOptions(KSP ksp);
PetscErrorCode KSPReset(KSP ksp);
PetscErrorCode KSPSetOperators(KSP ksp, Mat A, Mat P);
PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x);
PetscErrorCode KSPGetIterationNumber(KSP ksp, PetscInt* its);
PetscErrorCode KSPGetConvergedReason(KSP ksp, KSPConvergedReason* reason);
PetscErrorCode KSPDestroy(KSP* ksp);

/* the options database (PETSc's -<prefix>ksp_... command-line options) */
void lsref_options_set(const char* name, const char* value);
void lsref_options_clear(void);
#ifdef __cplusplus
}
#endif

#endif /* LSREF_SHIM_PETSC_H_ */
