/*
 * Single-rank, dense stand-in for the PETSc subset used by the TD-BEM
 * reference (SolverT.cpp, SolverStepLinearT.cpp, InputT.cpp, main.cpp).
 *
 * Test infrastructure only.  Semantics follow the PETSc manual pages for each
 * routine as the reference calls it; the one deliberate difference is
 * KSPSolve, which is an exact dense LU with partial pivoting instead of
 * PETSc's default GMRES(30) with rtol 1e-5 (SolverStepLinearT.cpp:503-504).
 * Matrices are dense row-major, vectors are plain arrays, and every object
 * is owned by the single process.
 */
#ifndef TDBEM_REF_SHIM_PETSCSYS_H
#define TDBEM_REF_SHIM_PETSCSYS_H

#include <stddef.h>
#include "mpi.h"

typedef int PetscErrorCode;
typedef int PetscInt;
typedef double PetscScalar;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;

typedef struct _shim_Mat* Mat;
typedef struct _shim_Vec* Vec;
typedef struct _shim_KSP* KSP;
typedef struct _shim_VecScatter* VecScatter;
typedef struct _shim_Viewer* PetscViewer;

typedef enum { INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { DIFFERENT_NONZERO_PATTERN = 0, SUBSET_NONZERO_PATTERN = 1,
               SAME_NONZERO_PATTERN = 2 } MatStructure;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { MAT_INITIAL_MATRIX = 0, MAT_REUSE_MATRIX = 1 } MatReuse;
typedef enum { SCATTER_FORWARD = 0, SCATTER_REVERSE = 1 } ScatterMode;
typedef const char* MatType;

#define MATSAME "same"
#define PETSC_COMM_WORLD 0
#define PETSC_DECIDE (-1)
#define PETSC_NULL NULL
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)

PetscErrorCode PetscInitialize(int* argc, char*** args, const char* file, const char* help);
PetscErrorCode PetscFinalize(void);
PetscErrorCode PetscStrcmp(const char* a, const char* b, PetscBool* flg);
PetscErrorCode PetscStrcpy(char* s, const char* t);

/* Mat */
PetscErrorCode MatCreateDense(MPI_Comm comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N,
                              PetscScalar* data, Mat* A);
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt idxm[], PetscInt n,
                            const PetscInt idxn[], const PetscScalar v[], InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t);
PetscErrorCode MatCopy(Mat A, Mat B, MatStructure str);
PetscErrorCode MatConvert(Mat A, MatType newtype, MatReuse reuse, Mat* B);
PetscErrorCode MatAXPY(Mat Y, PetscScalar a, Mat X, MatStructure str);
PetscErrorCode MatScale(Mat A, PetscScalar a);
PetscErrorCode MatZeroEntries(Mat A);
PetscErrorCode MatMult(Mat A, Vec x, Vec y);
PetscErrorCode MatMultAdd(Mat A, Vec x, Vec y, Vec z);
PetscErrorCode MatGetColumnVector(Mat A, Vec v, PetscInt col);
PetscErrorCode MatGetOwnershipRange(Mat A, PetscInt* lo, PetscInt* hi);
PetscErrorCode MatGetSize(Mat A, PetscInt* m, PetscInt* n);
PetscErrorCode MatDestroy(Mat* A);
PetscErrorCode MatView(Mat A, PetscViewer v);

/* Vec */
PetscErrorCode VecCreateMPI(MPI_Comm comm, PetscInt n, PetscInt N, Vec* v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt ix[], const PetscScalar y[],
                            InsertMode mode);
PetscErrorCode VecGetValues(Vec v, PetscInt n, const PetscInt ix[], PetscScalar y[]);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
PetscErrorCode VecCopy(Vec x, Vec y);
PetscErrorCode VecScale(Vec v, PetscScalar a);
PetscErrorCode VecGetArray(Vec v, PetscScalar** a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a);
PetscErrorCode VecGetOwnershipRange(Vec v, PetscInt* lo, PetscInt* hi);
PetscErrorCode VecDestroy(Vec* v);
PetscErrorCode VecView(Vec v, PetscViewer viewer);

PetscErrorCode VecScatterCreateToAll(Vec vin, VecScatter* ctx, Vec* vout);
PetscErrorCode VecScatterBegin(VecScatter ctx, Vec x, Vec y, InsertMode a, ScatterMode m);
PetscErrorCode VecScatterEnd(VecScatter ctx, Vec x, Vec y, InsertMode a, ScatterMode m);
PetscErrorCode VecScatterDestroy(VecScatter* ctx);

/* KSP: exact dense LU, refactored only when the operator's entries change */
PetscErrorCode KSPCreate(MPI_Comm comm, KSP* ksp);
PetscErrorCode KSPSetOperators(KSP ksp, Mat A, Mat P);
PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x);
PetscErrorCode KSPDestroy(KSP* ksp);

/* Counters used by the driver to report what the stand-in did. */
long shim_ksp_factorizations(void);

#endif
