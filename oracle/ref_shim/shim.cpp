/*
 * Implementation of the single-rank dense PETSc/MPI stand-in declared in
 * petscsys.h and mpi.h.  Test infrastructure only: it exists so the TD-BEM
 * reference sources (SolverT.cpp, SolverStepLinearT.cpp, main.cpp, ...) can
 * be compiled unmodified and run here to pin the oracle.
 *
 * Summation order of MatMult/MatMultAdd is the plain row-wise left-to-right
 * dot product; KSPSolve is Doolittle LU with partial pivoting (largest
 * absolute value, first index on ties) followed by forward/back substitution.
 */
#include "petscsys.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

struct _shim_Mat {
    int m, n;
    std::vector<double> a;  // row-major m x n
};
struct _shim_Vec {
    int n;
    std::vector<double> a;
};
struct _shim_KSP {
    Mat A = nullptr;
    std::vector<double> cached;  // copy of the operator last factorized
    std::vector<double> lu;      // packed L\U factors
    std::vector<int> piv;
    int n = 0;
};
struct _shim_VecScatter {
    int n;
};

static long g_factorizations = 0;
long shim_ksp_factorizations(void) { return g_factorizations; }

extern "C" {
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return 0; }
int MPI_Barrier(MPI_Comm) { return 0; }
}

PetscErrorCode PetscInitialize(int*, char***, const char*, const char*) { return 0; }
PetscErrorCode PetscFinalize(void) { return 0; }

PetscErrorCode PetscStrcmp(const char* a, const char* b, PetscBool* flg) {
    if (!a && !b) *flg = PETSC_TRUE;
    else if (!a || !b) *flg = PETSC_FALSE;
    else *flg = std::strcmp(a, b) == 0 ? PETSC_TRUE : PETSC_FALSE;
    return 0;
}
PetscErrorCode PetscStrcpy(char* s, const char* t) {
    if (t) std::strcpy(s, t);
    else s[0] = 0;
    return 0;
}

static void die(const char* what) {
    std::fprintf(stderr, "ref shim: %s\n", what);
    std::abort();
}

PetscErrorCode MatCreateDense(MPI_Comm, PetscInt, PetscInt, PetscInt M, PetscInt N,
                              PetscScalar* data, Mat* A) {
    Mat m = new _shim_Mat;
    m->m = M;
    m->n = N;
    m->a.assign((size_t)M * N, 0.0);
    if (data) std::memcpy(m->a.data(), data, sizeof(double) * (size_t)M * N);
    *A = m;
    return 0;
}
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt idxm[], PetscInt n,
                            const PetscInt idxn[], const PetscScalar v[], InsertMode mode) {
    for (int i = 0; i < m; i++) {
        if (idxm[i] < 0) continue;
        if (idxm[i] >= A->m) die("MatSetValues row out of range");
        for (int j = 0; j < n; j++) {
            if (idxn[j] < 0) continue;
            if (idxn[j] >= A->n) die("MatSetValues column out of range");
            double& dst = A->a[(size_t)idxm[i] * A->n + idxn[j]];
            if (mode == ADD_VALUES) dst += v[(size_t)i * n + j];
            else dst = v[(size_t)i * n + j];
        }
    }
    return 0;
}
PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType) { return 0; }
PetscErrorCode MatCopy(Mat A, Mat B, MatStructure) {
    if (A->m != B->m || A->n != B->n) die("MatCopy size mismatch");
    B->a = A->a;
    return 0;
}
PetscErrorCode MatConvert(Mat A, MatType, MatReuse, Mat* B) {
    Mat m = new _shim_Mat;
    *m = *A;
    *B = m;
    return 0;
}
PetscErrorCode MatAXPY(Mat Y, PetscScalar a, Mat X, MatStructure) {
    if (X->m != Y->m || X->n != Y->n) die("MatAXPY size mismatch");
    const size_t sz = Y->a.size();
    for (size_t i = 0; i < sz; i++) Y->a[i] += a * X->a[i];
    return 0;
}
PetscErrorCode MatScale(Mat A, PetscScalar a) {
    for (double& v : A->a) v *= a;
    return 0;
}
PetscErrorCode MatZeroEntries(Mat A) {
    std::fill(A->a.begin(), A->a.end(), 0.0);
    return 0;
}
PetscErrorCode MatMult(Mat A, Vec x, Vec y) {
    if (A->n != x->n || A->m != y->n) die("MatMult size mismatch");
    std::vector<double> out(A->m);
    for (int i = 0; i < A->m; i++) {
        const double* row = &A->a[(size_t)i * A->n];
        double s = 0.0;
        for (int j = 0; j < A->n; j++) s += row[j] * x->a[j];
        out[i] = s;
    }
    y->a = out;
    return 0;
}
PetscErrorCode MatMultAdd(Mat A, Vec x, Vec y, Vec z) {
    if (A->n != x->n || A->m != y->n || A->m != z->n) die("MatMultAdd size mismatch");
    std::vector<double> out(A->m);
    for (int i = 0; i < A->m; i++) {
        const double* row = &A->a[(size_t)i * A->n];
        double s = 0.0;
        for (int j = 0; j < A->n; j++) s += row[j] * x->a[j];
        out[i] = y->a[i] + s;
    }
    z->a = out;
    return 0;
}
PetscErrorCode MatGetColumnVector(Mat A, Vec v, PetscInt col) {
    if (v->n != A->m || col < 0 || col >= A->n) die("MatGetColumnVector range");
    for (int i = 0; i < A->m; i++) v->a[i] = A->a[(size_t)i * A->n + col];
    return 0;
}
PetscErrorCode MatGetOwnershipRange(Mat A, PetscInt* lo, PetscInt* hi) {
    *lo = 0;
    *hi = A->m;
    return 0;
}
PetscErrorCode MatGetSize(Mat A, PetscInt* m, PetscInt* n) {
    *m = A->m;
    *n = A->n;
    return 0;
}
PetscErrorCode MatDestroy(Mat* A) {
    delete *A;
    *A = nullptr;
    return 0;
}
PetscErrorCode MatView(Mat A, PetscViewer) {
    for (int i = 0; i < A->m; i++) {
        for (int j = 0; j < A->n; j++) std::printf(" %.6e", A->a[(size_t)i * A->n + j]);
        std::printf("\n");
    }
    return 0;
}

PetscErrorCode VecCreateMPI(MPI_Comm, PetscInt, PetscInt N, Vec* v) {
    Vec x = new _shim_Vec;
    x->n = N;
    x->a.assign(N, 0.0);
    *v = x;
    return 0;
}
PetscErrorCode VecSet(Vec v, PetscScalar a) {
    std::fill(v->a.begin(), v->a.end(), a);
    return 0;
}
PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt ix[], const PetscScalar y[],
                            InsertMode mode) {
    for (int i = 0; i < n; i++) {
        if (ix[i] < 0) continue;
        if (ix[i] >= v->n) die("VecSetValues out of range");
        if (mode == ADD_VALUES) v->a[ix[i]] += y[i];
        else v->a[ix[i]] = y[i];
    }
    return 0;
}
PetscErrorCode VecGetValues(Vec v, PetscInt n, const PetscInt ix[], PetscScalar y[]) {
    for (int i = 0; i < n; i++) {
        if (ix[i] < 0 || ix[i] >= v->n) die("VecGetValues out of range");
        y[i] = v->a[ix[i]];
    }
    return 0;
}
PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
PetscErrorCode VecCopy(Vec x, Vec y) {
    if (x->n != y->n) die("VecCopy size mismatch");
    y->a = x->a;
    return 0;
}
PetscErrorCode VecScale(Vec v, PetscScalar a) {
    for (double& x : v->a) x *= a;
    return 0;
}
PetscErrorCode VecGetArray(Vec v, PetscScalar** a) {
    *a = v->a.data();
    return 0;
}
PetscErrorCode VecRestoreArray(Vec, PetscScalar** a) {
    *a = nullptr;
    return 0;
}
PetscErrorCode VecGetOwnershipRange(Vec v, PetscInt* lo, PetscInt* hi) {
    *lo = 0;
    *hi = v->n;
    return 0;
}
PetscErrorCode VecDestroy(Vec* v) {
    delete *v;
    *v = nullptr;
    return 0;
}
PetscErrorCode VecView(Vec v, PetscViewer) {
    for (int i = 0; i < v->n; i++) std::printf("%.6e\n", v->a[i]);
    return 0;
}

PetscErrorCode VecScatterCreateToAll(Vec vin, VecScatter* ctx, Vec* vout) {
    VecScatter s = new _shim_VecScatter;
    s->n = vin->n;
    *ctx = s;
    VecCreateMPI(0, PETSC_DECIDE, vin->n, vout);
    return 0;
}
PetscErrorCode VecScatterBegin(VecScatter, Vec x, Vec y, InsertMode, ScatterMode) {
    y->a = x->a;
    return 0;
}
PetscErrorCode VecScatterEnd(VecScatter, Vec, Vec, InsertMode, ScatterMode) { return 0; }
PetscErrorCode VecScatterDestroy(VecScatter* ctx) {
    delete *ctx;
    *ctx = nullptr;
    return 0;
}

PetscErrorCode KSPCreate(MPI_Comm, KSP* ksp) {
    *ksp = new _shim_KSP;
    return 0;
}
PetscErrorCode KSPSetOperators(KSP ksp, Mat A, Mat) {
    ksp->A = A;
    return 0;
}

static void factorize(KSP k) {
    const int n = k->A->m;
    k->n = n;
    k->lu = k->A->a;
    k->piv.assign(n, 0);
    double* a = k->lu.data();
    for (int c = 0; c < n; c++) {
        int p = c;
        double best = std::fabs(a[(size_t)c * n + c]);
        for (int r = c + 1; r < n; r++) {
            const double v = std::fabs(a[(size_t)r * n + c]);
            if (v > best) { best = v; p = r; }
        }
        k->piv[c] = p;
        if (p != c)
            for (int j = 0; j < n; j++) std::swap(a[(size_t)c * n + j], a[(size_t)p * n + j]);
        const double d = a[(size_t)c * n + c];
        if (d == 0.0) die("KSPSolve: singular operator");
        for (int r = c + 1; r < n; r++) {
            double& l = a[(size_t)r * n + c];
            l /= d;
            if (l == 0.0) continue;
            const double* urow = &a[(size_t)c * n];
            double* rrow = &a[(size_t)r * n];
            for (int j = c + 1; j < n; j++) rrow[j] -= l * urow[j];
        }
    }
    k->cached = k->A->a;
    g_factorizations++;
}

PetscErrorCode KSPSolve(KSP k, Vec b, Vec x) {
    if (!k->A) die("KSPSolve without operator");
    const int n = k->A->m;
    if (k->cached.size() != k->A->a.size() ||
        std::memcmp(k->cached.data(), k->A->a.data(), sizeof(double) * k->A->a.size()) != 0)
        factorize(k);
    std::vector<double> y = b->a;
    for (int c = 0; c < n; c++)
        if (k->piv[c] != c) std::swap(y[c], y[k->piv[c]]);
    const double* a = k->lu.data();
    for (int r = 0; r < n; r++) {
        double s = y[r];
        for (int j = 0; j < r; j++) s -= a[(size_t)r * n + j] * y[j];
        y[r] = s;
    }
    for (int r = n - 1; r >= 0; r--) {
        double s = y[r];
        for (int j = r + 1; j < n; j++) s -= a[(size_t)r * n + j] * y[j];
        y[r] = s / a[(size_t)r * n + r];
    }
    x->a = y;
    return 0;
}
PetscErrorCode KSPDestroy(KSP* ksp) {
    delete *ksp;
    *ksp = nullptr;
    return 0;
}

const double* shim_mat_data(Mat A, int* m, int* n) {
    *m = A->m;
    *n = A->n;
    return A->a.data();
}
const double* shim_vec_data(Vec v, int* n) {
    *n = v->n;
    return v->a.data();
}
