// ref_shim.cpp - implementation of the single-rank MPI and PETSc stand-ins (mpi.h, petsc.h).
//
// TEST INFRASTRUCTURE ONLY: linked with the reference's unchanged sources into the parity
// library under oracle/_ref. Never part of the product library.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "petsc.h"

// ---------------------------------------------------------------------------
// MPI, one rank

static size_t type_size(MPI_Datatype t) {
    switch (t) {
    case MPI_CHAR: case MPI_UNSIGNED_CHAR: return 1;
    case MPI_SHORT: case MPI_UNSIGNED_SHORT: return 2;
    case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
    case MPI_LONG: case MPI_UNSIGNED_LONG: case MPI_LONG_LONG: case MPI_UNSIGNED_LONG_LONG: case MPI_DOUBLE: return 8;
    default: return 0;  // derived types: only ever broadcast, which copies nothing
    }
}

extern "C" {
int MPI_Initialized(int* flag) { *flag = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) { throw std::runtime_error("MPI_Abort(" + std::to_string(code) + ")"); }
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op, MPI_Comm) {
    if (sendbuf != recvbuf) std::memcpy(recvbuf, sendbuf, (size_t)count * type_size(type));
    return MPI_SUCCESS;
}
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int, MPI_Datatype,
                  MPI_Comm) {
    std::memcpy(recvbuf, sendbuf, (size_t)sendcount * type_size(sendtype));
    return MPI_SUCCESS;
}
int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) {
    throw std::runtime_error("MPI_Isend on a single rank");
}
int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) {
    throw std::runtime_error("MPI_Irecv on a single rank");
}
int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }
int MPI_Get_address(const void* location, MPI_Aint* address) {
    *address = (MPI_Aint)location;
    return MPI_SUCCESS;
}
int MPI_Type_create_struct(int, const int*, const MPI_Aint*, const MPI_Datatype*, MPI_Datatype* newtype) {
    *newtype = LSREF_MPI_FIRST_DERIVED;
    return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
int MPI_File_open(MPI_Comm, const char*, int, MPI_Info, MPI_File*) {
    throw std::runtime_error("MPI-IO is not part of the parity library");
}
int MPI_File_seek(MPI_File, MPI_Offset, int) { return MPI_ERR_OTHER; }
int MPI_File_write(MPI_File, const void*, int, MPI_Datatype, MPI_Status*) { return MPI_ERR_OTHER; }
int MPI_File_close(MPI_File*) { return MPI_ERR_OTHER; }
}

// ---------------------------------------------------------------------------
// PETSc objects

struct _p_Vec {
    std::vector<double> own;
    double* data = nullptr;
    PetscInt n = 0;
};

struct _p_Mat {
    PetscInt n = 0;
    std::vector<std::vector<std::pair<int, double>>> rows;  // entries in insertion order, sorted at assembly
    bool assembled = false;
};

struct _p_PC {
    std::string type = PCJACOBI;
};

struct _p_KSP {
    Mat A = nullptr;
    std::string prefix;
    std::string type = KSPGMRES;
    double rtol = 1e-5, abstol = 1e-50, dtol = 1e5;
    int max_it = 10000, restart = 30;
    bool nonzero_guess = false;
    int its = 0;
    KSPConvergedReason reason = KSP_CONVERGED_ITERATING;
    _p_PC pc;
};

static std::map<std::string, std::string>& options() {
    static std::map<std::string, std::string> db;
    return db;
}

extern "C" {
void lsref_options_set(const char* name, const char* value) { options()[name] = value ? value : ""; }
void lsref_options_clear(void) { options().clear(); }

PetscErrorCode PetscInitialize(int*, char***, const char*, const char*) { return 0; }
PetscErrorCode PetscFinalize(void) { return 0; }

PetscErrorCode VecCreate(MPI_Comm, Vec* v) {
    *v = new _p_Vec();
    return 0;
}
PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt) {
    v->n = n;
    v->own.assign((size_t)n, 0.0);
    v->data = v->own.data();
    return 0;
}
PetscErrorCode VecSetFromOptions(Vec) { return 0; }
PetscErrorCode VecDuplicate(Vec v, Vec* out) {
    *out = new _p_Vec();
    VecSetSizes(*out, v->n, PETSC_DECIDE);
    return 0;
}
PetscErrorCode VecDestroy(Vec* v) {
    delete *v;
    *v = nullptr;
    return 0;
}
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar value, InsertMode mode) {
    if (i < 0 || i >= v->n) throw std::runtime_error("VecSetValue: index out of range");
    if (mode == ADD_VALUES) v->data[i] += value;
    else v->data[i] = value;
    return 0;
}
PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
PetscErrorCode VecZeroEntries(Vec v) {
    for (PetscInt i = 0; i < v->n; ++i) v->data[i] = 0.0;
    return 0;
}
PetscErrorCode VecPlaceArray(Vec v, const PetscScalar* array) {
    v->data = const_cast<double*>(array);
    return 0;
}
PetscErrorCode VecResetArray(Vec v) {
    v->data = v->own.data();
    return 0;
}
PetscErrorCode VecMin(Vec v, PetscInt* loc, PetscReal* value) {
    PetscInt l = 0;
    for (PetscInt i = 1; i < v->n; ++i)
        if (v->data[i] < v->data[l]) l = i;
    if (loc) *loc = l;
    *value = v->n ? v->data[l] : 0.0;
    return 0;
}
PetscErrorCode VecMax(Vec v, PetscInt* loc, PetscReal* value) {
    PetscInt l = 0;
    for (PetscInt i = 1; i < v->n; ++i)
        if (v->data[i] > v->data[l]) l = i;
    if (loc) *loc = l;
    *value = v->n ? v->data[l] : 0.0;
    return 0;
}
PetscErrorCode VecNorm(Vec v, NormType type, PetscReal* value) {
    double acc = 0.0;
    for (PetscInt i = 0; i < v->n; ++i) {
        const double x = v->data[i];
        if (type == NORM_1) acc += std::fabs(x);
        else if (type == NORM_INFINITY) acc = std::fmax(acc, std::fabs(x));
        else acc += x * x;
    }
    *value = (type == NORM_2) ? std::sqrt(acc) : acc;
    return 0;
}

PetscErrorCode MatCreate(MPI_Comm, Mat* A) {
    *A = new _p_Mat();
    return 0;
}
PetscErrorCode MatSetSizes(Mat A, PetscInt m, PetscInt, PetscInt, PetscInt) {
    A->n = m;
    A->rows.assign((size_t)m, {});
    return 0;
}
PetscErrorCode MatSetType(Mat, MatType) { return 0; }
PetscErrorCode MatMPIAIJSetPreallocation(Mat, PetscInt, const PetscInt*, PetscInt, const PetscInt*) { return 0; }
PetscErrorCode MatSetOption(Mat, MatOption, PetscBool) { return 0; }
PetscErrorCode MatSetFromOptions(Mat) { return 0; }
PetscErrorCode MatSetValue(Mat A, PetscInt i, PetscInt j, PetscScalar value, InsertMode mode) {
    if (i < 0 || i >= A->n || j < 0 || j >= A->n) throw std::runtime_error("MatSetValue: index out of range");
    auto& row = A->rows[(size_t)i];
    for (auto& e : row)
        if (e.first == j) {
            // an existing entry: add in call order (AIJ's ap[k] += v), or replace
            if (mode == ADD_VALUES) e.second += value;
            else e.second = value;
            return 0;
        }
    row.emplace_back(j, value);  // a new entry takes the value as given
    A->assembled = false;
    return 0;
}
PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType) {
    for (auto& row : A->rows)
        std::sort(row.begin(), row.end(), [](const std::pair<int, double>& a, const std::pair<int, double>& b) {
            return a.first < b.first;
        });
    A->assembled = true;
    return 0;
}
PetscErrorCode MatZeroEntries(Mat A) {
    for (auto& row : A->rows)
        for (auto& e : row) e.second = 0.0;
    return 0;
}
PetscErrorCode MatDestroy(Mat* A) {
    delete *A;
    *A = nullptr;
    return 0;
}
PetscErrorCode MatAssembled(Mat A, PetscBool* flag) {
    *flag = A->assembled ? PETSC_TRUE : PETSC_FALSE;
    return 0;
}
PetscErrorCode MatCreateVecs(Mat A, Vec* right, Vec* left) {
    if (right) {
        VecCreate(0, right);
        VecSetSizes(*right, A->n, PETSC_DECIDE);
    }
    if (left) {
        VecCreate(0, left);
        VecSetSizes(*left, A->n, PETSC_DECIDE);
    }
    return 0;
}
PetscErrorCode MatGetDiagonal(Mat A, Vec d) {
    for (PetscInt i = 0; i < A->n; ++i) {
        double v = 0.0;
        for (const auto& e : A->rows[(size_t)i])
            if (e.first == i) v = e.second;
        d->data[i] = v;
    }
    return 0;
}
}  // extern "C"

// y = A x, each row's entries in ascending column order
static void mat_mult(const _p_Mat* A, const double* x, double* y) {
    for (PetscInt i = 0; i < A->n; ++i) {
        double acc = 0.0;
        for (const auto& e : A->rows[(size_t)i]) acc += e.second * x[e.first];
        y[i] = acc;
    }
}

// Restarted GMRES, classical Gram-Schmidt, left Jacobi preconditioning B = diag(A)^-1 (zero
// diagonal entries taken as 1); converged when ||B r|| <= max(rtol ||B b||, abstol).
static void gmres_solve(KSP ksp, const double* b, double* x) {
    const _p_Mat* A = ksp->A;
    const PetscInt n = A->n;
    const int m = ksp->restart > 0 ? ksp->restart : 30;
    std::vector<double> dinv((size_t)n), w((size_t)n), V((size_t)(m + 1) * n), H((size_t)(m + 1) * m);
    std::vector<double> cs((size_t)m), sn((size_t)m), g((size_t)m + 1), yv((size_t)m);
    for (PetscInt i = 0; i < n; ++i) {
        double d = 0.0;
        for (const auto& e : A->rows[(size_t)i])
            if (e.first == i) d = e.second;
        dinv[(size_t)i] = (d != 0.0) ? 1.0 / d : 1.0;
    }
    double bn = 0.0;
    for (PetscInt i = 0; i < n; ++i) bn += (dinv[i] * b[i]) * (dinv[i] * b[i]);
    bn = std::sqrt(bn);
    const double ttol = std::fmax(ksp->rtol * bn, ksp->abstol);
    int its = 0;
    ksp->reason = KSP_CONVERGED_ITERATING;
    for (;;) {
        mat_mult(A, x, w.data());
        double beta = 0.0;
        for (PetscInt i = 0; i < n; ++i) {
            V[(size_t)i] = dinv[i] * (b[i] - w[i]);
            beta += V[(size_t)i] * V[(size_t)i];
        }
        beta = std::sqrt(beta);
        if (!std::isfinite(beta)) { ksp->reason = KSP_DIVERGED_NANORINF; break; }
        if (beta <= ttol) { ksp->reason = (beta < ksp->abstol) ? KSP_CONVERGED_ATOL : KSP_CONVERGED_RTOL; break; }
        if (its >= ksp->max_it) { ksp->reason = KSP_DIVERGED_ITS; break; }
        for (PetscInt i = 0; i < n; ++i) V[(size_t)i] /= beta;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int done = 0;
        for (int j = 0; j < m; ++j) {
            double* vj = &V[(size_t)j * n];
            double* vn = &V[(size_t)(j + 1) * n];
            mat_mult(A, vj, w.data());
            for (PetscInt i = 0; i < n; ++i) vn[i] = dinv[i] * w[i];
            for (int q = 0; q <= j; ++q) {
                double h = 0.0;
                const double* vq = &V[(size_t)q * n];
                for (PetscInt i = 0; i < n; ++i) h += vn[i] * vq[i];
                H[(size_t)q * m + j] = h;
            }
            for (int q = 0; q <= j; ++q) {
                const double h = H[(size_t)q * m + j];
                const double* vq = &V[(size_t)q * n];
                for (PetscInt i = 0; i < n; ++i) vn[i] -= h * vq[i];
            }
            double hn = 0.0;
            for (PetscInt i = 0; i < n; ++i) hn += vn[i] * vn[i];
            hn = std::sqrt(hn);
            H[(size_t)(j + 1) * m + j] = hn;
            if (hn > 0.0)
                for (PetscInt i = 0; i < n; ++i) vn[i] /= hn;
            for (int q = 0; q < j; ++q) {
                const double a = H[(size_t)q * m + j], c = H[(size_t)(q + 1) * m + j];
                H[(size_t)q * m + j] = cs[q] * a + sn[q] * c;
                H[(size_t)(q + 1) * m + j] = -sn[q] * a + cs[q] * c;
            }
            const double a = H[(size_t)j * m + j], c = H[(size_t)(j + 1) * m + j];
            const double den = std::sqrt(a * a + c * c);
            cs[j] = den == 0.0 ? 1.0 : a / den;
            sn[j] = den == 0.0 ? 0.0 : c / den;
            H[(size_t)j * m + j] = cs[j] * a + sn[j] * c;
            H[(size_t)(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++its;
            done = j + 1;
            const double rn = std::fabs(g[j + 1]);
            if (!std::isfinite(rn)) { ksp->reason = KSP_DIVERGED_NANORINF; break; }
            if (rn <= ttol) { ksp->reason = (rn < ksp->abstol) ? KSP_CONVERGED_ATOL : KSP_CONVERGED_RTOL; break; }
            if (hn == 0.0) { ksp->reason = KSP_CONVERGED_RTOL; break; }
            if (its >= ksp->max_it) { ksp->reason = KSP_DIVERGED_ITS; break; }
        }
        for (int q = done - 1; q >= 0; --q) {
            double t = g[q];
            for (int c2 = q + 1; c2 < done; ++c2) t -= H[(size_t)q * m + c2] * yv[c2];
            yv[q] = H[(size_t)q * m + q] != 0.0 ? t / H[(size_t)q * m + q] : 0.0;
        }
        for (PetscInt i = 0; i < n; ++i) {
            double t = x[i];
            for (int q = 0; q < done; ++q) t += yv[q] * V[(size_t)q * n + i];
            x[i] = t;
        }
        if (ksp->reason != KSP_CONVERGED_ITERATING) break;
    }
    ksp->its = its;
}

extern "C" {
PetscErrorCode KSPCreate(MPI_Comm, KSP* ksp) {
    *ksp = new _p_KSP();
    return 0;
}
PetscErrorCode KSPSetType(KSP ksp, KSPType type) {
    ksp->type = type;
    return 0;
}
PetscErrorCode KSPSetOptionsPrefix(KSP ksp, const char* prefix) {
    ksp->prefix = prefix ? prefix : "";
    return 0;
}
PetscErrorCode KSPGetPC(KSP ksp, PC* pc) {
    *pc = &ksp->pc;
    return 0;
}
PetscErrorCode PCSetType(PC pc, PCType type) {
    pc->type = type;
    return 0;
}
PetscErrorCode KSPSetTolerances(KSP ksp, PetscReal rtol, PetscReal abstol, PetscReal dtol, PetscInt maxits) {
    if (rtol != PETSC_DEFAULT) ksp->rtol = rtol;
    if (abstol != PETSC_DEFAULT) ksp->abstol = abstol;
    if (dtol != PETSC_DEFAULT) ksp->dtol = dtol;
    if (maxits != PETSC_DEFAULT) ksp->max_it = maxits;
    return 0;
}
PetscErrorCode KSPSetInitialGuessNonzero(KSP ksp, PetscBool flag) {
    ksp->nonzero_guess = flag == PETSC_TRUE;
    return 0;
}
PetscErrorCode KSPSetFromOptions(KSP ksp) {
    auto& db = options();
    auto get = [&](const char* key) -> const std::string* {
        auto it = db.find(ksp->prefix + key);
        return it == db.end() ? nullptr : &it->second;
    };
    if (auto v = get("ksp_rtol")) ksp->rtol = std::stod(*v);
    if (auto v = get("ksp_atol")) ksp->abstol = std::stod(*v);
    if (auto v = get("ksp_max_it")) ksp->max_it = std::stoi(*v);
    if (auto v = get("ksp_gmres_restart")) ksp->restart = std::stoi(*v);
    return 0;
}
PetscErrorCode KSPReset(KSP ksp) {
    ksp->A = nullptr;
    return 0;
}
PetscErrorCode KSPSetOperators(KSP ksp, Mat A, Mat) {
    ksp->A = A;
    return 0;
}
PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x) {
    if (!ksp->A || !ksp->A->assembled) throw std::runtime_error("KSPSolve: no assembled operator");
    if (!ksp->nonzero_guess) VecZeroEntries(x);
    gmres_solve(ksp, b->data, x->data);
    return 0;
}
PetscErrorCode KSPGetIterationNumber(KSP ksp, PetscInt* its) {
    *its = ksp->its;
    return 0;
}
PetscErrorCode KSPGetConvergedReason(KSP ksp, KSPConvergedReason* reason) {
    *reason = ksp->reason;
    return 0;
}
PetscErrorCode KSPDestroy(KSP* ksp) {
    delete *ksp;
    *ksp = nullptr;
    return 0;
}
}  // extern "C"
