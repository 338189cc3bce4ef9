/*
 * petsc_shim.cpp -- sequential implementations behind petsc_shim.h.
 * TEST INFRASTRUCTURE: used only to build the reference for the oracle check.
 */
#include "petsc_shim.h"
#include <cmath>
#include <cstdarg>

void msx_shim_abort(const char *name)
{
    fprintf(stderr, "petsc-shim: %s is outside the explicit path and is not provided\n", name);
    abort();
}

/* ---------------- MPI, one rank ---------------- */
static size_t mpi_size(MPI_Datatype t)
{
    switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_LONG: return sizeof(long);
    default: return 1;
    }
}
int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)n * mpi_size(t));
    return 0;
}
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm)
{
    if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)sn * mpi_size(st));
    return 0;
}
int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *dis,
                MPI_Datatype, int, MPI_Comm)
{
    if (s != MPI_IN_PLACE) memcpy((char *)r + (size_t)dis[0] * mpi_size(st), s, (size_t)sn * mpi_size(st));
    return 0;
}
int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm)
{
    if (s != MPI_IN_PLACE) memcpy(r, s, (size_t)sn * mpi_size(st));
    return 0;
}
int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { msx_shim_abort("MPI_Send"); return 1; }
int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { msx_shim_abort("MPI_Recv"); return 1; }
int MPI_Init(int *, char ***) { return 0; }
int MPI_Finalize(void) { return 0; }

/* ---------------- PETSc basics ---------------- */
PetscErrorCode PetscInitialize(int *, char ***, const char *, const char *) { return 0; }
PetscErrorCode PetscFinalize(void) { return 0; }
PetscErrorCode PetscPrintf(MPI_Comm, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vprintf(fmt, ap);
    va_end(ap);
    return 0;
}
PetscErrorCode PetscOptionsGetInt(void *, const char *, const char *, PetscInt *, PetscBool *f)
{
    if (f) *f = PETSC_FALSE;
    return 0;
}
PetscErrorCode PetscOptionsGetBool(void *, const char *, const char *, PetscBool *, PetscBool *f)
{
    if (f) *f = PETSC_FALSE;
    return 0;
}

/* ---------------- sequential Vec ---------------- */
PetscErrorCode VecCreate(MPI_Comm, Vec *v)
{
    *v = new msx_shim_vec{0, nullptr, true};
    return 0;
}
PetscErrorCode VecSetSizes(Vec v, PetscInt local, PetscInt global)
{
    PetscInt n = global >= 0 ? global : local;
    if (v->own) delete[] v->a;
    v->n = n;
    v->a = new double[n > 0 ? n : 1]();
    v->own = true;
    return 0;
}
PetscErrorCode VecSetFromOptions(Vec) { return 0; }
PetscErrorCode VecCreateSeq(MPI_Comm c, PetscInt n, Vec *v)
{
    VecCreate(c, v);
    return VecSetSizes(*v, n, n);
}
PetscErrorCode VecCreateSeqWithArray(MPI_Comm, PetscInt, PetscInt n, const PetscScalar *a, Vec *v)
{
    *v = new msx_shim_vec{n, const_cast<double *>(a), false};
    return 0;
}
PetscErrorCode VecDuplicate(Vec s, Vec *v)
{
    VecCreate(0, v);
    return VecSetSizes(*v, s->n, s->n);
}
PetscErrorCode VecDestroy(Vec *v)
{
    if (v && *v) {
        if ((*v)->own) delete[] (*v)->a;
        delete *v;
        *v = nullptr;
    }
    return 0;
}
PetscErrorCode VecZeroEntries(Vec v)
{
    for (PetscInt i = 0; i < v->n; i++) v->a[i] = 0.0;
    return 0;
}
static PetscErrorCode check_index(Vec v, PetscInt i)
{
    if (i < 0 || i >= v->n) {
        fprintf(stderr, "petsc-shim: index %d out of range [0,%d)\n", i, v->n);
        abort();
    }
    return 0;
}
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar x, InsertMode m)
{
    check_index(v, i);
    if (m == ADD_VALUES) v->a[i] += x;
    else v->a[i] = x;
    return 0;
}
PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt *ix, const PetscScalar *y, InsertMode m)
{
    for (PetscInt k = 0; k < n; k++) VecSetValue(v, ix[k], y[k], m);
    return 0;
}
PetscErrorCode VecGetValues(Vec v, PetscInt n, const PetscInt *ix, PetscScalar *y)
{
    for (PetscInt k = 0; k < n; k++) { check_index(v, ix[k]); y[k] = v->a[ix[k]]; }
    return 0;
}
PetscErrorCode VecGetArray(Vec v, PetscScalar **a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArray(Vec, PetscScalar **a) { if (a) *a = nullptr; return 0; }
PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
PetscErrorCode VecCopy(Vec x, Vec y)
{
    for (PetscInt i = 0; i < x->n && i < y->n; i++) y->a[i] = x->a[i];
    return 0;
}
/* y = y + alpha*x, element by element */
PetscErrorCode VecAXPY(Vec y, PetscScalar alpha, Vec x)
{
    for (PetscInt i = 0; i < y->n; i++) y->a[i] += alpha * x->a[i];
    return 0;
}
PetscErrorCode VecScale(Vec x, PetscScalar alpha)
{
    for (PetscInt i = 0; i < x->n; i++) x->a[i] *= alpha;
    return 0;
}
/* w = x ./ y */
PetscErrorCode VecPointwiseDivide(Vec w, Vec x, Vec y)
{
    for (PetscInt i = 0; i < w->n; i++) w->a[i] = x->a[i] / y->a[i];
    return 0;
}
PetscErrorCode VecNorm(Vec x, NormType t, PetscReal *r)
{
    double s = 0;
    for (PetscInt i = 0; i < x->n; i++) {
        double v = std::fabs(x->a[i]);
        if (t == NORM_INFINITY) s = v > s ? v : s;
        else if (t == NORM_1) s += v;
        else s += v * v;
    }
    *r = (t == NORM_2 || t == NORM_FROBENIUS) ? std::sqrt(s) : s;
    return 0;
}
PetscErrorCode VecGetSize(Vec x, PetscInt *n) { *n = x->n; return 0; }
PetscErrorCode VecGetOwnershipRange(Vec x, PetscInt *lo, PetscInt *hi)
{
    *lo = 0;
    *hi = x->n;
    return 0;
}

/* LAPACK stand-ins with C linkage; the reference declares the real signatures. */
extern "C" void dsyevr_() { msx_shim_abort("dsyevr_"); }
extern "C" void dgeev_() { msx_shim_abort("dgeev_"); }
extern "C" double dlamch_() { msx_shim_abort("dlamch_"); return 0; }
