/*
 * petsc_shim.h -- minimal single-process stand-in for the parts of PETSc,
 * MPI and LAPACK that MuPhiSim v1.1 declares.  Written for this project; it
 * lets the reference's own sources compile and run sequentially so that the
 * oracle can be checked against the real reference.  TEST INFRASTRUCTURE.
 *
 * Implemented for real: the sequential Vec calls of the explicit solver path
 * (src/solvers/nonlinearSystem.cpp:17-776,1006-1202), PetscInitialize/Finalize
 * and single-rank MPI.  Every other entry point aborts loudly when called.
 */
#ifndef MSX_PETSC_SHIM_H
#define MSX_PETSC_SHIM_H
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>

void msx_shim_abort(const char *name);

/* ---------------- scalar types and enums ---------------- */
typedef int PetscErrorCode;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef enum { INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3 } NormType;
typedef enum { SCATTER_FORWARD = 0, SCATTER_REVERSE = 1 } ScatterMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { PETSC_COPY_VALUES = 0, PETSC_OWN_POINTER = 1, PETSC_USE_POINTER = 2 } PetscCopyMode;
typedef enum { DIFFERENT_NONZERO_PATTERN = 0, SUBSET_NONZERO_PATTERN = 1, SAME_NONZERO_PATTERN = 2 } MatStructure;
typedef int KSPConvergedReason;
typedef const char *KSPType;
typedef const char *PCType;
typedef const char *MatType;
typedef const char *MatSolverType;
#define KSPPREONLY "preonly"
#define KSPGMRES "gmres"
#define KSPCG "cg"
#define PCJACOBI "jacobi"
#define PCNONE "none"
#define PCLU "lu"
#define MATAIJ "aij"
#define MATSOLVERMUMPS "mumps"
#define PETSC_DECIDE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_NULL NULL

/* ---------------- MPI (single rank) ---------------- */
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 1
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_LONG 3
#define MPI_CHAR 4
#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
int MPI_Comm_rank(MPI_Comm, int *r);
int MPI_Comm_size(MPI_Comm, int *s);
int MPI_Barrier(MPI_Comm);
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm);
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm);
int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int, MPI_Comm);
int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rc, const int *dis,
                MPI_Datatype rt, int, MPI_Comm);
int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm);
int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm);
int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *);
int MPI_Init(int *, char ***);
int MPI_Finalize(void);

/* ---------------- PETSc objects ---------------- */
struct msx_shim_vec { PetscInt n; double *a; bool own; };
typedef msx_shim_vec *Vec;
typedef struct msx_shim_opaque *Mat;
typedef struct msx_shim_opaque *KSP;
typedef struct msx_shim_opaque *PC;
typedef struct msx_shim_opaque *IS;
typedef struct msx_shim_opaque *VecScatter;
typedef struct msx_shim_opaque *SNES;
typedef struct msx_shim_opaque *PetscViewer;
typedef struct msx_shim_opaque *PetscObject;
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)

#define CHKERRV(e) do { if (e) { fprintf(stderr, "petsc-shim error %d\n", (int)(e)); return; } } while (0)
#define CHKERRQ(e) do { if (e) { fprintf(stderr, "petsc-shim error %d\n", (int)(e)); return (e); } } while (0)

PetscErrorCode PetscInitialize(int *, char ***, const char *, const char *);
PetscErrorCode PetscFinalize(void);
PetscErrorCode PetscPrintf(MPI_Comm, const char *fmt, ...);
PetscErrorCode PetscOptionsGetInt(void *, const char *, const char *, PetscInt *, PetscBool *);
PetscErrorCode PetscOptionsGetBool(void *, const char *, const char *, PetscBool *, PetscBool *);
inline PetscErrorCode PetscMemcpy(void *d, const void *s, size_t n) { if (n) memcpy(d, s, n); return 0; }
inline PetscErrorCode PetscObjectSetName(void *, const char *) { return 0; }

/* sequential Vec, implemented in petsc_shim.cpp */
PetscErrorCode VecCreate(MPI_Comm, Vec *);
PetscErrorCode VecCreateSeq(MPI_Comm, PetscInt, Vec *);
PetscErrorCode VecCreateSeqWithArray(MPI_Comm, PetscInt, PetscInt, const PetscScalar *, Vec *);
PetscErrorCode VecSetSizes(Vec, PetscInt, PetscInt);
PetscErrorCode VecSetFromOptions(Vec);
PetscErrorCode VecDuplicate(Vec, Vec *);
PetscErrorCode VecDestroy(Vec *);
PetscErrorCode VecZeroEntries(Vec);
PetscErrorCode VecSetValue(Vec, PetscInt, PetscScalar, InsertMode);
PetscErrorCode VecSetValues(Vec, PetscInt, const PetscInt *, const PetscScalar *, InsertMode);
PetscErrorCode VecGetValues(Vec, PetscInt, const PetscInt *, PetscScalar *);
PetscErrorCode VecGetArray(Vec, PetscScalar **);
PetscErrorCode VecRestoreArray(Vec, PetscScalar **);
PetscErrorCode VecAssemblyBegin(Vec);
PetscErrorCode VecAssemblyEnd(Vec);
PetscErrorCode VecCopy(Vec, Vec);
PetscErrorCode VecAXPY(Vec, PetscScalar, Vec);
PetscErrorCode VecScale(Vec, PetscScalar);
PetscErrorCode VecPointwiseDivide(Vec, Vec, Vec);
PetscErrorCode VecNorm(Vec, NormType, PetscReal *);
PetscErrorCode VecGetSize(Vec, PetscInt *);
PetscErrorCode VecGetOwnershipRange(Vec, PetscInt *, PetscInt *);

/* Everything below is outside the explicit path: abort if ever reached. */
#define MSX_SHIM_ABORT_STUB(name) \
    template <class... T> inline PetscErrorCode name(T...) { msx_shim_abort(#name); return 1; }
MSX_SHIM_ABORT_STUB(VecView)
MSX_SHIM_ABORT_STUB(VecScatterCreate)
MSX_SHIM_ABORT_STUB(VecScatterBegin)
MSX_SHIM_ABORT_STUB(VecScatterEnd)
MSX_SHIM_ABORT_STUB(VecScatterDestroy)
MSX_SHIM_ABORT_STUB(ISCreateGeneral)
MSX_SHIM_ABORT_STUB(ISDestroy)
MSX_SHIM_ABORT_STUB(MatCreate)
MSX_SHIM_ABORT_STUB(MatSetSizes)
MSX_SHIM_ABORT_STUB(MatSetType)
MSX_SHIM_ABORT_STUB(MatSetFromOptions)
MSX_SHIM_ABORT_STUB(MatSetUp)
MSX_SHIM_ABORT_STUB(MatSeqAIJSetPreallocation)
MSX_SHIM_ABORT_STUB(MatMPIAIJSetPreallocation)
MSX_SHIM_ABORT_STUB(MatSetValues)
MSX_SHIM_ABORT_STUB(MatGetValues)
MSX_SHIM_ABORT_STUB(MatAssemblyBegin)
MSX_SHIM_ABORT_STUB(MatAssemblyEnd)
MSX_SHIM_ABORT_STUB(MatZeroEntries)
MSX_SHIM_ABORT_STUB(MatDestroy)
MSX_SHIM_ABORT_STUB(MatAXPY)
MSX_SHIM_ABORT_STUB(MatMult)
MSX_SHIM_ABORT_STUB(MatGetLocalSize)
MSX_SHIM_ABORT_STUB(MatView)
MSX_SHIM_ABORT_STUB(KSPCreate)
MSX_SHIM_ABORT_STUB(KSPDestroy)
MSX_SHIM_ABORT_STUB(KSPSetOperators)
MSX_SHIM_ABORT_STUB(KSPSetType)
MSX_SHIM_ABORT_STUB(KSPGetPC)
MSX_SHIM_ABORT_STUB(KSPSetTolerances)
MSX_SHIM_ABORT_STUB(KSPSetFromOptions)
MSX_SHIM_ABORT_STUB(KSPSolve)
MSX_SHIM_ABORT_STUB(KSPGetConvergedReason)
MSX_SHIM_ABORT_STUB(KSPGetIterationNumber)
MSX_SHIM_ABORT_STUB(KSPSetReusePreconditioner)
MSX_SHIM_ABORT_STUB(PCSetType)
MSX_SHIM_ABORT_STUB(PCSetFromOptions)
MSX_SHIM_ABORT_STUB(PCSetReusePreconditioner)
MSX_SHIM_ABORT_STUB(PCFactorSetMatSolverType)

/* LAPACK (dsyevr_, dgeev_, dlamch_) is declared by the reference itself;
 * petsc_shim.cpp defines aborting C-linkage stand-ins. */
#endif
