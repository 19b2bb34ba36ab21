/*
 * Opaque PETSc stand-in used ONLY to compile the reference's own C++
 * translation units into the CPU oracle (oracle/_ref).  It is test
 * infrastructure: nothing in the product links it.
 *
 * The oracle harness sets CrsMat::use_petsc = false right after the solid is
 * constructed (module/solid/implicit/implicit_mpm_solid.h:24 sets it true), so
 * the reference takes its native path: BuildDiagonalPreconditioner
 * (module/solver/crsmat.cpp:178) + GPBiCGSafe (module/solver/solver.cpp:19).
 * Every PETSc entry point below therefore aborts if it is ever reached.
 */
#pragma once
#include <mpi.h>
#include <cstdio>
#include <cstdlib>
/* The real petscsys.h pulls in the C headers <stdlib.h> and <math.h>.  In C++
 * these resolve to the library's wrappers, which bring the floating-point
 * overloads of abs() into the global namespace.  module/shape_function.cpp:43
 * calls unqualified abs(double) and reaches petsc.h through
 * material_point.h -> solver/crsmat.h; without these two includes it would
 * bind to int abs(int) and truncate the linear hat function to 1. */
#include <stdlib.h>
#include <math.h>

typedef int PetscInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef int PetscErrorCode;
typedef int PetscMPIInt;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef struct _p_Mat *Mat;
typedef struct _p_Vec *Vec;
typedef struct _p_KSP *KSP;
typedef struct _p_PC *PC;
typedef struct _p_IS *IS;
typedef struct _p_VecScatter *VecScatter;
typedef struct _p_ISLocalToGlobalMapping *ISLocalToGlobalMapping;
typedef const char *KSPType;
typedef const char *PCType;
typedef const char *MatType;
typedef enum { KSP_CONVERGED_ITERATING = 0, KSP_DIVERGED_ITS = -3 } KSPConvergedReason;
typedef enum { INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_INFINITY = 3 } NormType;
typedef enum { SCATTER_FORWARD = 0, SCATTER_REVERSE = 1 } ScatterMode;
typedef enum { PETSC_COPY_VALUES = 0, PETSC_OWN_POINTER = 1, PETSC_USE_POINTER = 2 } PetscCopyMode;
typedef enum {
    MAT_NEW_NONZERO_ALLOCATION_ERR = 1,
    MAT_NEW_NONZERO_LOCATION_ERR = 2,
    MAT_KEEP_NONZERO_PATTERN = 3,
    MAT_IGNORE_OFF_PROC_ENTRIES = 4,
    MAT_NO_OFF_PROC_ENTRIES = 5,
    MAT_SYMMETRIC = 6,
    MAT_ROW_ORIENTED = 7
} MatOption;
typedef enum { PC_COMPOSITE_ADDITIVE = 0, PC_COMPOSITE_MULTIPLICATIVE = 1, PC_COMPOSITE_SCHUR = 4 } PCCompositeType;

#define PETSC_DETERMINE (-1)
#define PETSC_DECIDE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_CURRENT (-2)
#define PETSC_NULLPTR nullptr
#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define PETSC_COMM_SELF MPI_COMM_SELF
#define KSPFGMRES "fgmres"
#define KSPBCGS "bcgs"
#define KSPGMRES "gmres"
#define KSPPREONLY "preonly"
#define PCNONE "none"
#define PCHYPRE "hypre"
#define PCFIELDSPLIT "fieldsplit"
#define PCJACOBI "jacobi"
#define MATAIJ "aij"
#define MATMPIAIJ "mpiaij"
#define MATBAIJ "baij"

static inline PetscErrorCode petsc_stub_unreachable(const char *name) {
    std::fprintf(stderr, "oracle: PETSc stub %s reached (use_petsc must be false)\n", name);
    std::abort();
    return 1;
}

#define ORACLE_PETSC_STUB(name)                                                                                        \
    template <class... A> static inline PetscErrorCode name(A &&...) { return petsc_stub_unreachable(#name); }

ORACLE_PETSC_STUB(PetscInitialize)
ORACLE_PETSC_STUB(PetscFinalize)
ORACLE_PETSC_STUB(PetscOptionsSetValue)
ORACLE_PETSC_STUB(PetscOptionsClearValue)
ORACLE_PETSC_STUB(MatCreate)
ORACLE_PETSC_STUB(MatSetSizes)
ORACLE_PETSC_STUB(MatSetType)
ORACLE_PETSC_STUB(MatSetBlockSize)
ORACLE_PETSC_STUB(MatSetOption)
ORACLE_PETSC_STUB(MatSeqAIJSetPreallocation)
ORACLE_PETSC_STUB(MatMPIAIJSetPreallocation)
ORACLE_PETSC_STUB(MatSetLocalToGlobalMapping)
ORACLE_PETSC_STUB(MatSetValues)
ORACLE_PETSC_STUB(MatSetValuesBlocked)
ORACLE_PETSC_STUB(MatSetValuesLocal)
ORACLE_PETSC_STUB(MatAssemblyBegin)
ORACLE_PETSC_STUB(MatAssemblyEnd)
ORACLE_PETSC_STUB(MatZeroEntries)
ORACLE_PETSC_STUB(MatZeroRowsColumns)
ORACLE_PETSC_STUB(MatZeroRows)
ORACLE_PETSC_STUB(MatMult)
ORACLE_PETSC_STUB(MatDestroy)
ORACLE_PETSC_STUB(MatGetOwnershipRange)
ORACLE_PETSC_STUB(VecCreateMPI)
ORACLE_PETSC_STUB(VecCreateSeq)
ORACLE_PETSC_STUB(VecDuplicate)
ORACLE_PETSC_STUB(VecDestroy)
ORACLE_PETSC_STUB(VecSetValues)
ORACLE_PETSC_STUB(VecAssemblyBegin)
ORACLE_PETSC_STUB(VecAssemblyEnd)
ORACLE_PETSC_STUB(VecZeroEntries)
ORACLE_PETSC_STUB(VecGetArrayRead)
ORACLE_PETSC_STUB(VecRestoreArrayRead)
ORACLE_PETSC_STUB(VecGetArray)
ORACLE_PETSC_STUB(VecRestoreArray)
ORACLE_PETSC_STUB(VecAYPX)
ORACLE_PETSC_STUB(VecPointwiseMult)
ORACLE_PETSC_STUB(VecNorm)
ORACLE_PETSC_STUB(VecSum)
ORACLE_PETSC_STUB(VecSet)
ORACLE_PETSC_STUB(VecScatterCreate)
ORACLE_PETSC_STUB(VecScatterBegin)
ORACLE_PETSC_STUB(VecScatterEnd)
ORACLE_PETSC_STUB(VecScatterDestroy)
ORACLE_PETSC_STUB(ISCreateGeneral)
ORACLE_PETSC_STUB(ISCreateStride)
ORACLE_PETSC_STUB(ISDestroy)
ORACLE_PETSC_STUB(ISLocalToGlobalMappingCreate)
ORACLE_PETSC_STUB(ISLocalToGlobalMappingDestroy)
ORACLE_PETSC_STUB(KSPCreate)
ORACLE_PETSC_STUB(KSPDestroy)
ORACLE_PETSC_STUB(KSPSetType)
ORACLE_PETSC_STUB(KSPSetOperators)
ORACLE_PETSC_STUB(KSPGetPC)
ORACLE_PETSC_STUB(KSPSetTolerances)
ORACLE_PETSC_STUB(KSPSetInitialGuessNonzero)
ORACLE_PETSC_STUB(KSPSetFromOptions)
ORACLE_PETSC_STUB(KSPSetUp)
ORACLE_PETSC_STUB(KSPSolve)
ORACLE_PETSC_STUB(KSPGetIterationNumber)
ORACLE_PETSC_STUB(KSPGetConvergedReason)
ORACLE_PETSC_STUB(KSPSetReusePreconditioner)
ORACLE_PETSC_STUB(PCSetType)
ORACLE_PETSC_STUB(PCReset)
ORACLE_PETSC_STUB(PCSetReusePreconditioner)
ORACLE_PETSC_STUB(PCHYPRESetType)
ORACLE_PETSC_STUB(PCFieldSplitSetFields)
ORACLE_PETSC_STUB(PCFieldSplitSetType)
ORACLE_PETSC_STUB(PCFieldSplitSetBlockSize)
ORACLE_PETSC_STUB(PCFieldSplitSetIS)
ORACLE_PETSC_STUB(PCFieldSplitSetSchurFactType)
ORACLE_PETSC_STUB(PCFieldSplitSetSchurPre)
ORACLE_PETSC_STUB(PCSetUp)
ORACLE_PETSC_STUB(PCFieldSplitGetSubKSP)
ORACLE_PETSC_STUB(PetscFree)
ORACLE_PETSC_STUB(PetscPrintf)

#define PetscCall(x) (void)(x)
#define CHKERRQ(x) (void)(x)
