/*
 * petsc-lite: the small slice of the PETSc / MPI C API that BioFEM-IA's
 * hot-path sources (src/active_strain.c, src/math.c, src/bending.c, src/io.c,
 * src/external.c) need in order to compile and run at np = 1.
 *
 * TEST INFRASTRUCTURE ONLY.  This header exists so that the reference's own
 * C files can be compiled unmodified into oracle/_ref/ (see oracle/build_ref.py)
 * and used as the checker for the restated oracle and the CUDA path.  Nothing
 * in the product library includes it.
 *
 * Semantics follow the public PETSc 3.22 / MPI-3 API at one rank:
 *   - PetscInt = int32, PetscReal = PetscScalar = double;
 *   - Vec is a plain host array (VecSetValues ADD/INSERT, assembly is a no-op);
 *   - MPI collectives copy send -> recv (or nothing for MPI_IN_PLACE);
 *   - options come from a process-local table filled by PetscLiteSetOption();
 *   - Mat, viewers and binary I/O return PETSC_ERR_SUP (never on the hot path).
 */
#ifndef PETSC_LITE_PETSCSYS_H
#define PETSC_LITE_PETSCSYS_H

#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int    PetscInt;
typedef int    PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef int    PetscErrorCode;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef void *PetscOptions;
typedef double PetscLogDouble;

/* wall-clock seconds (PETSc's PetscTime) */
static inline PetscErrorCode PetscTime(PetscLogDouble *t)
{
  struct timespec ts_;
  clock_gettime(CLOCK_MONOTONIC, &ts_);
  *t = (PetscLogDouble)ts_.tv_sec + 1e-9 * (PetscLogDouble)ts_.tv_nsec;
  return 0;
}

#define PETSC_SUCCESS 0
#define PETSC_COMM_WORLD ((MPI_Comm)1)
#define PETSC_COMM_SELF  ((MPI_Comm)2)
#define PETSC_NULL NULL
#define PETSC_DECIDE (-1)
#define PetscInt_FMT "d"
#define PETSC_PI 3.14159265358979323846264338327950288419716939937510582
#define PETSC_MAX_REAL 1.7976931348623157e+308

/* error codes (PETSc numbering) */
#define PETSC_ERR_MEM             55
#define PETSC_ERR_SUP             56
#define PETSC_ERR_ORDER           58
#define PETSC_ERR_ARG_WRONG       62
#define PETSC_ERR_ARG_SIZ         60
#define PETSC_ERR_ARG_OUTOFRANGE  63
#define PETSC_ERR_FILE_OPEN       65
#define PETSC_ERR_FILE_READ       66
#define PETSC_ERR_FILE_WRITE      67
#define PETSC_ERR_FILE_UNEXPECTED 79
#define PETSC_ERR_FP              72
#define PETSC_ERR_LIB             76
#define PETSC_ERR_PLIB            77
#define PETSC_ERR_ARG_NULL        85

/* MPI datatypes / ops: the datatype value is its element size in bytes */
#define MPIU_REAL   ((MPI_Datatype)8)
#define MPIU_INT    ((MPI_Datatype)4)
#define MPI_INT     ((MPI_Datatype)4)
#define MPI_DOUBLE  ((MPI_Datatype)8)
#define MPI_SUM     ((MPI_Op)1)
#define MPI_MAX     ((MPI_Op)2)
#define MPI_MIN     ((MPI_Op)3)
#define MPI_IN_PLACE ((void *)1)

typedef enum { PETSC_INT = 0, PETSC_REAL = 1, PETSC_SCALAR = 1 } PetscDataType;

/* ---- error handling ---- */
PetscErrorCode PetscLiteError_(PetscErrorCode code, const char *file, int line, const char *fmt, ...);

#define PetscFunctionBegin
#define PetscFunctionBeginUser
#define PetscFunctionReturn(x) return (x)
#define CHKERRQ(e) do { PetscErrorCode e_lite_ = (e); if (e_lite_) return e_lite_; } while (0)
#define PetscCall(x) do { PetscErrorCode e_lite_ = (x); if (e_lite_) return e_lite_; } while (0)
#define PetscCallMPI(x) PetscCall(x)
#define PetscCheck(cond, comm, code, ...) \
  do { if (!(cond)) return PetscLiteError_((code), __FILE__, __LINE__, __VA_ARGS__); } while (0)
#define SETERRQ(comm, code, ...) return PetscLiteError_((code), __FILE__, __LINE__, __VA_ARGS__)
#define SETERRQ1 SETERRQ

/* ---- memory ---- */
#define PetscMalloc(sz, pp)   (*(void **)(pp) = malloc((size_t)(sz) ? (size_t)(sz) : 1), 0)
#define PetscMalloc1(n, pp)   (*(void **)(pp) = malloc(((size_t)(n) ? (size_t)(n) : 1) * sizeof(**(pp))), 0)
#define PetscCalloc1(n, pp)   (*(void **)(pp) = calloc(((size_t)(n) ? (size_t)(n) : 1), sizeof(**(pp))), 0)
#define PetscFree(p)          (free(p), (p) = NULL, 0)
#define PetscMemzero(p, n)    (memset((p), 0, (size_t)(n)), 0)
#define PetscMemcpy(d, s, n)  (memcpy((d), (s), (size_t)(n)), 0)

/* ---- printing (silent unless PETSC_LITE_VERBOSE is set) ---- */
PetscErrorCode PetscPrintf(MPI_Comm comm, const char *fmt, ...);
PetscErrorCode PetscFPrintf(MPI_Comm comm, FILE *fd, const char *fmt, ...);
PetscErrorCode PetscBarrier(void *obj);

/* ---- real math ---- */
#define PetscSqrtReal(a)  sqrt(a)
#define PetscPowReal(a, b) pow((a), (b))
#define PetscCosReal(a)   cos(a)
#define PetscSinReal(a)   sin(a)
#define PetscExpReal(a)   exp(a)
#define PetscAbsReal(a)   fabs(a)
#define PetscRealPart(a)  (a)
#define PetscMin(a, b)    (((a) < (b)) ? (a) : (b))
#define PetscMax(a, b)    (((a) < (b)) ? (b) : (a))

/* ---- options database ---- */
void PetscLiteSetOption(const char *name, const char *value);
void PetscLiteClearOptions(void);
PetscErrorCode PetscOptionsGetInt(PetscOptions o, const char pre[], const char name[], PetscInt *v, PetscBool *set);
PetscErrorCode PetscOptionsGetReal(PetscOptions o, const char pre[], const char name[], PetscReal *v, PetscBool *set);
PetscErrorCode PetscOptionsGetBool(PetscOptions o, const char pre[], const char name[], PetscBool *v, PetscBool *set);
PetscErrorCode PetscOptionsGetString(PetscOptions o, const char pre[], const char name[], char *v, size_t len, PetscBool *set);

/* ---- MPI at one rank ---- */
int MPI_Comm_rank(MPI_Comm comm, PetscMPIInt *rank);
int MPI_Comm_size(MPI_Comm comm, PetscMPIInt *size);
int MPI_Allreduce(const void *send, void *recv, int n, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *send, void *recv, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Bcast(void *buf, int n, MPI_Datatype t, int root, MPI_Comm comm);
#define MPIU_Allreduce MPI_Allreduce

/* ---- misc ---- */
PetscErrorCode PetscSortIntWithArray(PetscInt n, PetscInt keys[], PetscInt vals[]);

#ifdef __cplusplus
}
#endif

#include "petsc_lite_objects.h"

#endif
