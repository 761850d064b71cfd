/*
 * petsc-lite objects: Vec (host array), and opaque Mat / SNES / DM / PetscSF /
 * Tao / PetscViewer handles.  TEST INFRASTRUCTURE ONLY (see petscsys.h).
 */
#ifndef PETSC_LITE_OBJECTS_H
#define PETSC_LITE_OBJECTS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct PetscLiteVec_ { PetscInt n; PetscScalar *a; } *Vec;
typedef struct PetscLiteOpaque_ *Mat;
typedef struct PetscLiteOpaque_ *SNES;
typedef int SNESConvergedReason;   /* an enum in PETSc */
typedef struct PetscLiteOpaque_ *DM;
typedef struct PetscLiteOpaque_ *PetscSF;
typedef struct PetscLiteOpaque_ *Tao;
typedef struct PetscLiteOpaque_ *PetscViewer;
typedef const char *MatType;
#define MATDENSE "dense"

typedef enum { INSERT_VALUES = 0, ADD_VALUES = 1 } InsertMode;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3 } NormType;
typedef enum { FILE_MODE_READ = 0, FILE_MODE_WRITE = 1, FILE_MODE_APPEND = 2 } PetscFileMode;

PetscErrorCode VecCreateSeq(MPI_Comm c, PetscInt n, Vec *v);
PetscErrorCode VecCreateMPI(MPI_Comm c, PetscInt nlocal, PetscInt N, Vec *v);
PetscErrorCode VecDuplicate(Vec x, Vec *y);
PetscErrorCode VecDestroy(Vec *v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecCopy(Vec x, Vec y);
PetscErrorCode VecGetArray(Vec v, PetscScalar **a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a);
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt idx[], const PetscScalar y[], InsertMode m);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
PetscErrorCode VecNorm(Vec v, NormType t, PetscReal *r);
PetscErrorCode VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y);
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x);
PetscErrorCode VecScale(Vec x, PetscScalar a);
PetscErrorCode VecGetSize(Vec v, PetscInt *n);
PetscErrorCode VecGetOwnershipRange(Vec v, PetscInt *lo, PetscInt *hi);
PetscErrorCode VecView(Vec v, PetscViewer w);
PetscErrorCode VecLoad(Vec v, PetscViewer w);

PetscErrorCode PetscViewerBinaryOpen(MPI_Comm c, const char name[], PetscFileMode m, PetscViewer *w);
PetscErrorCode PetscViewerDestroy(PetscViewer *w);
PetscErrorCode PetscViewerBinaryGetDescriptor(PetscViewer w, int *fd);
PetscErrorCode PetscBinaryWrite(int fd, const void *p, PetscInt n, PetscDataType t);
PetscErrorCode PetscBinaryRead(int fd, void *p, PetscInt n, PetscInt *count, PetscDataType t);
PetscErrorCode PetscRealView(PetscInt n, const PetscReal v[], PetscViewer w);

PetscErrorCode MatCreate(MPI_Comm c, Mat *m);
PetscErrorCode MatSetSizes(Mat m, PetscInt a, PetscInt b, PetscInt c, PetscInt d);
PetscErrorCode MatSetFromOptions(Mat m);
PetscErrorCode MatSetType(Mat m, MatType t);
PetscErrorCode MatSetUp(Mat m);
PetscErrorCode MatZeroEntries(Mat m);
PetscErrorCode MatGetSize(Mat m, PetscInt *a, PetscInt *b);
PetscErrorCode MatCreateSeqDense(MPI_Comm c, PetscInt a, PetscInt b, PetscScalar *d, Mat *m);

/* An array-backed sequential block matrix with PETSc SeqBAIJ's storage:
   block rows by a CSR pattern (i, j over blocks), each bs x bs block's values
   column by column (a[k bs^2 + c bs + r] is row r, column c of block k). */
typedef enum { MAT_FINAL_ASSEMBLY = 0, MAT_FLUSH_ASSEMBLY = 1 } MatAssemblyType;
PetscErrorCode MatCreateSeqBAIJWithArrays(MPI_Comm c, PetscInt bs, PetscInt m, PetscInt n, PetscInt i[], PetscInt j[],
                                          PetscScalar a[], Mat *mat);
PetscErrorCode MatSeqBAIJGetArray(Mat A, PetscScalar **a);
PetscErrorCode MatSeqBAIJRestoreArray(Mat A, PetscScalar **a);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t);
PetscErrorCode MatMult(Mat A, Vec x, Vec y);
PetscErrorCode MatDestroy(Mat *A);

#ifdef __cplusplus
}
#endif
#endif
