/*
 * gpu_snes.h -- the PETSc side of the GB300 path: SNES residual and Jacobian
 * callbacks over the C-ABI of include/biofem_gpu.h, for a BioFEM-IA build
 * that links libbiofem_gpu.so.  The callbacks keep the reference's shapes:
 * FormFunctionFEM(SNES, Vec x, Vec R, void *ctx) (main.c:120, 757) and the
 * Jacobian slot of SNESSetJacobian (main.c:462-466), here with an assembled
 * SeqBAIJ(bs = 3) matrix instead of the matrix-free MFFD operator.
 */
#ifndef BIOFEM_GPU_SNES_H
#define BIOFEM_GPU_SNES_H

#include <petscsnes.h>

#include "biofem_gpu.h"

typedef struct {
  BiofemGpuMesh *gpu;     /* the mesh resident on the GPU */
  PetscInt       n_dof;   /* 3 (n_v + n_ghosts): the Vec layout of x and R */
  PetscInt       nnzb;    /* 3x3 blocks of the tangent */
  PetscInt      *rowptr, *colind;   /* SeqBAIJ pattern (block rows = nodes, real then ghost) */
  PetscScalar   *vals;    /* 9 nnzb block values, the storage of J */
  Mat            J;       /* SeqBAIJ(3) over rowptr / colind / vals */
  float         *kf;      /* BIOFEM_FP32_BULK handles: the FP32 values, widened into vals */
} GpuSnesCtx;

/* Prepare the mesh on the GPU (PrepareGpuMesh) and create J.  The handle is
   made with BIOFEM_BLOCK_COL_MAJOR whatever p->block_layout says, so that the
   library writes each block in SeqBAIJ's column-by-column storage.  With
   p->precision = BIOFEM_FP32_BULK the tangent comes in FP32 and is widened
   into J's (PetscScalar) storage after each call. */
PetscErrorCode GpuSnesSetup(GpuSnesCtx *g, const BiofemMeshDesc *d, const BiofemParams *p);
PetscErrorCode GpuSnesDestroy(GpuSnesCtx *g);

/* SNESSetFunction(snes, R, FormFunctionFEMGPU, &g) */
PetscErrorCode FormFunctionFEMGPU(SNES snes, Vec x, Vec R, void *ctx);
/* SNESSetJacobian(snes, g.J, g.J, FormJacobianFEMGPU, &g) */
PetscErrorCode FormJacobianFEMGPU(SNES snes, Vec x, Mat J, Mat P, void *ctx);

#endif
