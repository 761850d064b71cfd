/*
 * PETSc SNES callbacks over the GB300 C-ABI (see gpu_snes.h).  Needs PETSc's
 * headers (or the petsc-lite shim the tests compile it against) and
 * libbiofem_gpu.so; no CUDA header.
 */
#include "gpu_snes.h"

#include <stdlib.h>

#define GPU_SNES_CHECK(rc)                                                                      \
  do {                                                                                          \
    const int rc_ = (rc);                                                                       \
    PetscCheck(!rc_, PETSC_COMM_SELF, rc_, "biofem_gpu: %s", BiofemGpuLastError());              \
  } while (0)

PetscErrorCode GpuSnesSetup(GpuSnesCtx *g, const BiofemMeshDesc *d, const BiofemParams *p)
{
  BiofemParams prm = *p;
  BiofemMeshInfo info;
  int32_t *rp = NULL, *ci = NULL;

  PetscFunctionBeginUser;
  prm.block_layout = BIOFEM_BLOCK_COL_MAJOR;
  GPU_SNES_CHECK(PrepareGpuMesh(d, &prm, &g->gpu));
  GPU_SNES_CHECK(GetGpuMeshInfo(g->gpu, &info));
  g->n_dof = info.n_dof;
  g->nnzb = (PetscInt)info.nnzb;
  const PetscInt nb = info.n_v + info.n_ghosts;
  /* the pattern comes as int32; PetscInt may be wider */
  rp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nb + 1));
  ci = (int32_t *)malloc(sizeof(int32_t) * (size_t)g->nnzb);
  PetscCheck(rp && ci, PETSC_COMM_SELF, PETSC_ERR_MEM, "pattern allocation");
  GPU_SNES_CHECK(GetGpuCsrPattern(g->gpu, rp, ci));
  PetscCall(PetscMalloc1(nb + 1, &g->rowptr));
  PetscCall(PetscMalloc1(g->nnzb, &g->colind));
  PetscCall(PetscCalloc1(9 * g->nnzb, &g->vals));
  g->kf = NULL;
  if (prm.precision == BIOFEM_FP32_BULK) {
    g->kf = (float *)malloc(sizeof(float) * 9 * (size_t)g->nnzb);
    PetscCheck(g->kf, PETSC_COMM_SELF, PETSC_ERR_MEM, "FP32 tangent buffer");
  }
  for (PetscInt i = 0; i <= nb; i++) g->rowptr[i] = rp[i];
  for (PetscInt k = 0; k < g->nnzb; k++) g->colind[k] = ci[k];
  free(rp);
  free(ci);
  PetscCall(MatCreateSeqBAIJWithArrays(PETSC_COMM_SELF, 3, 3 * nb, 3 * nb, g->rowptr, g->colind, g->vals, &g->J));
  PetscFunctionReturn(0);
}

PetscErrorCode GpuSnesDestroy(GpuSnesCtx *g)
{
  PetscFunctionBeginUser;
  PetscCall(MatDestroy(&g->J));
  PetscCall(PetscFree(g->rowptr));
  PetscCall(PetscFree(g->colind));
  PetscCall(PetscFree(g->vals));
  free(g->kf);
  g->kf = NULL;
  if (g->gpu) GPU_SNES_CHECK(DestroyGpuMesh(g->gpu));
  g->gpu = NULL;
  PetscFunctionReturn(0);
}

/* FormFunctionFEM's body (main.c:767-1032) on the GPU: R = Fint - Fext (+ Fdyn),
   clamp rows x - X, ghost rows 0, scaled by 1 / max(|Fext|_inf, 1). */
PetscErrorCode FormFunctionFEMGPU(SNES snes, Vec x, Vec R, void *ctx)
{
  GpuSnesCtx *g = (GpuSnesCtx *)ctx;
  const PetscScalar *xx;
  PetscScalar *rr;
  int rc;

  PetscFunctionBeginUser;
  (void)snes;
  PetscCall(VecGetArrayRead(x, &xx));
  PetscCall(VecGetArray(R, &rr));
  rc = RunGpuResidual(g->gpu, xx, rr);
  PetscCall(VecRestoreArray(R, &rr));
  PetscCall(VecRestoreArrayRead(x, &xx));
  GPU_SNES_CHECK(rc);
  PetscFunctionReturn(0);
}

/* K = dR/dx written by the library straight into P's SeqBAIJ storage, each
   3x3 block column by column (the handle's BIOFEM_BLOCK_COL_MAJOR layout). */
PetscErrorCode FormJacobianFEMGPU(SNES snes, Vec x, Mat J, Mat P, void *ctx)
{
  GpuSnesCtx *g = (GpuSnesCtx *)ctx;
  const PetscScalar *xx;
  PetscScalar *vals;
  int rc;

  PetscFunctionBeginUser;
  (void)snes;
  PetscCall(VecGetArrayRead(x, &xx));
  PetscCall(MatSeqBAIJGetArray(P, &vals));
  rc = RunGpuResidualJacobian(g->gpu, xx, NULL, g->kf ? (void *)g->kf : (void *)vals);
  if (!rc && g->kf)
    for (PetscInt k = 0; k < 9 * g->nnzb; k++) vals[k] = (PetscScalar)g->kf[k];
  PetscCall(MatSeqBAIJRestoreArray(P, &vals));
  PetscCall(VecRestoreArrayRead(x, &xx));
  GPU_SNES_CHECK(rc);
  PetscCall(MatAssemblyBegin(P, MAT_FINAL_ASSEMBLY));
  PetscCall(MatAssemblyEnd(P, MAT_FINAL_ASSEMBLY));
  if (J != P) {
    PetscCall(MatAssemblyBegin(J, MAT_FINAL_ASSEMBLY));
    PetscCall(MatAssemblyEnd(J, MAT_FINAL_ASSEMBLY));
  }
  PetscFunctionReturn(0);
}
