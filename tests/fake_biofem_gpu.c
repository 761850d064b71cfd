/* A stand-in for libbiofem_gpu.so with the entry points the PETSc adapter
   (biofem-ia_gb300/petsc/) and tests/petsc_adapter_harness.c call, for the
   CPU test of the adapter (tests/test_petsc_adapter.py): no GPU, a small
   tridiagonal block pattern and deterministic, non-symmetric block values
   written in the layout the handle asks for.  PrepareGpuMesh writes what it
   receives to the file named by BIOFEM_FAKE_DUMP (when set), so the test can
   check the adapter's FE -> mesh description copy. */
#include <stdio.h>
#include <stdlib.h>

#include "biofem_gpu.h"

struct BiofemGpuMesh_ {
  int nt, layout;
};

static void dump(const BiofemMeshDesc *d, const BiofemParams *p)
{
  const char *path = getenv("BIOFEM_FAKE_DUMP");
  if (!path) return;
  FILE *f = fopen(path, "wb");
  if (!f) return;
  int sb = 0;
  for (int r = 0; r < d->n_edge; r++) sb += d->n_bnodes[r];
  const int32_t hdr[11] = {d->n_v, d->n_elmt, d->n_edge, sb, p->n_qp, p->c33_subitr_nums, p->clamp_edge,
                           p->precision, p->basis, p->thickness_normal, p->block_layout};
  const double r[5] = {p->mu, p->bulk_modulus, p->h0, p->gamma, p->pressure};
  fwrite(hdr, 4, 11, f); fwrite(r, 8, 5, f);
  fwrite(d->tri, 4, 3 * (size_t)d->n_elmt, f); fwrite(d->xyz0, 8, 3 * (size_t)d->n_v, f);
  fwrite(d->n_bnodes, 4, (size_t)d->n_edge, f); fwrite(d->bnodes, 4, (size_t)sb, f);
  fwrite(d->n_fib, 8, 3 * (size_t)d->n_elmt, f); fwrite(d->gamma_scale, 8, (size_t)d->n_elmt, f);
  fwrite(&d->n_elmt_base, 4, 1, f);
  fclose(f);
}

int PrepareGpuMesh(const BiofemMeshDesc *d, const BiofemParams *p, BiofemGpuMesh **out)
{
  dump(d, p);
  BiofemGpuMesh *m = malloc(sizeof(*m));
  int sb = 0;
  for (int r = 0; r < d->n_edge; r++) sb += d->n_bnodes[r];
  m->nt = d->n_v + sb;
  m->layout = p->block_layout;
  *out = m;
  return 0;
}

int DestroyGpuMesh(BiofemGpuMesh *m) { free(m); return 0; }
const char *BiofemGpuLastError(void) { return "fake"; }

/* rows i: blocks i-1, i, i+1 */
static long long nnzb_of(int nt) { return 3LL * nt - 2; }

int GetGpuMeshInfo(const BiofemGpuMesh *m, BiofemMeshInfo *info)
{
  info->n_v = m->nt; info->n_ghosts = 0; info->n_elmt = 0; info->n_dof = 3 * m->nt; info->n_irregular = 0;
  info->nnzb = nnzb_of(m->nt); info->n_contrib = 0; info->device_bytes = 0; info->precision = BIOFEM_FP64;
  return 0;
}

int GetGpuCsrPattern(const BiofemGpuMesh *m, int32_t *rowptr, int32_t *colind)
{
  int k = 0;
  for (int i = 0; i < m->nt; i++) {
    rowptr[i] = k;
    for (int j = i - 1; j <= i + 1; j++)
      if (j >= 0 && j < m->nt) colind[k++] = j;
  }
  rowptr[m->nt] = k;
  return 0;
}

int RunGpuResidual(BiofemGpuMesh *m, const double *x, double *R)
{
  for (int i = 0; i < 3 * m->nt; i++) R[i] = 2.0 * x[i] - 1.0;
  return 0;
}

/* entry (a, b) of block (i, j): 100 i + 10 j + 3 a + b + 0.5 (distinct, non-symmetric) */
int RunGpuResidualJacobian(BiofemGpuMesh *m, const double *x, double *R, void *Kvals)
{
  double *K = (double *)Kvals;
  if (R) RunGpuResidual(m, x, R);
  long long k = 0;
  for (int i = 0; i < m->nt; i++)
    for (int j = i - 1; j <= i + 1; j++) {
      if (j < 0 || j >= m->nt) continue;
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
          const double v = 100.0 * i + 10.0 * j + 3 * a + b + 0.5;
          K[9 * k + (m->layout == BIOFEM_BLOCK_COL_MAJOR ? 3 * b + a : 3 * a + b)] = v;
        }
      k++;
    }
  return 0;
}

int FormFunctionFEMGpu(void *snes, const double *x, double *R, void *ctx)
{
  (void)snes;
  return RunGpuResidual((BiofemGpuMesh *)ctx, x, R);
}

int FormJacobianFEMGpu(void *snes, const double *x, void *K, void *ctx)
{
  (void)snes;
  return RunGpuResidualJacobian((BiofemGpuMesh *)ctx, x, NULL, K);
}
