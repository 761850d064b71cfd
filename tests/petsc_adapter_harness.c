/* Driver of the PETSc adapter (biofem-ia_gb300/petsc/gpu_snes.c) and of the
   library's own SNES-shaped exports, for tests/test_petsc_adapter.py.
   Compiled against the petsc-lite shim (oracle/petsc_lite) and linked to
   libbiofem_gpu.so.  Reads one case from argv[1]:
     int32 n_v, n_elmt, n_edge, sum_bnodes, n_qp, c33_iters, clamp_edge, precision
     double mu, bulk, h0, gamma, pressure
     int32 tri[3 n_elmt]; double xyz0[3 n_v]; int32 n_bnodes[n_edge], bnodes[sum_bnodes];
     double fib[3 n_elmt], gamma_scale[n_elmt]; int32 n_dof; double x[n_dof], v[n_dof]
   and writes to argv[2] (doubles, n_dof each):
     R and J v through FormFunctionFEMGPU / FormJacobianFEMGPU (SeqBAIJ J, MatMult),
     R and K v through the library's FormFunctionFEMGpu / FormJacobianFEMGpu
     (row-major blocks, K v formed here from GetGpuCsrPattern). */
#include <stdio.h>
#include <stdlib.h>

#include "gpu_snes.h"

#define RD(p, sz, n) do { if (fread((p), (sz), (size_t)(n), f) != (size_t)(n)) return 3; } while (0)

int main(int argc, char **argv)
{
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t h[8];
  double r[5];
  RD(h, 4, 8);
  RD(r, 8, 5);
  const int nv = h[0], ne = h[1], nedge = h[2], sb = h[3];
  int32_t *tri = malloc(12 * (size_t)ne), *nb = malloc(4 * (size_t)nedge + 4), *bn = malloc(4 * (size_t)sb + 4);
  double *xyz = malloc(24 * (size_t)nv), *fib = malloc(24 * (size_t)ne), *gs = malloc(8 * (size_t)ne);
  RD(tri, 4, 3 * ne); RD(xyz, 8, 3 * nv); RD(nb, 4, nedge); RD(bn, 4, sb); RD(fib, 8, 3 * ne); RD(gs, 8, ne);
  int32_t ndof;
  RD(&ndof, 4, 1);
  double *x = malloc(8 * (size_t)ndof), *v = malloc(8 * (size_t)ndof);
  RD(x, 8, ndof); RD(v, 8, ndof);
  fclose(f);

  BiofemMeshDesc d = {nv, ne, nedge, tri, xyz, nb, bn, fib, gs, 0};
  BiofemParams p = {0};
  p.n_qp = h[4]; p.c33_subitr_nums = h[5]; p.clamp_edge = h[6]; p.precision = h[7];
  p.mu = r[0]; p.bulk_modulus = r[1]; p.h0 = r[2]; p.gamma = r[3]; p.pressure = r[4];

  /* the adapter: PETSc Vec / SeqBAIJ Mat */
  GpuSnesCtx g = {0};
  if (GpuSnesSetup(&g, &d, &p)) { fprintf(stderr, "setup: %s\n", BiofemGpuLastError()); return 4; }
  if (g.n_dof != ndof) return 5;
  Vec X, R, V, JV;
  VecCreateSeq(PETSC_COMM_SELF, ndof, &X); VecCreateSeq(PETSC_COMM_SELF, ndof, &R);
  VecCreateSeq(PETSC_COMM_SELF, ndof, &V); VecCreateSeq(PETSC_COMM_SELF, ndof, &JV);
  for (int i = 0; i < ndof; i++) { X->a[i] = x[i]; V->a[i] = v[i]; }
  if (FormFunctionFEMGPU(NULL, X, R, &g)) return 6;
  if (FormJacobianFEMGPU(NULL, X, g.J, g.J, &g)) return 7;
  if (MatMult(g.J, V, JV)) return 8;

  /* the library's exports, one more handle with row-major blocks */
  BiofemGpuMesh *m2 = NULL;
  if (PrepareGpuMesh(&d, &p, &m2)) return 9;
  BiofemMeshInfo info;
  GetGpuMeshInfo(m2, &info);
  double *R2 = malloc(8 * (size_t)ndof), *Kv = calloc((size_t)ndof, 8);
  const size_t kvals = 9 * (size_t)info.nnzb;
  const int f32 = p.precision == BIOFEM_FP32_BULK;
  void *K2 = malloc(kvals * (f32 ? 4 : 8));
  int32_t *rp = malloc(4 * (size_t)(info.n_v + info.n_ghosts + 1)), *ci = malloc(4 * (size_t)info.nnzb);
  GetGpuCsrPattern(m2, rp, ci);
  if (FormFunctionFEMGpu(NULL, x, R2, m2)) return 10;
  if (FormJacobianFEMGpu(NULL, x, K2, m2)) return 11;
  for (int i = 0; i < info.n_v + info.n_ghosts; i++)
    for (int k = rp[i]; k < rp[i + 1]; k++)
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
          const double kab = f32 ? (double)((float *)K2)[9 * (size_t)k + 3 * a + b] : ((double *)K2)[9 * (size_t)k + 3 * a + b];
          Kv[3 * i + a] += kab * v[3 * ci[k] + b];
        }
  DestroyGpuMesh(m2);
  GpuSnesDestroy(&g);

  FILE *o = fopen(argv[2], "wb");
  if (!o) return 12;
  fwrite(R->a, 8, (size_t)ndof, o); fwrite(JV->a, 8, (size_t)ndof, o);
  fwrite(R2, 8, (size_t)ndof, o); fwrite(Kv, 8, (size_t)ndof, o);
  fclose(o);
  return 0;
}
