/* Driver of the adapter's FE -> mesh description (biofem-ia_gb300/petsc/
   gpu_prepare.c) for tests/test_petsc_adapter.py: builds the reference's own
   FE with the reference build's ref_setup (oracle/_ref/libbiofem_ref.so),
   then calls GpuSnesPrepareFE, linked to the stand-in library
   (tests/fake_biofem_gpu.c) that records what it receives.  Input as
   tests/petsc_adapter_harness.c (the x and v vectors are not read). */
#include <stdio.h>
#include <stdlib.h>

#include "variables.h"
#include "gpu_snes.h"

extern int ref_setup(int n_v, int n_elmt, const int *tri, const double *xyz0, int n_edge, const int *n_bnodes,
                     const int *bnodes, const double *fib, const double *gamma_scale, int n_qp, int c33_iters,
                     double mu_in, double bulk_in, double h0_in, double gamma_in, double pressure, int clamp_edge0);
extern FE *ref_fem(void);
PetscErrorCode GpuSnesPrepareFE(FE *fem, PetscReal pressure, PetscInt clamp_ring, GpuSnesCtx *g);

#define RD(p, sz, n) do { if (fread((p), (sz), (size_t)(n), f) != (size_t)(n)) return 3; } while (0)

int main(int argc, char **argv)
{
  if (argc != 2) return 2;
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
  fclose(f);
  if (ref_setup(nv, ne, tri, xyz, nedge, nb, bn, fib, gs, h[4], h[5], r[0], r[1], r[2], r[3], r[4], h[6] >= 0))
    return 4;
  GpuSnesCtx g = {0};
  if (GpuSnesPrepareFE(ref_fem(), r[4], h[6], &g)) return 5;
  return GpuSnesDestroy(&g) ? 6 : 0;
}
