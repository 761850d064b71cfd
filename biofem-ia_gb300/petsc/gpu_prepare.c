/*
 * FE -> C-ABI mesh description for gpu_snes.c: the arrays io.c Input() fills
 * in IBMNodes (io.c:373-479; include/variables.h:44-89) and the active-strain
 * options in fem->act_data (active_strain.c:90-110).  Compiled inside the
 * reference's build (it includes the reference's variables.h).
 */
#include "variables.h"

#include "gpu_snes.h"

extern PetscReal h0;   /* main.c:22, -h0 */

/* pressure: the follower normal pressure P of SurfaceNormalPressure
   (external.c:589); the reference's FExternal (bcs.c:96-285) wires no load,
   so the caller names it (e.g. from an option it adds).  clamp_ring: the
   boundary ring EdgeDirectionalFix clamps in x, y, z (external.c:1706), -1
   for none. */
PetscErrorCode GpuSnesPrepareFE(FE *fem, PetscReal pressure, PetscInt clamp_ring, GpuSnesCtx *g)
{
  IBMNodes *ibm = fem->ibm;
  int32_t *tri, *nb, *bn;
  double *xyz, *fib;

  PetscFunctionBeginUser;
  PetscCall(PetscMalloc1(3 * ibm->n_elmt, &tri));
  PetscCall(PetscMalloc1(3 * ibm->n_v, &xyz));
  PetscCall(PetscMalloc1(3 * ibm->n_elmt, &fib));
  PetscCall(PetscMalloc1(ibm->n_edge, &nb));
  PetscCall(PetscMalloc1(ibm->sum_n_bnodes, &bn));
  for (PetscInt e = 0; e < ibm->n_elmt; e++) {
    tri[3 * e] = (int32_t)ibm->nv1[e]; tri[3 * e + 1] = (int32_t)ibm->nv2[e]; tri[3 * e + 2] = (int32_t)ibm->nv3[e];
    fib[3 * e] = ibm->n_fib[e].x; fib[3 * e + 1] = ibm->n_fib[e].y; fib[3 * e + 2] = ibm->n_fib[e].z;
  }
  for (PetscInt v = 0; v < ibm->n_v; v++) {
    xyz[3 * v] = ibm->x_bp0[v]; xyz[3 * v + 1] = ibm->y_bp0[v]; xyz[3 * v + 2] = ibm->z_bp0[v];
  }
  for (PetscInt r = 0; r < ibm->n_edge; r++) nb[r] = (int32_t)ibm->n_bnodes[r];
  for (PetscInt i = 0; i < ibm->sum_n_bnodes; i++) bn[i] = (int32_t)ibm->bnodes[i];
  BiofemMeshDesc d = {(int32_t)ibm->n_v, (int32_t)ibm->n_elmt, (int32_t)ibm->n_edge, tri, xyz, nb, bn, fib,
                      ibm->gamma_scale, (int32_t)ibm->n_elmt_base};
  BiofemParams p = {0};
  p.n_qp = (int32_t)fem->act_data.n_qp;
  p.c33_subitr_nums = (int32_t)fem->act_data.C33_subitr_nums;
  p.mu = fem->act_data.mu;
  p.bulk_modulus = fem->act_data.K;
  p.h0 = h0;
  p.gamma = fem->act_data.muscle_act_params.gamma;
  p.pressure = pressure;
  p.clamp_edge = (int32_t)clamp_ring;
  p.precision = BIOFEM_FP64;
  p.basis = BIOFEM_BASIS_REFERENCE;
  PetscErrorCode rc = GpuSnesSetup(g, &d, &p);
  PetscCall(PetscFree(tri)); PetscCall(PetscFree(xyz)); PetscCall(PetscFree(fib));
  PetscCall(PetscFree(nb)); PetscCall(PetscFree(bn));
  PetscFunctionReturn(rc);
}
