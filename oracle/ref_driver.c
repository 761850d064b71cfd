/*
 * np = 1 driver around the reference's OWN hot-path C files.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled together with the unmodified reference
 * sources src/active_strain.c, src/math.c, src/bending.c, src/io.c and
 * src/external.c (and the petsc-lite shim) into oracle/_ref/libbiofem_ref.so by
 * oracle/build_ref.py.  It exists only in the container that holds the
 * reference sources; tests use it to pin the restated oracle
 * (oracle/oracle.cpp) and to generate the committed golden fixtures.
 *
 * Built a second time with src/main.c (FDynamic, xAccVel) and src/material.c
 * (Mass, Damp) into oracle/_ref/libbiofem_ref_dyn.so (-DREF_DRIVER_WITH_MAIN,
 * main renamed, the externals main.c references but the dynamic term never
 * calls resolved by abort stubs that oracle/build_ref.py generates).
 *
 * What is restated here (everything else is the reference's own code):
 *   - main.c globals the compiled files read (main.c:22-77), with the values
 *     the hot path needs (-inverse 0, -bending 0, -curvature 6, tisteps 1);
 *   - FEM_DMPlexGeomSetup / FEM_DMPlexGeomUpdate / FEM_DMPlexGeomBuildNodeMap /
 *     FEM_DMPlexGeomSyncGhostDOFs at one rank, where the cell layout, vertex
 *     layout and DOF map are the identity (dmplex_geom.c:799-1011);
 *   - the init order of the LV loaders (lv_geometry_unstructured.c:239,405-406):
 *     GlobalGhostInit -> IrrVer -> Patch, then geom0, then Init()'s
 *     AreaNormal/GlobalGhost/dA0 (main.c:1439-1452);
 *   - FormFunctionFEM's serial sequence (main.c:757-1032) with FExternal
 *     replaced by the follower SurfaceNormalPressure(P) (external.c:589), or
 *     the dead-load SurfaceConstNormalPressure(P) (external.c:699), and the
 *     clamp EdgeDirectionalFix(0, d) for d = 0,1,2 (external.c:1706).
 */
#include "variables.h"
#include "active_strain.h"

/* ---- main.c globals read by the compiled reference files ---- */
#ifndef REF_DRIVER_WITH_MAIN
/* Built without src/main.c: its globals are restated here.  Built with it
   (oracle/_ref/libbiofem_ref_dyn.so, for FDynamic and xAccVel) main.c defines
   them, and ref_setup assigns the values the hot path needs. */
PetscReal E = 0.0, mu = 0.0, rho = 0.0, h0 = 0.0, dt = 0.0;
PetscReal char_length_x = 1.0, char_length_y = 1.0, char_length_z = 1.0;
PetscInt  dof = 3, contact = 0, ConstitutiveLawNonLinear = 0, curvature = 6;
PetscInt  ti = 0, tistart = 0, tisteps = 1, manufactured = 0, inverse = 0;
PetscInt  legacy_restart_in = 0, lv_geom_process = 0, muscle_activation = 1;
PetscInt  manufactured_fexternal_export = 0, prescribed_force_field = 0;
PetscInt  ressmooth = 0, par_jac = 0, Adam = 0;
PetscInt  n_Fung_Coeffs = 9, n_lin_model_coeffs = 2;
char      in_dir[256] = "./";
char      out_dir[256] = "./";
#else
extern PetscReal E, mu, rho, h0, dt, dampfactor, newmark_gamma;
extern PetscInt  dof, contact, ConstitutiveLawNonLinear, curvature, ti, tistart, tisteps, manufactured, inverse;
extern PetscInt  legacy_restart_in, lv_geom_process, muscle_activation, manufactured_fexternal_export;
extern PetscInt  prescribed_force_field, ressmooth, par_jac, Adam, damping, timeinteg, bending;
#endif
PetscReal manufactured_gamma0 = 0.0, manufactured_T = 1.0;

/* ---- reference functions defined in the compiled files ---- */
extern PetscErrorCode Create(IBMNodes *ibm, FE *fem, PetscInt ibi);
extern PetscErrorCode InitVecs(FE *fem);
extern PetscErrorCode AreaNormal(IBMNodes *ibm);
extern PetscErrorCode GlobalGhostInit(IBMNodes *ibm);
extern PetscErrorCode GlobalGhost(IBMNodes *ibm);
extern PetscErrorCode IrrVer(IBMNodes *ibm);
extern PetscErrorCode Patch(IBMNodes *ibm);
extern PetscErrorCode SurfaceNormalPressure(PetscReal P, FE *fem);
extern PetscErrorCode SurfaceConstNormalPressure(PetscReal P, FE *fem);
extern PetscErrorCode EdgeDirectionalFix(PetscInt edge_n, PetscInt dir, FE *fem, Vec R);

/* ---- never-called externals of the legacy parts of the compiled files ---- */
#define REF_ABORT_STUB(name) \
  PetscErrorCode name() { fprintf(stderr, "oracle/_ref: %s is off the hot path\n", #name); abort(); }
#ifndef REF_DRIVER_WITH_MAIN
REF_ABORT_STUB(BendingNonLinear)
REF_ABORT_STUB(CalcCurvStressStrainxyz)
REF_ABORT_STUB(MembraneNonLinear)
REF_ABORT_STUB(StressLinear)
REF_ABORT_STUB(StressManufactured)
#endif
REF_ABORT_STUB(GhostLoc)
REF_ABORT_STUB(GetManufacturedActiveStrainOptions)
REF_ABORT_STUB(ManufacturedKinematicsAndFExternalSetInitial)

/* ---- DMPlex geometry context at one rank (dmplex_geom.c restated) ---- */
PetscErrorCode FEM_DMPlexGeomUpdate(FE *fem)
{
  /* dmplex_geom.c:881-900: the SF broadcast is a no-op at np = 1 */
  DMPlexGeomCtx *ctx = &fem->geom_ctx;
  for (PetscInt lc = 0; lc < ctx->layout.nLocalCells; ++lc) {
    const PetscInt ec = ctx->layout.orig_cell[lc];
    if (ec < 0 || ec >= fem->ibm->n_elmt) continue;
    PetscCall(ElemUpdateGeomSubdiv(fem, ec));
  }
  return 0;
}

static PetscErrorCode RefGeomCtxSetupNp1_(FE *fem)
{
  /* dmplex_geom.c:799-879 at one rank: identity cell/vertex layout, ghosts
     appended after the real vertices, geom0 once for every cell. */
  DMPlexGeomCtx *ctx = &fem->geom_ctx;
  IBMNodes *ibm = fem->ibm;
  const PetscInt nTotal = ibm->n_v + ibm->n_ghosts;
  memset(ctx, 0, sizeof(*ctx));
  ctx->layout.nLocalCells = ibm->n_elmt;
  PetscMalloc1(ibm->n_elmt, &ctx->layout.orig_cell);
  for (PetscInt ec = 0; ec < ibm->n_elmt; ec++) ctx->layout.orig_cell[ec] = ec;
  ctx->nLocalVerts = ibm->n_v;
  PetscMalloc1(ibm->n_v, &ctx->origVert);
  PetscMalloc1(ibm->n_v, &ctx->ownerRank);
  for (PetscInt v = 0; v < ibm->n_v; v++) { ctx->origVert[v] = v; ctx->ownerRank[v] = 0; }
  PetscMalloc1(nTotal, &ctx->ibm_to_local_idx);
  for (PetscInt v = 0; v < nTotal; v++) ctx->ibm_to_local_idx[v] = v;
  ctx->nOwnedVerts = nTotal;
  for (PetscInt ec = 0; ec < ibm->n_elmt; ec++) PetscCall(ElemUpdateGeom0Subdiv(fem, ec));
  ctx->initialized = PETSC_TRUE;
  return 0;
}

static PetscErrorCode RefBuildNodeMapNp1_(FE *fem)
{
  /* dmplex_geom.c:915-958 at one rank: dof0(v) = 3 v */
  DMPlexGeomCtx *ctx = &fem->geom_ctx;
  const PetscInt nTotal = fem->ibm->n_v + fem->ibm->n_ghosts;
  PetscMalloc1(nTotal, &ctx->ibm_to_global_dof0);
  for (PetscInt v = 0; v < nTotal; v++) ctx->ibm_to_global_dof0[v] = dof * v;
  return 0;
}

static PetscErrorCode RefSyncGhostDOFs_(FE *fem, Vec R)
{
  /* dmplex_geom.c:991-1011 */
  IBMNodes *ibm = fem->ibm;
  PetscReal *RR;
  PetscCall(VecGetArray(R, &RR));
  for (PetscInt gc = 0; gc < ibm->n_ghosts; ++gc) {
    PetscInt li = fem->geom_ctx.ibm_to_local_idx[ibm->n_v + gc];
    RR[li * dof] = 0.0; RR[li * dof + 1] = 0.0; RR[li * dof + 2] = 0.0;
  }
  PetscCall(VecRestoreArray(R, &RR));
  return 0;
}

/* ---- the one body this driver holds ---- */
static FE       g_fem;
static IBMNodes g_ibm;
static int      g_ready = 0;
static double   g_pressure = 0.0;
static int      g_clamp = 1;
static int      g_dead_load = 0;   /* SurfaceConstNormalPressure instead of SurfaceNormalPressure */
static int      g_cart_fib_act = 1;

/* Options of the next ref_setup: dead_load 1 applies the pressure with
   SurfaceConstNormalPressure (external.c:699), iso_act 1 sets -cart_fib_act 0
   (the isotropic active gradient, active_strain.c:1238-1255). */
int ref_set_load_options(int dead_load, int iso_act)
{
  g_dead_load = dead_load != 0;
  g_cart_fib_act = iso_act ? 0 : 1;
  return 0;
}

/* ibm->n_elmt_base of the next ref_setup: 0, or the count of base elements
   (the elements from n_elmt_base on are apex-cap triangles). */
static int g_elmt_base = 0;
int ref_set_elmt_base(int n_elmt_base)
{
  g_elmt_base = n_elmt_base;
  return 0;
}

static void RefFreeAll_(void)
{
  /* The reference never frees a body before exit; the driver leaks the
     previous body on re-setup rather than restate Free().  Tests build a
     handful of meshes per process, so this is bounded. */
  memset(&g_fem, 0, sizeof(g_fem));
  memset(&g_ibm, 0, sizeof(g_ibm));
  g_ready = 0;
}

static void RefSetOptionReal_(const char *name, double v)
{
  char buf[64];
  snprintf(buf, sizeof(buf), "%.17g", v);
  PetscLiteSetOption(name, buf);
}

static void RefSetOptionInt_(const char *name, int v)
{
  char buf[32];
  snprintf(buf, sizeof(buf), "%d", v);
  PetscLiteSetOption(name, buf);
}

/*
 * Build the body from plain arrays (the fields Input() fills, io.c:373-479,
 * 0-based), then initialise it in the LV-loader order and run Init()'s
 * geometric part.  tri: 3*n_elmt, xyz0: 3*n_v, bnodes: sum(n_bnodes).
 */
int ref_setup(int n_v, int n_elmt, const int *tri, const double *xyz0,
              int n_edge, const int *n_bnodes, const int *bnodes,
              const double *fib, const double *gamma_scale,
              int n_qp, int c33_iters, double mu_in, double bulk_in, double h0_in,
              double gamma_in, double pressure, int clamp_edge0)
{
  RefFreeAll_();
  PetscLiteClearOptions();
  RefSetOptionInt_("-num_gaussian_quad_points", n_qp);
  RefSetOptionInt_("-C33_subitr_nums", c33_iters);
  RefSetOptionInt_("-cart_fib_act", g_cart_fib_act);
  RefSetOptionReal_("-muscle_act_gamma", gamma_in);
  RefSetOptionInt_("-gamma_ramp_type", 0);
  RefSetOptionReal_("-bulk_modulus", bulk_in);
  mu = mu_in;
  h0 = h0_in;
  /* the hot path's switches (main.c defaults differ: -inverse 1, no muscle activation) */
  contact = 0; ConstitutiveLawNonLinear = 0; curvature = 6; manufactured = 0; inverse = 0;
  lv_geom_process = 0; muscle_activation = 1; ressmooth = 0; par_jac = 0; Adam = 0;
  ti = 0; tistart = 0; tisteps = 1;
  g_pressure = pressure;
  g_clamp = clamp_edge0;

  IBMNodes *ibm = &g_ibm;
  FE *fem = &g_fem;
  fem->ibm = ibm;
  fem->dof = dof;
  ibm->ibi = 0;
  ibm->n_v = n_v;
  ibm->n_elmt = n_elmt;
  ibm->n_edge = n_edge;
  if (g_elmt_base < 0 || g_elmt_base > n_elmt) return PETSC_ERR_ARG_OUTOFRANGE;
  ibm->n_elmt_base = g_elmt_base;
  int sum = 0;
  for (int e = 0; e < n_edge; e++) sum += n_bnodes[e];
  ibm->n_ghosts = sum; /* one ghost per boundary node per closed ring */
  PetscCall(Create(ibm, fem, 0));

  for (int v = 0; v < n_v; v++) {
    ibm->x_bp[v] = xyz0[3 * v];     ibm->y_bp[v] = xyz0[3 * v + 1];     ibm->z_bp[v] = xyz0[3 * v + 2];
    ibm->x_bp0[v] = ibm->x_bp[v];   ibm->y_bp0[v] = ibm->y_bp[v];       ibm->z_bp0[v] = ibm->z_bp[v];
  }
  for (int ec = 0; ec < n_elmt; ec++) {
    ibm->nv1[ec] = tri[3 * ec]; ibm->nv2[ec] = tri[3 * ec + 1]; ibm->nv3[ec] = tri[3 * ec + 2];
    ibm->n_fib[ec].x = fib[3 * ec]; ibm->n_fib[ec].y = fib[3 * ec + 1]; ibm->n_fib[ec].z = fib[3 * ec + 2];
    ibm->gamma_scale[ec] = gamma_scale[ec];
  }
  ibm->sum_n_bnodes = sum;
  for (int e = 0; e < n_edge; e++) ibm->n_bnodes[e] = n_bnodes[e];
  PetscMalloc1(sum, &ibm->bnodes);
  for (int i = 0; i < sum; i++) ibm->bnodes[i] = bnodes[i];

  /* topology (LV-loader order) */
  PetscCall(GlobalGhostInit(ibm));
  PetscCall(IrrVer(ibm));
  PetscCall(Patch(ibm));

  /* main.c:268-289 */
  PetscCall(InitActStrainProblem(fem, 0));
  PetscCall(RefGeomCtxSetupNp1_(fem));
  PetscCall(InitVecs(fem));
  PetscCall(RefBuildNodeMapNp1_(fem));

  /* Init() geometric part, main.c:1443-1452 (curvature == 6) */
  PetscCall(GlobalGhostInit(ibm));
  PetscCall(AreaNormal(ibm));
  if (ibm->n_ghosts > 0) PetscCall(GlobalGhost(ibm));
  for (int ec = 0; ec < ibm->n_elmt + 2 * ibm->n_ghosts; ec++) {
    ibm->dA0[ec] = ibm->dA[ec];
    ibm->Nf_x[ec] = ibm->nf_x[ec]; ibm->Nf_y[ec] = ibm->nf_y[ec]; ibm->Nf_z[ec] = ibm->nf_z[ec];
  }
  g_ready = 1;
  return 0;
}

/* The body ref_setup built (for tests that hand the reference's FE to code
   written against it, e.g. the PETSc adapter's FE -> mesh description). */
FE *ref_fem(void) { return g_ready ? &g_fem : NULL; }

int ref_sizes(int *n_ghosts, int *n_dof)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  *n_ghosts = g_ibm.n_ghosts;
  *n_dof = dof * (g_ibm.n_v + g_ibm.n_ghosts);
  return 0;
}

/* patch16: 16*n_elmt; ire/val/irv: n_elmt; gtri: 3*(n_elmt+2*n_ghosts);
   xyz0_full: 3*(n_v+n_ghosts) (reference coordinates including ghosts); dA0: n_elmt */
int ref_topology(int *patch16, int *ire, int *val, int *irv, int *gtri, double *xyz0_full, double *dA0)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  IBMNodes *ibm = &g_ibm;
  for (int i = 0; i < 16 * ibm->n_elmt; i++) patch16[i] = ibm->patch[i];
  for (int ec = 0; ec < ibm->n_elmt; ec++) { ire[ec] = ibm->ire[ec]; val[ec] = ibm->val[ec]; irv[ec] = ibm->irv[ec]; dA0[ec] = ibm->dA0[ec]; }
  for (int ec = 0; ec < ibm->n_elmt + 2 * ibm->n_ghosts; ec++) {
    gtri[3 * ec] = ibm->nv1[ec]; gtri[3 * ec + 1] = ibm->nv2[ec]; gtri[3 * ec + 2] = ibm->nv3[ec];
  }
  for (int v = 0; v < ibm->n_v + ibm->n_ghosts; v++) {
    xyz0_full[3 * v] = ibm->x_bp0[v]; xyz0_full[3 * v + 1] = ibm->y_bp0[v]; xyz0_full[3 * v + 2] = ibm->z_bp0[v];
  }
  return 0;
}

/*
 * FormFunctionFEM at np = 1 (main.c:757-1032).  x, R, Fint, Fext are
 * 3*(n_v+n_ghosts) long; Fint/Fext may be NULL.
 */
int ref_residual(const double *x, double *R, double *Fint_out, double *Fext_out)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  FE *fem = &g_fem;
  IBMNodes *ibm = &g_ibm;
  const PetscInt ndof = dof * (ibm->n_v + ibm->n_ghosts);
  Vec Rv;
  PetscCall(VecDuplicate(fem->Fint, &Rv));

  /* main.c:767-793, parallel branch at one rank: owned real vertices only */
  for (PetscInt v = 0; v < ibm->n_v; v++) {
    ibm->x_bp[v] = x[v * dof]; ibm->y_bp[v] = x[v * dof + 1]; ibm->z_bp[v] = x[v * dof + 2];
  }
  PetscCall(AreaNormal(ibm));
  if (ibm->n_ghosts > 0) PetscCall(GlobalGhost(ibm));

  PetscCall(VecSet(fem->Fext, 0.0));
  PetscCall(VecSet(fem->Fint, 0.0));
  PetscCall(VecSet(fem->Fdyn, 0.0));
  PetscCall(VecSet(Rv, 0.0));
  PetscCall(FInternalAct(fem));
  /* FExternal (bcs.c:96) wires no load on this path; the follower pressure
     helper is called in its place. */
  if (g_pressure != 0.0) {
    if (g_dead_load) PetscCall(SurfaceConstNormalPressure(g_pressure, fem));
    else PetscCall(SurfaceNormalPressure(g_pressure, fem));
  }
  PetscCall(VecWAXPY(Rv, -1., fem->Fext, fem->Fint));
  PetscCall(VecAXPY(Rv, 1., fem->Fdyn));
  if (g_clamp) {
    PetscCall(EdgeDirectionalFix(0, 0, fem, Rv));
    PetscCall(EdgeDirectionalFix(0, 1, fem, Rv));
    PetscCall(EdgeDirectionalFix(0, 2, fem, Rv));
  }
  PetscCall(RefSyncGhostDOFs_(fem, Rv));
  PetscReal fext_inf = 0.0;
  PetscCall(VecNorm(fem->Fext, NORM_INFINITY, &fext_inf));
  PetscCall(VecScale(Rv, 1.0 / PetscMax(fext_inf, 1.0)));

  for (PetscInt i = 0; i < ndof; i++) R[i] = Rv->a[i];
  if (Fint_out) for (PetscInt i = 0; i < ndof; i++) Fint_out[i] = fem->Fint->a[i];
  if (Fext_out) for (PetscInt i = 0; i < ndof; i++) Fext_out[i] = fem->Fext->a[i];
  PetscCall(VecDestroy(&Rv));
  return 0;
}

/* Per-element state after the last ref_residual: S^ij (n_qp*9, row-major),
   C33 (n_qp), current geom (24: a1,a2,n,gc1,gc2,Aaa,Abb,Aab). */
int ref_elem_state(int ec, double *S, double *C33, double *geom24)
{
  if (!g_ready || ec < 0 || ec >= g_ibm.n_elmt) return PETSC_ERR_ARG_OUTOFRANGE;
  ElemActData *ead = &g_fem.act_data.elem_act_data[ec];
  for (int q = 0; q < g_fem.act_data.n_qp; q++) {
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) S[9 * q + 3 * i + j] = ead->S[q].Cont[i][j];
    C33[q] = ead->C[q].Cov[2][2];
  }
  const SubdivGeomQP *G = &ead->geom[0];
  const Cmpnts *vs[8] = {&G->ndx21, &G->ndx31, &G->nn, &G->gc1, &G->gc2, &G->Aaa, &G->Abb, &G->Aab};
  for (int k = 0; k < 8; k++) { geom24[3 * k] = vs[k]->x; geom24[3 * k + 1] = vs[k]->y; geom24[3 * k + 2] = vs[k]->z; }
  return 0;
}

/* ---- on-disk formats: the reference's own writers and readers ---- */
extern PetscErrorCode LocationOut(FE *fem, PetscInt ti, PetscInt ibi, const char *out_dir);
extern PetscErrorCode LocationIn(FE *fem, PetscInt ti, PetscInt ibi, const char *out_dir);
extern PetscErrorCode Output(FE *fem, PetscInt ti, PetscInt ibi, const char *out_dir);
extern PetscErrorCode Write3DShellVTK(FE *fem, PetscInt ti, PetscInt ibi, const char *out_dir);
extern PetscErrorCode UpdateElementThickness(FE *fem);

/* LocationOut (io.c:1272) of the given state.  dmplex = 1 keeps the driver's
   DMPlex context (raw ibm-order files), 0 takes the serial VecView path. */
int ref_location_out(const char *dir, int ti_out, int ibi, const double *x, const double *xn, const double *xd,
                     const double *xdd, int dmplex)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  FE *fem = &g_fem;
  const PetscInt ndof = dof * (g_ibm.n_v + g_ibm.n_ghosts);
  Vec v[4] = {fem->x, fem->xn, fem->xd, fem->xdd};
  const double *src[4] = {x, xn, xd, xdd};
  for (int k = 0; k < 4; k++) for (PetscInt i = 0; i < ndof; i++) v[k]->a[i] = src[k][i];
  const PetscBool init = fem->geom_ctx.initialized;
  fem->geom_ctx.initialized = dmplex ? PETSC_TRUE : PETSC_FALSE;
  PetscErrorCode rc = LocationOut(fem, ti_out, ibi, dir);
  fem->geom_ctx.initialized = init;
  return rc;
}

/* LocationIn (io.c:1513) into x, xn, xd, xdd (each 3 (n_v + n_ghosts)). */
int ref_location_in(const char *dir, int ti_in, int ibi, double *x, double *xn, double *xd, double *xdd, int dmplex)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  FE *fem = &g_fem;
  const PetscInt ndof = dof * (g_ibm.n_v + g_ibm.n_ghosts);
  const PetscBool init = fem->geom_ctx.initialized;
  fem->geom_ctx.initialized = dmplex ? PETSC_TRUE : PETSC_FALSE;
  PetscErrorCode rc = LocationIn(fem, ti_in, ibi, dir);
  fem->geom_ctx.initialized = init;
  if (rc) return rc;
  Vec v[4] = {fem->x, fem->xn, fem->xd, fem->xdd};
  double *dst[4] = {x, xn, xd, xdd};
  for (int k = 0; k < 4; k++) for (PetscInt i = 0; i < ndof; i++) dst[k][i] = v[k]->a[i];
  return 0;
}

/* Output (io.c:540) after a residual evaluation at x.  The driver has no
   FDynamic: Fdyn and the velocity xd are the caller's.  The nodal mass is
   Init's (main.c:1465-1470) for density rho_in; IE is zeroed as FormFunctionFEM
   does (main.c:831); lv sets lv_geom_process (the nfib cell field). */
int ref_output_vtk(const char *dir, int ti_out, int ibi, const double *x, const double *Fdyn, const double *xd,
                   double rho_in, int lv)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  FE *fem = &g_fem;
  IBMNodes *ibm = &g_ibm;
  const PetscInt ndof = dof * (ibm->n_v + ibm->n_ghosts);
  double *R = (double *)malloc(sizeof(double) * (size_t)ndof);
  int rc = ref_residual(x, R, NULL, NULL);
  free(R);
  if (rc) return rc;
  for (PetscInt i = 0; i < ndof; i++) { fem->Fdyn->a[i] = Fdyn[i]; fem->xd->a[i] = xd[i]; }
  rho = rho_in;
  for (PetscInt v = 0; v < ibm->n_v; v++) ibm->m[v] = 0.;
  for (PetscInt ec = 0; ec < ibm->n_elmt; ec++) {
    const PetscReal mass = 1. / 3. * rho * ibm->dA0[ec] * h0;
    ibm->m[ibm->nv1[ec]] += mass; ibm->m[ibm->nv2[ec]] += mass; ibm->m[ibm->nv3[ec]] += mass;
  }
  for (PetscInt v = 0; v < ibm->n_v; v++) fem->IE[v] = 0.;
  const PetscInt lv_was = lv_geom_process;
  lv_geom_process = lv;
  rc = Output(fem, ti_out, ibi, dir);
  lv_geom_process = lv_was;
  return rc;
}

/* UpdateElementThickness (active_strain.c:2198) after a residual evaluation at
   x, then Write3DShellVTK (io.c:983) when dir is not NULL. */
int ref_thickness(const char *dir, int ti_out, int ibi, const double *x, double *thickness)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  FE *fem = &g_fem;
  IBMNodes *ibm = &g_ibm;
  const PetscInt ndof = dof * (ibm->n_v + ibm->n_ghosts);
  double *R = (double *)malloc(sizeof(double) * (size_t)ndof);
  int rc = ref_residual(x, R, NULL, NULL);
  free(R);
  if (rc) return rc;
  PetscCall(UpdateElementThickness(fem));
  for (PetscInt ec = 0; ec < ibm->n_elmt; ec++) thickness[ec] = ibm->thickness[ec];
  if (dir) PetscCall(Write3DShellVTK(fem, ti_out, ibi, dir));
  return 0;
}

#ifdef REF_DRIVER_WITH_MAIN
/* ---- the dynamic term: main.c's own FDynamic and xAccVel ---- */
extern PetscErrorCode FDynamic(FE *fem);
extern PetscErrorCode xAccVel(FE *fem);

/* The -dt, -rho, -newmark_gamma, -dampfactor, -timeinteg and -damping
   options (main.c globals). */
int ref_set_dynamics(double dt_in, double rho_in, double newmark_gamma_in, double dampfactor_in, int timeinteg_in,
                     int damping_in)
{
  dt = dt_in; rho = rho_in; newmark_gamma = newmark_gamma_in; dampfactor = dampfactor_in;
  timeinteg = timeinteg_in; damping = damping_in;
  return 0;
}

static void RefSetVec_(Vec v, const double *a, PetscInt n) { for (PetscInt i = 0; i < n; i++) v->a[i] = a[i]; }

/* FDynamic (main.c:1157-1364) at the state (x, xn, xnm1, xd, xdd), each
   3 (n_v + n_ghosts): x goes to ibm->x_bp with the ghost positions by
   GlobalGhost, as FormFunctionFEM does before FDynamic (main.c:767-813);
   Fdyn receives fem->Fdyn.  dmplex = 1 runs it with the driver's DMPlex
   context (the path an active-strain run takes, main.c:326-331: real
   triangles, VecSetValues), 0 the serial path (every triangle, ghost and
   bridging ones included). */
int ref_fdynamic(const double *x, const double *xn, const double *xnm1, const double *xd, const double *xdd,
                 double *Fdyn, int dmplex)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  FE *fem = &g_fem;
  IBMNodes *ibm = &g_ibm;
  const PetscInt ndof = dof * (ibm->n_v + ibm->n_ghosts);
  for (PetscInt v = 0; v < ibm->n_v; v++) {
    ibm->x_bp[v] = x[v * dof]; ibm->y_bp[v] = x[v * dof + 1]; ibm->z_bp[v] = x[v * dof + 2];
  }
  PetscCall(AreaNormal(ibm));
  if (ibm->n_ghosts > 0) PetscCall(GlobalGhost(ibm));
  RefSetVec_(fem->x, x, ndof); RefSetVec_(fem->xn, xn, ndof); RefSetVec_(fem->xnm1, xnm1, ndof);
  RefSetVec_(fem->xd, xd, ndof); RefSetVec_(fem->xdd, xdd, ndof);
  PetscCall(VecSet(fem->Fdyn, 0.0));
  const PetscBool init = fem->geom_ctx.initialized;
  fem->geom_ctx.initialized = dmplex ? PETSC_TRUE : PETSC_FALSE;
  PetscErrorCode rc = FDynamic(fem);
  fem->geom_ctx.initialized = init;
  if (rc) return rc;
  for (PetscInt i = 0; i < ndof; i++) Fdyn[i] = fem->Fdyn->a[i];
  return 0;
}

/* xAccVel (main.c:1367-1412) from the converged x and the state (xn, xd,
   xdd); xd and xdd are updated in place.  dmplex as for ref_fdynamic
   (1: the n_v real nodes, 0: n_v + n_ghosts). */
int ref_xaccvel(const double *x, const double *xn, double *xd, double *xdd, int dmplex)
{
  if (!g_ready) return PETSC_ERR_ORDER;
  FE *fem = &g_fem;
  const PetscInt ndof = dof * (g_ibm.n_v + g_ibm.n_ghosts);
  RefSetVec_(fem->x, x, ndof); RefSetVec_(fem->xn, xn, ndof); RefSetVec_(fem->xd, xd, ndof);
  RefSetVec_(fem->xdd, xdd, ndof);
  const PetscBool init = fem->geom_ctx.initialized;
  fem->geom_ctx.initialized = dmplex ? PETSC_TRUE : PETSC_FALSE;
  PetscErrorCode rc = xAccVel(fem);
  fem->geom_ctx.initialized = init;
  if (rc) return rc;
  for (PetscInt i = 0; i < ndof; i++) { xd[i] = fem->xd->a[i]; xdd[i] = fem->xdd->a[i]; }
  return 0;
}
#endif
