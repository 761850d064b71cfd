/*
 * biofem_gpu.h -- C-ABI of the GB300 (sm_103a) element residual / tangent /
 * assembly path for BioFEM-IA's active-strain Kirchhoff-Love shell.
 *
 * Shaped like the reference's GPU bridge, include/cuda_bridge.h:10-15
 * (InitCudaWorkspace / DestroyCudaWorkspace / PrepareCudaHostWorkspace /
 * Run*Kernel, all extern "C", PetscErrorCode return), but taking plain
 * arrays instead of FE* so that callers need neither PETSc nor CUDA headers.
 * A PETSc build binds these from its SNES callbacks.
 *
 * Conventions
 *   - Every entry point returns an int that is PetscErrorCode-compatible:
 *     0 = success, otherwise a PETSc error number (56 unsupported, 58 wrong
 *     order, 62 bad argument, 63 out of range, 72 floating point, 76 CUDA
 *     library error, 77 internal).  BiofemGpuLastError() gives the message.
 *   - Index type is int32 (PetscInt default), reals are double (PetscReal).
 *   - Vectors use the reference's Vec layout: 3*(n_v + n_ghosts) entries,
 *     node-major (x, y, z), real nodes first, then one ghost node per
 *     boundary-ring node (io.c:329-345, dmplex_geom.c:836-857).
 *   - The tangent is a 3x3-block CSR (BSR) matrix over the same node
 *     numbering.  Block values are row-major within the block, or column-major
 *     (PETSc SeqBAIJ storage) when BiofemParams.block_layout asks for it.
 *   - Host-side API is single-threaded per mesh handle; different handles may
 *     be driven from different host threads (error messages are per thread).
 */
#ifndef BIOFEM_GPU_H
#define BIOFEM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mesh arrays, 0-based, as io.c Input() fills IBMNodes (io.c:373-479;
   include/variables.h:44-89).  Boundary rings are closed loops with one ghost
   node per ring node (bending.c:1670-1757). */
typedef struct {
  int32_t n_v;                 /* real nodes */
  int32_t n_elmt;              /* real triangles */
  int32_t n_edge;              /* boundary rings */
  const int32_t *tri;          /* 3*n_elmt corners (nv1, nv2, nv3) */
  const double  *xyz0;         /* 3*n_v reference coordinates (x_bp0, y_bp0, z_bp0 interleaved) */
  const int32_t *n_bnodes;     /* n_edge ring lengths */
  const int32_t *bnodes;       /* sum(n_bnodes) ring node ids in ring order */
  const double  *n_fib;        /* 3*n_elmt fibre directions (ibm->n_fib) */
  const double  *gamma_scale;  /* n_elmt per-element activation multiplier (ibm->gamma_scale) */
  int32_t n_elmt_base;         /* ibm->n_elmt_base: 0, or the count of subdivision elements, the
                                  elements from it on being flat apex-cap triangles (bending.c:1204-1294,
                                  active_strain.c:444-470, 1801-1853) */
} BiofemMeshDesc;

/* Options of the path (active_strain.c:90-110, main.c:190-252). */
typedef struct {
  int32_t n_qp;                /* -num_gaussian_quad_points, 1..6 (6 is an extension) */
  int32_t c33_subitr_nums;     /* -C33_subitr_nums, >= 1 */
  double  mu;                  /* -mu */
  double  bulk_modulus;        /* -bulk_modulus */
  double  h0;                  /* -h0 */
  double  gamma;               /* -muscle_act_gamma (gamma_ramp_type 0) */
  double  pressure;            /* follower normal pressure P (external.c:589), 0 = none */
  int32_t clamp_edge;          /* ring clamped in x,y,z by EdgeDirectionalFix (external.c:1706); -1 = none */
  int32_t precision;           /* BIOFEM_FP64 or BIOFEM_FP32_BULK */
  int32_t basis;               /* BIOFEM_BASIS_REFERENCE (default) or BIOFEM_BASIS_EXACT */
  int32_t thickness_normal;    /* 0 (reference): g_alpha = a_alpha + theta3 a3,alpha with a3,alpha the derivative of
                                  a1 x a2 over |a1 x a2| (active_strain.c:745-762, 896-982); 1 (extension): its
                                  tangential part n,alpha only.  The two agree where |a1 x a2| is uniform; on
                                  non-uniform patches (ghost-reflected boundary patches of a fine mesh) the
                                  normal part J,alpha/J n folds the thickness points once h << h0 */
  int32_t block_layout;        /* storage of each 3x3 block of the tangent the RunGpuResidualJacobian* calls
                                  return: BIOFEM_BLOCK_ROW_MAJOR (0, default) or BIOFEM_BLOCK_COL_MAJOR (1, the
                                  layout of PETSc SeqBAIJ storage, so MatSeqBAIJGetArray's array can be passed) */
  int32_t pressure_kind;       /* BIOFEM_PRESSURE_FOLLOWER (0, default): SurfaceNormalPressure, the current normal
                                  and area (external.c:589-624), with its load stiffness in K;
                                  BIOFEM_PRESSURE_DEAD (1): SurfaceConstNormalPressure, the reference normal and
                                  area dA0 (external.c:699-730), no load stiffness */
  int32_t activation_kind;     /* BIOFEM_ACTIVATION_FIBRE (0, default; -cart_fib_act 1): Fa = I - gamma f f^T;
                                  BIOFEM_ACTIVATION_ISOTROPIC (1; -cart_fib_act 0): Fa = diag(1 - gamma,
                                  1 - gamma, 1/(1 - gamma)^2) in the Cartesian basis (active_strain.c:1238-1255) */
} BiofemParams;

enum { BIOFEM_FP64 = 0, BIOFEM_FP32_BULK = 1 };
enum { BIOFEM_BLOCK_ROW_MAJOR = 0, BIOFEM_BLOCK_COL_MAJOR = 1 };
enum { BIOFEM_PRESSURE_FOLLOWER = 0, BIOFEM_PRESSURE_DEAD = 1 };
enum { BIOFEM_ACTIVATION_FIBRE = 0, BIOFEM_ACTIVATION_ISOTROPIC = 1 };
/* Centroid basis-derivative tables.  REFERENCE: the four-decimal values of
   active_strain.c:69-88 (parity with the reference).  EXACT (extension): the
   rationals they round; the four-decimal second-derivative rows sum to
   -1e-4, -1e-4, 2e-4 instead of 0, so a flat sheet acquires a curvature
   ~1e-4 |x| / h^2 at the thickness points, which folds them once the mesh
   is much finer than the shell (h below ~h0/4). */
enum { BIOFEM_BASIS_REFERENCE = 0, BIOFEM_BASIS_EXACT = 1 };

typedef struct {
  int32_t n_v, n_ghosts, n_elmt, n_dof;
  int32_t n_irregular;         /* elements on the one-step-subdivision branch */
  int64_t nnzb;                /* 3x3 blocks in the tangent pattern */
  int64_t n_contrib;           /* element-block contributions (assembly map size) */
  int64_t device_bytes;        /* device memory held by the handle: mesh arrays, and once a Newton solve has
                                  run, its GMRES work and multigrid hierarchy */
  int32_t precision;           /* BIOFEM_FP64 or BIOFEM_FP32_BULK */
} BiofemMeshInfo;

typedef struct BiofemGpuMesh_ BiofemGpuMesh;

/* Replaces InitCudaWorkspace (cuda_bridge.h:10): selects the device, creates
   the stream.  Idempotent. */
int InitGpuWorkspace(void);
/* Replaces DestroyCudaWorkspace (cuda_bridge.h:11): frees every mesh handle
   still alive and the stream. */
int DestroyGpuWorkspace(void);

/* Replaces PrepareCudaHostWorkspace (cuda_bridge.h:12) and the one-time
   geometry of FEM_DMPlexGeomSetup (dmplex_geom.c:799-879): builds the
   subdivision topology (GlobalGhostInit/IrrVer/Patch, bending.c:1188-1757),
   dA0 (main.c:1447-1452), the reference geometry of every element, the
   assembly maps and the tangent pattern, and uploads everything. */
int PrepareGpuMesh(const BiofemMeshDesc *mesh, const BiofemParams *params, BiofemGpuMesh **out);
/* Same, with the handle's setup, host-array calls and teardown ordered on
   `stream` (cudaStream_t; NULL = the workspace stream).  Device memory comes
   from the stream-ordered pool, so handles can be created and destroyed on
   concurrent streams without synchronising the device. */
int PrepareGpuMeshOnStream(const BiofemMeshDesc *mesh, const BiofemParams *params, void *stream, BiofemGpuMesh **out);
int DestroyGpuMesh(BiofemGpuMesh *m);
int GetGpuMeshInfo(const BiofemGpuMesh *m, BiofemMeshInfo *info);

/* Host copies of the topology the handle uses (same layout as IBMNodes):
   patch 16*n_elmt, ire/val/irv n_elmt, gtri 3*(n_elmt+2*n_ghosts),
   xyz0_full 3*(n_v+n_ghosts), dA0 n_elmt.  Any pointer may be NULL. */
int GetGpuTopology(const BiofemGpuMesh *m, int32_t *patch, int32_t *ire, int32_t *val, int32_t *irv,
                   int32_t *gtri, double *xyz0_full, double *dA0);
/* Ghost rule of every ghost node g (GlobalGhostInit/GlobalGhost,
   bending.c:1670-1814): x_g = x[nv2] + x[nv1] - x[nv3]; ghost3 holds
   (nv1, nv2, nv3) per ghost, 3*n_ghosts entries. */
int GetGpuGhostMap(const BiofemGpuMesh *m, int32_t *ghost3);
/* Tangent pattern: rowptr (n_v+n_ghosts+1), colind (nnzb). */
int GetGpuCsrPattern(const BiofemGpuMesh *m, int32_t *rowptr, int32_t *colind);

/* FormFunctionFEM body (main.c:757-1032): R(x) with host arrays of n_dof
   entries; copies in, computes, copies out.  Replaces the CPU residual the
   reference's SNES callback evaluates. */
int RunGpuResidual(BiofemGpuMesh *m, const double *x, double *R);
/* R(x) and the tangent K = dR/dx (new: the reference is matrix-free,
   main.c:464-466).  Kvals has 9*nnzb entries: double for a BIOFEM_FP64
   handle, float for a BIOFEM_FP32_BULK handle (whose residual runs in
   float-float numbers on the FP32 pipe and whose tangent is formed in FP32
   on patch-local shifted coordinates).
   R may be NULL. */
int RunGpuResidualJacobian(BiofemGpuMesh *m, const double *x, double *R, void *Kvals);

/* Device-resident variants: pointers are device memory, work is enqueued on
   `stream` (a cudaStream_t; NULL = the CUDA default stream) and not
   synchronised.  BiofemGpuSync() waits and reports device-side errors. */
int RunGpuResidualDevice(BiofemGpuMesh *m, const double *d_x, double *d_R, void *stream);
int RunGpuResidualJacobianDevice(BiofemGpuMesh *m, const double *d_x, double *d_R, void *d_Kvals, void *stream);
int BiofemGpuSync(BiofemGpuMesh *m, void *stream);

/* Residual for callers that cannot allocate device memory when they call:
   a serving loop or host code that has reserved a fixed HBM budget (its own
   pool) and must not have the library reach cudaMalloc, which can fail under
   the budget, fragments the pool and synchronises the device.  No
   counterpart in the reference.  Same result as RunGpuResidualDevice for a
   prepared handle (the same element kernel: FP64, or float-float for an
   FP32-bulk handle); d_x / d_R are device pointers the caller owns; allocates
   nothing.  The per-call work arrays live in one fixed 8 MiB device array
   (1,048,576 doubles) that each GPU loading the library holds until exit:
   meshes needing more than 4*(n_v+n_ghosts) + 51*n_elmt + 1 doubles (about
   19,000 triangles) are rejected with error 63.  All calls share that array:
   calls that overlap on the GPU race and must be serialised.  The first call
   on a device looks up the array's address (once per device); make it before
   any stream capture.  The handle's device must be current (else error 62).
   Element errors (a vanishing CC3333) come back, as for the other device
   variants, through BiofemGpuSync(handle, stream) as error 72. */
int RunGpuResidualNoAlloc(BiofemGpuMesh *m, const double *d_x, double *d_R, void *stream);

/* One quasi-static load step: Newton on R(x) = 0 with the assembled tangent
   (new: replaces the matrix-free SNES newtonls/MFFD/GMRES solve of
   main.c:461-551).  Linear solves: restarted GMRES(gmres_restart) with right
   block-Jacobi(3x3) preconditioning, FP64 vectors on the device.  x (host,
   n_dof entries) holds the start on entry and the solution on exit. */
typedef struct {
  double  rtol;              /* stop when ||R|| <= rtol ||R0||  (1e-10) */
  double  atol;              /* or ||R|| <= atol (0 = off) */
  int32_t max_newton;        /* Newton iterations (20) */
  int32_t gmres_restart;     /* Krylov subspace size m, 1..200; 0 = 30 below 50k DOFs, else 100 */
  int32_t gmres_max_it;      /* total GMRES iterations per solve (20000) */
  double  gmres_rtol;        /* relative linear tolerance (1e-9) */
  int32_t line_search;       /* 1 = backtracking on ||R|| */
  int32_t preconditioner;    /* BIOFEM_PC_AMG (default) or BIOFEM_PC_BJACOBI */
  int32_t forcing;           /* 0: every linear solve to gmres_rtol; 1: Eisenstat-Walker (version 2) forcing
                                terms, as PETSc's -snes_ksp_ew: eta_0 = 0.3, eta_k = (|R_k|/|R_k-1|)^1.618,
                                safeguarded, at most 0.9, at least gmres_rtol and 0.5 (Newton target)/|R_k| */
} BiofemNewtonOptions;

/* Preconditioners of the Newton linear solve: smoothed-aggregation multigrid
   (rigid-body near-null space, FP32 V-cycle) or block-Jacobi on the 3x3
   diagonal blocks.  The reference's matrix-free SNES has neither (no
   assembled operator to precondition with). */
#define BIOFEM_PC_AMG 0
#define BIOFEM_PC_BJACOBI 1

typedef struct {
  int32_t newton_its, gmres_its_total, gmres_its_last, residual_evals, jacobian_evals, converged;
  double  r0, rfinal, gmres_relres_last;
  double  rhist[64];         /* ||R|| after each Newton iteration (rhist[0] = ||R0||) */
} BiofemNewtonStats;

void BiofemNewtonDefaults(BiofemNewtonOptions *o);
int RunGpuNewtonSolve(BiofemGpuMesh *m, double *x, const BiofemNewtonOptions *opt, BiofemNewtonStats *stats);
/* Same on a device vector d_x (updated in place). */
int RunGpuNewtonSolveDevice(BiofemGpuMesh *m, double *d_x, const BiofemNewtonOptions *opt, BiofemNewtonStats *stats,
                            void *stream);

/* Dynamic term and time stepping (main.c:420-567, FDynamic main.c:1157-1290,
   Mass/Damp material.c:100-139, xAccVel main.c:1367-1412).  With dynamics
   on, R = (Fint - Fext) + Fdyn and K gains d Fdyn / dx on the diagonal:
   per element and corner M = rho h0 A0 / 3 (A0 the flat reference area),
   C = dampfactor M when damping, and with beta = (gamma_nm + 1/2)^2 / 4
     Newmark (timeinteg 0): Fd = M M1 x + C C1 x - M (M1 xn + M2 xd + M3 xdd)
                                  - C (C1 xn + C2 xd + C3 xdd),
     central (timeinteg 1): Fd = M (x - 2 xn + xnm1) / dt^2 + C (x - xn) / dt.
   The corner sum runs over every triangle, ghost and bridging triangles
   included (the serial FDynamic loop, main.c:1293).  SetGpuDynamics(m, NULL)
   switches the term off; each SetGpuDynamics call restarts the state
   (3*(n_v+n_ghosts) each) at xn = xnm1 = the reference coordinates and
   xd = xdd = 0 (Init, main.c:1515-1540); the state calls set or read it (NULL
   entries are skipped).  RunGpuDynamicUpdate(m, x) ends a step from the
   converged x: xAccVel's acceleration and velocity updates (main.c:1367-1412),
   then xnm1 <- xn, xn <- x.  SetGpuElementGamma(m, g) recomputes the per-element activation
   constants with g[e] in place of gamma * gamma_scale[e] (the value of
   GammaOfTimeDelayed times gamma_scale, active_strain.c:1156-1212). */
typedef struct {
  double  dt, rho, newmark_gamma, dampfactor;
  int32_t timeinteg, damping;
} BiofemDynParams;
int SetGpuDynamics(BiofemGpuMesh *m, const BiofemDynParams *params);
int SetGpuDynamicState(BiofemGpuMesh *m, const double *xn, const double *xnm1, const double *xd, const double *xdd);
int GetGpuDynamicState(BiofemGpuMesh *m, double *xn, double *xnm1, double *xd, double *xdd);
int RunGpuDynamicUpdate(BiofemGpuMesh *m, const double *x);
int SetGpuElementGamma(BiofemGpuMesh *m, const double *gamma_e);

/* Output quantities of a state x (host arrays, 3*(n_v+n_ghosts) each): the
   unscaled node forces Fint, Fext and Fdyn of FormFunctionFEM
   (main.c:829-845; Fdyn zero while the dynamic term is off) and the residual
   R; any output pointer may be NULL. */
int RunGpuResidualParts(BiofemGpuMesh *m, const double *x, double *R, double *Fint, double *Fext, double *Fdyn);
/* Wall thickness per element of a state x (UpdateElementThickness,
   active_strain.c:2198-2224): h0 sqrt(mean over the thickness points of C33
   after the sub-iterations); n_elmt values. */
int RunGpuElementThickness(BiofemGpuMesh *m, const double *x, double *thickness);

/* On-disk formats (host only; formats.cpp).
   Checkpoints: LocationOut / LocationIn (io.c:1272-1376, 1513-1640) write and
   read "<dir>/<tag><ibi>_<ti>.dat" for tag x, xn, xd, xdd, each n_dof =
   3*(n_v+n_ghosts) doubles in original-vertex order, big-endian:
   BIOFEM_CKPT_VERTEX_ORDER the values alone (the DMPlex path, any process
   count), BIOFEM_CKPT_VEC a PETSc VecView record (int32 classid 1211214, int32
   length, values; the serial path).  BiofemLocationIn accepts both (and a
   VecView record with 64-bit header integers), choosing by the file size. */
#define BIOFEM_CKPT_VERTEX_ORDER 0
#define BIOFEM_CKPT_VEC 1
int BiofemLocationOut(const char *dir, int32_t ti, int32_t ibi, int64_t n_dof, const double *x, const double *xn,
                      const double *xd, const double *xdd, int32_t layout);
int BiofemLocationIn(const char *dir, int32_t ti, int32_t ibi, int64_t n_dof, double *x, double *xn, double *xd,
                     double *xdd);
/* "<dir>/surface<ibi>_<ti>.vtk" (Output, io.c:540-964, with muscle
   activation on and no contact): points x, triangles, point data contact (0),
   m, IE (0), disp = x - X, Fint, Fext, Fdyn, Fcnt (0), u = xd, Res = Fint -
   Fext + Fdyn; cell data nfib (when fib is given, the LV loader's field), dA
   (flat area on x), dA0 (given, or the flat area on X), gamma.  Node arrays
   hold the n_v real nodes; NULL force / velocity / mass arrays print zeros. */
typedef struct {
  int32_t n_v, n_elmt;
  const int32_t *tri;      /* 3 n_elmt corners */
  const double *x, *X;     /* 3 n_v current and reference positions */
  const double *mass;      /* n_v lumped mass (Init, main.c:1465-1470) */
  const double *Fint, *Fext, *Fdyn, *xd;   /* 3 n_v each */
  const double *dA0;       /* n_elmt */
  const double *gamma_e;   /* n_elmt activation of the step (required) */
  const double *fib;       /* 3 n_elmt fibre directions */
} BiofemSurfaceFields;
int BiofemWriteSurfaceVTK(const char *dir, int32_t ti, int32_t ibi, const BiofemSurfaceFields *fields);
/* "<dir>/shell3d<ibi>_<ti>.vtk" (Write3DShellVTK, io.c:983-1064): one layer of
   wedges, each surface node offset by half its node-averaged thickness along
   its area-weighted normal. */
int BiofemWriteShell3dVTK(const char *dir, int32_t ti, int32_t ibi, int32_t n_v, int32_t n_elmt, const int32_t *tri,
                          const double *x, const double *thickness_e);

/* Serving loop for load-step requests (new; the reference runs each case as
   a separate batch job, bin/biofem:352-456).  Continuous batching: requests
   are admitted first-fit in arrival order whenever one of max_slots slots is
   free and their device-memory estimate fits hbm_budget_bytes; admitted
   requests run concurrently on their own streams (mesh setup + Newton load
   step), and finished ones free their slot and memory immediately.
   ServeSubmit copies the request; requests that can never fit the budget are
   refused with 55.  ServeWait blocks for one ticket, returns its x, Newton
   statistics and the submit / admission / finish times (seconds since
   ServeCreate).  ServeStatsGet: in_use, peak_in_use bytes, active,
   peak_active, queued, completed. */
typedef struct BiofemServe_ BiofemServe;
int ServeCreate(int64_t hbm_budget_bytes, int32_t max_slots, BiofemServe **out);
int ServeSubmit(BiofemServe *s, const BiofemMeshDesc *mesh, const BiofemParams *params,
                const BiofemNewtonOptions *opt, const double *x0, int64_t *ticket);
int ServeWait(BiofemServe *s, int64_t ticket, double *x_out, BiofemNewtonStats *stats, double times[3]);
int ServeStatsGet(BiofemServe *s, int64_t out[6]);
int ServeDestroy(BiofemServe *s);
/* Device-memory estimate the serving loop admits a request by. */
int BiofemServeEstimateBytes(int32_t n_v, int32_t n_elmt, int32_t n_ghosts, int32_t precision,
                             int32_t gmres_restart, int64_t *bytes);

/* SNES-callback-shaped wrappers (main.c:120 FormFunctionFEM(SNES, Vec, Vec,
   void*) and the Jacobian slot SNESSetJacobian, main.c:462-466) taking host
   arrays; ctx is the BiofemGpuMesh*.  `snes` is passed through unused. */
int FormFunctionFEMGpu(void *snes, const double *x, double *R, void *ctx);
int FormJacobianFEMGpu(void *snes, const double *x, void *Kvals, void *ctx);

/* Per-kernel CUDA-event timing of the device calls (off by default): slot i
   is the i-th launch of the call (residual: positions, element residual,
   node gather, scale; jacobian: positions, element tangent, node gather,
   row assembly, scale).  Times accumulate over calls until re-enabled. */
int EnableGpuKernelTiming(BiofemGpuMesh *m, int on);
int GetGpuKernelTimes(const BiofemGpuMesh *m, double *ms, int32_t nslots, int32_t *calls);

/* Number of kernels one RunGpuResidual* / RunGpuResidualJacobian* call
   launches (for launch accounting). */
int GetGpuLaunchCounts(const BiofemGpuMesh *m, int32_t *residual_launches, int32_t *jacobian_launches);

/* Host-only build of the same topology, maps and tangent pattern without a
   GPU (no CUDA call is made): lets a caller or a test inspect the tables.
   The handle only serves GetGpuMeshInfo / GetGpuTopology / GetGpuCsrPattern
   and must be released with DestroyHostMesh. */
int BuildHostMesh(const BiofemMeshDesc *mesh, const BiofemParams *params, BiofemGpuMesh **out);
int DestroyHostMesh(BiofemGpuMesh *m);

/* Centroid basis-derivative tables the kernels use: 11 tables x 5 rows x 16
   (table 0 = regular patch, active_strain.c:69-88; table v = the one-step
   subdivision weights of valence v, active_strain.c:594-666). */
int GetGpuBasisTables(double *out);
/* The same for either table kind. */
int GetGpuBasisTablesKind(int32_t basis, double *out);

const char *BiofemGpuLastError(void);

#ifdef __cplusplus
}
#endif
#endif
