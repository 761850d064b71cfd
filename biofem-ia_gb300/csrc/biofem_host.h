/*
 * Internal declarations shared by the host bridge, the topology builder and
 * the CUDA kernels.  Not part of the C-ABI (include/biofem_gpu.h is).
 */
#ifndef BIOFEM_HOST_H
#define BIOFEM_HOST_H

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/biofem_gpu.h"

namespace biofem {

constexpr int kMaxQp = 6;
constexpr int kRefPerQp = 20;     /* FP64 reference constants per (element, qp) */
constexpr int kRefPerElem = 4;    /* gamma, gamma', c1, pref0 */
constexpr int kGeomShape = 18;    /* primal element geometry stored for the FP64 tangent (elem_geom_store) */
constexpr int kGeomPrimal = kGeomShape + 17;   /* + the primal resultants (elem_res_store) */
constexpr int kCapTable = 11;     /* flat apex-cap triangle: a1 = x2 - x1, a2 = x3 - x1, no curvature */
constexpr int kNumTables = 12;    /* 0 = regular 12-node patch, v = 3..10 irregular, kCapTable */
constexpr int kDeStride = 240;    /* per-element tangent block: D = df/dy (15 x 15, row-major), */
constexpr int kDePres = 225;      /* then the three follower-pressure corner vectors (9) */
constexpr int kMaxRowBlocks = 1023;   /* tangent blocks per row the row assembly handles (10-bit slot targets) */
constexpr int kRowRec = 20;           /* ints per row-assembly record (80 bytes, 16-byte aligned) */
constexpr unsigned kRowSlotGhost = 1u << 31;   /* record slot target of a ghost slot: three packed parents */
constexpr unsigned kRowSlotDup = 1u << 30;     /* with kRowSlotGhost: a slot repeating an earlier slot's real node
                                                  (an open boundary that is no ring); its target in the first two
                                                  10-bit fields, 1023 (no block) in the third */

/* Topology in IBMNodes layout (see topology.cpp). */
struct HostTopo {
  int n_v = 0, n_elmt = 0, n_ghosts = 0, n_edge = 0;
  int n_elmt_base = 0;                             /* > 0: elements from n_elmt_base on are apex-cap triangles */
  std::vector<int> tri_all;                        /* 3*(n_elmt + 2 n_ghosts) */
  std::vector<int> ghost_nv1, ghost_nv2, ghost_nv3;/* per ghost: x_g = x_nv2 + x_nv1 - x_nv3 */
  std::vector<int> ire, irv, val, patch;           /* patch: 16*n_elmt, the reference's tables */
  std::vector<int> dpatch;                         /* the kernels' stencils: patch, cap corners in slots 0-2 */
  std::vector<double> xyz0_full;                   /* 3*(n_v + n_ghosts) */
};

int build_topology(const BiofemMeshDesc &d, HostTopo &T, std::string &err);

/* Parameters every element kernel needs (passed by value). */
struct KParams {
  int ne, nt, nv, ng, nq, iters;
  int tnormal;               /* thickness metric from the tangential part of a3,alpha */
  int pres_dead;             /* pressure with the reference normal and area (no load stiffness) */
  int iso_act;               /* isotropic active gradient (-cart_fib_act 0) */
  double mu, K, hhalf;
  double theta[kMaxQp], w[kMaxQp];
  double pressure;
  double gamma;
  /* dynamic term (FDynamic, main.c:1157-1290): lumped corner mass rho h0 A0 / 3,
     optional damping c M, Newmark (0) or central (1) differences */
  int dyn, dyn_central, dyn_damp;
  double dyn_rhoh0, dyn_dt, dyn_dampf, dyn_M1, dyn_M2, dyn_M3, dyn_C1, dyn_C2, dyn_C3, dyn_U2, dyn_U3;
  /* FP32 copies for the FP32-bulk kernels (filled on the host) */
  float muf, Kf, hhalff, pres6f;
  float thetaf[kMaxQp], wf[kMaxQp];
  /* float-float copies (hi, lo) for the FP32-bulk residual (filled on the host) */
  float mu2[2], K2[2], hhalf2[2];
  float theta2[kMaxQp][2], w2[kMaxQp][2];
};

/* Device views of one mesh handle. */
struct DevMesh {
  /* topology / per-element constants */
  const int *patch;          /* 16*ne */
  const int *einfo;          /* ne: nen | (table << 8) */
  const int *ecorner;        /* ne: patch slots of nv1, nv2, nv3 (5 bits each) */
  const double *eref;        /* (kRefPerQp*nq + kRefPerElem) * ne, SoA */
  const float *erefF;        /* the same in FP32 (FP32-bulk handles only) */
  const void *erefFF;        /* the same as float-float pairs (FP32-bulk handles only; ff.cuh FF) */
  const void *ntabFF;        /* basis tables and their row sums as float-float pairs (FP32-bulk handles) */
  const double *ntab;        /* kNumTables * 5 * 16 basis-derivative tables */
  const float *ntabF;        /* the same in FP32, followed by the kNumTables*5 row sums */
  const int *etri;           /* 3*ne triangle corners (pressure) */
  const int *ghost3;         /* 3*ng (nv1, nv2, nv3) */
  const double *X;           /* 3*nt reference positions (Vec layout) */
  const unsigned char *rowkind; /* nt: 0 free real row, 1 clamped row, 2 ghost row */
  /* residual gather lists */
  const int *rptr, *ridx;    /* nt+1, into fb scratch (slot*3*ne + e) */
  const int *rrec;           /* kRowRec ints per contribution (same order): e | slot << 27, einfo, ecorner, 0,
                                the slot targets in the row (row assembly of the tangent) */
  const int *pptr, *pidx;    /* nt+1, elements whose corner is the node */
  /* tangent pattern */
  const int *rowptr, *colind;   /* BSR pattern, columns sorted per row */
  long long nnzb;
  int maxblk;                /* most blocks in one row */
  int ntabs;                 /* basis tables the row assembly stages: kCapTable, or kNumTables with cap elements */
  /* work arrays */
  double *pos;               /* 4*nt padded positions */
  double *fb;                /* 48*ne element forces */
  double *fp;                /* 3*ne element pressure forces */
  double *De;                /* kDeStride*ne element tangent blocks df/dy (FP64 handles) */
  float *DeF;                /* the same in FP32 (FP32-bulk handles) */
  int *status;               /* device error flag */
  double *dA0;               /* n_elmt flat reference areas of the real triangles (AreaNormal at Init) */
  int *dptr, *didx;          /* per node, the real triangles with that corner, in triangle order */
  double *xn, *xnm1, *xd, *xdd;   /* 3*nt dynamic state (previous positions, velocity, acceleration) */
  double *dyn_diag;          /* nt: d Fdyn / d x on the diagonal of each free row */
  double *gmq;               /* FP64 handles: 6 nq x ne thickness-point metrics, k_elem_residual -> k_elem_tangent */
  double *gpr;               /* FP64 handles: kGeomPrimal x ne primal geometry and resultants, k_elem_residual -> k_elem_tangent */
  double *gtape;             /* FP64 handles: nq x (6 + 23 C33 iterations) x ne primal stress values, likewise */
  unsigned long long *fmax;  /* max |Fext| as ordered bits */
};

/* kernel launchers (kernels.cu); return cudaError_t as int */
int launch_ref_prep(const DevMesh &m, const KParams &p, const double *fib, const double *gscale, double *eref_out, void *stream);
int launch_positions(const DevMesh &m, const KParams &p, const double *x, void *stream);
int launch_elem_residual(const DevMesh &m, const KParams &p, void *stream, bool store_metric = false);
int launch_elem_tangent(const DevMesh &m, const KParams &p, void *stream);
int launch_node_gather(const DevMesh &m, const KParams &p, const double *x, double *R, void *stream,
                       double *parts = nullptr);
int launch_elem_thickness(const DevMesh &m, const KParams &p, double h0, double *th, void *stream);
int launch_row_assemble(const DevMesh &m, const KParams &p, void *K, bool f32, bool colmajor, void *stream);
int launch_row_records(const DevMesh &m, const KParams &p, int *rrec, void *stream);   /* once per mesh */
extern thread_local bool t_blocking_waits;   /* solver host waits sleep instead of spinning (serving workers) */
int row_assemble_configure(int maxblk, bool f32, int ntabs);   /* dynamic shared memory of the row assembly */
size_t row_assemble_smem(int maxblk, bool f32, int ntabs);
int row_assemble_max_blocks(bool f32);             /* blocks per row each row assembly handles */
int launch_scale(const DevMesh &m, const KParams &p, double *R, void *stream);
int launch_elem_tangent_f32(const DevMesh &m, const KParams &p, void *stream);
int launch_elem_residual_ff(const DevMesh &m, const KParams &p, void *stream);
int launch_to_ff(const double *a, void *b, long long n, void *stream);
int launch_to_float(const double *a, float *b, long long n, void *stream);
int launch_dyn_diag(const DevMesh &m, const KParams &p, void *stream);
int launch_dyn_update(const DevMesh &m, const KParams &p, const double *x, void *stream);
int upload_tables(double *d_ntab);

/* device Newton / GMRES (solver.cu) */
struct SolverWork;
SolverWork *solver_create(int n, int nb, int m, void *stream, int *rc);
void solver_destroy(SolverWork *w);
double *solver_xbuf(SolverWork *w);
int solver_m(const SolverWork *w);
long long solver_device_bytes(const SolverWork *w);
typedef int (*ResidualFn)(void *ctx, const double *x, double *R, void *stream);
typedef int (*JacobianFn)(void *ctx, const double *x, double *R, void *K, void *stream);
struct AmgHier;
int newton_device(const DevMesh &dm, const KParams &kp, bool f32, void *dK, double *dR, double *x,
                  const BiofemNewtonOptions &o, BiofemNewtonStats &s, SolverWork *w, AmgHier *amg, cudaStream_t st,
                  ResidualFn residual, JacobianFn jacobian, void *ctx, std::string &err);
void host_tables(double *out, int basis);   /* kNumTables*5*16 host copy of the basis tables */

} /* namespace biofem */

#endif
