/*
 * C-ABI bridge (include/biofem_gpu.h): mesh handles, one-time setup and the
 * residual / tangent entry points.  Replaces the reference's
 * src/cuda_wrapper.cpp + the host half of src/cuda_kernel.cu: instead of a
 * global workspace re-uploaded on every call, each mesh handle keeps its
 * topology, reference geometry, assembly maps and work arrays resident in
 * HBM; a call moves only x in and R (and K) out.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <type_traits>
#include <vector>

#include "amg.h"
#include "ff.cuh"
#include "biofem_host.h"

namespace biofem {

static thread_local std::string g_last_error;
static std::mutex g_mu;
static cudaStream_t g_stream = nullptr;
static bool g_init = false;

static int fail(int code, const std::string &msg)
{
  g_last_error = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                             \
  do {                                                                                             \
    cudaError_t e_ = (expr);                                                                       \
    if (e_ != cudaSuccess) return fail(76, std::string(#expr) + ": " + cudaGetErrorString(e_));    \
  } while (0)

/* ---------------- basis-derivative tables ---------------- */
/* Centroid derivatives of the 12 regular box-spline basis functions in the
   reference's node ordering, four-decimal values (active_strain.c:69-88);
   parity with the reference needs these exact constants. */
static const double kNaC[2][12] = {
  {-0.0247, -0.0309, 0.0000, -0.4815, -0.1852, 0.0247, 0.4815, 0.0000, -0.0062, 0.0309, 0.1852, 0.0062},
  {-0.0309, -0.0247, -0.1852, -0.4815, 0.0000, -0.0062, 0.0000, 0.4815, 0.0247, 0.0062, 0.1852, 0.0309}};
static const double kNabC[3][12] = {
  {0.1111, 0.2222, -0.2222, -0.2222, 0.4444, 0.1111, -0.2222, -0.8889, 0.0000, 0.2222, 0.4444, 0.0000},
  {0.2222, 0.1111, 0.4444, -0.2222, -0.2222, 0.0000, -0.8889, -0.2222, 0.1111, 0.0000, 0.4444, 0.2222},
  {0.1667, 0.1667, -0.1111, 0.2222, -0.1111, -0.0556, -0.4444, -0.4444, -0.0556, 0.0556, 0.5556, 0.0556}};

/* One Loop-subdivision step around an extraordinary vertex of valence v,
   restricted to the rows the centroid evaluation reads.  Each rule is
   (row = rb*v + ro, col = cb*v + co, weight), applied in order so that for
   small v later rules overwrite earlier ones exactly as the reference's
   assignment sequence does (active_strain.c:594-630). */
struct SubdivRule { signed char rb, ro, cb, co; double wgt; signed char min_v; };
static const SubdivRule kRules[] = {
  /* edge points next to the extraordinary vertex */
  {0, 1, 0, 0, 0.375, 0}, {0, 1, 0, 1, 0.375, 0}, {0, 1, 0, 2, 0.125, 0}, {0, 1, 1, 0, 0.125, 0},
  {0, 2, 0, 0, 0.375, 0}, {0, 2, 0, 1, 0.125, 0}, {0, 2, 0, 2, 0.375, 0}, {0, 2, 0, 3, 0.125, 0},
  {1, -4, 0, 0, 0.375, 6}, {1, -4, 1, -5, 0.125, 6}, {1, -4, 1, -4, 0.375, 6}, {1, -4, 1, -3, 0.125, 6},
  {1, -3, 0, 0, 0.375, 5}, {1, -3, 1, -4, 0.125, 5}, {1, -3, 1, -3, 0.375, 5}, {1, -3, 1, -2, 0.125, 5},
  {1, -2, 0, 0, 0.375, 0}, {1, -2, 1, -3, 0.125, 0}, {1, -2, 1, -2, 0.375, 0}, {1, -2, 1, -1, 0.125, 0},
  {1, -1, 0, 0, 0.375, 0}, {1, -1, 1, -2, 0.125, 0}, {1, -1, 1, -1, 0.375, 0}, {1, -1, 1, 0, 0.125, 0},
  {1, 0, 0, 0, 0.375, 0}, {1, 0, 0, 1, 0.125, 0}, {1, 0, 1, -1, 0.125, 0}, {1, 0, 1, 0, 0.375, 0},
  /* the second ring */
  {1, 1, 0, 0, 0.125, 0}, {1, 1, 0, 1, 0.375, 0}, {1, 1, 1, 0, 0.375, 0}, {1, 1, 1, 1, 0.125, 0},
  {1, 2, 0, 0, 0.0625, 0}, {1, 2, 0, 1, 0.625, 0}, {1, 2, 0, 2, 0.0625, 0}, {1, 2, 1, 0, 0.0625, 0},
  {1, 2, 1, 1, 0.0625, 0}, {1, 2, 1, 2, 0.0625, 0}, {1, 2, 1, 3, 0.0625, 0},
  {1, 3, 0, 0, 0.125, 0}, {1, 3, 0, 1, 0.375, 0}, {1, 3, 0, 2, 0.375, 0}, {1, 3, 1, 3, 0.125, 0},
  {1, 4, 0, 0, 0.0625, 0}, {1, 4, 0, 1, 0.0625, 0}, {1, 4, 1, -1, 0.0625, 0}, {1, 4, 1, 0, 0.625, 0},
  {1, 4, 1, 1, 0.0625, 0}, {1, 4, 1, 4, 0.0625, 0}, {1, 4, 1, 5, 0.0625, 0},
  {1, 5, 0, 0, 0.125, 0}, {1, 5, 1, -1, 0.375, 0}, {1, 5, 1, 0, 0.375, 0}, {1, 5, 1, 5, 0.125, 0},
  {1, 6, 0, 1, 0.375, 0}, {1, 6, 1, 0, 0.125, 0}, {1, 6, 1, 1, 0.375, 0}, {1, 6, 1, 2, 0.125, 0},
  {1, 9, 0, 1, 0.125, 0}, {1, 9, 1, 0, 0.375, 0}, {1, 9, 1, 1, 0.375, 0}, {1, 9, 1, 4, 0.125, 0},
};

/* rows of the refined net that form the regular 12-node sub-patch holding
   the centroid, in regular-patch order (active_strain.c:608-610) */
static void subpatch_rows(int v, int rows[12])
{
  const int r[12] = {v + 9, v + 6, v + 4, v + 1, v + 2, v + 5, v, 1, v + 3, v - 1, 0, 2};
  for (int i = 0; i < 12; i++) rows[i] = r[i];
}

/* basis BIOFEM_BASIS_REFERENCE: the four-decimal constants above;
   BIOFEM_BASIS_EXACT: the rationals they round (k/324 for the first
   derivatives, k/108 for the second), whose rows sum to zero, so that a flat
   uniform patch has exactly zero second derivatives.  The irregular tables
   are built from whichever regular table is chosen.  Table kCapTable is the
   flat apex-cap triangle on its corners (slots 0-2): a1 = x2 - x1,
   a2 = x3 - x1 and no second derivatives (active_strain.c:448-470). */
void host_tables(double *out, int basis)
{
  std::fill(out, out + kNumTables * 80, 0.0);
  for (int i = 0; i < 12; i++) {
    for (int r = 0; r < 2; r++)
      out[r * 16 + i] = basis ? std::nearbyint(kNaC[r][i] * 324.0) / 324.0 : kNaC[r][i];
    for (int r = 0; r < 3; r++)
      out[(2 + r) * 16 + i] = basis ? std::nearbyint(kNabC[r][i] * 108.0) / 108.0 : kNabC[r][i];
  }
  const double pi = 3.14159265358979323846264338327950288419716939937510582;
  for (int v = 3; v < kCapTable; v++) {
    const int nen = v + 6, nr = v + 12;
    std::vector<double> B((size_t)nr * nen, 0.0);
    /* Loop's vertex rule, weight w(v) = (5/8 - (3/8 + cos(2 pi / v)/4)^2) / v */
    const double w = (1.0 / (double)v) * (0.625 - std::pow(0.375 + 0.25 * std::cos(2 * pi / (double)v), 2.0));
    B[0] = 1 - v * w;
    for (int j = 0; j < v; j++) B[1 + j] = w;
    for (const SubdivRule &r : kRules) {
      if (r.min_v && v < r.min_v) continue;
      const int row = r.rb * v + r.ro, col = r.cb * v + r.co;
      if (row < 0 || row >= nr || col < 0 || col >= nen) continue;
      B[(size_t)row * nen + col] = r.wgt;
    }
    int rows[12];
    subpatch_rows(v, rows);
    const double *Nrow[5] = {out, out + 16, out + 32, out + 48, out + 64};   /* the chosen regular table */
    const double scale[5] = {-2.0, -2.0, 4.0, 4.0, 4.0};
    for (int rr = 0; rr < 5; rr++)
      for (int j = 0; j < nen; j++) {
        double s = 0.0;
        for (int i = 0; i < 12; i++) s = s + B[(size_t)rows[i] * nen + j] * Nrow[rr][i];
        out[v * 80 + rr * 16 + j] = scale[rr] * s;
      }
  }
  double *cap = out + kCapTable * 80;
  cap[0] = -1.0; cap[1] = 1.0;             /* a1 */
  cap[16 + 0] = -1.0; cap[16 + 2] = 1.0;   /* a2 */
}

} /* namespace biofem */

using namespace biofem;

/* optional per-kernel timing of the device calls (events on the call's stream) */
static const int kMaxTimed = 8;
struct KernelTimer {
  bool on = false;
  int n = 0;
  cudaEvent_t ev[kMaxTimed + 1] = {};
  float acc_ms[kMaxTimed] = {};
  int calls = 0;
};

/* ---------------- the mesh handle ---------------- */
struct BiofemGpuMesh_ {
  HostTopo topo;
  BiofemParams prm{};
  KParams kp{};
  std::vector<double> dA0;
  std::vector<int> rowptr, colind;
  long long nnzb = 0, ncontrib = 0;
  int n_irregular = 0, maxblk = 1;
  size_t bytes = 0;
  std::vector<void *> allocs;
  DevMesh dm{};
  double *d_x = nullptr, *d_R = nullptr;   /* staging for host-array calls */
  void *d_K = nullptr;                      /* K values: double (FP64) or float (FP32-bulk) */
  SolverWork *solver = nullptr;             /* Newton/GMRES work, created on first solve */
  double *d_fib = nullptr, *d_gam = nullptr;   /* fibres; per-element activation of SetGpuElementGamma */
  AmgHier *amg = nullptr;                   /* multigrid hierarchy, created on first multigrid solve */
  std::vector<unsigned char> rowkind;       /* host copy: 0 free, 1 clamped, 2 ghost */
  cudaStream_t st = nullptr;                /* stream of the host-array calls and of setup/teardown */
  cudaStream_t side = nullptr;              /* second stream: independent kernels of one call overlap */
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  KernelTimer timer;
  int device = -1;                          /* the device the handle's arrays live on */
};

static std::set<BiofemGpuMesh *> g_meshes;
static std::mutex g_meshes_mu;

namespace biofem {
/* accessors for the no-allocation residual (noalloc.cu) */
int noalloc_fail(int code, const std::string &msg) { return fail(code, msg); }
/* the calling thread's last error for the host-only modules (formats.cpp) */
int host_fail(int code, const std::string &msg) { return fail(code, msg); }
const DevMesh *mesh_devview(const BiofemGpuMesh *m, const KParams **kp, int *device)
{
  if (!m || !m->dm.patch) return nullptr;
  *kp = &m->kp;
  *device = m->device;
  return &m->dm;
}
} /* namespace biofem */
static KernelTimer &timer_of(BiofemGpuMesh *m) { return m->timer; }

/* device-variant stream argument: a cudaStream_t; NULL is the CUDA default stream */
static inline cudaStream_t pick_stream(void *s) { return (cudaStream_t)s; }

static inline void tmark(BiofemGpuMesh *m, cudaStream_t st, int i)
{
  KernelTimer &t = timer_of(m);
  if (t.on && i <= kMaxTimed) { cudaEventRecord(t.ev[i], st); t.n = i; }
}

template <class T>
static int dalloc(BiofemGpuMesh *m, T **p, size_t n)
{
  void *q = nullptr;
  cudaError_t e = cudaMallocAsync(&q, std::max<size_t>(n, 1) * sizeof(T), m->st);
  if (e != cudaSuccess) return fail(55, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
  m->allocs.push_back(q);
  m->bytes += std::max<size_t>(n, 1) * sizeof(T);
  *p = reinterpret_cast<T *>(q);
  return 0;
}

template <class T>
static int dupload(BiofemGpuMesh *m, T **p, const std::vector<T> &h)
{
  int rc = dalloc(m, p, h.size());
  if (rc) return rc;
  if (!h.empty()) CUDA_TRY(cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, m->st));
  return 0;
}

static void free_mesh(BiofemGpuMesh *m)
{
  if (m->st) cudaStreamSynchronize(m->st);
  if (m->solver) solver_destroy(m->solver);
  if (m->amg) amg_destroy(m->amg);
  for (int i = 0; i <= kMaxTimed; i++) if (m->timer.ev[i]) cudaEventDestroy(m->timer.ev[i]);
  for (void *p : m->allocs) cudaFreeAsync(p, m->st);
  m->allocs.clear();
  if (m->st) cudaStreamSynchronize(m->st);
  if (m->side) { cudaStreamSynchronize(m->side); cudaStreamDestroy(m->side); }
  if (m->ev_fork) cudaEventDestroy(m->ev_fork);
  if (m->ev_join) cudaEventDestroy(m->ev_join);
  delete m;
}

/* Host-side build of every map; no CUDA calls (usable without a GPU). */
/* Flat reference area of triangle t (real, ghost or bridging), the
   expression of AreaNormal (io.c:1646-1669) on the reference coordinates. */
static double tri_area0(const HostTopo &T, int t)
{
  const double *X = T.xyz0_full.data();
  const int a = T.tri_all[3 * (size_t)t], b = T.tri_all[3 * (size_t)t + 1], c = T.tri_all[3 * (size_t)t + 2];
  const double d21[3] = {X[3 * b] - X[3 * a], X[3 * b + 1] - X[3 * a + 1], X[3 * b + 2] - X[3 * a + 2]};
  const double d31[3] = {X[3 * c] - X[3 * a], X[3 * c + 1] - X[3 * a + 1], X[3 * c + 2] - X[3 * a + 2]};
  const double cx = d21[1] * d31[2] - d31[1] * d21[2], cy = -d21[0] * d31[2] + d31[0] * d21[2], cz = d21[0] * d31[1] - d31[0] * d21[1];
  return 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
}

static int build_host_maps(BiofemGpuMesh *m, const BiofemMeshDesc &d, const BiofemParams &prm,
                           std::vector<int> &einfo, std::vector<int> &ecorner, std::vector<unsigned char> &rowkind,
                           std::vector<int> &rptr, std::vector<int> &ridx, std::vector<int> &pptr,
                           std::vector<int> &pidx)
{
  std::string err;
  int rc = build_topology(d, m->topo, err);
  if (rc) return fail(rc, err);
  const HostTopo &T = m->topo;
  const int ne = T.n_elmt, nv = T.n_v, ng = T.n_ghosts, nt = nv + ng;
  if (prm.clamp_edge >= d.n_edge) return fail(63, "clamp_edge beyond the number of boundary rings");

  if (ne >= (1 << 27)) return fail(63, "more than 2^27 elements");
  einfo.assign(ne, 0);
  ecorner.assign(ne, 0);
  m->n_irregular = 0;
  const int ncap_from = T.n_elmt_base > 0 ? T.n_elmt_base : ne;
  for (int e = 0; e < ne; e++) {
    const bool cap = e >= ncap_from;
    const int nen = cap ? 3 : T.ire[e] ? T.val[e] + 6 : 12;
    const int tab = cap ? kCapTable : T.ire[e] ? T.val[e] : 0;
    if (T.ire[e]) m->n_irregular++;
    einfo[e] = nen | (tab << 8);
    /* patch slots holding the triangle's corners (first occurrence) */
    int packed = 0;
    for (int k = 0; k < 3; k++) {
      const int node = T.tri_all[3 * (size_t)e + k];
      int slot = -1;
      for (int a = 0; a < nen && slot < 0; a++) if (T.dpatch[16 * (size_t)e + a] == node) slot = a;
      if (slot < 0) return fail(77, "a triangle corner is missing from its own patch");
      packed |= slot << (5 * k);
    }
    ecorner[e] = packed;
  }

  rowkind.assign(nt, 0);
  for (int g = nv; g < nt; g++) rowkind[g] = 2;
  if (prm.clamp_edge >= 0) {
    int start = 0;
    for (int r = 0; r < prm.clamp_edge; r++) start += d.n_bnodes[r];
    for (int i = 0; i < d.n_bnodes[prm.clamp_edge]; i++) rowkind[d.bnodes[start + i]] = 1;
  }

  /* residual gather lists: (element, slot) in element order for real rows */
  rptr.assign(nt + 1, 0);
  for (int e = 0; e < ne; e++) {
    const int nen = einfo[e] & 0xff;
    for (int a = 0; a < nen; a++) {
      const int node = T.dpatch[16 * (size_t)e + a];
      if (node < nv) rptr[node + 1]++;
    }
  }
  for (int i = 0; i < nt; i++) rptr[i + 1] += rptr[i];
  ridx.assign(rptr[nt], 0);
  std::vector<int> r_elem(rptr[nt]);   /* the contribution's element, for the pattern sweep below */
  {
    std::vector<int> fill(rptr.begin(), rptr.end() - 1);
    for (int e = 0; e < ne; e++) {
      const int nen = einfo[e] & 0xff;
      for (int a = 0; a < nen; a++) {
        const int node = T.dpatch[16 * (size_t)e + a];
        if (node < nv) {
          const int c = fill[node]++;
          ridx[c] = (int)((long long)3 * a * ne + e);
          r_elem[c] = e;
        }
      }
    }
  }
  /* corner lists (pressure load, dynamic term): elements having the node
     as a corner, in element order */
  pptr.assign(nt + 1, 0);
  for (int e = 0; e < ne; e++) for (int k = 0; k < 3; k++) pptr[T.tri_all[3 * (size_t)e + k] + 1]++;
  for (int i = 0; i < nt; i++) pptr[i + 1] += pptr[i];
  pidx.assign(pptr[nt], 0);
  {
    std::vector<int> fill(pptr.begin(), pptr.end() - 1);
    for (int e = 0; e < ne; e++) for (int k = 0; k < 3; k++) pidx[fill[T.tri_all[3 * (size_t)e + k]]++] = e;
  }

  /* column expansion of a patch slot: real node, or the ghost's parents */
  auto expand = [&](int node, int cols[3], int sg[3]) -> int {
    if (node < nv) { cols[0] = node; sg[0] = 1; return 1; }
    const int g = node - nv;
    cols[0] = T.ghost_nv2[g]; sg[0] = 1;
    cols[1] = T.ghost_nv1[g]; sg[1] = 1;
    cols[2] = T.ghost_nv3[g]; sg[2] = -1;
    return 3;
  };

  /* BSR pattern: the columns of row i are the real nodes of every patch
     holding i, a ghost slot standing for its three parents (the chain rule of
     x_g = x_nv2 + x_nv1 - x_nv3), sorted; n_contrib counts the (element, row
     slot, column slot, parent) terms the row assembly adds. */
  m->rowptr.assign(nt + 1, 0);
  m->colind.clear();
  m->colind.reserve((size_t)nt * 40);
  std::vector<int> mark(nt, -1);
  std::vector<int> cols_acc;
  long long ncontrib = 0;
  int maxblk = 1;
  for (int i = 0; i < nt; i++) {
    if (rowkind[i] != 0) {
      m->colind.push_back(i);
      m->rowptr[i + 1] = (int)m->colind.size();
      continue;
    }
    cols_acc.clear();
    cols_acc.push_back(i);
    mark[i] = i;
    for (int c = rptr[i]; c < rptr[i + 1]; c++) {
      const int e = r_elem[c];
      const int nen = einfo[e] & 0xff;
      for (int b = 0; b < nen; b++) {
        int cols[3], sg[3];
        const int k = expand(T.dpatch[16 * (size_t)e + b], cols, sg);
        ncontrib += k;
        for (int q = 0; q < k; q++)
          if (mark[cols[q]] != i) { mark[cols[q]] = i; cols_acc.push_back(cols[q]); }
      }
    }
    std::sort(cols_acc.begin(), cols_acc.end());
    m->colind.insert(m->colind.end(), cols_acc.begin(), cols_acc.end());
    if (m->colind.size() >= (size_t)1 << 31) return fail(63, "tangent pattern exceeds int32");
    maxblk = std::max(maxblk, (int)cols_acc.size());
    m->rowptr[i + 1] = (int)m->colind.size();
  }
  if (maxblk > kMaxRowBlocks) return fail(63, "a tangent row has more blocks than the row assembly handles");
  m->nnzb = (long long)m->colind.size();
  m->ncontrib = ncontrib;
  m->maxblk = maxblk;
  /* dA0 on the host too (GetGpuTopology) */
  m->dA0.assign(ne, 0.0);
  for (int e = 0; e < ne; e++) m->dA0[e] = tri_area0(T, e);
  return 0;
}

static int check_params(const BiofemParams &p)
{
  if (p.n_qp < 1 || p.n_qp > kMaxQp) return fail(63, "n_qp must be between 1 and 6");
  if (p.c33_subitr_nums < 1) return fail(62, "C33_subitr_nums must be >= 1");
  if (!(p.h0 > 0.0)) return fail(62, "h0 must be positive");
  if (p.precision != BIOFEM_FP64 && p.precision != BIOFEM_FP32_BULK) return fail(62, "unknown precision");
  if (p.basis != BIOFEM_BASIS_REFERENCE && p.basis != BIOFEM_BASIS_EXACT) return fail(62, "unknown basis tables");
  if (p.thickness_normal != 0 && p.thickness_normal != 1) return fail(62, "thickness_normal must be 0 or 1");
  if (p.block_layout != BIOFEM_BLOCK_ROW_MAJOR && p.block_layout != BIOFEM_BLOCK_COL_MAJOR)
    return fail(62, "unknown block layout");
  if (p.pressure_kind != BIOFEM_PRESSURE_FOLLOWER && p.pressure_kind != BIOFEM_PRESSURE_DEAD)
    return fail(62, "unknown pressure kind");
  if (p.activation_kind != BIOFEM_ACTIVATION_FIBRE && p.activation_kind != BIOFEM_ACTIVATION_ISOTROPIC)
    return fail(62, "unknown activation kind");
  return 0;
}

static void gauss(int n, double *th, double *w)
{
  switch (n) {
  case 1: th[0] = 0.0; w[0] = 2.0; break;
  case 2: th[0] = -0.5773502691896257; th[1] = 0.5773502691896257; w[0] = w[1] = 1.0; break;
  case 3: th[0] = -0.7745966692414834; th[1] = 0.0; th[2] = 0.7745966692414834;
          w[0] = w[2] = 0.5555555555555556; w[1] = 0.8888888888888888; break;
  case 4: th[0] = -0.8611363115940526; th[1] = -0.3399810435848563; th[2] = 0.3399810435848563; th[3] = 0.8611363115940526;
          w[0] = w[3] = 0.3478548451374538; w[1] = w[2] = 0.6521451548625461; break;
  case 5: th[0] = -0.9061798459386640; th[1] = -0.5384693101056831; th[2] = 0.0; th[3] = 0.5384693101056831; th[4] = 0.9061798459386640;
          w[0] = w[4] = 0.2369268850561891; w[1] = w[3] = 0.4786286704993665; w[2] = 0.5688888888888889; break;
  default: th[0] = -0.9324695142031521; th[1] = -0.6612093864662645; th[2] = -0.2386191860831969;
           th[3] = 0.2386191860831969; th[4] = 0.6612093864662645; th[5] = 0.9324695142031521;
           w[0] = w[5] = 0.1713244923791704; w[1] = w[4] = 0.3607615730481386; w[2] = w[3] = 0.4679139345726910; break;
  }
}

extern "C" {

int InitGpuWorkspace(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_init) return 0;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(76, std::string("no CUDA device: ") + cudaGetErrorString(e));
  CUDA_TRY(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
  /* keep freed handle memory in the stream-ordered pool for reuse (serving
     creates and destroys handles continuously) */
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  g_init = true;
  return 0;
}

int DestroyGpuWorkspace(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  {
    std::lock_guard<std::mutex> lk2(g_meshes_mu);
    for (BiofemGpuMesh *m : g_meshes) free_mesh(m);
    g_meshes.clear();
  }
  if (g_stream) cudaStreamDestroy(g_stream);
  g_stream = nullptr;
  g_init = false;
  return 0;
}

const char *BiofemGpuLastError(void) { return g_last_error.c_str(); }

/* Host-only: topology + maps without touching the GPU (used by tests and by
   callers that want the tables).  Returns a handle whose device views are empty. */
int BuildHostMesh(const BiofemMeshDesc *mesh, const BiofemParams *params, BiofemGpuMesh **out)
{
  if (!mesh || !params || !out) return fail(85, "null argument");
  int rc = check_params(*params);
  if (rc) return rc;
  BiofemGpuMesh *m = new BiofemGpuMesh();
  m->prm = *params;
  std::vector<int> einfo, ecorner, rptr, ridx, pptr, pidx;
  std::vector<unsigned char> rowkind;
  rc = build_host_maps(m, *mesh, *params, einfo, ecorner, rowkind, rptr, ridx, pptr, pidx);
  if (rc) { delete m; return rc; }
  *out = m;
  return 0;
}

int DestroyHostMesh(BiofemGpuMesh *m) { delete m; return 0; }

int PrepareGpuMesh(const BiofemMeshDesc *mesh, const BiofemParams *params, BiofemGpuMesh **out)
{
  if (!g_init) { int rc = InitGpuWorkspace(); if (rc) return rc; }
  return PrepareGpuMeshOnStream(mesh, params, g_stream, out);
}

int PrepareGpuMeshOnStream(const BiofemMeshDesc *mesh, const BiofemParams *params, void *stream, BiofemGpuMesh **out)
{
  if (!mesh || !params || !out) return fail(85, "null argument");
  int rc = check_params(*params);
  if (rc) return rc;
  if (!g_init) { rc = InitGpuWorkspace(); if (rc) return rc; }
  BiofemGpuMesh *m = new BiofemGpuMesh();
  m->prm = *params;
  m->st = stream ? (cudaStream_t)stream : g_stream;
  if (cudaGetDevice(&m->device) != cudaSuccess) { delete m; return fail(76, "cudaGetDevice failed"); }
  std::vector<int> einfo, ecorner, rptr, ridx, pptr, pidx;
  std::vector<unsigned char> rowkind;
  rc = build_host_maps(m, *mesh, *params, einfo, ecorner, rowkind, rptr, ridx, pptr, pidx);
  if (rc) { delete m; return rc; }
  if (cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&m->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    free_mesh(m);
    return fail(76, "side stream or events could not be created");
  }
  m->rowkind = rowkind;
  const HostTopo &T = m->topo;
  const int ne = T.n_elmt, nv = T.n_v, ng = T.n_ghosts, nt = nv + ng;

  KParams &kp = m->kp;
  kp.ne = ne; kp.nt = nt; kp.nv = nv; kp.ng = ng; kp.nq = params->n_qp; kp.iters = params->c33_subitr_nums;
  kp.tnormal = params->thickness_normal;
  kp.pres_dead = params->pressure_kind == BIOFEM_PRESSURE_DEAD;
  kp.iso_act = params->activation_kind == BIOFEM_ACTIVATION_ISOTROPIC;
  kp.mu = params->mu; kp.K = params->bulk_modulus; kp.hhalf = 0.5 * params->h0;
  kp.pressure = params->pressure; kp.gamma = params->gamma;
  gauss(params->n_qp, kp.theta, kp.w);
  kp.muf = (float)kp.mu; kp.Kf = (float)kp.K; kp.hhalff = (float)kp.hhalf; kp.pres6f = (float)(kp.pressure / 6.0);
  for (int q = 0; q < kMaxQp; q++) { kp.thetaf[q] = (float)kp.theta[q]; kp.wf[q] = (float)kp.w[q]; }
  {
    auto split = [](double d, float out[2]) { const FF f(d); out[0] = f.hi; out[1] = f.lo; };
    split(kp.mu, kp.mu2); split(kp.K, kp.K2); split(kp.hhalf, kp.hhalf2);
    for (int q = 0; q < kMaxQp; q++) { split(kp.theta[q], kp.theta2[q]); split(kp.w[q], kp.w2[q]); }
  }

  DevMesh &dm = m->dm;
  std::vector<int> ghost3(3 * (size_t)ng);
  for (int g = 0; g < ng; g++) { ghost3[3 * g] = T.ghost_nv1[g]; ghost3[3 * g + 1] = T.ghost_nv2[g]; ghost3[3 * g + 2] = T.ghost_nv3[g]; }
  std::vector<int> etri(T.tri_all.begin(), T.tri_all.begin() + 3 * (size_t)ne);
  std::vector<double> tabs(kNumTables * 80);
  host_tables(tabs.data(), params->basis);
  std::vector<float> tabsF(kNumTables * 85);
  std::vector<FF> tabsFF(kNumTables * 85);
  for (int i = 0; i < kNumTables * 80; i++) { tabsF[i] = (float)tabs[i]; tabsFF[i] = FF(tabs[i]); }
  for (int i = 0; i < kNumTables * 5; i++) {
    double acc = 0.0;
    for (int k = 0; k < 16; k++) acc += tabs[i * 16 + k];
    tabsF[kNumTables * 80 + i] = (float)acc;
    tabsFF[kNumTables * 80 + i] = FF(acc);
  }
  std::vector<double> fib(mesh->n_fib, mesh->n_fib + 3 * (size_t)ne), gsc(mesh->gamma_scale, mesh->gamma_scale + ne);

#define UP(field, vec) do { rc = dupload(m, const_cast<std::remove_const<std::remove_pointer<decltype(dm.field)>::type>::type **>(&dm.field), vec); if (rc) { free_mesh(m); return rc; } } while (0)
  UP(patch, T.dpatch); UP(einfo, einfo); UP(ecorner, ecorner); UP(ntab, tabs); UP(ntabF, tabsF); UP(etri, etri); UP(ghost3, ghost3);
  UP(X, T.xyz0_full); UP(rowkind, rowkind); UP(rptr, rptr); UP(ridx, ridx); UP(pptr, pptr); UP(pidx, pidx);
  UP(rowptr, m->rowptr); UP(colind, m->colind);
#undef UP
  {   /* the row-assembly records, built on the device from the arrays above */
    int *d_rrec = nullptr;
    if ((rc = dalloc(m, &d_rrec, (size_t)kRowRec * rptr[nt]))) { free_mesh(m); return rc; }
    dm.rrec = d_rrec;
  }
  dm.nnzb = m->nnzb;
  dm.maxblk = m->maxblk;
  dm.ntabs = (T.n_elmt_base > 0 && T.n_elmt_base < ne) ? kNumTables : kCapTable;
  if (m->maxblk > row_assemble_max_blocks(params->precision != BIOFEM_FP64)) {
    free_mesh(m);
    return fail(63, "a tangent row has more blocks than the FP32 row assembly holds in registers");
  }
  {
    cudaError_t ce = (cudaError_t)row_assemble_configure(m->maxblk, params->precision != BIOFEM_FP64, dm.ntabs);
    if (ce != cudaSuccess) { free_mesh(m); return fail(76, std::string("row assembly configuration: ") + cudaGetErrorString(ce)); }
  }
  double *d_fib = nullptr, *d_gsc = nullptr, *d_eref = nullptr;
  const size_t nref = (size_t)(kRefPerQp * kp.nq + kRefPerElem) * ne;
  if ((rc = dupload(m, &d_fib, fib)) || (rc = dupload(m, &d_gsc, gsc)) || (rc = dalloc(m, &d_eref, nref)) ||
      (rc = dalloc(m, &dm.pos, 4 * (size_t)nt)) || (rc = dalloc(m, &dm.fb, 48 * (size_t)ne)) ||
      (rc = dalloc(m, &dm.fp, 3 * (size_t)ne)) ||
      (rc = dalloc(m, &dm.status, 1)) || (rc = dalloc(m, &dm.fmax, 1)) ||
      (rc = dalloc(m, &m->d_x, 3 * (size_t)nt)) || (rc = dalloc(m, &m->d_R, 3 * (size_t)nt))) {
    free_mesh(m);
    return rc;
  }
  float *d_erefF = nullptr;
  if (params->precision == BIOFEM_FP64) {
    double *dK = nullptr;
    if ((rc = dalloc(m, &dm.De, (size_t)kDeStride * ne)) || (rc = dalloc(m, &dK, 9 * (size_t)m->nnzb)) ||
        (rc = dalloc(m, &dm.gmq, 6 * (size_t)kp.nq * ne)) || (rc = dalloc(m, &dm.gpr, (size_t)kGeomPrimal * ne)) ||
        (rc = dalloc(m, &dm.gtape, (size_t)(6 + 23 * kp.iters) * kp.nq * ne))) {
      free_mesh(m);
      return rc;
    }
    m->d_K = dK;
  } else {
    float *dK = nullptr;
    FF *d_erefFF = nullptr, *d_ntabFF = nullptr;
    if ((rc = dalloc(m, &dm.DeF, (size_t)kDeStride * ne)) || (rc = dalloc(m, &dK, 9 * (size_t)m->nnzb)) ||
        (rc = dalloc(m, &d_erefF, nref)) || (rc = dalloc(m, &d_erefFF, nref)) || (rc = dupload(m, &d_ntabFF, tabsFF))) {
      free_mesh(m);
      return rc;
    }
    dm.erefFF = d_erefFF;
    dm.ntabFF = d_ntabFF;
    m->d_K = dK;
  }
  dm.eref = d_eref;
  dm.erefF = d_erefF;
  m->d_fib = d_fib;
  CUDA_TRY(cudaMemsetAsync(dm.status, 0, sizeof(int), m->st));
  CUDA_TRY(cudaMemsetAsync(dm.fp, 0, 3 * sizeof(double) * (size_t)ne, m->st));
  /* reference positions (ghosts included) -> one-time reference geometry */
  if ((rc = launch_positions(dm, kp, dm.X, m->st)) || (rc = launch_ref_prep(dm, kp, d_fib, d_gsc, d_eref, m->st)) ||
      (rc = launch_row_records(dm, kp, const_cast<int *>(dm.rrec), m->st))) {
    free_mesh(m);
    return fail(76, std::string("reference preparation launch: ") + cudaGetErrorString((cudaError_t)rc));
  }
  if (d_erefF && ((rc = launch_to_float(d_eref, d_erefF, (long long)nref, m->st)) ||
                  (rc = launch_to_ff(d_eref, const_cast<void *>(dm.erefFF), (long long)nref, m->st)))) {
    free_mesh(m);
    return fail(76, std::string("reference conversion launch: ") + cudaGetErrorString((cudaError_t)rc));
  }
  cudaError_t e = cudaStreamSynchronize(m->st);
  if (e != cudaSuccess) { free_mesh(m); return fail(76, std::string("reference preparation: ") + cudaGetErrorString(e)); }
  {
    std::lock_guard<std::mutex> lk(g_meshes_mu);
    g_meshes.insert(m);
  }
  *out = m;
  return 0;
}

int DestroyGpuMesh(BiofemGpuMesh *m)
{
  if (!m) return 0;
  bool mine = false;
  {
    std::lock_guard<std::mutex> lk(g_meshes_mu);
    mine = g_meshes.erase(m) > 0;
  }
  if (mine) free_mesh(m);
  return 0;
}

int GetGpuMeshInfo(const BiofemGpuMesh *m, BiofemMeshInfo *info)
{
  if (!m || !info) return fail(85, "null argument");
  info->n_v = m->topo.n_v; info->n_ghosts = m->topo.n_ghosts; info->n_elmt = m->topo.n_elmt;
  info->n_dof = 3 * (m->topo.n_v + m->topo.n_ghosts);
  info->n_irregular = m->n_irregular;
  info->nnzb = m->nnzb; info->n_contrib = m->ncontrib;
  info->device_bytes = (int64_t)m->bytes + solver_device_bytes(m->solver) + amg_device_bytes(m->amg);
  info->precision = m->prm.precision;
  return 0;
}

int GetGpuTopology(const BiofemGpuMesh *m, int32_t *patch, int32_t *ire, int32_t *val, int32_t *irv,
                   int32_t *gtri, double *xyz0_full, double *dA0)
{
  if (!m) return fail(85, "null argument");
  const HostTopo &T = m->topo;
  if (patch) std::copy(T.patch.begin(), T.patch.end(), patch);
  if (ire) std::copy(T.ire.begin(), T.ire.end(), ire);
  if (val) std::copy(T.val.begin(), T.val.end(), val);
  if (irv) std::copy(T.irv.begin(), T.irv.end(), irv);
  if (gtri) std::copy(T.tri_all.begin(), T.tri_all.end(), gtri);
  if (xyz0_full) std::copy(T.xyz0_full.begin(), T.xyz0_full.end(), xyz0_full);
  if (dA0) std::copy(m->dA0.begin(), m->dA0.end(), dA0);
  return 0;
}

int GetGpuGhostMap(const BiofemGpuMesh *m, int32_t *ghost3)
{
  if (!m || !ghost3) return fail(85, "null argument");
  const HostTopo &T = m->topo;
  for (int g = 0; g < T.n_ghosts; g++) {
    ghost3[3 * g] = T.ghost_nv1[g]; ghost3[3 * g + 1] = T.ghost_nv2[g]; ghost3[3 * g + 2] = T.ghost_nv3[g];
  }
  return 0;
}

int GetGpuCsrPattern(const BiofemGpuMesh *m, int32_t *rowptr, int32_t *colind)
{
  if (!m) return fail(85, "null argument");
  if (rowptr) std::copy(m->rowptr.begin(), m->rowptr.end(), rowptr);
  if (colind) std::copy(m->colind.begin(), m->colind.end(), colind);
  return 0;
}

int GetGpuLaunchCounts(const BiofemGpuMesh *m, int32_t *res, int32_t *jac)
{
  if (!m) return fail(85, "null argument");
  if (res) *res = 4;   /* positions, element residual, node gather, scale */
  /* positions, element residual (FP64), element tangent, node gather,
     row assembly, scale */
  if (jac) *jac = 6;
  return 0;
}

static void timer_collect(BiofemGpuMesh *m)
{
  KernelTimer &t = m->timer;
  if (!t.on || t.n == 0) return;
  cudaEventSynchronize(t.ev[t.n]);
  for (int i = 0; i < t.n; i++) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t.ev[i], t.ev[i + 1]);
    t.acc_ms[i] += ms;
  }
  t.calls++;
  t.n = 0;
}

/* The element residual of the handle's form: FP64 (k_elem_residual) or, for
   FP32-bulk handles, float-float on the FP32 pipe (k_elem_residual_ff). */
static int launch_residual_elements(BiofemGpuMesh *m, cudaStream_t st)
{
  return m->prm.precision == BIOFEM_FP64 ? launch_elem_residual(m->dm, m->kp, st)
                                         : launch_elem_residual_ff(m->dm, m->kp, st);
}

int RunGpuResidualDevice(BiofemGpuMesh *m, const double *d_x, double *d_R, void *stream)
{
  if (!m || !d_x || !d_R) return fail(85, "null argument");
  cudaStream_t st = pick_stream(stream);
  int rc = 0;
  tmark(m, st, 0);
  if (!rc) { rc = launch_positions(m->dm, m->kp, d_x, st); tmark(m, st, 1); }
  if (!rc) { rc = launch_residual_elements(m, st); tmark(m, st, 2); }
  if (!rc) { rc = launch_node_gather(m->dm, m->kp, d_x, d_R, st); tmark(m, st, 3); }
  if (!rc) { rc = launch_scale(m->dm, m->kp, d_R, st); tmark(m, st, 4); }
  if (rc) return fail(76, std::string("residual launch: ") + cudaGetErrorString((cudaError_t)rc));
  timer_collect(m);
  return 0;
}

static int residual_jacobian(BiofemGpuMesh *m, const double *d_x, double *d_R, void *d_K, void *stream, bool colmajor);

/* d_K may also be the device view of a mapped page-locked host buffer: the
   row assembly writes each row's values once, contiguously */
int RunGpuResidualJacobianDevice(BiofemGpuMesh *m, const double *d_x, double *d_R, void *d_K, void *stream)
{
  if (!m) return fail(85, "null argument");
  return residual_jacobian(m, d_x, d_R, d_K, stream, m->prm.block_layout == BIOFEM_BLOCK_COL_MAJOR);
}

/* colmajor: each 3x3 block stored column by column (PETSc SeqBAIJ); the
   Newton solve's own calls always take row-major blocks */
static int residual_jacobian(BiofemGpuMesh *m, const double *d_x, double *d_R, void *d_K, void *stream, bool colmajor)
{
  if (!m || !d_x || !d_R || !d_K) return fail(85, "null argument");
  if (!m->dm.patch) return fail(58, "host-only handle");
  cudaStream_t st = pick_stream(stream);
  int rc = 0;
  /* Independent kernels run side by side on the handle's second stream: the
     node gather beside the FP64 tangent, the FP32 tangent beside the
     float-float residual and the gather.  The row assembly waits for both
     (it reads D and the gather's max |Fext|).  With per-kernel timing on,
     every launch stays on the call's stream so that the events bracket one
     kernel each. */
  const bool overlap = !m->timer.on;
  cudaStream_t sd = overlap ? m->side : st;
  auto fork = [&]() {
    if (!overlap || rc) return;
    rc = (int)cudaEventRecord(m->ev_fork, st);
    if (!rc) rc = (int)cudaStreamWaitEvent(sd, m->ev_fork, 0);
  };
  auto join = [&]() {
    if (!overlap || rc) return;
    rc = (int)cudaEventRecord(m->ev_join, sd);
    if (!rc) rc = (int)cudaStreamWaitEvent(st, m->ev_join, 0);
  };
  tmark(m, st, 0);
  if (m->prm.precision == BIOFEM_FP64) {
    /* R from the residual kernel, so that the Jacobian call returns exactly
       the residual call's R */
    double *K = static_cast<double *>(d_K);
    if (!rc) { rc = launch_positions(m->dm, m->kp, d_x, st); tmark(m, st, 1); }
    if (!rc) { rc = launch_elem_residual(m->dm, m->kp, st, true); tmark(m, st, 2); }
    if (overlap) {
      fork();
      if (!rc) rc = launch_node_gather(m->dm, m->kp, d_x, d_R, sd);
      if (!rc) rc = launch_elem_tangent(m->dm, m->kp, st);
      join();
    } else {
      if (!rc) { rc = launch_elem_tangent(m->dm, m->kp, st); tmark(m, st, 3); }
      if (!rc) { rc = launch_node_gather(m->dm, m->kp, d_x, d_R, st); tmark(m, st, 4); }
    }
    if (!rc) { rc = launch_row_assemble(m->dm, m->kp, K, false, colmajor, st); tmark(m, st, 5); }
    if (!rc) { rc = launch_scale(m->dm, m->kp, d_R, st); tmark(m, st, 6); }
  } else {
    /* FP32-bulk: residual in float-float, tangent (D, K) in FP32 */
    float *K = static_cast<float *>(d_K);
    if (!rc) { rc = launch_positions(m->dm, m->kp, d_x, st); tmark(m, st, 1); }
    if (overlap) {
      fork();
      if (!rc) rc = launch_elem_tangent_f32(m->dm, m->kp, sd);
      if (!rc) rc = launch_elem_residual_ff(m->dm, m->kp, st);
      if (!rc) rc = launch_node_gather(m->dm, m->kp, d_x, d_R, st);
      join();
    } else {
      if (!rc) { rc = launch_elem_residual_ff(m->dm, m->kp, st); tmark(m, st, 2); }
      if (!rc) { rc = launch_elem_tangent_f32(m->dm, m->kp, st); tmark(m, st, 3); }
      if (!rc) { rc = launch_node_gather(m->dm, m->kp, d_x, d_R, st); tmark(m, st, 4); }
    }
    if (!rc) { rc = launch_row_assemble(m->dm, m->kp, K, true, colmajor, st); tmark(m, st, 5); }
    if (!rc) { rc = launch_scale(m->dm, m->kp, d_R, st); tmark(m, st, 6); }
  }
  if (rc) return fail(76, std::string("jacobian launch: ") + cudaGetErrorString((cudaError_t)rc));
  timer_collect(m);
  return 0;
}

/* Per-kernel event timing of the device calls: on = 1 starts (and clears)
   accumulation, 0 stops.  Timing synchronises on the last event of every call. */
int EnableGpuKernelTiming(BiofemGpuMesh *m, int on)
{
  if (!m) return fail(85, "null argument");
  KernelTimer &t = m->timer;
  if (on && !t.ev[0])
    for (int i = 0; i <= kMaxTimed; i++) CUDA_TRY(cudaEventCreate(&t.ev[i]));
  t.on = on != 0;
  t.n = 0; t.calls = 0;
  for (int i = 0; i < kMaxTimed; i++) t.acc_ms[i] = 0.f;
  return 0;
}

/* Accumulated milliseconds per kernel slot (launch order of the last kind of
   call) and the number of calls timed. */
int GetGpuKernelTimes(const BiofemGpuMesh *m, double *ms, int32_t nslots, int32_t *calls)
{
  if (!m || !ms) return fail(85, "null argument");
  for (int i = 0; i < nslots && i < kMaxTimed; i++) ms[i] = m->timer.acc_ms[i];
  if (calls) *calls = m->timer.calls;
  return 0;
}

int BiofemGpuSync(BiofemGpuMesh *m, void *stream)
{
  if (!m) return fail(85, "null argument");
  cudaStream_t st = pick_stream(stream);
  CUDA_TRY(cudaStreamSynchronize(st));
  int status = 0;
  CUDA_TRY(cudaMemcpyAsync(&status, m->dm.status, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (status) {
    CUDA_TRY(cudaMemsetAsync(m->dm.status, 0, sizeof(int), st));
    return fail(72, "CC3333 too small in the C33 solve (ModElemC33, active_strain.c:1676)");
  }
  return 0;
}

int RunGpuResidual(BiofemGpuMesh *m, const double *x, double *R)
{
  if (!m || !x || !R) return fail(85, "null argument");
  const size_t n = 3 * (size_t)(m->topo.n_v + m->topo.n_ghosts);
  CUDA_TRY(cudaMemcpyAsync(m->d_x, x, n * sizeof(double), cudaMemcpyHostToDevice, m->st));
  int rc = RunGpuResidualDevice(m, m->d_x, m->d_R, m->st);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(R, m->d_R, n * sizeof(double), cudaMemcpyDeviceToHost, m->st));
  return BiofemGpuSync(m, m->st);
}

int RunGpuResidualJacobian(BiofemGpuMesh *m, const double *x, double *R, void *K)
{
  if (!m || !x || !K) return fail(85, "null argument");
  const size_t n = 3 * (size_t)(m->topo.n_v + m->topo.n_ghosts);
  const size_t kbytes = 9 * (size_t)m->nnzb * (m->prm.precision == BIOFEM_FP64 ? sizeof(double) : sizeof(float));
  /* A page-locked, device-mapped K buffer (cudaHostAlloc / cudaMallocHost /
     cudaHostRegister) is written by the row assembly itself, each value once,
     so the copy-out overlaps the assembly instead of following it. */
  void *dK = m->d_K;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, K) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer)
    dK = a.devicePointer;
  else
    cudaGetLastError();
  CUDA_TRY(cudaMemcpyAsync(m->d_x, x, n * sizeof(double), cudaMemcpyHostToDevice, m->st));
  int rc = RunGpuResidualJacobianDevice(m, m->d_x, m->d_R, dK, m->st);
  if (rc) return rc;
  if (R) CUDA_TRY(cudaMemcpyAsync(R, m->d_R, n * sizeof(double), cudaMemcpyDeviceToHost, m->st));
  if (dK == m->d_K) CUDA_TRY(cudaMemcpyAsync(K, m->d_K, kbytes, cudaMemcpyDeviceToHost, m->st));
  return BiofemGpuSync(m, m->st);
}

int RunGpuResidualParts(BiofemGpuMesh *m, const double *x, double *R, double *Fint, double *Fext, double *Fdyn)
{
  if (!m || !x) return fail(85, "null argument");
  if (!m->dm.patch) return fail(58, "host-only handle");
  const size_t n = 3 * (size_t)(m->topo.n_v + m->topo.n_ghosts);
  cudaStream_t st = m->st;
  double *parts = nullptr;
  CUDA_TRY(cudaMallocAsync((void **)&parts, 3 * n * sizeof(double), st));
  CUDA_TRY(cudaMemcpyAsync(m->d_x, x, n * sizeof(double), cudaMemcpyHostToDevice, st));
  int rc = launch_positions(m->dm, m->kp, m->d_x, st);
  if (!rc) rc = launch_residual_elements(m, st);
  if (!rc) rc = launch_node_gather(m->dm, m->kp, m->d_x, m->d_R, st, parts);
  if (!rc) rc = launch_scale(m->dm, m->kp, m->d_R, st);
  if (rc) {
    cudaFreeAsync(parts, st);
    return fail(76, std::string("residual launch: ") + cudaGetErrorString((cudaError_t)rc));
  }
  double *out[4] = {R, Fint, Fext, Fdyn};
  const double *src[4] = {m->d_R, parts, parts + n, parts + 2 * n};
  for (int k = 0; k < 4; k++)
    if (out[k]) CUDA_TRY(cudaMemcpyAsync(out[k], src[k], n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaFreeAsync(parts, st));
  return BiofemGpuSync(m, st);
}

int RunGpuElementThickness(BiofemGpuMesh *m, const double *x, double *thickness)
{
  if (!m || !x || !thickness) return fail(85, "null argument");
  if (!m->dm.patch) return fail(58, "host-only handle");
  const size_t n = 3 * (size_t)(m->topo.n_v + m->topo.n_ghosts), ne = (size_t)m->kp.ne;
  cudaStream_t st = m->st;
  double *d_th = nullptr;
  CUDA_TRY(cudaMallocAsync((void **)&d_th, ne * sizeof(double), st));
  CUDA_TRY(cudaMemcpyAsync(m->d_x, x, n * sizeof(double), cudaMemcpyHostToDevice, st));
  int rc = launch_positions(m->dm, m->kp, m->d_x, st);
  if (!rc) rc = launch_elem_thickness(m->dm, m->kp, m->prm.h0, d_th, st);
  if (rc) {
    cudaFreeAsync(d_th, st);
    return fail(76, std::string("thickness launch: ") + cudaGetErrorString((cudaError_t)rc));
  }
  CUDA_TRY(cudaMemcpyAsync(thickness, d_th, ne * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaFreeAsync(d_th, st));
  return BiofemGpuSync(m, st);
}

int FormFunctionFEMGpu(void *snes, const double *x, double *R, void *ctx)
{
  (void)snes;
  return RunGpuResidual(reinterpret_cast<BiofemGpuMesh *>(ctx), x, R);
}

int FormJacobianFEMGpu(void *snes, const double *x, void *K, void *ctx)
{
  (void)snes;
  return RunGpuResidualJacobian(reinterpret_cast<BiofemGpuMesh *>(ctx), x, nullptr, K);
}

void BiofemNewtonDefaults(BiofemNewtonOptions *o)
{
  if (!o) return;
  o->rtol = 1e-10; o->atol = 0.0; o->max_newton = 20;
  o->gmres_restart = 0; o->gmres_max_it = 20000; o->gmres_rtol = 1e-9; o->line_search = 1;
  o->preconditioner = BIOFEM_PC_AMG;
  o->forcing = 0;
}

static int newton_residual_cb(void *ctx, const double *x, double *R, void *stream)
{
  return RunGpuResidualDevice(static_cast<BiofemGpuMesh *>(ctx), x, R, stream);
}

static int newton_jacobian_cb(void *ctx, const double *x, double *R, void *K, void *stream)
{
  return residual_jacobian(static_cast<BiofemGpuMesh *>(ctx), x, R, K, stream, false);
}

int RunGpuNewtonSolveDevice(BiofemGpuMesh *m, double *d_x, const BiofemNewtonOptions *opt, BiofemNewtonStats *stats,
                            void *stream)
{
  if (!m || !d_x || !stats) return fail(85, "null argument");
  if (!m->dm.patch) return fail(58, "host-only handle");
  BiofemNewtonOptions o;
  if (opt) o = *opt; else BiofemNewtonDefaults(&o);
  if (o.preconditioner != BIOFEM_PC_AMG && o.preconditioner != BIOFEM_PC_BJACOBI)
    return fail(63, "unknown preconditioner");
  if (o.forcing != 0 && o.forcing != 1) return fail(63, "unknown forcing-term rule");
  const bool use_amg = o.preconditioner == BIOFEM_PC_AMG;
  if (o.gmres_restart == 0) o.gmres_restart = (!use_amg && 3 * m->kp.nt > 50000) ? 100 : 30;   /* auto */
  if (o.gmres_restart < 1 || o.gmres_restart > 200 || o.max_newton < 0 || o.gmres_max_it < 1)
    return fail(63, "Newton options out of range");
  const int n = 3 * m->kp.nt;
  if (!m->solver || solver_m(m->solver) != o.gmres_restart) {
    if (m->solver) solver_destroy(m->solver);
    int rc = 0;
    m->solver = solver_create(n, m->kp.nt, o.gmres_restart, (void *)pick_stream(stream), &rc);
    if (!m->solver) return fail(55, std::string("Newton work allocation: ") + cudaGetErrorString((cudaError_t)rc));
  }
  if (use_amg && !m->amg) {
    int rc = 0;
    m->amg = amg_create(m->kp.nt, m->rowptr, m->colind, m->rowkind, m->topo.xyz0_full, m->topo.tri_all.data(),
                        m->kp.ne, m->dm.rowptr, m->dm.colind, m->prm.precision != BIOFEM_FP64,
                        pick_stream(stream), &rc);
    if (!m->amg) return fail(55, std::string("multigrid allocation: ") + cudaGetErrorString((cudaError_t)rc));
  }
  std::string err;
  cudaStream_t st = pick_stream(stream);
  int rc = newton_device(m->dm, m->kp, m->prm.precision != BIOFEM_FP64, m->d_K, m->d_R, d_x, o, *stats, m->solver,
                         use_amg ? m->amg : nullptr, st,
                         newton_residual_cb, newton_jacobian_cb, m, err);
  if (rc) return fail(rc > 1000 ? 76 : rc, "Newton " + err + " step failed: " + g_last_error);
  return BiofemGpuSync(m, stream);
}

int RunGpuNewtonSolve(BiofemGpuMesh *m, double *x, const BiofemNewtonOptions *opt, BiofemNewtonStats *stats)
{
  if (!m || !x || !stats) return fail(85, "null argument");
  if (!m->dm.patch) return fail(58, "host-only handle");
  BiofemNewtonOptions o;
  if (opt) o = *opt; else BiofemNewtonDefaults(&o);
  const size_t n = 3 * (size_t)m->kp.nt;
  double *dx = m->d_x;
  CUDA_TRY(cudaMemcpyAsync(dx, x, n * sizeof(double), cudaMemcpyHostToDevice, m->st));
  int rc = RunGpuNewtonSolveDevice(m, dx, &o, stats, m->st);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(x, dx, n * sizeof(double), cudaMemcpyDeviceToHost, m->st));
  CUDA_TRY(cudaStreamSynchronize(m->st));
  return 0;
}

/* ---------------- dynamic term and time-dependent activation ---------------- */
int SetGpuDynamics(BiofemGpuMesh *m, const BiofemDynParams *d)
{
  if (!m) return fail(85, "null argument");
  if (!m->dm.patch) return fail(58, "host-only handle");
  KParams &kp = m->kp;
  if (!d) { kp.dyn = 0; return 0; }
  if (!(d->dt > 0.0) || d->rho < 0.0 || (d->timeinteg != 0 && d->timeinteg != 1))
    return fail(62, "dynamic parameters out of range");
  const size_t n = 3 * (size_t)kp.nt;
  if (!m->dm.xn) {
    /* lumped mass over the real triangles (FDynamic with the DMPlex context
       of an active-strain run, main.c:1178-1270): flat reference areas and,
       per node, its corner triangles in triangle order */
    const HostTopo &T = m->topo;
    const int ntri = T.n_elmt, nt = kp.nt;
    std::vector<double> area(ntri);
    for (int t = 0; t < ntri; t++) area[t] = tri_area0(T, t);
    std::vector<int> dptr(nt + 1, 0), didx(3 * (size_t)ntri);
    for (int t = 0; t < ntri; t++) for (int k = 0; k < 3; k++) dptr[T.tri_all[3 * (size_t)t + k] + 1]++;
    for (int i = 0; i < nt; i++) dptr[i + 1] += dptr[i];
    std::vector<int> fill(dptr.begin(), dptr.end() - 1);
    for (int t = 0; t < ntri; t++) for (int k = 0; k < 3; k++) didx[fill[T.tri_all[3 * (size_t)t + k]]++] = t;
    int rc;
    if ((rc = dalloc(m, &m->dm.xn, n)) || (rc = dalloc(m, &m->dm.xnm1, n)) || (rc = dalloc(m, &m->dm.xd, n)) ||
        (rc = dalloc(m, &m->dm.xdd, n)) || (rc = dalloc(m, &m->dm.dyn_diag, (size_t)nt)) ||
        (rc = dupload(m, &m->dm.dA0, area)) || (rc = dupload(m, &m->dm.dptr, dptr)) || (rc = dupload(m, &m->dm.didx, didx)))
      return rc;
    CUDA_TRY(cudaStreamSynchronize(m->st));   /* the host vectors above go out of scope */
  }
  /* Init (main.c:1515-1540): xn = xnm1 = x = the reference coordinates, xd = xdd = 0 */
  CUDA_TRY(cudaMemcpyAsync(m->dm.xn, m->dm.X, n * sizeof(double), cudaMemcpyDeviceToDevice, m->st));
  CUDA_TRY(cudaMemcpyAsync(m->dm.xnm1, m->dm.X, n * sizeof(double), cudaMemcpyDeviceToDevice, m->st));
  CUDA_TRY(cudaMemsetAsync(m->dm.xd, 0, n * sizeof(double), m->st));
  CUDA_TRY(cudaMemsetAsync(m->dm.xdd, 0, n * sizeof(double), m->st));
  /* the constants of FDynamic (main.c:1171-1176) and xAccVel (main.c:1383-1385) */
  const double dt = d->dt, G = d->newmark_gamma, B = 0.25 * (G + 0.5) * (G + 0.5);
  kp.dyn = 1; kp.dyn_central = d->timeinteg; kp.dyn_damp = d->damping != 0;
  kp.dyn_rhoh0 = d->rho * m->prm.h0; kp.dyn_dt = dt; kp.dyn_dampf = d->dampfactor;
  kp.dyn_M1 = 1. / (B * std::pow(dt, 2)); kp.dyn_M2 = 1. / (B * dt); kp.dyn_M3 = (1. / (2 * B)) - 1.;
  kp.dyn_C1 = G / (B * dt); kp.dyn_C2 = (G / B) - 1; kp.dyn_C3 = dt * (G / (2. * B) - 1);
  kp.dyn_U2 = (1. - G) * dt; kp.dyn_U3 = G * dt;
  int rc = launch_dyn_diag(m->dm, kp, m->st);
  if (rc) return fail(76, std::string("dynamic diagonal launch: ") + cudaGetErrorString((cudaError_t)rc));
  CUDA_TRY(cudaStreamSynchronize(m->st));
  return 0;
}

int SetGpuDynamicState(BiofemGpuMesh *m, const double *xn, const double *xnm1, const double *xd, const double *xdd)
{
  if (!m) return fail(85, "null argument");
  if (!m->dm.xn) return fail(58, "dynamics not enabled (SetGpuDynamics)");
  const size_t bytes = 3 * sizeof(double) * (size_t)m->kp.nt;
  const double *src[4] = {xn, xnm1, xd, xdd};
  double *dst[4] = {m->dm.xn, m->dm.xnm1, m->dm.xd, m->dm.xdd};
  for (int k = 0; k < 4; k++)
    if (src[k]) CUDA_TRY(cudaMemcpyAsync(dst[k], src[k], bytes, cudaMemcpyHostToDevice, m->st));
  CUDA_TRY(cudaStreamSynchronize(m->st));
  return 0;
}

int GetGpuDynamicState(BiofemGpuMesh *m, double *xn, double *xnm1, double *xd, double *xdd)
{
  if (!m) return fail(85, "null argument");
  if (!m->dm.xn) return fail(58, "dynamics not enabled (SetGpuDynamics)");
  const size_t bytes = 3 * sizeof(double) * (size_t)m->kp.nt;
  double *dst[4] = {xn, xnm1, xd, xdd};
  const double *src[4] = {m->dm.xn, m->dm.xnm1, m->dm.xd, m->dm.xdd};
  for (int k = 0; k < 4; k++)
    if (dst[k]) CUDA_TRY(cudaMemcpyAsync(dst[k], src[k], bytes, cudaMemcpyDeviceToHost, m->st));
  CUDA_TRY(cudaStreamSynchronize(m->st));
  return 0;
}

int RunGpuDynamicUpdate(BiofemGpuMesh *m, const double *x)
{
  if (!m || !x) return fail(85, "null argument");
  if (!m->dm.xn) return fail(58, "dynamics not enabled (SetGpuDynamics)");
  const size_t n = 3 * (size_t)m->kp.nt;
  CUDA_TRY(cudaMemcpyAsync(m->d_x, x, n * sizeof(double), cudaMemcpyHostToDevice, m->st));
  int rc = launch_dyn_update(m->dm, m->kp, m->d_x, m->st);
  if (rc) return fail(76, std::string("dynamic update launch: ") + cudaGetErrorString((cudaError_t)rc));
  CUDA_TRY(cudaStreamSynchronize(m->st));
  return 0;
}

int SetGpuElementGamma(BiofemGpuMesh *m, const double *gamma_e)
{
  if (!m || !gamma_e) return fail(85, "null argument");
  if (!m->dm.patch) return fail(58, "host-only handle");
  const int ne = m->kp.ne;
  if (!m->d_gam) { int rc = dalloc(m, &m->d_gam, (size_t)ne); if (rc) return rc; }
  CUDA_TRY(cudaMemcpyAsync(m->d_gam, gamma_e, sizeof(double) * ne, cudaMemcpyHostToDevice, m->st));
  /* reference constants with gamma_e in place of gamma * gamma_scale */
  KParams kp = m->kp;
  kp.gamma = 1.0;
  int rc = launch_positions(m->dm, kp, m->dm.X, m->st);
  if (!rc) rc = launch_ref_prep(m->dm, kp, m->d_fib, m->d_gam, const_cast<double *>(m->dm.eref), m->st);
  const size_t nref = (size_t)(kRefPerQp * kp.nq + kRefPerElem) * ne;
  if (!rc && m->dm.erefF) rc = launch_to_float(m->dm.eref, const_cast<float *>(m->dm.erefF), (long long)nref, m->st);
  if (!rc && m->dm.erefFF) rc = launch_to_ff(m->dm.eref, const_cast<void *>(m->dm.erefFF), (long long)nref, m->st);
  if (rc) return fail(76, std::string("activation update launch: ") + cudaGetErrorString((cudaError_t)rc));
  CUDA_TRY(cudaStreamSynchronize(m->st));
  return 0;
}

/* Basis-derivative tables (regular + irregular valences 3..10), 11*5*16. */
/* the 11 subdivision tables (the cap table is internal) */
int GetGpuBasisTables(double *out)
{
  if (!out) return fail(85, "null argument");
  double tabs[kNumTables * 80];
  host_tables(tabs, BIOFEM_BASIS_REFERENCE);
  std::copy(tabs, tabs + kCapTable * 80, out);
  return 0;
}

int GetGpuBasisTablesKind(int32_t basis, double *out)
{
  if (!out) return fail(85, "null argument");
  if (basis != BIOFEM_BASIS_REFERENCE && basis != BIOFEM_BASIS_EXACT) return fail(63, "unknown basis tables");
  double tabs[kNumTables * 80];
  host_tables(tabs, basis);
  std::copy(tabs, tabs + kCapTable * 80, out);
  return 0;
}

} /* extern "C" */
