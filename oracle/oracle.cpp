/*
 * CPU restatement of BioFEM-IA's element residual path  -- TEST INFRASTRUCTURE.
 *
 * This file is the oracle: it restates, operation for operation, the
 * reference's FP64 algorithm for one residual evaluation of the active-strain
 * Kirchhoff-Love shell (the FormFunctionFEM sequence at np = 1).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs load it, and only as the
 * checker or the timed CPU baseline; the product library never links it.
 *
 * Every function cites the reference function it follows.  Arithmetic is
 * written in the reference's evaluation order, so that with Scalar = double
 * and -ffp-contract=off the results are bitwise equal to the reference build
 * (oracle/_ref, pinned by tests/test_oracle_pin.py).
 *
 * The element pipeline is a template over the scalar type of the CURRENT
 * configuration.  Instantiated with Dual<N> (forward-mode dual numbers), the
 * same code yields exact directional derivatives of the residual, which are
 * the checker for the GPU tangent stiffness (the reference has no tangent:
 * its Newton solve is matrix-free, main.c:464-466).
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

static const int kMissing = 1000000;   /* bending.c:1291 sentinel */
static const int kMaxQp = 6;

/* ---------------- dual numbers ---------------- */
template <int N> struct Dual {
  double v;
  double d[N];
  Dual() : v(0.0) { for (int i = 0; i < N; i++) d[i] = 0.0; }
  Dual(double a) : v(a) { for (int i = 0; i < N; i++) d[i] = 0.0; }
};
template <int N> inline Dual<N> operator+(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = a.v + b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = a.v - b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N> &a) { Dual<N> r; r.v = -a.v; for (int i = 0; i < N; i++) r.d[i] = -a.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = a.v * b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> inline Dual<N> operator*(double a, const Dual<N> &b) { Dual<N> r; r.v = a * b.v; for (int i = 0; i < N; i++) r.d[i] = a * b.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N> &a, double b) { Dual<N> r; r.v = a.v * b; for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b; return r; }
template <int N> inline Dual<N> operator/(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = a.v / b.v; for (int i = 0; i < N; i++) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v); return r; }
template <int N> inline Dual<N> operator/(double a, const Dual<N> &b) { Dual<N> r; r.v = a / b.v; for (int i = 0; i < N; i++) r.d[i] = -a * b.d[i] / (b.v * b.v); return r; }
template <int N> inline Dual<N> operator/(const Dual<N> &a, double b) { Dual<N> r; r.v = a.v / b; for (int i = 0; i < N; i++) r.d[i] = a.d[i] / b; return r; }
template <int N> inline Dual<N> operator+(const Dual<N> &a, double b) { Dual<N> r = a; r.v = a.v + b; return r; }
template <int N> inline Dual<N> operator+(double a, const Dual<N> &b) { Dual<N> r = b; r.v = a + b.v; return r; }
template <int N> inline Dual<N> operator-(const Dual<N> &a, double b) { Dual<N> r = a; r.v = a.v - b; return r; }
template <int N> inline Dual<N> operator-(double a, const Dual<N> &b) { Dual<N> r; r.v = a - b.v; for (int i = 0; i < N; i++) r.d[i] = -b.d[i]; return r; }
template <int N> inline Dual<N> &operator+=(Dual<N> &a, const Dual<N> &b) { a = a + b; return a; }
template <int N> inline Dual<N> &operator/=(Dual<N> &a, const Dual<N> &b) { a = a / b; return a; }
template <int N> inline Dual<N> sqrt(const Dual<N> &a) { Dual<N> r; r.v = std::sqrt(a.v); for (int i = 0; i < N; i++) r.d[i] = a.d[i] / (2.0 * r.v); return r; }
template <int N> inline double val(const Dual<N> &a) { return a.v; }
inline double val(double a) { return a; }
using std::sqrt;

/* ---------------- 3-vectors (math.c:1-72) ---------------- */
template <class T> struct V3 { T x, y, z; };
template <class T> inline V3<T> PLUS(const V3<T> &a, const V3<T> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> MINUS(const V3<T> &a, const V3<T> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> CROSS(const V3<T> &a, const V3<T> &b)
{   /* math.c:27-37 */
  V3<T> r;
  r.x = a.y * b.z - b.y * a.z;
  r.y = -a.x * b.z + b.x * a.z;
  r.z = a.x * b.y - b.x * a.y;
  return r;
}
template <class T> inline T DOT(const V3<T> &a, const V3<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T SIZE(const V3<T> &a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
template <class T> inline V3<T> UNIT(const V3<T> &a)
{   /* math.c:46-55 */
  T n = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return {a.x / n, a.y / n, a.z / n};
}
template <class S, class T> inline V3<T> AMULT(const S &al, const V3<T> &a) { return {al * a.x, al * a.y, al * a.z}; }

/* ---------------- 3x3 helpers (math.c:75-182) ---------------- */
template <class T> inline void INV(const T A[3][3], T B[3][3])
{   /* math.c:75-89: cofactor inverse, no singularity guard */
  T T11 = A[0][0], T12 = A[0][1], T13 = A[0][2];
  T T21 = A[1][0], T22 = A[1][1], T23 = A[1][2];
  T T31 = A[2][0], T32 = A[2][1], T33 = A[2][2];
  T det = T11 * (T33 * T22 - T32 * T23) - T21 * (T33 * T12 - T32 * T13) + T31 * (T23 * T12 - T22 * T13);
  T c = 1 / det;
  B[0][0] = c * (T33 * T22 - T32 * T23);   B[0][1] = -c * (T33 * T12 - T32 * T13); B[0][2] = c * (T23 * T12 - T22 * T13);
  B[1][0] = -c * (T33 * T21 - T31 * T23);  B[1][1] = c * (T33 * T11 - T31 * T13);  B[1][2] = -c * (T23 * T11 - T21 * T13);
  B[2][0] = c * (T32 * T21 - T31 * T22);   B[2][1] = -c * (T32 * T11 - T31 * T12); B[2][2] = c * (T22 * T11 - T21 * T12);
}
template <class A, class B, class C> inline void MATMULT(const A a[3][3], const B b[3][3], C c[3][3])
{   /* math.c:92-119 */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      c[i][j] = 0.0;
      for (int k = 0; k < 3; k++) c[i][j] = c[i][j] + a[i][k] * b[k][j];
    }
}
template <class T> inline T DET3x3(const T A[3][3])
{   /* math.c:145-151 */
  return A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1])
       - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0])
       + A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
}
template <class G, class T> inline void RaiseIndices2(const G g[3][3], const T a[3][3], T out[3][3])
{   /* math.c:154-167 */
  T tmp[3][3];
  MATMULT(g, a, tmp);
  MATMULT(tmp, g, out);
}

/* ---------------- element tables ---------------- */
/* Centroid derivatives of the 12 regular box-spline basis functions,
   four-decimal values as tabulated in active_strain.c:69-88. */
static const double kNaRef[2][12] = {
  {-0.0247, -0.0309, 0.0000, -0.4815, -0.1852, 0.0247, 0.4815, 0.0000, -0.0062, 0.0309, 0.1852, 0.0062},
  {-0.0309, -0.0247, -0.1852, -0.4815, 0.0000, -0.0062, 0.0000, 0.4815, 0.0247, 0.0062, 0.1852, 0.0309}};
static const double kNabRef[3][12] = {
  {0.1111, 0.2222, -0.2222, -0.2222, 0.4444, 0.1111, -0.2222, -0.8889, 0.0000, 0.2222, 0.4444, 0.0000},
  {0.2222, 0.1111, 0.4444, -0.2222, -0.2222, 0.0000, -0.8889, -0.2222, 0.1111, 0.0000, 0.4444, 0.2222},
  {0.1667, 0.1667, -0.1111, 0.2222, -0.1111, -0.0556, -0.4444, -0.4444, -0.0556, 0.0556, 0.5556, 0.0556}};

/* Active tables: the reference's four-decimal values (default), or, as an
   extension for meshes much finer than the shell thickness, the exact
   rationals they round (first derivatives k/324, second derivatives k/108,
   rows summing to zero).  Set by oracle_set_basis before oracle_setup. */
static double kNa[2][12], kNab[3][12];
static int set_basis_tables(int kind)
{
  if (kind != 0 && kind != 1) return 63;
  for (int r = 0; r < 2; r++) for (int i = 0; i < 12; i++)
    kNa[r][i] = kind ? std::nearbyint(kNaRef[r][i] * 324.0) / 324.0 : kNaRef[r][i];
  for (int r = 0; r < 3; r++) for (int i = 0; i < 12; i++)
    kNab[r][i] = kind ? std::nearbyint(kNabRef[r][i] * 108.0) / 108.0 : kNabRef[r][i];
  return 0;
}
static const int g_tables_init = set_basis_tables(0);

/* Gauss-Legendre points/weights on [-1,1] (active_strain.c:174-230 for n = 1..5;
   n = 6 is an extension: the reference stops at 5). */
static int gauss_rule(int n, double *th, double *w)
{
  switch (n) {
  case 1: th[0] = 0.0; w[0] = 2.0; return 0;
  case 2: th[0] = -0.5773502691896257; th[1] = 0.5773502691896257; w[0] = w[1] = 1.0; return 0;
  case 3: th[0] = -0.7745966692414834; th[1] = 0.0; th[2] = 0.7745966692414834;
          w[0] = w[2] = 0.5555555555555556; w[1] = 0.8888888888888888; return 0;
  case 4: th[0] = -0.8611363115940526; th[1] = -0.3399810435848563; th[2] = 0.3399810435848563; th[3] = 0.8611363115940526;
          w[0] = w[3] = 0.3478548451374538; w[1] = w[2] = 0.6521451548625461; return 0;
  case 5: th[0] = -0.9061798459386640; th[1] = -0.5384693101056831; th[2] = 0.0; th[3] = 0.5384693101056831; th[4] = 0.9061798459386640;
          w[0] = w[4] = 0.2369268850561891; w[1] = w[3] = 0.4786286704993665; w[2] = 0.5688888888888889; return 0;
  case 6: th[0] = -0.9324695142031521; th[1] = -0.6612093864662645; th[2] = -0.2386191860831969;
          th[3] = 0.2386191860831969; th[4] = 0.6612093864662645; th[5] = 0.9324695142031521;
          w[0] = w[5] = 0.1713244923791704; w[1] = w[4] = 0.3607615730481386; w[2] = w[3] = 0.4679139345726910; return 0;
  default: return 63;
  }
}

/* ---------------- mesh + parameters ---------------- */
struct Params {
  int n_qp, c33_iters, clamp;
  double mu, K, h0, gamma, pressure;
  double theta[kMaxQp], w[kMaxQp];
  int dead_load = 0;   /* 1: SurfaceConstNormalPressure (external.c:699-730) instead of the follower load */
  int iso_act = 0;     /* 1: -cart_fib_act 0, the isotropic active gradient (active_strain.c:1238-1255) */
};

/* load / activation options of the next setup (oracle_set_load_options) */
static int g_dead_load = 0, g_iso_act = 0;
/* n_elmt_base of the next setup (oracle_set_elmt_base) */
static int g_elmt_base = 0;

struct Mesh {
  int n_v = 0, n_elmt = 0, n_ghosts = 0, n_edge = 0;
  int n_elmt_base = 0;                     /* > 0: elements ec >= n_elmt_base are apex-cap triangles */
  std::vector<int> nv1, nv2, nv3;          /* n_elmt + 2 n_ghosts */
  std::vector<int> n_bnodes, bnodes;
  std::vector<int> ire, irv, val, patch;   /* patch: 16 n_elmt */
  std::vector<int> ghost_nv3;              /* per ghost, the reflected interior node */
  std::vector<double> x0, y0, z0;          /* n_v + n_ghosts reference coordinates */
  std::vector<double> fib, gscale, dA0;
};

/* Apex-cap element (ec >= n_elmt_base when n_elmt_base > 0): a flat
   constant-strain triangle closing the apex (bending.c:1282-1294,
   active_strain.c:448-470, 1807-1853). */
inline bool is_cap(const Mesh &m, int ec) { return m.n_elmt_base > 0 && ec >= m.n_elmt_base; }

/* ---------------- topology (bending.c) ---------------- */
/* The reference's searches scan every triangle for each query
   (O(N_e^2) overall).  Every query looks for triangles holding a given node,
   and the result of each is the last match in triangle order, so scanning only
   the triangles incident to that node, in increasing index, gives the same
   tables (the fast mode, oracle_set_fast_topology; tests pin both modes
   against the reference build).  scan_tris(node, f) calls f(i) for the
   candidate triangles i in increasing order. */
static int g_fast_topology = 0;

struct TriScan {
  const Mesh &m;
  int ntri;
  bool fast;
  std::vector<int> ptr, idx;   /* node -> incident triangles (fast mode) */
  TriScan(const Mesh &mm, int nt, int nnode, bool f) : m(mm), ntri(nt), fast(f)
  {
    if (!fast) return;
    ptr.assign(nnode + 1, 0);
    for (int i = 0; i < nt; i++) {
      const int c[3] = {m.nv1[i], m.nv2[i], m.nv3[i]};
      for (int k = 0; k < 3; k++)
        if (c[k] >= 0 && c[k] < nnode && (k == 0 || c[k] != c[0]) && (k < 2 || c[k] != c[1])) ptr[c[k] + 1]++;
    }
    for (int v = 0; v < nnode; v++) ptr[v + 1] += ptr[v];
    idx.assign(ptr[nnode], 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < nt; i++) {
      const int c[3] = {m.nv1[i], m.nv2[i], m.nv3[i]};
      for (int k = 0; k < 3; k++)
        if (c[k] >= 0 && c[k] < nnode && (k == 0 || c[k] != c[0]) && (k < 2 || c[k] != c[1])) idx[fill[c[k]]++] = i;
    }
  }
  template <class F> void operator()(int node, F f) const
  {
    if (!fast) { for (int i = 0; i < ntri; i++) f(i); return; }
    if (node < 0 || node + 1 >= (int)ptr.size()) return;   /* no triangle holds it */
    for (int k = ptr[node]; k < ptr[node + 1]; k++) f(idx[k]);
  }
};

/* GlobalGhostInit, bending.c:1670-1757.  Writes ghost coordinates into
   (x, y, z) and the reference arrays, and the 2 triangles of every ghost. */
static void global_ghost_init(Mesh &m, std::vector<double> &x, std::vector<double> &y, std::vector<double> &z)
{
  int count = 0, nv3 = 0;
  m.ghost_nv3.assign(m.n_ghosts, 0);
  const TriScan scan(m, m.n_elmt, m.n_v, g_fast_topology != 0);
  for (int edge_n = 0; edge_n < m.n_edge; edge_n++) {
    int start = 0, end = 0;
    for (int e = 0; e < edge_n + 1; e++) end += m.n_bnodes[e];
    start = end - m.n_bnodes[edge_n];
    const int n_local = end - start;
    const int ring_first = count;
    /* the apex ring (edge 0) reflects through base elements only, bending.c:1687 */
    const int ec_limit = (edge_n == 0 && m.n_elmt_base > 0) ? m.n_elmt_base : m.n_elmt;
    for (int li = 0; li < n_local; li++) {
      const int i = start + li, inext = start + (li + 1) % n_local;
      const int nv1 = m.bnodes[inext], nv2 = m.bnodes[i];
      scan(nv1, [&](int ec) {
        if (ec >= ec_limit) return;
        int c = 0;
        if (nv1 == m.nv1[ec] || nv1 == m.nv2[ec] || nv1 == m.nv3[ec]) c++;
        if (nv2 == m.nv1[ec] || nv2 == m.nv2[ec] || nv2 == m.nv3[ec]) c++;
        if (c == 2) {
          if (m.nv1[ec] != nv1 && m.nv1[ec] != nv2) nv3 = m.nv1[ec];
          else if (m.nv2[ec] != nv1 && m.nv2[ec] != nv2) nv3 = m.nv2[ec];
          else nv3 = m.nv3[ec];
        }
      });
      const int g = m.n_v + count;
      x[g] = x[nv2] + x[nv1] - x[nv3];
      y[g] = y[nv2] + y[nv1] - y[nv3];
      z[g] = z[nv2] + z[nv1] - z[nv3];
      m.x0[g] = x[g]; m.y0[g] = y[g]; m.z0[g] = z[g];
      m.ghost_nv3[count] = nv3;
      m.nv2[m.n_elmt + 2 * count] = nv2;
      m.nv1[m.n_elmt + 2 * count] = nv1;
      m.nv3[m.n_elmt + 2 * count] = g;
      const int gprev = (li == 0) ? (m.n_v + ring_first + n_local - 1) : (g - 1);
      m.nv1[m.n_elmt + 2 * count + 1] = g;
      m.nv2[m.n_elmt + 2 * count + 1] = nv2;
      m.nv3[m.n_elmt + 2 * count + 1] = gprev;
      count++;
    }
  }
}

/* IrrVer, bending.c:1188-1267: only base elements (ec < n_elmt_base, when
   set) count towards a node's valence (bending.c:1204-1210); irv is set over
   every element. */
static void irrver(Mesh &m)
{
  std::vector<int> irr(m.n_v, 0), elmt;
  elmt.reserve(64);
  for (int ec = 0; ec < m.n_elmt; ec++) { m.ire[ec] = 0; m.irv[ec] = 0; m.val[ec] = 6; }
  const int nb = (int)m.bnodes.size();
  const bool fast = g_fast_topology != 0;
  const TriScan scan(m, m.n_elmt, m.n_v, fast);
  const int ec_limit = (m.n_elmt_base > 0) ? m.n_elmt_base : m.n_elmt;
  std::vector<char> bflag;
  if (fast) { bflag.assign(m.n_v, 0); for (int i = 0; i < nb; i++) if (m.bnodes[i] >= 0 && m.bnodes[i] < m.n_v) bflag[m.bnodes[i]] = 1; }
  for (int nc = 0; nc < m.n_v; nc++) {
    int count = 0, bcount = 0, is_b = 0;
    elmt.clear();
    if (fast) is_b = bflag[nc];
    else for (int i = 0; i < nb; i++) if (nc == m.bnodes[i]) { is_b = 1; break; }
    scan(nc, [&](int ec) {
      if (ec >= ec_limit) return;
      if (nc == m.nv1[ec] || nc == m.nv2[ec] || nc == m.nv3[ec]) { elmt.push_back(ec); count++; }
    });
    if (is_b) bcount = count + 3;
    if (bcount == 0) {
      if (count != 6) { irr[nc] = 1; for (int e : elmt) { m.ire[e] = 1; m.val[e] = count; } }
    } else {
      if (bcount != 6) { irr[nc] = 1; for (int e : elmt) { m.ire[e] = 1; m.val[e] = bcount; } }
    }
  }
  for (int ec = 0; ec < m.n_elmt; ec++) {
    if (fast) {   /* the corners in increasing node order: the scan over nc keeps the last */
      int c[3] = {m.nv1[ec], m.nv2[ec], m.nv3[ec]};
      std::sort(c, c + 3);
      for (int k = 0; k < 3; k++) {
        const int nc = c[k];
        if (nc < 0 || nc >= m.n_v || irr[nc] != 1) continue;
        if (nc == m.nv1[ec]) m.irv[ec] = 1;
        if (nc == m.nv2[ec]) m.irv[ec] = 2;
        if (nc == m.nv3[ec]) m.irv[ec] = 3;
      }
      continue;
    }
    for (int nc = 0; nc < m.n_v; nc++)
      if (irr[nc] == 1) {
        if (nc == m.nv1[ec]) m.irv[ec] = 1;
        if (nc == m.nv2[ec]) m.irv[ec] = 2;
        if (nc == m.nv3[ec]) m.irv[ec] = 3;
      }
  }
}

/* One shared-edge search step of Patch(): if triangle (a,b,c) holds both
   p[A] and p[B], pick its first corner outside `excl` (and, when skip_self,
   only for i != ec). bending.c:1302-1619 repeats this pattern. */
static inline void patch_pick(int *p, int A, int B, int n1, int n2, int n3, int e1, int e2, int e3, bool guard, int out)
{
  int mm = 0;
  if (p[A] == n1 || p[A] == n2 || p[A] == n3) mm++;
  if (p[B] == n1 || p[B] == n2 || p[B] == n3) mm++;
  if (mm == 2) {
    if (n1 != e1 && n1 != e2 && n1 != e3 && guard) p[out] = n1;
    else if (n2 != e1 && n2 != e2 && n2 != e3 && guard) p[out] = n2;
    else if (n3 != e1 && n3 != e2 && n3 != e3 && guard) p[out] = n3;
  }
}

/* Patch, bending.c:1270-1667.  A cap element's patch holds only its corners,
   in slots 3, 6 and 7, and the sentinel elsewhere (bending.c:1282-1294).  In
   every pick the node
   p[A] is a corner of the element (p[3], p[6], p[7] regular; p[0], p[1], p[v]
   irregular), and no pick overwrites a corner slot for valence v >= 4, so a
   triangle can match only if it holds one of the three corners: the fast mode
   runs the reference's loops, picks in the same order, over the triangles
   incident to the corners in increasing index (valence 3, where slot v - 2 = 1
   is a corner, keeps the full scan). */
static void patch_build(Mesh &m)
{
  const int ntot = m.n_elmt + 2 * m.n_ghosts;
  const bool fast = g_fast_topology != 0;
  const TriScan scan(m, ntot, m.n_v + m.n_ghosts, fast);
  std::vector<int> cand, all;
  all.resize(ntot);
  for (int i = 0; i < ntot; i++) all[i] = i;
  int p[64];
  for (int ec = 0; ec < m.n_elmt; ec++) {
    const int v = m.val[ec];
    if (is_cap(m, ec)) {
      for (int i = 0; i < 16; i++) m.patch[16 * ec + i] = kMissing;
      m.patch[16 * ec + 3] = m.nv1[ec];
      m.patch[16 * ec + 6] = m.nv2[ec];
      m.patch[16 * ec + 7] = m.nv3[ec];
      continue;
    }
    const std::vector<int> *tris = &all;
    if (fast && v >= 4) {
      cand.clear();
      const int c[3] = {m.nv1[ec], m.nv2[ec], m.nv3[ec]};
      for (int k = 0; k < 3; k++) scan(c[k], [&](int i) { cand.push_back(i); });
      std::sort(cand.begin(), cand.end());
      cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
      tris = &cand;
    }
    for (int i = 0; i < v + 6; i++) p[i] = kMissing;
    if (m.ire[ec] == 0) {
      p[3] = m.nv1[ec]; p[6] = m.nv2[ec]; p[7] = m.nv3[ec];
      for (int i : *tris) {
        const int a = m.nv1[i], b = m.nv2[i], c = m.nv3[i];
        const bool g = (i != ec);
        patch_pick(p, 3, 6, a, b, c, p[3], p[6], p[6], g, 2);
        patch_pick(p, 3, 7, a, b, c, p[3], p[7], p[7], g, 4);
        patch_pick(p, 6, 7, a, b, c, p[6], p[7], p[7], g, 10);
      }
      for (int i : *tris) {
        const int a = m.nv1[i], b = m.nv2[i], c = m.nv3[i];
        patch_pick(p, 3, 2, a, b, c, p[3], p[2], p[6], true, 0);
        patch_pick(p, 3, 4, a, b, c, p[3], p[4], p[7], true, 1);
        patch_pick(p, 6, 2, a, b, c, p[6], p[2], p[3], true, 5);
        patch_pick(p, 6, 10, a, b, c, p[6], p[10], p[7], true, 9);
        patch_pick(p, 7, 10, a, b, c, p[7], p[10], p[6], true, 11);
        patch_pick(p, 7, 4, a, b, c, p[7], p[4], p[3], true, 8);
      }
    } else if (m.ire[ec] == 1) {
      if (m.irv[ec] == 1) { p[0] = m.nv1[ec]; p[1] = m.nv2[ec]; p[v] = m.nv3[ec]; }
      else if (m.irv[ec] == 2) { p[0] = m.nv2[ec]; p[1] = m.nv3[ec]; p[v] = m.nv1[ec]; }
      else if (m.irv[ec] == 3) { p[0] = m.nv3[ec]; p[1] = m.nv1[ec]; p[v] = m.nv2[ec]; }
      for (int i : *tris) {
        const int a = m.nv1[i], b = m.nv2[i], c = m.nv3[i];
        const bool g = (i != ec);
        patch_pick(p, 0, 1, a, b, c, p[0], p[1], p[1], g, 2);
        patch_pick(p, 0, v, a, b, c, p[0], p[v], p[v], g, v - 1);
        patch_pick(p, 1, v, a, b, c, p[1], p[v], p[v], g, v + 1);
      }
      for (int i : *tris) {
        const int a = m.nv1[i], b = m.nv2[i], c = m.nv3[i];
        patch_pick(p, 0, 2, a, b, c, p[0], p[2], p[1], true, 3);
        patch_pick(p, 0, v - 1, a, b, c, p[0], p[v - 1], p[v], true, v - 2);
        patch_pick(p, 1, 2, a, b, c, p[1], p[2], p[0], true, v + 3);
        patch_pick(p, 1, v + 1, a, b, c, p[1], p[v + 1], p[v], true, v + 2);
        patch_pick(p, v, v + 1, a, b, c, p[v], p[v + 1], p[1], true, v + 4);
        patch_pick(p, v, v - 1, a, b, c, p[v], p[v - 1], p[0], true, v + 5);
      }
      if (m.val[ec] > 6) {
        for (int k = 0; k < v - 6; k++)
          for (int i : *tris) {
            const int a = m.nv1[i], b = m.nv2[i], c = m.nv3[i];
            patch_pick(p, 0, 3 + k, a, b, c, p[0], p[3 + k], p[2 + k], true, k + 4);
            patch_pick(p, 0, v - 2 - k, a, b, c, p[0], p[v - 2 - k], p[v - 1 - k], true, v - 3 - k);
          }
      }
    }
    /* sentinel fix-up, bending.c:1637-1650 */
    int fix = -1, gfix = -1;
    for (int i = 0; i < v + 6 && i < 16; i++) {
      if (p[i] == kMissing) continue;
      if (fix < 0) fix = p[i];
      if (p[i] >= m.n_v) { gfix = p[i]; break; }
    }
    if (gfix >= 0) fix = gfix;
    if (fix >= 0) for (int i = 0; i < v + 6 && i < 16; i++) if (p[i] == kMissing) p[i] = fix;
    for (int i = 0; i < 16; i++) m.patch[16 * ec + i] = kMissing;
    for (int i = 0; i < v + 6 && i < 16; i++) m.patch[16 * ec + i] = p[i];
  }
}

/* ---------------- element pipeline ---------------- */
template <class T> struct Geom {
  int nen = 12;
  V3<T> a1, a2, n, gc1, gc2, Aaa, Abb, Aab;
  double INa0[16], INa1[16], INab0[16], INab1[16], INab2[16];
};

/* One-step subdivision operator for an irregular patch (active_strain.c:594-666):
   fills IN arrays (derivative weights of the nen = v+6 control points).
   The entries of the subdivision matrix are Loop's rules (vertex, edge and
   face masks) in the reference's node ordering; they are written in the same
   order as the reference writes them, so overlapping rows for small v resolve
   identically. */
static int irregular_weights(int v, double *INa0, double *INa1, double *INab0, double *INab1, double *INab2)
{
  const int nen = v + 6;
  if (v + 12 > 64 || nen > 16 || v < 3) return 56;
  static thread_local double B1[64][64];
  const double w = (1.0 / (double)v) * (0.625 - std::pow(0.375 + 0.25 * std::cos(2 * 3.14159265358979323846264338327950288419716939937510582 / (double)v), 2.0));
  for (int i = 0; i < v + 12; i++) for (int j = 0; j < nen; j++) B1[i][j] = 0.0;
  B1[0][0] = 1 - v * w; for (int j = 0; j < v; j++) B1[0][1 + j] = w;
  B1[1][0] = 0.375; B1[1][1] = 0.375; B1[1][2] = 0.125; B1[1][v] = 0.125;
  B1[2][0] = 0.375; B1[2][1] = 0.125; B1[2][2] = 0.375; B1[2][3] = 0.125;
  if (v > 5) { B1[v - 4][0] = 0.375; B1[v - 4][v - 5] = 0.125; B1[v - 4][v - 4] = 0.375; B1[v - 4][v - 3] = 0.125; }
  if (v > 4) { B1[v - 3][0] = 0.375; B1[v - 3][v - 4] = 0.125; B1[v - 3][v - 3] = 0.375; B1[v - 3][v - 2] = 0.125; }
  B1[v - 2][0] = 0.375; B1[v - 2][v - 3] = 0.125; B1[v - 2][v - 2] = 0.375; B1[v - 2][v - 1] = 0.125;
  B1[v - 1][0] = 0.375; B1[v - 1][v - 2] = 0.125; B1[v - 1][v - 1] = 0.375; B1[v - 1][v] = 0.125;
  B1[v][0] = 0.375; B1[v][1] = 0.125; B1[v][v - 1] = 0.125; B1[v][v] = 0.375;
  B1[v + 1][0] = 0.125; B1[v + 1][1] = 0.375; B1[v + 1][v] = 0.375; B1[v + 1][v + 1] = 0.125;
  B1[v + 2][0] = 0.0625; B1[v + 2][1] = 0.625; B1[v + 2][2] = 0.0625; B1[v + 2][v] = 0.0625; B1[v + 2][v + 1] = 0.0625; B1[v + 2][v + 2] = 0.0625; B1[v + 2][v + 3] = 0.0625;
  B1[v + 3][0] = 0.125; B1[v + 3][1] = 0.375; B1[v + 3][2] = 0.375; B1[v + 3][v + 3] = 0.125;
  B1[v + 4][0] = 0.0625; B1[v + 4][1] = 0.0625; B1[v + 4][v - 1] = 0.0625; B1[v + 4][v] = 0.625; B1[v + 4][v + 1] = 0.0625; B1[v + 4][v + 4] = 0.0625; B1[v + 4][v + 5] = 0.0625;
  B1[v + 5][0] = 0.125; B1[v + 5][v - 1] = 0.375; B1[v + 5][v] = 0.375; B1[v + 5][v + 5] = 0.125;
  B1[v + 6][1] = 0.375; B1[v + 6][v] = 0.125; B1[v + 6][v + 1] = 0.375; B1[v + 6][v + 2] = 0.125;
  B1[v + 7][1] = 0.375; B1[v + 7][v + 1] = 0.125; B1[v + 7][v + 2] = 0.375; B1[v + 7][v + 3] = 0.125;
  B1[v + 8][1] = 0.375; B1[v + 8][2] = 0.125; B1[v + 8][v + 2] = 0.125; B1[v + 8][v + 3] = 0.375;
  B1[v + 9][1] = 0.125; B1[v + 9][v] = 0.375; B1[v + 9][v + 1] = 0.375; B1[v + 9][v + 4] = 0.125;
  B1[v + 10][v] = 0.375; B1[v + 10][v + 1] = 0.125; B1[v + 10][v + 4] = 0.375; B1[v + 10][v + 5] = 0.125;
  B1[v + 11][v - 1] = 0.125; B1[v + 11][v] = 0.375; B1[v + 11][v + 4] = 0.125; B1[v + 11][v + 5] = 0.375;
  /* B3 = B2 * B1 where B2 picks 12 rows of B1 (one 1.0 per row) */
  const int pick[12] = {v + 9, v + 6, v + 4, v + 1, v + 2, v + 5, v, 1, v + 3, v - 1, 0, 2};
  for (int j = 0; j < nen; j++) {
    double s1 = 0., s2 = 0., s3 = 0., s4 = 0., s5 = 0.;
    for (int i = 0; i < 12; i++) {
      /* (B2 B1)[i][j] summed over m < v+12: exactly B1[pick[i]][j] */
      double b3 = 0.0;
      for (int mm = 0; mm < v + 12; mm++) b3 = b3 + ((mm == pick[i]) ? 1.0 : 0.0) * B1[mm][j];
      s1 = s1 + b3 * kNa[0][i]; s2 = s2 + b3 * kNa[1][i];
      s3 = s3 + b3 * kNab[0][i]; s4 = s4 + b3 * kNab[1][i]; s5 = s5 + b3 * kNab[2][i];
    }
    INa0[j] = -2.0 * s1; INa1[j] = -2.0 * s2;
    INab0[j] = 4.0 * s3; INab1[j] = 4.0 * s4; INab2[j] = 4.0 * s5;
  }
  return 0;
}

/* ElemUpdateGeomSubdivFromCoords_, active_strain.c:428-724 */
template <class T>
static int elem_geom(const Mesh &m, int ec, const T *xb, const T *yb, const T *zb, Geom<T> &G)
{
  const int *pt = &m.patch[16 * ec];
  if (is_cap(m, ec)) {   /* flat triangle, active_strain.c:448-470 */
    const int n1 = m.nv1[ec], n2 = m.nv2[ec], n3 = m.nv3[ec];
    G.a1 = {xb[n2] - xb[n1], yb[n2] - yb[n1], zb[n2] - zb[n1]};
    G.a2 = {xb[n3] - xb[n1], yb[n3] - yb[n1], zb[n3] - zb[n1]};
    G.Aaa = {0.0, 0.0, 0.0}; G.Abb = {0.0, 0.0, 0.0}; G.Aab = {0.0, 0.0, 0.0};
    G.nen = 12;
  } else if (m.ire[ec] == 0) {
    T x[12], y[12], z[12];
    for (int i = 0; i < 12; i++) {
      if (pt[i] == kMissing) return 77;
      x[i] = xb[pt[i]]; y[i] = yb[pt[i]]; z[i] = zb[pt[i]];
    }
    G.Aaa = {0.0, 0.0, 0.0}; G.Abb = {0.0, 0.0, 0.0}; G.Aab = {0.0, 0.0, 0.0};
    for (int i = 0; i < 12; i++) {
      G.Aaa.x = G.Aaa.x + kNab[0][i] * x[i]; G.Aaa.y = G.Aaa.y + kNab[0][i] * y[i]; G.Aaa.z = G.Aaa.z + kNab[0][i] * z[i];
      G.Abb.x = G.Abb.x + kNab[1][i] * x[i]; G.Abb.y = G.Abb.y + kNab[1][i] * y[i]; G.Abb.z = G.Abb.z + kNab[1][i] * z[i];
      G.Aab.x = G.Aab.x + kNab[2][i] * x[i]; G.Aab.y = G.Aab.y + kNab[2][i] * y[i]; G.Aab.z = G.Aab.z + kNab[2][i] * z[i];
    }
    G.a1 = {0.0, 0.0, 0.0}; G.a2 = {0.0, 0.0, 0.0};
    for (int i = 0; i < 12; i++) {
      G.a1.x = G.a1.x + kNa[0][i] * x[i]; G.a1.y = G.a1.y + kNa[0][i] * y[i]; G.a1.z = G.a1.z + kNa[0][i] * z[i];
      G.a2.x = G.a2.x + kNa[1][i] * x[i]; G.a2.y = G.a2.y + kNa[1][i] * y[i]; G.a2.z = G.a2.z + kNa[1][i] * z[i];
    }
    G.nen = 12;
  } else {
    const int v = m.val[ec], nen = v + 6;
    for (int i = 0; i < nen; i++) if (pt[i] == kMissing) return 77;
    int rc = irregular_weights(v, G.INa0, G.INa1, G.INab0, G.INab1, G.INab2);
    if (rc) return rc;
    G.Aaa = {0.0, 0.0, 0.0}; G.Abb = {0.0, 0.0, 0.0}; G.Aab = {0.0, 0.0, 0.0};
    for (int i = 0; i < nen; i++) {
      const T X = xb[pt[i]], Y = yb[pt[i]], Z = zb[pt[i]];
      G.Aaa.x = G.Aaa.x + G.INab0[i] * X; G.Aaa.y = G.Aaa.y + G.INab0[i] * Y; G.Aaa.z = G.Aaa.z + G.INab0[i] * Z;
      G.Abb.x = G.Abb.x + G.INab1[i] * X; G.Abb.y = G.Abb.y + G.INab1[i] * Y; G.Abb.z = G.Abb.z + G.INab1[i] * Z;
      G.Aab.x = G.Aab.x + G.INab2[i] * X; G.Aab.y = G.Aab.y + G.INab2[i] * Y; G.Aab.z = G.Aab.z + G.INab2[i] * Z;
    }
    G.a1 = {0.0, 0.0, 0.0}; G.a2 = {0.0, 0.0, 0.0};
    for (int i = 0; i < nen; i++) {
      const T X = xb[pt[i]], Y = yb[pt[i]], Z = zb[pt[i]];
      G.a1.x = G.a1.x + G.INa0[i] * X; G.a1.y = G.a1.y + G.INa0[i] * Y; G.a1.z = G.a1.z + G.INa0[i] * Z;
      G.a2.x = G.a2.x + G.INa1[i] * X; G.a2.y = G.a2.y + G.INa1[i] * Y; G.a2.z = G.a2.z + G.INa1[i] * Z;
    }
    G.nen = nen;
  }
  G.n = UNIT(CROSS(G.a1, G.a2));
  G.gc1 = CROSS(G.a2, G.n);
  G.gc1 = AMULT(1.0 / DOT(G.a1, G.gc1), G.gc1);
  G.gc2 = CROSS(G.n, G.a1);
  G.gc2 = AMULT(1.0 / DOT(G.a2, G.gc2), G.gc2);
  return 0;
}

/* 1: the thickness metric uses the tangential part of a3,alpha (n,alpha), an
   extension; 0: the reference's unnormalised derivative.  Set by
   oracle_set_thickness_normal before oracle_setup. */
static int g_tnormal = 0;

/* Compute_a3_alpha_, active_strain.c:745-762 */
template <class T>
static void a3_alpha(const Geom<T> &G, V3<T> &a31, V3<T> &a32)
{
  T s = SIZE(CROSS(G.a1, G.a2));
  a31 = PLUS(CROSS(G.Aaa, G.a2), CROSS(G.a1, G.Aab));
  a32 = PLUS(CROSS(G.Aab, G.a2), CROSS(G.a1, G.Abb));
  a31.x /= s; a31.y /= s; a31.z /= s;
  a32.x /= s; a32.y /= s; a32.z /= s;
  if (g_tnormal) {
    const T d1 = DOT(a31, G.n), d2 = DOT(a32, G.n);
    a31 = MINUS(a31, AMULT(d1, G.n));
    a32 = MINUS(a32, AMULT(d2, G.n));
  }
}

template <class T> inline void metric(const V3<T> g[3], T gm[3][3])
{
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) gm[i][j] = DOT(g[i], g[j]);
}

/* Reference-side state of one element (depends only on X, fibre, gamma). */
struct RefElem {
  Geom<double> geom0;
  double G0cov[kMaxQp][3][3], G0con[kMaxQp][3][3];
  double FaCon[kMaxQp][3][3], FaiCov[kMaxQp][3][3];
};

/* geom0 + the reference half of ElemUpdateG (active_strain.c:896-982) +
   ElemActDefGrad (active_strain.c:1196-1329, cart_fib_act = 1, constant gamma). */
static int ref_elem(const Mesh &m, const Params &P, int ec, RefElem &R)
{
  int rc = elem_geom<double>(m, ec, m.x0.data(), m.y0.data(), m.z0.data(), R.geom0);
  if (rc) return rc;
  V3<double> a31, a32;
  a3_alpha(R.geom0, a31, a32);
  const double hhalf = 0.5 * P.h0;
  const double gam = P.gamma * m.gscale[ec];
  const double nf[3] = {m.fib[3 * ec], m.fib[3 * ec + 1], m.fib[3 * ec + 2]};
  double Fc[3][3], Fic[3][3], S[3][3], ST[3][3], tmp[3][3], FaCov[3][3];
  if (!P.iso_act) {   /* cart_fib_act = 1: I - gamma f f^T */
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) Fc[i][j] = (i == j ? 1.0 : 0.0) - gam * nf[i] * nf[j];
  } else {            /* cart_fib_act = 0: diag(1 - gamma, 1 - gamma, 1 / ((1 - gamma)^2)) */
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) Fc[i][j] = 0.0;
    Fc[0][0] = 1.0 - gam;
    Fc[1][1] = 1.0 - gam;
    Fc[2][2] = 1.0 / (Fc[0][0] * Fc[1][1]);
  }
  for (int q = 0; q < P.n_qp; q++) {
    const double th3 = hhalf * P.theta[q];
    V3<double> g0[3];
    g0[0] = PLUS(R.geom0.a1, AMULT(th3, a31));
    g0[1] = PLUS(R.geom0.a2, AMULT(th3, a32));
    g0[2] = R.geom0.n;
    metric(g0, R.G0cov[q]);
    INV(R.G0cov[q], R.G0con[q]);
    for (int j = 0; j < 3; j++) { S[0][j] = g0[j].x; S[1][j] = g0[j].y; S[2][j] = g0[j].z; }
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) ST[i][j] = S[j][i];
    MATMULT(ST, Fc, tmp);
    MATMULT(tmp, S, FaCov);
    INV(Fc, Fic);
    MATMULT(ST, Fic, tmp);
    MATMULT(tmp, S, R.FaiCov[q]);
    RaiseIndices2(R.G0con[q], FaCov, R.FaCon[q]);
  }
  return 0;
}

/* Current-configuration element pipeline for one element:
   ElemUpdateG (current half) -> ElemCGDefTens -> ElemC33Solve -> ElemUpdFint.
   Fb has 3*nen entries (zeroed here). */
template <class T>
static int elem_forces(const Mesh &m, const Params &P, int ec, const RefElem &R,
                       const T *xb, const T *yb, const T *zb, T *Fb,
                       T Sout[kMaxQp][3][3] = nullptr, T C33out[kMaxQp] = nullptr, Geom<T> *Gout = nullptr)
{
  Geom<T> G;
  int rc = elem_geom<T>(m, ec, xb, yb, zb, G);
  if (rc) return rc;
  if (Gout) *Gout = G;
  V3<T> a31, a32;
  a3_alpha(G, a31, a32);
  const double hhalf = 0.5 * P.h0;
  const int nq = P.n_qp;

  T gmCov[kMaxQp][3][3], gmCon[kMaxQp][3][3];
  T Ccov[kMaxQp][3][3], Cinv[kMaxQp][3][3];
  T S[kMaxQp][3][3];
  for (int q = 0; q < nq; q++) {
    const double th3 = hhalf * P.theta[q];
    V3<T> g[3];
    g[0] = PLUS(G.a1, AMULT(th3, a31));
    g[1] = PLUS(G.a2, AMULT(th3, a32));
    g[2] = G.n;
    metric(g, gmCov[q]);
    INV(gmCov[q], gmCon[q]);
    /* ElemCGDefTens, active_strain.c:1332-1378 (C.Cont / C_inv.Cov unused downstream) */
    for (int i = 0; i < 2; i++) for (int j = 0; j < 2; j++) { Ccov[q][i][j] = gmCov[q][i][j]; Cinv[q][i][j] = gmCon[q][i][j]; }
    for (int a = 0; a < 2; a++) { Ccov[q][a][2] = 0.0; Ccov[q][2][a] = 0.0; Cinv[q][a][2] = 0.0; Cinv[q][2][a] = 0.0; }
    Ccov[q][2][2] = 1.0; Cinv[q][2][2] = 1.0;
  }

  /* ElemC33Solve, active_strain.c:2048-2138 */
  for (int it = 0; it < P.c33_iters; it++) {
    for (int q = 0; q < nq; q++) {
      const double (*G0)[3] = R.G0cov[q];
      const double (*G0c)[3] = R.G0con[q];
      const double (*Fa)[3] = R.FaCon[q];
      const double (*Fi)[3] = R.FaiCov[q];
      /* ElemElasCGDefTens, :1381-1434 */
      T CeiCon[3][3], CeiCov[3][3], CeCon[3][3], CeCov[3][3];
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) CeiCon[i][j] = 0.0;
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
        for (int mm = 0; mm < 3; mm++) for (int p = 0; p < 3; p++) for (int qq = 0; qq < 3; qq++) for (int l = 0; l < 3; l++)
          CeiCon[i][j] = CeiCon[i][j] + Fa[i][mm] * G0[mm][p] * Cinv[q][p][qq] * Fa[l][j] * G0[l][qq];
      RaiseIndices2(G0, CeiCon, CeiCov);   /* LowerIndices2 == the same two products with gm0.Cov */
      INV(CeiCov, CeCon);
      RaiseIndices2(G0, CeCon, CeCov);
      /* ElemElasStress, :1437-1491 */
      T detCe = DET3x3(CeCov);
      double detG0 = DET3x3(G0);
      T Je = sqrt(detCe / detG0);
      T Se[3][3];
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
        T t1 = P.mu * (G0c[i][j] - CeiCon[i][j]);
        T t2 = P.K * CeiCon[i][j] * (Je * Je - Je);
        Se[i][j] = t1 + t2;
      }
      /* ElemTotStress, :1494-1532 */
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) S[q][i][j] = 0.0;
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
        for (int w = 0; w < 3; w++) for (int p = 0; p < 3; p++) for (int z = 0; z < 3; z++) for (int s = 0; s < 3; s++)
          S[q][i][j] = S[q][i][j] + 0.5 * Fi[w][p] * Fi[z][s] * G0c[s][j] * (Se[p][z] * G0c[w][i] + Se[p][i] * G0c[w][z]);
      /* ElemElsTangMatTens, :1535-1589 */
      T Je2 = Je * Je;
      T alpha = P.K * (Je2 - Je) - P.mu;
      T beta = 0.5 * P.K * Je * (2.0 * Je - 1.0);
      static thread_local T CCe[3][3][3][3];
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++)
        CCe[i][j][k][l] = (2.0 * beta) * CeiCon[i][j] * CeiCon[k][l] - alpha * (CeiCon[i][k] * CeiCon[l][j] + CeiCon[i][l] * CeiCon[k][j]);
      /* ElemTotTangMatTens, :1592-1651 (only CC3333 is filled) */
      T CC = 0.0;
      {
        const int i = 2, j = 2, k = 2, l = 2;
        for (int g = 0; g < 3; g++) for (int h = 0; h < 3; h++) for (int mm = 0; mm < 3; mm++) for (int n = 0; n < 3; n++)
          for (int p = 0; p < 3; p++) for (int s = 0; s < 3; s++) for (int w = 0; w < 3; w++) for (int z = 0; z < 3; z++)
            CC = CC + 0.25 * Fi[w][p] * Fi[z][s] * Fi[g][h] * Fi[n][mm] * G0c[s][j] * G0c[mm][l]
                      * (G0c[g][k] * (CCe[h][n][p][z] * G0c[w][i] + CCe[h][n][p][i] * G0c[w][z])
                         + G0c[g][n] * (CCe[h][k][p][z] * G0c[w][i] + CCe[h][k][p][i] * G0c[w][z]));
      }
      /* ModElemC33, :1654-1707 */
      T S33 = S[q][2][2];
      if (!(std::fabs(val(CC)) > 1e-14)) return 72;   /* PETSC_ERR_FP */
      T dC = -1.0 * S33 / CC;
      {
        T old = Ccov[q][2][2];
        Ccov[q][2][2] = old + dC;
        if (val(DET3x3(Ccov[q])) <= 0.0) {
          double lo = 0.0, hi = 1.0;
          for (int bk = 0; bk < 16; bk++) {
            double mid = 0.5 * (lo + hi);
            Ccov[q][2][2] = old + mid * dC;
            if (val(DET3x3(Ccov[q])) > 0.0) lo = mid; else hi = mid;
          }
          dC = dC * lo;
          Ccov[q][2][2] = old + dC;
        }
      }
    }
    /* raise/INV/lower after the update, :2095-2108 (only C_inv.Cont is used) */
    for (int q = 0; q < nq; q++) INV(Ccov[q], Cinv[q]);
  }

  if (Sout) for (int q = 0; q < nq; q++) for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) Sout[q][i][j] = S[q][i][j];
  if (C33out) for (int q = 0; q < nq; q++) C33out[q] = Ccov[q][2][2];

  /* ElemUpdFint, active_strain.c:1762-1995 */
  const double A0 = m.dA0[ec];
  const double half_h0 = 0.5 * P.h0;
  const double pref0 = 0.5 * P.h0 * A0;
  const int nen = G.nen;
  for (int i = 0; i < 3 * nen; i++) Fb[i] = 0.0;
  if (is_cap(m, ec)) {
    /* constant-strain membrane force into the patch slots of the corners,
       active_strain.c:1807-1853 */
    const int tri_nodes[3] = {m.nv1[ec], m.nv2[ec], m.nv3[ec]};
    const double dN[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
    int tri_slot[3] = {-1, -1, -1};
    const int nslot = m.val[ec] + 6;
    for (int a = 0; a < 3; a++) {
      for (int i = 0; i < nslot && i < 16; i++)
        if (m.patch[16 * ec + i] == tri_nodes[a]) { tri_slot[a] = i; break; }
      if (tri_slot[a] < 0) return 62;
    }
    const V3<T> d21 = G.a1, d31 = G.a2;
    for (int q = 0; q < nq; q++) {
      const double wq = P.w[q];
      const T Sv[3] = {S[q][0][0], S[q][1][1], S[q][0][1]};
      for (int a = 0; a < 3; a++) {
        const int base = 3 * tri_slot[a];
        const double Na0 = dN[a][0], Na1 = dN[a][1];
        const T Bm0x = Na0 * d21.x, Bm0y = Na0 * d21.y, Bm0z = Na0 * d21.z;
        const T Bm1x = Na1 * d31.x, Bm1y = Na1 * d31.y, Bm1z = Na1 * d31.z;
        const T Bm2x = Na0 * d31.x + Na1 * d21.x;
        const T Bm2y = Na0 * d31.y + Na1 * d21.y;
        const T Bm2z = Na0 * d31.z + Na1 * d21.z;
        Fb[base + 0] = Fb[base + 0] + pref0 * wq * (Bm0x * Sv[0] + Bm1x * Sv[1] + Bm2x * Sv[2]);
        Fb[base + 1] = Fb[base + 1] + pref0 * wq * (Bm0y * Sv[0] + Bm1y * Sv[1] + Bm2y * Sv[2]);
        Fb[base + 2] = Fb[base + 2] + pref0 * wq * (Bm0z * Sv[0] + Bm1z * Sv[1] + Bm2z * Sv[2]);
      }
    }
    return 0;
  }
  const bool reg = (m.ire[ec] == 0);
  for (int q = 0; q < nq; q++) {
    const double wq = P.w[q], xi = P.theta[q];
    T Sv[3] = {S[q][0][0], S[q][1][1], S[q][0][1]};
    for (int a = 0; a < nen; a++) {
      const double na0 = reg ? kNa[0][a] : G.INa0[a];
      const double na1 = reg ? kNa[1][a] : G.INa1[a];
      const double nb0 = reg ? kNab[0][a] : G.INab0[a];
      const double nb1 = reg ? kNab[1][a] : G.INab1[a];
      const double nb2 = reg ? kNab[2][a] : G.INab2[a];
      const V3<T> ng = PLUS(AMULT(na0, G.gc1), AMULT(na1, G.gc2));
      const T b1 = DOT(ng, G.Aaa), b2 = DOT(ng, G.Abb), b3 = DOT(ng, G.Aab);
      const T Bs0 = -(nb0 + b1), Bs1 = -(nb1 + b2), Bs2 = -2.0 * (nb2 + b3);
      const T a1c[3] = {G.a1.x, G.a1.y, G.a1.z}, a2c[3] = {G.a2.x, G.a2.y, G.a2.z}, nc[3] = {G.n.x, G.n.y, G.n.z};
      for (int d = 0; d < 3; d++) {
        T Bm0 = na0 * a1c[d], Bm1 = na1 * a2c[d], Bm2 = na0 * a2c[d] + na1 * a1c[d];
        T mem, bend;
        if (reg) {
          mem = 0.0; mem = mem + Bm0 * Sv[0]; mem = mem + Bm1 * Sv[1]; mem = mem + Bm2 * Sv[2];
          bend = 0.0; bend = bend + (Bs0 * nc[d]) * Sv[0]; bend = bend + (Bs1 * nc[d]) * Sv[1]; bend = bend + (Bs2 * nc[d]) * Sv[2];
        } else {
          mem = Bm0 * Sv[0] + Bm1 * Sv[1] + Bm2 * Sv[2];
          bend = (Bs0 * nc[d]) * Sv[0] + (Bs1 * nc[d]) * Sv[1] + (Bs2 * nc[d]) * Sv[2];
        }
        Fb[3 * a + d] = Fb[3 * a + d] + pref0 * wq * (mem + bend * (half_h0 * xi));
      }
    }
  }
  return 0;
}

/* ---------------- whole-residual restatement ---------------- */
/* Time integration state of FDynamic / xAccVel (main.c:1157-1412).
   Newmark's Beta is tied to Gama, Beta = (Gama + 1/2)^2 / 4 (main.c:1171). */
struct Dyn {
  bool on = false;
  int central = 0, damp = 0;
  double dt = 0, rhoh0 = 0, dampf = 0;
  double M1 = 0, M2 = 0, M3 = 0, C1 = 0, C2 = 0, C3 = 0, U2 = 0, U3 = 0;
  std::vector<double> dA0;                 /* flat reference area of every triangle (real ones used) */
  std::vector<double> xn, xnm1, xd, xdd;   /* 3 (n_v + n_ghosts) */
};

struct Body {
  Mesh m;
  Params P;
  std::vector<RefElem> ref;
  Dyn D;
  bool ready = false;
};

/* AreaNormal (io.c:1646-1669) for the real elements only: the residual reads
   dA/nf of ec < n_elmt (SurfaceNormalPressure, external.c:589-624). */
template <class T>
static void area_normal(const Mesh &m, const T *x, const T *y, const T *z, int ec, T &dA, V3<T> &nf)
{
  const int a = m.nv1[ec], b = m.nv2[ec], c = m.nv3[ec];
  V3<T> x1 = {x[a], y[a], z[a]}, x2 = {x[b], y[b], z[b]}, x3 = {x[c], y[c], z[c]};
  V3<T> cr = CROSS(MINUS(x2, x1), MINUS(x3, x1));
  nf = UNIT(cr);
  dA = 0.5 * SIZE(cr);
}

/* GlobalGhost (bending.c:1763-1814): ghost = x[nv2] + x[nv1] - x[nv3]. */
template <class T>
static void global_ghost(const Mesh &m, T *x, T *y, T *z)
{
  int count = 0;
  for (int edge_n = 0; edge_n < m.n_edge; edge_n++) {
    int end = 0;
    for (int e = 0; e < edge_n + 1; e++) end += m.n_bnodes[e];
    const int start = end - m.n_bnodes[edge_n], n_local = end - start;
    for (int li = 0; li < n_local; li++) {
      const int nv1 = m.bnodes[start + (li + 1) % n_local], nv2 = m.bnodes[start + li];
      const int nv3 = m.ghost_nv3[count];
      const int g = m.n_v + count;
      x[g] = x[nv2] + x[nv1] - x[nv3];
      y[g] = y[nv2] + y[nv1] - y[nv3];
      z[g] = z[nv2] + z[nv1] - z[nv3];
      count++;
    }
  }
}

static int g_threads = 1;

/* FormFunctionFEM at np = 1, main.c:757-1032 (see oracle/ref_driver.c for the
   load and BC choices).  x and R have 3 (n_v + n_ghosts) entries. */
template <class T>
static int residual(const Body &B, const T *x, T *R, T *Fint_out = nullptr, T *Fext_out = nullptr,
                    T *Fdyn_out = nullptr)
{
  const Mesh &m = B.m;
  const int ntot = m.n_v + m.n_ghosts, ndof = 3 * ntot;
  std::vector<T> xb(ntot), yb(ntot), zb(ntot);
  for (int v = 0; v < m.n_v; v++) { xb[v] = x[3 * v]; yb[v] = x[3 * v + 1]; zb[v] = x[3 * v + 2]; }
  for (int v = m.n_v; v < ntot; v++) { xb[v] = m.x0[v]; yb[v] = m.y0[v]; zb[v] = m.z0[v]; }
  global_ghost(m, xb.data(), yb.data(), zb.data());

  std::vector<T> Fint(ndof, T(0.0)), Fext(ndof, T(0.0));
  /* FInternalAct, active_strain.c:2226-2267: element loop, then scatter in
     element order (ghost and sentinel slots dropped). */
  std::vector<T> Fb((size_t)m.n_elmt * 48);
  std::vector<int> rcs(m.n_elmt, 0);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(g_threads) if (g_threads > 1)
#endif
  for (int ec = 0; ec < m.n_elmt; ec++)
    rcs[ec] = elem_forces<T>(m, B.P, ec, B.ref[ec], xb.data(), yb.data(), zb.data(), &Fb[(size_t)ec * 48]);
  for (int ec = 0; ec < m.n_elmt; ec++) if (rcs[ec]) return rcs[ec];
  for (int ec = 0; ec < m.n_elmt; ec++) {
    const int nen = (m.ire[ec] == 0) ? 12 : m.val[ec] + 6;
    for (int i = 0; i < nen; i++) {
      const int node = m.patch[16 * ec + i];
      if (node == kMissing || node < 0 || node >= m.n_v) continue;
      for (int d = 0; d < 3; d++) Fint[3 * node + d] = Fint[3 * node + d] + Fb[(size_t)ec * 48 + 3 * i + d];
    }
  }
  /* SurfaceNormalPressure(P), external.c:589-624: current normal and area;
     SurfaceConstNormalPressure(P), external.c:699-730: the reference normal
     Nf and area dA0 of Init (AreaNormal on the reference coordinates) */
  if (B.P.pressure != 0.0) {
    const double Pp = B.P.pressure;
    for (int ec = 0; ec < m.n_elmt; ec++) {
      T dA; V3<T> n;
      if (B.P.dead_load) {
        double dA0; V3<double> N;
        area_normal(m, m.x0.data(), m.y0.data(), m.z0.data(), ec, dA0, N);
        dA = T(dA0); n = {T(N.x), T(N.y), T(N.z)};
      } else {
        area_normal(m, xb.data(), yb.data(), zb.data(), ec, dA, n);
      }
      const int c[3] = {m.nv1[ec], m.nv2[ec], m.nv3[ec]};
      for (int k = 0; k < 3; k++) {
        Fext[3 * c[k]] = Fext[3 * c[k]] + n.x * Pp * dA / 3.;
        Fext[3 * c[k] + 1] = Fext[3 * c[k] + 1] + n.y * Pp * dA / 3.;
        Fext[3 * c[k] + 2] = Fext[3 * c[k] + 2] + n.z * Pp * dA / 3.;
      }
    }
  }
  /* FDynamic, main.c:1157-1270 (the path of an active-strain run, whose
     DMPlex context is initialised, main.c:326-331): every real triangle, in
     triangle order, adds M (M1 x - ...) per corner, M = rho h0 dA0 / 3 (Mass,
     material.c:100-119) and C = dampfactor M (Damp, material.c:122-137). */
  std::vector<T> Fdyn(ndof, T(0.0));
  if (B.D.on) {
    const Dyn &D = B.D;
    const T *xc[3] = {xb.data(), yb.data(), zb.data()};
    for (int ec = 0; ec < m.n_elmt; ec++) {
      const double M = D.rhoh0 * D.dA0[ec] / 3;
      const double C = D.damp ? D.dampf * M : 0.0;
      const int c[3] = {m.nv1[ec], m.nv2[ec], m.nv3[ec]};
      for (int k = 0; k < 3; k++)
        for (int d = 0; d < 3; d++) {
          const int o = 3 * c[k] + d;
          const T xv = xc[d][c[k]];
          T f;
          if (!D.central) {
            const double facc = M * (D.M1 * D.xn[o] + D.M2 * D.xd[o] + D.M3 * D.xdd[o]);
            const double fvel = C * (D.C1 * D.xn[o] + D.C2 * D.xd[o] + D.C3 * D.xdd[o]);
            f = M * D.M1 * xv + C * D.C1 * xv - facc - fvel;
          } else {
            f = M * (xv - 2 * D.xn[o] + D.xnm1[o]) / (D.dt * D.dt) + C * (xv - D.xn[o]) / D.dt;
          }
          Fdyn[o] = Fdyn[o] + f;
        }
    }
  }
  /* R = -1*Fext + Fint + 1*Fdyn, main.c:844-845 */
  for (int i = 0; i < ndof; i++) R[i] = (-1. * Fext[i] + Fint[i]) + 1. * Fdyn[i];
  /* EdgeDirectionalFix(0, d), external.c:1706-1741: R := x_bp - x_bp0 */
  if (B.P.clamp && m.n_edge > 0) {
    for (int nbc = 0; nbc < m.n_bnodes[0]; nbc++) {
      const int nb = m.bnodes[nbc];
      R[3 * nb] = xb[nb] - m.x0[nb];
      R[3 * nb + 1] = yb[nb] - m.y0[nb];
      R[3 * nb + 2] = zb[nb] - m.z0[nb];
    }
  }
  /* FEM_DMPlexGeomSyncGhostDOFs, dmplex_geom.c:991-1011 */
  for (int v = m.n_v; v < ntot; v++) { R[3 * v] = 0.0; R[3 * v + 1] = 0.0; R[3 * v + 2] = 0.0; }
  /* R *= 1/max(|Fext|_inf, 1), main.c:1020-1026 */
  double finf = 0.0;
  for (int i = 0; i < ndof; i++) finf = std::max(finf, std::fabs(val(Fext[i])));
  const double scale = 1.0 / std::max(finf, 1.0);
  for (int i = 0; i < ndof; i++) R[i] = R[i] * scale;
  if (Fint_out) for (int i = 0; i < ndof; i++) Fint_out[i] = Fint[i];
  if (Fext_out) for (int i = 0; i < ndof; i++) Fext_out[i] = Fext[i];
  if (Fdyn_out) for (int i = 0; i < ndof; i++) Fdyn_out[i] = Fdyn[i];
  return 0;
}

static Body *g_body = nullptr;

} /* namespace oracle */

using namespace oracle;

extern "C" {

/* Build a body from plain arrays (Input(), io.c:373-479, 0-based) and
   initialise it in the LV-loader order: GlobalGhostInit -> IrrVer -> Patch ->
   geom0 -> dA0 (bending.c, active_strain.c, main.c:1443-1452).
   build_topology = 0 takes patch/ire/val/irv/ghost triangles from the caller. */
int oracle_setup(int n_v, int n_elmt, const int *tri, const double *xyz0,
                 int n_edge, const int *n_bnodes, const int *bnodes,
                 const double *fib, const double *gamma_scale,
                 int n_qp, int c33_iters, double mu, double K, double h0,
                 double gamma, double pressure, int clamp_edge0)
{
  delete g_body;
  g_body = new Body();
  Body &B = *g_body;
  Mesh &m = B.m;
  Params &P = B.P;
  if (gauss_rule(n_qp, P.theta, P.w)) return 63;
  if (c33_iters < 1) return 62;
  P.n_qp = n_qp; P.c33_iters = c33_iters; P.mu = mu; P.K = K; P.h0 = h0;
  P.gamma = gamma; P.pressure = pressure; P.clamp = clamp_edge0;
  P.dead_load = g_dead_load; P.iso_act = g_iso_act;
  m.n_v = n_v; m.n_elmt = n_elmt; m.n_edge = n_edge;
  if (g_elmt_base < 0 || g_elmt_base > n_elmt) return 63;
  m.n_elmt_base = g_elmt_base;
  m.n_bnodes.assign(n_bnodes, n_bnodes + n_edge);
  int sum = 0;
  for (int e = 0; e < n_edge; e++) sum += n_bnodes[e];
  m.n_ghosts = sum;
  m.bnodes.assign(bnodes, bnodes + sum);
  const int ntri = n_elmt + 2 * sum, ntot = n_v + sum;
  m.nv1.assign(ntri, 0); m.nv2.assign(ntri, 0); m.nv3.assign(ntri, 0);
  for (int ec = 0; ec < n_elmt; ec++) { m.nv1[ec] = tri[3 * ec]; m.nv2[ec] = tri[3 * ec + 1]; m.nv3[ec] = tri[3 * ec + 2]; }
  m.x0.assign(ntot, 0.0); m.y0.assign(ntot, 0.0); m.z0.assign(ntot, 0.0);
  for (int v = 0; v < n_v; v++) { m.x0[v] = xyz0[3 * v]; m.y0[v] = xyz0[3 * v + 1]; m.z0[v] = xyz0[3 * v + 2]; }
  m.fib.assign(fib, fib + 3 * n_elmt);
  m.gscale.assign(gamma_scale, gamma_scale + n_elmt);
  m.ire.assign(n_elmt, 0); m.irv.assign(n_elmt, 0); m.val.assign(n_elmt, 6); m.patch.assign(16 * n_elmt, kMissing);
  std::vector<double> x = m.x0, y = m.y0, z = m.z0;
  global_ghost_init(m, x, y, z);
  irrver(m);
  patch_build(m);
  m.dA0.assign(n_elmt, 0.0);
  for (int ec = 0; ec < n_elmt; ec++) {
    double dA; V3<double> n;
    area_normal(m, m.x0.data(), m.y0.data(), m.z0.data(), ec, dA, n);
    m.dA0[ec] = dA;
  }
  B.ref.resize(n_elmt);
  for (int ec = 0; ec < n_elmt; ec++) {
    int rc = ref_elem(m, P, ec, B.ref[ec]);
    if (rc) return rc;
  }
  B.ready = true;
  return 0;
}

/* Same as oracle_setup but with the subdivision topology supplied by the
   caller (patch/ire/val/irv, the ghost triangles and the reflected interior
   node of every ghost): skips the O(N^2) GlobalGhostInit/IrrVer/Patch
   searches for large meshes.  Tables must equal the reference's (the
   product's O(N) builder is checked bitwise against them). */
int oracle_setup_given_topology(int n_v, int n_elmt, const int *tri_all, const double *xyz0_full,
                                int n_edge, const int *n_bnodes, const int *bnodes,
                                const int *patch16, const int *ire, const int *val, const int *irv,
                                const int *ghost_nv3, const double *fib, const double *gamma_scale,
                                int n_qp, int c33_iters, double mu, double K, double h0,
                                double gamma, double pressure, int clamp_edge0)
{
  delete g_body;
  g_body = new Body();
  Body &B = *g_body;
  Mesh &m = B.m;
  Params &P = B.P;
  if (gauss_rule(n_qp, P.theta, P.w)) return 63;
  if (c33_iters < 1) return 62;
  P.n_qp = n_qp; P.c33_iters = c33_iters; P.mu = mu; P.K = K; P.h0 = h0;
  P.gamma = gamma; P.pressure = pressure; P.clamp = clamp_edge0;
  P.dead_load = g_dead_load; P.iso_act = g_iso_act;
  m.n_v = n_v; m.n_elmt = n_elmt; m.n_edge = n_edge;
  if (g_elmt_base < 0 || g_elmt_base > n_elmt) return 63;
  m.n_elmt_base = g_elmt_base;
  m.n_bnodes.assign(n_bnodes, n_bnodes + n_edge);
  int sum = 0;
  for (int e = 0; e < n_edge; e++) sum += n_bnodes[e];
  m.n_ghosts = sum;
  m.bnodes.assign(bnodes, bnodes + sum);
  const int ntri = n_elmt + 2 * sum, ntot = n_v + sum;
  m.nv1.resize(ntri); m.nv2.resize(ntri); m.nv3.resize(ntri);
  for (int t = 0; t < ntri; t++) { m.nv1[t] = tri_all[3 * t]; m.nv2[t] = tri_all[3 * t + 1]; m.nv3[t] = tri_all[3 * t + 2]; }
  m.x0.resize(ntot); m.y0.resize(ntot); m.z0.resize(ntot);
  for (int v = 0; v < ntot; v++) { m.x0[v] = xyz0_full[3 * v]; m.y0[v] = xyz0_full[3 * v + 1]; m.z0[v] = xyz0_full[3 * v + 2]; }
  m.fib.assign(fib, fib + 3 * n_elmt);
  m.gscale.assign(gamma_scale, gamma_scale + n_elmt);
  m.ire.assign(ire, ire + n_elmt); m.val.assign(val, val + n_elmt); m.irv.assign(irv, irv + n_elmt);
  m.patch.assign(patch16, patch16 + 16 * n_elmt);
  m.ghost_nv3.assign(ghost_nv3, ghost_nv3 + sum);
  m.dA0.assign(n_elmt, 0.0);
  for (int ec = 0; ec < n_elmt; ec++) {
    double dA; V3<double> n;
    area_normal(m, m.x0.data(), m.y0.data(), m.z0.data(), ec, dA, n);
    m.dA0[ec] = dA;
  }
  B.ref.resize(n_elmt);
  for (int ec = 0; ec < n_elmt; ec++) {
    int rc = ref_elem(m, P, ec, B.ref[ec]);
    if (rc) return rc;
  }
  B.ready = true;
  return 0;
}

int oracle_set_threads(int n) { g_threads = n > 0 ? n : 1; return 0; }

/* ibm->n_elmt_base of the next setup: 0 (every element a subdivision
   element) or the count of base elements, the rest being apex-cap
   triangles. */
int oracle_set_elmt_base(int n_elmt_base) { g_elmt_base = n_elmt_base; return 0; }

/* 1: oracle_setup builds the topology with the corner-incident scans (O(N),
   same tables); 0: with the reference's full scans (O(N_e^2)). */
int oracle_set_fast_topology(int on) { g_fast_topology = on != 0; return 0; }

/* Options of the next setup: dead_load 1 takes SurfaceConstNormalPressure
   (external.c:699-730) for the pressure, iso_act 1 the isotropic active
   gradient of -cart_fib_act 0 (active_strain.c:1238-1255). */
int oracle_set_load_options(int dead_load, int iso_act)
{
  g_dead_load = dead_load != 0;
  g_iso_act = iso_act != 0;
  return 0;
}

/* Switch the dynamic term on (dt > 0) or off (dt <= 0): the -dt, -rho,
   -newmark_gamma, -dampfactor, -timeinteg, -damping options of main.c.
   The state starts at xn = xnm1 = the reference coordinates, xd = xdd = 0. */
int oracle_set_dynamics(double dt, double rho, double newmark_gamma, double dampfactor, int timeinteg, int damping)
{
  if (!g_body || !g_body->ready) return 58;
  Body &B = *g_body;
  const Mesh &m = B.m;
  Dyn &D = B.D;
  if (!(dt > 0.0)) { D = Dyn(); return 0; }
  if (timeinteg != 0 && timeinteg != 1) return 66;
  const double G = newmark_gamma, Be = 0.25 * (G + 0.5) * (G + 0.5);
  D.on = true; D.central = timeinteg; D.damp = damping != 0;
  D.dt = dt; D.rhoh0 = rho * B.P.h0; D.dampf = dampfactor;
  /* FDynamic's constants (main.c:1175-1176) and xAccVel's velocity update
     weights (main.c:1383-1385) */
  D.M1 = 1. / (Be * pow(dt, 2)); D.M2 = 1. / (Be * dt); D.M3 = (1. / (2 * Be)) - 1.;
  D.C1 = G / (Be * dt); D.C2 = (G / Be) - 1; D.C3 = dt * (G / (2. * Be) - 1);
  D.U2 = (1. - G) * dt; D.U3 = G * dt;
  const int ntri = m.n_elmt + 2 * m.n_ghosts, ntot = m.n_v + m.n_ghosts;
  D.dA0.assign(ntri, 0.0);
  for (int ec = 0; ec < ntri; ec++) {
    double dA; V3<double> n;
    area_normal(m, m.x0.data(), m.y0.data(), m.z0.data(), ec, dA, n);
    D.dA0[ec] = dA;
  }
  D.xn.assign(3 * (size_t)ntot, 0.0);
  for (int v = 0; v < ntot; v++) { D.xn[3 * v] = m.x0[v]; D.xn[3 * v + 1] = m.y0[v]; D.xn[3 * v + 2] = m.z0[v]; }
  D.xnm1 = D.xn;
  D.xd.assign(3 * (size_t)ntot, 0.0);
  D.xdd.assign(3 * (size_t)ntot, 0.0);
  return 0;
}

/* Any of the four may be null (left unchanged); each has 3 (n_v + n_ghosts) entries. */
int oracle_set_dynamic_state(const double *xn, const double *xnm1, const double *xd, const double *xdd)
{
  if (!g_body || !g_body->ready || !g_body->D.on) return 58;
  Dyn &D = g_body->D;
  const size_t n = D.xn.size();
  if (xn) std::copy(xn, xn + n, D.xn.begin());
  if (xnm1) std::copy(xnm1, xnm1 + n, D.xnm1.begin());
  if (xd) std::copy(xd, xd + n, D.xd.begin());
  if (xdd) std::copy(xdd, xdd + n, D.xdd.begin());
  return 0;
}

int oracle_get_dynamic_state(double *xn, double *xnm1, double *xd, double *xdd)
{
  if (!g_body || !g_body->ready || !g_body->D.on) return 58;
  const Dyn &D = g_body->D;
  std::copy(D.xn.begin(), D.xn.end(), xn);
  std::copy(D.xnm1.begin(), D.xnm1.end(), xnm1);
  std::copy(D.xd.begin(), D.xd.end(), xd);
  std::copy(D.xdd.begin(), D.xdd.end(), xdd);
  return 0;
}

/* xAccVel (main.c:1367-1412; with the DMPlex context over the n_v real
   nodes), then xnm1 <- xn, xn <- x over every entry (main.c:571-572). */
int oracle_dynamic_update(const double *x)
{
  if (!g_body || !g_body->ready || !g_body->D.on) return 58;
  Dyn &D = g_body->D;
  const size_t n = D.xn.size(), nreal = 3 * (size_t)g_body->m.n_v;
  for (size_t j = 0; j < nreal; j++) {
    const double xddn = D.xdd[j];
    D.xdd[j] = D.M1 * (x[j] - D.xn[j]) - D.M2 * D.xd[j] - D.M3 * D.xdd[j];
    D.xd[j] = D.xd[j] + D.U2 * xddn + D.U3 * D.xdd[j];
  }
  D.xnm1 = D.xn;
  std::copy(x, x + n, D.xn.begin());
  return 0;
}

/* Per-element activation gamma_e (ElemActDefGrad, active_strain.c:1207-1212:
   GammaOfTimeDelayed(delay_e) * gamma_scale_e), taken as given: the body's
   scalar gamma becomes 1 and gamma_scale the caller's values; the reference
   geometry per element is rebuilt. */
int oracle_set_element_gamma(const double *gamma_e)
{
  if (!g_body || !g_body->ready) return 58;
  Body &B = *g_body;
  B.P.gamma = 1.0;
  B.m.gscale.assign(gamma_e, gamma_e + B.m.n_elmt);
  for (int ec = 0; ec < B.m.n_elmt; ec++) {
    int rc = ref_elem(B.m, B.P, ec, B.ref[ec]);
    if (rc) return rc;
  }
  return 0;
}

int oracle_sizes(int *n_ghosts, int *n_dof)
{
  if (!g_body || !g_body->ready) return 58;
  *n_ghosts = g_body->m.n_ghosts;
  *n_dof = 3 * (g_body->m.n_v + g_body->m.n_ghosts);
  return 0;
}

int oracle_topology(int *patch16, int *ire, int *val, int *irv, int *gtri, double *xyz0_full, double *dA0, int *ghost_nv3)
{
  if (!g_body || !g_body->ready) return 58;
  const Mesh &m = g_body->m;
  std::copy(m.patch.begin(), m.patch.end(), patch16);
  std::copy(m.ire.begin(), m.ire.end(), ire);
  std::copy(m.val.begin(), m.val.end(), val);
  std::copy(m.irv.begin(), m.irv.end(), irv);
  for (int ec = 0; ec < m.n_elmt + 2 * m.n_ghosts; ec++) { gtri[3 * ec] = m.nv1[ec]; gtri[3 * ec + 1] = m.nv2[ec]; gtri[3 * ec + 2] = m.nv3[ec]; }
  for (int v = 0; v < m.n_v + m.n_ghosts; v++) { xyz0_full[3 * v] = m.x0[v]; xyz0_full[3 * v + 1] = m.y0[v]; xyz0_full[3 * v + 2] = m.z0[v]; }
  std::copy(m.dA0.begin(), m.dA0.end(), dA0);
  if (ghost_nv3) std::copy(m.ghost_nv3.begin(), m.ghost_nv3.end(), ghost_nv3);
  return 0;
}

int oracle_residual(const double *x, double *R, double *Fint, double *Fext)
{
  if (!g_body || !g_body->ready) return 58;
  return residual<double>(*g_body, x, R, Fint, Fext);
}

/* R and the unscaled Fint, Fext, Fdyn of main.c:829-845 */
int oracle_residual_parts(const double *x, double *R, double *Fint, double *Fext, double *Fdyn)
{
  if (!g_body || !g_body->ready) return 58;
  return residual<double>(*g_body, x, R, Fint, Fext, Fdyn);
}

/* Directional derivative J v of the residual (exact, forward mode). */
int oracle_jvp(const double *x, const double *v, double *R, double *Jv)
{
  if (!g_body || !g_body->ready) return 58;
  const int ndof = 3 * (g_body->m.n_v + g_body->m.n_ghosts);
  std::vector<Dual<1>> xd(ndof), Rd(ndof);
  for (int i = 0; i < ndof; i++) { xd[i].v = x[i]; xd[i].d[0] = v[i]; }
  int rc = residual<Dual<1>>(*g_body, xd.data(), Rd.data());
  if (rc) return rc;
  for (int i = 0; i < ndof; i++) { if (R) R[i] = Rd[i].v; Jv[i] = Rd[i].d[0]; }
  return 0;
}

/* J V for up to 8 directions V (8 x ndof, row major), JV the same layout. */
int oracle_jmv8(const double *x, const double *V, int nvec, double *JV)
{
  if (!g_body || !g_body->ready) return 58;
  if (nvec < 1 || nvec > 8) return 63;
  const int ndof = 3 * (g_body->m.n_v + g_body->m.n_ghosts);
  std::vector<Dual<8>> xd(ndof), Rd(ndof);
  for (int i = 0; i < ndof; i++) {
    xd[i] = Dual<8>(x[i]);
    for (int k = 0; k < nvec; k++) xd[i].d[k] = V[(size_t)k * ndof + i];
  }
  int rc = residual<Dual<8>>(*g_body, xd.data(), Rd.data());
  if (rc) return rc;
  for (int k = 0; k < nvec; k++)
    for (int i = 0; i < ndof; i++) JV[(size_t)k * ndof + i] = Rd[i].d[k];
  return 0;
}

/* Dense Jacobian (column major, ndof x ndof) for small meshes, 8 columns per pass. */
int oracle_jacobian_dense(const double *x, double *J)
{
  if (!g_body || !g_body->ready) return 58;
  const int ndof = 3 * (g_body->m.n_v + g_body->m.n_ghosts);
  std::vector<Dual<8>> xd(ndof), Rd(ndof);
  for (int c0 = 0; c0 < ndof; c0 += 8) {
    for (int i = 0; i < ndof; i++) { xd[i] = Dual<8>(x[i]); }
    for (int k = 0; k < 8 && c0 + k < ndof; k++) xd[c0 + k].d[k] = 1.0;
    int rc = residual<Dual<8>>(*g_body, xd.data(), Rd.data());
    if (rc) return rc;
    for (int k = 0; k < 8 && c0 + k < ndof; k++)
      for (int i = 0; i < ndof; i++) J[(size_t)(c0 + k) * ndof + i] = Rd[i].d[k];
  }
  return 0;
}

/* Per-element state for x (regular/irregular alike): S (n_qp*9), C33 (n_qp),
   current geometry (24: a1, a2, n, gc1, gc2, Aaa, Abb, Aab), Fb (3*nen). */
int oracle_elem_state(const double *x, int ec, double *S, double *C33, double *geom24, double *Fb)
{
  if (!g_body || !g_body->ready) return 58;
  const Body &B = *g_body;
  const Mesh &m = B.m;
  if (ec < 0 || ec >= m.n_elmt) return 63;
  const int ntot = m.n_v + m.n_ghosts;
  std::vector<double> xb(ntot), yb(ntot), zb(ntot);
  for (int v = 0; v < m.n_v; v++) { xb[v] = x[3 * v]; yb[v] = x[3 * v + 1]; zb[v] = x[3 * v + 2]; }
  for (int v = m.n_v; v < ntot; v++) { xb[v] = m.x0[v]; yb[v] = m.y0[v]; zb[v] = m.z0[v]; }
  global_ghost(m, xb.data(), yb.data(), zb.data());
  double Sq[kMaxQp][3][3], c33[kMaxQp], fb[48];
  Geom<double> G;
  int rc = elem_forces<double>(m, B.P, ec, B.ref[ec], xb.data(), yb.data(), zb.data(), fb, Sq, c33, &G);
  if (rc) return rc;
  for (int q = 0; q < B.P.n_qp; q++) {
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) S[9 * q + 3 * i + j] = Sq[q][i][j];
    C33[q] = c33[q];
  }
  const V3<double> *vs[8] = {&G.a1, &G.a2, &G.n, &G.gc1, &G.gc2, &G.Aaa, &G.Abb, &G.Aab};
  for (int k = 0; k < 8; k++) { geom24[3 * k] = vs[k]->x; geom24[3 * k + 1] = vs[k]->y; geom24[3 * k + 2] = vs[k]->z; }
  if (Fb) for (int i = 0; i < 3 * G.nen; i++) Fb[i] = fb[i];
  return 0;
}

/* IN arrays of the one-step subdivision for valence v (5 x (v+6), row major). */
int oracle_set_basis(int kind) { (void)g_tables_init; return set_basis_tables(kind); }

int oracle_set_thickness_normal(int on)
{
  if (on != 0 && on != 1) return 63;
  g_tnormal = on;
  return 0;
}

int oracle_irregular_weights(int v, double *out)
{
  const int nen = v + 6;
  return irregular_weights(v, out, out + nen, out + 2 * nen, out + 3 * nen, out + 4 * nen);
}

/* CPU baseline of R+K: for elements [e0, e1) evaluate the element force and
   its derivative w.r.t. the element's patch coordinates (forward mode over
   all 3*nen patch coordinates at once, Dual<48>), using `threads` OpenMP
   threads, then assemble the element forces in element order.  Returns a
   checksum in *chk (keeps the work observable).  This is the reference's
   own per-element algorithm (active_strain.c) with its tangent taken
   exactly; the reference itself has no tangent. */
int oracle_rk_sample(const double *x, int e0, int e1, int threads, double *chk)
{
  if (!g_body || !g_body->ready) return 58;
  const Body &B = *g_body;
  const Mesh &m = B.m;
  if (e0 < 0 || e1 > m.n_elmt || e0 > e1) return 63;
  const int ntot = m.n_v + m.n_ghosts;
  std::vector<double> xb(ntot), yb(ntot), zb(ntot);
  for (int v = 0; v < m.n_v; v++) { xb[v] = x[3 * v]; yb[v] = x[3 * v + 1]; zb[v] = x[3 * v + 2]; }
  for (int v = m.n_v; v < ntot; v++) { xb[v] = m.x0[v]; yb[v] = m.y0[v]; zb[v] = m.z0[v]; }
  global_ghost(m, xb.data(), yb.data(), zb.data());
  const int ne = e1 - e0;
  std::vector<double> part((size_t)ne, 0.0);
  std::vector<int> rcs(ne, 0);
#ifdef _OPENMP
#pragma omp parallel num_threads(threads > 0 ? threads : 1)
#endif
  {
    /* per-thread coordinate copies carrying the element's seeds */
    std::vector<Dual<48>> xd(ntot), yd(ntot), zd(ntot);
    for (int v = 0; v < ntot; v++) { xd[v] = Dual<48>(xb[v]); yd[v] = Dual<48>(yb[v]); zd[v] = Dual<48>(zb[v]); }
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 8)
#endif
    for (int k = 0; k < ne; k++) {
      const int ec = e0 + k;
      const int nen = (m.ire[ec] == 0) ? 12 : m.val[ec] + 6;
      const int *pt = &m.patch[16 * ec];
      for (int a = 0; a < nen; a++) {
        const int n = pt[a];
        xd[n].d[3 * a] = 1.0; yd[n].d[3 * a + 1] = 1.0; zd[n].d[3 * a + 2] = 1.0;
      }
      Dual<48> Fb[48];
      rcs[k] = elem_forces<Dual<48>>(m, B.P, ec, B.ref[ec], xd.data(), yd.data(), zd.data(), Fb);
      double s = 0.0;
      for (int i = 0; i < 3 * nen; i++) { s += Fb[i].v; for (int j = 0; j < 3 * nen; j++) s += 1e-3 * Fb[i].d[j]; }
      part[k] = s;
      for (int a = 0; a < nen; a++) {
        const int n = pt[a];
        for (int j = 0; j < 48; j++) { xd[n].d[j] = 0.0; yd[n].d[j] = 0.0; zd[n].d[j] = 0.0; }
      }
    }
  }
  for (int k = 0; k < ne; k++) if (rcs[k]) return rcs[k];
  double c = 0.0;
  for (int k = 0; k < ne; k++) c += part[k];
  *chk = c;
  return 0;
}

/* CPU baseline of the residual alone (the only thing the reference evaluates:
   its Newton is Jacobian-free, main.c:464-466): the element forces of
   elements [e0, e1) by the reference's per-element algorithm
   (FInternalAct's loop body, active_strain.c:2226-2267) on `threads` OpenMP
   threads, checksum in *chk. */
int oracle_r_sample(const double *x, int e0, int e1, int threads, double *chk)
{
  if (!g_body || !g_body->ready) return 58;
  const Body &B = *g_body;
  const Mesh &m = B.m;
  if (e0 < 0 || e1 > m.n_elmt || e0 > e1) return 63;
  const int ntot = m.n_v + m.n_ghosts;
  std::vector<double> xb(ntot), yb(ntot), zb(ntot);
  for (int v = 0; v < m.n_v; v++) { xb[v] = x[3 * v]; yb[v] = x[3 * v + 1]; zb[v] = x[3 * v + 2]; }
  for (int v = m.n_v; v < ntot; v++) { xb[v] = m.x0[v]; yb[v] = m.y0[v]; zb[v] = m.z0[v]; }
  global_ghost(m, xb.data(), yb.data(), zb.data());
  const int ne = e1 - e0;
  std::vector<double> part((size_t)ne, 0.0);
  std::vector<int> rcs(ne, 0);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads > 0 ? threads : 1)
#endif
  for (int k = 0; k < ne; k++) {
    const int ec = e0 + k;
    const int nen = (m.ire[ec] == 0) ? 12 : m.val[ec] + 6;
    double Fb[48];
    rcs[k] = elem_forces<double>(m, B.P, ec, B.ref[ec], xb.data(), yb.data(), zb.data(), Fb);
    double s = 0.0;
    for (int i = 0; i < 3 * nen; i++) s += Fb[i];
    part[k] = s;
  }
  for (int k = 0; k < ne; k++) if (rcs[k]) return rcs[k];
  double c = 0.0;
  for (int k = 0; k < ne; k++) c += part[k];
  *chk = c;
  return 0;
}

void oracle_teardown(void) { delete g_body; g_body = nullptr; }

} /* extern "C" */
