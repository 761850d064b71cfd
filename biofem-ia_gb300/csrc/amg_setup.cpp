/*
 * Host symbolic setup of the smoothed-aggregation hierarchy (see amg.h).
 * Everything here depends only on the mesh (pattern, identity rows,
 * reference positions), so it runs once per mesh handle.
 */
#include <algorithm>
#include <cmath>

#include "amg.h"

namespace biofem {
namespace {

/* Greedy aggregation on a node graph.  Pass 1 makes an aggregate of every
   free node whose free neighbours are all still unassigned (the node and those
   neighbours); pass 2 attaches each remaining free node to the pass-1
   aggregate of its first assigned neighbour; pass 3 groups what is left with
   its unassigned free neighbours.  Returns the number of aggregates. */
int aggregate(int n, const std::vector<int> &gptr, const std::vector<int> &gadj, const std::vector<char> &free_,
              std::vector<int> &agg)
{
  agg.assign(n, -1);
  int na = 0;
  for (int i = 0; i < n; i++) {
    if (!free_[i] || agg[i] >= 0) continue;
    bool clean = true;
    for (int k = gptr[i]; k < gptr[i + 1] && clean; k++) {
      const int j = gadj[k];
      if (free_[j] && agg[j] >= 0) clean = false;
    }
    if (!clean) continue;
    agg[i] = na;
    for (int k = gptr[i]; k < gptr[i + 1]; k++)
      if (free_[gadj[k]]) agg[gadj[k]] = na;
    na++;
  }
  const std::vector<int> first = agg;
  for (int i = 0; i < n; i++) {
    if (!free_[i] || agg[i] >= 0) continue;
    for (int k = gptr[i]; k < gptr[i + 1]; k++)
      if (first[gadj[k]] >= 0) { agg[i] = first[gadj[k]]; break; }
  }
  for (int i = 0; i < n; i++) {
    if (!free_[i] || agg[i] >= 0) continue;
    agg[i] = na;
    for (int k = gptr[i]; k < gptr[i + 1]; k++)
      if (free_[gadj[k]] && agg[gadj[k]] < 0) agg[gadj[k]] = na;
    na++;
  }
  return na;
}

/* Tentative prolongator: per aggregate, the member rows of the near-null
   space B (bs rows per node, 6 columns) are orthonormalised by Gram-Schmidt
   applied twice; Q holds the orthonormal rows, the coefficients R become the
   coarse near-null space (6 rows per aggregate).  A column that vanishes marks
   its coarse unknown dead. */
void tentative(int n, int bs, int na, const std::vector<int> &agg, const std::vector<double> &B, std::vector<float> &Q,
               std::vector<double> &Bc, std::vector<unsigned char> &dead)
{
  constexpr int k6 = kAmgCoarseBs;
  std::vector<int> aptr(na + 1, 0), amem;
  for (int i = 0; i < n; i++) if (agg[i] >= 0) aptr[agg[i] + 1]++;
  for (int a = 0; a < na; a++) aptr[a + 1] += aptr[a];
  amem.resize(aptr[na]);
  {
    std::vector<int> fill(aptr.begin(), aptr.end() - 1);
    for (int i = 0; i < n; i++) if (agg[i] >= 0) amem[fill[agg[i]]++] = i;
  }
  Q.assign((size_t)n * bs * k6, 0.f);
  Bc.assign((size_t)na * k6 * k6, 0.0);
  dead.assign((size_t)na * k6, 0);
  std::vector<double> M;
  for (int a = 0; a < na; a++) {
    const int cnt = aptr[a + 1] - aptr[a], rows = cnt * bs;
    M.assign((size_t)rows * k6, 0.0);
    for (int m = 0; m < cnt; m++) {
      const int i = amem[aptr[a] + m];
      for (int r = 0; r < bs; r++)
        for (int c = 0; c < k6; c++) M[(size_t)(m * bs + r) * k6 + c] = B[((size_t)i * bs + r) * k6 + c];
    }
    double R[k6][k6] = {};
    for (int c = 0; c < k6; c++) {
      double n0 = 0.0;
      for (int r = 0; r < rows; r++) n0 += M[(size_t)r * k6 + c] * M[(size_t)r * k6 + c];
      n0 = std::sqrt(n0);
      for (int pass = 0; pass < 2; pass++)
        for (int p = 0; p < c; p++) {
          double s = 0.0;
          for (int r = 0; r < rows; r++) s += M[(size_t)r * k6 + p] * M[(size_t)r * k6 + c];
          R[p][c] += s;
          for (int r = 0; r < rows; r++) M[(size_t)r * k6 + c] -= s * M[(size_t)r * k6 + p];
        }
      double nr = 0.0;
      for (int r = 0; r < rows; r++) nr += M[(size_t)r * k6 + c] * M[(size_t)r * k6 + c];
      nr = std::sqrt(nr);
      if (!(nr > 1e-10 * n0) || nr == 0.0) {
        for (int r = 0; r < rows; r++) M[(size_t)r * k6 + c] = 0.0;
        dead[(size_t)a * k6 + c] = 1;
      } else {
        for (int r = 0; r < rows; r++) M[(size_t)r * k6 + c] /= nr;
        R[c][c] = nr;
      }
    }
    for (int m = 0; m < cnt; m++) {
      const int i = amem[aptr[a] + m];
      for (int r = 0; r < bs; r++)
        for (int c = 0; c < k6; c++) Q[((size_t)i * bs + r) * k6 + c] = (float)M[(size_t)(m * bs + r) * k6 + c];
    }
    for (int p = 0; p < k6; p++)
      for (int c = 0; c < k6; c++) Bc[((size_t)a * k6 + p) * k6 + c] = R[p][c];
  }
}

/* Row-wise union of column sets: out row i = sorted union over the sets
   named by src(i); marker-array merge, linear in the total input size. */
template <class RowSources>
void union_pattern(int nrows, int ncols, RowSources src, std::vector<int> &ptr, std::vector<int> &col,
                   std::vector<int> &blkrow)
{
  std::vector<int> mark(ncols, -1), buf;
  ptr.assign(nrows + 1, 0);
  col.clear();
  for (int i = 0; i < nrows; i++) {
    buf.clear();
    src(i, [&](int c) { if (mark[c] != i) { mark[c] = i; buf.push_back(c); } });
    std::sort(buf.begin(), buf.end());
    col.insert(col.end(), buf.begin(), buf.end());
    ptr[i + 1] = (int)col.size();
  }
  blkrow.resize(col.size());
  for (int i = 0; i < nrows; i++)
    for (int k = ptr[i]; k < ptr[i + 1]; k++) blkrow[k] = i;
}

void diag_index(int n, const std::vector<int> &ptr, const std::vector<int> &col, std::vector<int> &diag)
{
  diag.assign(n, -1);
  for (int i = 0; i < n; i++)
    for (int k = ptr[i]; k < ptr[i + 1]; k++)
      if (col[k] == i) { diag[i] = k; break; }
}

}  // namespace

int amg_symbolic(int nt, const std::vector<int> &rowptr, const std::vector<int> &colind,
                 const std::vector<unsigned char> &rowkind, const std::vector<double> &X, const int *tri, int ntri,
                 std::vector<AmgLevelHost> &levels)
{
  constexpr int k6 = kAmgCoarseBs;
  levels.clear();
  /* level 0: free rows, near-null space (translations + infinitesimal
     rotations about the free nodes' centroid), triangle-edge graph */
  std::vector<char> free_(nt);
  double cen[3] = {0, 0, 0};
  int nfree = 0;
  for (int i = 0; i < nt; i++) {
    free_[i] = rowkind[i] == 0;
    if (free_[i]) { for (int d = 0; d < 3; d++) cen[d] += X[3 * (size_t)i + d]; nfree++; }
  }
  for (int d = 0; d < 3; d++) cen[d] /= std::max(nfree, 1);
  std::vector<double> B((size_t)nt * 3 * k6, 0.0);
  for (int i = 0; i < nt; i++) {
    if (!free_[i]) continue;
    const double cx = X[3 * (size_t)i] - cen[0], cy = X[3 * (size_t)i + 1] - cen[1], cz = X[3 * (size_t)i + 2] - cen[2];
    double *b = &B[(size_t)i * 3 * k6];
    b[0 * k6 + 0] = 1.0; b[1 * k6 + 1] = 1.0; b[2 * k6 + 2] = 1.0;
    b[1 * k6 + 3] = -cz; b[2 * k6 + 3] = cy;         /* rotation about x */
    b[0 * k6 + 4] = cz;  b[2 * k6 + 4] = -cx;        /* rotation about y */
    b[0 * k6 + 5] = -cy; b[1 * k6 + 5] = cx;         /* rotation about z */
  }
  std::vector<int> gptr(nt + 1, 0), gadj;
  {
    std::vector<std::vector<int>> nb(nt);
    for (int e = 0; e < ntri; e++)
      for (int a = 0; a < 3; a++) {
        const int u = tri[3 * e + a], v = tri[3 * e + (a + 1) % 3];
        nb[u].push_back(v);
        nb[v].push_back(u);
      }
    for (int i = 0; i < nt; i++) {
      std::sort(nb[i].begin(), nb[i].end());
      nb[i].erase(std::unique(nb[i].begin(), nb[i].end()), nb[i].end());
      gptr[i + 1] = gptr[i] + (int)nb[i].size();
    }
    gadj.reserve(gptr[nt]);
    for (int i = 0; i < nt; i++) gadj.insert(gadj.end(), nb[i].begin(), nb[i].end());
  }

  AmgLevelHost L0;
  L0.n = nt; L0.bs = 3;
  L0.rowptr = rowptr; L0.colind = colind;
  diag_index(nt, L0.rowptr, L0.colind, L0.diag);
  levels.push_back(std::move(L0));

  for (int lev = 0; lev < kAmgMaxLevels - 1; lev++) {
    AmgLevelHost &L = levels.back();
    if ((long long)L.n * L.bs <= kAmgMaxDense) break;
    std::vector<int> agg;
    const int na = aggregate(L.n, gptr, gadj, free_, agg);
    if (na == 0 || (long long)na * k6 >= (long long)L.n * L.bs) break;     /* no coarsening: stop here */
    L.na = na;
    L.agg = agg;
    std::vector<double> Bc;
    tentative(L.n, L.bs, na, agg, B, L.Q, Bc, L.dead);
    /* P: fine row -> aggregates of its operator neighbours (free rows only) */
    union_pattern(L.n, na, [&](int i, auto add) {
      if (L.agg[i] < 0) return;
      for (int k = L.rowptr[i]; k < L.rowptr[i + 1]; k++)
        if (L.agg[L.colind[k]] >= 0) add(L.agg[L.colind[k]]);
    }, L.prow, L.pcol, L.pblkrow);
    /* P^T by counting sort on the aggregate */
    L.rrow.assign(na + 1, 0);
    for (int c : L.pcol) L.rrow[c + 1]++;
    for (int a = 0; a < na; a++) L.rrow[a + 1] += L.rrow[a];
    L.rcol.resize(L.pcol.size());
    L.rmap.resize(L.pcol.size());
    {
      std::vector<int> fill(L.rrow.begin(), L.rrow.end() - 1);
      for (int i = 0; i < L.n; i++)
        for (int k = L.prow[i]; k < L.prow[i + 1]; k++) {
          const int slot = fill[L.pcol[k]]++;
          L.rcol[slot] = i;
          L.rmap[slot] = k;
        }
    }
    /* T = A P, needed on free rows only (P^T reads no other row) */
    union_pattern(L.n, na, [&](int i, auto add) {
      if (L.agg[i] < 0) return;
      for (int k = L.rowptr[i]; k < L.rowptr[i + 1]; k++) {
        const int j = L.colind[k];
        for (int q = L.prow[j]; q < L.prow[j + 1]; q++) add(L.pcol[q]);
      }
    }, L.trow, L.tcol, L.tblkrow);
    /* next operator P^T A P */
    union_pattern(na, na, [&](int a, auto add) {
      for (int r = L.rrow[a]; r < L.rrow[a + 1]; r++) {
        const int i = L.rcol[r];
        for (int q = L.trow[i]; q < L.trow[i + 1]; q++) add(L.tcol[q]);
      }
    }, L.crow, L.ccol, L.cblkrow);

    AmgLevelHost C;
    C.n = na; C.bs = k6;
    C.rowptr = L.crow; C.colind = L.ccol;
    diag_index(na, C.rowptr, C.colind, C.diag);
    /* next level's graph: the operator pattern without the diagonal; all
       coarse nodes are free */
    gptr.assign(na + 1, 0);
    gadj.clear();
    for (int a = 0; a < na; a++) {
      for (int k = C.rowptr[a]; k < C.rowptr[a + 1]; k++)
        if (C.colind[k] != a) gadj.push_back(C.colind[k]);
      gptr[a + 1] = (int)gadj.size();
    }
    free_.assign(na, 1);
    B.swap(Bc);
    levels.push_back(std::move(C));
  }
  return (int)levels.size();
}

}  // namespace biofem
