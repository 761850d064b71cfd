/*
 * Subdivision-surface topology in O(N): ghost ring, irregular-vertex
 * classification and the 12 / v+6 patch stencils.
 *
 * Produces tables bit-identical to the reference's O(N^2) searches
 * GlobalGhostInit (bending.c:1670-1757), IrrVer (bending.c:1188-1267) and
 * Patch (bending.c:1270-1667), including their apex-cap rules: with
 * n_elmt_base > 0 the elements from n_elmt_base on are flat cap triangles,
 * which count towards no node's valence (bending.c:1204-1222), take no part
 * in the apex ring's ghost reflection (bending.c:1683-1687) and whose patch
 * holds only their corners, in slots 3, 6 and 7 (bending.c:1282-1294).  The reference scans every triangle for each
 * stencil query and keeps the LAST triangle that matches; every query of
 * Patch() involves one of the element's three corner nodes, so scanning only
 * the triangles incident to those corners, in increasing triangle index,
 * performs the same sequence of matches and writes.
 */
#include <algorithm>
#include <string>
#include <vector>

#include "biofem_host.h"

namespace biofem {

/* The reference's Patch() marks an unresolved stencil slot with the node id
   1000000 (bending.c:1291), which collides with real node ids from 10^6 nodes
   on.  The search here marks it with -1, which no node id can equal; the
   slots past the stencil (16 - nen of them) are still filled with 1000000 so
   that the tables equal the reference's bit for bit. */
static const int kUnset = -1;
static const int kMissing = 1000000;

/* node -> incident triangles (increasing triangle index), CSR */
static void incidence(int n_nodes, int n_tri, const std::vector<int> &tri, std::vector<int> &ptr, std::vector<int> &idx)
{
  ptr.assign(n_nodes + 1, 0);
  for (int t = 0; t < n_tri; t++)
    for (int k = 0; k < 3; k++) ptr[tri[3 * t + k] + 1]++;
  for (int i = 0; i < n_nodes; i++) ptr[i + 1] += ptr[i];
  idx.assign(ptr[n_nodes], 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int t = 0; t < n_tri; t++)
    for (int k = 0; k < 3; k++) {
      const int n = tri[3 * t + k];
      /* a triangle listing a node twice is recorded once */
      bool dup = false;
      for (int kk = 0; kk < k; kk++) if (tri[3 * t + kk] == n) dup = true;
      if (!dup) idx[fill[n]++] = t;
    }
  /* rows may be shorter than reserved when a triangle repeats a node */
  std::vector<int> ptr2(n_nodes + 1, 0), idx2;
  idx2.reserve(idx.size());
  for (int i = 0; i < n_nodes; i++) {
    for (int j = ptr[i]; j < fill[i]; j++) idx2.push_back(idx[j]);
    ptr2[i + 1] = (int)idx2.size();
  }
  ptr.swap(ptr2);
  idx.swap(idx2);
}

/* One shared-edge query of Patch(): triangle (a,b,c) holds both p[A] and p[B]
   -> write its first corner outside {e1,e2,e3} (guarded) into p[out]. */
static inline void pick(int *p, int A, int B, int a, int b, int c, int e1, int e2, int e3, bool guard, int out)
{
  int mm = 0;
  if (p[A] == a || p[A] == b || p[A] == c) mm++;
  if (p[B] == a || p[B] == b || p[B] == c) mm++;
  if (mm == 2) {
    if (a != e1 && a != e2 && a != e3 && guard) p[out] = a;
    else if (b != e1 && b != e2 && b != e3 && guard) p[out] = b;
    else if (c != e1 && c != e2 && c != e3 && guard) p[out] = c;
  }
}

int build_topology(const BiofemMeshDesc &d, HostTopo &T, std::string &err)
{
  const int nv = d.n_v, ne = d.n_elmt, nedge = d.n_edge;
  if (nv <= 0 || ne <= 0 || nedge < 0) { err = "empty mesh"; return 62; }
  int ng = 0;
  for (int e = 0; e < nedge; e++) {
    if (d.n_bnodes[e] < 3) { err = "a boundary ring needs at least 3 nodes"; return 62; }
    ng += d.n_bnodes[e];
  }
  if ((long long)nv + ng >= (1LL << 31) - 1) { err = "n_v + n_ghosts must fit in int32"; return 63; }
  for (int i = 0; i < 3 * ne; i++)
    if (d.tri[i] < 0 || d.tri[i] >= nv) { err = "triangle corner out of range"; return 63; }
  for (int i = 0; i < ng; i++)
    if (d.bnodes[i] < 0 || d.bnodes[i] >= nv) { err = "boundary node out of range"; return 63; }

  const int nbase = d.n_elmt_base;
  if (nbase < 0 || nbase > ne) { err = "n_elmt_base outside [0, n_elmt]"; return 63; }
  const int ec_limit = nbase > 0 ? nbase : ne;   /* elements counted by IrrVer */
  T.n_v = nv; T.n_elmt = ne; T.n_ghosts = ng; T.n_edge = nedge; T.n_elmt_base = nbase;
  const int ntri = ne + 2 * ng, ntot = nv + ng;
  T.tri_all.assign(3 * (size_t)ntri, 0);
  std::copy(d.tri, d.tri + 3 * (size_t)ne, T.tri_all.begin());
  T.xyz0_full.assign(3 * (size_t)ntot, 0.0);
  std::copy(d.xyz0, d.xyz0 + 3 * (size_t)nv, T.xyz0_full.begin());
  T.ghost_nv1.assign(ng, 0); T.ghost_nv2.assign(ng, 0); T.ghost_nv3.assign(ng, 0);

  std::vector<int> rptr, ridx;  /* real triangles only */
  incidence(nv, ne, T.tri_all, rptr, ridx);

  /* ---- GlobalGhostInit (bending.c:1670-1757) ---- */
  int count = 0, start = 0;
  for (int edge_n = 0; edge_n < nedge; edge_n++) {
    const int n_local = d.n_bnodes[edge_n];
    const int ring_first = count;
    const int ring_limit = (edge_n == 0) ? ec_limit : ne;   /* the apex ring reflects through base elements */
    for (int li = 0; li < n_local; li++) {
      const int nv1 = d.bnodes[start + (li + 1) % n_local], nv2 = d.bnodes[start + li];
      int nv3 = -1;
      /* last real triangle holding both nv1 and nv2 */
      for (int j = rptr[nv1]; j < rptr[nv1 + 1]; j++) {
        const int ec = ridx[j];
        if (ec >= ring_limit) break;   /* increasing triangle index */
        const int a = T.tri_all[3 * ec], b = T.tri_all[3 * ec + 1], c = T.tri_all[3 * ec + 2];
        if (!(nv2 == a || nv2 == b || nv2 == c)) continue;
        if (a != nv1 && a != nv2) nv3 = a;
        else if (b != nv1 && b != nv2) nv3 = b;
        else nv3 = c;
      }
      if (nv3 < 0) { err = "boundary ring edge belongs to no triangle"; return 62; }
      const int g = nv + count;
      for (int k = 0; k < 3; k++)
        T.xyz0_full[3 * (size_t)g + k] = T.xyz0_full[3 * (size_t)nv2 + k] + T.xyz0_full[3 * (size_t)nv1 + k] - T.xyz0_full[3 * (size_t)nv3 + k];
      T.ghost_nv1[count] = nv1; T.ghost_nv2[count] = nv2; T.ghost_nv3[count] = nv3;
      const size_t t0 = 3 * (size_t)(ne + 2 * count);
      T.tri_all[t0 + 0] = nv1; T.tri_all[t0 + 1] = nv2; T.tri_all[t0 + 2] = g;
      const int gprev = (li == 0) ? (nv + ring_first + n_local - 1) : (g - 1);
      T.tri_all[t0 + 3] = g; T.tri_all[t0 + 4] = nv2; T.tri_all[t0 + 5] = gprev;
      count++;
    }
    start += n_local;
  }

  /* ---- IrrVer (bending.c:1188-1267) ---- */
  std::vector<char> is_b(nv, 0);
  for (int i = 0; i < ng; i++) is_b[d.bnodes[i]] = 1;
  std::vector<char> irr(nv, 0);
  std::vector<int> nval(nv, 6);
  for (int n = 0; n < nv; n++) {
    int cnt = 0;   /* base elements holding n */
    for (int j = rptr[n]; j < rptr[n + 1] && ridx[j] < ec_limit; j++) cnt++;
    if (!is_b[n]) { if (cnt != 6) { irr[n] = 1; nval[n] = cnt; } }
    else if (cnt + 3 != 6) { irr[n] = 1; nval[n] = cnt + 3; }
  }
  T.ire.assign(ne, 0); T.irv.assign(ne, 0); T.val.assign(ne, 6);
  for (int ec = 0; ec < ne; ec++) {
    /* the largest-index irregular corner wins both val (node loop) and irv */
    int best = -1;
    for (int k = 0; k < 3; k++) {
      const int n = T.tri_all[3 * ec + k];
      if (irr[n] && n > best) best = n;
    }
    if (best >= 0) {
      if (ec < ec_limit) { T.ire[ec] = 1; T.val[ec] = nval[best]; }   /* cap elements keep ire 0, val 6 */
      for (int k = 0; k < 3; k++) if (T.tri_all[3 * ec + k] == best) T.irv[ec] = k + 1;
    }
  }

  /* ---- Patch (bending.c:1270-1667) over corner-incident triangles ---- */
  std::vector<int> aptr, aidx;  /* all triangles incl. ghost ones */
  incidence(ntot, ntri, T.tri_all, aptr, aidx);
  T.patch.assign(16 * (size_t)ne, kMissing);
  std::vector<int> cand;
  cand.reserve(64);
  int p[64];
  for (int ec = 0; ec < ne; ec++) {
    const int v = T.val[ec];
    if (ec >= ec_limit) {
      T.patch[16 * (size_t)ec + 3] = T.tri_all[3 * ec];
      T.patch[16 * (size_t)ec + 6] = T.tri_all[3 * ec + 1];
      T.patch[16 * (size_t)ec + 7] = T.tri_all[3 * ec + 2];
      continue;
    }
    if (v + 6 > 16 || v < 3) { err = "element valence outside the 16-wide patch (3 <= v <= 10)"; return 56; }
    for (int i = 0; i < v + 6; i++) p[i] = kUnset;
    const int n1 = T.tri_all[3 * ec], n2 = T.tri_all[3 * ec + 1], n3 = T.tri_all[3 * ec + 2];
    cand.clear();
    for (int n : {n1, n2, n3})
      for (int j = aptr[n]; j < aptr[n + 1]; j++) cand.push_back(aidx[j]);
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    auto tri3 = [&](int i, int &a, int &b, int &c) { a = T.tri_all[3 * i]; b = T.tri_all[3 * i + 1]; c = T.tri_all[3 * i + 2]; };
    int a, b, c;
    if (T.ire[ec] == 0) {
      p[3] = n1; p[6] = n2; p[7] = n3;
      for (int i : cand) {
        tri3(i, a, b, c);
        const bool g = (i != ec);
        pick(p, 3, 6, a, b, c, p[3], p[6], p[6], g, 2);
        pick(p, 3, 7, a, b, c, p[3], p[7], p[7], g, 4);
        pick(p, 6, 7, a, b, c, p[6], p[7], p[7], g, 10);
      }
      for (int i : cand) {
        tri3(i, a, b, c);
        pick(p, 3, 2, a, b, c, p[3], p[2], p[6], true, 0);
        pick(p, 3, 4, a, b, c, p[3], p[4], p[7], true, 1);
        pick(p, 6, 2, a, b, c, p[6], p[2], p[3], true, 5);
        pick(p, 6, 10, a, b, c, p[6], p[10], p[7], true, 9);
        pick(p, 7, 10, a, b, c, p[7], p[10], p[6], true, 11);
        pick(p, 7, 4, a, b, c, p[7], p[4], p[3], true, 8);
      }
    } else {
      if (T.irv[ec] == 1) { p[0] = n1; p[1] = n2; p[v] = n3; }
      else if (T.irv[ec] == 2) { p[0] = n2; p[1] = n3; p[v] = n1; }
      else if (T.irv[ec] == 3) { p[0] = n3; p[1] = n1; p[v] = n2; }
      for (int i : cand) {
        tri3(i, a, b, c);
        const bool g = (i != ec);
        pick(p, 0, 1, a, b, c, p[0], p[1], p[1], g, 2);
        pick(p, 0, v, a, b, c, p[0], p[v], p[v], g, v - 1);
        pick(p, 1, v, a, b, c, p[1], p[v], p[v], g, v + 1);
      }
      for (int i : cand) {
        tri3(i, a, b, c);
        pick(p, 0, 2, a, b, c, p[0], p[2], p[1], true, 3);
        pick(p, 0, v - 1, a, b, c, p[0], p[v - 1], p[v], true, v - 2);
        pick(p, 1, 2, a, b, c, p[1], p[2], p[0], true, v + 3);
        pick(p, 1, v + 1, a, b, c, p[1], p[v + 1], p[v], true, v + 2);
        pick(p, v, v + 1, a, b, c, p[v], p[v + 1], p[1], true, v + 4);
        pick(p, v, v - 1, a, b, c, p[v], p[v - 1], p[0], true, v + 5);
      }
      if (v > 6) {
        for (int k = 0; k < v - 6; k++)
          for (int i : cand) {
            tri3(i, a, b, c);
            pick(p, 0, 3 + k, a, b, c, p[0], p[3 + k], p[2 + k], true, k + 4);
            pick(p, 0, v - 2 - k, a, b, c, p[0], p[v - 2 - k], p[v - 1 - k], true, v - 3 - k);
          }
      }
    }
    int fix = -1, gfix = -1;
    for (int i = 0; i < v + 6; i++) {
      if (p[i] == kUnset) continue;
      if (fix < 0) fix = p[i];
      if (p[i] >= nv) { gfix = p[i]; break; }
    }
    if (gfix >= 0) fix = gfix;
    if (fix >= 0) for (int i = 0; i < v + 6; i++) if (p[i] == kUnset) p[i] = fix;
    for (int i = 0; i < v + 6; i++) {
      if (p[i] == kUnset) { err = "patch stencil incomplete after ghost resolution"; return 77; }
      T.patch[16 * (size_t)ec + i] = p[i];
    }
  }

  /* the stencils the kernels read: a cap element's three corners in slots
     0-2 (the cap basis table acts on those), the rest a copy of the first
     corner (never read) */
  T.dpatch = T.patch;
  for (int ec = ec_limit; ec < ne; ec++) {
    int *q = &T.dpatch[16 * (size_t)ec];
    for (int k = 0; k < 16; k++) q[k] = T.tri_all[3 * ec + (k < 3 ? k : 0)];
  }
  return 0;
}

} /* namespace biofem */
