/*
 * On-disk formats of the shell solver: checkpoints (LocationOut / LocationIn,
 * io.c:1272-1376 and io.c:1513-1640) and the VTK files of a time step (Output,
 * io.c:540-964; Write3DShellVTK, io.c:983-1064).  Host code, C-ABI in
 * include/biofem_gpu.h.
 *
 * Checkpoint files are "<dir>/<tag><ibi>_<ti>.dat" (tag x, xn, xd, xdd; ibi one
 * digit, ti five), each one vector of 3 (n_v + n_ghosts) doubles in original-
 * vertex order, big-endian as every PETSc binary file:
 *   BIOFEM_CKPT_VERTEX_ORDER  the values alone, as PetscBinaryWrite writes them
 *                             on the DMPlex path (io.c:1285-1334), restartable at
 *                             any process count;
 *   BIOFEM_CKPT_VEC           a PETSc VecView record: int32 VEC_FILE_CLASSID
 *                             (1211214), int32 length, the values (the serial
 *                             path, io.c:1335-1356).
 * LocationIn reads either (and a VecView record with 64-bit header integers),
 * telling them apart by the file size.
 *
 * VTK files are legacy ASCII with the reference's exact printf formats, so
 * the same state gives the same bytes.
 */
#include <cerrno>
#include <cstdarg>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <sys/types.h>

#include "../../include/biofem_gpu.h"

namespace biofem {
int host_fail(int code, const std::string &msg);   /* sets the calling thread's last error (bridge.cu) */
}

namespace {

constexpr int32_t kVecClassId = 1211214;

void put_be64(unsigned char *p, double v)
{
  uint64_t u;
  std::memcpy(&u, &v, 8);
  for (int k = 7; k >= 0; k--) { p[k] = (unsigned char)(u & 0xffu); u >>= 8; }
}

double get_be64(const unsigned char *p)
{
  uint64_t u = 0;
  for (int k = 0; k < 8; k++) u = (u << 8) | p[k];
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}

void put_be32(unsigned char *p, int32_t v)
{
  uint32_t u = (uint32_t)v;
  for (int k = 3; k >= 0; k--) { p[k] = (unsigned char)(u & 0xffu); u >>= 8; }
}

int64_t get_be_int(const unsigned char *p, int bytes)
{
  uint64_t u = 0;
  for (int k = 0; k < bytes; k++) u = (u << 8) | p[k];
  if (bytes == 4) return (int64_t)(int32_t)(uint32_t)u;
  return (int64_t)u;
}

std::string dir_of(const char *dir)
{
  return (dir && dir[0]) ? std::string(dir) : std::string(".");
}

std::string ckpt_name(const std::string &dir, const char *tag, int ibi, int ti)
{
  char buf[64];
  std::snprintf(buf, sizeof(buf), "/%s%1.1d_%5.5d.dat", tag, ibi, ti);
  return dir + buf;
}

int write_vector(const std::string &path, const double *v, int64_t n, int layout)
{
  const size_t head = layout == BIOFEM_CKPT_VEC ? 8 : 0;
  std::vector<unsigned char> buf(head + 8 * (size_t)n);
  if (layout == BIOFEM_CKPT_VEC) {
    put_be32(buf.data(), kVecClassId);
    put_be32(buf.data() + 4, (int32_t)n);
  }
  for (int64_t i = 0; i < n; i++) put_be64(buf.data() + head + 8 * (size_t)i, v[i]);
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return biofem::host_fail(90, "cannot open " + path + ": " + std::strerror(errno));
  const size_t w = std::fwrite(buf.data(), 1, buf.size(), f);
  const int c = std::fclose(f);
  if (w != buf.size() || c != 0) return biofem::host_fail(90, "short write to " + path);
  return 0;
}

int read_vector(const std::string &path, double *v, int64_t n)
{
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return biofem::host_fail(91, "cannot open " + path + ": " + std::strerror(errno));
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t r;
  while ((r = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + r);
  std::fclose(f);
  /* a self-consistent VecView record (its header's length matches the file
     size) is one; otherwise the file must hold exactly the n values */
  const size_t sz = buf.size();
  size_t head = 0;
  int64_t len = -1;
  if (sz >= 8 && get_be_int(buf.data(), 4) == kVecClassId && (sz - 8) % 8 == 0 &&
      get_be_int(buf.data() + 4, 4) == (int64_t)((sz - 8) / 8)) {
    head = 8; len = get_be_int(buf.data() + 4, 4);            /* VecView, 32-bit PetscInt */
  } else if (sz >= 16 && get_be_int(buf.data(), 8) == kVecClassId && (sz - 16) % 8 == 0 &&
             get_be_int(buf.data() + 8, 8) == (int64_t)((sz - 16) / 8)) {
    head = 16; len = get_be_int(buf.data() + 8, 8);           /* VecView, 64-bit PetscInt */
  } else if (sz % 8 == 0) {
    len = (int64_t)(sz / 8);                                   /* the values alone */
  }
  if (len != n)
    return biofem::host_fail(92, path + ": " + std::to_string(sz) + " bytes hold " +
                                     (len < 0 ? std::string("no checkpoint vector") : std::to_string(len) + " values") +
                                     ", the mesh has " + std::to_string(n));
  for (int64_t i = 0; i < n; i++) v[i] = get_be64(buf.data() + head + 8 * (size_t)i);
  return 0;
}

void make_dir(const std::string &d)
{
  mkdir(d.c_str(), 0777);   /* io.c:1283: an existing directory is fine */
}

/* printf into a growing buffer (one fwrite per file) */
struct Out {
  std::string s;
  void operator()(const char *fmt, ...) __attribute__((format(printf, 2, 3)))
  {
    char tmp[256];
    va_list ap;
    va_start(ap, fmt);
    const int k = std::vsnprintf(tmp, sizeof(tmp), fmt, ap);
    va_end(ap);
    if (k < (int)sizeof(tmp)) { s.append(tmp, (size_t)(k > 0 ? k : 0)); return; }
    std::vector<char> big((size_t)k + 1);
    va_start(ap, fmt);
    std::vsnprintf(big.data(), big.size(), fmt, ap);
    va_end(ap);
    s.append(big.data(), (size_t)k);
  }
  int save(const std::string &path) const
  {
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return biofem::host_fail(90, "cannot open " + path + ": " + std::strerror(errno));
    const size_t w = std::fwrite(s.data(), 1, s.size(), f);
    const int c = std::fclose(f);
    if (w != s.size() || c != 0) return biofem::host_fail(90, "short write to " + path);
    return 0;
  }
};

/* AreaNormal's area (io.c:1646-1669) of triangle e on coordinates P */
double flat_area(const double *P, const int32_t *tri, int e)
{
  const int a = tri[3 * e], b = tri[3 * e + 1], c = tri[3 * e + 2];
  const double d21[3] = {P[3 * b] - P[3 * a], P[3 * b + 1] - P[3 * a + 1], P[3 * b + 2] - P[3 * a + 2]};
  const double d31[3] = {P[3 * c] - P[3 * a], P[3 * c + 1] - P[3 * a + 1], P[3 * c + 2] - P[3 * a + 2]};
  const double cx = d21[1] * d31[2] - d31[1] * d21[2];
  const double cy = -d21[0] * d31[2] + d31[0] * d21[2];
  const double cz = d21[0] * d31[1] - d31[0] * d21[1];
  return 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
}

} /* namespace */

extern "C" {

int BiofemLocationOut(const char *dir, int32_t ti, int32_t ibi, int64_t n_dof, const double *x, const double *xn,
                      const double *xd, const double *xdd, int32_t layout)
{
  if (!x || !xn || !xd || !xdd || n_dof <= 0) return biofem::host_fail(85, "null argument");
  if (layout != BIOFEM_CKPT_VERTEX_ORDER && layout != BIOFEM_CKPT_VEC) return biofem::host_fail(62, "unknown checkpoint layout");
  if (layout == BIOFEM_CKPT_VEC && n_dof > INT32_MAX) return biofem::host_fail(62, "vector too long for a 32-bit VecView header");
  const std::string d = dir_of(dir);
  make_dir(d);
  const char *tag[4] = {"x", "xn", "xd", "xdd"};
  const double *v[4] = {x, xn, xd, xdd};
  for (int k = 0; k < 4; k++) {
    int rc = write_vector(ckpt_name(d, tag[k], ibi, ti), v[k], n_dof, layout);
    if (rc) return rc;
  }
  return 0;
}

int BiofemLocationIn(const char *dir, int32_t ti, int32_t ibi, int64_t n_dof, double *x, double *xn, double *xd,
                     double *xdd)
{
  if (!x || !xn || !xd || !xdd || n_dof <= 0) return biofem::host_fail(85, "null argument");
  const std::string d = dir_of(dir);
  const char *tag[4] = {"x", "xn", "xd", "xdd"};
  double *v[4] = {x, xn, xd, xdd};
  for (int k = 0; k < 4; k++) {
    int rc = read_vector(ckpt_name(d, tag[k], ibi, ti), v[k], n_dof);
    if (rc) return rc;
  }
  return 0;
}

int BiofemWriteSurfaceVTK(const char *dir, int32_t ti, int32_t ibi, const BiofemSurfaceFields *f)
{
  if (!f || !f->tri || !f->x || !f->X || !f->gamma_e) return biofem::host_fail(85, "null argument");
  const int nv = f->n_v, ne = f->n_elmt;
  if (nv <= 0 || ne <= 0) return biofem::host_fail(62, "empty surface");
  for (int i = 0; i < 3 * ne; i++)
    if (f->tri[i] < 0 || f->tri[i] >= nv) return biofem::host_fail(63, "triangle corner out of range");
  const std::string d = dir_of(dir);
  make_dir(d);
  char name[64];
  std::snprintf(name, sizeof(name), "/surface%2.2d_%5.5d.vtk", ibi, ti);
  auto vec3 = [&](const double *a, int i, int k) { return a ? a[3 * i + k] : 0.0; };
  Out o;
  o("# vtk DataFile Version 2.0\n");
  o("Surface Grid\n");
  o("ASCII\n");
  o("DATASET UNSTRUCTURED_GRID\n");
  o("POINTS  %d float\n", nv);
  for (int i = 0; i < nv; i++) o("%f %f %f\n", f->x[3 * i], f->x[3 * i + 1], f->x[3 * i + 2]);
  o("CELLS %d %d\n", ne, 4 * ne);
  for (int e = 0; e < ne; e++) o("%d  %d %d %d\n", 3, f->tri[3 * e], f->tri[3 * e + 1], f->tri[3 * e + 2]);
  o("CELL_TYPES %d\n", ne);
  for (int e = 0; e < ne; e++) o("%d\n", 5);
  o("POINT_DATA %d\n", nv);
  /* no contact on this path: the contact flags and the bending energy IE are 0 */
  o("SCALARS contact integer\n");
  o("LOOKUP_TABLE default\n");
  for (int i = 0; i < nv; i++) o("%d\n", 0);
  o("SCALARS m float\n");
  o("LOOKUP_TABLE default\n");
  for (int i = 0; i < nv; i++) o("%f \n", f->mass ? f->mass[i] : 0.0);
  o("SCALARS IE float\n");
  o("LOOKUP_TABLE default\n");
  for (int i = 0; i < nv; i++) o("%f \n", 0.0);
  o("VECTORS disp float\n");
  for (int i = 0; i < nv; i++)
    o("%f %f %f\n", f->x[3 * i] - f->X[3 * i], f->x[3 * i + 1] - f->X[3 * i + 1], f->x[3 * i + 2] - f->X[3 * i + 2]);
  const char *lab[5] = {"Fint", "Fext", "Fdyn", "Fcnt", "u"};
  const double *src[5] = {f->Fint, f->Fext, f->Fdyn, nullptr, f->xd};
  for (int k = 0; k < 5; k++) {
    o("VECTORS %s float\n", lab[k]);
    for (int i = 0; i < nv; i++) o("%f %f %f\n", vec3(src[k], i, 0), vec3(src[k], i, 1), vec3(src[k], i, 2));
  }
  /* R = Fint - Fext + Fdyn (io.c:724-749) */
  o("VECTORS Res float\n");
  for (int i = 0; i < nv; i++)
    o("%f %f %f\n", vec3(f->Fint, i, 0) - vec3(f->Fext, i, 0) + vec3(f->Fdyn, i, 0),
      vec3(f->Fint, i, 1) - vec3(f->Fext, i, 1) + vec3(f->Fdyn, i, 1),
      vec3(f->Fint, i, 2) - vec3(f->Fext, i, 2) + vec3(f->Fdyn, i, 2));
  o("CELL_DATA %d\n", ne);
  if (f->fib) {
    o("VECTORS nfib float\n");
    for (int e = 0; e < ne; e++) o("%f %f %f\n", f->fib[3 * e], f->fib[3 * e + 1], f->fib[3 * e + 2]);
  }
  o("SCALARS dA float\n");
  o("LOOKUP_TABLE default\n");
  for (int e = 0; e < ne; e++) o("%f \n", flat_area(f->x, f->tri, e));
  o("SCALARS dA0 float\n");
  o("LOOKUP_TABLE default\n");
  for (int e = 0; e < ne; e++) o("%f \n", f->dA0 ? f->dA0[e] : flat_area(f->X, f->tri, e));
  o("SCALARS gamma float\n");
  o("LOOKUP_TABLE default\n");
  for (int e = 0; e < ne; e++) o("%f \n", f->gamma_e[e]);
  return o.save(d + name);
}

int BiofemWriteShell3dVTK(const char *dir, int32_t ti, int32_t ibi, int32_t n_v, int32_t n_elmt, const int32_t *tri,
                          const double *x, const double *thickness_e)
{
  if (!tri || !x || !thickness_e) return biofem::host_fail(85, "null argument");
  if (n_v <= 0 || n_elmt <= 0) return biofem::host_fail(62, "empty surface");
  for (int i = 0; i < 3 * n_elmt; i++)
    if (tri[i] < 0 || tri[i] >= n_v) return biofem::host_fail(63, "triangle corner out of range");
  /* area-weighted node normals and node-averaged thickness (io.c:992-1024) */
  std::vector<double> nx(n_v, 0.0), ny(n_v, 0.0), nz(n_v, 0.0), tsum(n_v, 0.0), th(n_v, 0.0);
  std::vector<int> tcnt(n_v, 0);
  for (int e = 0; e < n_elmt; e++) {
    const int c[3] = {tri[3 * e], tri[3 * e + 1], tri[3 * e + 2]};
    const double e1[3] = {x[3 * c[1]] - x[3 * c[0]], x[3 * c[1] + 1] - x[3 * c[0] + 1], x[3 * c[1] + 2] - x[3 * c[0] + 2]};
    const double e2[3] = {x[3 * c[2]] - x[3 * c[0]], x[3 * c[2] + 1] - x[3 * c[0] + 1], x[3 * c[2] + 2] - x[3 * c[0] + 2]};
    const double fn[3] = {e1[1] * e2[2] - e2[1] * e1[2], -e1[0] * e2[2] + e2[0] * e1[2], e1[0] * e2[1] - e2[0] * e1[1]};
    for (int k = 0; k < 3; k++) {
      nx[c[k]] += fn[0]; ny[c[k]] += fn[1]; nz[c[k]] += fn[2];
      tsum[c[k]] += thickness_e[e]; tcnt[c[k]]++;
    }
  }
  for (int v = 0; v < n_v; v++) {
    const double len = std::sqrt(nx[v] * nx[v] + ny[v] * ny[v] + nz[v] * nz[v]);
    if (len > 1.0e-14) { nx[v] /= len; ny[v] /= len; nz[v] /= len; }
    th[v] = (tcnt[v] > 0) ? tsum[v] / (double)tcnt[v] : 0.0;
  }
  const std::string d = dir_of(dir);
  make_dir(d);
  char name[64];
  std::snprintf(name, sizeof(name), "/shell3d%2.2d_%5.5d.vtk", ibi, ti);
  Out o;
  o("# vtk DataFile Version 2.0\nLV 3D shell (visualization only)\nASCII\nDATASET UNSTRUCTURED_GRID\n");
  o("POINTS %d float\n", 2 * n_v);
  for (int v = 0; v < n_v; v++) {
    const double h2 = 0.5 * th[v];
    o("%f %f %f\n", x[3 * v] - h2 * nx[v], x[3 * v + 1] - h2 * ny[v], x[3 * v + 2] - h2 * nz[v]);
  }
  for (int v = 0; v < n_v; v++) {
    const double h2 = 0.5 * th[v];
    o("%f %f %f\n", x[3 * v] + h2 * nx[v], x[3 * v + 1] + h2 * ny[v], x[3 * v + 2] + h2 * nz[v]);
  }
  o("CELLS %d %d\n", n_elmt, 7 * n_elmt);
  for (int e = 0; e < n_elmt; e++) {
    const int n1 = tri[3 * e], n2 = tri[3 * e + 1], n3 = tri[3 * e + 2];
    o("6 %d %d %d %d %d %d\n", n1, n2, n3, n1 + n_v, n2 + n_v, n3 + n_v);
  }
  o("CELL_TYPES %d\n", n_elmt);
  for (int e = 0; e < n_elmt; e++) o("13\n");
  o("POINT_DATA %d\n", 2 * n_v);
  o("SCALARS layer float 1\nLOOKUP_TABLE default\n");
  for (int v = 0; v < n_v; v++) o("0.0\n");
  for (int v = 0; v < n_v; v++) o("1.0\n");
  o("SCALARS thickness float 1\nLOOKUP_TABLE default\n");
  for (int v = 0; v < n_v; v++) o("%f\n", th[v]);
  for (int v = 0; v < n_v; v++) o("%f\n", th[v]);
  return o.save(d + name);
}

} /* extern "C" */
