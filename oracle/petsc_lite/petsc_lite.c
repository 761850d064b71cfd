/*
 * petsc-lite implementation (TEST INFRASTRUCTURE ONLY; see petscsys.h).
 * One rank, host arrays, no threads.
 */
#include "petscsys.h"

#include <fcntl.h>
#include <unistd.h>

static int lite_verbose_(void) { return getenv("PETSC_LITE_VERBOSE") != NULL; }

PetscErrorCode PetscLiteError_(PetscErrorCode code, const char *file, int line, const char *fmt, ...)
{
  va_list ap;
  fprintf(stderr, "[petsc-lite] error %d at %s:%d: ", code, file, line);
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  fprintf(stderr, "\n");
  return code;
}

PetscErrorCode PetscPrintf(MPI_Comm comm, const char *fmt, ...)
{
  (void)comm;
  if (!lite_verbose_()) return 0;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  return 0;
}

PetscErrorCode PetscFPrintf(MPI_Comm comm, FILE *fd, const char *fmt, ...)
{
  (void)comm;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(fd ? fd : stderr, fmt, ap);
  va_end(ap);
  return 0;
}

PetscErrorCode PetscBarrier(void *obj) { (void)obj; return 0; }

/* ---------------- options ---------------- */
#define LITE_MAX_OPTS 128
static char lite_opt_name_[LITE_MAX_OPTS][64];
static char lite_opt_val_[LITE_MAX_OPTS][64];
static int  lite_nopt_ = 0;

void PetscLiteClearOptions(void) { lite_nopt_ = 0; }

void PetscLiteSetOption(const char *name, const char *value)
{
  for (int i = 0; i < lite_nopt_; i++) {
    if (strcmp(lite_opt_name_[i], name) == 0) {
      snprintf(lite_opt_val_[i], sizeof(lite_opt_val_[i]), "%s", value);
      return;
    }
  }
  if (lite_nopt_ >= LITE_MAX_OPTS) return;
  snprintf(lite_opt_name_[lite_nopt_], sizeof(lite_opt_name_[0]), "%s", name);
  snprintf(lite_opt_val_[lite_nopt_], sizeof(lite_opt_val_[0]), "%s", value);
  lite_nopt_++;
}

static const char *lite_find_(const char *name)
{
  for (int i = 0; i < lite_nopt_; i++)
    if (strcmp(lite_opt_name_[i], name) == 0) return lite_opt_val_[i];
  return NULL;
}

PetscErrorCode PetscOptionsGetInt(PetscOptions o, const char pre[], const char name[], PetscInt *v, PetscBool *set)
{
  (void)o; (void)pre;
  const char *s = lite_find_(name);
  if (s) *v = (PetscInt)strtol(s, NULL, 10);
  if (set) *set = s ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

PetscErrorCode PetscOptionsGetReal(PetscOptions o, const char pre[], const char name[], PetscReal *v, PetscBool *set)
{
  (void)o; (void)pre;
  const char *s = lite_find_(name);
  if (s) *v = strtod(s, NULL);
  if (set) *set = s ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

PetscErrorCode PetscOptionsGetBool(PetscOptions o, const char pre[], const char name[], PetscBool *v, PetscBool *set)
{
  (void)o; (void)pre;
  const char *s = lite_find_(name);
  if (s) *v = (s[0] == '1' || s[0] == 't' || s[0] == 'T' || s[0] == 'y') ? PETSC_TRUE : PETSC_FALSE;
  if (set) *set = s ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

PetscErrorCode PetscOptionsGetString(PetscOptions o, const char pre[], const char name[], char *v, size_t len, PetscBool *set)
{
  (void)o; (void)pre;
  const char *s = lite_find_(name);
  if (s && len) snprintf(v, len, "%s", s);
  if (set) *set = s ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

/* ---------------- MPI at one rank ---------------- */
int MPI_Comm_rank(MPI_Comm comm, PetscMPIInt *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, PetscMPIInt *size) { (void)comm; *size = 1; return 0; }

int MPI_Allreduce(const void *send, void *recv, int n, MPI_Datatype t, MPI_Op op, MPI_Comm comm)
{
  (void)op; (void)comm;
  if (send != MPI_IN_PLACE && n > 0) memcpy(recv, send, (size_t)n * (size_t)t);
  return 0;
}

int MPI_Reduce(const void *send, void *recv, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm)
{
  (void)root;
  return MPI_Allreduce(send, recv, n, t, op, comm);
}

int MPI_Bcast(void *buf, int n, MPI_Datatype t, int root, MPI_Comm comm)
{
  (void)buf; (void)n; (void)t; (void)root; (void)comm;
  return 0;
}

PetscErrorCode PetscSortIntWithArray(PetscInt n, PetscInt keys[], PetscInt vals[])
{
  for (PetscInt i = 1; i < n; i++) {
    PetscInt k = keys[i], v = vals[i], j = i - 1;
    while (j >= 0 && keys[j] > k) { keys[j + 1] = keys[j]; vals[j + 1] = vals[j]; j--; }
    keys[j + 1] = k; vals[j + 1] = v;
  }
  return 0;
}

/* ---------------- Vec ---------------- */
PetscErrorCode VecCreateSeq(MPI_Comm c, PetscInt n, Vec *v)
{
  (void)c;
  *v = (Vec)calloc(1, sizeof(**v));
  (*v)->n = n;
  (*v)->a = (PetscScalar *)calloc((size_t)(n > 0 ? n : 1), sizeof(PetscScalar));
  return 0;
}

PetscErrorCode VecCreateMPI(MPI_Comm c, PetscInt nlocal, PetscInt N, Vec *v)
{
  return VecCreateSeq(c, N >= 0 ? N : nlocal, v);
}

PetscErrorCode VecDuplicate(Vec x, Vec *y) { return VecCreateSeq(0, x->n, y); }

PetscErrorCode VecDestroy(Vec *v)
{
  if (v && *v) { free((*v)->a); free(*v); *v = NULL; }
  return 0;
}

PetscErrorCode VecSet(Vec v, PetscScalar a)
{
  for (PetscInt i = 0; i < v->n; i++) v->a[i] = a;
  return 0;
}

PetscErrorCode VecCopy(Vec x, Vec y) { memcpy(y->a, x->a, sizeof(PetscScalar) * (size_t)x->n); return 0; }
PetscErrorCode VecGetArray(Vec v, PetscScalar **a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a) { (void)v; *a = NULL; return 0; }
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a) { (void)v; *a = NULL; return 0; }

PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt idx[], const PetscScalar y[], InsertMode m)
{
  for (PetscInt i = 0; i < n; i++) {
    if (idx[i] < 0) continue;
    if (idx[i] >= v->n) return PetscLiteError_(PETSC_ERR_ARG_OUTOFRANGE, __FILE__, __LINE__, "VecSetValues index %d >= %d", idx[i], v->n);
    if (m == ADD_VALUES) v->a[idx[i]] += y[i]; else v->a[idx[i]] = y[i];
  }
  return 0;
}

PetscErrorCode VecAssemblyBegin(Vec v) { (void)v; return 0; }
PetscErrorCode VecAssemblyEnd(Vec v) { (void)v; return 0; }

PetscErrorCode VecNorm(Vec v, NormType t, PetscReal *r)
{
  PetscReal s = 0.0;
  for (PetscInt i = 0; i < v->n; i++) {
    PetscReal a = fabs(v->a[i]);
    if (t == NORM_INFINITY) { if (a > s) s = a; }
    else if (t == NORM_1) s += a;
    else s += a * a;
  }
  *r = (t == NORM_2 || t == NORM_FROBENIUS) ? sqrt(s) : s;
  return 0;
}

PetscErrorCode VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y)
{
  for (PetscInt i = 0; i < w->n; i++) w->a[i] = a * x->a[i] + y->a[i];
  return 0;
}

PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x)
{
  for (PetscInt i = 0; i < y->n; i++) y->a[i] += a * x->a[i];
  return 0;
}

PetscErrorCode VecScale(Vec x, PetscScalar a)
{
  for (PetscInt i = 0; i < x->n; i++) x->a[i] *= a;
  return 0;
}

PetscErrorCode VecGetSize(Vec v, PetscInt *n) { *n = v->n; return 0; }
PetscErrorCode VecGetOwnershipRange(Vec v, PetscInt *lo, PetscInt *hi) { *lo = 0; *hi = v->n; return 0; }

#define LITE_UNSUPPORTED(name) \
  return PetscLiteError_(PETSC_ERR_SUP, __FILE__, __LINE__, "%s is not part of petsc-lite", name)

/* Binary viewer: PETSc's documented file layout, every item big-endian
   (PetscBinaryWrite / PetscBinaryRead); VecView writes the record
   VEC_FILE_CLASSID (1211214), the length, the values, with 32-bit PetscInt.
   No ".info" side file is written. */
/* The one object the opaque handles point at: a binary viewer (fd) or an
   array-backed SeqBAIJ matrix (the rest); SNES, DM and the others are never created. */
struct PetscLiteOpaque_ {
  int fd;
  PetscInt bs, mb, nb;
  const PetscInt *i, *j;
  PetscScalar *a;
  int locked;   /* between MatSeqBAIJGetArray and MatSeqBAIJRestoreArray */
};
#define LITE_VEC_FILE_CLASSID 1211214

static void lite_swap_(unsigned char *b, size_t size, size_t n)
{
  for (size_t i = 0; i < n; i++) {
    unsigned char *e = b + i * size;
    for (size_t k = 0; k < size / 2; k++) { unsigned char t = e[k]; e[k] = e[size - 1 - k]; e[size - 1 - k] = t; }
  }
}

static int lite_little_endian_(void) { const unsigned one = 1; return *(const unsigned char *)&one == 1; }

PetscErrorCode PetscBinaryWrite(int fd, const void *p, PetscInt n, PetscDataType t)
{
  const size_t size = t == PETSC_INT ? sizeof(PetscInt) : sizeof(PetscReal);
  unsigned char *b = (unsigned char *)malloc(size * (size_t)(n > 0 ? n : 1));
  memcpy(b, p, size * (size_t)n);
  if (lite_little_endian_()) lite_swap_(b, size, (size_t)n);
  const ssize_t w = write(fd, b, size * (size_t)n);
  free(b);
  if (w != (ssize_t)(size * (size_t)n)) return PetscLiteError_(PETSC_ERR_FILE_WRITE, __FILE__, __LINE__, "short write");
  return 0;
}

PetscErrorCode PetscBinaryRead(int fd, void *p, PetscInt n, PetscInt *count, PetscDataType t)
{
  const size_t size = t == PETSC_INT ? sizeof(PetscInt) : sizeof(PetscReal);
  size_t got = 0;
  while (got < size * (size_t)n) {
    const ssize_t r = read(fd, (unsigned char *)p + got, size * (size_t)n - got);
    if (r <= 0) break;
    got += (size_t)r;
  }
  if (lite_little_endian_()) lite_swap_((unsigned char *)p, size, got / size);
  if (count) *count = (PetscInt)(got / size);
  else if (got != size * (size_t)n) return PetscLiteError_(PETSC_ERR_FILE_READ, __FILE__, __LINE__, "short read");
  return 0;
}

PetscErrorCode PetscViewerBinaryOpen(MPI_Comm c, const char name[], PetscFileMode m, PetscViewer *w)
{
  (void)c;
  const int fd = m == FILE_MODE_READ ? open(name, O_RDONLY) : open(name, O_WRONLY | O_CREAT | O_TRUNC, 0666);
  if (fd < 0) return PetscLiteError_(PETSC_ERR_FILE_OPEN, __FILE__, __LINE__, "cannot open %s", name);
  *w = (PetscViewer)malloc(sizeof(**w));
  (*w)->fd = fd;
  return 0;
}

PetscErrorCode PetscViewerDestroy(PetscViewer *w)
{
  if (w && *w) { close((*w)->fd); free(*w); *w = NULL; }
  return 0;
}

PetscErrorCode PetscViewerBinaryGetDescriptor(PetscViewer w, int *fd)
{
  if (!w) return PetscLiteError_(PETSC_ERR_ARG_NULL, __FILE__, __LINE__, "null viewer");
  *fd = w->fd;
  return 0;
}

PetscErrorCode VecView(Vec v, PetscViewer w)
{
  PetscInt head[2] = {LITE_VEC_FILE_CLASSID, v->n};
  PetscCall(PetscBinaryWrite(w->fd, head, 2, PETSC_INT));
  return PetscBinaryWrite(w->fd, v->a, v->n, PETSC_REAL);
}

PetscErrorCode VecLoad(Vec v, PetscViewer w)
{
  PetscInt head[2];
  PetscCall(PetscBinaryRead(w->fd, head, 2, NULL, PETSC_INT));
  if (head[0] != LITE_VEC_FILE_CLASSID || head[1] != v->n)
    return PetscLiteError_(PETSC_ERR_FILE_UNEXPECTED, __FILE__, __LINE__, "not a Vec record of length %d", (int)v->n);
  return PetscBinaryRead(w->fd, v->a, v->n, NULL, PETSC_REAL);
}
PetscErrorCode PetscRealView(PetscInt n, const PetscReal v[], PetscViewer w) { (void)n; (void)v; (void)w; LITE_UNSUPPORTED("PetscRealView"); }

PetscErrorCode MatCreate(MPI_Comm c, Mat *m) { (void)c; (void)m; LITE_UNSUPPORTED("MatCreate"); }
PetscErrorCode MatSetSizes(Mat m, PetscInt a, PetscInt b, PetscInt c, PetscInt d)
{ (void)m; (void)a; (void)b; (void)c; (void)d; LITE_UNSUPPORTED("MatSetSizes"); }
PetscErrorCode MatSetFromOptions(Mat m) { (void)m; LITE_UNSUPPORTED("MatSetFromOptions"); }
PetscErrorCode MatSetType(Mat m, MatType t) { (void)m; (void)t; LITE_UNSUPPORTED("MatSetType"); }
PetscErrorCode MatSetUp(Mat m) { (void)m; LITE_UNSUPPORTED("MatSetUp"); }
PetscErrorCode MatZeroEntries(Mat m) { (void)m; LITE_UNSUPPORTED("MatZeroEntries"); }
PetscErrorCode MatGetSize(Mat m, PetscInt *a, PetscInt *b) { (void)m; (void)a; (void)b; LITE_UNSUPPORTED("MatGetSize"); }
PetscErrorCode MatCreateSeqDense(MPI_Comm c, PetscInt a, PetscInt b, PetscScalar *d, Mat *m)
{ (void)c; (void)a; (void)b; (void)d; (void)m; LITE_UNSUPPORTED("MatCreateSeqDense"); }

/* The block matrix of MatCreateSeqBAIJWithArrays is the only Mat kind the
   shim creates (its fields are in struct PetscLiteOpaque_ above). */
PetscErrorCode MatCreateSeqBAIJWithArrays(MPI_Comm c, PetscInt bs, PetscInt m, PetscInt n, PetscInt i[], PetscInt j[],
                                          PetscScalar a[], Mat *mat)
{
  (void)c;
  if (!mat || !i || !j || !a || bs < 1 || m % bs || n % bs)
    return PetscLiteError_(PETSC_ERR_ARG_WRONG, __FILE__, __LINE__, "bad SeqBAIJ arguments");
  struct PetscLiteOpaque_ *A = (struct PetscLiteOpaque_ *)calloc(1, sizeof(*A));
  A->bs = bs; A->mb = m / bs; A->nb = n / bs; A->i = i; A->j = j; A->a = a;
  *mat = A;
  return 0;
}

PetscErrorCode MatSeqBAIJGetArray(Mat A, PetscScalar **a)
{
  if (!A || A->locked) return PetscLiteError_(PETSC_ERR_ORDER, __FILE__, __LINE__, "array already taken");
  A->locked = 1;
  *a = A->a;
  return 0;
}

PetscErrorCode MatSeqBAIJRestoreArray(Mat A, PetscScalar **a)
{
  if (!A || !A->locked || *a != A->a) return PetscLiteError_(PETSC_ERR_ORDER, __FILE__, __LINE__, "array not taken");
  A->locked = 0;
  *a = NULL;
  return 0;
}

PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t) { (void)t; return A && !A->locked ? 0 : PETSC_ERR_ORDER; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t) { (void)t; return A && !A->locked ? 0 : PETSC_ERR_ORDER; }

/* y = A x with the column-by-column block storage */
PetscErrorCode MatMult(Mat A, Vec x, Vec y)
{
  if (!A || x->n != A->nb * A->bs || y->n != A->mb * A->bs)
    return PetscLiteError_(PETSC_ERR_ARG_SIZ, __FILE__, __LINE__, "MatMult sizes");
  const PetscInt bs = A->bs;
  for (PetscInt I = 0; I < A->mb; I++) {
    for (PetscInt r = 0; r < bs; r++) y->a[I * bs + r] = 0.0;
    for (PetscInt k = A->i[I]; k < A->i[I + 1]; k++) {
      const PetscScalar *blk = A->a + (size_t)k * bs * bs;
      const PetscScalar *xj = x->a + (size_t)A->j[k] * bs;
      for (PetscInt cc = 0; cc < bs; cc++)
        for (PetscInt r = 0; r < bs; r++) y->a[I * bs + r] += blk[cc * bs + r] * xj[cc];
    }
  }
  return 0;
}

PetscErrorCode MatDestroy(Mat *A)
{
  if (A && *A) { free(*A); *A = NULL; }
  return 0;
}
