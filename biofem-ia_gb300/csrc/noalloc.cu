/*
 * RunGpuResidualNoAlloc: the residual entry point for callers that cannot
 * allocate device memory at call time.
 *
 * Who needs it: a caller that runs under a fixed device-memory budget it has
 * already reserved (a serving loop admitting meshes by HBM budget, or a host
 * code that owns all device memory through its own pool) must not have a
 * library call reach cudaMalloc, which can fail under the budget, fragments
 * the pool, and synchronises the device.  This variant allocates nothing:
 * the caller passes the prepared mesh handle, x and R (device pointers), and
 * the per-call work arrays of the residual (node positions, element forces,
 * pressure corner forces, the |Fext| maximum) live in one file-scope device
 * array of fixed size, BIOFEM_NOALLOC_SCRATCH_DOUBLES doubles (8 MiB), that
 * every GPU which loads the library holds until the process exits.
 *
 * Limit: 4*(n_v + n_ghosts) + 51*n_elmt + 1 doubles must fit in the array
 * (about 19,000 triangles on a flat mesh); larger meshes get error 63.
 *
 * Sharing: all calls use the same array and it keeps the last call's
 * contents.  Calls whose work overlaps on the GPU (different streams, or
 * different host threads) race on it; serialise them.  The |Fext| maximum
 * is cleared by every call; every other entry is written before it is read.
 *
 * First call on a device: it looks up the array's device address with
 * cudaGetSymbolAddress (once per device, that device current) and caches
 * it.  Make that first call before any stream capture.
 *
 * Device: the handle's mesh arrays live on the device that was current when
 * it was prepared; a call made with another device current is refused
 * (error 62), so that no launch mixes one device's array with another's mesh.
 *
 * Errors: as for the other device variants, a vanishing CC3333 inside the
 * element kernel (ModElemC33, active_strain.c:1676) sets the handle's status
 * word, which BiofemGpuSync(handle, stream) turns into error 72; calls on
 * the same handle that overlap on the GPU share that word.
 */
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "biofem_host.h"

#define BIOFEM_NOALLOC_SCRATCH_DOUBLES (1 << 20)   /* 8 MiB */

namespace biofem {

static __device__ __align__(256) double g_noalloc_scratch[BIOFEM_NOALLOC_SCRATCH_DOUBLES];

static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[64] = {};   /* device address per device ordinal */

/* error reporting shared with bridge.cu */
int noalloc_fail(int code, const std::string &msg);
const DevMesh *mesh_devview(const BiofemGpuMesh *m, const KParams **kp, int *device);

static int noalloc_scratch(double **out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(76, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return noalloc_fail(63, "device ordinal beyond 63");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return noalloc_fail(76, std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[dev];
  return 0;
}

} /* namespace biofem */

using namespace biofem;

extern "C" int RunGpuResidualNoAlloc(BiofemGpuMesh *m, const double *d_x, double *d_R, void *stream)
{
  if (!m || !d_x || !d_R) return noalloc_fail(85, "null argument");
  const KParams *kp = nullptr;
  int mdev = -1, cur = -1;
  const DevMesh *dm = mesh_devview(m, &kp, &mdev);
  if (!dm || !kp) return noalloc_fail(58, "mesh handle has no device data (host-only handle?)");
  if (cudaGetDevice(&cur) != cudaSuccess) return noalloc_fail(76, "cudaGetDevice failed");
  if (cur != mdev)
    return noalloc_fail(62, "the mesh handle lives on device " + std::to_string(mdev) + " but device " +
                                std::to_string(cur) + " is current");
  const long long need = 4LL * kp->nt + 51LL * kp->ne + 1;
  if (need > BIOFEM_NOALLOC_SCRATCH_DOUBLES)
    return noalloc_fail(63, "mesh too large for the no-allocation residual: needs " + std::to_string(need) +
                                " scratch doubles, the fixed array holds " +
                                std::to_string(BIOFEM_NOALLOC_SCRATCH_DOUBLES));
  double *base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc) return rc;
  /* carve the fixed array: positions, element forces, pressure forces, |Fext| max */
  DevMesh v = *dm;
  v.pos = base;
  v.fb = base + 4LL * kp->nt;
  v.fp = v.fb + 48LL * kp->ne;
  v.fmax = reinterpret_cast<unsigned long long *>(v.fp + 3LL * kp->ne);
  cudaStream_t st = (cudaStream_t)stream;
  /* the element kernel of the handle's precision (FP32-bulk handles carry the
     float-float constants), so the result is RunGpuResidualDevice's */
  if ((rc = launch_positions(v, *kp, d_x, st)) ||
      (rc = v.erefFF ? launch_elem_residual_ff(v, *kp, st) : launch_elem_residual(v, *kp, st)) ||
      (rc = launch_node_gather(v, *kp, d_x, d_R, st)) || (rc = launch_scale(v, *kp, d_R, st)))
    return noalloc_fail(76, std::string("no-alloc residual launch: ") + cudaGetErrorString((cudaError_t)rc));
  return 0;
}
