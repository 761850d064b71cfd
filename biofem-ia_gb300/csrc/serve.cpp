/*
 * Serving loop for quasi-static load-step requests (the `biofem sweep`
 * workload, bin/biofem:352-456, as a resident service instead of a batch of
 * separate jobs).
 *
 * Continuous batching: a request is admitted as soon as a slot is free and
 * its device-memory estimate fits the HBM budget; admitted requests run
 * concurrently, each on its own CUDA stream and host worker thread (mesh
 * setup, Newton with the assembled tangent, GMRES/block-Jacobi), so the
 * kernels of different requests overlap on the GPU, and a finished request
 * returns its memory and slot to the next waiting one at once.  Admission is
 * first-fit in arrival order: a request that does not fit yet does not block
 * smaller ones behind it.  Device memory comes from the stream-ordered pool,
 * so handles are created and destroyed without synchronising the device.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "biofem_host.h"

namespace biofem {
int noalloc_fail(int code, const std::string &msg);   /* sets the calling thread's last error (bridge.cu) */
}

namespace {

struct ServeReq {
  int64_t ticket = 0;
  std::vector<int32_t> tri, nb, bn;
  std::vector<double> xyz, fib, gs, x;
  BiofemMeshDesc desc{};
  BiofemParams prm{};
  BiofemNewtonOptions opt{};
  int64_t est = 0;
  double t_submit = 0, t_start = 0, t_done = 0;
  int rc = 0;
  bool done = false;
  BiofemNewtonStats st{};
  std::string err;
};

double now_s(std::chrono::steady_clock::time_point t0)
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct BiofemServe_ {
  int64_t budget = 0;
  int max_slots = 1;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv, cv_done;
  std::deque<ServeReq *> queue;
  std::map<int64_t, ServeReq *> reqs;
  int64_t next_ticket = 1, in_use = 0, peak_in_use = 0, completed = 0;
  int active = 0, peak_active = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
};

extern "C" int BiofemServeEstimateBytes(int32_t n_v, int32_t n_elmt, int32_t n_ghosts, int32_t precision,
                                        int32_t gmres_restart, int64_t *bytes);

static void worker_main(BiofemServe_ *E)
{
  cudaSetDevice(E->device);
  biofem::t_blocking_waits = true;
  /* one stream per worker, reused by every request it serves */
  cudaStream_t s = nullptr;
  const int src = (int)cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { if (s) cudaStreamDestroy(s); } } guard{s};
  for (;;) {
    ServeReq *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(E->mu);
      for (;;) {
        if (E->stop && E->queue.empty()) return;
        if (E->active < E->max_slots) {
          for (auto it = E->queue.begin(); it != E->queue.end(); ++it) {
            if (E->in_use + (*it)->est <= E->budget) { r = *it; E->queue.erase(it); break; }
          }
        }
        if (r) break;
        E->cv.wait(lk);
      }
      E->in_use += r->est;
      E->active++;
      if (E->in_use > E->peak_in_use) E->peak_in_use = E->in_use;
      if (E->active > E->peak_active) E->peak_active = E->active;
      r->t_start = now_s(E->t0);
    }
    int rc = src;
    BiofemGpuMesh *h = nullptr;
    if (!rc) rc = PrepareGpuMeshOnStream(&r->desc, &r->prm, (void *)s, &h);
    if (!rc) rc = RunGpuNewtonSolve(h, r->x.data(), &r->opt, &r->st);
    if (rc) r->err = BiofemGpuLastError();
    if (h) DestroyGpuMesh(h);
    {
      std::lock_guard<std::mutex> lk(E->mu);
      E->in_use -= r->est;
      E->active--;
      E->completed++;
      r->rc = rc;
      r->t_done = now_s(E->t0);
      r->done = true;
    }
    E->cv.notify_all();
    E->cv_done.notify_all();
  }
}

extern "C" {

int BiofemServeEstimateBytes(int32_t n_v, int32_t n_elmt, int32_t n_ghosts, int32_t precision,
                             int32_t gmres_restart, int64_t *bytes)
{
  if (!bytes) return 85;
  const int64_t nt = (int64_t)n_v + n_ghosts;
  const int m = gmres_restart > 0 ? gmres_restart : 30;
  /* per element: tangent block df/dy (240 values), forces, thickness-point
     metrics, primal geometry, resultants and C33 values (FP64; 3 points,
     3 sub-iterations), reference constants, row-assembly lists and records
     (80 bytes for each of the element's ~12 row contributions); per node:
     tangent row (~37 blocks), pattern, flexible-GMRES bases V and Z,
     multigrid hierarchy (FP32 copy of the tangent for FP64 handles, P, A P,
     the coarse operators) */
  const int64_t per_elem = (precision == BIOFEM_FP64 ? 6800 : 3500) + 12 * 80;
  const int64_t per_node = (precision == BIOFEM_FP64 ? 3500 + 1400 : 2100) + (int64_t)(2 * m + 8) * 24 + 3450;
  *bytes = (per_elem * n_elmt + per_node * nt) * 5 / 4 + (8 << 20);
  return 0;
}

int ServeCreate(int64_t hbm_budget_bytes, int32_t max_slots, BiofemServe **out)
{
  if (!out || max_slots < 1 || hbm_budget_bytes <= 0) return 62;
  int rc = InitGpuWorkspace();
  if (rc) return rc;
  BiofemServe_ *E = new BiofemServe_();
  E->budget = hbm_budget_bytes;
  E->max_slots = max_slots;
  cudaGetDevice(&E->device);
  for (int i = 0; i < max_slots; i++) E->workers.emplace_back(worker_main, E);
  *out = E;
  return 0;
}

int ServeSubmit(BiofemServe *E, const BiofemMeshDesc *d, const BiofemParams *prm, const BiofemNewtonOptions *opt,
                const double *x0, int64_t *ticket)
{
  if (!E || !d || !prm || !x0 || !ticket) return 85;
  ServeReq *r = new ServeReq();
  int ng = 0;
  for (int e = 0; e < d->n_edge; e++) ng += d->n_bnodes[e];
  const size_t ndof = 3 * (size_t)(d->n_v + ng);
  r->tri.assign(d->tri, d->tri + 3 * (size_t)d->n_elmt);
  r->xyz.assign(d->xyz0, d->xyz0 + 3 * (size_t)d->n_v);
  r->nb.assign(d->n_bnodes, d->n_bnodes + d->n_edge);
  r->bn.assign(d->bnodes, d->bnodes + ng);
  r->fib.assign(d->n_fib, d->n_fib + 3 * (size_t)d->n_elmt);
  r->gs.assign(d->gamma_scale, d->gamma_scale + d->n_elmt);
  r->x.assign(x0, x0 + ndof);
  r->desc = *d;
  r->desc.tri = r->tri.data(); r->desc.xyz0 = r->xyz.data(); r->desc.n_bnodes = r->nb.data();
  r->desc.bnodes = r->bn.data(); r->desc.n_fib = r->fib.data(); r->desc.gamma_scale = r->gs.data();
  r->prm = *prm;
  if (opt) r->opt = *opt; else BiofemNewtonDefaults(&r->opt);
  BiofemServeEstimateBytes(d->n_v, d->n_elmt, ng, prm->precision, r->opt.gmres_restart, &r->est);
  std::lock_guard<std::mutex> lk(E->mu);
  if (r->est > E->budget) { delete r; return 55; }   /* PETSC_ERR_MEM: can never be admitted */
  r->ticket = E->next_ticket++;
  r->t_submit = now_s(E->t0);
  E->reqs[r->ticket] = r;
  E->queue.push_back(r);
  *ticket = r->ticket;
  E->cv.notify_all();
  return 0;
}

/* Wait for a request; x_out receives the converged x (n_dof entries).
   times: submit, start (admission) and finish, seconds since ServeCreate. */
int ServeWait(BiofemServe *E, int64_t ticket, double *x_out, BiofemNewtonStats *st, double times[3])
{
  if (!E) return 85;
  ServeReq *r = nullptr;
  {
    std::unique_lock<std::mutex> lk(E->mu);
    auto it = E->reqs.find(ticket);
    if (it == E->reqs.end()) return 63;
    r = it->second;
    E->cv_done.wait(lk, [&] { return r->done; });
    E->reqs.erase(it);
  }
  if (x_out) std::copy(r->x.begin(), r->x.end(), x_out);
  if (st) *st = r->st;
  if (times) { times[0] = r->t_submit; times[1] = r->t_start; times[2] = r->t_done; }
  const int rc = r->rc;
  const std::string err = r->err;
  delete r;
  return rc ? biofem::noalloc_fail(rc, "served request: " + err) : 0;
}

int ServeStatsGet(BiofemServe *E, int64_t out[6])
{
  if (!E || !out) return 85;
  std::lock_guard<std::mutex> lk(E->mu);
  out[0] = E->in_use; out[1] = E->peak_in_use; out[2] = E->active; out[3] = E->peak_active;
  out[4] = (int64_t)E->queue.size(); out[5] = E->completed;
  return 0;
}

int ServeDestroy(BiofemServe *E)
{
  if (!E) return 0;
  {
    std::lock_guard<std::mutex> lk(E->mu);
    E->stop = true;
  }
  E->cv.notify_all();
  for (std::thread &t : E->workers) t.join();
  for (auto &kv : E->reqs) delete kv.second;
  delete E;
  return 0;
}

} /* extern "C" */
