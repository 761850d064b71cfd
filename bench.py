#!/usr/bin/env python
"""Benchmark of the element residual + tangent + assembly path ("K+R assembly").

One step = one evaluation of R(x) and K(x) = dR/dx of the whole mesh,
assembled into the global vector and the 3x3-block CSR tangent, through the
C-ABI (libbiofem_gpu.so).  Default workload: the 256x192-cell flat membrane
(98,304 triangles, 3 thickness points, 3 C33 sub-iterations, follower
pressure, clamped boundary ring), FP64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  --impl reference times the reference's CPU
algorithm (the restated oracle, oracle/oracle.cpp: the reference's element
code with its tangent taken exactly by forward-mode dual numbers) on the
host's cores for a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "biofem-ia_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "K+R assembly elems/s & %HBM; served load-steps/s, p50/p99; FP32 vs FP64"
# dram__bytes_read.sum + dram__bytes_write.sum per launch on the 256x192
# workload, from one ncu capture of each kernel (profiles/, bytes)
DRAM_BYTES_C2 = {"elem_residual": 60.582e6 + 193.670e6, "elem_tangent": 241.039e6 + 160.028e6,
                 "row_assemble": 289.613e6 + 106.150e6, "elem_residual_ff": 59.955e6 + 2.915e6,
                 "elem_tangent_fp32": 36.505e6 + 33.795e6, "row_assemble_fp32": 195.243e6 + 48.489e6}
# sm__pipe_fp64_cycles_active (fraction of peak sustained active) per kernel
# in the same captures
FP64_PIPE_ACTIVE_C2 = {"elem_residual": 0.884, "elem_tangent": 0.893, "row_assemble": 0.937}
# FP64 FMA throughput of this GB300, measured by the DFMA loop of the FP64 pipe
# probe (biofem-ia_gb300/csrc/probe_fp64.cu): TFLOP/s
FP64_DFMA_TFLOPS = 1.057
KERNELS_FP64 = ["positions", "elem_residual", "elem_tangent", "node_gather", "row_assemble", "scale"]
KERNELS_FP32 = ["positions", "elem_residual_ff", "elem_tangent_fp32", "node_gather", "row_assemble_fp32", "scale"]
UNIT = "elems/s"
L2_FLUSH_BYTES = 256 << 20
CPU_SAMPLE_ELEMS = 2048
REF_SAMPLE_ELEMS = 2048


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="C2_flat_256x192")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solve", action="store_true", help="skip the Newton and serving measurements")
    ap.add_argument("--no-c3", action="store_true", help="skip the C3 (1024x768) and C4 (ellipsoid) measurements")
    ap.add_argument("--serve-requests", type=int, default=512)
    return ap.parse_args()


def workload(name):
    from biofem import configs
    return configs.ALL[name]


def algorithmic_bytes(info, topo, nnzb):
    """Canonical algorithmic bytes of one R+K evaluation (FP64 K values):
    4*sum(nen) patch ids + 2*24*(N_v+N_g) for x and X + 32*N_e fibre and
    activation + 24*N_v residual + 72*nnzb tangent values."""
    nen = np.where(topo["ire"] == 0, 12, topo["val"] + 6)
    nt = info.n_v + info.n_ghosts
    return int(4 * nen.sum() + 48 * nt + 32 * info.n_elmt + 24 * info.n_v + 72 * nnzb)


def canonical_flops(n_elmt, n_qp):
    """F_alg = q [2(3*3*m + m*m*3) + 2*m*3] per element, m = 36."""
    m = 36
    return n_elmt * n_qp * (2 * (9 * m + m * m * 3) + 2 * m * 3)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        smax = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[4 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_oracle(w, mesh):
    """The oracle set up on `mesh` by the reference's own table builders
    (GlobalGhostInit, IrrVer, Patch restated; corner-incident scans, the same
    tables as the reference's full scans) -- no GPU library involved."""
    from oracle.pyoracle import Oracle
    from biofem import configs
    o = Oracle().set_fast_topology(True)
    try:
        o.setup(mesh, w, configs.MU, configs.BULK, configs.H0)
    finally:
        o.set_fast_topology(False)
    return o


def cpu_rk(o, n_elmt, x_full, n_elems, threads, steps=1, warmup=0, residual_only=False):
    """The reference's element algorithm on the host (oracle `o`): R and the
    element tangents (or, with residual_only, R alone) of a bounded window of
    n_elems consecutive elements; each step takes the next window, spread over
    the mesh.  Returns (elems/s, seconds, n_elems)."""
    x = np.ascontiguousarray(x_full)
    chk = ctypes.c_double()
    n_elems = min(n_elems, n_elmt)
    span = max(1, n_elmt - n_elems + 1)
    fn = o.lib.oracle_r_sample if residual_only else o.lib.oracle_rk_sample
    times = []
    for s in range(warmup + steps):
        e0 = (n_elmt // 2 + s * 7919 * n_elems) % span
        t0 = time.perf_counter()
        rc = fn(x.ctypes.data_as(ctypes.c_void_p), e0, e0 + n_elems, threads, ctypes.byref(chk))
        dt = time.perf_counter() - t0
        if rc:
            raise RuntimeError(f"oracle element sample failed: {rc}")
        if s >= warmup:
            times.append(dt)
    return n_elems * len(times) / sum(times), sum(times), n_elems


def cpu_jfnk_step(threads):
    """One Newton step of the reference's own solver path (Jacobian-free
    Newton, unpreconditioned GMRES(30) on finite-difference J v) on C1, on
    the oracle residual with `threads` OpenMP threads: its wall time and how
    many residual evaluations it took."""
    from biofem import configs
    w = configs.C1
    mesh = w.build_mesh()
    o = cpu_oracle(w, mesh)
    o.set_threads(threads)
    x0 = w.initial_x(mesh, o.topology().xyz0_full)
    _, _, st = o.jfnk_newton_step(x0)
    return {"workload": f"{w.name} ({mesh.n_elmt} triangles), first Newton step from the reference state",
            "seconds": st["seconds"], "residual_evaluations": st["residual_evaluations"],
            "gmres_its": st["gmres_its"], "lin_converged": bool(st["lin_converged"]), "cores": threads,
            "kind": "port"}


def bench_config(w, mesh, world):
    """The workload description both arms print."""
    return {"workload": f"{w.name} R+K FP64: {mesh.n_elmt} triangles, {mesh.n_v} nodes, {mesh.n_ghosts} ghosts, "
                        f"{w.n_qp} thickness points, {w.c33_iters} C33 sub-iterations, P={w.pressure}, clamped ring",
            "l2": "GPU arm: flushed between timed steps (256 MiB device write outside the events)",
            "parallelism": f"replicas x{world}"}


SAMPLE_NOTE = ("reference element algorithm (oracle/oracle.cpp, bitwise equal to the reference build) + exact "
               "element tangent by Dual<48> forward mode, OpenMP over elements")


def cpu_baseline_block(w, mesh, o, x, threads, n_sample, steps=1, warmup=0):
    """cpu_baseline: R+K of a bounded element sample on all host threads, the
    residual alone (what the reference evaluates: its Newton is Jacobian-free)
    on all threads and on one, and one reference JFNK Newton step on C1."""
    val, tot, n = cpu_rk(o, mesh.n_elmt, x, n_sample, threads, steps=steps, warmup=warmup)
    cpu = {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{steps} x {n} consecutive elements of {w.name} (moving windows): {SAMPLE_NOTE}, {tot:.1f} s"}
    rval, rtot, rn = cpu_rk(o, mesh.n_elmt, x, 4 * n_sample, threads, residual_only=True)
    r1val, r1tot, r1n = cpu_rk(o, mesh.n_elmt, x, 4 * n_sample, 1, residual_only=True)
    cpu["residual_only"] = {"value": rval, "unit": UNIT, "cores": threads, "one_core_value": r1val,
                            "sample": f"{rn} elements on {threads} threads ({rtot:.2f} s), {r1n} on one "
                                      f"({r1tot:.2f} s): element forces only"}
    try:   # the reference's solver step, for scale beside the device Newton load step
        cpu["jfnk_newton_step"] = cpu_jfnk_step(threads)
    except Exception as exc:   # reported, never fatal to the line
        cpu["jfnk_newton_step"] = {"error": f"{type(exc).__name__}: {exc}"}
    return cpu


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest rank's time: every rank's timed region is reduced with MAX
    (replicas: no data exchange inside the timed region)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_rank: int, seconds: float) -> float:
    """Weak scaling: every rank processes its own copy of the workload, so the
    job rate is all ranks' units over the slowest rank's time."""
    return world * units_per_rank / seconds


def newton_bench(reps=3):
    """One quasi-static load step (Newton + multigrid-preconditioned device
    GMRES to ||R|| <= 1e-10 ||R0||) on C1 and C2, FP64 and FP32-bulk tangents;
    wall time of RunGpuNewtonSolve (host x in and out), best of reps."""
    from biofem import configs
    from biofem.gpu import GpuShell
    out = {}
    for w in (configs.C1, configs.C2):
        m = w.build_mesh()
        for prec, tag in ((0, "fp64"), (1, "fp32_bulk")):
            sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=prec)
            x0 = w.initial_x(m, sh.topology()["xyz0_full"])
            best, st = None, None
            for _ in range(reps):
                t0 = time.perf_counter()
                x, st = sh.newton(x0, rtol=1e-10)
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
            out[f"{w.name}_{tag}"] = {"ms": best * 1e3, "newton_its": st["newton_its"],
                                      "gmres_its": st["gmres_its_total"], "converged": st["converged"],
                                      "rel_residual": st["rfinal"] / st["r0"]}
            sh.close()
    return out


def dynamics_bench(steps=10):
    """The implicit time loop (main.c:420-573): per step the element activation
    gamma_e(t) (full sin^2 beat over the run, GammaOfTimeDelayed ramp 1, with a
    wavefront delay on C4), a Newton solve with the Newmark inertial and damping
    term in R and K (FDynamic), then xAccVel.  Wall time per step through the
    public calls (host x in and out), FP64 and FP32-bulk tangents."""
    from biofem import configs
    from biofem.dynamics import Activation, Dynamics, time_loop
    from biofem.gpu import GpuShell
    out = {}
    for w, dt in ((configs.C2, 1e-3), (configs.C4, 5e-3)):
        m = w.build_mesh()
        act = Activation(0.1, ramp_type=1)
        delay = None
        if "lv" in w.name:   # activation wavefront from the apex: delay proportional to height
            z = m.xyz0[m.tri].mean(axis=1)[:, 2]
            delay = 0.3 * steps * dt * (z - z.min()) / max(z.max() - z.min(), 1e-30)
        for prec, tag in ((0, "fp64"), (1, "fp32_bulk")):
            sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=prec)
            x0 = w.initial_x(m, sh.topology()["xyz0_full"])
            dyn = Dynamics(dt=dt, rho=1.0, newmark_gamma=0.5, dampfactor=5.0, damping=1)
            time_loop(sh, m, x0, dyn, act, 2, delay=delay, rtol=1e-10, max_newton=30)   # warm-up
            t0 = time.perf_counter()
            x, rec = time_loop(sh, m, x0, dyn, act, steps, delay=delay, rtol=1e-10, max_newton=30)
            wall = time.perf_counter() - t0
            out[f"{w.name}_{tag}"] = {
                "ms_per_time_step": wall / steps * 1e3, "steps": steps, "dt": dt,
                "newton_its_mean": float(np.mean([r.stats.get("newton_its", 0) for r in rec])),
                "gmres_its_total": int(sum(r.stats.get("gmres_its_total", 0) for r in rec)),
                "all_converged": all(r.converged for r in rec),
                "max_displacement": float(np.abs((x - x0)[: 3 * m.n_v]).max())}
            sh.close()
    return out


def case_bench(w, steps=5, warmup=2):
    """One large workload: R+K time of the FP64 and FP32-bulk forms (device
    pointers, L2 flushed between steps), a warm Newton load step with each,
    and their agreement (K Frobenius error, residual identity, displacement).
    C3: 1024x768 cells, 1,572,864 triangles, 6 thickness points, random fibre
    angle and lambda_a, exact basis tables and tangential thickness metric
    (extensions that keep this resolution well posed).  C4: the ~200k-triangle
    truncated ellipsoid with isolated valence-5/7 vertices, helix fibres,
    internal pressure, reference tables."""
    import torch
    from biofem import configs
    from biofem.gpu import GpuShell, BIOFEM_FP64, BIOFEM_FP32_BULK
    m = w.build_mesh()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    out, keep = {}, {}
    for prec, tag, kt in ((BIOFEM_FP64, "fp64", torch.float64), (BIOFEM_FP32_BULK, "fp32_bulk", torch.float32)):
        t0 = time.perf_counter()
        sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=prec)
        prep = time.perf_counter() - t0
        n_irregular = int(sh.info.n_irregular)
        x0 = w.initial_x(m, sh.topology()["xyz0_full"])
        dx = torch.tensor(x0, device=dev)
        dR = torch.empty_like(dx)
        dK = torch.empty(9 * sh.nnzb, dtype=kt, device=dev)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = []
        with torch.cuda.stream(stream):
            for i in range(warmup + steps):
                flush.zero_()
                ev0.record(stream)
                sh.jacobian_device(dx.data_ptr(), dR.data_ptr(), dK.data_ptr(), sp)
                ev1.record(stream)
                ev1.synchronize()
                if i >= warmup:
                    ms.append(ev0.elapsed_time(ev1))
            sh.sync(sp)
        best = None
        for _ in range(2):
            t0 = time.perf_counter()
            x, st = sh.newton(x0, rtol=1e-10, max_newton=12, gmres_max_it=1000)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        out[tag] = {"rk_ms": min(ms), "rk_elems_per_s": m.n_elmt / (min(ms) * 1e-3), "prep_s": prep,
                    "newton_ms": best * 1e3, "newton_its": st["newton_its"], "gmres_its": st["gmres_its_total"],
                    "converged": st["converged"], "rel_residual": st["rfinal"] / st["r0"]}
        keep[tag] = (dK.double() if kt == torch.float32 else dK, dR.clone(), torch.tensor(x - x0, device=dev))
        sh.close()
        del dx, dR, dK
    K64, R64, u64 = keep["fp64"]
    K32, R32, u32 = keep["fp32_bulk"]
    out["K_frobenius_rel_err_fp32_vs_fp64"] = float(torch.linalg.norm(K32 - K64) / torch.linalg.norm(K64))
    out["R_rel_err_fp32_vs_fp64"] = float(torch.linalg.norm(R32 - R64) / torch.linalg.norm(R64))
    out["displacement_rel_err_fp32_vs_fp64"] = float(torch.linalg.norm(u32 - u64) / torch.linalg.norm(u64))
    out["workload"] = (f"{w.name}: {m.n_elmt} triangles, {m.n_v} nodes, {m.n_ghosts} ghosts, q={w.n_qp}, "
                       f"basis tables {'exact' if w.basis else 'reference'}, thickness metric "
                       f"{'n,alpha' if w.tnormal else 'reference'}")
    if w.basis or w.tnormal:
        out["formulation"] = ("builder formulation (exact tables, tangential thickness metric): the reference's "
                              "four-decimal tables and a3,alpha thickness metric are ill-posed at this h")
    else:
        out["formulation"] = "reference algebra (one-step subdivision tables on irregular patches)"
    out["irregular_elements"] = n_irregular
    del keep, K64, K32
    torch.cuda.empty_cache()
    return out


def serve_bench(n_req=512, slots=16, budget=40 << 30, load=0.8):
    """Load-step serving stream (C5): flat sheets with nx log-uniform in
    [16, 256], ny = round(0.75 nx), seeded smooth imperfection, lambda_a,
    fibre angle and pressure per request; 5 Newton iterations at most, each to
    ||R|| <= 1e-10 ||R0||.  Sequential plain FP64 solves (mesh preparation +
    load step, one after another) against the serving loop (continuous
    batching, FP32-bulk tangents) run to capacity and under Poisson arrivals
    at `load` x capacity."""
    from biofem import configs
    from biofem.gpu import GpuShell, Serve, BIOFEM_FP64, BIOFEM_FP32_BULK
    # at most 300 GMRES iterations per Newton step: a request whose sheet carries
    # no pre-tension (lambda_a near 1) has a near-singular tangent, and one such
    # request ran 20,000 iterations for 7 s, the makespan's whole tail
    newton = dict(max_newton=5, rtol=1e-10, forcing=1, gmres_max_it=300)
    reqs = []
    for i in range(n_req):
        w = configs.serve_request(i)
        m = w.build_mesh()
        h = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
        reqs.append((w, m, w.initial_x(m, h.topology()["xyz0_full"])))
        h.close()
    w, m, x0 = reqs[0]
    for prec in (BIOFEM_FP64, BIOFEM_FP32_BULK):         # warm-up
        sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=prec)
        sh.newton(x0, **newton)
        sh.close()
    t0 = time.perf_counter()
    seq = []
    for w, m, x0 in reqs:
        sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=BIOFEM_FP64)
        seq.append(sh.newton(x0, **newton))
        sh.close()
    seq_s = time.perf_counter() - t0

    def served(prec, arrivals=None):
        srv = Serve(budget, slots)
        t_start = time.perf_counter()
        tickets = []
        for k, (w, m, x0) in enumerate(reqs):
            if arrivals is not None:
                wait = arrivals[k] - (time.perf_counter() - t_start)
                if wait > 0:
                    time.sleep(wait)
            tickets.append(srv.submit(m, w, configs.MU, configs.BULK, configs.H0, x0, precision=prec, **newton))
        res = [srv.wait(t) for t in tickets]
        stats = srv.stats()
        srv.close()
        t_sub = np.array([r[2][0] for r in res])
        t_end = np.array([r[2][2] for r in res])
        return res, float(t_end.max() - t_sub.min()), t_end - t_sub, stats

    res32, span32, _, st32 = served(BIOFEM_FP32_BULK)
    cap32 = n_req / span32
    res64, span64, _, _ = served(BIOFEM_FP64)
    # the same stream with the GMRES cap lifted: how many requests converge
    # within the 5 Newton iterations when every linear solve may finish
    newton_capped = dict(newton)
    newton.update(gmres_max_it=20000)
    res_nc, span_nc, _, _ = served(BIOFEM_FP32_BULK)
    newton.clear()
    newton.update(newton_capped)
    rng = np.random.default_rng(20261203 + 5)
    arrivals = np.cumsum(rng.exponential(1.0 / (load * cap32), size=n_req))
    arrivals -= arrivals[0]
    resp, spanp, lat, stp = served(BIOFEM_FP32_BULK, arrivals)
    conv_seq = [s[1]["converged"] for s in seq]
    conv32 = [r[1]["converged"] for r in res32]
    conv64 = [r[1]["converged"] for r in res64]
    conv_nc = [r[1]["converged"] for r in res_nc]
    diffs = [np.linalg.norm(r[0] - s[0]) / max(np.linalg.norm(s[0] - q[2]), 1e-300)
             for r, s, q in zip(res32, seq, reqs) if r[1]["converged"] and s[1]["converged"]]
    same64 = all(np.array_equal(r[0], s[0]) for r, s in zip(res64, seq))
    rel_seq = np.array([s[1]["rfinal"] / s[1]["r0"] for s in seq])
    rel32 = np.array([r[1]["rfinal"] / r[1]["r0"] for r in res32])
    return {
        "requests": n_req, "slots": slots, "hbm_budget_gb": budget / 2**30,
        "mesh_sizes_nx": [q[0].nx for q in reqs],
        "newton": "at most 5 iterations to ||R|| <= 1e-10 ||R0||, multigrid-preconditioned device GMRES "
                  "(at most 300 iterations per step), Eisenstat-Walker forcing terms (both arms)",
        "sequential_fp64_load_steps_per_s": n_req / seq_s,
        "served_fp32_bulk_capacity_load_steps_per_s": cap32,
        "served_fp64_capacity_load_steps_per_s": n_req / span64,
        "speedup_served_fp32_vs_sequential_fp64": cap32 / (n_req / seq_s),
        "poisson": {"offered_load": load, "arrival_rate_per_s": load * cap32,
                    "throughput_load_steps_per_s": n_req / spanp,
                    "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                    "peak_active": stp["peak_active"]},
        "peak_hbm_bytes_admitted": st32["peak_in_use"], "peak_active_capacity_run": st32["peak_active"],
        "converged_sequential_fp64": int(sum(conv_seq)), "converged_served_fp32_bulk": int(sum(conv32)),
        "converged_load_steps_per_s": {"sequential_fp64": sum(conv_seq) / seq_s,
                                       "served_fp32_bulk": sum(conv32) / span32,
                                       "served_fp64": sum(conv64) / span64},
        "gmres_cap_lifted": {"converged_served_fp32_bulk": int(sum(conv_nc)), "makespan_s": span_nc,
                             "load_steps_per_s": n_req / span_nc,
                             "converged_load_steps_per_s": sum(conv_nc) / span_nc,
                             "note": "same stream and Newton limit (5 iterations), at most 20,000 GMRES "
                                     "iterations per step"},
        "final_rel_residual_p50_p90_sequential_fp64": [float(np.percentile(rel_seq, 50)), float(np.percentile(rel_seq, 90))],
        "final_rel_residual_p50_p90_served_fp32_bulk": [float(np.percentile(rel32, 50)), float(np.percentile(rel32, 90))],
        "max_rel_diff_fp32_served_vs_fp64_sequential_converged": float(max(diffs)) if diffs else None,
        "served_fp64_equals_sequential_fp64_bitwise": bool(same64),
    }


def reference_gpu_geometry(w, mesh, t, x, steps, warmup):
    """The reference's own GPU kernels (src/cuda_kernel.cu, unmodified, from
    oracle/_ref/ref_cuda_kernel.cubin) on this workload: SubdivGeomKernel_ on
    the current state and MetricTensorKernel_ over every thickness point, the
    geometry half of one residual evaluation (the reference computes stress,
    forces and assembly on the host)."""
    try:
        import torch
        from oracle import ref_cuda
        if not torch.cuda.is_available():
            return {"unavailable": "no GPU"}
        if not ref_cuda.available():
            return {"unavailable": "ref_cuda_kernel.cubin not built (reference sources absent at build time)"}
        k = ref_cuda.RefCudaKernels()
        theta = np.polynomial.legendre.leggauss(w.n_qp)[0]
        from biofem import configs
        b = k.prepare(mesh, t, x, t.xyz0_full.ravel(), w.n_qp, configs.H0, theta)
        r = k.time_geometry(b, steps=max(steps, 3), warmup=max(warmup, 3))
        if r["status_nonzero"] or r["metric_status_nonzero"]:
            return {"unavailable": f"reference kernels reported element errors: {r}"}
        r["elems_per_s"] = mesh.n_elmt / ((r["SubdivGeomKernel_ms"] + r["MetricTensorKernel_ms"]) * 1e-3)
        r["launch"] = "as LaunchCudaSubdivGeomKernelImpl / LaunchCudaMetricTensorKernelImpl: one 256-thread block " \
                      "per element; 256-thread blocks over element x thickness point; device-resident inputs, " \
                      "L2 flushed between steps"
        del b
        torch.cuda.empty_cache()
        return r
    except Exception as exc:   # reported, never fatal to the line
        return {"unavailable": f"{type(exc).__name__}: {exc}"}


def run_reference(args):
    """The reference's CPU implementation of the path on this host's cores:
    the oracle (a restatement of the reference's element algorithm, pinned
    bitwise to the reference build) set up by its own table builders, R and
    exact element tangents of a bounded element sample per step.  Loads no
    GPU library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    w = workload(args.workload)
    mesh = w.build_mesh()
    o = cpu_oracle(w, mesh)
    topo = o.topology()
    x = w.initial_x(mesh, topo.xyz0_full)
    # the GPU geometry first: the oracle library holds one mesh, and the JFNK
    # step of cpu_baseline_block sets it up again on C1
    gpu_geom = reference_gpu_geometry(w, mesh, topo, x, args.steps, args.warmup)
    threads = os.cpu_count() or 1
    cpu = cpu_baseline_block(w, mesh, o, x, threads, REF_SAMPLE_ELEMS, steps=args.steps, warmup=args.warmup)
    val = cpu["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * REF_SAMPLE_ELEMS / val,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded flat membrane, row-alternating diagonals)",
        "config": dict(bench_config(w, mesh, args.gpus), sample_elements_per_step=min(REF_SAMPLE_ELEMS, mesh.n_elmt)),
        "cpu_baseline": cpu,
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "ms_per_step is the time of one sample window; the rate is the reference algorithm's elements/s",
        "reference_gpu_geometry": gpu_geom,
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from biofem import configs
    from biofem.gpu import GpuShell, load_library
    load_library()
    w = workload(args.workload)
    mesh = w.build_mesh()
    sh = GpuShell(mesh, w, configs.MU, configs.BULK, configs.H0)
    topo = sh.topology()
    x_host = w.initial_x(mesh, topo["xyz0_full"])
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    dx = torch.tensor(x_host, device=dev)
    dR = torch.empty_like(dx)
    dK = torch.empty(9 * sh.nnzb, dtype=torch.float64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    n_launch_res, n_launch_jac = sh.launch_counts()

    def step():
        sh.jacobian_device(dx.data_ptr(), dR.data_ptr(), dK.data_ptr(), sp)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            step()
        sh.sync(sp)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        clocks = ClockSampler(local)
        clocks.start()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()                     # L2 flush between timed steps (outside the events)
            starts[i].record(stream)
            step()
            ends[i].record(stream)
        torch.cuda.synchronize()
        sh.sync(sp)
        clk = clocks.stop()
        ms_steps = [s.elapsed_time(e) for s, e in zip(starts, ends)]
        ms = max_over_ranks(sum(ms_steps) / args.steps, dist, dev)

        # per-kernel durations (separate pass; the library records events between launches)
        sh.kernel_timing(True)
        for _ in range(args.steps):
            flush.zero_()
            step()
        kms, calls = sh.kernel_times(n_launch_jac)
        sh.kernel_timing(False)
        kms = (kms / max(calls, 1)).tolist()

        # residual-only step for reference
        for _ in range(3):
            sh.residual_device(dx.data_ptr(), dR.data_ptr(), sp)
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r_ms = []
        for _ in range(args.steps):
            flush.zero_()
            r0.record(stream)
            sh.residual_device(dx.data_ptr(), dR.data_ptr(), sp)
            r1.record(stream)
            r1.synchronize()
            r_ms.append(r0.elapsed_time(r1))
        sh.sync(sp)

    # FP32-bulk form on the same workload: residual FP64, tangent FP32
    from biofem.gpu import BIOFEM_FP32_BULK
    s32 = GpuShell(mesh, w, configs.MU, configs.BULK, configs.H0, precision=BIOFEM_FP32_BULK)
    dK32 = torch.empty(9 * s32.nnzb, dtype=torch.float32, device=dev)
    dR32 = torch.empty_like(dx)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            s32.jacobian_device(dx.data_ptr(), dR32.data_ptr(), dK32.data_ptr(), sp)
        s32.sync(sp)
        f_ms = []
        for _ in range(args.steps):
            flush.zero_()
            r0.record(stream)
            s32.jacobian_device(dx.data_ptr(), dR32.data_ptr(), dK32.data_ptr(), sp)
            r1.record(stream)
            r1.synchronize()
            f_ms.append(r0.elapsed_time(r1))
        s32.sync(sp)
        s32.kernel_timing(True)
        n32 = s32.launch_counts()[1]
        for _ in range(args.steps):
            flush.zero_()
            s32.jacobian_device(dx.data_ptr(), dR32.data_ptr(), dK32.data_ptr(), sp)
        k32, c32 = s32.kernel_times(n32)
        s32.kernel_timing(False)
    torch.cuda.synchronize()
    K64h = dK.cpu().numpy()
    K32h = dK32.cpu().numpy().astype(np.float64)
    fp32_frob = float(np.linalg.norm(K32h - K64h) / np.linalg.norm(K64h))
    R64h = dR.cpu().numpy()
    fp32_rrel = float(np.linalg.norm(dR32.cpu().numpy() - R64h) / np.linalg.norm(R64h))
    f32_step = sum(f_ms) / len(f_ms)
    hx = torch.tensor(x_host).pin_memory()
    # the FP32-bulk form end to end through the public host call (FP32 K out);
    # a failure is reported in the line, and every rank still joins the max
    e32_local, e2e32 = float("nan"), None
    try:
        hR32 = torch.empty(s32.n_dof, dtype=torch.float64).pin_memory()
        hK32 = torch.empty(9 * s32.nnzb, dtype=torch.float32).pin_memory()
        for _ in range(2):
            s32.residual_jacobian_host_ptrs(hx.data_ptr(), hR32.data_ptr(), hK32.data_ptr())
        e32_t = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s32.residual_jacobian_host_ptrs(hx.data_ptr(), hR32.data_ptr(), hK32.data_ptr())
            e32_t.append(time.perf_counter() - t0)
        e32_local = sum(e32_t) / len(e32_t)
        k32_same = bool(np.array_equal(hK32.numpy(), dK32.cpu().numpy()))
    except Exception as exc:
        e2e32 = {"error": f"{type(exc).__name__}: {exc}"}
    e32_s = max_over_ranks(e32_local, dist, dev)
    if e2e32 is None:
        e2e32 = {"value": whole_job_rate(world, mesh.n_elmt, e32_s), "unit": UNIT, "h2d_bytes_per_step": 8 * s32.n_dof,
                 "d2h_bytes_per_step": 8 * s32.n_dof + 36 * s32.nnzb, "K_equals_device_call": k32_same}
    s32.close()

    # end to end through the public host API: pinned x in, R and K out
    hR = torch.empty(sh.n_dof, dtype=torch.float64).pin_memory()
    hK = torch.empty(9 * sh.nnzb, dtype=torch.float64).pin_memory()
    for _ in range(2):
        sh.residual_jacobian_host_ptrs(hx.data_ptr(), hR.data_ptr(), hK.data_ptr())
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sh.residual_jacobian_host_ptrs(hx.data_ptr(), hR.data_ptr(), hK.data_ptr())
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(sum(e2e_t) / len(e2e_t), dist, dev)
    # consistency: the host call returns the same R as the device call
    Rdev = dR.cpu().numpy()
    sh.residual_host_ptrs(hx.data_ptr(), hR.data_ptr())
    same = bool(np.array_equal(Rdev, hR.numpy()))

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    newton = newton_bench() if not args.no_solve else None
    from biofem import configs as _cfg
    c3 = case_bench(_cfg.C3) if not args.no_c3 else None
    c4 = case_bench(_cfg.C4) if not args.no_c3 else None
    serving = serve_bench(n_req=args.serve_requests) if not args.no_solve else None
    dynamics = dynamics_bench() if not args.no_solve else None

    info = sh.info
    ne = info.n_elmt
    value = whole_job_rate(world, ne, ms * 1e-3)
    b_alg = algorithmic_bytes(info, topo, sh.nnzb)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    step_gbs = b_alg / (ms * 1e-3) / 1e9
    dom = int(np.argmax(kms))
    dom_name = KERNELS_FP64[dom]
    kern_gbs = b_alg / (kms[dom] * 1e-3) / 1e9
    f_alg = canonical_flops(ne, w.n_qp)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline_block(w, mesh, cpu_oracle(w, mesh), x_host, os.cpu_count() or 1, CPU_SAMPLE_ELEMS)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded flat membrane, row-alternating diagonals)",
        "config": dict(bench_config(w, mesh, world),
                       tangent={"format": "3x3-block CSR, row-major blocks, FP64 values", "nnzb": sh.nnzb}),
        "roofline": {"bound": "hbm", "kernel": f"k_{dom_name}", "achieved": kern_gbs, "peak": hbm_peak,
                     "unit": "GB/s", "frac": kern_gbs / hbm_peak, "traffic": DRAM_BYTES_C2.get(dom_name),
                     "peak_source": peak_src, "step_achieved_gbs": step_gbs,
                     "note": "of measured HBM copy bandwidth; achieved = canonical algorithmic bytes of one R+K "
                             "evaluation (patch ids, x and X, fibre and activation, R, K values once) / the dominant "
                             "kernel's live launch time (CUDA events on the launch stream); traffic = dram read + "
                             "write of one launch of that kernel on C2 from an ncu capture; the step is FP64-pipe "
                             "bound, see compute_roofline"},
        "compute_roofline": {"kernel": "whole R+K step", "bound": "fp64", "step_ms": ms,
                             "canonical_flops_per_step": f_alg,
                             "achieved_tflops_canonical": f_alg / (ms * 1e-3) / 1e12,
                             "peak_tflops": FP64_DFMA_TFLOPS,
                             "frac": f_alg / (ms * 1e-3) / 1e12 / FP64_DFMA_TFLOPS,
                             "peak_source": "measured DFMA loop on this GB300 (FP64 pipe probe)",
                             "fp64_pipe_active_frac": FP64_PIPE_ACTIVE_C2,
                             "note": "canonical F_alg (the B^T D B contraction at every thickness point) over the "
                                     "whole step time; the contraction itself runs in k_row_assemble on the 15 "
                                     "generalised coordinates (about 18.4 kflop per element, against 25.9 kflop "
                                     "canonical at q = 3); fp64_pipe_active_frac is sm__pipe_fp64_cycles_active per "
                                     "kernel on C2 (ncu)"},
        "kernels_ms": dict(zip(KERNELS_FP64, kms)),
        "residual_only": {"ms_per_step": sum(r_ms) / len(r_ms), "elems_per_s": ne / (sum(r_ms) / len(r_ms) * 1e-3)},
        "e2e": {"value": whole_job_rate(world, ne, e2e_s), "unit": UNIT, "h2d_bytes_per_step": 8 * sh.n_dof,
                "d2h_bytes_per_step": 8 * sh.n_dof + 72 * sh.nnzb, "host_equals_device_R": same},
        "fp32_bulk": {"ms_per_step": f32_step, "elems_per_s": world * ne / (f32_step * 1e-3),
                      "speedup_vs_fp64": ms / f32_step,
                      "K_frobenius_rel_err_vs_fp64": fp32_frob, "R_rel_err_vs_fp64": fp32_rrel,
                      "kernels_ms": dict(zip(KERNELS_FP32, (k32 / max(c32, 1)).tolist())),
                      "roofline_hbm_frac": (b_alg - 36 * sh.nnzb) / (f32_step * 1e-3) / 1e9 / hbm_peak,
                      "dominant_kernel": KERNELS_FP32[int(np.argmax(k32))],
                      "dominant_kernel_traffic": DRAM_BYTES_C2.get(KERNELS_FP32[int(np.argmax(k32))]),
                      "e2e": e2e32,
                      "note": "residual in float-float arithmetic on the FP32 pipe (about 48 bits), node sums FP64; "
                              "tangent FP32 on patch-local shifted coordinates; K values FP32"},
        "gpu_launches": n_launch_jac * args.steps,
        "clocks": clk,
    }
    if newton:
        line["newton_load_step"] = newton
    if serving:
        line["serving"] = serving
    if dynamics:
        line["dynamics"] = dynamics
    if c3:
        line["C3"] = c3
    if c4:
        line["C4"] = c4
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
