"""The reference's own GPU kernels, run unmodified (TEST INFRASTRUCTURE ONLY).

oracle/build_ref.py compiles the reference's src/cuda_kernel.cu for sm_103a
into oracle/_ref/ref_cuda_kernel.cubin (device code only, so it loads on any
host).  This module loads that cubin through the CUDA driver API (ctypes on
libcuda), finds SubdivGeomKernel_ and MetricTensorKernel_ by name, and
launches them exactly as the reference's LaunchCudaSubdivGeomKernelImpl /
LaunchCudaMetricTensorKernelImpl do (src/cuda_kernel.cu:1032-1196): one
256-thread block per element for the subdivision geometry, 256-thread blocks
over element x thickness point for the metric tensors.  Device buffers and
events come from torch (its primary context is the one current here).

Used by bench.py --impl reference (the reference's GPU geometry timed on the
same GPU) and by tests/test_reference_gpu_kernels.py (its output checked
against the oracle's element geometry).  PetscInt is int32 in the petsc-lite
build the cubin is compiled against.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "ref_cuda_kernel.cubin"
GEOM_STRIDE = 24          # kCudaGeomStride_
IRREGULAR_STRIDE = 80     # kCudaIrregularStride_ = 5 x patch width 16
BASIS_STRIDE = 18         # kCudaBasisStride_
METRIC_STRIDE = 18        # kCudaMetricStride_
GEOM_THREADS = 256        # kCudaGeomThreadsPerElement_
MAX_PATCH = 16


def available() -> bool:
    return CUBIN.is_file()


class RefCudaKernels:
    def __init__(self, cubin: Path = CUBIN):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")          # make the primary context current
        self.cu = ctypes.CDLL("libcuda.so.1")
        cu = self.cu
        ctx = ctypes.c_void_p()
        self._check(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self._image = cubin.read_bytes()
        self.mod = ctypes.c_void_p()
        self._check(cu.cuModuleLoadData(ctypes.byref(self.mod), ctypes.c_char_p(self._image)), "cuModuleLoadData")
        count = ctypes.c_uint()
        self._check(cu.cuModuleGetFunctionCount(ctypes.byref(count), self.mod), "cuModuleGetFunctionCount")
        funcs = (ctypes.c_void_p * count.value)()
        self._check(cu.cuModuleEnumerateFunctions(funcs, count, self.mod), "cuModuleEnumerateFunctions")
        self.funcs = {}
        for f in funcs:
            name = ctypes.c_char_p()
            self._check(cu.cuFuncGetName(ctypes.byref(name), ctypes.c_void_p(f)), "cuFuncGetName")
            self.funcs[name.value.decode()] = ctypes.c_void_p(f)
        self.subdiv = self._find("SubdivGeomKernel_")
        self.metric = self._find("MetricTensorKernel_")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def _find(self, stem):
        hits = [f for n, f in self.funcs.items() if stem in n]
        if len(hits) != 1:
            raise RuntimeError(f"{stem}: {len(hits)} matches among {sorted(self.funcs)}")
        return hits[0]

    def _launch(self, f, grid, block, args, stream):
        vals = []
        for a in args:
            if isinstance(a, float):
                vals.append(ctypes.c_double(a))
            elif isinstance(a, int):
                vals.append(ctypes.c_int(a))
            else:                                  # a torch tensor: its device pointer
                vals.append(ctypes.c_void_p(a.data_ptr()))
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        self._check(self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, ctypes.c_void_p(stream), params, None),
                    "cuLaunchKernel")

    # -- inputs -------------------------------------------------------------
    @staticmethod
    def node_coordinates(mesh, topo, x):
        """xb, yb, zb over real and ghost nodes for the iterate x (3 per node):
        ghost g = x_nv2 + x_nv1 - x_nv3 along each boundary ring (GlobalGhost,
        bending.c:1763-1814)."""
        nv = mesh.n_v
        ng = int(np.asarray(mesh.n_bnodes).sum())
        p = np.array(x[: 3 * (nv + ng)], dtype=np.float64).reshape(-1, 3)
        bn = np.asarray(mesh.bnodes)
        count, start = 0, 0
        for n_local in np.asarray(mesh.n_bnodes):
            for li in range(n_local):
                nv1, nv2 = bn[start + (li + 1) % n_local], bn[start + li]
                p[nv + count] = p[nv2] + p[nv1] - p[topo.ghost_nv3[count]]
                count += 1
            start += n_local
        return np.ascontiguousarray(p.T)

    def prepare(self, mesh, topo, x_cur, x_ref, n_qp, h0, theta):
        """Device buffers for one mesh: the subdivision inputs of the current
        and reference states and every output array, sized as the reference's
        Launch*Impl functions size them."""
        import torch
        dev = torch.device("cuda")
        ne = mesh.n_elmt
        patch = np.asarray(topo.patch, dtype=np.int32).reshape(ne, MAX_PATCH)
        nen = np.where(np.asarray(topo.ire) == 0, 12, np.asarray(topo.val) + 6)
        ntot = mesh.n_v + int(np.asarray(mesh.n_bnodes).sum())
        # every node the kernel reads (slots < nen) is a real or ghost node
        used = np.arange(MAX_PATCH)[None, :] < nen[:, None]
        if nen.max() > MAX_PATCH or patch[used].min() < 0 or patch[used].max() >= ntot:
            raise ValueError("patch outside the node arrays")
        if not np.isin(np.asarray(topo.ire), (0, 1)).all():
            raise ValueError("ire must be 0 or 1")
        t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
        b = {"ne": ne, "nq": n_qp, "h0": float(h0)}
        b["ire"] = t(topo.ire, torch.int32)
        b["val"] = t(topo.val, torch.int32)
        b["patch"] = t(patch.ravel(), torch.int32)
        for tag, x in (("cur", x_cur), ("ref", x_ref)):
            c = self.node_coordinates(mesh, topo, x)
            b[f"xyz_{tag}"] = [t(c[k], torch.float64) for k in range(3)]
            b[f"geom_{tag}"] = torch.zeros(GEOM_STRIDE * ne, dtype=torch.float64, device=dev)
        b["meta"] = torch.zeros(3 * ne, dtype=torch.int32, device=dev)
        b["status"] = torch.zeros(ne, dtype=torch.int32, device=dev)
        b["irregular"] = torch.zeros(IRREGULAR_STRIDE * ne, dtype=torch.float64, device=dev)
        b["theta"] = t(theta, torch.float64)
        nq = ne * n_qp
        b["mstatus"] = torch.zeros(nq, dtype=torch.int32, device=dev)
        for k in ("basis_cur", "basis_ref", "metric_cur", "metric_ref"):
            b[k] = torch.zeros(BASIS_STRIDE * nq, dtype=torch.float64, device=dev)
        return b

    # -- launches -----------------------------------------------------------
    def subdiv_geom(self, b, tag, stream):
        x, y, z = b[f"xyz_{tag}"]
        self._launch(self.subdiv, b["ne"], GEOM_THREADS,
                     [b["ne"], b["ire"], b["val"], b["patch"], x, y, z, b["meta"], b["status"], b[f"geom_{tag}"],
                      b["irregular"]], stream)

    def metric_tensor(self, b, stream):
        total = b["ne"] * b["nq"]
        self._launch(self.metric, (total + 255) // 256, 256,
                     [b["ne"], b["nq"], b["h0"], b["theta"], b["geom_cur"], b["geom_ref"], b["mstatus"],
                      b["basis_cur"], b["basis_ref"], b["metric_cur"], b["metric_ref"]], stream)

    def time_geometry(self, b, steps=10, warmup=3, flush_bytes=256 << 20):
        """Device time of the reference's GPU geometry of one residual
        evaluation: SubdivGeomKernel_ on the current state and
        MetricTensorKernel_ on current + reference geometry (the reference
        geometry is computed once beforehand, as the reference keeps geom0).
        L2 flushed between steps outside the events.  Returns ms per kernel
        (mean over steps)."""
        import torch
        s = torch.cuda.current_stream()
        sp = s.cuda_stream
        flush = torch.empty(flush_bytes, dtype=torch.uint8, device="cuda")
        self.subdiv_geom(b, "ref", sp)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        t_geom, t_metric = [], []
        for i in range(warmup + steps):
            flush.zero_()
            ev[0].record(s)
            self.subdiv_geom(b, "cur", sp)
            ev[1].record(s)
            self.metric_tensor(b, sp)
            ev[2].record(s)
            ev[2].synchronize()
            if i >= warmup:
                t_geom.append(ev[0].elapsed_time(ev[1]))
                t_metric.append(ev[1].elapsed_time(ev[2]))
        torch.cuda.synchronize()
        return {"SubdivGeomKernel_ms": float(np.mean(t_geom)), "MetricTensorKernel_ms": float(np.mean(t_metric)),
                "status_nonzero": int((b["status"] != 0).sum().item()),
                "metric_status_nonzero": int((b["mstatus"] != 0).sum().item())}
