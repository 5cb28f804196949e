"""Benchmark: continuous FE Laplacian matvec on the deformed 64^3 mesh.

Workload (the metric's configuration): 64x64x64 hexahedral cells on [0,1]^3
mapped by x_i <- x_i + 0.05 sin(2 pi x_j) sin(2 pi x_k), Gauss quadrature
with n = p+1 points, precomputed merged 6-entry geometry per quadrature point,
homogeneous Dirichlet boundary, input uniform[-1,1].  Headline: degree 4,
FP32 operator.  The JSON line also carries the degree 2..8 sweep in FP32 and
FP64, each apply with its relative error against the FP64 CPU oracle on the
same mesh and vector, and the FP32-inner / FP64-refined CG against the plain
FP64 CG on the same operator.

One step = one operator apply y = A x with x and the geometry resident in
HBM (the working set, 0.9 GB at p=4 FP32, exceeds the 129 MB L2, so no
explicit flush).  e2e = the same apply through the C ABI with the input
copied from pinned host memory and the result copied back every step (steps
pipelined on three streams with double-buffered device vectors).

CPU leg (``cpu_baseline``, and the whole of ``--impl reference``): the FP64
oracle port of the reference's cell algorithm (gather -> even-odd sum
factorisation -> scatter), built -O3 for the host CPU with OpenMP over all
host threads, timed on the full workload.  The same leg uses the oracle's
strict build (-O2, no floating-point contraction) to state the error of every
GPU apply of the sweep.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Laplacian matvec GDoF/s + % HBM peak, FP32 vs FP64 at stated rel. error"
# DRAM bytes (read + write) of one apply = 8 colour launches of the default
# workload, measured by ncu with warm caches as in the timed loop
# (--metrics dram__bytes_read.sum,dram__bytes_write.sum --cache-control none
#  -k regex:line_vmult -s 24 -c 8 on this script with --steps 5 --warmup 3).
MEASURED_TRAFFIC = {(4, 64): 985454848}
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum summed over the 8 colour launches "
                  "of one apply, caches warm (--cache-control none)")
UNIT = "GDoF/s"
DEFORM = 0.05
CPU_REPEATS = 5          # the CPU baseline reports the best of this many applies


def algorithmic_bytes(p, n_dofs, n_cells, s):
    """x read once, y written once, 6 geometry entries per quadrature point
    (node indices are computed, not stored)"""
    return 2 * s * n_dofs + 6 * s * (p + 1) ** 3 * n_cells


def workload_config(p, ncells):
    """the workload keys both arms report, identical in both (the continuous
    node count includes the Dirichlet boundary nodes)"""
    return {"workload": "continuous Laplacian matvec, deformed %d^3 hex mesh, p=%d" % (ncells, p),
            "degree": p, "n_cells": [ncells] * 3, "n_dofs": (p * ncells + 1) ** 3, "deform": DEFORM,
            "geometry": "merged 6-entry JxW J^-1 J^-T per Gauss point, precomputed",
            "dirichlet": True}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def host_cpu():
    model = platform.processor() or platform.machine()
    try:
        import subprocess
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name:"):
                return {"machine": platform.machine(), "model": line.split(":", 1)[1].strip(),
                        "nproc": os.cpu_count()}
    except (OSError, ValueError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu part", "hardware"):
                    model = line.split(":", 1)[1].strip()
                    if key == "model name":
                        break
    except OSError:
        pass
    return {"machine": platform.machine(), "model": model, "nproc": os.cpu_count()}


class ClockSampler:
    """SM clock and throttle reasons sampled during the timed region through
    NVML (libnvidia-ml, read-only queries) every 2 ms in a thread."""

    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap"}

    def __init__(self, gpu_index=0):
        import ctypes
        import threading
        self.samples, self.reasons, self.max_mhz = [], set(), None
        self.stop_evt = threading.Event()
        self.thread = None
        self.nvml = None
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return
            h = ctypes.c_void_p()
            if nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(gpu_index), ctypes.byref(h)) != 0:
                return
            mx = ctypes.c_uint()
            if nv.nvmlDeviceGetMaxClockInfo(h, ctypes.c_int(1), ctypes.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            fn = None
            for name in ("nvmlDeviceGetCurrentClocksEventReasons",
                         "nvmlDeviceGetCurrentClocksThrottleReasons"):
                try:
                    fn = getattr(nv, name)
                    break
                except AttributeError:
                    continue
            self.reason_fn = fn
            self.nvml, self.h = nv, h
        except OSError:
            self.nvml = None

    def _sample(self):
        import ctypes
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        if self.nvml.nvmlDeviceGetClockInfo(self.h, ctypes.c_int(1), ctypes.byref(clk)) == 0:
            self.samples.append(float(clk.value))
        if self.reason_fn is not None and self.reason_fn(self.h, ctypes.byref(rs)) == 0:
            for bit, name in self.REASONS.items():
                if rs.value & bit:
                    self.reasons.add(name)

    def _run(self):
        # every 0.5 ms: the headline's timed region lasts a few milliseconds
        while not self.stop_evt.is_set():
            self._sample()
            self.stop_evt.wait(0.0005)

    def sample_now(self):
        """one sample from the calling thread (while queued work runs)"""
        if self.nvml is not None:
            self._sample()

    def start(self):
        import threading
        if self.nvml is not None:
            self.thread = threading.Thread(target=self._run, daemon=True)
            self.thread.start()

    def stop(self):
        if self.thread is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvml unavailable"]}
        self.stop_evt.set()
        self.thread.join()
        return {"sm_mhz": statistics.median(self.samples) if self.samples else None,
                "sm_max_mhz": self.max_mhz, "reasons": sorted(self.reasons),
                "samples": len(self.samples)}


def dist_setup(n_gpus, backend="nccl"):
    """one process per GPU (torchrun environment); the replicas share no data,
    the process group only carries the barrier and the max over ranks"""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def check_status(op, what):
    """a bounded wait inside a kernel that timed out invalidates the applies
    it belongs to: the run fails instead of reporting them"""
    s = op.device_status()
    if s != 0:
        raise SystemExit("device status %d after %s: results invalid" % (s, what))


# --------------------------------------------------------------------------
# CPU leg: the oracle port timed on the host cores (cpu_baseline and the
# reference arm), and the oracle's strict build stating the GPU's errors
# --------------------------------------------------------------------------
def perf_build_flags():
    """the gcc flags of the timed oracle build (recorded when it was built)"""
    from oracle import build as obuild
    return obuild.perf_build_flags()


def _cpu_env():
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")


def cpu_cont_setup(p, ncells):
    """mesh, precomputed geometry and input of the continuous workload for
    the timed port (the geometry precomputed as on the GPU)"""
    import numpy as np

    _cpu_env()
    from oracle import oracle as O

    m = O.mesh(p, (ncells,) * 3, deform=DEFORM)
    G = O.cont_geometry(m)
    x = np.random.default_rng(20241203).uniform(-1, 1, O.cont_n_dofs(m))
    return O, m, G, x


def cpu_time_best(fn, repeats):
    ts = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return min(ts), ts


def cpu_cont_baseline(p, ncells, repeats=CPU_REPEATS):
    """best of `repeats` full applies of the port on the whole workload"""
    import numpy as np

    O, m, G, x = cpu_cont_setup(p, ncells)
    L = O.perf_lib()
    threads = os.cpu_count() or 1
    y = np.empty_like(x)
    O.cont_apply(m, G, x, n_threads=threads, y=y, L=L)  # warm-up (page-in, thread pool)
    best, ts = cpu_time_best(lambda: O.cont_apply(m, G, x, n_threads=threads, y=y, L=L), repeats)
    n = O.cont_n_dofs(m)
    return {"value": round(n / best / 1e9, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "the full %d^3 deformed p=%d workload (%d DoFs), FP64, precomputed geometry, best of %d "
                      "applies (%s s)" % (ncells, p, n, repeats, ", ".join("%.3f" % t for t in ts)),
            "build": "gcc " + perf_build_flags() + ", OMP_PROC_BIND=close",
            "host": host_cpu()}


def cpu_check_sweep(sweep, ncells):
    """relative error of every sweep apply against the FP64 oracle (strict
    build) on the same mesh and vector; geometry computed per cell"""
    import numpy as np

    _cpu_env()
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    for ent in sweep:
        host = ent.pop("_host", None)
        if host is None:
            continue
        x, y64, y32 = host
        m = O.mesh(ent["degree"], (ncells,) * 3, deform=DEFORM)
        yo = O.cont_apply(m, None, x, n_threads=threads)
        nrm = float(np.linalg.norm(yo))
        ent["fp64_rel_err_vs_oracle"] = float("%.3g" % (np.linalg.norm(y64 - yo) / nrm))
        ent["fp32_rel_err_vs_oracle"] = float("%.3g" % (np.linalg.norm(y32.astype(np.float64) - yo) / nrm))
        del yo, host


def cpu_dg_baselines(configs):
    """the port's DG SIPG apply (config 3) and DG advection apply (config 5)
    on the full 48^3 meshes, best of CPU_REPEATS, beside the GPU numbers"""
    import numpy as np

    _cpu_env()
    from oracle import oracle as O

    L = O.perf_lib()
    threads = os.cpu_count() or 1
    out = {}
    h = 1.0 / 48
    g = O.dg(5, (48, 48, 48), (h, h, h), penalty=1.0)
    n = O.dg_n_dofs(g)
    x = np.random.default_rng(3).standard_normal(n)
    y = np.empty_like(x)
    O.dg_sipg_apply(g, x, L=L, y=y)
    best, ts = cpu_time_best(lambda: O.dg_sipg_apply(g, x, L=L, y=y), CPU_REPEATS)
    out["dg_sipg_p5_48c_cg"] = {"cpu_port_apply_fp64_gdofs": round(n / best / 1e9, 4), "cores": threads,
                                "sample": "full 48^3 p=5 apply, best of %d" % CPU_REPEATS}
    g = O.dg(4, (48, 48, 48), (h, h, h), velocity=(1.0, 0.5, 0.25), inverse_mass=1)
    n = O.dg_n_dofs(g)
    x = np.random.default_rng(5).uniform(-1, 1, n)
    y = np.empty_like(x)
    O.dg_advect_apply(g, x, L=L, y=y)
    best, ts = cpu_time_best(lambda: O.dg_advect_apply(g, x, L=L, y=y), CPU_REPEATS)
    out["dg_advect_p4_48c_8rhs"] = {"cpu_port_apply_fp64_gdofs_per_rhs": round(n / best / 1e9, 4),
                                    "cores": threads,
                                    "sample": "full 48^3 p=4 apply of one right-hand side (with M^-1), best of %d"
                                              % CPU_REPEATS}
    for key, ent in out.items():
        if configs and key in configs:
            cfg = configs[key]
            cfg["cpu_baseline"] = ent
            if key == "dg_sipg_p5_48c_cg":
                cfg["fp32_apply_over_cpu"] = round(cfg["apply_fp32_gdofs"] / ent["cpu_port_apply_fp64_gdofs"], 1)
                cfg["fp64_apply_over_cpu"] = round(cfg["apply_fp64_gdofs"] / ent["cpu_port_apply_fp64_gdofs"], 1)
            else:
                c = ent["cpu_port_apply_fp64_gdofs_per_rhs"]
                cfg["fp32_forward_over_cpu"] = round(cfg["fp32"]["forward_gdofs_total_8rhs"] / c, 1)
                cfg["fp64_forward_over_cpu"] = round(cfg["fp64"]["forward_gdofs_total_8rhs"] / c, 1)
    return out


def run_reference(args):
    """the reference's CPU algorithm (the oracle port, -O3, all host threads)
    on the same workload: each step is one full apply"""
    import numpy as np

    rank, world, _ = dist_setup(args.gpus)
    if rank != 0:
        return
    p, nc = args.degree, args.ncells
    O, m, G, x = cpu_cont_setup(p, nc)
    L = O.perf_lib()
    threads = os.cpu_count() or 1
    y = np.empty_like(x)
    n = O.cont_n_dofs(m)
    for _ in range(args.warmup):
        O.cont_apply(m, G, x, n_threads=threads, y=y, L=L)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.cont_apply(m, G, x, n_threads=threads, y=y, L=L)
        ts.append(time.perf_counter() - t0)
    best, med = min(ts), statistics.median(ts)
    value = n / best / 1e9
    base = {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "the full %d^3 deformed p=%d workload (%d DoFs) every step, FP64, precomputed geometry; "
                      "value from the best of %d steps (median %.4f s, best %.4f s)" % (nc, p, n, len(ts), med, best),
            "build": "gcc " + perf_build_flags() + ", OMP_PROC_BIND=close",
            "host": host_cpu()}
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(best * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": workload_config(p, nc),
            "cpu_baseline": base,
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def time_apply(op, x, y, steps, warmup, stream, what="apply"):
    import torch
    for _ in range(warmup):
        op.vmult(x, y, stream=stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        op.vmult(x, y, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    check_status(op, what)
    return e0.elapsed_time(e1) / 1e3 / steps


def solve_entry(code, st):
    return {"status": code, "iterations": st.iterations, "outer": st.outer_iterations,
            "rel_residual": float("%.3g" % st.rel_residual), "seconds": round(st.seconds, 3),
            "operator_applies": st.operator_applies}


def cont_cg_sweep(degrees, ncells):
    """the mixed-precision target: FP32-inner / FP64-refined CG against plain FP64
    CG to 1e-10 on the continuous Laplacian of the deformed mesh, Chebyshev(5)
    Jacobi preconditioner for both, right-hand side uniform[-1,1]"""
    import numpy as np
    import torch

    from sum_factorization_kernels_gb300 import sfgpu

    out = {"n_cells": [ncells] * 3, "rtol": 1e-10, "preconditioner": "Chebyshev(5) of D^-1 A, both solves",
           "degrees": {}}
    for q in degrees:
        op = sfgpu.Operator(sfgpu.OP_LAPLACE, degree=q, n_cells=(ncells,) * 3, deform=DEFORM)
        b = torch.tensor(np.random.default_rng(30 + q).uniform(-1, 1, op.n_dofs), device="cuda")
        res = {"n_dofs": op.n_dofs}
        for name, mode in (("mixed_fp32_inner", sfgpu.SOLVE_MIXED), ("all_fp64", sfgpu.SOLVE_FP64)):
            opts = sfgpu.default_solve_opts(mode=mode, precond=sfgpu.PRECOND_CHEBYSHEV, cheb_degree=5,
                                            rtol=1e-10, max_iter=20000)
            # preconditioner setup (diagonal, eigenvalue estimate) is cached per handle
            op.cg_solve(b, torch.zeros_like(b), sfgpu.default_solve_opts(mode=mode, max_iter=1, rtol=0.5))
            xs = torch.zeros_like(b)
            code, st = op.cg_solve(b, xs, opts)
            res[name] = solve_entry(code, st)
        check_status(op, "continuous CG p=%d" % q)
        if res["mixed_fp32_inner"]["seconds"] > 0:
            res["fp64_over_mixed_wall_time"] = round(res["all_fp64"]["seconds"] / res["mixed_fp32_inner"]["seconds"], 2)
        out["degrees"][str(q)] = res
        del op, b
        torch.cuda.empty_cache()
    return out


def secondary_configs(stream, peak):
    """the other configurations of the metric, measured once each: config 1
    (Q4 16^3 affine FP64, error vs the reference's golden vector), config 3
    (DG SIPG p=5 48^3 CG to 1e-10: FP32-inner/FP64-refined vs all-FP64; the
    same problem with the precomputed tensor-product SIPG operator),
    config 4 (variable kappa p=4 32^3: forward and adjoint), config 5 (DG
    advection p=4 48^3, 8 right-hand sides: forward / transpose, LSRK(5,4)
    time steps, dot test), the mass / convection variants of the cell
    operator (p=4 affine 64^3 FP32) and the unstructured-mesh input
    (p=4 48^3 FP32)"""
    import numpy as np
    import torch

    from sum_factorization_kernels_gb300 import sfgpu

    out = {}
    # ---- config 1 ----
    op = sfgpu.Operator(sfgpu.OP_LAPLACE, degree=4, n_cells=(16, 16, 16))
    x = torch.tensor(np.random.default_rng(20241203).uniform(-1.0, 1.0, op.n_dofs), device="cuda")
    y = torch.empty_like(x)
    t = time_apply(op, x, y, 50, 5, stream, "config 1")
    g = np.load(os.path.join(ROOT, "tests", "golden", "cont.npz"))
    idx = g["q4_16_sample_idx"]
    yh = y.cpu().numpy()
    err = float(np.linalg.norm(yh[idx] - g["q4_16_sample_y"]) / np.linalg.norm(g["q4_16_sample_y"]))
    out["q4_affine_16c_fp64"] = {"n_dofs": op.n_dofs, "gdofs": round(op.n_dofs / t / 1e9, 3),
                                 "rel_err_vs_reference_golden": float("%.3g" % err)}
    del op, x, y
    # ---- config 3 ----
    op = sfgpu.Operator(sfgpu.OP_DG_SIPG, degree=5, n_cells=(48, 48, 48))
    N = op.n_dofs
    b = torch.tensor(np.random.default_rng(3).standard_normal(N), device="cuda")
    xd32 = torch.randn(N, device="cuda", dtype=torch.float32)
    yd32 = torch.empty_like(xd32)
    t32 = time_apply(op, xd32, yd32, 20, 3, stream, "config 3 FP32")
    xd64 = xd32.double()
    yd64 = torch.empty_like(xd64)
    t64 = time_apply(op, xd64, yd64, 5, 2, stream, "config 3 FP64")
    res = {"n_dofs": N, "apply_fp32_gdofs": round(N / t32 / 1e9, 3),
           "apply_fp32_hbm_frac": round(2 * 4 * N / t32 / 1e9 / peak, 4),
           "apply_fp64_gdofs": round(N / t64 / 1e9, 3)}
    for name, mode in (("mixed_fp32_inner", sfgpu.SOLVE_MIXED), ("all_fp64", sfgpu.SOLVE_FP64)):
        xs = torch.zeros_like(b)
        opts = sfgpu.default_solve_opts(mode=mode, precond=sfgpu.PRECOND_CHEBYSHEV, cheb_degree=5,
                                        rtol=1e-10, project_constant=1, max_iter=4000)
        op.cg_solve(b, torch.zeros_like(b), opts)  # preconditioner setup (cached per handle)
        code, st = op.cg_solve(b, xs, opts)
        res[name] = solve_entry(code, st)
    check_status(op, "config 3 CG")
    if res["mixed_fp32_inner"]["seconds"] > 0:
        res["fp64_over_mixed_wall_time"] = round(res["all_fp64"]["seconds"] / res["mixed_fp32_inner"]["seconds"], 2)
    out["dg_sipg_p5_48c_cg"] = res
    del op
    # the same SIPG problem class in the tensor-product form with precomputed
    # 1D matrices (PrecomputedDGLaplacian): apply and mixed-precision CG
    op = sfgpu.Operator(sfgpu.OP_DG_PRECOMPUTED, degree=5, n_cells=(48, 48, 48), length=(1.0, 1.0, 1.0))
    t32 = time_apply(op, xd32, yd32, 20, 3, stream, "precomputed FP32")
    t64 = time_apply(op, xd64, yd64, 5, 2, stream, "precomputed FP64")
    res = {"n_dofs": N, "apply_fp32_gdofs": round(N / t32 / 1e9, 3),
           "apply_fp32_hbm_frac": round(2 * 4 * N / t32 / 1e9 / peak, 4),
           "apply_fp64_gdofs": round(N / t64 / 1e9, 3)}
    xs = torch.zeros_like(b)
    opts = sfgpu.default_solve_opts(mode=sfgpu.SOLVE_MIXED, precond=sfgpu.PRECOND_CHEBYSHEV, cheb_degree=5,
                                    rtol=1e-10, project_constant=1, max_iter=4000)
    op.cg_solve(b, torch.zeros_like(b), opts)
    code, st = op.cg_solve(b, xs, opts)
    res["mixed_fp32_inner"] = solve_entry(code, st)
    check_status(op, "precomputed CG")
    out["dg_precomputed_p5_48c"] = res
    del op, b, xd32, yd32, xd64, yd64
    torch.cuda.empty_cache()
    # ---- config 4 ----
    op = sfgpu.Operator(sfgpu.OP_LAPLACE, degree=4, n_cells=(32, 32, 32), deform=0.05)
    nq = op.n_cells * 125
    kap = torch.exp(0.5 * torch.randn(nq, dtype=torch.float64, device="cuda"))
    op.set_coefficient(kap)
    res = {"n_dofs": op.n_dofs}
    for prec, dt in (("fp32", torch.float32), ("fp64", torch.float64)):
        xx = (torch.rand(op.n_dofs, device="cuda", dtype=torch.float64) * 2 - 1).to(dt)
        yy = torch.empty_like(xx)
        tf = time_apply(op, xx, yy, 20, 3, stream, "config 4 forward")
        dk = torch.empty(nq, dtype=dt, device="cuda")
        for _ in range(3):
            op.kappa_gradient(xx, yy, dk)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            op.kappa_gradient(xx, yy, dk)
        e1.record()
        torch.cuda.synchronize()
        check_status(op, "config 4 dkappa")
        tg = e0.elapsed_time(e1) / 1e3 / 10
        res[prec] = {"forward_gdofs": round(op.n_dofs / tf / 1e9, 3),
                     "dkappa_gdofs": round(op.n_dofs / tg / 1e9, 3)}
    out["kappa_p4_32c"] = res
    del op
    torch.cuda.empty_cache()
    # ---- config 5 ----
    op = sfgpu.Operator(sfgpu.OP_DG_ADVECT, degree=4, n_cells=(48, 48, 48), velocity=(1.0, 0.5, 0.25),
                        inverse_mass=1)
    N = op.n_dofs
    res = {"n_dofs_per_rhs": N, "nrhs": 8}
    for prec, dt in (("fp32", torch.float32), ("fp64", torch.float64)):
        xx = (torch.rand(8 * N, device="cuda", dtype=torch.float64) * 2 - 1).to(dt)
        yy = torch.empty_like(xx)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        for _ in range(3):
            op.vmult_batched(xx, yy, 8, stream=stream)
            op.vmult_transpose_batched(xx, yy, 8, stream=stream)
        torch.cuda.synchronize()
        reps = 10 if prec == "fp32" else 3
        ev[0].record(stream)
        for _ in range(reps):
            op.vmult_batched(xx, yy, 8, stream=stream)
        ev[1].record(stream)
        for _ in range(reps):
            op.vmult_transpose_batched(xx, yy, 8, stream=stream)
        ev[2].record(stream)
        # LSRK(5,4) time steps (do_time_step): five fused operator stages
        old, tmp = torch.zeros_like(xx), torch.zeros_like(xx)
        op.lsrk_step(xx, old, tmp, 1e-3, nrhs=8, stream=stream)
        ev[3].record(stream)
        for _ in range(reps):
            op.lsrk_step(xx, old, tmp, 1e-3, nrhs=8, stream=stream)
        ev[4].record(stream)
        torch.cuda.synchronize()
        check_status(op, "config 5 %s" % prec)
        tf = ev[0].elapsed_time(ev[1]) / 1e3 / reps
        tt = ev[1].elapsed_time(ev[2]) / 1e3 / reps
        ts = ev[3].elapsed_time(ev[4]) / 1e3 / reps
        res[prec] = {"forward_gdofs_total_8rhs": round(8 * N / tf / 1e9, 3),
                     "forward_hbm_frac": round(2 * dt.itemsize * 8 * N / tf / 1e9 / peak, 4),
                     "transpose_gdofs_total_8rhs": round(8 * N / tt / 1e9, 3),
                     # DoF-steps per second; 5 stages x (src, upd read; vec_np, vec_tm written),
                     # the reference's memory model (test_dg_advect.cc:111-113)
                     "lsrk_step_gdofs_total_8rhs": round(8 * N / ts / 1e9, 3),
                     "lsrk_step_hbm_frac": round(20 * dt.itemsize * 8 * N / ts / 1e9 / peak, 4)}
    # the cell-and-face kernel (SF_KERNEL_GENERIC) on the same FP32 batch
    op.set_kernel_variant(sfgpu.KERNEL_GENERIC)
    xx = (torch.rand(8 * N, device="cuda", dtype=torch.float64) * 2 - 1).to(torch.float32)
    yy = torch.empty_like(xx)
    for _ in range(3):
        op.vmult_batched(xx, yy, 8, stream=stream)
        op.vmult_transpose_batched(xx, yy, 8, stream=stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(stream)
    for _ in range(10):
        op.vmult_batched(xx, yy, 8, stream=stream)
    ev[1].record(stream)
    for _ in range(10):
        op.vmult_transpose_batched(xx, yy, 8, stream=stream)
    ev[2].record(stream)
    torch.cuda.synchronize()
    check_status(op, "config 5 cell-and-face kernel")
    res["fp32"]["cell_face_kernel"] = {
        "forward_gdofs_total_8rhs": round(8 * N / (ev[0].elapsed_time(ev[1]) / 1e4) / 1e9, 3),
        "transpose_gdofs_total_8rhs": round(8 * N / (ev[1].elapsed_time(ev[2]) / 1e4) / 1e9, 3)}
    op.set_kernel_variant(sfgpu.KERNEL_AUTO)
    del xx, yy
    x64 = torch.rand(8 * N, device="cuda", dtype=torch.float64) * 2 - 1
    y64 = torch.rand(8 * N, device="cuda", dtype=torch.float64) * 2 - 1
    ax, aty = torch.empty_like(x64), torch.empty_like(y64)
    op.vmult_batched(x64, ax, 8)
    op.vmult_transpose_batched(y64, aty, 8)
    worst = 0.0
    for r in range(8):
        s_ = slice(r * N, (r + 1) * N)
        lhs, rhs = float(torch.dot(ax[s_], y64[s_])), float(torch.dot(x64[s_], aty[s_]))
        worst = max(worst, abs(lhs - rhs) / float(ax[s_].norm() * y64[s_].norm()))
    check_status(op, "config 5 dot test")
    res["adjoint_dot_test_rel"] = float("%.3g" % worst)
    out["dg_advect_p4_48c_8rhs"] = res
    del op
    torch.cuda.empty_cache()
    # ---- the cell operator's DO_MASS_MATRIX / DO_CONVECTION variants:
    # continuous mass matrix and convection form, p=4, affine 64^3, FP32
    # (vectors only: 2 s N algorithmic bytes); default kernel (assembled
    # Kronecker products) and the line-ownership kernel (SF_KERNEL_GENERIC) ----
    res = {}
    for name, kind in (("mass", sfgpu.OP_MASS), ("convection", sfgpu.OP_CONVECTION)):
        op = sfgpu.Operator(kind, degree=4, n_cells=(64, 64, 64), velocity=(1.0, 2.0, 3.0))
        x = torch.rand(op.n_dofs, device="cuda", dtype=torch.float32) * 2 - 1
        y = torch.empty_like(x)
        t = time_apply(op, x, y, 30, 5, stream, name)
        op.set_kernel_variant(sfgpu.KERNEL_GENERIC)
        tg = time_apply(op, x, y, 30, 5, stream, name + " (line kernel)")
        res[name] = {"gdofs": round(op.n_dofs / t / 1e9, 3), "hbm_frac": round(8 * op.n_dofs / t / 1e9 / peak, 4),
                     "kernel": "assembled Kronecker products (z pass + x-y tiles)",
                     "line_kernel_gdofs": round(op.n_dofs / tg / 1e9, 3)}
        del op, x, y
    # the DO_FACES builds on the cell-major vector of the same 64^3 cells
    # (n^3 entries per cell; 2 s C n^3 algorithmic bytes); default kernel
    # (sums of 1D line operators) and the face-array kernel
    for name, kind in (("laplace_faces", sfgpu.OP_LAPLACE_FACES), ("convection_faces", sfgpu.OP_CONVECTION_FACES)):
        op = sfgpu.Operator(kind, degree=4, n_cells=(64, 64, 64), velocity=(1.0, 2.0, 3.0))
        x = torch.rand(op.n_dofs, device="cuda", dtype=torch.float32) * 2 - 1
        y = torch.empty_like(x)
        t = time_apply(op, x, y, 30, 5, stream, name)
        op.set_kernel_variant(sfgpu.KERNEL_GENERIC)
        tg = time_apply(op, x, y, 30, 5, stream, name + " (face-array kernel)")
        res[name] = {"gdofs": round(op.n_dofs / t / 1e9, 3), "hbm_frac": round(8 * op.n_dofs / t / 1e9 / peak, 4),
                     "n_dofs": op.n_dofs, "kernel": "sums of 1D line operators",
                     "face_array_kernel_gdofs": round(op.n_dofs / tg / 1e9, 3)}
        del op, x, y
    out["cell_variants_p4_64c_affine_fp32"] = res
    # ---- unstructured hexahedral input: the 48^3 p=4 box given as cell-node
    # index arrays (lexicographic numbering) and per-cell merged geometry
    # (affine tensor times Gauss weights); bytes: vectors, geometry, indices
    # and the per-column masks ----
    from sum_factorization_kernels_gb300.timing import unstructured_box
    p_, nc_ = 4, 48
    n_ = p_ + 1
    idx, geo, N = unstructured_box(p_, nc_)
    op = sfgpu.Operator.unstructured(p_, idx, geo, N, dirichlet=None, precisions=2)
    del geo, idx
    x = torch.rand(N, device="cuda", dtype=torch.float32) * 2 - 1
    y = torch.empty_like(x)
    t = time_apply(op, x, y, 30, 5, stream, "unstructured")
    C = nc_ ** 3
    bytes_apply = 8 * N + C * (6 * n_ ** 3 * 4 + n_ ** 3 * 4 + n_ ** 2 * 4)
    out["unstructured_p4_48c_fp32"] = {"n_dofs": N, "gdofs": round(N / t / 1e9, 3),
                                       "hbm_frac": round(bytes_apply / t / 1e9 / peak, 4),
                                       "algorithmic_bytes_per_apply": bytes_apply}
    del op, x, y
    torch.cuda.empty_cache()
    return out


def run_ours(args):
    import numpy as np
    import torch

    from sum_factorization_kernels_gb300 import sfgpu

    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    peak, peak_kind = measured_peaks()
    p = args.degree
    NCELLS = (args.ncells,) * 3

    # ---- headline: FP32, degree p, inputs resident ----
    op = sfgpu.Operator(sfgpu.OP_LAPLACE, degree=p, n_cells=NCELLS, deform=DEFORM)
    N, C = op.n_dofs, op.n_cells
    assert N == workload_config(p, args.ncells)["n_dofs"]
    gen = torch.Generator(device="cuda").manual_seed(1234 + rank)
    x64 = torch.rand(N, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
    x32 = x64.float()
    y32 = torch.empty_like(x32)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            op.vmult(x32, y32, stream=stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        op.vmult(x32, y32, stream=stream)
    e1.record(stream)
    clocks.sample_now()  # the queued applies are running
    torch.cuda.synchronize()
    barrier(world)
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    clk = clocks.stop()
    check_status(op, "the timed applies")
    t_step = max_over_ranks(t_step, world)
    value = N * world / t_step / 1e9
    bytes_apply = algorithmic_bytes(p, N, C, 4)
    achieved = bytes_apply / t_step / 1e9
    launches_per_apply = 8  # one launch per colour class

    # ---- e2e: pinned host input -> device -> apply -> host, every step ----
    # Steps are pipelined on three streams with two device buffer pairs:
    # step k+1's host-to-device copy and step k-1's device-to-host copy run
    # while step k's apply runs.  Every step copies its whole input in and
    # its whole result out inside the timed region.
    xh = torch.empty(N, dtype=torch.float32, pin_memory=True)
    xh.copy_(x32.cpu())
    yh = [torch.empty(N, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    xd = [torch.empty_like(x32) for _ in range(2)]
    yd = [torch.empty_like(x32) for _ in range(2)]
    # each copy is split into E2E_CHUNKS pieces on as many streams (several
    # copy engines); one cudaMemcpyAsync per piece
    nch = max(1, args.e2e_chunks)
    bounds = [N * i // nch for i in range(nch + 1)]
    s_in = [torch.cuda.Stream() for _ in range(nch)]
    s_out = [torch.cuda.Stream() for _ in range(nch)]
    ev_in = [[torch.cuda.Event() for _ in range(nch)] for _ in range(2)]
    ev_apply = [torch.cuda.Event() for _ in range(2)]
    ev_out = [[torch.cuda.Event() for _ in range(nch)] for _ in range(2)]
    for e in ev_apply + [e for row in ev_out for e in row]:
        e.record(stream)
    torch.cuda.synchronize()

    def e2e_steps(k_steps):
        for k in range(k_steps):
            b = k & 1
            for c in range(nch):
                lo, hi = bounds[c], bounds[c + 1]
                s_in[c].wait_event(ev_apply[b])   # xd[b] no longer read
                with torch.cuda.stream(s_in[c]):
                    xd[b][lo:hi].copy_(xh[lo:hi], non_blocking=True)
                ev_in[b][c].record(s_in[c])
                stream.wait_event(ev_in[b][c])
                stream.wait_event(ev_out[b][c])   # yd[b] already copied out
            op.vmult(xd[b], yd[b], stream=stream)
            ev_apply[b].record(stream)
            for c in range(nch):
                lo, hi = bounds[c], bounds[c + 1]
                s_out[c].wait_event(ev_apply[b])
                with torch.cuda.stream(s_out[c]):
                    yh[b][lo:hi].copy_(yd[b][lo:hi], non_blocking=True)
                ev_out[b][c].record(s_out[c])

    e2e_steps(args.warmup)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    e2e_steps(args.steps)
    torch.cuda.synchronize()
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    check_status(op, "the e2e applies")
    e2e = {"value": N * world / t_e2e / 1e9, "unit": UNIT, "h2d_bytes_per_step": 4 * N,
           "d2h_bytes_per_step": 4 * N,
           "pipelined": "2 device buffer pairs: H2D of step k+1 and D2H of step k-1 overlap the apply of step k; "
                        "each copy in %d pieces on %d streams" % (nch, nch)}
    if not torch.equal(yh[(args.steps - 1) & 1], yd[(args.steps - 1) & 1].cpu()):
        raise SystemExit("e2e: the result read back differs from the device result")
    del op, xh, yh, xd, yd, x64, x32, y32
    torch.cuda.empty_cache()

    # ---- the degree sweep, FP32 and FP64; inputs from a seeded host
    # generator so the CPU leg checks every apply on the same vector ----
    sweep = []
    fp64_value = None
    check = rank == 0 and world == 1 and not args.no_cpu
    if not args.no_sweep:
        degrees = [int(d) for d in args.sweep.split(",")]
        for q in degrees:
            opq = sfgpu.Operator(sfgpu.OP_LAPLACE, degree=q, n_cells=NCELLS, deform=DEFORM)
            Nq = opq.n_dofs
            xh64 = np.random.default_rng(4000 + q).uniform(-1, 1, Nq)
            xq64 = torch.from_numpy(xh64).cuda()
            xq32 = xq64.float()
            yq64 = torch.empty_like(xq64)
            yq32 = torch.empty_like(xq32)
            reps64 = max(2, min(args.steps, 6))
            t64 = time_apply(opq, xq64, yq64, reps64, 2, stream, "FP64 sweep p=%d" % q)
            t32 = time_apply(opq, xq32, yq32, max(3, args.steps), 2, stream, "FP32 sweep p=%d" % q)
            err = float((yq32.double() - yq64).norm() / yq64.norm())
            b32 = algorithmic_bytes(q, Nq, opq.n_cells, 4)
            b64 = algorithmic_bytes(q, Nq, opq.n_cells, 8)
            ent = {"degree": q, "n_dofs": Nq,
                   "fp32_gdofs": round(Nq / t32 / 1e9, 3), "fp32_hbm_frac": round(b32 / t32 / 1e9 / peak, 4),
                   "fp64_gdofs": round(Nq / t64 / 1e9, 3), "fp64_hbm_frac": round(b64 / t64 / 1e9 / peak, 4),
                   "fp32_rel_err_vs_fp64": float("%.3g" % err)}
            if check:
                ent["_host"] = (xh64, yq64.cpu().numpy(), yq32.cpu().numpy())
            sweep.append(ent)
            if q == p:
                fp64_value = ent["fp64_gdofs"]
            del opq, xq64, xq32, yq64, yq32
            torch.cuda.empty_cache()

    cg = None
    if not args.no_cg and world == 1:
        cg = cont_cg_sweep([int(d) for d in args.cg_degrees.split(",")], args.cg_ncells)

    configs = None
    if not args.no_configs and world == 1:
        configs = secondary_configs(stream, peak)
        if cg is not None:
            configs["cont_cg_p4_8"] = cg
    elif cg is not None:
        configs = {"cont_cg_p4_8": cg}

    # ---- CPU leg (rank 0, one GPU): the port timed on the full workload,
    # the oracle's errors of every sweep apply, DG baselines ----
    cpu = None
    if check:
        cpu = cpu_cont_baseline(p, args.ncells)
        cpu_check_sweep(sweep, args.ncells)
        if configs is not None and not args.no_configs:
            cpu_dg_baselines(configs)
    for ent in sweep:
        ent.pop("_host", None)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(p, args.ncells),
            "details": {"parallelism": "replicas" if world > 1 else "single GPU",
                        "l2": "working set %.2f GB > 129 MB L2, no flush" % (bytes_apply / 1e9),
                        "fp64_gdofs_same_degree": fp64_value},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": MEASURED_TRAFFIC.get((p, args.ncells)),
                         "traffic_source": TRAFFIC_SOURCE if (p, args.ncells) in MEASURED_TRAFFIC else None,
                         "peak_kind": peak_kind,
                         "kernel": "line_vmult_kernel<%d,float,deformed> (8 colour launches per apply)" % (p + 1),
                         "algorithmic_bytes_per_apply": bytes_apply},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk,
            "gpu_launches": launches_per_apply * args.steps,
            "sweep": sweep,
            "configs": configs,
        }
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--degree", type=int, default=4)
    ap.add_argument("--ncells", type=int, default=64, help="cells per direction")
    ap.add_argument("--sweep", default="2,3,4,5,6,7,8")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU leg (baseline and oracle errors)")
    ap.add_argument("--no-configs", action="store_true", help="skip configs 1, 3, 4, 5")
    ap.add_argument("--no-cg", action="store_true", help="skip the continuous CG comparison")
    ap.add_argument("--cg-degrees", default="4,5,6,7,8")
    ap.add_argument("--cg-ncells", type=int, default=64)
    ap.add_argument("--e2e-chunks", type=int, default=1, help="pieces per host-device copy in the e2e leg")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
