"""Benchmark: continuous FE Laplacian matvec on the deformed 64^3 mesh.

Workload (the metric's configuration): 64x64x64 hexahedral cells on [0,1]^3
mapped by x_i <- x_i + 0.05 sin(2 pi x_j) sin(2 pi x_k), Gauss quadrature
with n = p+1 points, precomputed merged 6-entry geometry per quadrature point,
homogeneous Dirichlet boundary, input uniform[-1,1].  Headline: degree 4,
FP32 operator; the JSON line also carries the degree 2..8 sweep in FP32 and
FP64 with the relative error of every FP32 apply against the FP64 apply.

One step = one operator apply y = A x with x and the geometry resident in
HBM (the working set, 0.9 GB at p=4 FP32, exceeds the 129 MB L2, so no
explicit flush).  e2e = the same apply through the C ABI with the input
copied from pinned host memory and the result copied back every step (steps
pipelined on three streams with double-buffered device vectors).

``--impl reference`` times the reference's CPU algorithm for the same apply
on the host cores (the FP64 oracle port, OpenMP over all host threads) on a
bounded sample of cells and prints the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
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
MEASURED_TRAFFIC = {(4, 64): 985032704}
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum summed over the 8 colour launches "
                  "of one apply, caches warm (--cache-control none)")
UNIT = "GDoF/s"
REF_BUDGET_S = 120.0  # CPU seconds of the --impl reference run's timed steps
DEFORM = 0.05


def algorithmic_bytes(p, n_dofs, n_cells, s):
    """x read once, y written once, 6 geometry entries per quadrature point
    (node indices are computed, not stored)"""
    return 2 * s * n_dofs + 6 * s * (p + 1) ** 3 * n_cells


def workload_config(p, ncells):
    """the workload keys both arms report (the continuous node count
    includes the Dirichlet boundary nodes)"""
    return {"workload": "continuous Laplacian matvec, deformed %d^3 hex mesh, p=%d" % (ncells, p),
            "degree": p, "n_cells": [ncells] * 3, "n_dofs": (p * ncells + 1) ** 3, "deform": DEFORM,
            "geometry": "merged 6-entry JxW J^-1 J^-T per Gauss point, in the apply's precision",
            "dirichlet": True}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


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

    def _run(self):
        import ctypes
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop_evt.is_set():
            if self.nvml.nvmlDeviceGetClockInfo(self.h, ctypes.c_int(1), ctypes.byref(clk)) == 0:
                self.samples.append(float(clk.value))
            if self.reason_fn is not None and self.reason_fn(self.h, ctypes.byref(rs)) == 0:
                for bit, name in self.REASONS.items():
                    if rs.value & bit:
                        self.reasons.add(name)
            self.stop_evt.wait(0.002)

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


def cpu_reference(p, seconds=12.0, n_threads=None):
    """time the FP64 oracle port of the reference's cell algorithm (gather ->
    even-odd sum factorisation -> scatter) on a bounded sample mesh"""
    import numpy as np

    from oracle import oracle as O

    threads = n_threads or os.cpu_count() or 1
    nc = (16, 16, 16)
    m = O.mesh(p, nc, deform=DEFORM)
    G = O.cont_geometry(m)
    x = np.random.default_rng(1).uniform(-1, 1, O.cont_n_dofs(m))
    O.cont_apply(m, G, x, n_threads=threads)  # warm-up
    reps, t0 = 0, time.perf_counter()
    while True:
        O.cont_apply(m, G, x, n_threads=threads)
        reps += 1
        el = time.perf_counter() - t0
        if el >= seconds or reps >= 100000:
            break
    n_dofs = O.cont_n_dofs(m)
    return {"value": n_dofs * reps / el / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "16^3 cells of the deformed mesh, p=%d, FP64, %d applies in %.1f s" % (p, reps, el)}


def run_reference(args):
    rank, world, _ = dist_setup(args.gpus)
    if rank != 0:
        return
    p = args.degree
    per_step = []
    base = None
    # each step is a bounded sample: the whole run stays within about
    # REF_BUDGET_S seconds of CPU time whatever --steps is
    step_s = max(0.05, min(args.ref_seconds, REF_BUDGET_S / max(1, args.steps)))
    for _ in range(args.warmup):
        cpu_reference(p, seconds=min(1.0, step_s))
    for _ in range(args.steps):
        r = cpu_reference(p, seconds=step_s)
        per_step.append(r["value"])
        base = r
    value = statistics.median(per_step)
    base["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": workload_config(p, args.ncells),
            "cpu_baseline": base,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def time_apply(op, x, y, steps, warmup, stream):
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
    return e0.elapsed_time(e1) / 1e3 / steps


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
    t = time_apply(op, x, y, 50, 5, stream)
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
    t32 = time_apply(op, xd32, yd32, 20, 3, stream)
    xd64 = xd32.double()
    yd64 = torch.empty_like(xd64)
    t64 = time_apply(op, xd64, yd64, 5, 2, stream)
    res = {"n_dofs": N, "apply_fp32_gdofs": round(N / t32 / 1e9, 3),
           "apply_fp32_hbm_frac": round(2 * 4 * N / t32 / 1e9 / peak, 4),
           "apply_fp64_gdofs": round(N / t64 / 1e9, 3)}
    for name, mode in (("mixed_fp32_inner", sfgpu.SOLVE_MIXED), ("all_fp64", sfgpu.SOLVE_FP64)):
        xs = torch.zeros_like(b)
        opts = sfgpu.default_solve_opts(mode=mode, precond=sfgpu.PRECOND_CHEBYSHEV, cheb_degree=5,
                                        rtol=1e-10, project_constant=1, max_iter=4000)
        op.cg_solve(b, torch.zeros_like(b), opts)  # preconditioner setup (cached per handle)
        code, st = op.cg_solve(b, xs, opts)
        res[name] = {"status": code, "iterations": st.iterations, "outer": st.outer_iterations,
                     "rel_residual": float("%.3g" % st.rel_residual), "seconds": round(st.seconds, 3),
                     "operator_applies": st.operator_applies}
    if res["mixed_fp32_inner"]["seconds"] > 0:
        res["fp64_over_mixed_wall_time"] = round(res["all_fp64"]["seconds"] / res["mixed_fp32_inner"]["seconds"], 2)
    out["dg_sipg_p5_48c_cg"] = res
    del op
    # the same SIPG problem class in the tensor-product form with precomputed
    # 1D matrices (PrecomputedDGLaplacian): apply and mixed-precision CG
    op = sfgpu.Operator(sfgpu.OP_DG_PRECOMPUTED, degree=5, n_cells=(48, 48, 48), length=(1.0, 1.0, 1.0))
    t32 = time_apply(op, xd32, yd32, 20, 3, stream)
    t64 = time_apply(op, xd64, yd64, 5, 2, stream)
    res = {"n_dofs": N, "apply_fp32_gdofs": round(N / t32 / 1e9, 3),
           "apply_fp32_hbm_frac": round(2 * 4 * N / t32 / 1e9 / peak, 4),
           "apply_fp64_gdofs": round(N / t64 / 1e9, 3)}
    xs = torch.zeros_like(b)
    opts = sfgpu.default_solve_opts(mode=sfgpu.SOLVE_MIXED, precond=sfgpu.PRECOND_CHEBYSHEV, cheb_degree=5,
                                    rtol=1e-10, project_constant=1, max_iter=4000)
    op.cg_solve(b, torch.zeros_like(b), opts)
    code, st = op.cg_solve(b, xs, opts)
    res["mixed_fp32_inner"] = {"status": code, "iterations": st.iterations, "outer": st.outer_iterations,
                               "rel_residual": float("%.3g" % st.rel_residual), "seconds": round(st.seconds, 3),
                               "operator_applies": st.operator_applies}
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
        tf = time_apply(op, xx, yy, 20, 3, stream)
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
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
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
        ev.append(torch.cuda.Event(enable_timing=True))
        ev[4].record(stream)
        torch.cuda.synchronize()
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
    res["adjoint_dot_test_rel"] = float("%.3g" % worst)
    out["dg_advect_p4_48c_8rhs"] = res
    del op
    torch.cuda.empty_cache()
    # ---- the cell operator's DO_MASS_MATRIX / DO_CONVECTION variants:
    # continuous mass matrix and convection form, p=4, affine 64^3, FP32
    # (vectors only: 2 s N algorithmic bytes) ----
    res = {}
    for name, kind in (("mass", sfgpu.OP_MASS), ("convection", sfgpu.OP_CONVECTION)):
        op = sfgpu.Operator(kind, degree=4, n_cells=(64, 64, 64), velocity=(1.0, 2.0, 3.0))
        x = torch.rand(op.n_dofs, device="cuda", dtype=torch.float32) * 2 - 1
        y = torch.empty_like(x)
        t = time_apply(op, x, y, 30, 5, stream)
        res[name] = {"gdofs": round(op.n_dofs / t / 1e9, 3), "hbm_frac": round(8 * op.n_dofs / t / 1e9 / peak, 4)}
        del op, x, y
    # the DO_FACES builds on the cell-major vector of the same 64^3 cells
    # (n^3 entries per cell; 2 s C n^3 algorithmic bytes)
    for name, kind in (("laplace_faces", sfgpu.OP_LAPLACE_FACES), ("convection_faces", sfgpu.OP_CONVECTION_FACES)):
        op = sfgpu.Operator(kind, degree=4, n_cells=(64, 64, 64), velocity=(1.0, 2.0, 3.0))
        x = torch.rand(op.n_dofs, device="cuda", dtype=torch.float32) * 2 - 1
        y = torch.empty_like(x)
        t = time_apply(op, x, y, 30, 5, stream)
        res[name] = {"gdofs": round(op.n_dofs / t / 1e9, 3), "hbm_frac": round(8 * op.n_dofs / t / 1e9 / peak, 4),
                     "n_dofs": op.n_dofs}
        del op, x, y
    out["cell_variants_p4_64c_affine_fp32"] = res
    # ---- unstructured hexahedral input: the 48^3 p=4 box given as cell-node
    # index arrays (lexicographic numbering) and per-cell merged geometry
    # (affine tensor times Gauss weights); bytes: vectors, geometry, indices
    # and the per-column masks ----
    p_, nc_ = 4, 48
    n_ = p_ + 1
    S_, D_, xq_, wq_ = sfgpu.shape_tables(p_)
    Nx = p_ * nc_ + 1
    cz, cy, cx = np.meshgrid(np.arange(n_), np.arange(n_), np.arange(n_), indexing="ij")
    kk, jj, ii = np.meshgrid(np.arange(nc_), np.arange(nc_), np.arange(nc_), indexing="ij")
    idx = (((kk.ravel()[:, None] * p_ + cz.ravel()[None, :]) * Nx + (jj.ravel()[:, None] * p_ + cy.ravel()[None, :]))
           * Nx + (ii.ravel()[:, None] * p_ + cx.ravel()[None, :])).astype(np.int32)
    w3 = (wq_[:, None, None] * wq_[None, :, None] * wq_[None, None, :]).ravel()
    h = 1.0 / nc_
    g1 = np.zeros((6, n_ ** 3))
    g1[:3] = h * w3                             # JxW / h_d^2 = h
    geo = np.broadcast_to(g1, (nc_ ** 3, 6, n_ ** 3))
    N = Nx ** 3
    op = sfgpu.Operator.unstructured(p_, idx, geo, N, dirichlet=None, precisions=2)
    del geo, idx
    x = torch.rand(N, device="cuda", dtype=torch.float32) * 2 - 1
    y = torch.empty_like(x)
    t = time_apply(op, x, y, 30, 5, stream)
    C = nc_ ** 3
    bytes_apply = 8 * N + C * (6 * n_ ** 3 * 4 + n_ ** 3 * 4 + n_ ** 2 * 4)
    out["unstructured_p4_48c_fp32"] = {"n_dofs": N, "gdofs": round(N / t / 1e9, 3),
                                       "hbm_frac": round(bytes_apply / t / 1e9 / peak, 4),
                                       "algorithmic_bytes_per_apply": bytes_apply}
    del op, x, y
    torch.cuda.empty_cache()
    return out


def run_ours(args):
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
    torch.cuda.synchronize()
    barrier(world)
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    clk = clocks.stop()
    t_step = max_over_ranks(t_step, world)
    value = N * world / t_step / 1e9
    bytes_apply = algorithmic_bytes(p, N, C, 4)
    achieved = bytes_apply / t_step / 1e9
    launches_per_apply = 8  # one launch per colour class

    # ---- the other kernel variant at the headline degree (plane ownership) ----
    variants = {"line_gdofs": round(value / world, 3)}
    for name, var in (("pair_fp32x2_gdofs", sfgpu.KERNEL_PAIR),):
        op.set_kernel_variant(var)
        tv = time_apply(op, x32, y32, max(10, args.steps // 2), 3, stream)
        variants[name] = round(N / tv / 1e9, 3)
    op.set_kernel_variant(sfgpu.KERNEL_AUTO)

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
    e2e = {"value": N * world / t_e2e / 1e9, "unit": UNIT, "h2d_bytes_per_step": 4 * N,
           "d2h_bytes_per_step": 4 * N,
           "pipelined": "2 device buffer pairs: H2D of step k+1 and D2H of step k-1 overlap the apply of step k; "
                        "each copy in %d pieces on %d streams" % (nch, nch)}
    if not torch.equal(yh[(args.steps - 1) & 1], yd[(args.steps - 1) & 1].cpu()):
        raise SystemExit("e2e: the result read back differs from the device result")

    # ---- FP64 at the headline degree and the degree sweep ----
    sweep = []
    fp64_value = None
    if not args.no_sweep:
        y64 = torch.empty_like(x64)
        del op, xh, yh, xd, yd
        torch.cuda.empty_cache()
        degrees = [int(d) for d in args.sweep.split(",")]
        for q in degrees:
            opq = sfgpu.Operator(sfgpu.OP_LAPLACE, degree=q, n_cells=NCELLS, deform=DEFORM)
            Nq = opq.n_dofs
            xq64 = torch.rand(Nq, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
            xq32 = xq64.float()
            yq64 = torch.empty_like(xq64)
            yq32 = torch.empty_like(xq32)
            reps64 = max(2, min(args.steps, 6))
            t64 = time_apply(opq, xq64, yq64, reps64, 2, stream)
            t32 = time_apply(opq, xq32, yq32, max(3, args.steps), 2, stream)
            err = float((yq32.double() - yq64).norm() / yq64.norm())
            variants_q = {}
            for name, var in (("line", sfgpu.KERNEL_GENERIC), ("pair_fp32x2", sfgpu.KERNEL_PAIR)):
                opq.set_kernel_variant(var)
                tv = time_apply(opq, xq32, yq32, max(3, args.steps // 2), 2, stream)
                variants_q[name] = round(Nq / tv / 1e9, 3)
            opq.set_kernel_variant(sfgpu.KERNEL_AUTO)
            b32 = algorithmic_bytes(q, Nq, opq.n_cells, 4)
            b64 = algorithmic_bytes(q, Nq, opq.n_cells, 8)
            ent = {"degree": q, "n_dofs": Nq,
                   "fp32_gdofs": round(Nq / t32 / 1e9, 3), "fp32_hbm_frac": round(b32 / t32 / 1e9 / peak, 4),
                   "fp64_gdofs": round(Nq / t64 / 1e9, 3), "fp64_hbm_frac": round(b64 / t64 / 1e9 / peak, 4),
                   "fp32_rel_err_vs_fp64": float("%.3g" % err), "fp32_variants_gdofs": variants_q}
            sweep.append(ent)
            if q == p:
                fp64_value = ent["fp64_gdofs"]
            del opq, xq64, xq32, yq64, yq32
            torch.cuda.empty_cache()

    configs = None
    if not args.no_configs and world == 1:
        configs = secondary_configs(stream, peak)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_reference(p, seconds=args.ref_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": dict(workload_config(p, args.ncells),
                           parallelism="replicas" if world > 1 else "single GPU",
                           l2="working set %.2f GB > 129 MB L2, no flush" % (bytes_apply / 1e9),
                           fp64_gdofs_same_degree=fp64_value, kernel_variants=variants),
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
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip configs 1, 3, 4, 5")
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--e2e-chunks", type=int, default=1, help="pieces per host-device copy in the e2e leg")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
