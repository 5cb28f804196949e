"""Time single operator applies through the C ABI (CUDA events, inputs in
device memory): ``python -m sum_factorization_kernels_gb300.timing KIND ...``.

KIND is ``laplace`` (continuous, the deformed mesh; ``--deform 0`` for the
affine one), ``sipg`` (DG SIPG),
``advect`` (DG upwind advection with inverse mass), ``precomputed`` (DG
SIPG in tensor-product form with precomputed 1D matrices), ``mass`` /
``convection`` (continuous, affine), ``unstructured`` (the affine box given
as cell-node index arrays and per-cell geometry) or ``faces`` /
``convection_faces`` (the DO_FACES cell operators on cell-major vectors).  Prints one line with the
apply rate summed over the right-hand sides and the vector traffic it implies.
Used to drive profiler captures of one kernel on a small case.

KIND ``sweeps`` times the shared-memory slab sweeps alone (sf_sweep_benchmark)
with the CUDA-core even-odd contraction in FP32 and FP64 and with the tensor
cores (TF32 x3 and TF32), on ncells^3 cells of (degree+1)^3 values, and
prints each rate and each FP32 path's relative error against the FP64 path.
"""
from __future__ import annotations

import argparse

import torch

from . import sfgpu as sf


def unstructured_box(degree: int, ncells: int):
    """the unit box of ncells^3 affine cells as an unstructured mesh: cell-node
    indices in the lexicographic numbering and the merged tensor h w_q on the
    diagonal"""
    import numpy as np
    p, n = degree, degree + 1
    Nx = p * ncells + 1
    cz, cy, cx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    kk, jj, ii = np.meshgrid(np.arange(ncells), np.arange(ncells), np.arange(ncells), indexing="ij")
    idx = (((kk.ravel()[:, None] * p + cz.ravel()[None, :]) * Nx + (jj.ravel()[:, None] * p + cy.ravel()[None, :]))
           * Nx + (ii.ravel()[:, None] * p + cx.ravel()[None, :])).astype(np.int32)
    _, _, _, wq = sf.shape_tables(degree)
    w3 = (wq[:, None, None] * wq[None, :, None] * wq[None, None, :]).ravel()
    g1 = np.zeros((6, n ** 3))
    g1[:3] = w3 / ncells
    geo = np.broadcast_to(g1, (ncells ** 3, 6, n ** 3))
    return idx, geo, Nx ** 3


def make_operator(kind: str, degree: int, ncells: int, deform: float = 0.05):
    n = (ncells,) * 3
    if kind == "mass":
        return sf.Operator(sf.OP_MASS, degree=degree, n_cells=n)
    if kind == "convection":
        return sf.Operator(sf.OP_CONVECTION, degree=degree, n_cells=n, velocity=(1.0, 2.0, 3.0))
    if kind == "unstructured":
        idx, geo, nn = unstructured_box(degree, ncells)
        return sf.Operator.unstructured(degree, idx, geo, nn)
    if kind == "laplace":
        return sf.Operator(sf.OP_LAPLACE, degree=degree, n_cells=n, deform=deform)
    if kind == "sipg":
        return sf.Operator(sf.OP_DG_SIPG, degree=degree, n_cells=n)
    if kind == "advect":
        return sf.Operator(sf.OP_DG_ADVECT, degree=degree, n_cells=n, velocity=(1.0, 0.5, 0.25), inverse_mass=1)
    if kind == "precomputed":
        return sf.Operator(sf.OP_DG_PRECOMPUTED, degree=degree, n_cells=n)
    if kind == "faces":
        return sf.Operator(sf.OP_LAPLACE_FACES, degree=degree, n_cells=n)
    if kind == "convection_faces":
        return sf.Operator(sf.OP_CONVECTION_FACES, degree=degree, n_cells=n, velocity=(1.0, 2.0, 3.0))
    raise ValueError("unknown operator kind %r" % kind)


def sweeps(degree: int, ncells: int, rounds: int, reps: int, warmup: int) -> None:
    n3 = (degree + 1) ** 3
    cells = ncells ** 3
    g = torch.Generator(device="cuda").manual_seed(3)
    x64 = torch.rand(cells * n3, device="cuda", dtype=torch.float64, generator=g) * 2 - 1
    x32 = x64.float()
    x64 = x32.double()
    results = {}
    for name, method, x in (("eo_fp64", sf.SWEEP_EO_FP64, x64), ("eo_fp32", sf.SWEEP_EO_FP32, x32),
                            ("mma_tf32x3", sf.SWEEP_MMA_TF32X3, x32), ("mma_tf32", sf.SWEEP_MMA_TF32, x32)):
        y = torch.empty_like(x)

        def run():
            sf.check(sf.lib().sf_sweep_benchmark(degree, method, cells, rounds, x.data_ptr(), y.data_ptr(),
                                                 torch.cuda.current_stream().cuda_stream))

        for _ in range(warmup):
            run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            run()
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / reps
        results[name] = (t, y)
    ref = results["eo_fp64"][1]
    for name, (t, y) in results.items():
        err = float((y.double() - ref).norm() / ref.norm())
        # values swept per second: every round sweeps all values along x and along y
        print("sweeps p=%d %d^3 cells rounds=%d %-10s %.3f ms  %.1f G line-values/s  rel. error vs FP64 %.2e"
              % (degree, ncells, rounds, name, t * 1e3, 2 * rounds * cells * n3 / t / 1e9, err))


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("kind", choices=["laplace", "sipg", "advect", "precomputed", "mass", "convection",
                                     "unstructured", "faces", "convection_faces", "sweeps"])
    ap.add_argument("--degree", type=int, default=4)
    ap.add_argument("--ncells", type=int, default=32, help="cells per direction")
    ap.add_argument("--prec", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--nrhs", type=int, default=1)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--transpose", action="store_true", help="time the transposed apply")
    ap.add_argument("--rounds", type=int, default=16, help="sweeps: x and y sweeps per round")
    ap.add_argument("--deform", type=float, default=0.05, help="laplace: mapping amplitude (0: affine)")
    ap.add_argument("--generic", action="store_true",
                    help="select SF_KERNEL_GENERIC: the cell-and-face kernels of the DG operators and DO_FACES "
                         "forms, the line-ownership kernel of the affine continuous operators")
    a = ap.parse_args(argv)
    if a.kind == "sweeps":
        sweeps(a.degree, a.ncells, a.rounds, a.reps, a.warmup)
        return
    op = make_operator(a.kind, a.degree, a.ncells, a.deform)
    if a.generic:
        op.set_kernel_variant(sf.KERNEL_GENERIC)
    dt = torch.float32 if a.prec == "fp32" else torch.float64
    n = op.n_dofs
    g = torch.Generator(device="cuda").manual_seed(1)
    x = (torch.rand(a.nrhs * n, device="cuda", dtype=torch.float64, generator=g) * 2 - 1).to(dt)
    y = torch.empty_like(x)

    def apply():
        if a.transpose:
            op.vmult_transpose_batched(x, y, a.nrhs)
        elif a.nrhs > 1:
            op.vmult_batched(x, y, a.nrhs)
        else:
            op.vmult(x, y)

    for _ in range(a.warmup):
        apply()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        apply()
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / a.reps
    status = op.device_status()
    print("%s%s p=%d %d^3 %s nrhs=%d: %.3f GDoF/s (summed over right-hand sides), %.1f GB/s of vector "
          "traffic, %.1f us per apply, device status %d"
          % (a.kind + (" (generic)" if a.generic else ""), " (transpose)" if a.transpose else "", a.degree, a.ncells, a.prec, a.nrhs, a.nrhs * n / t / 1e9,
             2 * a.nrhs * n * x.element_size() / t / 1e9, t * 1e6, status))
    if status != 0:
        raise SystemExit("device status %d" % status)


if __name__ == "__main__":
    main()
