"""The operators evaluated as sums of 1D line operators or Kronecker products,
at the bench's sizes, against the FP64 oracle on the same vectors: DG
advection p=4 on 48^3 periodic cells (forward with the inverse mass, the
transpose with the inverse mass in one launch), the DO_FACES Laplacian and
convection forms on 48^3 cells, and the affine continuous Laplacian and mass
matrix on 64^3 cells with Dirichlet conditions.  At these sizes the grids run
many blocks per SM and the z pass of the Kronecker form walks long lines.
The advection kernels also keep two size-independent properties there:
conservation and constants transported unchanged."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


def _check(torch, apply, x, ref, p, factor=4):
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, factor * FP32_TOL[p])):
        xd = to_dev(torch, x, dtype)
        y = torch.full_like(xd, float("nan"))
        apply(xd, y)
        torch.cuda.synchronize()
        assert rel(to_np(y), ref) < tol, dtype


def test_advect_48c_vs_oracle():
    torch = torch_cuda()
    sf = _sf()
    p, nc, vel = 4, (48, 48, 48), (1.0, 0.5, 0.25)
    h = tuple(1.0 / n for n in nc)
    op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=nc, velocity=vel, inverse_mass=1)
    g = O.dg(p, nc, h, velocity=vel, inverse_mass=1)
    x = np.random.default_rng(48).uniform(-1, 1, op.n_dofs)
    _check(torch, op.vmult, x, O.dg_advect_apply(g, x), p)
    _check(torch, op.vmult_transpose, x, O.dg_advect_apply_transpose(g, x), p)
    assert op.device_status() == 0


@pytest.mark.parametrize("conv", [False, True])
def test_cell_faces_48c_vs_oracle(conv):
    torch = torch_cuda()
    sf = _sf()
    p, nc, b = 4, (48, 48, 48), (1.0, 0.5, 0.25)
    h = tuple(1.0 / n for n in nc)
    op = sf.Operator(sf.OP_CONVECTION_FACES if conv else sf.OP_LAPLACE_FACES, degree=p, n_cells=nc, velocity=b)
    x = np.random.default_rng(49).uniform(-1, 1, op.n_dofs)
    ref = O.cell_faces_apply(p, conv, op.n_dofs // (p + 1) ** 3, h, x, b)
    _check(torch, op.vmult, x, ref, p, factor=2)
    assert op.device_status() == 0


def test_affine_continuous_64c_vs_oracle():
    torch = torch_cuda()
    sf = _sf()
    p, nc = 4, (64, 64, 64)
    m = O.mesh(p, nc)
    x = np.random.default_rng(64).uniform(-1, 1, O.cont_n_dofs(m))
    lap = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc)
    _check(torch, lap.vmult, x, O.cont_apply(m, None, x, n_threads=os.cpu_count() or 1), p)
    mass = sf.Operator(sf.OP_MASS, degree=p, n_cells=nc)
    _check(torch, mass.vmult, x, O.cont_apply_op(m, O.OP_MASS, x), p)
    assert lap.device_status() == 0 and mass.device_status() == 0


def test_advect_48c_conserves_and_transports_constants():
    """size-independent properties at the bench's size, both kernels, FP64:
    the entries of A u sum to zero and A 1 = 0 on the periodic mesh (without
    and with the inverse mass)"""
    torch = torch_cuda()
    sf = _sf()
    p, nc, vel = 4, (48, 48, 48), (1.0, 0.5, 0.25)
    for invm in (0, 1):
        op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=nc, velocity=vel, inverse_mass=invm)
        gen = torch.Generator(device="cuda:0").manual_seed(invm)
        u = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=gen) * 2 - 1
        one = torch.ones_like(u)
        for variant in (sf.KERNEL_AUTO, sf.KERNEL_GENERIC):
            op.set_kernel_variant(variant)
            au, a1 = torch.empty_like(u), torch.empty_like(u)
            op.vmult(u, au)
            op.vmult(one, a1)
            torch.cuda.synchronize()
            if not invm:
                assert abs(float(au.sum())) < 1e-12 * float(au.abs().sum()), variant
            assert float(a1.abs().max()) < 1e-12 * float(au.abs().max()), (invm, variant)
        assert op.device_status() == 0
