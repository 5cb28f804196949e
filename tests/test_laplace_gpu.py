"""Continuous FE Laplacian on the GPU against the oracle and the golden
vectors of the reference's cell operator (through the C ABI)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


@pytest.mark.parametrize("p", range(1, 9))
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_affine_golden(golden, p, prec):
    torch = torch_cuda()
    sf = _sf()
    g = golden("cont.npz")
    nc = tuple(int(v) for v in g["nc_%d" % p])
    op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc, length=tuple(g["len_%d" % p]))
    dtype = torch.float64 if prec == "fp64" else torch.float32
    x = to_dev(torch, g["x_%d" % p], dtype)
    y = torch.empty_like(x)
    op.vmult(x, y)
    torch.cuda.synchronize()
    err = rel(to_np(y), g["y_%d" % p])
    assert err < (FP64_TOL if prec == "fp64" else FP32_TOL[p]), err


def test_q4_16_golden(golden):
    torch = torch_cuda()
    sf = _sf()
    g = golden("cont.npz")
    op = sf.Operator(sf.OP_LAPLACE, degree=4, n_cells=(16, 16, 16))
    x = np.random.default_rng(20241203).uniform(-1.0, 1.0, op.n_dofs)
    xd = to_dev(torch, x, torch.float64)
    yd = torch.empty_like(xd)
    op.vmult(xd, yd)
    y = to_np(yd)
    idx = g["q4_16_sample_idx"]
    assert rel(y[idx], g["q4_16_sample_y"]) < FP64_TOL
    assert abs(np.linalg.norm(y) - g["q4_16_norm2"][0]) < 1e-12 * g["q4_16_norm2"][0]


@pytest.mark.parametrize("p", range(1, 9))
@pytest.mark.parametrize("basis", [0, 1])
def test_deformed_vs_oracle(p, basis):
    torch = torch_cuda()
    sf = _sf()
    nc = (3, 2, 3) if p <= 5 else (2, 2, 2)
    L = (1.0, 0.7, 1.1)
    op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc, length=L, basis=basis, deform=0.05)
    m = O.mesh(p, nc, basis=basis, length=L, deform=0.05)
    x = np.random.default_rng(p).uniform(-1, 1, op.n_dofs)
    y_ref = O.cont_apply(m, O.cont_geometry(m), x)
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, FP32_TOL[p])):
        xd = to_dev(torch, x, dtype)
        yd = torch.empty_like(xd)
        op.vmult(xd, yd)
        assert rel(to_np(yd), y_ref) < tol


@pytest.mark.parametrize("p", [2, 4, 7])
def test_external_geometry_and_kappa(p):
    torch = torch_cuda()
    sf = _sf()
    nc = (2, 3, 2)
    m = O.mesh(p, nc, deform=0.08)
    G = O.cont_geometry(m)
    rng = np.random.default_rng(11)
    kappa = np.exp(0.5 * rng.standard_normal(np.prod(nc) * (p + 1) ** 3))
    op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc)
    op.set_geometry(to_dev(torch, G, torch.float64))
    op.set_coefficient(to_dev(torch, kappa, torch.float64))
    x = rng.uniform(-1, 1, op.n_dofs)
    y_ref = O.cont_apply(m, G, x, kappa=kappa)
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, FP32_TOL[p])):
        xd = to_dev(torch, x, dtype)
        yd = torch.empty_like(xd)
        op.vmult(xd, yd)
        assert rel(to_np(yd), y_ref) < tol


@pytest.mark.parametrize("p", [1, 3, 4, 8])
def test_kappa_gradient_vs_oracle(p):
    torch = torch_cuda()
    sf = _sf()
    nc = (2, 2, 3)
    op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc, deform=0.05)
    m = O.mesh(p, nc, deform=0.05)
    G = O.cont_geometry(m)
    rng = np.random.default_rng(5)
    u = rng.uniform(-1, 1, op.n_dofs)
    lam = rng.uniform(-1, 1, op.n_dofs)
    ref = O.cont_kappa_grad(m, G, u, lam)
    out = torch.empty(op.n_cells * (p + 1) ** 3, dtype=torch.float64, device="cuda:0")
    op.kappa_gradient(to_dev(torch, u, torch.float64), to_dev(torch, lam, torch.float64), out)
    assert rel(to_np(out), ref) < FP64_TOL


def test_symmetry_and_boundary_rows_large():
    """size-independent properties at a full-size-like case: <Ax,y> = <x,Ay>,
    identity boundary rows, zero row sums for interior rows on the
    constant function (no boundary)"""
    torch = torch_cuda()
    sf = _sf()
    op = sf.Operator(sf.OP_LAPLACE, degree=4, n_cells=(24, 20, 16), deform=0.05)
    g = torch.Generator(device="cuda:0").manual_seed(1)
    x = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=g) * 2 - 1
    y = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=g) * 2 - 1
    ax, ay = torch.empty_like(x), torch.empty_like(y)
    op.vmult(x, ax)
    op.vmult(y, ay)
    a, b = float(torch.dot(ax, y)), float(torch.dot(x, ay))
    assert abs(a - b) <= 1e-12 * max(abs(a), float(ax.norm() * y.norm()))
    op2 = sf.Operator(sf.OP_LAPLACE, degree=4, n_cells=(24, 20, 16), deform=0.05, dirichlet=0)
    one = torch.ones_like(x)
    r = torch.empty_like(x)
    op2.vmult(one, r)
    assert float(r.abs().max()) < 1e-12


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 8])
@pytest.mark.parametrize("case", ["deformed", "kappa", "affine", "neumann_odd"])
def test_fp32_kernels_vs_fp64(p, case):
    """the packed FP32 line kernel (several cells per warp group, so odd and
    unit cell counts leave partly filled groups) against the FP64 apply"""
    torch = torch_cuda()
    sf = _sf()
    nc = {"deformed": (7, 6, 5), "kappa": (5, 4, 6), "affine": (6, 5, 3), "neumann_odd": (1, 3, 5)}[case]
    op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc, length=(1.0, 0.9, 1.1),
                     deform=0.0 if case == "affine" else 0.05, dirichlet=0 if case == "neumann_odd" else 1)
    rng = np.random.default_rng(p)
    if case == "kappa":
        op.set_coefficient(to_dev(torch, np.exp(0.5 * rng.standard_normal(op.n_cells * (p + 1) ** 3)),
                                  torch.float64))
    x64 = to_dev(torch, rng.uniform(-1, 1, op.n_dofs), torch.float64)
    y64 = torch.empty_like(x64)
    op.vmult(x64, y64)
    x = x64.float()
    y = torch.full_like(x, float("nan"))
    op.vmult(x, y)
    torch.cuda.synchronize()
    assert rel(to_np(y), to_np(y64)) < FP32_TOL[p]
    assert op.device_status() == 0


def test_fp32_full_size_vs_fp64():
    """64^3 deformed p=4: FP32 applies against the FP64 apply, twice in a row
    (geometry staging and colour ordering are stateless)"""
    torch = torch_cuda()
    sf = _sf()
    op = sf.Operator(sf.OP_LAPLACE, degree=4, n_cells=(64, 64, 64), deform=0.05)
    g = torch.Generator(device="cuda:0").manual_seed(5)
    x64 = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=g) * 2 - 1
    y64 = torch.empty_like(x64)
    op.vmult(x64, y64)
    x32 = x64.float()
    for variant in (sf.KERNEL_AUTO, sf.KERNEL_GENERIC):
        op.set_kernel_variant(variant)
        for _ in range(2):
            y32 = torch.full_like(x32, float("nan"))
            op.vmult(x32, y32)
            assert float((y32.double() - y64).norm() / y64.norm()) < 3e-7
    assert op.device_status() == 0
