"""Continuous mass matrix (SF_OP_MASS) and convection form (SF_OP_CONVECTION)
on the GPU through the C ABI: against the golden vectors of the reference's
DO_MASS_MATRIX / DO_CONVECTION builds (Hermite-like basis, velocity
(1, 2, 3), Dirichlet), against the oracle (GLL basis, degree 2, no
Dirichlet, other velocities), and size-independent identities at 48^3."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


@pytest.mark.parametrize("p", [1, 3, 4, 5, 6, 7, 8])
def test_cellops_golden(golden, p):
    torch = torch_cuda()
    sf = _sf()
    g = golden("cell_ops.npz")
    nc = tuple(int(v) for v in g["nc_%d" % p])
    length = tuple(float(v) for v in g["len_%d" % p])
    x = g["cont_x_%d" % p]
    for kind, key in ((sf.OP_MASS, "cont_mass_%d"), (sf.OP_CONVECTION, "cont_conv_%d")):
        op = sf.Operator(kind, degree=p, n_cells=nc, length=length, basis=sf.BASIS_HERMITE,
                         velocity=(1.0, 2.0, 3.0))
        for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 2 * FP32_TOL[p])):
            xd = to_dev(torch, x, dtype)
            y = torch.full_like(xd, float("nan"))
            op.vmult(xd, y)
            assert rel(to_np(y), g[key % p]) < tol, (kind, dtype)
        assert op.device_status() == 0


@pytest.mark.parametrize("dirichlet", [0, 1])
@pytest.mark.parametrize("p", [2, 4, 7])
def test_cellops_vs_oracle(p, dirichlet):
    """GLL basis, anisotropic box, odd cell counts, a general velocity"""
    torch = torch_cuda()
    sf = _sf()
    nc, length, b = (5, 3, 4), (1.0, 0.6, 0.9), (0.7, -1.3, 0.4)
    m = O.mesh(p, nc, length=length, dirichlet=dirichlet)
    x = np.random.default_rng(p + 10 * dirichlet).uniform(-1, 1, O.cont_n_dofs(m))
    for kind, ref in ((sf.OP_MASS, O.cont_apply_op(m, O.OP_MASS, x)),
                      (sf.OP_CONVECTION, O.cont_apply_op(m, O.OP_CONVECTION, x, b))):
        op = sf.Operator(kind, degree=p, n_cells=nc, length=length, dirichlet=dirichlet, velocity=b)
        for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 2 * FP32_TOL[p])):
            y = torch.empty(op.n_dofs, dtype=dtype, device="cuda:0")
            op.vmult(to_dev(torch, x, dtype), y)
            assert rel(to_np(y), ref) < tol, (kind, dtype)


def test_mass_identities_48():
    """48^3 cells, p=4 (12.2 M DoF), no Dirichlet: the mass matrix is
    symmetric positive definite and integrates constants to the volume; the
    convection form sums to zero over all test functions,
    sum_i (u, b . grad phi_i) = (u, b . grad 1) = 0"""
    torch = torch_cuda()
    sf = _sf()
    nc, length = (48, 48, 48), (1.0, 2.0, 0.5)
    mass = sf.Operator(sf.OP_MASS, degree=4, n_cells=nc, length=length, dirichlet=0)
    conv = sf.Operator(sf.OP_CONVECTION, degree=4, n_cells=nc, length=length, dirichlet=0,
                       velocity=(1.0, 0.5, 0.25))
    g = torch.Generator(device="cuda:0").manual_seed(3)
    x = torch.rand(mass.n_dofs, dtype=torch.float64, device="cuda:0", generator=g) - 0.5
    z = torch.rand(mass.n_dofs, dtype=torch.float64, device="cuda:0", generator=g) - 0.5
    mx, mz = torch.empty_like(x), torch.empty_like(z)
    mass.vmult(x, mx)
    mass.vmult(z, mz)
    assert abs(float(torch.dot(mx, z)) - float(torch.dot(x, mz))) < 1e-12 * float(mx.norm() * z.norm())
    assert float(torch.dot(mx, x)) > 0
    one, m1 = torch.ones_like(x), torch.empty_like(x)
    mass.vmult(one, m1)
    assert abs(float(m1.sum()) - 1.0) < 1e-12           # volume 1 x 2 x 0.5
    c = torch.empty_like(x)
    conv.vmult(x, c)
    assert abs(float(c.sum())) < 1e-11 * float(c.abs().sum())
    y32 = torch.empty(mass.n_dofs, dtype=torch.float32, device="cuda:0")
    mass.vmult(x.float(), y32)
    assert float((y32.double() - mx).norm() / mx.norm()) < 2 * FP32_TOL[4]


def test_cellops_unsupported():
    torch = torch_cuda()
    sf = _sf()
    with pytest.raises(sf.SFError) as e:
        sf.Operator(sf.OP_MASS, degree=3, n_cells=(4, 4, 4), deform=0.05)
    assert e.value.code == sf.SF_ERR_UNSUPPORTED
    op = sf.Operator(sf.OP_CONVECTION, degree=3, n_cells=(4, 4, 4))
    x = torch.zeros(op.n_dofs, dtype=torch.float64, device="cuda:0")
    y = torch.empty_like(x)
    with pytest.raises(sf.SFError) as e:
        op.vmult_transpose(x, y)
    assert e.value.code == sf.SF_ERR_UNSUPPORTED
    with pytest.raises(sf.SFError) as e:
        op.diagonal(y)
    assert e.value.code == sf.SF_ERR_UNSUPPORTED


def test_mass_cg_unpreconditioned():
    """CG on the mass matrix (SPD) without a preconditioner, FP64 and
    FP32-inner/FP64-refined"""
    torch = torch_cuda()
    sf = _sf()
    op = sf.Operator(sf.OP_MASS, degree=3, n_cells=(6, 5, 4), length=(1.0, 0.8, 0.7))
    b = torch.tensor(np.random.default_rng(5).standard_normal(op.n_dofs), device="cuda:0")
    for mode in (0, 1):
        x = torch.zeros_like(b)
        opts = sf.default_solve_opts(mode=mode, precond=0, rtol=1e-10)
        code, st = op.cg_solve(b, x, opts)
        assert code == 0, sf.lib().sf_last_error()
        r = torch.empty_like(x)
        op.vmult(x, r)
        assert float((r - b).norm() / b.norm()) < 1e-9


@pytest.mark.parametrize("basis", [0, 1])
@pytest.mark.parametrize("p", range(1, 9))
def test_affine_kronecker_passes_equal_line_kernel(p, basis):
    """The affine continuous Laplacian, mass and convection forms through the
    Kronecker passes (default) and the line-ownership kernel
    (SF_KERNEL_GENERIC): both against the oracle and each other, GLL and
    Hermite-like bases, with and without Dirichlet conditions, a
    one-cell-thick mesh and two right-hand sides"""
    torch = torch_cuda()
    sf = _sf()
    b = (0.7, -1.3, 0.4)
    for nc, length, dirichlet in (((5, 3, 4), (1.0, 0.6, 0.9), 1), ((1, 3, 2), (0.5, 1.0, 0.8), 0),
                                  ((2, 1, 3), (1.0, 0.4, 0.75), 1)):
        m = O.mesh(p, nc, basis=basis, length=length, dirichlet=dirichlet)
        N = O.cont_n_dofs(m)
        X = np.random.default_rng(p + 3 * basis + sum(nc)).uniform(-1, 1, 2 * N)
        for kind, okind in ((sf.OP_LAPLACE, None), (sf.OP_MASS, O.OP_MASS), (sf.OP_CONVECTION, O.OP_CONVECTION)):
            refs = [O.cont_apply(m, None, X[r * N:(r + 1) * N]) if okind is None
                    else O.cont_apply_op(m, okind, X[r * N:(r + 1) * N], b) for r in range(2)]
            op = sf.Operator(kind, degree=p, n_cells=nc, length=length, dirichlet=dirichlet, velocity=b,
                             basis=basis)
            out = {}
            for variant in (sf.KERNEL_AUTO, sf.KERNEL_GENERIC):
                op.set_kernel_variant(variant)
                for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 4 * FP32_TOL[p])):
                    y = torch.full((2 * N,), float("nan"), dtype=dtype, device="cuda:0")
                    op.vmult_batched(to_dev(torch, X, dtype), y, 2)
                    for r in range(2):
                        assert rel(to_np(y[r * N:(r + 1) * N]), refs[r]) < tol, (kind, nc, variant, dtype, r)
                    if dtype == torch.float64:
                        out[variant] = to_np(y)
            assert rel(out[sf.KERNEL_AUTO], out[sf.KERNEL_GENERIC]) < FP64_TOL, (kind, nc)
            assert op.device_status() == 0
