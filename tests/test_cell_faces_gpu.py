"""The DO_FACES builds of the cell operator (SF_OP_LAPLACE_FACES,
SF_OP_CONVECTION_FACES) on the GPU through the C ABI: against the golden
vectors of the reference's DO_FACES builds (one Cartesian cell with inverse
Jacobian diag(4, 2, 4/3), velocity (1, 2, 3)), against the oracle on
anisotropic multi-cell meshes (degree 2 included) and at 48^3 through the
block-diagonal structure."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


def _kinds(sf):
    return ((sf.OP_LAPLACE_FACES, False), (sf.OP_CONVECTION_FACES, True))


@pytest.mark.parametrize("p", [1, 3, 4, 5, 6, 7, 8])
def test_cell_faces_golden(golden, p):
    torch = torch_cuda()
    sf = _sf()
    g = golden("cell_ops.npz")
    x = g["cell_x_%d" % p]
    for kind, key in ((sf.OP_LAPLACE_FACES, "cell_faces_%d"), (sf.OP_CONVECTION_FACES, "cell_faces_conv_%d")):
        op = sf.Operator(kind, degree=p, n_cells=(1, 1, 1), length=(0.25, 0.5, 0.75), velocity=(1.0, 2.0, 3.0))
        assert op.n_dofs == (p + 1) ** 3
        for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 2 * FP32_TOL[p])):
            xd = to_dev(torch, x, dtype)
            y = torch.full_like(xd, float("nan"))
            op.vmult(xd, y)
            assert rel(to_np(y), g[key % p]) < tol, (kind, dtype)
        assert op.device_status() == 0


@pytest.mark.parametrize("p", [1, 2, 4, 7, 8])
def test_cell_faces_vs_oracle(p):
    """anisotropic cells, a general velocity, a partly filled last block,
    three right-hand sides in one launch"""
    torch = torch_cuda()
    sf = _sf()
    nc, length, b = (3, 2, 5), (0.9, 0.5, 1.3), (0.7, -1.3, 0.4)
    h = tuple(L / n for L, n in zip(length, nc))
    C = nc[0] * nc[1] * nc[2]
    N = C * (p + 1) ** 3
    X = np.random.default_rng(p).uniform(-1, 1, 3 * N)
    for kind, conv in _kinds(sf):
        op = sf.Operator(kind, degree=p, n_cells=nc, length=length, velocity=b)
        refs = [O.cell_faces_apply(p, conv, C, h, X[r * N:(r + 1) * N], b) for r in range(3)]
        for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 2 * FP32_TOL[p])):
            xd = to_dev(torch, X, dtype)
            y = torch.full_like(xd, float("nan"))
            op.vmult_batched(xd, y, 3)
            for r in range(3):
                assert rel(to_np(y[r * N:(r + 1) * N]), refs[r]) < tol, (kind, dtype, r)
            y1 = torch.empty(N, dtype=dtype, device="cuda:0")
            op.vmult(xd[N:2 * N].contiguous(), y1)
            assert torch.equal(y1, y[N:2 * N])
        assert op.device_status() == 0


@pytest.mark.parametrize("p", range(1, 9))
def test_cell_faces_line_operators_equal_face_kernel(p):
    """SF_OP_LAPLACE_FACES and SF_OP_CONVECTION_FACES through the line-operator
    kernel (default: sum_f L_f (x) M1 (x) M1, plus the rank-one face term of
    the Laplacian) and through the face-array kernel: both against the oracle
    and each other, two right-hand sides in one launch"""
    torch = torch_cuda()
    sf = _sf()
    nc, length, b = (3, 2, 5), (0.9, 0.5, 1.3), (0.7, -1.3, 0.4)
    h = tuple(L / n for L, n in zip(length, nc))
    C = nc[0] * nc[1] * nc[2]
    N = C * (p + 1) ** 3
    X = np.random.default_rng(70 + p).uniform(-1, 1, 2 * N)
    for kind, conv in _kinds(sf):
        refs = [O.cell_faces_apply(p, conv, C, h, X[r * N:(r + 1) * N], b) for r in range(2)]
        op = sf.Operator(kind, degree=p, n_cells=nc, length=length, velocity=b)
        out = {}
        for variant in (sf.KERNEL_AUTO, sf.KERNEL_GENERIC):
            op.set_kernel_variant(variant)
            for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 2 * FP32_TOL[p])):
                xd = to_dev(torch, X, dtype)
                y = torch.full_like(xd, float("nan"))
                op.vmult_batched(xd, y, 2)
                for r in range(2):
                    assert rel(to_np(y[r * N:(r + 1) * N]), refs[r]) < tol, (kind, variant, dtype, r)
                if dtype == torch.float64:
                    out[variant] = to_np(y)
        assert rel(out[sf.KERNEL_AUTO], out[sf.KERNEL_GENERIC]) < FP64_TOL, kind
        assert op.device_status() == 0


def test_cell_faces_block_diagonal_48():
    """48^3 cells, p=4 (13.8 M entries): cells do not couple (changing one
    cell's input changes that cell's output only, bit for bit elsewhere), and
    FP32 agrees with FP64"""
    torch = torch_cuda()
    sf = _sf()
    for kind, _ in _kinds(sf):
        op = sf.Operator(kind, degree=4, n_cells=(48, 48, 48), length=(1.0, 2.0, 0.5), velocity=(1.0, 0.5, 0.25))
        gen = torch.Generator(device="cuda:0").manual_seed(kind)
        x = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=gen) - 0.5
        y, y2 = torch.empty_like(x), torch.empty_like(x)
        op.vmult(x, y)
        e = 12345
        x2 = x.clone()
        x2[e * 125:(e + 1) * 125] = 0.0
        op.vmult(x2, y2)
        assert torch.equal(y[:e * 125], y2[:e * 125]) and torch.equal(y[(e + 1) * 125:], y2[(e + 1) * 125:])
        assert float(y2[e * 125:(e + 1) * 125].abs().max()) == 0.0
        y32 = torch.empty(op.n_dofs, dtype=torch.float32, device="cuda:0")
        op.vmult(x.float(), y32)
        assert float((y32.double() - y).norm() / y.norm()) < 2 * FP32_TOL[4]
        assert op.device_status() == 0


def test_cell_faces_unsupported_calls():
    torch = torch_cuda()
    sf = _sf()
    op = sf.Operator(sf.OP_LAPLACE_FACES, degree=3, n_cells=(2, 2, 2))
    x = torch.zeros(op.n_dofs, dtype=torch.float64, device="cuda:0")
    y = torch.empty_like(x)
    for call in (lambda: op.vmult_transpose(x, y), lambda: op.diagonal(y)):
        with pytest.raises(sf.SFError) as e:
            call()
        assert e.value.code == sf.SF_ERR_UNSUPPORTED
    with pytest.raises(sf.SFError) as e:
        op.chebyshev_step(x, x, x, y, torch.empty_like(x), 0.5, 0.5)
    assert e.value.code == sf.SF_ERR_UNSUPPORTED
    code, _ = op.cg_solve(x, y, sf.default_solve_opts(mode=0, precond=0))
    assert code == sf.SF_ERR_STATE
