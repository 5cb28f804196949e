"""DG SIPG Laplacian and DG upwind advection on the GPU against the golden
vectors of the reference's own DG evaluators and the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


def _lengths(nc, h):
    return tuple(float(n) * float(hh) for n, hh in zip(nc, h))


@pytest.mark.parametrize("p", [1, 3, 4, 5, 6, 7, 8])
def test_sipg_golden(golden, p):
    torch = torch_cuda()
    sf = _sf()
    g = golden("dg_sipg.npz")
    nc = tuple(int(v) for v in g["nc_%d" % p])
    op = sf.Operator(sf.OP_DG_SIPG, degree=p, n_cells=nc, length=_lengths(nc, g["h_%d" % p]))
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 4 * FP32_TOL[p])):
        x = to_dev(torch, g["x_%d" % p], dtype)
        y = torch.empty_like(x)
        op.vmult(x, y)
        assert rel(to_np(y), g["y_%d" % p]) < tol


def test_sipg_chebyshev_golden(golden):
    torch = torch_cuda()
    sf = _sf()
    g = golden("dg_sipg.npz")
    nc = tuple(int(v) for v in g["nc_5"])
    op = sf.Operator(sf.OP_DG_SIPG, degree=5, n_cells=nc, length=_lengths(nc, g["h_5"]))
    d = lambda a: to_dev(torch, a, torch.float64)  # noqa: E731
    b, dinv, x, t = d(g["cheb_b"]), d(g["cheb_dinv"]), d(g["x_5"]), d(g["cheb_t"])
    xn = torch.empty_like(x)
    op.chebyshev_step(b, dinv, x, xn, t, 0.7, 0.3)
    assert rel(to_np(xn), g["cheb_xnew"]) < FP64_TOL
    assert rel(to_np(t), g["cheb_tnew"]) < FP64_TOL


@pytest.mark.parametrize("p", range(1, 9))
@pytest.mark.parametrize("penalty", [1.0, 2.5])
def test_sipg_tensor_form_equals_cell_face_kernel(p, penalty):
    """SF_OP_DG_SIPG evaluated in tensor-product form (default) and by the
    cell-and-face kernel: the same operator, the same Chebyshev step and
    diagonal, both against the oracle (anisotropic cells, 1-cell-thick y)"""
    torch = torch_cuda()
    sf = _sf()
    nc, h = (4, 1, 3), (0.3, 0.2, 0.45)
    op = sf.Operator(sf.OP_DG_SIPG, degree=p, n_cells=nc, length=_lengths(nc, h), penalty=penalty)
    g = O.dg(p, nc, h, penalty=penalty)
    rng = np.random.default_rng(p)
    x = rng.standard_normal(op.n_dofs)
    y_ref = O.dg_sipg_apply(g, x)
    d_ref = O.dg_sipg_diagonal(g)
    b0, t0 = rng.standard_normal(op.n_dofs), rng.standard_normal(op.n_dofs)
    out = {}
    for variant in (sf.KERNEL_AUTO, sf.KERNEL_GENERIC):
        op.set_kernel_variant(variant)
        for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 4 * FP32_TOL[p])):
            xd = to_dev(torch, x, dtype)
            y = torch.empty_like(xd)
            op.vmult(xd, y)
            assert rel(to_np(y), y_ref) < tol, (variant, dtype)
            d = torch.empty_like(xd)
            op.diagonal(d)
            assert rel(to_np(d), d_ref) < tol, (variant, dtype)
        b = to_dev(torch, b0, torch.float64)
        dinv = 1.0 / to_dev(torch, d_ref, torch.float64)
        t = to_dev(torch, t0, torch.float64)
        xn = torch.empty_like(b)
        op.chebyshev_step(b, dinv, to_dev(torch, x, torch.float64), xn, t, 0.7, 0.3)
        out[variant] = (to_np(xn), to_np(t))
    assert rel(out[sf.KERNEL_AUTO][0], out[sf.KERNEL_GENERIC][0]) < FP64_TOL
    assert rel(out[sf.KERNEL_AUTO][1], out[sf.KERNEL_GENERIC][1]) < FP64_TOL
    assert op.device_status() == 0


@pytest.mark.parametrize("p", range(1, 9))
def test_advect_golden(golden, p):
    torch = torch_cuda()
    sf = _sf()
    g = golden("dg_advect.npz")
    nc = tuple(int(v) for v in g["nc_%d" % p])
    op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=nc, length=_lengths(nc, g["h_%d" % p]),
                     velocity=(1.0, 0.15, -0.05), inverse_mass=1)
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 4 * FP32_TOL[p])):
        x = to_dev(torch, g["x_%d" % p], dtype)
        y = torch.empty_like(x)
        op.vmult(x, y)
        assert rel(to_np(y), g["y_%d" % p]) < tol


@pytest.mark.parametrize("p", [1, 2, 4, 7])
@pytest.mark.parametrize("invm", [0, 1])
def test_advect_forward_transpose_vs_oracle(p, invm):
    torch = torch_cuda()
    sf = _sf()
    nc, h = (3, 4, 2), (0.25, 0.2, 0.4)
    vel = (1.0, 0.5, 0.25)
    op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=nc, length=_lengths(nc, h), velocity=vel,
                     inverse_mass=invm)
    d = O.dg(p, nc, h, velocity=vel, inverse_mass=invm)
    x = np.random.default_rng(p).uniform(-1, 1, op.n_dofs)
    xd = to_dev(torch, x, torch.float64)
    y = torch.empty_like(xd)
    op.vmult(xd, y)
    assert rel(to_np(y), O.dg_advect_apply(d, x)) < FP64_TOL
    op.vmult_transpose(xd, y)
    assert rel(to_np(y), O.dg_advect_apply_transpose(d, x)) < FP64_TOL


@pytest.mark.parametrize("p", range(1, 9))
def test_advect_line_operators_equal_cell_face_kernel(p):
    """SF_OP_DG_ADVECT through the line-operator kernel (default) and the
    cell-and-face kernel: forward and transpose with and without the inverse
    mass, three right-hand sides in one launch, a Runge-Kutta stage and a
    Chebyshev step; the applies against the oracle (anisotropic cells,
    one-cell-thick y, a negative velocity component)"""
    torch = torch_cuda()
    sf = _sf()
    nc, h, vel = (4, 1, 3), (0.3, 0.2, 0.45), (1.0, 0.5, -0.25)
    rng = np.random.default_rng(40 + p)
    for invm in (0, 1):
        op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=nc, length=_lengths(nc, h), velocity=vel,
                         inverse_mass=invm)
        g = O.dg(p, nc, h, velocity=vel, inverse_mass=invm)
        N = op.n_dofs
        x = rng.uniform(-1, 1, 3 * N)
        refs = [O.dg_advect_apply(g, x[r * N:(r + 1) * N]) for r in range(3)]
        refs_t = [O.dg_advect_apply_transpose(g, x[r * N:(r + 1) * N]) for r in range(3)]
        b0, t0, d0 = rng.uniform(-1, 1, N), rng.uniform(-1, 1, N), rng.uniform(0.5, 1, N)
        out = {}
        for variant in (sf.KERNEL_AUTO, sf.KERNEL_GENERIC):
            op.set_kernel_variant(variant)
            for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 4 * FP32_TOL[p])):
                xd = to_dev(torch, x, dtype)
                y = torch.empty_like(xd)
                op.vmult_batched(xd, y, 3)
                for r in range(3):
                    assert rel(to_np(y[r * N:(r + 1) * N]), refs[r]) < tol, (variant, invm, dtype, r)
                op.vmult_transpose_batched(xd, y, 3)
                for r in range(3):
                    assert rel(to_np(y[r * N:(r + 1) * N]), refs_t[r]) < tol, (variant, invm, dtype, r)
            xd = to_dev(torch, x, torch.float64)
            upd = to_dev(torch, b0, torch.float64).repeat(3)
            vnp, vtm = torch.empty_like(xd), torch.empty_like(xd)
            op.rk_stage(xd, upd, vnp, vtm, 0.3, -0.2, nrhs=3)
            xn, t = torch.empty(N, dtype=torch.float64, device="cuda:0"), to_dev(torch, t0, torch.float64)
            op.chebyshev_step(to_dev(torch, b0, torch.float64), to_dev(torch, d0, torch.float64),
                              xd[:N].contiguous(), xn, t, 0.7, 0.3)
            out[variant] = [to_np(v) for v in (vnp, vtm, xn, t)]
        for a_, b_ in zip(out[sf.KERNEL_AUTO], out[sf.KERNEL_GENERIC]):
            assert rel(a_, b_) < FP64_TOL, invm
        assert op.device_status() == 0


def test_advect_adjoint_dot_test_full_size():
    """<A x, y> = <x, A^T y> to 1e-12 (FP64) on the 48^3 p=4 mesh, 8 right-hand
    sides in one launch, with and without the inverse mass matrix"""
    torch = torch_cuda()
    sf = _sf()
    for invm in (1, 0):
        op = sf.Operator(sf.OP_DG_ADVECT, degree=4, n_cells=(48, 48, 48), velocity=(1.0, 0.5, 0.25),
                         inverse_mass=invm)
        N = op.n_dofs
        gen = torch.Generator(device="cuda:0").manual_seed(3)
        x = torch.rand(8 * N, dtype=torch.float64, device="cuda:0", generator=gen) * 2 - 1
        y = torch.rand(8 * N, dtype=torch.float64, device="cuda:0", generator=gen) * 2 - 1
        ax, aty = torch.empty_like(x), torch.empty_like(y)
        op.vmult_batched(x, ax, 8)
        op.vmult_transpose_batched(y, aty, 8)
        for r in range(8):
            s = slice(r * N, (r + 1) * N)
            lhs = float(torch.dot(ax[s], y[s]))
            rhs = float(torch.dot(x[s], aty[s]))
            scale = float(ax[s].norm() * y[s].norm())
            assert abs(lhs - rhs) <= 1e-12 * scale, (invm, r, lhs, rhs)
        # batched == single applies
        one = torch.empty(N, dtype=torch.float64, device="cuda:0")
        op.vmult(x[N:2 * N].contiguous(), one)
        assert torch.equal(one, ax[N:2 * N])


@pytest.mark.parametrize("p", [3, 5])
def test_sipg_diagonal_vs_oracle(p):
    torch = torch_cuda()
    sf = _sf()
    nc, h = (3, 2, 2), (0.3, 0.5, 0.2)
    op = sf.Operator(sf.OP_DG_SIPG, degree=p, n_cells=nc, length=_lengths(nc, h), penalty=1.5)
    ref = O.dg_sipg_diagonal(O.dg(p, nc, h, penalty=1.5))
    out = torch.empty(op.n_dofs, dtype=torch.float64, device="cuda:0")
    op.diagonal(out)
    assert rel(to_np(out), ref) < 1e-12


def test_sipg_symmetry_and_constant_nullspace():
    torch = torch_cuda()
    sf = _sf()
    op = sf.Operator(sf.OP_DG_SIPG, degree=5, n_cells=(24, 20, 16), length=(1.0, 0.8, 0.6))
    gen = torch.Generator(device="cuda:0").manual_seed(2)
    x = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=gen) * 2 - 1
    y = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=gen) * 2 - 1
    ax, ay = torch.empty_like(x), torch.empty_like(y)
    op.vmult(x, ax)
    op.vmult(y, ay)
    a, b = float(torch.dot(ax, y)), float(torch.dot(x, ay))
    assert abs(a - b) <= 1e-12 * float(ax.norm() * y.norm())
    op.vmult(torch.ones_like(x), ax)
    assert float(ax.abs().max()) < 1e-10 * float(ay.abs().max())
