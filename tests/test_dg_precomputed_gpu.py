"""Tensor-product DG SIPG Laplacian with precomputed 1D matrices
(SF_OP_DG_PRECOMPUTED) on the GPU through the C ABI, against the golden
vectors of the reference's PrecomputedDGLaplacian (couplings corrected),
the oracle, and size-independent identities at full size."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


def _op(sf, p, nc, h=(1.0, 1.0, 1.0)):
    return sf.Operator(sf.OP_DG_PRECOMPUTED, degree=p, n_cells=nc,
                       length=tuple(n * hh for n, hh in zip(nc, h)))


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6, 8])
def test_precomputed_golden(golden, p):
    torch = torch_cuda()
    sf = _sf()
    g = golden("dg_precomputed.npz")
    nc = tuple(int(v) for v in g["nc_%d" % p])
    op = _op(sf, p, nc)
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 4 * FP32_TOL[p])):
        x = to_dev(torch, g["x_%d" % p].astype(np.float64), dtype)
        y = torch.full_like(x, float("nan"))
        op.vmult(x, y)
        assert rel(to_np(y), g["y_%d" % p]) < tol
    assert op.device_status() == 0


@pytest.mark.parametrize("p", [2, 4, 7])
def test_precomputed_anisotropic_vs_oracle(p):
    """anisotropic cells, odd and unit cell counts (wrap-around onto the
    cell itself), both precisions; transpose = apply (symmetric)"""
    torch = torch_cuda()
    sf = _sf()
    nc, h = (5, 1, 3), (0.3, 0.7, 0.45)
    op = _op(sf, p, nc, h)
    d = O.dg(p, nc, h)
    x = np.random.default_rng(p).uniform(-1, 1, O.dg_n_dofs(d))
    ref = O.dg_precomputed_apply(d, x)
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 4 * FP32_TOL[p])):
        xd = to_dev(torch, x, dtype)
        y, yt = torch.empty_like(xd), torch.empty_like(xd)
        op.vmult(xd, y)
        op.vmult_transpose(xd, yt)
        assert rel(to_np(y), ref) < tol
        assert float((y - yt).abs().max()) == 0.0


def test_precomputed_batched_diagonal_chebyshev():
    torch = torch_cuda()
    sf = _sf()
    p, nc, h = 3, (4, 3, 2), (0.5, 0.4, 0.6)
    op = _op(sf, p, nc, h)
    d = O.dg(p, nc, h)
    n = O.dg_n_dofs(d)
    rng = np.random.default_rng(11)
    X = rng.uniform(-1, 1, 3 * n)
    xd = to_dev(torch, X, torch.float64)
    yd = torch.empty_like(xd)
    op.vmult_batched(xd, yd, 3)
    for r in range(3):
        assert rel(to_np(yd[r * n:(r + 1) * n]), O.dg_precomputed_apply(d, X[r * n:(r + 1) * n])) < FP64_TOL
    diag = torch.empty(n, dtype=torch.float64, device="cuda:0")
    op.diagonal(diag)
    assert rel(to_np(diag), O.dg_precomputed_diagonal(d)) < FP64_TOL
    # fused Chebyshev step: t <- c_tm t + c_np D^-1 (A x_old - b); x_new = x_old - t
    b, t0, xo = rng.standard_normal(n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    dinv = 1.0 / O.dg_precomputed_diagonal(d)
    xn_ref, t_ref = O.chebyshev_update(O.dg_precomputed_apply(d, xo), b, dinv, xo, t0, 0.7, 0.3)
    tt = to_dev(torch, t0, torch.float64)
    xn = torch.empty(n, dtype=torch.float64, device="cuda:0")
    op.chebyshev_step(to_dev(torch, b, torch.float64), to_dev(torch, dinv, torch.float64),
                      to_dev(torch, xo, torch.float64), xn, tt, 0.7, 0.3)
    assert rel(to_np(xn), xn_ref) < FP64_TOL
    assert rel(to_np(tt), t_ref) < FP64_TOL


def test_precomputed_full_size_identities():
    """48^3 cells, p=5 (23.9 M DoF): constants in the null space,
    <A x, z> = <x, A z>, FP32 against FP64"""
    torch = torch_cuda()
    sf = _sf()
    op = _op(sf, 5, (48, 48, 48), (1.0 / 48,) * 3)
    g = torch.Generator(device="cuda:0").manual_seed(7)
    x = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=g) - 0.5
    z = torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=g) - 0.5
    ax, az = torch.empty_like(x), torch.empty_like(z)
    op.vmult(x, ax)
    op.vmult(z, az)
    s = float(torch.dot(ax, z))
    assert abs(s - float(torch.dot(x, az))) < 1e-11 * float(ax.norm() * z.norm())
    one, r = torch.ones_like(x), torch.empty_like(x)
    op.vmult(one, r)
    assert float(r.abs().max()) < 1e-10 * float(ax.abs().max())
    y32 = torch.empty(op.n_dofs, dtype=torch.float32, device="cuda:0")
    op.vmult(x.float(), y32)
    assert float((y32.double() - ax).norm() / ax.norm()) < 4 * FP32_TOL[5]
    assert op.device_status() == 0


@pytest.mark.parametrize("mode", [0, 1])
def test_precomputed_cg_periodic(mode):
    """CG with Chebyshev preconditioning on the diagonal, FP64 and
    FP32-inner/FP64-refined, mean-free right-hand side"""
    torch = torch_cuda()
    sf = _sf()
    op = _op(sf, 4, (8, 8, 8), (1.0 / 8,) * 3)
    b = torch.tensor(np.random.default_rng(3).standard_normal(op.n_dofs), device="cuda:0")
    x = torch.zeros_like(b)
    opts = sf.default_solve_opts(mode=mode, precond=2, rtol=1e-10, project_constant=1)
    code, st = op.cg_solve(b, x, opts)
    assert code == 0, sf.lib().sf_last_error()
    assert st.rel_residual <= 1e-10
    bp = b - b.mean()
    r = torch.empty_like(x)
    op.vmult(x, r)
    assert float((r - bp).norm() / bp.norm()) < 1e-9
