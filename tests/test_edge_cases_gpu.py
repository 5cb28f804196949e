"""Edge cases on the GPU through the C ABI, against the oracle: meshes one
cell thick in some direction and the single-cell mesh, for every operator
kind.  On the continuous meshes most colour classes are then empty, the
packed kernels run partly filled cell groups, and with Dirichlet conditions
on a single cell of degree 1 every node is fixed (y = x).  On the periodic DG
meshes a cell is its own neighbour across the faces of a one-cell direction.
Unstructured meshes of one cell, a batch of one right-hand side, and calls
whose output overlaps another vector of the call."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu

MESHES = [(1, 1, 1), (1, 1, 4), (2, 1, 1), (1, 3, 1)]
H = (0.5, 0.4, 0.3)


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


def _length(nc):
    return tuple(n * h for n, h in zip(nc, H))


def _check(torch, op, x, ref, p, fp32_factor=2, transpose=False):
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, fp32_factor * FP32_TOL[p])):
        xd = to_dev(torch, x, dtype)
        y = torch.full_like(xd, float("nan"))
        (op.vmult_transpose if transpose else op.vmult)(xd, y)
        assert rel(to_np(y), ref) < tol, dtype
    assert op.device_status() == 0


@pytest.mark.parametrize("nc", MESHES)
@pytest.mark.parametrize("p", [1, 4, 8])
def test_continuous_thin_meshes(p, nc):
    torch = torch_cuda()
    sf = _sf()
    b = (0.7, -1.3, 0.4)
    rng = np.random.default_rng(p + 7 * sum(nc))
    for dirichlet in (0, 1):
        m = O.mesh(p, nc, length=_length(nc), deform=0.05, dirichlet=dirichlet)
        x = rng.uniform(-1, 1, O.cont_n_dofs(m))
        op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc, length=_length(nc), deform=0.05,
                         dirichlet=dirichlet)
        ref = O.cont_apply(m, O.cont_geometry(m), x)
        _check(torch, op, x, ref, p)
        if dirichlet and p == 1 and nc == (1, 1, 1):
            assert rel(ref, x) == 0.0                  # every node fixed
        ma = O.mesh(p, nc, length=_length(nc), dirichlet=dirichlet)
        for kind, okind in ((sf.OP_MASS, O.OP_MASS), (sf.OP_CONVECTION, O.OP_CONVECTION)):
            op = sf.Operator(kind, degree=p, n_cells=nc, length=_length(nc), dirichlet=dirichlet, velocity=b)
            _check(torch, op, x, O.cont_apply_op(ma, okind, x, b), p)


@pytest.mark.parametrize("nz", [16383, 16384])
def test_affine_plane_limit_of_kronecker_passes(nz):
    """the Kronecker passes of affine operators launch one x-y block per node
    plane, at most 65535 planes along z: p = 4 on 1 x 1 x 16383 cells (65533
    planes) runs them, 1 x 1 x 16384 (65537 planes) the line-ownership
    kernel; both precisions equal the oracle either way"""
    torch = torch_cuda()
    sf = _sf()
    p, nc = 4, (1, 1, nz)
    m = O.mesh(p, nc, length=_length(nc), dirichlet=1)
    x = np.random.default_rng(nz).uniform(-1, 1, O.cont_n_dofs(m))
    lap = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc, length=_length(nc))
    _check(torch, lap, x, O.cont_apply(m, None, x), p)
    mass = sf.Operator(sf.OP_MASS, degree=p, n_cells=nc, length=_length(nc))
    _check(torch, mass, x, O.cont_apply_op(m, O.OP_MASS, x), p)


@pytest.mark.parametrize("nc", MESHES)
@pytest.mark.parametrize("p", [1, 4, 8])
def test_dg_thin_meshes(p, nc):
    torch = torch_cuda()
    sf = _sf()
    vel = (1.0, 0.5, 0.25)
    d = O.dg(p, nc, H, penalty=1.5)
    x = np.random.default_rng(p + 11 * sum(nc)).uniform(-1, 1, O.dg_n_dofs(d))
    op = sf.Operator(sf.OP_DG_SIPG, degree=p, n_cells=nc, length=_length(nc), penalty=1.5)
    _check(torch, op, x, O.dg_sipg_apply(d, x), p, fp32_factor=4)
    op = sf.Operator(sf.OP_DG_PRECOMPUTED, degree=p, n_cells=nc, length=_length(nc))
    _check(torch, op, x, O.dg_precomputed_apply(O.dg(p, nc, H), x), p, fp32_factor=4)
    for invm in (0, 1):
        da = O.dg(p, nc, H, velocity=vel, inverse_mass=invm)
        op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=nc, length=_length(nc), velocity=vel,
                         inverse_mass=invm)
        _check(torch, op, x, O.dg_advect_apply(da, x), p, fp32_factor=4)
        _check(torch, op, x, O.dg_advect_apply_transpose(da, x), p, fp32_factor=4, transpose=True)


@pytest.mark.parametrize("p", [1, 3, 8])
def test_unstructured_single_cell(p):
    """one deformed cell, listed in a rotated and reflected frame with
    renumbered nodes, with and without Dirichlet nodes; both kernels"""
    torch = torch_cuda()
    sf = _sf()
    m = O.mesh(p, (1, 1, 1), length=(0.6, 0.5, 0.4), deform=0.05)
    G = O.cont_geometry(m).reshape(1, -1)
    idx, dmask = O.structured_as_unstructured(m)
    n, N = p + 1, O.cont_n_dofs(m)
    rng = np.random.default_rng(p)
    perm = rng.permutation(N)
    i2, g2 = O.reorient_cell(perm[idx[0]], G[0], n, np.array([2, 0, 1]), np.array([1, 0, 1]))
    d2 = np.empty(N, dtype=np.uint8)
    d2[perm] = dmask
    x = rng.uniform(-1, 1, N)
    for dm in (None, d2):
        ref = O.unstructured_apply(p, O.BASIS_GLL, i2[None], g2[None], N, x, dm)
        op = sf.Operator.unstructured(p, i2[None], g2[None], N, dirichlet=dm)
        _check(torch, op, x, ref, p)


def test_batch_of_one_equals_single_apply():
    torch = torch_cuda()
    sf = _sf()
    for kind, kw in ((sf.OP_LAPLACE, {"deform": 0.05}), (sf.OP_DG_SIPG, {}), (sf.OP_DG_ADVECT, {}),
                     (sf.OP_DG_PRECOMPUTED, {})):
        op = sf.Operator(kind, degree=3, n_cells=(3, 1, 2), length=(0.9, 0.3, 0.6), **kw)
        gen = torch.Generator(device="cuda:0").manual_seed(kind)
        for dtype in (torch.float64, torch.float32):
            x = (torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=gen) - 0.5).to(dtype)
            y1, yb = torch.empty_like(x), torch.empty_like(x)
            op.vmult(x, y1)
            op.vmult_batched(x, yb, 1)
            assert torch.equal(y1, yb), (kind, dtype)
        assert op.device_status() == 0


def test_overlapping_outputs_are_rejected():
    """an output that overlaps another vector of the call is refused with
    SF_ERR_INVALID before anything is launched (views into one buffer); the
    reference's in-place vector update (ax the same vector as x_new) runs
    and follows its formula"""
    torch = torch_cuda()
    sf = _sf()
    dev = "cuda:0"
    for kind, kw in ((sf.OP_LAPLACE, {"deform": 0.05}), (sf.OP_LAPLACE, {}), (sf.OP_DG_SIPG, {}),
                     (sf.OP_DG_ADVECT, {"inverse_mass": 1})):
        op = sf.Operator(kind, degree=2, n_cells=(2, 2, 2), **kw)
        n = op.n_dofs
        buf = torch.zeros(4 * n, dtype=torch.float64, device=dev)
        rejected = [
            lambda: op.vmult(buf[:n], buf[n // 2:n // 2 + n]),                 # y starts inside x
            lambda: op.vmult_transpose(buf[n // 2:n // 2 + n], buf[:n]),       # x starts inside y
            lambda: op.vmult_batched(buf[:2 * n], buf[n:3 * n], 2),            # second x is first y
        ]
        if kind == sf.OP_DG_ADVECT:
            rejected.append(lambda: op.vmult_transpose_batched(buf[:2 * n], buf[n:3 * n], 2))
        if kind != sf.OP_DG_ADVECT:
            b, d, t = (torch.ones(n, dtype=torch.float64, device=dev) for _ in range(3))
            x = buf[:n]
            rejected += [lambda: op.chebyshev_step(b, d, x, b, t, 0.5, 0.5),   # x_new is b
                         lambda: op.chebyshev_step(b, d, x, buf[n:2 * n], x, 0.5, 0.5),  # t is x_old
                         lambda: op.chebyshev_step(b, d, x, t, t, 0.5, 0.5)]   # x_new is t
        for call in rejected:
            with pytest.raises(sf.SFError) as e:
                call()
            assert e.value.code == sf.SF_ERR_INVALID and "overlap" in str(e.value)
        assert op.device_status() == 0
    g = torch.Generator(device=dev).manual_seed(5)
    ax, b, d, xo, t = (torch.rand(1000, dtype=torch.float64, device=dev, generator=g) for _ in range(5))
    t_ref = 0.6 * t + 0.45 * d * (ax - b)
    x_ref = xo - t_ref
    sf.vector_update(ax, b, d, xo, ax, t, 0.45, 0.6)
    torch.cuda.synchronize()
    assert float((t - t_ref).abs().max()) < 4e-15 and float((ax - x_ref).abs().max()) < 4e-15
    with pytest.raises(sf.SFError) as e:
        sf.vector_update(ax, b, d, xo, t, t, 0.45, 0.6)
    assert e.value.code == sf.SF_ERR_INVALID
