"""Continuous Laplacian on unstructured hexahedral meshes
(sf_create_unstructured) on the GPU: the structured deformed mesh written as
index arrays, renumbered and with every cell in a random local frame,
against the oracle and against the structured operator; batched applies and
CG without a preconditioner."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


def scrambled_mesh(p, nc, seed, basis=O.BASIS_GLL, deform=0.05, length=(1.0, 0.7, 0.9)):
    """structured deformed mesh as a renumbered, reoriented unstructured one"""
    m = O.mesh(p, nc, basis=basis, length=length, deform=deform)
    G = O.cont_geometry(m)
    N = O.cont_n_dofs(m)
    idx, dmask = O.structured_as_unstructured(m)
    n, ncell = p + 1, idx.shape[0]
    rng = np.random.default_rng(seed)
    perm_nodes = rng.permutation(N)
    perm_cells = rng.permutation(ncell)
    Gc = G.reshape(ncell, -1)
    idx2, G2 = np.empty_like(idx), np.empty_like(Gc)
    for new_e, e in enumerate(perm_cells):
        idx2[new_e], G2[new_e] = O.reorient_cell(perm_nodes[idx[e]], Gc[e], n, rng.permutation(3),
                                                 rng.integers(0, 2, 3))
    d2 = np.empty(N, dtype=np.uint8)
    d2[perm_nodes] = dmask
    return m, G, idx, dmask, idx2, G2, d2, perm_nodes


@pytest.mark.parametrize("p", [1, 2, 4, 6, 8])
def test_unstructured_vs_oracle_and_structured(p):
    torch = torch_cuda()
    sf = _sf()
    m, G, idx, dmask, idx2, G2, d2, perm = scrambled_mesh(p, (4, 3, 3), seed=p)
    N = O.cont_n_dofs(m)
    x = np.random.default_rng(100 + p).uniform(-1, 1, N)
    x2 = np.empty(N)
    x2[perm] = x
    ref2 = O.unstructured_apply(p, O.BASIS_GLL, idx2, G2, N, x2, d2)
    op = sf.Operator.unstructured(p, idx2, G2, N, dirichlet=d2)
    st = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=(4, 3, 3), length=(1.0, 0.7, 0.9), deform=0.05)
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, 2 * FP32_TOL[p])):
        y = torch.full((N,), float("nan"), dtype=dtype, device="cuda:0")
        op.vmult(to_dev(torch, x2, dtype), y)
        assert rel(to_np(y), ref2) < tol, dtype
        ys = torch.empty(N, dtype=dtype, device="cuda:0")
        st.vmult(to_dev(torch, x, dtype), ys)
        assert rel(to_np(y)[perm], to_np(ys)) < tol, dtype
    assert op.device_status() == 0


def test_unstructured_no_dirichlet_hermite_batched():
    torch = torch_cuda()
    sf = _sf()
    p = 3
    m, G, idx, dmask, idx2, G2, d2, perm = scrambled_mesh(p, (3, 3, 2), seed=7, basis=O.BASIS_HERMITE)
    N = O.cont_n_dofs(m)
    op = sf.Operator.unstructured(p, idx2, G2, N, dirichlet=None, basis=sf.BASIS_HERMITE)
    X = np.random.default_rng(8).uniform(-1, 1, 3 * N)
    xd = to_dev(torch, X, torch.float64)
    yd = torch.empty_like(xd)
    op.vmult_batched(xd, yd, 3)
    for r in range(3):
        ref = O.unstructured_apply(p, O.BASIS_HERMITE, idx2, G2, N, X[r * N:(r + 1) * N], None)
        assert rel(to_np(yd[r * N:(r + 1) * N]), ref) < FP64_TOL
    # no Dirichlet nodes: constants are in the null space
    one, r1 = torch.ones(N, dtype=torch.float64, device="cuda:0"), torch.empty(N, dtype=torch.float64,
                                                                             device="cuda:0")
    op.vmult(one, r1)
    assert float(r1.abs().max()) < 1e-12


def test_unstructured_cg_and_errors():
    torch = torch_cuda()
    sf = _sf()
    p = 2
    m, G, idx, dmask, idx2, G2, d2, perm = scrambled_mesh(p, (5, 4, 4), seed=3)
    N = O.cont_n_dofs(m)
    op = sf.Operator.unstructured(p, idx2, G2, N, dirichlet=d2)
    b = torch.tensor(np.random.default_rng(4).standard_normal(N), device="cuda:0")
    x = torch.zeros_like(b)
    code, st = op.cg_solve(b, x, sf.default_solve_opts(mode=1, precond=0, rtol=1e-10))
    assert code == 0, sf.lib().sf_last_error()
    r = torch.empty_like(x)
    op.vmult(x, r)
    assert float((r - b).norm() / b.norm()) < 1e-9
    with pytest.raises(sf.SFError) as e:
        op.diagonal(r)
    assert e.value.code == sf.SF_ERR_UNSUPPORTED
    bad = idx2.copy()
    bad[0, 0] = N
    with pytest.raises(sf.SFError) as e:
        sf.Operator.unstructured(p, bad, G2, N)
    assert e.value.code == sf.SF_ERR_INVALID
