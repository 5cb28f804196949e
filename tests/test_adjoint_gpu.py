"""Hand-written adjoint of the variable-coefficient Laplacian: dL/dx and
dL/dkappa of L = 1/2 |A(kappa) x - b|^2 against central finite differences
(step 1e-6, FP64) and against the gradient assembled on the CPU by the
oracle; the torch.autograd wrapper passes gradcheck."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


def test_gradcheck_small():
    torch = torch_cuda()
    sf = _sf()
    from sum_factorization_kernels_gb300.autograd import laplace_apply
    p, nc = 2, (2, 2, 1)
    op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc, deform=0.05, precisions=1)
    g = torch.Generator(device="cuda:0").manual_seed(0)
    x = (torch.rand(op.n_dofs, dtype=torch.float64, device="cuda:0", generator=g) - 0.5).requires_grad_()
    k = torch.exp(0.5 * torch.randn(op.n_cells * (p + 1) ** 3, dtype=torch.float64, device="cuda:0",
                                    generator=g)).requires_grad_()
    assert torch.autograd.gradcheck(lambda xx, kk: laplace_apply(op, xx, kk), (x, k), eps=1e-6,
                                    atol=1e-7, rtol=1e-6)


def test_config4_full_size_gradients():
    """p=4, 32^3 deformed cells, kappa log-normal(0, 0.5) per Gauss point"""
    torch = torch_cuda()
    sf = _sf()
    from sum_factorization_kernels_gb300.autograd import laplace_apply
    p, nc = 4, (32, 32, 32)
    op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=nc, deform=0.05, precisions=1)
    rng = np.random.default_rng(20241203)
    nq = op.n_cells * (p + 1) ** 3
    kappa = np.exp(0.5 * rng.standard_normal(nq))
    x = rng.uniform(-1, 1, op.n_dofs)
    b = rng.uniform(-1, 1, op.n_dofs)
    xd = to_dev(torch, x, torch.float64).requires_grad_()
    kd = to_dev(torch, kappa, torch.float64).requires_grad_()
    bd = to_dev(torch, b, torch.float64)

    def loss(xx, kk):
        r = laplace_apply(op, xx, kk) - bd
        return 0.5 * torch.dot(r, r)

    L = loss(xd, kd)
    gx, gk = torch.autograd.grad(L, (xd, kd))
    # CPU-assembled reference gradient (oracle): r = A x - b, dL/dx = A r,
    # dL/dkappa = grad x . G grad r
    m = O.mesh(p, nc, deform=0.05)
    G = O.cont_geometry(m)
    r = O.cont_apply(m, G, x, kappa=kappa) - b
    assert rel(to_np(gx), O.cont_apply(m, G, r, kappa=kappa)) < 1e-12
    assert rel(to_np(gk), O.cont_kappa_grad(m, G, x, r)) < 1e-12
    # central differences, step 1e-6 (relative), on sampled entries.  The
    # difference L(+) - L(-) = 1/2 (r+ - r-).(r+ + r-) is evaluated in that
    # form: the two residuals differ only near the perturbed entry, so the
    # difference carries no cancellation error of the full-size sums.
    def resid(xx, kk):
        with torch.no_grad():
            return laplace_apply(op, xx, kk) - bd

    def central(xp, kp, xm, km, h):
        rp, rm = resid(xp, kp), resid(xm, km)
        return 0.5 * float(torch.dot(rp - rm, rp + rm)) / (2 * h)

    x0, k0 = xd.detach(), kd.detach()
    for q in rng.choice(nq, 6, replace=False):
        h = 1e-6 * kappa[q]
        kp, km = k0.clone(), k0.clone()
        kp[q] += h
        km[q] -= h
        fd = central(x0, kp, x0, km, h)
        assert abs(fd - float(gk[q])) <= 1e-6 * max(abs(fd), 1e-3 * float(gk.abs().max())), q
    picks = [int(i) for i in rng.choice(op.n_dofs, 400, replace=False)]
    interior = [i for i in picks if abs(float(gx[i])) > 1e-3 * float(gx.abs().max())][:6]
    assert interior
    for i in interior:
        h = 1e-6
        xp, xm = x0.clone(), x0.clone()
        xp[i] += h
        xm[i] -= h
        fd = central(xp, k0, xm, k0, h)
        assert abs(fd - float(gx[i])) <= 1e-6 * max(abs(fd), 1e-3 * float(gx.abs().max())), i
