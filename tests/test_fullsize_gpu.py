"""The headline workload at its full size against the FP64 oracle: the
continuous Laplacian on the deformed 64^3 mesh, FP64 and FP32 applies on the
same vector as the oracle (whose cell operator is pinned to the reference's
by the golden vectors), degrees 2, 4 and 8.  At this size the persistent
walk runs many steps per group over full colour classes, and the 32-bit
in-plane node offsets reach their largest values of the benchmark."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_np, torch_cuda

pytestmark = pytest.mark.gpu

NC = 64
DEFORM = 0.05


@pytest.mark.parametrize("p", [2, 4, 8])
def test_deformed_64c_vs_oracle(p):
    torch = torch_cuda()
    from sum_factorization_kernels_gb300 import sfgpu as sf

    op = sf.Operator(sf.OP_LAPLACE, degree=p, n_cells=(NC,) * 3, deform=DEFORM)
    m = O.mesh(p, (NC,) * 3, deform=DEFORM)
    assert op.n_dofs == O.cont_n_dofs(m)
    x = np.random.default_rng(640 + p).uniform(-1, 1, op.n_dofs)
    # the oracle computes each cell's merged tensor where it uses it
    y_ref = O.cont_apply(m, None, x, n_threads=os.cpu_count() or 1)
    x64 = torch.from_numpy(x).to("cuda:0")
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, FP32_TOL[p])):
        xd = x64.to(dtype)
        y = torch.full_like(xd, float("nan"))
        op.vmult(xd, y)
        torch.cuda.synchronize()
        err = rel(to_np(y), y_ref)
        assert err < tol, (p, dtype, err)
    assert op.device_status() == 0
