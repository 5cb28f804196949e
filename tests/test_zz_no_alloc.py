"""sf_vmult_transpose_static: the transposed advection apply for callers that
cannot allocate device memory while they run (applications that hand out all
device memory from their own pool or a fixed budget).  Its intermediate
vector lives in a fixed 4 MiB array inside the library.  The results must
match sf_vmult_transpose_batched on two calls in a row (the shared array
keeps the previous call's contents); sizes beyond the array and overlapping
vectors must be refused.

This file is collected last (test_zz_*) so that a failing run that stops at
the first failure has already run every other test."""
import pytest

from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_np, torch_cuda

pytestmark = pytest.mark.gpu


def test_static_scratch_transpose_matches_allocating_path():
    torch = torch_cuda()
    from sum_factorization_kernels_gb300 import sfgpu as sf
    p, nrhs = 3, 3
    op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=(6, 5, 4), length=(1.2, 1.0, 0.8),
                     velocity=(1.0, 0.5, 0.25), inverse_mass=1)
    N = op.n_dofs
    assert nrhs * N * 8 <= 4 << 20
    gen = torch.Generator(device="cuda:0").manual_seed(9)
    for dtype, tol in ((torch.float64, FP64_TOL), (torch.float32, FP32_TOL[p])):
        for call in range(2):  # two calls in a row share the static array
            x = (torch.rand(nrhs * N, device="cuda:0", generator=gen, dtype=torch.float64) * 2 - 1).to(dtype)
            y_ref = torch.empty_like(x)
            y_new = torch.full_like(x, float("nan"))
            op.vmult_transpose_batched(x, y_ref, nrhs)
            op.vmult_transpose_static(x, y_new, nrhs)
            torch.cuda.synchronize()
            assert torch.isfinite(y_new).all()
            assert rel(to_np(y_new), to_np(y_ref)) < tol, (dtype, call)


def test_static_scratch_rejects_oversized_requests():
    torch = torch_cuda()
    from sum_factorization_kernels_gb300 import sfgpu as sf
    op = sf.Operator(sf.OP_DG_ADVECT, degree=4, n_cells=(12, 12, 12), inverse_mass=1)
    N = op.n_dofs  # 216000 values: 1.7 MB in FP64, 8 right-hand sides exceed 4 MiB
    x = torch.zeros(8 * N, dtype=torch.float64, device="cuda:0")
    y = torch.zeros_like(x)
    code = sf.lib().sf_vmult_transpose_static(op._h, sf.FP64, 8, x.data_ptr(), y.data_ptr(), None)
    assert code == -1
    assert b"exceeds the static scratch" in sf.lib().sf_last_error()
    # y starting one entry into x
    assert sf.lib().sf_vmult_transpose_static(op._h, sf.FP64, 1, x.data_ptr(), x.data_ptr() + 8, None) == -1
    assert b"overlap" in sf.lib().sf_last_error()
    lap = sf.Operator(sf.OP_LAPLACE, degree=2, n_cells=(2, 2, 2))
    assert sf.lib().sf_vmult_transpose_static(lap._h, sf.FP64, 1, x.data_ptr(), y.data_ptr(), None) == -9
