"""Helpers for the GPU parity tests (device placement, error norms)."""
import numpy as np
import pytest


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def to_dev(torch, x, dtype):
    return torch.tensor(np.asarray(x), dtype=dtype, device="cuda:0")


def to_np(t):
    return t.detach().double().cpu().numpy()


# relative tolerance of an FP32 operator apply against the FP64 oracle, per
# degree (random input; measured errors are 2-5x below these)
FP32_TOL = {1: 2e-6, 2: 2e-6, 3: 3e-6, 4: 3e-6, 5: 4e-6, 6: 5e-6, 7: 6e-6, 8: 8e-6}
FP64_TOL = 1e-12
