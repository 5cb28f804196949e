"""Builds the C++ driver of include/sfgpu.hpp against libsfgpu.so and the
oracle, runs it on the GPU and checks its exit status."""
import os
import subprocess

import pytest

from tests.gpu_util import torch_cuda

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_evaluator_classes(tmp_path):
    torch_cuda()
    from oracle import build as obuild
    from sum_factorization_kernels_gb300 import _build
    lib = _build.build()
    olib = obuild.build_oracle()
    exe = str(tmp_path / "cpp_api_check")
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle"), "-I", cuda + "/include",
           os.path.join(ROOT, "tests", "cpp", "cpp_api_check.cc"), "-o", exe,
           lib, olib, "-L", cuda + "/lib64", "-lcudart",
           "-Wl,-rpath," + os.path.dirname(lib) + ":" + os.path.dirname(olib) + ":" + cuda + "/lib64"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
