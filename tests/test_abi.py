"""The C-ABI library loads and exports every function include/sfgpu.h
declares; argument validation works without touching a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lib():
    from sum_factorization_kernels_gb300 import _build, sfgpu
    if not os.path.exists(sfgpu.LIB_PATH):
        _build.build()
    return sfgpu, sfgpu.lib()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "sfgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sf_[a-z_0-9]+)\s*\(", src)))


def test_exports_every_declared_symbol():
    sfgpu, L = _lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(sfgpu.EXPORTS)


def test_validation_without_gpu():
    sfgpu, L = _lib()
    d = sfgpu.Desc()
    d.kind, d.degree = sfgpu.OP_LAPLACE, 9
    for k in range(3):
        d.n_cells[k], d.length[k] = 2, 1.0
    d.precisions = 3
    h = C.c_void_p()
    assert L.sf_create(C.byref(d), C.byref(h)) == -3  # degree 9 unsupported
    d.degree = 0
    assert L.sf_create(C.byref(d), C.byref(h)) == -3
    d.degree = 3
    d.n_cells[1] = 0
    assert L.sf_create(C.byref(d), C.byref(h)) == -1
    d.n_cells[1] = 2
    d.precisions = 0
    assert L.sf_create(C.byref(d), C.byref(h)) == -1
    assert L.sf_create(None, C.byref(h)) == -2
    assert L.sf_vmult(None, 0, None, None, None) == -2
    assert L.sf_destroy(None) == -2
    assert b"NULL" in L.sf_last_error()
    assert L.sf_convert(10, 0, None, 1, None, None) == -2
    assert L.sf_convert(10, 0, 8, 1, 6, None) == -8  # misaligned output
    assert L.sf_vector_update(-1, 0, 8, 8, 8, 8, 8, 8, 0.0, 0.0, None) == -1


def test_vector_update_overlap_rules_without_gpu():
    """outputs that overlap each other or an input are refused by address
    range before anything is launched (the addresses are never touched)"""
    _, L = _lib()
    n, es = 100, 8
    ax, b, dinv, xo, xn, t = (0x100000 + k * 0x1000 for k in range(6))

    def call(ax=ax, b=b, dinv=dinv, xo=xo, xn=xn, t=t):
        return L.sf_vector_update(n, 0, ax, b, dinv, xo, xn, t, 0.5, 0.5, None)

    assert call(t=xn) == -1 and b"x_new and t" in L.sf_last_error()
    assert call(t=xn + (n - 1) * es) == -1                     # last entry of x_new
    assert call(b=t + es) == -1 and b"t and b" in L.sf_last_error()
    assert call(xo=xn - es) == -1 and b"x_new and x_old" in L.sf_last_error()
    assert call(dinv=xn) == -1 and b"x_new and diag_inv" in L.sf_last_error()
    assert call(ax=xn + es) == -1 and b"x_new and ax" in L.sf_last_error()
    assert call(ax=t) == -1 and b"t and ax" in L.sf_last_error()


def test_shape_tables_match_oracle():
    import numpy as np
    from oracle import oracle as O
    sfgpu, _ = _lib()
    for p in range(1, 9):
        for basis in (0, 1):
            S, D, x, w = sfgpu.shape_tables(p, basis)
            a = O.shape_arrays(p, basis)
            assert np.abs(S - a["S"]).max() < 2e-15
            assert np.abs(D - a["D"]).max() < 2e-15 * np.abs(a["D"]).max()
            assert np.abs(x - a["xq"]).max() < 2e-16
            assert np.abs(w - a["wq"]).max() < 2e-15


def test_size_limits_without_gpu():
    """meshes past the index limits are refused before any device memory is
    touched: 2^31 cells, a continuous node plane block of 2^31 entries (the
    kernels' 32-bit node offsets), 2^40 vector entries"""
    sfgpu, L = _lib()
    h = C.c_void_p()

    def desc(kind, degree, nc):
        d = sfgpu.Desc()
        d.kind, d.degree, d.precisions, d.penalty = kind, degree, 3, 1.0
        for k in range(3):
            d.n_cells[k], d.length[k] = nc[k], 1.0
        return d

    for kind, degree, nc, what in ((sfgpu.OP_LAPLACE, 1, (2048, 2048, 512), b"2^31 - 1 cells"),
                                   (sfgpu.OP_LAPLACE, 8, (20000, 20000, 1), b"node plane"),
                                   (sfgpu.OP_DG_SIPG, 8, (1200, 1200, 1200), b"too large")):
        assert L.sf_create(C.byref(desc(kind, degree, nc)), C.byref(h)) == sfgpu.SF_ERR_INVALID, nc
        assert what in L.sf_last_error()
        assert not h.value


def test_unstructured_validation_without_gpu():
    """sf_create_unstructured checks its host arrays before any device work:
    node indices in range, each node once per cell, degree, basis, counts"""
    import numpy as np
    sfgpu, L = _lib()
    p, n3 = 1, 8
    idx = np.arange(2 * n3, dtype=np.int32)
    idx[n3:] -= 4                       # second cell shares a face with the first
    geo = np.zeros(2 * 6 * n3)
    h = C.c_void_p()

    def create(cells, n_cells=2, n_nodes=12, degree=p, basis=0, precisions=3, geometry=geo):
        return L.sf_create_unstructured(degree, basis, n_cells, n_nodes, cells.ctypes.data,
                                        None if geometry is None else geometry.ctypes.data, None,
                                        precisions, C.byref(h))

    assert create(idx, geometry=None) == sfgpu.SF_ERR_NULL
    assert create(idx, degree=9) == sfgpu.SF_ERR_UNSUPPORTED
    assert create(idx, basis=5) == sfgpu.SF_ERR_INVALID
    assert create(idx, n_cells=0) == sfgpu.SF_ERR_INVALID
    assert create(idx, n_nodes=0) == sfgpu.SF_ERR_INVALID
    assert create(idx, precisions=0) == sfgpu.SF_ERR_INVALID
    bad = idx.copy()
    bad[3] = 12
    assert create(bad) == sfgpu.SF_ERR_INVALID
    assert b"out of range" in L.sf_last_error()
    bad = idx.copy()
    bad[n3 + 5] = bad[n3 + 2]
    assert create(bad) == sfgpu.SF_ERR_INVALID
    assert b"same node twice" in L.sf_last_error()
    assert not h.value


def test_operator_kinds_without_gpu():
    """kinds past the enum and the unstructured kind are refused by sf_create
    before any device work; the face-term kinds pass the kind check and reach
    the degree check"""
    sfgpu, L = _lib()
    h = C.c_void_p()
    d = sfgpu.Desc()
    d.degree, d.precisions = 3, 3
    for k in range(3):
        d.n_cells[k], d.length[k] = 2, 1.0
    for kind in (-1, 9, 100):
        d.kind = kind
        assert L.sf_create(C.byref(d), C.byref(h)) == sfgpu.SF_ERR_INVALID, kind
    d.kind = sfgpu.OP_LAPLACE_UNSTRUCTURED
    assert L.sf_create(C.byref(d), C.byref(h)) == sfgpu.SF_ERR_INVALID
    assert b"sf_create_unstructured" in L.sf_last_error()
    d.degree = 9
    for kind in (sfgpu.OP_LAPLACE_FACES, sfgpu.OP_CONVECTION_FACES):
        d.kind = kind
        assert L.sf_create(C.byref(d), C.byref(h)) == sfgpu.SF_ERR_UNSUPPORTED, kind
    assert not h.value


def test_cpp_layer_builds_without_gpu(tmp_path):
    """the C++ driver of include/sfgpu.hpp (the reference's evaluator-class
    pattern) compiles without warnings and links against the library and
    the oracle; running it needs a GPU"""
    import subprocess
    from oracle import build as obuild
    sfgpu, _ = _lib()
    olib = obuild.build_oracle()
    cuda = "/usr/local/cuda"
    exe = str(tmp_path / "cpp_api_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle"), "-I", cuda + "/include",
           os.path.join(ROOT, "tests", "cpp", "cpp_api_check.cc"), "-o", exe,
           sfgpu.LIB_PATH, olib, "-L", cuda + "/lib64", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(exe)
    # the member templates that take the caller's vectors, in both modes
    src = tmp_path / "members.cc"
    src.write_text('#include "sfgpu.hpp"\n'
                   "void use(sfgpu::EvaluationDGAdvection<4, double> &e, sfgpu::EvaluationDGLaplacian<3, float> &l,\n"
                   "         sfgpu::DeviceVector<double> &v, sfgpu::DeviceVector<float> &w)\n"
                   "{\n"
                   "  e.do_rk_stage<true>(v, v, v, v, 0.0, 0.1, 0.2);\n"
                   "  e.do_rk_stage<false>(v, v, v, v, 0.0, 0.1, 0.2);\n"
                   "  l.do_cheby_iter<true>(w, w, w, w, w, 0.5f, 0.5f);\n"
                   "  l.do_cheby_iter<false>(w, w, w, w, w, 0.5f, 0.5f);\n"
                   "}\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I",
                        os.path.join(ROOT, "include"), "-I", cuda + "/include", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_python_vector_checks_without_gpu():
    """the Python layer refuses vectors the library could write past or
    misread (it cannot see buffer sizes): host tensors, non-contiguous views,
    the wrong precision, too few entries; None and integer addresses pass"""
    torch = pytest.importorskip("torch")
    sfgpu, _ = _lib()

    class FakeCuda:  # the attributes of a CUDA tensor that the check reads
        is_cuda = True

        def __init__(self, n, dtype, contiguous=True):
            self.n, self.dtype, self.contig = n, dtype, contiguous

        def is_contiguous(self):
            return self.contig

        def numel(self):
            return self.n

        def data_ptr(self):
            return 0x7000

    f64, f32 = torch.float64, torch.float32
    assert sfgpu.vec(None, 10, sfgpu.FP64, "x") is None
    assert sfgpu.vec(0x1234, 10, sfgpu.FP64, "x") == 0x1234
    assert sfgpu.vec(FakeCuda(10, f64), 10, sfgpu.FP64, "x") == 0x7000
    assert sfgpu.vec(FakeCuda(12, f32), 10, sfgpu.FP32, "x") == 0x7000
    with pytest.raises(ValueError, match="CUDA tensor"):
        sfgpu.vec(torch.zeros(10, dtype=f64), 10, sfgpu.FP64, "x")
    with pytest.raises(ValueError, match="contiguous"):
        sfgpu.vec(FakeCuda(10, f64, contiguous=False), 10, sfgpu.FP64, "x")
    with pytest.raises(TypeError, match="computes in float64"):
        sfgpu.vec(FakeCuda(10, f32), 10, sfgpu.FP64, "y")
    with pytest.raises(ValueError, match="holds 9 entries; this call needs 10"):
        sfgpu.vec(FakeCuda(9, f64), 10, sfgpu.FP64, "y")


def test_binding_arity_matches_header():
    """every ctypes signature of the Python layer has as many parameters as
    the prototype in include/sfgpu.h (a mismatch would shift arguments)"""
    _, L = _lib()
    src = open(os.path.join(ROOT, "include", "sfgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = re.findall(r"\b(sf_[a-z_0-9]+)\s*\(([^;{]*?)\)\s*;", src)
    assert len(protos) >= 20
    checked = 0
    for name, params in protos:
        params = " ".join(params.split())
        n = 0 if params in ("", "void") else params.count(",") + 1
        argtypes = getattr(getattr(L, name), "argtypes", None)
        if argtypes is None:
            continue
        assert len(argtypes) == n, (name, len(argtypes), n)
        checked += 1
    assert checked >= 20, checked
