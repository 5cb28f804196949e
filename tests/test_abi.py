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
