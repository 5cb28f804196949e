"""ctypes bindings of the reference's own code compiled here (oracle/_ref/).

TEST INFRASTRUCTURE ONLY, and only on the build host that has the reference
checkout: tests/golden/gen_golden.py uses it to write golden fixtures, and
the CPU tests use it, when present, to cross-check the oracle restatement.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_libs = {}
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def available() -> bool:
    return os.path.isdir(_build.REF_INC)


def _lib(name):
    if name not in _libs:
        path = os.path.join(_build.OUT_REF, "lib%s.so" % name)
        if not os.path.exists(path):
            _build.build_ref()
        _libs[name] = C.CDLL(path)
    return _libs[name]


def apply_1d(nn, type_, cor, add, do_dg, coef_eo, x, out_init=None, dg=None, face=None):
    L = _lib("ref_kernel")
    L.sfref_apply_1d.argtypes = [C.c_int] * 5 + [_dp, _dp, _dp, _dp, _dp]
    coef = np.zeros(nn * nn)
    coef[: len(coef_eo)] = coef_eo
    out = np.zeros(nn) if out_init is None else np.array(out_init, dtype=np.float64)
    dgv = np.zeros(2 * nn) if dg is None else np.array(dg, dtype=np.float64)
    fc = np.zeros(4) if face is None else np.array(face, dtype=np.float64)
    rc = L.sfref_apply_1d(nn, type_, int(cor), int(add), do_dg, coef,
                          np.ascontiguousarray(x, dtype=np.float64), out, dgv, fc)
    if rc != 0:
        raise ValueError("combination not instantiated")
    return out, fc


def gauss(n):
    L = _lib("ref_kernel")
    L.sfref_gauss.argtypes = [C.c_int, _dp, _dp]
    p, w = np.zeros(n), np.zeros(n)
    L.sfref_gauss(n, p, w)
    return p, w


def gll(n):
    L = _lib("ref_kernel")
    L.sfref_gll.argtypes = [C.c_int, _dp]
    p = np.zeros(n)
    L.sfref_gll(n, p)
    return p


def hermite(degree, x):
    L = _lib("ref_kernel")
    L.sfref_hermite.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
    x = np.ascontiguousarray(x, dtype=np.float64)
    v = np.zeros((degree + 1) * len(x))
    d = np.zeros_like(v)
    L.sfref_hermite(degree, len(x), x, v, d)
    return v.reshape(degree + 1, len(x)), d.reshape(degree + 1, len(x))


def gll_tables(degree):
    L = _lib("ref_cell_gll")
    L.sfref_gll_tables.argtypes = [C.c_int, _dp, _dp, _dp]
    n = degree + 1
    st = (n + 1) // 2
    s, d, w = np.zeros(n * st), np.zeros(n * st), np.zeros(n ** 3)
    L.sfref_gll_tables(degree, s, d, w)
    return s, d, w


def gll_cell(degree, G6, x):
    L = _lib("ref_cell_gll")
    L.sfref_gll_cell.argtypes = [C.c_int, _dp, _dp, _dp]
    out = np.zeros((degree + 1) ** 3)
    L.sfref_gll_cell(degree, np.ascontiguousarray(G6, dtype=np.float64),
                     np.ascontiguousarray(x, dtype=np.float64), out)
    return out


def herm_tables(degree):
    L = _lib("ref_cell_hermite")
    L.sfref_herm_tables.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
    n = degree + 1
    st = (n + 1) // 2
    s, d, w, h = np.zeros(n * st), np.zeros(n * st), np.zeros(n ** 3), np.zeros(1)
    L.sfref_herm_tables(degree, s, d, w, h)
    return s, d, w, h[0]


def herm_cell(degree, ij, jxw, x, variant=None):
    """the reference's Cartesian cell operator (Hermite-like basis): the
    Laplacian, or with variant "mass" / "convection" its DO_MASS_MATRIX /
    DO_CONVECTION build (convection velocity (1, 2, 3))"""
    L = _lib("ref_cell_hermite" if variant is None else "ref_cell_" + variant)
    L.sfref_herm_cell.argtypes = [C.c_int, _dp, C.c_double, _dp, _dp]
    out = np.zeros((degree + 1) ** 3)
    L.sfref_herm_cell(degree, np.ascontiguousarray(ij, dtype=np.float64), jxw,
                      np.ascontiguousarray(x, dtype=np.float64), out)
    return out


def dg_sipg(degree, n_cells, h, x, b=None, dinv=None, t=None, c_np=0.0, c_tm=0.0):
    L = _lib("ref_dg")
    L.sfref_dg_sipg.argtypes = [C.c_int, _ip, _dp, C.c_int, _dp, _dp, _dp, _dp,
                                C.c_double, C.c_double, _dp]
    N = len(x)
    mode = 0 if b is None else 1
    b = np.zeros(N) if b is None else np.ascontiguousarray(b, dtype=np.float64)
    dinv = np.zeros(N) if dinv is None else np.ascontiguousarray(dinv, dtype=np.float64)
    t = np.zeros(N) if t is None else np.array(t, dtype=np.float64)
    y = np.zeros(N)
    rc = L.sfref_dg_sipg(degree, np.array(n_cells, dtype=np.int32), np.array(h, dtype=np.float64),
                         mode, np.ascontiguousarray(x, dtype=np.float64), b, dinv, t, c_np, c_tm, y)
    assert rc == 0
    return (y, t) if mode else y


def dg_advect(degree, n_cells, h, x):
    L = _lib("ref_dg")
    L.sfref_dg_advect.argtypes = [C.c_int, _ip, _dp, _dp, _dp]
    y = np.zeros(len(x))
    rc = L.sfref_dg_advect(degree, np.array(n_cells, dtype=np.int32), np.array(h, dtype=np.float64),
                           np.ascontiguousarray(x, dtype=np.float64), y)
    assert rc == 0
    return y


def dg_rk_stage(degree, n_cells, h, src, upd, c_np, c_tm, vec_tm=None):
    """the reference's do_rk_stage<true>: returns (vec_np, vec_tm)"""
    L = _lib("ref_dg")
    L.sfref_dg_rk_stage.argtypes = [C.c_int, _ip, _dp, _dp, _dp, C.c_double, C.c_double, _dp, _dp]
    N = len(src)
    vnp = np.zeros(N)
    vtm = np.zeros(N) if vec_tm is None else np.array(vec_tm, dtype=np.float64)
    rc = L.sfref_dg_rk_stage(degree, np.array(n_cells, dtype=np.int32), np.array(h, dtype=np.float64),
                             np.ascontiguousarray(src, dtype=np.float64),
                             np.ascontiguousarray(upd, dtype=np.float64), c_np, c_tm, vnp, vtm)
    assert rc == 0
    return vnp, vtm


def dg_time_steps(degree, n_cells, h, x, nsteps, dt):
    """nsteps of the reference's do_time_step (LSRK(5,4)) from sol_new = x"""
    L = _lib("ref_dg")
    L.sfref_dg_time_steps.argtypes = [C.c_int, _ip, _dp, C.c_int, C.c_double, _dp]
    y = np.array(x, dtype=np.float64)
    rc = L.sfref_dg_time_steps(degree, np.array(n_cells, dtype=np.int32), np.array(h, dtype=np.float64),
                               nsteps, dt, y)
    assert rc == 0
    return y


def dg_precomputed(degree, n_cells, x):
    """the reference's PrecomputedDGLaplacian::matrix_vector_product (unit cells)"""
    L = _lib("ref_dg")
    L.sfref_dg_precomputed.argtypes = [C.c_int, _ip, _dp, _dp]
    y = np.zeros(len(x))
    rc = L.sfref_dg_precomputed(degree, np.array(n_cells, dtype=np.int32),
                                np.ascontiguousarray(x, dtype=np.float64), y)
    assert rc == 0
    return y


def dg_tables(degree):
    L = _lib("ref_dg")
    L.sfref_dg_tables.argtypes = [C.c_int, _dp, _dp]
    n = degree + 1
    st = (n + 1) // 2
    f, s = np.zeros(2 * n), np.zeros(n * st)
    L.sfref_dg_tables(degree, f, s)
    return f, s
