"""ctypes bindings of the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; it is the oracle, never the product path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_lib = None

SFO_MAX_N = 10
BASIS_GLL, BASIS_HERMITE = 0, 1


class Shape(C.Structure):
    _fields_ = [
        ("degree", C.c_int), ("n", C.c_int), ("basis", C.c_int),
        ("xq", C.c_double * SFO_MAX_N), ("wq", C.c_double * SFO_MAX_N),
        ("xgll", C.c_double * SFO_MAX_N),
        ("S", C.c_double * (SFO_MAX_N * SFO_MAX_N)),
        ("D", C.c_double * (SFO_MAX_N * SFO_MAX_N)),
        ("Sinv", C.c_double * (SFO_MAX_N * SFO_MAX_N)),
        ("face_v", (C.c_double * SFO_MAX_N) * 2),
        ("face_d", (C.c_double * SFO_MAX_N) * 2),
        ("hermite_d0", C.c_double),
        ("S_eo", C.c_double * (SFO_MAX_N * SFO_MAX_N)),
        ("D_eo", C.c_double * (SFO_MAX_N * SFO_MAX_N)),
        ("Sinv_eo", C.c_double * (SFO_MAX_N * SFO_MAX_N)),
        ("face_eo", C.c_double * (2 * SFO_MAX_N)),
    ]


class Mesh(C.Structure):
    _fields_ = [("degree", C.c_int), ("basis", C.c_int), ("n_cells", C.c_int * 3),
                ("length", C.c_double * 3), ("deform", C.c_double),
                ("dirichlet", C.c_int)]


class DG(C.Structure):
    _fields_ = [("degree", C.c_int), ("n_cells", C.c_int * 3), ("h", C.c_double * 3),
                ("penalty", C.c_double), ("velocity", C.c_double * 3),
                ("inverse_mass", C.c_int)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def _load(path):
    L = C.CDLL(path)
    L.sfo_shape_init.argtypes = [C.c_int, C.c_int, C.POINTER(Shape)]
    L.sfo_apply_1d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp,
                               C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.sfo_cont_n_dofs.argtypes = [C.POINTER(Mesh)]
    L.sfo_cont_n_dofs.restype = C.c_longlong
    L.sfo_cont_geometry.argtypes = [C.POINTER(Mesh), _dp]
    L.sfo_cont_apply.argtypes = [C.POINTER(Mesh), C.c_void_p, C.c_void_p, _dp, _dp, C.c_int]
    L.sfo_cont_kappa_grad.argtypes = [C.POINTER(Mesh), _dp, _dp, _dp, _dp]
    L.sfo_cont_diagonal.argtypes = [C.POINTER(Mesh), _dp, C.c_void_p, _dp]
    L.sfo_cell_apply.argtypes = [C.POINTER(Shape), _dp, C.c_int, _dp, _dp]
    L.sfo_cell_op.argtypes = [C.POINTER(Shape), C.c_int, _dp, C.c_double, _dp, _dp, _dp]
    L.sfo_cell_faces.argtypes = [C.POINTER(Shape), C.c_int, _dp, C.c_double, _dp, _dp, _dp]
    L.sfo_cell_faces_apply.argtypes = [C.c_int, C.c_int, C.c_longlong, _dp, _dp, _dp, _dp]
    L.sfo_cont_apply_op.argtypes = [C.POINTER(Mesh), C.c_int, _dp, _dp, _dp]
    L.sfo_unstructured_apply.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_void_p,
                                         _dp, C.c_void_p, _dp, _dp]
    L.sfo_dg_n_dofs.argtypes = [C.POINTER(DG)]
    L.sfo_dg_n_dofs.restype = C.c_longlong
    for f in ("sfo_dg_sipg_apply", "sfo_dg_advect_apply", "sfo_dg_advect_apply_transpose"):
        getattr(L, f).argtypes = [C.POINTER(DG), _dp, _dp]
    L.sfo_dg_sipg_diagonal.argtypes = [C.POINTER(DG), _dp]
    L.sfo_dg_precomputed_apply.argtypes = [C.POINTER(DG), _dp, _dp]
    L.sfo_dg_precomputed_diagonal.argtypes = [C.POINTER(DG), _dp]
    L.sfo_dg_precomputed_matrices.argtypes = [C.c_int, _dp, _dp, _dp]
    L.sfo_dg_rk_stage.argtypes = [C.POINTER(DG), _dp, _dp, _dp, _dp, C.c_double, C.c_double]
    L.sfo_dg_lsrk_step.argtypes = [C.POINTER(DG), C.c_double, _dp, _dp, _dp]
    L.sfo_chebyshev_update.argtypes = [C.c_longlong, _dp, _dp, _dp, _dp, _dp, _dp,
                                       C.c_double, C.c_double]
    return L


def lib():
    """the strict build (-O2, ISO C: no floating-point contraction)"""
    global _lib
    if _lib is None:
        _lib = _load(_build.build_oracle())
    return _lib


_perf = None


def perf_lib():
    """the same source built for timing (-O3, host CPU tuning, contraction
    allowed): the CPU baseline; results agree with lib() to rounding"""
    global _perf
    if _perf is None:
        _perf = _load(_build.build_oracle_perf())
    return _perf


def shape(degree: int, basis: int = BASIS_GLL) -> Shape:
    s = Shape()
    if lib().sfo_shape_init(degree, basis, C.byref(s)) != 0:
        raise ValueError("unsupported degree %d" % degree)
    return s


def shape_arrays(degree: int, basis: int = BASIS_GLL) -> dict:
    s = shape(degree, basis)
    n = degree + 1
    st = (n + 1) // 2

    def mat(a):
        return np.array(a[: n * n], dtype=np.float64).reshape(n, n)

    return {
        "xq": np.array(s.xq[:n]), "wq": np.array(s.wq[:n]), "xgll": np.array(s.xgll[:n]),
        "S": mat(s.S), "D": mat(s.D), "Sinv": mat(s.Sinv),
        "face_v": np.array([s.face_v[0][:n], s.face_v[1][:n]]),
        "face_d": np.array([s.face_d[0][:n], s.face_d[1][:n]]),
        "hermite_d0": s.hermite_d0,
        "S_eo": np.array(s.S_eo[: n * st]), "D_eo": np.array(s.D_eo[: n * st]),
        "Sinv_eo": np.array(s.Sinv_eo[: n * st]), "face_eo": np.array(s.face_eo[: 2 * n]),
    }


def apply_1d(nn, type_, cor, add, coef_eo, x, out_init=None, do_dg=0, dg=None, face=None):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(nn) if out_init is None else np.array(out_init, dtype=np.float64)
    addp = out.ctypes.data if add else None
    dgp = np.ascontiguousarray(dg, dtype=np.float64) if dg is not None else None
    facep = np.zeros(4) if face is None else np.array(face, dtype=np.float64)
    lib().sfo_apply_1d(nn, 1, type_, int(cor), int(add), np.ascontiguousarray(coef_eo, dtype=np.float64),
                       x, out, addp, do_dg, dgp.ctypes.data if dgp is not None else None,
                       facep.ctypes.data)
    return out, facep


def mesh(degree, n_cells, basis=BASIS_GLL, length=(1.0, 1.0, 1.0), deform=0.0, dirichlet=1):
    m = Mesh()
    m.degree = degree
    m.basis = basis
    for d in range(3):
        m.n_cells[d] = n_cells[d]
        m.length[d] = length[d]
    m.deform = deform
    m.dirichlet = dirichlet
    return m


def cont_n_dofs(m: Mesh) -> int:
    return int(lib().sfo_cont_n_dofs(C.byref(m)))


def cont_geometry(m: Mesh) -> np.ndarray:
    n = m.degree + 1
    C_ = m.n_cells[0] * m.n_cells[1] * m.n_cells[2]
    G = np.zeros(C_ * 6 * n ** 3)
    lib().sfo_cont_geometry(C.byref(m), G)
    return G


def cont_apply(m: Mesh, G, x, kappa=None, n_threads=0, y=None, L=None):
    """y = A x; G None computes each cell's geometry on the fly (no
    [cell][6][n^3] array); L selects the library build (default: the
    strict build)"""
    y = np.zeros(cont_n_dofs(m)) if y is None else y
    k = np.ascontiguousarray(kappa, dtype=np.float64) if kappa is not None else None
    g = None if G is None else np.ascontiguousarray(G).ctypes.data
    (L or lib()).sfo_cont_apply(C.byref(m), g, k.ctypes.data if k is not None else None,
                                np.ascontiguousarray(x, dtype=np.float64), y, n_threads)
    return y


def cont_kappa_grad(m: Mesh, G, u, lam):
    n = m.degree + 1
    C_ = m.n_cells[0] * m.n_cells[1] * m.n_cells[2]
    dk = np.zeros(C_ * n ** 3)
    lib().sfo_cont_kappa_grad(C.byref(m), np.ascontiguousarray(G), np.ascontiguousarray(u, dtype=np.float64),
                              np.ascontiguousarray(lam, dtype=np.float64), dk)
    return dk


def cont_diagonal(m: Mesh, G, kappa=None):
    d = np.zeros(cont_n_dofs(m))
    k = np.ascontiguousarray(kappa, dtype=np.float64) if kappa is not None else None
    lib().sfo_cont_diagonal(C.byref(m), np.ascontiguousarray(G), k.ctypes.data if k is not None else None, d)
    return d


def cell_apply(degree, basis, G, x, geo_stride):
    s = shape(degree, basis)
    out = np.zeros((degree + 1) ** 3)
    lib().sfo_cell_apply(C.byref(s), np.ascontiguousarray(G, dtype=np.float64), geo_stride,
                         np.ascontiguousarray(x, dtype=np.float64), out)
    return out


OP_MASS, OP_CONVECTION = 1, 2


def cell_op(degree, basis, kind, ij, jxw, b, x):
    """mass (kind 1) or convection (kind 2) operator of one Cartesian cell"""
    s = shape(degree, basis)
    out = np.zeros((degree + 1) ** 3)
    lib().sfo_cell_op(C.byref(s), kind, np.ascontiguousarray(ij, dtype=np.float64), jxw,
                      np.ascontiguousarray(b, dtype=np.float64), np.ascontiguousarray(x, dtype=np.float64), out)
    return out


def cell_faces(degree, conv, ij, jxw, b, x):
    """the DO_FACES build of the Hermite-like cell operator: Cartesian
    Laplacian (conv False) or convection form (conv True) of one cell plus the
    face terms between its own faces at 0 and 1"""
    s = shape(degree, BASIS_HERMITE)
    out = np.zeros((degree + 1) ** 3)
    lib().sfo_cell_faces(C.byref(s), int(bool(conv)), np.ascontiguousarray(ij, dtype=np.float64), jxw,
                         np.ascontiguousarray(b, dtype=np.float64), np.ascontiguousarray(x, dtype=np.float64),
                         out)
    return out


def cell_faces_apply(degree, conv, n_cells, h, x, b=(0.0, 0.0, 0.0)):
    """cell_faces on every cell of a cell-major vector (n^3 entries per cell)
    with cell size h"""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib().sfo_cell_faces_apply(degree, int(bool(conv)), int(n_cells), np.ascontiguousarray(h, dtype=np.float64),
                               np.ascontiguousarray(b, dtype=np.float64), x, y)
    return y


def cont_apply_op(m: Mesh, kind, x, b=(0.0, 0.0, 0.0)):
    """mass (kind 1) or convection (kind 2) operator on the affine continuous mesh"""
    y = np.zeros(cont_n_dofs(m))
    lib().sfo_cont_apply_op(C.byref(m), kind, np.ascontiguousarray(b, dtype=np.float64),
                            np.ascontiguousarray(x, dtype=np.float64), y)
    return y


def unstructured_apply(degree, basis, idx, G, n_nodes, x, dirichlet=None):
    """Laplacian on an unstructured hexahedral mesh (idx int32 [cell][nq])"""
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    nq = (degree + 1) ** 3
    d = None if dirichlet is None else np.ascontiguousarray(dirichlet, dtype=np.uint8)
    y = np.zeros(n_nodes)
    lib().sfo_unstructured_apply(degree, basis, idx.size // nq, n_nodes, idx.ctypes.data,
                                 np.ascontiguousarray(G, dtype=np.float64),
                                 None if d is None else d.ctypes.data,
                                 np.ascontiguousarray(x, dtype=np.float64), y)
    return y


def structured_as_unstructured(m: Mesh):
    """index array [cell][nq] and Dirichlet mask of a structured mesh in the
    global lexicographic numbering (cells x fastest)"""
    p, n = m.degree, m.degree + 1
    nc = [m.n_cells[d] for d in range(3)]
    Nx, Ny, Nz = p * nc[0] + 1, p * nc[1] + 1, p * nc[2] + 1
    c, b, a = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    k, j, i = np.meshgrid(np.arange(nc[2]), np.arange(nc[1]), np.arange(nc[0]), indexing="ij")
    X = (i.ravel()[:, None] * p + a.ravel()[None, :])
    Y = (j.ravel()[:, None] * p + b.ravel()[None, :])
    Z = (k.ravel()[:, None] * p + c.ravel()[None, :])
    idx = ((Z * Ny + Y) * Nx + X).astype(np.int32)
    N = Nx * Ny * Nz
    dmask = np.zeros(N, dtype=np.uint8)
    if m.dirichlet:
        g = np.arange(N)
        Xg, Yg, Zg = g % Nx, (g // Nx) % Ny, g // (Nx * Ny)
        dmask[(Xg == 0) | (Yg == 0) | (Zg == 0) | (Xg == Nx - 1) | (Yg == Ny - 1) | (Zg == Nz - 1)] = 1
    return idx, dmask


def reorient_cell(idx_e, G_e, n, perm, flips):
    """the same cell described in another local frame: new axis d is old
    axis perm[d], reflected when flips[d]; returns the node indices and the
    merged tensor (P^T G P per point) in the new frame"""
    Gm = np.zeros((n, n, n, 3, 3))
    g = G_e.reshape(6, n, n, n)
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    for e, (r, s) in enumerate(pairs):
        Gm[..., r, s] = g[e]
        Gm[..., s, r] = g[e]
    P = np.zeros((3, 3))
    for d in range(3):
        P[perm[d], d] = -1.0 if flips[d] else 1.0
    old = idx_e.reshape(n, n, n)
    new_idx = np.zeros_like(old)
    new_G = np.zeros((6, n, n, n))
    for cz in range(n):
        for cy in range(n):
            for cx in range(n):
                newc = (cx, cy, cz)
                oldc = [0, 0, 0]
                for d in range(3):
                    v = newc[d]
                    oldc[perm[d]] = n - 1 - v if flips[d] else v
                ox, oy, oz = oldc
                new_idx[cz, cy, cx] = old[oz, oy, ox]
                Gn = P.T @ Gm[oz, oy, ox] @ P
                for e, (r, s) in enumerate(pairs):
                    new_G[e, cz, cy, cx] = Gn[r, s]
    return new_idx.ravel(), new_G.ravel()


def dg(degree, n_cells, h, penalty=1.0, velocity=(1.0, 0.5, 0.25), inverse_mass=1):
    g = DG()
    g.degree = degree
    for d in range(3):
        g.n_cells[d] = n_cells[d]
        g.h[d] = h[d]
        g.velocity[d] = velocity[d]
    g.penalty = penalty
    g.inverse_mass = inverse_mass
    return g


def dg_n_dofs(g: DG) -> int:
    return int(lib().sfo_dg_n_dofs(C.byref(g)))


def _dg_call(name, g, x, L=None, y=None):
    y = np.zeros(dg_n_dofs(g)) if y is None else y
    getattr(L or lib(), name)(C.byref(g), np.ascontiguousarray(x, dtype=np.float64), y)
    return y


def dg_sipg_apply(g, x, L=None, y=None):
    return _dg_call("sfo_dg_sipg_apply", g, x, L, y)


def dg_advect_apply(g, x, L=None, y=None):
    return _dg_call("sfo_dg_advect_apply", g, x, L, y)


def dg_advect_apply_transpose(g, x):
    return _dg_call("sfo_dg_advect_apply_transpose", g, x)


def dg_precomputed_apply(g, x):
    return _dg_call("sfo_dg_precomputed_apply", g, x)


def dg_precomputed_diagonal(g):
    d = np.zeros(dg_n_dofs(g))
    lib().sfo_dg_precomputed_diagonal(C.byref(g), d)
    return d


def dg_precomputed_matrices(degree):
    n = degree + 1
    M, L, iv = np.zeros(n * n), np.zeros(n * n), np.zeros(2)
    lib().sfo_dg_precomputed_matrices(degree, M, L, iv)
    return M.reshape(n, n), L.reshape(n, n), iv


def dg_rk_stage(g, src, upd, vec_np, vec_tm, c_np, c_tm):
    """fused Runge-Kutta stage, vec_np / vec_tm updated in place (float64
    contiguous arrays; upd may be the same array as vec_np or vec_tm)"""
    lib().sfo_dg_rk_stage(C.byref(g), src, upd, vec_np, vec_tm, c_np, c_tm)


def dg_lsrk_step(g, dt, sol_new, sol_old, sol_tmp):
    """one LSRK(5,4) step, all three arrays updated in place"""
    lib().sfo_dg_lsrk_step(C.byref(g), dt, sol_new, sol_old, sol_tmp)


def dg_sipg_diagonal(g):
    d = np.zeros(dg_n_dofs(g))
    lib().sfo_dg_sipg_diagonal(C.byref(g), d)
    return d


def chebyshev_update(ax, b, dinv, x_old, t, c_np, c_tm):
    x_new = np.zeros_like(x_old)
    t = np.array(t, dtype=np.float64)
    lib().sfo_chebyshev_update(len(x_old), ax, b, dinv, x_old, x_new, t, c_np, c_tm)
    return x_new, t
