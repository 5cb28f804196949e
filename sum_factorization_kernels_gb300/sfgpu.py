"""ctypes binding of the sfgpu C ABI (include/sfgpu.h).

Loads the in-tree ``libsfgpu.so`` built for sm_103a and fails loudly when it
is missing: there is no CPU fallback.  Arrays are passed as device pointers:
a CUDA ``torch.Tensor`` (checked to be contiguous, of the call's precision
and long enough, since the library cannot see buffer sizes) or an integer
address (passed on unchecked).  PyTorch is only the allocator here.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsfgpu.so")

SF_OK = 0
STATUS = {0: "SF_OK", -1: "SF_ERR_INVALID", -2: "SF_ERR_NULL", -3: "SF_ERR_UNSUPPORTED",
          -4: "SF_ERR_CUDA", -5: "SF_ERR_OOM", -6: "SF_ERR_NOT_CONVERGED",
          -7: "SF_ERR_BREAKDOWN", -8: "SF_ERR_ALIGN", -9: "SF_ERR_STATE"}
(SF_ERR_INVALID, SF_ERR_NULL, SF_ERR_UNSUPPORTED, SF_ERR_CUDA, SF_ERR_OOM, SF_ERR_NOT_CONVERGED,
 SF_ERR_BREAKDOWN, SF_ERR_ALIGN, SF_ERR_STATE) = range(-1, -10, -1)
FP64, FP32 = 0, 1
OP_LAPLACE, OP_DG_SIPG, OP_DG_ADVECT, OP_DG_PRECOMPUTED, OP_MASS, OP_CONVECTION = 0, 1, 2, 3, 4, 5
OP_LAPLACE_UNSTRUCTURED = 6
OP_LAPLACE_FACES, OP_CONVECTION_FACES = 7, 8   # DO_FACES builds, cell-major vectors
BASIS_GLL, BASIS_HERMITE = 0, 1
SOLVE_FP64, SOLVE_MIXED = 0, 1
PRECOND_NONE, PRECOND_JACOBI, PRECOND_CHEBYSHEV = 0, 1, 2
KERNEL_AUTO, KERNEL_GENERIC = 0, 1
SWEEP_EO_FP32, SWEEP_MMA_TF32X3, SWEEP_MMA_TF32, SWEEP_EO_FP64 = 0, 1, 2, 3

EXPORTS = [
    "sf_last_error", "sf_version", "sf_create", "sf_destroy", "sf_sizes", "sf_set_geometry",
    "sf_set_coefficient", "sf_vmult", "sf_vmult_transpose", "sf_vmult_batched",
    "sf_vmult_transpose_batched", "sf_chebyshev_step", "sf_vector_update", "sf_diagonal",
    "sf_kappa_gradient", "sf_solve_opts_default", "sf_cg_solve", "sf_convert", "sf_dot",
    "sf_shape_tables", "sf_set_kernel_variant", "sf_device_status", "sf_vmult_transpose_static",
    "sf_rk_stage", "sf_lsrk_step", "sf_create_unstructured", "sf_sweep_benchmark",
]


class SFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code


class Desc(C.Structure):
    _fields_ = [("kind", C.c_int), ("degree", C.c_int), ("n_cells", C.c_int * 3),
                ("length", C.c_double * 3), ("basis", C.c_int), ("deform", C.c_double),
                ("dirichlet", C.c_int), ("penalty", C.c_double), ("velocity", C.c_double * 3),
                ("inverse_mass", C.c_int), ("precisions", C.c_int)]


class SolveOpts(C.Structure):
    _fields_ = [("mode", C.c_int), ("precond", C.c_int), ("cheb_degree", C.c_int),
                ("cheb_range", C.c_double), ("eig_iterations", C.c_int), ("rtol", C.c_double),
                ("max_iter", C.c_int), ("inner_rtol", C.c_double), ("project_constant", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer_iterations", C.c_int),
                ("rel_residual", C.c_double), ("lambda_max", C.c_double),
                ("seconds", C.c_double), ("operator_applies", C.c_int)]


_lib = None


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libsfgpu.so not built (run __graft_entry__.build()); "
                              "there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        vp, i, d, ll = C.c_void_p, C.c_int, C.c_double, C.c_longlong
        L.sf_last_error.restype = C.c_char_p
        L.sf_version.restype = C.c_char_p
        L.sf_create.argtypes = [C.POINTER(Desc), C.POINTER(vp)]
        L.sf_create_unstructured.argtypes = [C.c_int, C.c_int, ll, ll, vp, vp, vp, C.c_int, C.POINTER(vp)]
        L.sf_destroy.argtypes = [vp]
        L.sf_sizes.argtypes = [vp, C.POINTER(ll), C.POINTER(ll)]
        L.sf_set_geometry.argtypes = [vp, vp]
        L.sf_set_coefficient.argtypes = [vp, vp]
        L.sf_vmult.argtypes = [vp, i, vp, vp, vp]
        L.sf_vmult_transpose.argtypes = [vp, i, vp, vp, vp]
        L.sf_vmult_batched.argtypes = [vp, i, i, vp, vp, vp]
        L.sf_vmult_transpose_batched.argtypes = [vp, i, i, vp, vp, vp]
        L.sf_chebyshev_step.argtypes = [vp, i, vp, vp, vp, vp, vp, d, d, vp]
        L.sf_vector_update.argtypes = [ll, i, vp, vp, vp, vp, vp, vp, d, d, vp]
        L.sf_diagonal.argtypes = [vp, i, vp, vp]
        L.sf_kappa_gradient.argtypes = [vp, i, vp, vp, vp, vp]
        L.sf_solve_opts_default.argtypes = [C.POINTER(SolveOpts)]
        L.sf_solve_opts_default.restype = None
        L.sf_cg_solve.argtypes = [vp, vp, vp, C.POINTER(SolveOpts), C.POINTER(SolveStats), vp]
        L.sf_convert.argtypes = [ll, i, vp, i, vp, vp]
        L.sf_dot.argtypes = [ll, i, vp, vp, vp, vp]
        L.sf_shape_tables.argtypes = [i, i, vp, vp, vp, vp]
        L.sf_set_kernel_variant.argtypes = [vp, i]
        L.sf_vmult_transpose_static.argtypes = [vp, i, i, vp, vp, vp]
        L.sf_device_status.argtypes = [vp, C.POINTER(i)]
        L.sf_rk_stage.argtypes = [vp, i, i, vp, vp, vp, vp, d, d, vp]
        L.sf_lsrk_step.argtypes = [vp, i, i, vp, vp, vp, d, vp]
        L.sf_sweep_benchmark.argtypes = [i, i, ll, i, vp, vp, vp]
        _lib = L
    return _lib


def check(code):
    if code != SF_OK:
        raise SFError(code, lib().sf_last_error().decode())
    return code


def ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    return a.data_ptr()


def prec_of(t):
    import torch
    if t.dtype == torch.float64:
        return FP64
    if t.dtype == torch.float32:
        return FP32
    raise TypeError("vectors must be float32 or float64, got %s" % t.dtype)


def vec(t, n, prec, name):
    """device address of a vector argument.  The library cannot see buffer
    sizes (a short buffer would be written past its end), so a tensor must
    be a contiguous CUDA tensor of the call's precision with at least n
    entries; None and integer addresses are passed on unchecked."""
    if t is None or isinstance(t, int):
        return t
    if not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor" % name)
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    if prec_of(t) != prec:
        raise TypeError("%s is %s; this call computes in %s" % (name, t.dtype, "float64" if prec == FP64
                                                                 else "float32"))
    if t.numel() < n:
        raise ValueError("%s holds %d entries; this call needs %d" % (name, t.numel(), n))
    return t.data_ptr()


def stream_ptr(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Operator:
    """One operator handle (sf_op).  Mirrors the evaluator classes of the
    reference: construction = initialize(), vmult = matrix_vector_product()
    / do_matvec(), chebyshev_step = do_cheby_iter<true>()."""

    def __init__(self, kind=OP_LAPLACE, degree=4, n_cells=(16, 16, 16), length=(1.0, 1.0, 1.0),
                 basis=BASIS_GLL, deform=0.0, dirichlet=1, penalty=1.0,
                 velocity=(1.0, 0.5, 0.25), inverse_mass=1, precisions=3):
        d = Desc()
        d.kind, d.degree = kind, degree
        for k in range(3):
            d.n_cells[k] = int(n_cells[k])
            d.length[k] = float(length[k])
            d.velocity[k] = float(velocity[k])
        d.basis, d.deform, d.dirichlet = basis, float(deform), int(dirichlet)
        d.penalty, d.inverse_mass, d.precisions = float(penalty), int(inverse_mass), int(precisions)
        self.desc = d
        h = C.c_void_p()
        check(lib().sf_create(C.byref(d), C.byref(h)))
        self._h = h
        nd, nc = C.c_longlong(), C.c_longlong()
        check(lib().sf_sizes(self._h, C.byref(nd), C.byref(nc)))
        self.n_dofs, self.n_cells = nd.value, nc.value
        self.degree = degree
        self.kind = kind

    @classmethod
    def unstructured(cls, degree, cell_nodes, merged6, n_nodes, dirichlet=None, basis=BASIS_GLL, precisions=3):
        """continuous Laplacian on an unstructured hexahedral mesh
        (sf_create_unstructured): cell_nodes int32 [cell][(p+1)^3], merged6
        float64 [cell][6][(p+1)^3], dirichlet uint8 [n_nodes] or None"""
        import numpy as np
        idx = np.ascontiguousarray(cell_nodes, dtype=np.int32).ravel()
        geo = np.ascontiguousarray(merged6, dtype=np.float64).ravel()
        n3 = (degree + 1) ** 3
        n_cells = idx.size // n3
        dmask = None if dirichlet is None else np.ascontiguousarray(dirichlet, dtype=np.uint8)
        self = cls.__new__(cls)
        h = C.c_void_p()
        check(lib().sf_create_unstructured(degree, basis, n_cells, int(n_nodes), idx.ctypes.data, geo.ctypes.data,
                                           None if dmask is None else dmask.ctypes.data, precisions,
                                           C.byref(h)))
        self._h = h
        self.desc = None
        self.n_dofs, self.n_cells = int(n_nodes), n_cells
        self.degree = degree
        self.kind = OP_LAPLACE_UNSTRUCTURED
        return self

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().sf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _cell_points(self):
        return self.n_cells * (self.degree + 1) ** 3

    def vmult(self, x, y, stream=None):
        pr, n = prec_of(x), self.n_dofs
        check(lib().sf_vmult(self._h, pr, vec(x, n, pr, "x"), vec(y, n, pr, "y"), stream_ptr(stream)))
        return y

    def vmult_transpose(self, x, y, stream=None):
        pr, n = prec_of(x), self.n_dofs
        check(lib().sf_vmult_transpose(self._h, pr, vec(x, n, pr, "x"), vec(y, n, pr, "y"), stream_ptr(stream)))
        return y

    def vmult_batched(self, x, y, nrhs, stream=None):
        pr, n = prec_of(x), int(nrhs) * self.n_dofs
        check(lib().sf_vmult_batched(self._h, pr, nrhs, vec(x, n, pr, "x"), vec(y, n, pr, "y"), stream_ptr(stream)))
        return y

    def vmult_transpose_batched(self, x, y, nrhs, stream=None):
        pr, n = prec_of(x), int(nrhs) * self.n_dofs
        check(lib().sf_vmult_transpose_batched(self._h, pr, nrhs, vec(x, n, pr, "x"), vec(y, n, pr, "y"),
                                               stream_ptr(stream)))
        return y

    def vmult_transpose_static(self, x, y, nrhs=1, stream=None):
        """transposed advection apply that allocates nothing (see sfgpu.h)"""
        pr, n = prec_of(x), int(nrhs) * self.n_dofs
        check(lib().sf_vmult_transpose_static(self._h, pr, nrhs, vec(x, n, pr, "x"), vec(y, n, pr, "y"),
                                              stream_ptr(stream)))
        return y

    def chebyshev_step(self, b, diag_inv, x_old, x_new, t, c_np, c_tm, stream=None):
        pr, n = prec_of(x_old), self.n_dofs
        check(lib().sf_chebyshev_step(self._h, pr, vec(b, n, pr, "b"), vec(diag_inv, n, pr, "diag_inv"),
                                      vec(x_old, n, pr, "x_old"), vec(x_new, n, pr, "x_new"), vec(t, n, pr, "t"),
                                      float(c_np), float(c_tm), stream_ptr(stream)))

    def rk_stage(self, src, upd, vec_np, vec_tm, c_np, c_tm, nrhs=1, stream=None):
        """do_rk_stage<true>: vec_np = upd + c_np A src, vec_tm = vec_np + c_tm A src"""
        pr, n = prec_of(src), int(nrhs) * self.n_dofs
        check(lib().sf_rk_stage(self._h, pr, int(nrhs), vec(src, n, pr, "src"), vec(upd, n, pr, "upd"),
                                vec(vec_np, n, pr, "vec_np"), vec(vec_tm, n, pr, "vec_tm"),
                                float(c_np), float(c_tm), stream_ptr(stream)))

    def lsrk_step(self, sol_new, sol_old, sol_tmp, dt, nrhs=1, stream=None):
        """do_time_step: one LSRK(5,4) step, sol_new advanced in place"""
        pr, n = prec_of(sol_new), int(nrhs) * self.n_dofs
        check(lib().sf_lsrk_step(self._h, pr, int(nrhs), vec(sol_new, n, pr, "sol_new"),
                                 vec(sol_old, n, pr, "sol_old"), vec(sol_tmp, n, pr, "sol_tmp"),
                                 float(dt), stream_ptr(stream)))

    def diagonal(self, out, stream=None):
        pr = prec_of(out)
        check(lib().sf_diagonal(self._h, pr, vec(out, self.n_dofs, pr, "out"), stream_ptr(stream)))
        return out

    def kappa_gradient(self, u, lam, out, stream=None):
        pr, n = prec_of(u), self.n_dofs
        check(lib().sf_kappa_gradient(self._h, pr, vec(u, n, pr, "u"), vec(lam, n, pr, "lam"),
                                      vec(out, self._cell_points(), pr, "out"), stream_ptr(stream)))
        return out

    def set_geometry(self, G):
        check(lib().sf_set_geometry(self._h, vec(G, 6 * self._cell_points(), FP64, "G")))

    def set_coefficient(self, kappa):
        check(lib().sf_set_coefficient(self._h, vec(kappa, self._cell_points(), FP64, "kappa")))

    def set_kernel_variant(self, variant):
        check(lib().sf_set_kernel_variant(self._h, int(variant)))

    def device_status(self):
        f = C.c_int()
        check(lib().sf_device_status(self._h, C.byref(f)))
        return f.value

    def cg_solve(self, b, x, opts=None, stream=None):
        o = default_solve_opts() if opts is None else opts
        st = SolveStats()
        code = lib().sf_cg_solve(self._h, vec(b, self.n_dofs, FP64, "b"), vec(x, self.n_dofs, FP64, "x"),
                                 C.byref(o), C.byref(st), stream_ptr(stream))
        return code, st


def default_solve_opts(**kw):
    o = SolveOpts()
    lib().sf_solve_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def dot(x, y, out, stream=None):
    pr, n = prec_of(x), x.numel()
    check(lib().sf_dot(n, pr, vec(x, n, pr, "x"), vec(y, n, pr, "y"), vec(out, 1, FP64, "out"),
                       stream_ptr(stream)))
    return out


def convert(x, y, stream=None):
    n = x.numel()
    check(lib().sf_convert(n, prec_of(x), vec(x, n, prec_of(x), "x"), prec_of(y), vec(y, n, prec_of(y), "y"),
                           stream_ptr(stream)))
    return y


def vector_update(ax, b, dinv, x_old, x_new, t, c_np, c_tm, stream=None):
    pr, n = prec_of(x_old), x_old.numel()
    check(lib().sf_vector_update(n, pr, vec(ax, n, pr, "ax"), vec(b, n, pr, "b"), vec(dinv, n, pr, "dinv"),
                                 vec(x_old, n, pr, "x_old"), vec(x_new, n, pr, "x_new"), vec(t, n, pr, "t"),
                                 float(c_np), float(c_tm), stream_ptr(stream)))


def shape_tables(degree, basis=BASIS_GLL):
    import numpy as np
    n = degree + 1
    S, D, x, w = (np.zeros(n * n), np.zeros(n * n), np.zeros(n), np.zeros(n))
    check(lib().sf_shape_tables(degree, basis, S.ctypes.data, D.ctypes.data, x.ctypes.data,
                                w.ctypes.data))
    return S.reshape(n, n), D.reshape(n, n), x, w
