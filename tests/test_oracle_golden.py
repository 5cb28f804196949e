"""The CPU oracle against the golden vectors made by the reference's own code.

These pins are what every GPU parity test inherits: the CUDA library is
compared with the oracle, and the oracle is compared here with the reference
(tests/golden/gen_golden.py).  Tolerances are relative, FP64.
"""
import numpy as np
import pytest

from oracle import oracle as O


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("p", range(1, 9))
def test_tables(golden, p):
    g = golden("tables.npz")
    n = p + 1
    a = O.shape_arrays(p, O.BASIS_GLL)
    np.testing.assert_allclose(a["xq"], g["gauss_x_%d" % n], rtol=0, atol=1e-15)
    np.testing.assert_allclose(a["wq"], g["gauss_w_%d" % n], rtol=0, atol=1e-15)
    np.testing.assert_allclose(a["xgll"], g["gll_x_%d" % n], rtol=0, atol=1e-15)
    scale = np.abs(g["gll_D_eo_%d" % p]).max()
    np.testing.assert_allclose(a["S_eo"], g["gll_S_eo_%d" % p], rtol=0, atol=1e-14)
    np.testing.assert_allclose(a["D_eo"], g["gll_D_eo_%d" % p], rtol=0, atol=1e-15 * scale)
    np.testing.assert_allclose(a["face_eo"], g["face_eo_%d" % p], rtol=0, atol=1e-13)
    np.testing.assert_allclose(a["Sinv_eo"], g["Sinv_eo_%d" % p], rtol=0, atol=1e-14)
    h = O.shape_arrays(p, O.BASIS_HERMITE)
    np.testing.assert_allclose(h["S_eo"], g["herm_S_eo_%d" % p], rtol=0, atol=1e-14)
    np.testing.assert_allclose(h["D_eo"], g["herm_D_eo_%d" % p], rtol=0, atol=1e-15 * scale)
    assert abs(h["hermite_d0"] - g["herm_d0_%d" % p][0]) <= 1e-13 * abs(g["herm_d0_%d" % p][0])


def test_kernel1d(golden):
    g = golden("kernel1d.npz")
    k = 0
    while "k%03d_meta" % k in g:
        nn, t, c, a, dgm = (int(v) for v in g["k%03d_meta" % k])
        y, f = O.apply_1d(nn, t, c, a, g["k%03d_coef" % k], g["k%03d_x" % k],
                          out_init=g["k%03d_o" % k], do_dg=dgm, dg=g["k%03d_dg" % k],
                          face=g["k%03d_fin" % k])
        assert rel(y, g["k%03d_y" % k]) < 1e-14, (nn, t, c, a, dgm)
        if dgm and c:
            assert rel(f[: 2 * dgm], g["k%03d_fout" % k][: 2 * dgm]) < 1e-14
        k += 1
    assert k >= 80


def test_kernel_even_odd_vs_plain():
    """even-odd kernel against the plain n x n contraction
    (the cross-check of test_multiplication.cc:912-1021)"""
    rng = np.random.default_rng(3)
    for p in range(1, 9):
        n = p + 1
        a = O.shape_arrays(p, O.BASIS_GLL)
        x = rng.standard_normal(n)
        for M, eo, t in ((a["S"], a["S_eo"], 0), (a["D"], a["D_eo"], 1)):
            y, _ = O.apply_1d(n, t, True, False, eo, x)
            assert rel(y, M @ x) < 1e-14
            y, _ = O.apply_1d(n, t, False, False, eo, x)
            assert rel(y, M.T @ x) < 1e-14


@pytest.mark.parametrize("p", range(1, 9))
def test_cell(golden, p):
    g = golden("cell.npz")
    n = p + 1
    a = O.shape_arrays(p, O.BASIS_GLL)
    W = np.einsum("k,j,i->kji", a["wq"], a["wq"], a["wq"]).ravel()
    G6 = g["gll_G6_%d" % p]
    G = np.concatenate([G6[e] * W for e in range(6)])
    y = O.cell_apply(p, O.BASIS_GLL, G, g["gll_x_%d" % p], n ** 3)
    assert rel(y, g["gll_y_%d" % p]) < 1e-14
    if p != 2:  # the reference drops a nonzero term for the degree-2 Hermite basis
        ij = np.array([4.0, 2.0, 4.0 / 3.0])
        jxw = 1.0 / np.prod(ij)
        G6 = np.array([jxw * ij[0] ** 2, jxw * ij[1] ** 2, jxw * ij[2] ** 2, 0, 0, 0])
        G = np.concatenate([G6[e] * W for e in range(6)])
        y = O.cell_apply(p, O.BASIS_HERMITE, G, g["herm_x_%d" % p], n ** 3)
        assert rel(y, g["herm_y_%d" % p]) < 1e-14


@pytest.mark.parametrize("p", range(1, 9))
def test_continuous_affine(golden, p):
    g = golden("cont.npz")
    nc = tuple(int(v) for v in g["nc_%d" % p])
    m = O.mesh(p, nc, length=tuple(g["len_%d" % p]))
    G = O.cont_geometry(m)
    y = O.cont_apply(m, G, g["x_%d" % p])
    assert rel(y, g["y_%d" % p]) < 1e-13


def test_continuous_q4_16(golden):
    g = golden("cont.npz")
    m = O.mesh(4, (16, 16, 16))
    N = O.cont_n_dofs(m)
    x = np.random.default_rng(20241203).uniform(-1.0, 1.0, N)
    y = O.cont_apply(m, O.cont_geometry(m), x)
    idx = g["q4_16_sample_idx"]
    assert rel(y[idx], g["q4_16_sample_y"]) < 1e-13
    assert abs(np.linalg.norm(y) - g["q4_16_norm2"][0]) < 1e-12 * g["q4_16_norm2"][0]


@pytest.mark.parametrize("p", [1, 3, 4, 5, 6, 7, 8])
def test_dg_sipg(golden, p):
    g = golden("dg_sipg.npz")
    d = O.dg(p, tuple(int(v) for v in g["nc_%d" % p]), tuple(g["h_%d" % p]))
    y = O.dg_sipg_apply(d, g["x_%d" % p])
    assert rel(y, g["y_%d" % p]) < 1e-14


def test_dg_chebyshev_step(golden):
    g = golden("dg_sipg.npz")
    d = O.dg(5, tuple(int(v) for v in g["nc_5"]), tuple(g["h_5"]))
    ax = O.dg_sipg_apply(d, g["x_5"])
    xn, tn = O.chebyshev_update(ax, g["cheb_b"], g["cheb_dinv"], g["x_5"], g["cheb_t"], 0.7, 0.3)
    assert rel(xn, g["cheb_xnew"]) < 1e-14
    assert rel(tn, g["cheb_tnew"]) < 1e-14


@pytest.mark.parametrize("p", range(1, 9))
def test_dg_advect(golden, p):
    g = golden("dg_advect.npz")
    d = O.dg(p, tuple(int(v) for v in g["nc_%d" % p]), tuple(g["h_%d" % p]),
             velocity=(1.0, 0.15, -0.05), inverse_mass=1)
    y = O.dg_advect_apply(d, g["x_%d" % p])
    assert rel(y, g["y_%d" % p]) < 1e-14


@pytest.mark.parametrize("p", [1, 2, 4, 5])
@pytest.mark.parametrize("case", ["a", "b"])
def test_dg_rk_stage(golden, p, case):
    """fused Runge-Kutta stage against the reference's do_rk_stage<true>
    (case b has c_tm = 0: vec_tm must stay untouched)"""
    g = golden("dg_rk.npz")
    d = O.dg(p, tuple(int(v) for v in g["nc_%d" % p]), tuple(g["h_%d" % p]),
             velocity=(1.0, 0.15, -0.05), inverse_mass=1)
    c_np, c_tm = (float(v) for v in g["c_%s_%d" % (case, p)])
    vnp = np.zeros_like(g["src_%d" % p])
    vtm = np.array(g["tm0_%d" % p])
    O.dg_rk_stage(d, np.array(g["src_%d" % p]), np.array(g["upd_%d" % p]), vnp, vtm, c_np, c_tm)
    assert rel(vnp, g["np_%s_%d" % (case, p)]) < 1e-14
    assert rel(vtm, g["tm_%s_%d" % (case, p)]) < 1e-14
    # the same stage with upd aliasing the output vectors, as do_time_step calls it
    u = np.array(g["upd_%d" % p])
    vtm2 = np.array(g["tm0_%d" % p]) if case == "b" else u
    if case == "a":
        O.dg_rk_stage(d, np.array(g["src_%d" % p]), u, vnp, u, c_np, c_tm)
        assert rel(u, g["tm_a_%d" % p]) < 1e-14
    else:
        O.dg_rk_stage(d, np.array(g["src_%d" % p]), u, u, vtm2, c_np, c_tm)
        assert rel(u, g["np_b_%d" % p]) < 1e-14


@pytest.mark.parametrize("p", [1, 2, 4, 5])
def test_dg_lsrk_steps(golden, p):
    """three LSRK(5,4) steps against the reference's do_time_step"""
    g = golden("dg_rk.npz")
    d = O.dg(p, tuple(int(v) for v in g["nc_%d" % p]), tuple(g["h_%d" % p]),
             velocity=(1.0, 0.15, -0.05), inverse_mass=1)
    x = np.array(g["x0_%d" % p])
    old, tmp = np.zeros_like(x), np.zeros_like(x)
    for _ in range(3):
        O.dg_lsrk_step(d, float(g["dt_%d" % p]), x, old, tmp)
    assert rel(x, g["steps3_%d" % p]) < 1e-13


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6, 8])
def test_dg_precomputed(golden, p):
    """tensor-product SIPG with precomputed 1D matrices against the
    reference's PrecomputedDGLaplacian (unit cells)"""
    g = golden("dg_precomputed.npz")
    d = O.dg(p, tuple(int(v) for v in g["nc_%d" % p]), (1.0, 1.0, 1.0))
    y = O.dg_precomputed_apply(d, g["x_%d" % p].astype(np.float64))
    assert rel(y, g["y_%d" % p]) < 1e-14


# mass matrix and convection form (the reference's DO_MASS_MATRIX and
# DO_CONVECTION builds of the cell operator, velocity (1, 2, 3)); the
# reference's transposed values kernel drops the middle point for odd n
# (matrix_vector_kernel.h:130-131), wrong for the Hermite-like degree-2
# basis, so degree 2 is pinned by the tensor-product identity
# M = JxW (S^T W S) x (S^T W S) x (S^T W S)
CELL_IJ = np.array([4.0, 2.0, 4.0 / 3.0])


@pytest.mark.parametrize("p", [1, 3, 4, 5, 6, 7, 8])
def test_cell_mass_convection(golden, p):
    g = golden("cell_ops.npz")
    jxw = 1.0 / np.prod(CELL_IJ)
    x = g["cell_x_%d" % p]
    assert rel(O.cell_op(p, O.BASIS_HERMITE, O.OP_MASS, CELL_IJ, jxw, (0, 0, 0), x), g["cell_mass_%d" % p]) < 1e-13
    assert rel(O.cell_op(p, O.BASIS_HERMITE, O.OP_CONVECTION, CELL_IJ, jxw, (1, 2, 3), x),
               g["cell_conv_%d" % p]) < 1e-13


@pytest.mark.parametrize("basis", [O.BASIS_GLL, O.BASIS_HERMITE])
@pytest.mark.parametrize("p", [2, 4])
def test_cell_mass_convection_tensor_identity(p, basis):
    """the oracle's sum-factorised variants equal the dense Kronecker forms
    built from its 1D tables: M = JxW M1 x M1 x M1 with M1 = S^T W S, and the
    convection form sum_d (ij_d b_d) JxW (S^T W D S in direction d)"""
    n = p + 1
    a = O.shape_arrays(p, basis)
    S = np.array(a["S"])[: n * n].reshape(n, n)
    D = np.array(a["D"])[: n * n].reshape(n, n)
    W = np.diag(np.array(a["wq"])[:n])
    jxw = 1.0 / np.prod(CELL_IJ)
    M1, C1 = S.T @ W @ S, (D @ S).T @ W @ S
    k = np.kron
    M = jxw * k(k(M1, M1), M1)
    b = np.array([1.0, 2.0, 3.0])
    Cv = jxw * (CELL_IJ[0] * b[0] * k(k(M1, M1), C1) + CELL_IJ[1] * b[1] * k(k(M1, C1), M1)
                + CELL_IJ[2] * b[2] * k(k(C1, M1), M1))
    x = np.random.default_rng(p).uniform(-1, 1, n ** 3)
    assert rel(O.cell_op(p, basis, O.OP_MASS, CELL_IJ, jxw, (0, 0, 0), x), M @ x) < 1e-14
    assert rel(O.cell_op(p, basis, O.OP_CONVECTION, CELL_IJ, jxw, b, x), Cv @ x) < 1e-14
    assert np.abs(M - M.T).max() < 1e-15


@pytest.mark.parametrize("p", [1, 3, 4, 5, 6, 7, 8])
def test_continuous_mass_convection(golden, p):
    g = golden("cell_ops.npz")
    nc = tuple(int(v) for v in g["nc_%d" % p])
    m = O.mesh(p, nc, basis=O.BASIS_HERMITE, length=tuple(g["len_%d" % p]))
    x = g["cont_x_%d" % p]
    assert rel(O.cont_apply_op(m, O.OP_MASS, x), g["cont_mass_%d" % p]) < 1e-13
    assert rel(O.cont_apply_op(m, O.OP_CONVECTION, x, (1, 2, 3)), g["cont_conv_%d" % p]) < 1e-13


# the DO_FACES builds of the cell operator (Laplacian and convection form)
# on one Cartesian cell; degree 2 again by a dense formulation
@pytest.mark.parametrize("p", [1, 3, 4, 5, 6, 7, 8])
def test_cell_faces(golden, p):
    g = golden("cell_ops.npz")
    jxw = 1.0 / np.prod(CELL_IJ)
    x = g["cell_x_%d" % p]
    assert rel(O.cell_faces(p, False, CELL_IJ, jxw, (0, 0, 0), x), g["cell_faces_%d" % p]) < 1e-13
    assert rel(O.cell_faces(p, True, CELL_IJ, jxw, (1, 2, 3), x), g["cell_faces_conv_%d" % p]) < 1e-13


def faces_dense(p, conv, ij, jxw, b):
    """the DO_FACES cell operator as a dense matrix from the 1D tables: the
    Kronecker cell term plus, per direction f, the face terms written with
    layer-selection matrices and the face interpolation S x S"""
    n = p + 1
    a = O.shape_arrays(p, O.BASIS_HERMITE)
    S, D, w, hd = a["S"], a["D"], a["wq"], a["hermite_d0"]
    W = np.diag(w)
    k = np.kron
    M1, L1, C1 = S.T @ W @ S, (D @ S).T @ W @ (D @ S), (D @ S).T @ W @ S
    if conv:
        A = jxw * (ij[0] * b[0] * k(k(M1, M1), C1) + ij[1] * b[1] * k(k(M1, C1), M1)
                   + ij[2] * b[2] * k(k(C1, M1), M1))
    else:
        A = jxw * (ij[0] ** 2 * k(k(M1, M1), L1) + ij[1] ** 2 * k(k(M1, L1), M1)
                   + ij[2] ** 2 * k(k(L1, M1), M1))
    F2 = k(S, S)
    grid = np.arange(n ** 3).reshape(n, n, n)        # [z, y, x]
    for f in range(3):
        d1, d2 = (f + 1) % 3, (f + 2) % 3

        def sel(layer):
            R = np.zeros((n * n, n ** 3))
            for i2 in range(n):
                for i1 in range(n):
                    c = [0, 0, 0]
                    c[f], c[d1], c[d2] = layer, i1, i2
                    R[i2 * n + i1, grid[c[2], c[1], c[0]]] = 1.0
            return R
        W2 = -np.diag(k(w, w)) * np.prod([1.0 / ij[e] for e in range(3) if e != f])
        uR, uL = F2 @ sel(p), F2 @ sel(0)
        if conv:
            flux = 0.5 * (b[f] * (uR + uL) + abs(b[f]) * (uR - uL))
            A += sel(p).T @ F2.T @ W2 @ flux - sel(0).T @ F2.T @ W2 @ flux
        else:
            nR, nL = F2 @ (hd * (sel(p - 1) - sel(p))), F2 @ (hd * (sel(1) - sel(0)))
            avg = 0.5 * (uR + uL)
            v = W2 @ (2 * n * n * ij[f] * avg - 0.5 * ij[f] * (nR + nL))
            td = F2 @ (W2 @ (ij[f] * avg))            # forward S, as the reference
            A += sel(p).T @ (F2.T @ -v - hd * td) + sel(p - 1).T @ (hd * td)
            A += sel(0).T @ (F2.T @ v - hd * td) + sel(1).T @ (hd * td)
    return A


@pytest.mark.parametrize("p", [1, 2, 4])
def test_cell_faces_dense(p):
    jxw = 1.0 / np.prod(CELL_IJ)
    b = np.array([0.7, -1.3, 0.4])
    x = np.random.default_rng(p).uniform(-1, 1, (p + 1) ** 3)
    for conv in (False, True):
        ref = faces_dense(p, conv, CELL_IJ, jxw, b) @ x
        assert rel(O.cell_faces(p, conv, CELL_IJ, jxw, b, x), ref) < 1e-14, conv
    # the cell-major apply is the cell operator on every cell
    h = 1.0 / CELL_IJ
    X = np.random.default_rng(10 + p).uniform(-1, 1, 3 * (p + 1) ** 3)
    Y = O.cell_faces_apply(p, True, 3, h, X, b)
    n3 = (p + 1) ** 3
    for e in range(3):
        assert rel(Y[e * n3:(e + 1) * n3], O.cell_faces(p, True, CELL_IJ, jxw, b, X[e * n3:(e + 1) * n3])) < 1e-15
