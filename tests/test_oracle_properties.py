"""Mathematical identities of the oracle itself (size-independent checks that
complement the golden vectors): symmetry, explicit transposes and diagonals,
the analytic advection derivative of the reference's self-check, central
finite differences for the kappa gradient, null spaces, boundary rows and
conservation, and the Kronecker-product and line-operator forms that the
structured kernels evaluate."""
import numpy as np
import pytest

from oracle import oracle as O


def dense(apply, n):
    A = np.zeros((n, n))
    e = np.zeros(n)
    for j in range(n):
        e[j] = 1.0
        A[:, j] = apply(e)
        e[j] = 0.0
    return A


@pytest.mark.parametrize("p,basis", [(1, 0), (2, 0), (3, 1), (4, 0)])
def test_continuous_matrix_symmetric_and_diagonal(p, basis):
    m = O.mesh(p, (2, 2, 2), basis=basis, deform=0.06)
    G = O.cont_geometry(m)
    kappa = np.exp(0.3 * np.random.default_rng(1).standard_normal(8 * (p + 1) ** 3))
    A = dense(lambda v: O.cont_apply(m, G, v, kappa=kappa), O.cont_n_dofs(m))
    assert np.abs(A - A.T).max() < 1e-13 * np.abs(A).max()
    assert np.allclose(np.diag(A), O.cont_diagonal(m, G, kappa=kappa), rtol=1e-13, atol=1e-15)
    w = np.linalg.eigvalsh(A)
    assert w.min() > 0  # SPD with identity Dirichlet rows


@pytest.mark.parametrize("p", [1, 3, 4])
def test_sipg_matrix_symmetric_positive(p):
    d = O.dg(p, (3, 2, 2), (0.3, 0.5, 0.2))
    A = dense(lambda v: O.dg_sipg_apply(d, v), O.dg_n_dofs(d))
    assert np.abs(A - A.T).max() < 1e-12 * np.abs(A).max()
    w = np.linalg.eigvalsh(0.5 * (A + A.T))
    assert w[0] > -1e-9 * w[-1]  # periodic: constant null space, PSD
    assert np.allclose(np.diag(A), O.dg_sipg_diagonal(d), rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("p,invm", [(1, 1), (2, 0), (3, 1), (4, 0)])
def test_advect_transpose_is_matrix_transpose(p, invm):
    d = O.dg(p, (2, 3, 2), (0.25, 0.2, 0.4), velocity=(1.0, 0.5, 0.25), inverse_mass=invm)
    n = O.dg_n_dofs(d)
    A = dense(lambda v: O.dg_advect_apply(d, v), n)
    At = dense(lambda v: O.dg_advect_apply_transpose(d, v), n)
    assert np.abs(At - A.T).max() < 1e-12 * np.abs(A).max()


def _wave(points, t, a):
    k = 4.0 * np.pi
    xs = [points[i] - t * a[i] for i in range(3)]
    u = np.sin(k * xs[0]) * np.cos(k * xs[1]) * np.cos(k * xs[2])
    dudt = -(a[0] * k * np.cos(k * xs[0]) * np.cos(k * xs[1]) * np.cos(k * xs[2])
             - a[1] * k * np.sin(k * xs[0]) * np.sin(k * xs[1]) * np.cos(k * xs[2])
             - a[2] * k * np.sin(k * xs[0]) * np.cos(k * xs[1]) * np.sin(k * xs[2]))
    return u, dudt


def test_advect_analytic_time_derivative_converges():
    """the reference's verify_derivative (evaluation_dg_advect.h:221-251):
    M^-1 A u at the GLL nodes approximates du/dt of the advected wave"""
    a = (1.0, 0.15, -0.05)
    errs = []
    nc = (4, 4, 4)
    for p in (3, 5, 7):
        n = p + 1
        h = 2.0 / nc[0]
        xg = O.shape_arrays(p, O.BASIS_GLL)["xgll"]
        pts = []
        for k in range(nc[2]):
            for j in range(nc[1]):
                for i in range(nc[0]):
                    c, b, aa = np.meshgrid(xg, xg, xg, indexing="ij")
                    pts.append([(i + aa) * h, (j + b) * h, (k + c) * h])
        P = [np.concatenate([q[dd].ravel() for q in pts]) for dd in range(3)]
        u, dudt = _wave(P, 0.0, a)
        d = O.dg(p, nc, (h, h, h), velocity=a, inverse_mass=1)
        errs.append(np.abs(O.dg_advect_apply(d, u) - dudt).max() / np.abs(dudt).max())
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 2e-2


def test_kappa_gradient_central_differences():
    """dL/dkappa of L = 1/2 |A(kappa) x - b|^2 against central differences
    with step 1e-6 (relative), FP64"""
    p, nc = 2, (2, 2, 2)
    m = O.mesh(p, nc, deform=0.05)
    G = O.cont_geometry(m)
    rng = np.random.default_rng(4)
    nq = 8 * (p + 1) ** 3
    kappa = np.exp(0.5 * rng.standard_normal(nq))
    x = rng.uniform(-1, 1, O.cont_n_dofs(m))
    b = rng.uniform(-1, 1, O.cont_n_dofs(m))

    def L(k):
        r = O.cont_apply(m, G, x, kappa=k) - b
        return 0.5 * r @ r

    r = O.cont_apply(m, G, x, kappa=kappa) - b
    g = O.cont_kappa_grad(m, G, x, r)
    for q in rng.choice(nq, 12, replace=False):
        hstep = 1e-6 * kappa[q]
        kp, km = kappa.copy(), kappa.copy()
        kp[q] += hstep
        km[q] -= hstep
        fd = (L(kp) - L(km)) / (2 * hstep)
        assert abs(fd - g[q]) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(g).max()), (q, fd, g[q])


def test_fast_division_formula():
    """the 64-bit multiply-high division used by the DG kernels' cell decode
    (m = floor((2^64-1)/d) + 1, q = floor(m n / 2^64)) is exact for 32-bit n"""
    rng = np.random.default_rng(7)
    ds = [2, 3, 5, 7, 48, 63, 64, 65, 1000, 2 ** 20, 2 ** 20 - 1, 2 ** 31 - 1, 2 ** 32 - 1]
    ds += [int(v) for v in rng.integers(2, 2 ** 32, 50)]
    ns = [0, 1, 2 ** 31 - 1, 2 ** 31, 2 ** 32 - 1] + [int(v) for v in rng.integers(0, 2 ** 32, 2000)]
    for d in ds:
        m = (2 ** 64 - 1) // d + 1
        for n in ns + [d - 1, d, d + 1, 2 * d - 1, 2 * d]:
            n &= 2 ** 32 - 1
            assert (m * n) >> 64 == n // d


@pytest.mark.parametrize("p", [2, 3])
def test_precomputed_sipg_matrix_properties(p):
    """symmetric, positive semi-definite with the constants as null space,
    diagonal equal to the assembled one, uniform scaling h -> s h scales the
    operator by s (anisotropic cells)"""
    d = O.dg(p, (3, 2, 2), (0.5, 0.8, 0.3))
    n = O.dg_n_dofs(d)
    A = dense(lambda x: O.dg_precomputed_apply(d, x), n)
    assert np.abs(A - A.T).max() < 1e-12 * np.abs(A).max()
    ev = np.linalg.eigvalsh(0.5 * (A + A.T))
    assert ev.min() > -1e-10 * ev.max()
    assert np.abs(A @ np.ones(n)).max() < 1e-12 * np.abs(A).max()
    assert np.abs(np.diag(A) - O.dg_precomputed_diagonal(d)).max() < 1e-12 * np.abs(A).max()
    d2 = O.dg(p, (3, 2, 2), (1.5, 2.4, 0.9))
    x = np.random.default_rng(p).uniform(-1, 1, n)
    assert np.abs(O.dg_precomputed_apply(d2, x) - 3.0 * A @ x).max() < 1e-12 * np.abs(A @ x).max() * 3


# unstructured hexahedral meshes (no counterpart in the reference): the
# structured mesh written as index arrays, renumbered, and with every cell
# described in a random local frame (axis permutation and reflections) gives
# the structured operator
@pytest.mark.parametrize("basis", [O.BASIS_GLL, O.BASIS_HERMITE])
@pytest.mark.parametrize("p", [1, 3, 4])
def test_unstructured_equals_structured(p, basis):
    m = O.mesh(p, (3, 2, 2), basis=basis, length=(1.0, 0.7, 0.9), deform=0.05)
    G = O.cont_geometry(m)
    N = O.cont_n_dofs(m)
    idx, dmask = O.structured_as_unstructured(m)
    x = np.random.default_rng(p).uniform(-1, 1, N)
    y = O.cont_apply(m, G, x)
    n, nc = p + 1, idx.shape[0]
    rng = np.random.default_rng(10 + p)
    perm_nodes = rng.permutation(N)             # new number of old node i
    perm_cells = rng.permutation(nc)
    Gc = G.reshape(nc, -1)
    idx2 = np.empty_like(idx)
    G2 = np.empty_like(Gc)
    for new_e, e in enumerate(perm_cells):
        a, g = O.reorient_cell(perm_nodes[idx[e]], Gc[e], n, rng.permutation(3), rng.integers(0, 2, 3))
        idx2[new_e], G2[new_e] = a, g
    x2 = np.empty(N)
    x2[perm_nodes] = x
    d2 = np.empty(N, dtype=np.uint8)
    d2[perm_nodes] = dmask
    y2 = O.unstructured_apply(p, basis, idx2, G2, N, x2, d2)
    assert np.abs(y2[perm_nodes] - y).max() < 1e-13 * np.abs(y).max()


@pytest.mark.parametrize("p", [1, 2, 5, 8])
@pytest.mark.parametrize("penalty", [1.0, 2.5])
def test_sipg_is_kronecker_sum(p, penalty):
    """On a periodic Cartesian mesh the SIPG operator (tau = penalty (p+1)^2
    / h_d) is L (x) M (x) M + M (x) L (x) M + M (x) M (x) L with 1D periodic
    DG stiffness-plus-face matrices L of 1D penalty penalty (p+1)^2 and 1D
    mass matrices M: the identity behind evaluating SF_OP_DG_SIPG with the
    tensor-product kernel"""
    n = p + 1
    sh = O.shape_arrays(p, O.BASIS_HERMITE)
    S, D, w = sh["S"], sh["D"], sh["wq"]
    v0, v1 = sh["face_v"][0] @ S, sh["face_v"][1] @ S
    d0, d1 = sh["face_d"][0] @ S, sh["face_d"][1] @ S
    dq = D @ S
    pen = penalty * (p + 1) ** 2
    M = (S * w[:, None]).T @ S
    L = ((dq * w[:, None]).T @ dq + pen * np.outer(v0, v0) + 0.5 * (np.outer(d0, v0) + np.outer(v0, d0))
         + pen * np.outer(v1, v1) - 0.5 * (np.outer(d1, v1) + np.outer(v1, d1)))
    C = -pen * np.outer(v0, v1) - 0.5 * np.outer(d0, v1) + 0.5 * np.outer(v0, d1)   # cell <- left neighbour
    nc, h = (3, 4, 2), (1 / 3, 0.25, 0.5)

    def lap1d(m, hh):
        A = np.zeros((m * n, m * n))
        for e in range(m):
            l, r = (e - 1) % m, (e + 1) % m
            A[e * n:(e + 1) * n, e * n:(e + 1) * n] += L / hh
            A[e * n:(e + 1) * n, l * n:(l + 1) * n] += C / hh
            A[e * n:(e + 1) * n, r * n:(r + 1) * n] += C.T / hh
        return A

    Ad = [lap1d(nc[d], h[d]) for d in range(3)]
    Md = [np.kron(np.eye(nc[d]), M * h[d]) for d in range(3)]
    x = np.random.default_rng(p).standard_normal(int(np.prod(nc)) * n ** 3)
    T = x.reshape(nc[2], nc[1], nc[0], n, n, n).transpose(0, 3, 1, 4, 2, 5).reshape(nc[2] * n, nc[1] * n, nc[0] * n)

    def app(Ax, Ay, Az):
        return np.einsum("ai,zyi->zya", Ax, np.einsum("bj,zjx->zbx", Ay, np.einsum("ck,kyx->cyx", Az, T)))

    Y = app(Ad[0], Md[1], Md[2]) + app(Md[0], Ad[1], Md[2]) + app(Md[0], Md[1], Ad[2])
    y = Y.reshape(nc[2], n, nc[1], n, nc[0], n).transpose(0, 2, 4, 1, 3, 5).ravel()
    ys = O.dg_sipg_apply(O.dg(p, nc, h, penalty=penalty), x)
    assert np.linalg.norm(y - ys) / np.linalg.norm(ys) < 1e-13


@pytest.mark.parametrize("p", range(1, 9))
def test_advect_is_sum_of_line_operators(p):
    """On a periodic Cartesian mesh with constant velocity the upwind DG
    advection operator (GLL nodes, Gauss points) separates by direction:
    M^-1 A = sum_d B_d (x) I (x) I and A = M sum_d B_d (x) I (x) I, with
    B_d = S^-1 W^-1 R_d S from the Gauss-point line residual R_d and each
    line coupled to the upwind (transpose: downwind) neighbour's nodal end
    value; M = jxw M1 (x) M1 (x) M1, M1 = S^T W S.  The identity behind the
    line-operator advection kernel, checked for the forward operator (with
    and without the inverse mass) and the transpose, on a mesh with a
    one-cell-thick direction and a negative velocity component; and the
    transpose with the inverse mass as one sum of line operators whose
    couplings read the neighbour's whole line"""
    n = p + 1
    sh = O.shape_arrays(p)
    S, D, Sinv, w, fv = sh["S"], sh["D"], sh["Sinv"], sh["wq"], sh["face_v"]
    M1 = S.T @ np.diag(w) @ S
    vel = (1.0, 0.5, -0.25)
    for nc, h in (((3, 4, 2), (0.25, 0.2, 0.4)), ((4, 1, 3), (0.3, 0.2, 0.45))):
        jxw = h[0] * h[1] * h[2]
        # (the transpose with the inverse mass is A^T M^-1: the transpose
        # case applied to M^-1 x)
        for invm, tr in ((0, False), (0, True), (1, False)):
            g = O.dg(p, nc, h, velocity=vel, inverse_mass=invm)
            x = np.random.default_rng(p).uniform(-1, 1, O.dg_n_dofs(g))
            inv = bool(invm)
            P = Sinv / w[None, :] / (jxw if inv else 1.0)
            X = x.reshape(nc[2], nc[1], nc[0], n, n, n)   # [cz][cy][cx][z][y][x]
            Y = np.zeros_like(X)
            for d, (cax, nax) in enumerate(((2, 5), (1, 4), (0, 3))):
                ij, ad = 1 / h[d], vel[d]
                c, jf = ad * ij * jxw, jxw * ij
                R = c * np.diag(w) @ D if tr else D.T @ np.diag(c * w)
                nb = []
                for side in range(2):
                    an = ad if side else -ad
                    fa = -0.5 * ((an + abs(an)) if tr else an) * jf
                    fb = -0.5 * abs(an) * jf
                    R = R + (fa if tr else fa + fb) * np.outer(fv[side], fv[side])
                    nb.append(P @ (fv[side] * (-fa if tr else fa - fb)))
                B = P @ R @ S
                lo = np.take(np.roll(X, 1, axis=cax), n - 1, axis=nax)
                hi = np.take(np.roll(X, -1, axis=cax), 0, axis=nax)
                Yd = np.moveaxis(X, nax, -1) @ B.T + lo[..., None] * nb[0] + hi[..., None] * nb[1]
                Y += np.moveaxis(Yd, -1, nax)
            if not inv:
                for nax in (5, 4, 3):
                    Y = np.moveaxis(np.moveaxis(Y, nax, -1) @ M1.T, -1, nax)
            ref = O.dg_advect_apply_transpose(g, x) if tr else O.dg_advect_apply(g, x)
            assert np.linalg.norm(Y.ravel() - ref) / np.linalg.norm(ref) < 1e-13, (nc, invm, tr)
        # the transpose with the inverse mass, A^T M^-1 = sum_d C_d (x) I (x) I / jxw with
        # C_d = M1 B'_d M1^-1, each coupling through a row of M1^-1 and the neighbour's line
        g = O.dg(p, nc, h, velocity=vel, inverse_mass=1)
        x = np.random.default_rng(p).uniform(-1, 1, O.dg_n_dofs(g))
        Minv = np.linalg.inv(M1)
        P = Sinv / w[None, :]
        X = x.reshape(nc[2], nc[1], nc[0], n, n, n)
        Y = np.zeros_like(X)
        for d, (cax, nax) in enumerate(((2, 5), (1, 4), (0, 3))):
            ij, ad = 1 / h[d], vel[d]
            c, jf = ad * ij * jxw, jxw * ij
            R = c * np.diag(w) @ D
            nb = []
            for side in range(2):
                an = ad if side else -ad
                fa = -0.5 * (an + abs(an)) * jf
                R = R + fa * np.outer(fv[side], fv[side])
                nb.append(M1 @ P @ (fv[side] * -fa) / jxw)
            C = M1 @ (P @ R @ S) @ Minv / jxw
            Xm = np.moveaxis(X, nax, -1)
            lo = np.roll(Xm, 1, axis=cax) @ Minv[n - 1]
            hi = np.roll(Xm, -1, axis=cax) @ Minv[0]
            Y += np.moveaxis(Xm @ C.T + lo[..., None] * nb[0] + hi[..., None] * nb[1], -1, nax)
        ref = O.dg_advect_apply_transpose(g, x)
        assert np.linalg.norm(Y.ravel() - ref) / np.linalg.norm(ref) < 1e-13, (nc, "transpose, inverse mass")


@pytest.mark.parametrize("p", range(1, 9))
def test_cell_faces_are_kronecker_sums(p):
    """The DO_FACES cell operators on a Cartesian cell (Hermite-like basis,
    M1 = S^T W S): convection = sum_f L_f (x) M1 (x) M1 with
    L_f = b_f ij_f jxw S^T D^T W S - jf (e_p - e_0) flux^T; Laplacian =
    sum_f (K_f + F1_f) (x) M1 (x) M1 + sum_f F2_f (x) Tp (x) Tp with
    Tp = S W S, K_f = jxw ij_f^2 (D S)^T W (D S) and rank-one face terms
    F1_f, F2_f: the identities behind the line-operator evaluation of
    SF_OP_CONVECTION_FACES and SF_OP_LAPLACE_FACES"""
    n = p + 1
    sh = O.shape_arrays(p, O.BASIS_HERMITE)
    S, D, w, hd = sh["S"], sh["D"], sh["wq"], sh["hermite_d0"]
    M1, Tp, DS = S.T @ np.diag(w) @ S, S @ np.diag(w) @ S, D @ S
    h = (0.3, 0.2, 0.45)
    ij, jxw = [1 / v for v in h], h[0] * h[1] * h[2]
    b = (1.0, 0.5, -0.25)
    E, n3 = np.eye(n), n ** 3
    for conv in (True, False):
        K = np.stack([O.cell_faces(p, conv, ij, jxw, b if conv else (0., 0., 0.), e) for e in np.eye(n3)], axis=1)
        Kc = np.zeros_like(K)
        for f in range(3):
            jf = jxw * ij[f]
            terms = []
            if conv:
                flux = 0.5 * (b[f] * (E[p] + E[0]) + abs(b[f]) * (E[p] - E[0]))
                L = b[f] * ij[f] * jxw * S.T @ D.T @ np.diag(w) @ S - jf * np.outer(E[p] - E[0], flux)
                terms.append((L, M1))
            else:
                rowv = n * n * ij[f] * (E[p] + E[0]) - 0.5 * ij[f] * hd * (E[p - 1] - E[p] + E[1] - E[0])
                L = jxw * ij[f] ** 2 * DS.T @ np.diag(w) @ DS + jf * np.outer(E[p] - E[0], rowv)
                F2 = -jf * ij[f] * hd * np.outer(-E[p] + E[p - 1] - E[0] + E[1], 0.5 * (E[p] + E[0]))
                terms += [(L, M1), (F2, Tp)]
            for A_f, T_t in terms:
                mats = [T_t, T_t, T_t]
                mats[f] = A_f
                Kc += np.kron(mats[2], np.kron(mats[1], mats[0]))
        assert np.abs(K - Kc).max() < 1e-13 * np.abs(K).max(), conv


@pytest.mark.parametrize("basis", [0, 1])
@pytest.mark.parametrize("p", range(1, 9))
def test_affine_continuous_operators_are_assembled_kronecker_products(p, basis):
    """On a structured affine mesh the assembled continuous mass, Laplacian and
    convection operators are M_z M_y M_x, sum_d K_d (x) M (x) M and
    sum_d C_d (x) M (x) M with assembled banded 1D matrices (cell matrices
    h M1, K1 / h, b C1); with Dirichlet conditions every 1D matrix loses its
    boundary rows and columns and the boundary rows become y = x: the
    identity behind the Kronecker passes of the affine continuous apply"""
    sh = O.shape_arrays(p, basis)
    S, D, w = sh["S"], sh["D"], sh["wq"]
    M1 = S.T @ np.diag(w) @ S
    K1 = (D @ S).T @ np.diag(w) @ (D @ S)
    C1 = S.T @ D.T @ np.diag(w) @ S
    b = (0.7, -1.3, 0.4)

    def assembled(A1, nc):
        G = np.zeros((nc * p + 1, nc * p + 1))
        for c in range(nc):
            G[c * p:c * p + p + 1, c * p:c * p + p + 1] += A1
        return G

    def app(Az, Ay, Ax, X):
        return np.einsum("ck,kyx->cyx", Az, np.einsum("bj,zjx->zbx", Ay, np.einsum("ai,zyi->zya", Ax, X)))

    for nc, length, dirichlet in (((3, 2, 4), (0.9, 0.5, 1.3), 1), ((2, 1, 3), (1.0, 0.4, 0.75), 0),
                                  ((1, 3, 2), (0.5, 1.0, 0.8), 1)):
        h = [length[d] / nc[d] for d in range(3)]
        m = O.mesh(p, nc, basis=basis, length=length, dirichlet=dirichlet)
        x = np.random.default_rng(p).uniform(-1, 1, O.cont_n_dofs(m))
        nn = [nc[d] * p + 1 for d in range(3)]
        Pd = [np.diag(np.r_[1 - dirichlet, np.ones(nn[d] - 2), 1 - dirichlet]) for d in range(3)]
        Md = [Pd[d] @ assembled(h[d] * M1, nc[d]) @ Pd[d] for d in range(3)]
        Kd = [Pd[d] @ assembled(K1 / h[d], nc[d]) @ Pd[d] for d in range(3)]
        Cd = [Pd[d] @ assembled(b[d] * C1, nc[d]) @ Pd[d] for d in range(3)]
        X = x.reshape(nn[2], nn[1], nn[0])
        bnd = np.zeros_like(X, dtype=bool)
        if dirichlet:
            bnd[0] = bnd[-1] = bnd[:, 0] = bnd[:, -1] = bnd[:, :, 0] = bnd[:, :, -1] = True
        cases = (("mass", O.cont_apply_op(m, O.OP_MASS, x, b), app(Md[2], Md[1], Md[0], X)),
                 ("convection", O.cont_apply_op(m, O.OP_CONVECTION, x, b),
                  app(Md[2], Md[1], Cd[0], X) + app(Md[2], Cd[1], Md[0], X) + app(Cd[2], Md[1], Md[0], X)),
                 ("laplacian", O.cont_apply(m, None, x),
                  app(Md[2], Md[1], Kd[0], X) + app(Md[2], Kd[1], Md[0], X) + app(Kd[2], Md[1], Md[0], X)))
        for name, ref, Y in cases:
            Y = np.where(bnd, X, Y).ravel()
            assert np.linalg.norm(Y - ref) / np.linalg.norm(ref) < 1e-13, (name, nc)


@pytest.mark.parametrize("p", [1, 2, 4, 7])
def test_continuous_null_space_boundary_rows_and_volume(p):
    """GLL basis, deformed box: without Dirichlet conditions the Laplacian
    annihilates constants (the nodal basis sums to one) and its quadratic
    form, the Dirichlet energy, is positive off the constants; with them the
    boundary rows are the identity and the interior rows ignore boundary
    values; the mass matrix integrates one to the box volume"""
    nc, length = (3, 2, 2), (0.9, 0.6, 0.5)
    rng = np.random.default_rng(p)
    m0 = O.mesh(p, nc, length=length, deform=0.05, dirichlet=0)
    G = O.cont_geometry(m0)
    n = O.cont_n_dofs(m0)
    x = rng.uniform(-1, 1, n)
    ax = O.cont_apply(m0, G, x)
    assert np.abs(O.cont_apply(m0, G, np.ones(n))).max() < 1e-13 * np.abs(ax).max()
    assert x @ ax > 0
    nn = [p * c + 1 for c in nc]
    Z, Y, X = np.meshgrid(*(np.arange(k) for k in nn[::-1]), indexing="ij")
    bnd = ((X == 0) | (X == nn[0] - 1) | (Y == 0) | (Y == nn[1] - 1) | (Z == 0) | (Z == nn[2] - 1)).ravel()
    m1 = O.mesh(p, nc, length=length, deform=0.05, dirichlet=1)
    y1 = O.cont_apply(m1, G, x)
    assert np.array_equal(y1[bnd], x[bnd])
    x0 = np.where(bnd, 0.0, x)
    assert np.allclose(y1[~bnd], O.cont_apply(m1, G, x0)[~bnd], rtol=0, atol=1e-14 * np.abs(y1).max())
    assert np.allclose(y1[~bnd], ax[~bnd] - O.cont_apply(m0, G, x - x0)[~bnd], rtol=0,
                       atol=1e-13 * np.abs(y1).max())
    ma = O.mesh(p, nc, length=length, dirichlet=0)
    one = np.ones(O.cont_n_dofs(ma))
    assert abs(one @ O.cont_apply_op(ma, O.OP_MASS, one) - np.prod(length)) < 1e-14


@pytest.mark.parametrize("p", [1, 3, 5, 8])
def test_advect_conserves_and_transports_constants(p):
    """periodic mesh, constant velocity, GLL nodal basis: the upwind fluxes
    cancel across faces and the basis sums to one, so the entries of A u sum
    to zero (conservation, 1^T A = 0) and A 1 = 0 (a constant state does not
    change), also with the inverse mass"""
    d = O.dg(p, (3, 2, 2), (0.3, 0.5, 0.2), velocity=(1.0, -0.5, 0.25), inverse_mass=0)
    u = np.random.default_rng(p).uniform(-1, 1, O.dg_n_dofs(d))
    one = np.ones_like(u)
    au = O.dg_advect_apply(d, u)
    assert abs(au.sum()) < 1e-14 * np.abs(au).sum()
    assert np.abs(O.dg_advect_apply(d, one)).max() < 1e-14 * np.abs(au).max()
    assert abs(O.dg_advect_apply_transpose(d, u).sum()) < 1e-14 * np.abs(au).sum()
    di = O.dg(p, (3, 2, 2), (0.3, 0.5, 0.2), velocity=(1.0, -0.5, 0.25), inverse_mass=1)
    assert np.abs(O.dg_advect_apply(di, one)).max() < 1e-13 * np.abs(O.dg_advect_apply(di, u)).max()


@pytest.mark.parametrize("p", [1, 3, 5, 8])
def test_dg_laplacians_periodic_null_space(p):
    """periodic meshes: the SIPG operator and its precomputed tensor-product
    form annihilate constants (the Hermite-like basis sums to one), so the
    entries of A u sum to zero as well (symmetry), and u^T A u > 0 off the
    constants"""
    mesh, h = (3, 2, 2), (0.3, 0.5, 0.2)
    for d, apply in ((O.dg(p, mesh, h, penalty=1.5), O.dg_sipg_apply), (O.dg(p, mesh, h), O.dg_precomputed_apply)):
        u = np.random.default_rng(p).uniform(-1, 1, O.dg_n_dofs(d))
        au = apply(d, u)
        assert np.abs(apply(d, np.ones_like(u))).max() < 1e-14 * np.abs(au).max()
        assert abs(au.sum()) < 1e-14 * np.abs(au).sum()
        assert u @ au > 0
