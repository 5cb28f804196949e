"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Run on a host that has the reference checkout (it compiles
``oracle/ref_src/*.cc`` against the reference's headers through
``oracle/build.py build_ref``):

    python tests/golden/gen_golden.py

Every array written here comes from the reference's compiled code
(``oracle/_ref/*.so``), never from the oracle restatement; the tests then
pin the oracle (and through it the CUDA library) to these vectors.  The
continuous-FE fixtures wrap the reference's cell operator in a gather /
scatter over the global lexicographic numbering that this library defines
(the reference has no global numbering).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import refbind as R  # noqa: E402

SEED = 20241203


def cont_index_arrays(degree, nc):
    """global index and Dirichlet flag of every cell-local node, x fastest"""
    p = degree
    n = p + 1
    Nx, Ny, Nz = p * nc[0] + 1, p * nc[1] + 1, p * nc[2] + 1
    c, b, a = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    idx, bnd = [], []
    for k in range(nc[2]):
        for j in range(nc[1]):
            for i in range(nc[0]):
                X, Y, Z = i * p + a, j * p + b, k * p + c
                idx.append(((Z * Ny + Y) * Nx + X).ravel())
                bnd.append(((X == 0) | (Y == 0) | (Z == 0) | (X == Nx - 1) | (Y == Ny - 1)
                            | (Z == Nz - 1)).ravel())
    return np.array(idx), np.array(bnd), Nx * Ny * Nz


def ref_cont_apply(degree, nc, length, x):
    """gather -> reference GLL cell operator (benchmark_loops.cc) -> scatter,
    homogeneous Dirichlet rows as identity"""
    idx, bnd, N = cont_index_arrays(degree, nc)
    h = np.array(length, dtype=np.float64) / np.array(nc)
    # merged tensor without quadrature weight: det(J) J^-2 on the diagonal
    detJ = h[0] * h[1] * h[2]
    G6 = np.array([detJ / h[0] ** 2, detJ / h[1] ** 2, detJ / h[2] ** 2, 0, 0, 0])
    y = np.zeros(N)
    for c in range(idx.shape[0]):
        u = np.where(bnd[c], 0.0, x[idx[c]])
        v = R.gll_cell(degree, G6, u)
        np.add.at(y, idx[c][~bnd[c]], v[~bnd[c]])
    allb = np.zeros(N, dtype=bool)
    allb[idx[bnd]] = True
    y[allb] = x[allb]
    return y, allb


def main():
    rng = np.random.default_rng(SEED)
    out = {}

    # quadrature, bases and even-odd tables
    for p in range(1, 9):
        n = p + 1
        out["gauss_x_%d" % n], out["gauss_w_%d" % n] = R.gauss(n)
        out["gll_x_%d" % n] = R.gll(n)
        s, d, w = R.gll_tables(p)
        out["gll_S_eo_%d" % p], out["gll_D_eo_%d" % p] = s, d
        s, d, w, h0 = R.herm_tables(p)
        out["herm_S_eo_%d" % p], out["herm_D_eo_%d" % p] = s, d
        out["herm_d0_%d" % p] = np.array([h0])
        f, si = R.dg_tables(p)
        out["face_eo_%d" % p], out["Sinv_eo_%d" % p] = f, si
    np.savez(os.path.join(HERE, "tables.npz"), **out)

    # 1D even-odd kernel on random coefficients (the transposed values kernel
    # for odd n is exercised with the real tables, see sf_oracle.c dev. (3))
    out = {}
    combos = [(0, 1, 0, 0), (0, 1, 1, 0), (1, 1, 0, 0), (1, 0, 0, 0), (1, 0, 1, 0),
              (1, 1, 0, 2), (1, 0, 0, 2), (1, 0, 1, 2), (0, 0, 0, 0), (0, 0, 1, 0)]
    k = 0
    for nn in range(2, 10):
        st = (nn + 1) // 2
        for (t, c, a, g) in combos:
            if t == 0 and c == 0 and nn % 2 == 1:
                coef = R.gll_tables(nn - 1)[0]
            else:
                coef = rng.standard_normal(nn * st)
            x = rng.standard_normal(nn)
            o = rng.standard_normal(nn)
            dg = rng.standard_normal(2 * nn)
            fc = rng.standard_normal(4)
            r, f = R.apply_1d(nn, t, c, a, g, coef, x, o, dg, fc)
            out["k%03d_meta" % k] = np.array([nn, t, c, a, g])
            out["k%03d_coef" % k], out["k%03d_x" % k], out["k%03d_o" % k] = coef, x, o
            out["k%03d_dg" % k], out["k%03d_fin" % k] = dg, fc
            out["k%03d_y" % k], out["k%03d_fout" % k] = r, f
            k += 1
    np.savez(os.path.join(HERE, "kernel1d.npz"), **out)

    # single cells: GLL basis with a full symmetric merged tensor, Hermite-like
    # basis with the reference's Cartesian Jacobian diag(4, 2, 4/3)
    out = {}
    for p in range(1, 9):
        n = p + 1
        G6 = rng.uniform(0.5, 1.5, 6) * np.array([1, 1, 1, .2, .2, .2])
        x = rng.uniform(-1, 1, n ** 3)
        out["gll_G6_%d" % p], out["gll_x_%d" % p] = G6, x
        out["gll_y_%d" % p] = R.gll_cell(p, G6, x)
        ij = np.array([4.0, 2.0, 4.0 / 3.0])
        jxw = 1.0 / np.prod(ij)
        out["herm_x_%d" % p] = x
        out["herm_y_%d" % p] = R.herm_cell(p, ij, jxw, x)
    np.savez(os.path.join(HERE, "cell.npz"), **out)

    # continuous Laplacian, affine box, homogeneous Dirichlet
    out = {}
    for p in range(1, 9):
        nc = (3, 2, 2) if p <= 4 else (2, 2, 2)
        length = (1.0, 0.8, 1.2)
        _, _, N = cont_index_arrays(p, nc)
        x = rng.uniform(-1, 1, N)
        y, bnd = ref_cont_apply(p, nc, length, x)
        x[bnd] = 0.0
        y[bnd] = 0.0
        out["x_%d" % p], out["y_%d" % p] = x, y
        out["nc_%d" % p], out["len_%d" % p] = np.array(nc), np.array(length)
    # the Q4 16^3 unit-cube case: x regenerated from its seed, y sampled
    p, nc = 4, (16, 16, 16)
    idx, bnd, N = cont_index_arrays(p, nc)
    x = np.random.default_rng(SEED).uniform(-1.0, 1.0, N)
    y, allb = ref_cont_apply(p, nc, (1.0, 1.0, 1.0), x)
    sample = np.sort(np.random.default_rng(SEED + 1).choice(N, 4096, replace=False))
    out["q4_16_sample_idx"] = sample
    out["q4_16_sample_y"] = y[sample]
    out["q4_16_norm2"] = np.array([np.linalg.norm(y)])
    out["q4_16_sum"] = np.array([y.sum()])
    np.savez(os.path.join(HERE, "cont.npz"), **out)

    # DG SIPG (penalty factor 1, the reference's) and its fused Chebyshev step
    out = {}
    for p in range(1, 9):
        if p == 2:
            continue  # reference drops a nonzero term for the degree-2 Hermite basis
        nc, h = ((3, 2, 4) if p <= 4 else (3, 2, 2)), (0.3, 0.5, 0.2)
        N = nc[0] * nc[1] * nc[2] * (p + 1) ** 3
        x = rng.uniform(-1, 1, N)
        out["x_%d" % p], out["y_%d" % p] = x, R.dg_sipg(p, nc, h, x)
        out["nc_%d" % p], out["h_%d" % p] = np.array(nc), np.array(h)
        if p == 5:
            b = rng.standard_normal(N)
            dinv = rng.uniform(0.5, 1.5, N)
            t = rng.uniform(-1, 1, N)
            xn, tn = R.dg_sipg(p, nc, h, x, b=b, dinv=dinv, t=t, c_np=0.7, c_tm=0.3)
            out.update(cheb_b=b, cheb_dinv=dinv, cheb_t=t, cheb_xnew=xn, cheb_tnew=tn)
    np.savez(os.path.join(HERE, "dg_sipg.npz"), **out)

    # DG upwind advection with M^-1, the reference's velocity (1, 0.15, -0.05)
    out = {}
    for p in range(1, 9):
        nc, h = ((3, 2, 4) if p <= 4 else (3, 2, 2)), (0.3, 0.5, 0.2)
        N = nc[0] * nc[1] * nc[2] * (p + 1) ** 3
        x = rng.uniform(-1, 1, N)
        out["x_%d" % p], out["y_%d" % p] = x, R.dg_advect(p, nc, h, x)
        out["nc_%d" % p], out["h_%d" % p] = np.array(nc), np.array(h)
    np.savez(os.path.join(HERE, "dg_advect.npz"), **out)


def rk_fixtures():
    """the reference's fused Runge-Kutta stage (do_rk_stage<true>) and its
    LSRK(5,4) time step (do_time_step), own seed so the other fixtures keep
    their values"""
    rng = np.random.default_rng(20241207)
    out = {}
    for p in (1, 2, 4, 5):
        nc, h = ((3, 2, 4) if p <= 4 else (3, 2, 2)), (0.3, 0.5, 0.2)
        N = nc[0] * nc[1] * nc[2] * (p + 1) ** 3
        src, upd, tm0 = rng.uniform(-1, 1, N), rng.uniform(-1, 1, N), rng.uniform(-1, 1, N)
        for case, (c_np, c_tm) in (("a", (0.013, -0.007)), ("b", (0.021, 0.0))):
            vnp, vtm = R.dg_rk_stage(p, nc, h, src, upd, c_np, c_tm, vec_tm=tm0)
            out["np_%s_%d" % (case, p)], out["tm_%s_%d" % (case, p)] = vnp, vtm
            out["c_%s_%d" % (case, p)] = np.array([c_np, c_tm])
        x0 = rng.uniform(-1, 1, N)
        dt = 0.2 * min(h) / (np.linalg.norm([1.0, 0.15, -0.05]) * p)
        out["src_%d" % p], out["upd_%d" % p], out["tm0_%d" % p] = src, upd, tm0
        out["x0_%d" % p], out["dt_%d" % p] = x0, np.array(dt)
        out["steps3_%d" % p] = R.dg_time_steps(p, nc, h, x0, 3, dt)
        out["nc_%d" % p], out["h_%d" % p] = np.array(nc), np.array(h)
    np.savez(os.path.join(HERE, "dg_rk.npz"), **out)


def precomputed_fixtures():
    """the reference's PrecomputedDGLaplacian on unit cells (periodic), with
    the neighbour-coupling and odd-n add-into lines patched (oracle/build.py
    PATCHES); inputs stored in FP32 to keep the file small"""
    rng = np.random.default_rng(20241208)
    out = {}
    for p in (1, 2, 3, 4, 5, 6, 8):
        nc = (3, 2, 2) if p <= 4 else (2, 2, 2)
        N = nc[0] * nc[1] * nc[2] * (p + 1) ** 3
        x = rng.uniform(-1, 1, N).astype(np.float32)
        out["x_%d" % p], out["y_%d" % p] = x, R.dg_precomputed(p, nc, x.astype(np.float64))
        out["nc_%d" % p] = np.array(nc)
    np.savez(os.path.join(HERE, "dg_precomputed.npz"), **out)


def ref_cont_apply_variant(degree, nc, length, x, variant):
    """gather -> the reference's Hermite-like Cartesian cell operator built
    with DO_MASS_MATRIX / DO_CONVECTION -> scatter, Dirichlet rows identity"""
    idx, bnd, N = cont_index_arrays(degree, nc)
    h = np.array(length, dtype=np.float64) / np.array(nc)
    ij, jxw = 1.0 / h, float(np.prod(h))
    y = np.zeros(N)
    for c in range(idx.shape[0]):
        u = np.where(bnd[c], 0.0, x[idx[c]])
        v = R.herm_cell(degree, ij, jxw, u, variant)
        np.add.at(y, idx[c][~bnd[c]], v[~bnd[c]])
    allb = np.zeros(N, dtype=bool)
    allb[idx[bnd]] = True
    y[allb] = x[allb]
    return y, allb


def cellop_fixtures():
    """the reference's DO_MASS_MATRIX and DO_CONVECTION builds of the
    Hermite-like cell operator (velocity (1, 2, 3)): single Cartesian cells
    with inverse Jacobian diag(4, 2, 4/3) and small affine boxes with
    homogeneous Dirichlet conditions; the DO_FACES builds (Laplacian and
    convection) on the same single cells (their face set-up takes the
    reference's fixed Jacobian diag(4, 2, 4/3), evaluation_cell_laplacian.h:
    46,84-100).  Degree 2 is stored too, but the
    reference's transposed values kernel drops the middle point for odd n
    (matrix_vector_kernel.h:130-131), which is wrong for the Hermite-like
    degree-2 basis (the reference's degree-2 mass matrix is not symmetric),
    so the tests pin degree 2 by the tensor-product identity instead."""
    rng = np.random.default_rng(20241209)
    out = {}
    ij = np.array([4.0, 2.0, 4.0 / 3.0])
    jxw = 1.0 / np.prod(ij)
    for p in range(1, 9):
        x = rng.uniform(-1, 1, (p + 1) ** 3)
        out["cell_x_%d" % p] = x
        out["cell_mass_%d" % p] = R.herm_cell(p, ij, jxw, x, "mass")
        out["cell_conv_%d" % p] = R.herm_cell(p, ij, jxw, x, "convection")
        out["cell_faces_%d" % p] = R.herm_cell(p, ij, jxw, x, "faces")
        out["cell_faces_conv_%d" % p] = R.herm_cell(p, ij, jxw, x, "faces_convection")
        nc = (3, 2, 2) if p <= 4 else (2, 2, 2)
        length = (1.0, 0.8, 1.2)
        _, _, N = cont_index_arrays(p, nc)
        xc = rng.uniform(-1, 1, N)
        for name, variant in (("mass", "mass"), ("conv", "convection")):
            y, bnd = ref_cont_apply_variant(p, nc, length, xc, variant)
            out["cont_%s_%d" % (name, p)] = np.where(bnd, 0.0, y)
        xc[bnd] = 0.0
        out["cont_x_%d" % p] = xc
        out["nc_%d" % p], out["len_%d" % p] = np.array(nc), np.array(length)
    np.savez(os.path.join(HERE, "cell_ops.npz"), **out)


if __name__ == "__main__":
    import sys
    if sys.argv[1:] == ["rk"]:
        rk_fixtures()
    elif sys.argv[1:] == ["precomputed"]:
        precomputed_fixtures()
    elif sys.argv[1:] == ["cellops"]:
        cellop_fixtures()
    else:
        main()
        rk_fixtures()
        precomputed_fixtures()
        cellop_fixtures()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
