/*
 * sf_oracle.h -- FP64 CPU oracle for the sum-factorization operators.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: the parity tests,
 * smoke() and the CPU-baseline leg of bench.py call it to produce the
 * expected results that the CUDA library must reproduce.  No product code
 * path links, loads or calls it.
 *
 * It is a plain-C restatement of the reference's algorithms
 * (KKraljic/sum_factorization_kernels, directory legacy/):
 *   - quadrature       gauss_formula.h:35-175
 *   - 1D bases         lagrange_polynomials.h:31-274
 *   - shape tables     evaluation_cell_laplacian.h:815-886 (Hermite-like),
 *                      src/benchmark_loops.cc:1387-1470 (GLL),
 *                      evaluation_dg_laplacian.h:615-695,
 *                      evaluation_dg_advect.h:729-825
 *   - 1D even-odd kernel matrix_vector_kernel.h:30-185
 *   - cell Laplacian   src/benchmark_loops.cc:1302-1385 (sweep order) with the
 *                      merged 6-entry quadrature-point tensor of
 *                      evaluation_cell_laplacian.h:392-415
 *   - DG SIPG          evaluation_dg_laplacian.h:130-510 (x-wrap index fixed)
 *   - DG advection     evaluation_dg_advect.h:286-676  (x-wrap index fixed)
 *   - Chebyshev update evaluation_dg_laplacian.h:485-502, 556-601
 * plus restatements, written from the mathematics, of the pieces the
 * reference does not have (continuous numbering with homogeneous Dirichlet,
 * deformed geometry, per-quadrature-point coefficient, adjoints, CG).
 *
 * Parity of this oracle is pinned against golden vectors produced by the
 * reference's own headers compiled here (tests/golden/, generated by
 * tests/golden/gen_golden.py through oracle/ref_wrap.cc).
 */
#ifndef SF_ORACLE_H
#define SF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define SFO_MAX_N 10

enum { SFO_BASIS_GLL = 0, SFO_BASIS_HERMITE = 1 };

typedef struct {
  int degree, n, basis;
  double xq[SFO_MAX_N], wq[SFO_MAX_N];   /* Gauss points/weights on [0,1] */
  double xgll[SFO_MAX_N];                /* Gauss-Lobatto points on [0,1] */
  /* full matrices */
  double S[SFO_MAX_N * SFO_MAX_N];    /* S[q*n+i] = phi_i(xq_q)                  */
  double D[SFO_MAX_N * SFO_MAX_N];    /* D[q*n+j] = l_j'(xq_q), Gauss-Lagrange   */
  double Sinv[SFO_MAX_N * SFO_MAX_N]; /* Sinv[i*n+q] = l_q(xgll_i)               */
  double face_v[2][SFO_MAX_N];        /* l_j(0), l_j(1)   (Gauss-Lagrange)       */
  double face_d[2][SFO_MAX_N];        /* l_j'(0), l_j'(1)                        */
  double hermite_d0;                  /* phi_0'(0) of the Hermite-like basis     */
  /* the reference's even-odd layouts */
  double S_eo[SFO_MAX_N * SFO_MAX_N];
  double D_eo[SFO_MAX_N * SFO_MAX_N];
  double Sinv_eo[SFO_MAX_N * SFO_MAX_N];
  double face_eo[2 * SFO_MAX_N];
} sfo_shape;

/* quadrature and bases */
void sfo_gauss(int n, double *points, double *weights);
void sfo_gll_points(int n, double *points);
int sfo_shape_init(int degree, int basis, sfo_shape *s);

/* restated 1D even-odd kernel (matrix_vector_kernel.h:30-185) */
void sfo_apply_1d(int nn, int stride, int type, int contract_over_rows,
                  int add_into, const double *coef_eo, const double *in,
                  double *out, const double *array_for_add, int do_dg,
                  const double *dg_coef, double *array_face);
/* plain n x n reference for the same contraction (test_multiplication.cc) */
void sfo_apply_1d_plain(int n, int stride, const double *M, int transpose,
                        const double *in, double *out);

/* ---------------- continuous Laplacian ---------------- */
typedef struct {
  int degree, basis;
  int n_cells[3];
  double length[3];        /* box [0,Lx]x[0,Ly]x[0,Lz]                       */
  double deform;           /* amplitude of x_i += a sin(2 pi x_j) sin(2 pi x_k) */
  int dirichlet;           /* 1: homogeneous Dirichlet on the whole boundary  */
} sfo_mesh;

long long sfo_cont_n_dofs(const sfo_mesh *m);
/* merged tensor G[cell][6][nq] = JxW * J^-1 J^-T (order xx,yy,zz,xy,xz,yz) */
void sfo_cont_geometry(const sfo_mesh *m, double *G);
/* y = A x (kappa may be NULL => 1).  Dirichlet rows: y_b = x_b.  G may be
 * NULL: each cell's merged tensor is then computed where it is used (the
 * same values as sfo_cont_geometry, without the [cell][6][nq] array). */
void sfo_cont_apply(const sfo_mesh *m, const double *G, const double *kappa,
                    const double *x, double *y, int n_threads);
/* dL/dkappa_q = grad(u)_q . G_q grad(lam)_q with Dirichlet entries zeroed */
void sfo_cont_kappa_grad(const sfo_mesh *m, const double *G, const double *u,
                         const double *lam, double *dk);
void sfo_cont_diagonal(const sfo_mesh *m, const double *G, const double *kappa,
                       double *diag);
/* apply the cell operator to one cell-local array (E-vector entry) with a
 * constant merged tensor (Cartesian) -- mirrors EvaluationCellLaplacian */
void sfo_cell_apply(const sfo_shape *s, const double *Gcell, int geo_stride,
                    const double *in, double *out);

/* mass matrix (kind 1) and convection form (u, b . grad v) (kind 2) of one
 * cell with inverse Jacobian diag(ij) and volume jxw: the DO_MASS_MATRIX and
 * DO_CONVECTION variants of evaluation_cell_laplacian.h (:299-326,
 * :328-354) */
void sfo_cell_op(const sfo_shape *s, int kind, const double *ij, double jxw,
                 const double *b, const double *in, double *out);
/* the DO_FACES build of the cell operator (evaluation_cell_laplacian.h:
 * 505-797): the Cartesian Laplacian (conv = 0) or the convection form
 * (conv = 1) of one cell plus face terms that couple the cell's faces at 0
 * and 1 in each direction, Hermite-like basis */
void sfo_cell_faces(const sfo_shape *s, int conv, const double *ij, double jxw, const double *b,
                    const double *in, double *out);
/* the same operator on every cell of a cell-major vector (n^3 entries per
 * cell) with cell size h */
void sfo_cell_faces_apply(int degree, int conv, long long n_cells, const double *h, const double *b,
                          const double *x, double *y);
/* y = A x on the affine continuous mesh (m->deform ignored) for those two
 * operators; Dirichlet rows as in sfo_cont_apply */
void sfo_cont_apply_op(const sfo_mesh *m, int kind, const double *b,
                       const double *x, double *y);

/* y = A x for the Laplacian on an unstructured hexahedral mesh: cell e's
 * local node q (x fastest) is idx[e nq + q], G[e][6][nq] its merged tensor,
 * dirichlet[node] != 0 (or NULL) homogeneous Dirichlet rows y = x */
void sfo_unstructured_apply(int degree, int basis, long long n_cells, long long n_nodes,
                            const int *idx, const double *G, const unsigned char *dirichlet,
                            const double *x, double *y);

/* ---------------- DG operators (cell-major layout, periodic) ------------- */
typedef struct {
  int degree;
  int n_cells[3];
  double h[3];             /* cell sizes                                       */
  double penalty;          /* SIPG: tau = penalty (p+1)^2 / h_d                */
  double velocity[3];      /* advection                                        */
  int inverse_mass;        /* advection: apply M^-1 (reference do_matvec)      */
} sfo_dg;

long long sfo_dg_n_dofs(const sfo_dg *g);
void sfo_dg_sipg_apply(const sfo_dg *g, const double *x, double *y);
void sfo_dg_sipg_diagonal(const sfo_dg *g, double *diag);
void sfo_dg_advect_apply(const sfo_dg *g, const double *x, double *y);
void sfo_dg_advect_apply_transpose(const sfo_dg *g, const double *x, double *y);
/* fused Runge-Kutta stage (evaluation_dg_advect.h:286-290,651-707):
 * r = advect_apply(src); vec_np = upd + c_np r; vec_tm = vec_np + c_tm r when
 * c_tm != 0 (vec_tm untouched otherwise).  upd may alias vec_np or vec_tm. */
void sfo_dg_rk_stage(const sfo_dg *g, const double *src, const double *upd,
                     double *vec_np, double *vec_tm, double c_np, double c_tm);
/* one step of the five-stage fourth-order low-storage Runge-Kutta scheme
 * (evaluation_dg_advect.h:190-214) with step dt: sol_new advanced in place,
 * sol_old and sol_tmp are the scheme's registers */
void sfo_dg_lsrk_step(const sfo_dg *g, double dt, double *sol_new, double *sol_old,
                      double *sol_tmp);

/* tensor-product SIPG Laplacian with precomputed 1D matrices
 * (precomputed_dg_laplacian.h:96-377), Hermite-like basis, periodic:
 *   A = sum_d c_d (L (+) couplings)_d x M x M,  c_d = hx hy hz / h_d^2
 * (c_d = 1 on the reference's unit cells).  M: 1D mass, L: 1D stiffness
 * with the own-face SIPG terms, penalty p(p+1); iv[0], iv[1]: couplings of
 * the end nodes with the neighbour's two nearest node layers (the reference
 * evaluates them at swapped face points, which makes them vanish). */
void sfo_dg_precomputed_matrices(int degree, double *M, double *L, double *iv);
void sfo_dg_precomputed_apply(const sfo_dg *g, const double *x, double *y);
void sfo_dg_precomputed_diagonal(const sfo_dg *g, double *diag);

/* ---------------- vector kernels ---------------- */
void sfo_chebyshev_update(long long n, const double *ax, const double *b,
                          const double *diag_inv, const double *x_old,
                          double *x_new, double *t, double c_np, double c_tm);

#ifdef __cplusplus
}
#endif
#endif
