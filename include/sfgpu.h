/*
 * sfgpu.h -- C ABI of the GB300 (sm_103a) matrix-free sum-factorization
 * operators.
 *
 * The reference (KKraljic/sum_factorization_kernels, directory legacy/) has
 * no library interface: its operator "API" is a family of template member
 * functions of evaluator classes that own their vectors.  Each entry point
 * below names the member function whose job it takes over; the vectors that
 * the reference keeps as private members are passed in here as caller-owned
 * device buffers.
 *
 * Conventions
 *  - Every function returns SF_OK (0) or a negative sf_status; no C++
 *    exception crosses the ABI.  sf_last_error() describes the last failure
 *    of the calling thread.
 *  - Vector and array pointers are DEVICE pointers unless a parameter name
 *    ends in _host.  They must be aligned to the element size; the library
 *    never frees them.  An output vector of an operator apply or Chebyshev
 *    step must not overlap any other vector of the call (checked by
 *    address range, SF_ERR_INVALID); inputs may share storage.  The
 *    Runge-Kutta stage and step and sf_vector_update state their own
 *    aliasing rules beside their declarations.
 *  - Work is ordered on the given stream (0 = legacy default stream) and is
 *    asynchronous unless stated otherwise.  A handle is not re-entrant: calls
 *    on one handle must not overlap; distinct handles are independent.
 *  - Precision: SF_FP64 vectors are double, SF_FP32 vectors are float.
 *
 * Vector layouts
 *  - continuous (SF_OP_LAPLACE, SF_OP_MASS, SF_OP_CONVECTION): global
 *    lexicographic nodes of the
 *    (p*nx+1) x (p*ny+1) x (p*nz+1) grid, x fastest; cell (i,j,k) local node
 *    (a,b,c) is global ((k*p+c)*(p*ny+1) + (j*p+b))*(p*nx+1) + (i*p+a).
 *    Restricted to one cell this is the reference's cell-local order
 *    (evaluation_cell_laplacian.h:157-160).  With homogeneous Dirichlet
 *    conditions the boundary nodes stay in the vector: the operator reads
 *    them as zero and its boundary rows are the identity (y_b = x_b).
 *  - DG (SF_OP_DG_SIPG, SF_OP_DG_ADVECT): cell-major, n^3 values per cell
 *    in the cell-local order, cells x fastest.  This is the reference's
 *    lane-interleaved layout (evaluation_dg_laplacian.h:162-166) with one
 *    lane.
 */
#ifndef SFGPU_H
#define SFGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SF_OK = 0,
  SF_ERR_INVALID = -1,      /* bad argument value                              */
  SF_ERR_NULL = -2,         /* required pointer is NULL                        */
  SF_ERR_UNSUPPORTED = -3,  /* degree / precision / operator combination       */
  SF_ERR_CUDA = -4,         /* CUDA runtime error (see sf_last_error)          */
  SF_ERR_OOM = -5,          /* device allocation failed                        */
  SF_ERR_NOT_CONVERGED = -6,/* solver hit its iteration limit                  */
  SF_ERR_BREAKDOWN = -7,    /* solver produced NaN/Inf or a non-positive curvature */
  SF_ERR_ALIGN = -8,        /* pointer not aligned to its element size         */
  SF_ERR_STATE = -9         /* call not valid for this handle's configuration  */
} sf_status;

typedef enum { SF_FP64 = 0, SF_FP32 = 1 } sf_prec;

typedef enum {
  SF_OP_LAPLACE = 0,   /* continuous FE Laplacian -div(kappa grad u)           */
  SF_OP_DG_SIPG = 1,   /* DG symmetric interior penalty Laplacian, periodic     */
  SF_OP_DG_ADVECT = 2, /* DG upwind advection, periodic                        */
  SF_OP_DG_PRECOMPUTED = 3, /* DG SIPG Laplacian in tensor-product form with
                          precomputed 1D mass and stiffness matrices, Hermite-
                          like basis, penalty p(p+1), periodic; replaces
                          PrecomputedDGLaplacian (precomputed_dg_laplacian.h:
                          44-377): sf_vmult = matrix_vector_product() */
  SF_OP_MASS = 4,      /* continuous mass matrix (u, v), affine meshes; the
                          DO_MASS_MATRIX variant of the cell Laplacian
                          (evaluation_cell_laplacian.h:299-326)              */
  SF_OP_CONVECTION = 5, /* continuous convection form (u, b . grad v) with a
                          constant b = desc.velocity, affine meshes; the
                          DO_CONVECTION variant (evaluation_cell_laplacian.h:
                          328-354), there with b = (1, 2, 3)                 */
  SF_OP_LAPLACE_UNSTRUCTURED = 6, /* continuous Laplacian on an unstructured
                          hexahedral mesh (sf_create_unstructured; the
                          reference has no mesh input at all)                */
  SF_OP_LAPLACE_FACES = 7, /* the DO_FACES build of the cell Laplacian
                          (evaluation_cell_laplacian.h:505-797): per
                          Cartesian cell of a cell-major vector (n^3 entries
                          per cell, Hermite-like basis), the cell Laplacian
                          plus face terms between the cell's own faces at 0
                          and 1; block diagonal, sf_vmult / sf_vmult_batched */
  SF_OP_CONVECTION_FACES = 8 /* the DO_FACES + DO_CONVECTION build: the cell
                          convection form (u, b . grad v), b = desc.velocity,
                          plus upwind fluxes between the cell's own faces    */
} sf_op_kind;

typedef enum { SF_BASIS_GLL = 0, SF_BASIS_HERMITE = 1 } sf_basis;

typedef struct {
  int kind;            /* sf_op_kind                                            */
  int degree;          /* 1..8                                                  */
  int n_cells[3];      /* hexahedral cells per direction                        */
  double length[3];    /* domain [0,Lx]x[0,Ly]x[0,Lz]                           */
  int basis;           /* continuous operators (DG SIPG and precomputed:
                          Hermite-like, DG advect: GLL)                         */
  double deform;       /* SF_OP_LAPLACE: amplitude a of the mapping
                          x_i <- x_i + a sin(2 pi x_j) sin(2 pi x_k), (i,j,k)
                          cyclic; 0 = affine (geometry not stored)            */
  int dirichlet;       /* continuous: 1 = homogeneous Dirichlet boundary       */
  double penalty;      /* SF_OP_DG_SIPG: tau = penalty (p+1)^2 / h_d (ref: 1)  */
  double velocity[3];  /* SF_OP_DG_ADVECT, SF_OP_CONVECTION                     */
  int inverse_mass;    /* SF_OP_DG_ADVECT: 1 = apply M^-1 (reference do_matvec) */
  int precisions;      /* bit 0: prepare FP64, bit 1: prepare FP32             */
} sf_desc;

typedef struct sf_op sf_op;

const char *sf_last_error(void);
const char *sf_version(void);

/* Replaces initialize() of the evaluator classes
 * (evaluation_cell_laplacian.h:34-101, evaluation_dg_laplacian.h:43-108,
 * evaluation_dg_advect.h:107-180, benchmark_loops.cc:1163-1200): builds the
 * shape tables and, for a deformed mesh, the per-quadrature-point geometry
 * on the device (FP64, plus an FP32 copy).  An affine continuous operator
 * (SF_OP_LAPLACE with deform 0, SF_OP_MASS, SF_OP_CONVECTION) whose node
 * grid fits the Kronecker passes (at most 65535 node planes along z) also
 * gets their work vectors: 2 (SF_OP_MASS: 1) vectors of n_dofs entries of
 * the widest prepared precision, so that no apply allocates.  Synchronous. */
int sf_create(const sf_desc *desc, sf_op **op);
int sf_destroy(sf_op *op);

/* The continuous Laplacian on an unstructured hexahedral mesh of degree
 * 1..8 (no counterpart in the reference, whose evaluators take structured
 * meshes only).  Host arrays, copied:
 *  - cell_nodes[e (p+1)^3 + (z (p+1) + y)(p+1) + x]: global index in
 *    [0, n_nodes) of node (x, y, z) of cell e, in the cell-local order of the
 *    structured layout (x fastest).  Each cell's orientation is the caller's:
 *    a rotated or reflected cell lists its nodes in its own local frame.
 *    A cell lists each node once (SF_ERR_INVALID otherwise).
 *  - merged6[e][6][(p+1)^3]: JxW J^-1 J^-T at the Gauss points of cell e in
 *    that local frame (order xx, yy, zz, xy, xz, yz; quadrature weight
 *    included), as sf_set_geometry.
 *  - dirichlet[node] != 0: homogeneous Dirichlet node (row y = x); may be
 *    NULL.
 * Cells are coloured greedily on the host (cells of one colour share no
 * node) and summed colour by colour without atomics.  The handle takes
 * sf_vmult, sf_vmult_batched, sf_chebyshev_step, and sf_cg_solve without a
 * preconditioner; n_dofs = n_nodes.  basis: sf_basis; precisions as in
 * sf_desc. */
int sf_create_unstructured(int degree, int basis, long long n_cells, long long n_nodes,
                           const int *cell_nodes, const double *merged6,
                           const unsigned char *dirichlet, int precisions, sf_op **op);
/* number of vector entries, number of cells */
int sf_sizes(const sf_op *op, long long *n_dofs, long long *n_cells);

/* Overrides the merged geometry of a SF_OP_LAPLACE handle with a deformed
 * layout: G[cell][6][n^3] (xx,yy,zz,xy,xz,yz; JxW * J^-1 J^-T per Gauss
 * point), FP64 device array.  Replaces the jacobian_data member
 * (benchmark_loops.cc:1177-1197). */
int sf_set_geometry(sf_op *op, const double *merged6);
/* Per-quadrature-point coefficient kappa[cell][n^3] (FP64 device array),
 * NULL to remove.  No reference counterpart (new in this library). */
int sf_set_coefficient(sf_op *op, const double *kappa);

/* y = A x.  Replaces matrix_vector_product() (evaluation_cell_laplacian.h:216,
 * benchmark_loops.cc:1302) and do_matvec() (evaluation_dg_laplacian.h:121,
 * evaluation_dg_advect.h:216). */
int sf_vmult(sf_op *op, int prec, const void *x, void *y, void *stream);
/* y = A^T x.  The Laplacians are symmetric (A^T = A); for advection this is
 * the transpose-upwind adjoint.  No reference counterpart. */
int sf_vmult_transpose(sf_op *op, int prec, const void *x, void *y, void *stream);
/* y[r] = A x[r] for r < nrhs (1..64); x and y hold nrhs vectors of n_dofs
 * entries back to back.  The DG and face-term operators treat all
 * right-hand sides in one launch; the continuous operators apply them one
 * after another on the stream. */
int sf_vmult_batched(sf_op *op, int prec, int nrhs, const void *x, void *y, void *stream);
int sf_vmult_transpose_batched(sf_op *op, int prec, int nrhs, const void *x, void *y,
                               void *stream);

/* The transposed advection apply of sf_vmult_transpose_batched() for callers
 * that cannot allocate device memory while they run: applications that hand
 * out all device memory from their own pool or reserve a fixed budget up
 * front, and loops that cannot take the device synchronisation an
 * allocation implies.  No counterpart in the reference.  (The default
 * line-operator path of sf_vmult_transpose_batched() applies K^T M^-1 in one
 * launch and needs no intermediate vector; its cell-and-face path,
 * SF_KERNEL_GENERIC, allocates one per handle on first use.)  This function
 * always runs the cell-and-face two-pass form, with the intermediate vector
 * of the inverse-mass form in a 4 MiB array compiled into the library
 * (reserved on every GPU that loads it, until process exit) instead of a
 * cudaMalloc'd buffer; it allocates nothing.  Only for SF_OP_DG_ADVECT
 * handles; nrhs * n_dofs * element size must not exceed 4 MiB
 * (SF_ERR_INVALID otherwise).  Every call looks up the array's device
 * address in the current context (so calls after cudaDeviceReset() use the
 * reloaded array), and the first call with each degree and precision loads
 * that kernel.
 * All calls share the array (nothing in it needs to start at zero), so
 * calls whose work overlaps on the GPU race: keep them on one stream or
 * synchronise between them. */
int sf_vmult_transpose_static(sf_op *op, int prec, int nrhs, const void *x, void *y,
                              void *stream);

/* Fused Chebyshev step, replaces do_cheby_iter<true>
 * (evaluation_dg_laplacian.h:513-554, fused update :485-502):
 *   t     <- c_tm * t + c_np * diag_inv .* (A x_old - b)
 *   x_new <- x_old - t
 * (the reference reads its member vector sol_rhs for b; this uses b). */
int sf_chebyshev_step(sf_op *op, int prec, const void *b, const void *diag_inv,
                      const void *x_old, void *x_new, void *t, double c_np,
                      double c_tm, void *stream);
/* Fused Runge-Kutta stage of the DG advection operator, replaces
 * do_rk_stage<true> (evaluation_dg_advect.h:679-707, stage update
 * :651-667):  r = A src (with the inverse mass when the handle has
 * inverse_mass = 1, the reference's operator), then
 *   vec_np = upd + c_np * r   and, when c_tm != 0,   vec_tm = vec_np + c_tm * r
 * (vec_tm is not touched when c_tm == 0 and may then be NULL).  upd may be the
 * same vector as src, vec_np or vec_tm, as in the reference's do_time_step;
 * any other overlap (src with an output, vec_np with vec_tm, upd partly
 * over another vector) is refused with SF_ERR_INVALID.  nrhs vectors of
 * n_dofs entries each, contiguous.  The reference's current_time argument
 * only names the exact solution's transport direction, which here is the
 * handle's velocity. */
int sf_rk_stage(sf_op *op, int prec, int nrhs, const void *src, const void *upd, void *vec_np,
                void *vec_tm, double c_np, double c_tm, void *stream);
/* One step of the five-stage fourth-order low-storage Runge-Kutta scheme of
 * do_time_step (evaluation_dg_advect.h:190-214) with step dt: five fused
 * stages with the reference's coefficients and register rotation; sol_new
 * is advanced in place, sol_old and sol_tmp are the scheme's two registers
 * (contents on entry are not used; three vectors that do not overlap). */
int sf_lsrk_step(sf_op *op, int prec, int nrhs, void *sol_new, void *sol_old, void *sol_tmp, double dt,
                 void *stream);
/* The same update without the operator, replaces
 * emulate_cheby_vector_updates() (evaluation_dg_laplacian.h:556-601):
 *   t <- c_tm * t + c_np * diag_inv .* (ax - b);  x_new <- x_old - t
 * ax may be x_new itself (the reference's emulation passes sol_new as both);
 * otherwise the outputs x_new and t overlap neither each other nor an input
 * (SF_ERR_INVALID).  Inputs may share storage. */
int sf_vector_update(long long n, int prec, const void *ax, const void *b,
                     const void *diag_inv, const void *x_old, void *x_new, void *t,
                     double c_np, double c_tm, void *stream);

/* Diagonal of A (for Jacobi / Chebyshev).  The reference uses a placeholder
 * of ones (evaluation_dg_laplacian.h:88). */
int sf_diagonal(sf_op *op, int prec, void *diag, void *stream);

/* d(loss)/d(kappa_q) = grad(u)_q . G_q grad(lam)_q per Gauss point
 * (FP64/FP32 u, lam; output [cell][n^3] of the same precision), gradients
 * recomputed.  With lam = A x - b and u = x this is the kappa-gradient of
 * 1/2 |A(kappa) x - b|^2.  No reference counterpart. */
int sf_kappa_gradient(sf_op *op, int prec, const void *u, const void *lam, void *dkappa,
                      void *stream);

/* Kernel selection.  Continuous operators: SF_KERNEL_AUTO evaluates the
 * affine structured ones without a coefficient (SF_OP_LAPLACE with deform 0
 * and no sf_set_coefficient, SF_OP_MASS, SF_OP_CONVECTION) as Kronecker
 * products of assembled 1D matrices (a pass along z, then x-y tiles of each
 * node plane) in FP64, and in FP32 where that measured faster (the
 * Laplacian and mass matrix at every degree, convection up to degree 5);
 * everything else (deformed, coefficient, unstructured, more than 65535
 * node planes along z, the remaining FP32 cases) runs on the packed
 * line-ownership kernel (one thread per line of a cell, several cells per
 * warp group); SF_KERNEL_GENERIC selects the line-ownership kernel for all
 * of them.  Both give the same operator to rounding.  SF_OP_DG_SIPG:
 * SF_KERNEL_AUTO evaluates the operator in its tensor-product form (on
 * these Cartesian meshes the SIPG bilinear form is exactly
 * L (x) M (x) M + M (x) L (x) M + M (x) M (x) L with 1D stiffness-plus-face
 * matrices L of penalty * (p+1)^2 and 1D mass matrices M: the kernel of
 * SF_OP_DG_PRECOMPUTED), SF_KERNEL_GENERIC the cell-and-face
 * kernel that follows the reference's EvaluationDGLaplacian step by step;
 * both give the same operator to rounding.  SF_OP_DG_ADVECT: SF_KERNEL_AUTO
 * evaluates M^-1 A as a sum of 1D line operators, sum_d B_d (x) I (x) I
 * with each line coupled to the upwind neighbour's end node (constant
 * velocity, Cartesian cells), and A and A^T as M times such a sum;
 * SF_KERNEL_GENERIC the cell-and-face kernel that follows the reference's
 * EvaluationDGAdvection step by step; the same operator to rounding.
 * SF_OP_LAPLACE_FACES and SF_OP_CONVECTION_FACES: SF_KERNEL_AUTO evaluates
 * the cell operator as sum_f L_f (x) M1 (x) M1 (1D stiffness- or
 * convection-plus-own-face matrices L_f, 1D mass M1; for the Laplacian plus
 * a rank-one face term per direction), SF_KERNEL_GENERIC the face-array
 * kernel.  Other values are rejected with SF_ERR_INVALID.  No reference
 * counterpart. */
typedef enum {
  SF_KERNEL_AUTO = 0,
  SF_KERNEL_GENERIC = 1
} sf_kernel_variant;
int sf_set_kernel_variant(sf_op *op, int variant);
/* Device-side error flags of the handle's kernels (bit 0: a bounded wait
 * for an asynchronous copy timed out; the result of that apply is invalid).
 * Synchronous.  No reference counterpart. */
int sf_device_status(sf_op *op, int *flags);

/* ---------------- conjugate gradients ---------------- */
typedef enum {
  SF_SOLVE_FP64 = 0,        /* plain CG, FP64 operator                          */
  SF_SOLVE_MIXED = 1        /* FP32 preconditioned CG with reliable updates by
                               the true FP64 residual, FP64 refinement steps
                               as the fallback                                 */
} sf_solve_mode;

typedef enum { SF_PRECOND_NONE = 0, SF_PRECOND_JACOBI = 1, SF_PRECOND_CHEBYSHEV = 2 } sf_precond;

typedef struct {
  int mode;              /* sf_solve_mode                                        */
  int precond;           /* sf_precond                                           */
  int cheb_degree;       /* Chebyshev polynomial degree (default 5)              */
  double cheb_range;     /* smoothing range lambda_max / lambda_min (default 15) */
  int eig_iterations;    /* Lanczos steps for lambda_max (default 12)            */
  double rtol;           /* relative residual target |b - A x| / |b|             */
  int max_iter;          /* total inner iterations allowed                       */
  double inner_rtol;     /* SF_SOLVE_MIXED: reliable-update factor (0.03): the
                            FP32 CG replaces its residual by the true FP64
                            residual b - A x whenever the recursive one has
                            dropped by this factor since the last replacement */
  int project_constant;  /* 1: remove the mean from b and x (periodic SIPG)      */
} sf_solve_opts;

typedef struct {
  int iterations;        /* CG iterations (inner, for SF_SOLVE_MIXED)            */
  int outer_iterations;  /* SF_SOLVE_MIXED: FP64 true-residual updates of the
                            iterate (reliable updates and refinement steps)  */
  double rel_residual;   /* final |b - A x| / |b| in FP64                        */
  double lambda_max;     /* estimate used by the Chebyshev preconditioner        */
  double seconds;        /* wall time of the solve (device synchronised)         */
  int operator_applies;  /* number of operator applications                      */
} sf_solve_stats;

void sf_solve_opts_default(sf_solve_opts *opts);
/* Solves A x = b (FP64 device vectors, x holds the initial guess).  No
 * reference counterpart: the reference has no solver.  Synchronous. */
int sf_cg_solve(sf_op *op, const double *b, double *x, const sf_solve_opts *opts,
                sf_solve_stats *stats, void *stream);

/* ---------------- design measurements ---------------- */
/* The slab sweeps of the operator kernels in isolation: n_cells cells of
 * (degree+1)^3 values (cell-major, x fastest) are loaded into shared memory,
 * `rounds` times the interpolation matrix S (Gauss points of the GLL basis)
 * is applied along x and then along y, and the result is written to out.
 * method selects the arithmetic: SF_SWEEP_EO_FP32 / SF_SWEEP_EO_FP64 the
 * CUDA-core even-odd contraction of the operator kernels (one thread per
 * line), SF_SWEEP_MMA_TF32X3 the tensor cores (mma.sync m16n8k8, TF32
 * operands split into high part and remainder, three products, FP32
 * accumulation), SF_SWEEP_MMA_TF32 one TF32 product.  in/out are float
 * (double for SF_SWEEP_EO_FP64).  No reference counterpart: it measures the
 * choice between the two arithmetic units for matrix_vector_kernel.h:30-185. */
typedef enum {
  SF_SWEEP_EO_FP32 = 0,
  SF_SWEEP_MMA_TF32X3 = 1,
  SF_SWEEP_MMA_TF32 = 2,
  SF_SWEEP_EO_FP64 = 3
} sf_sweep_method;
int sf_sweep_benchmark(int degree, int method, long long n_cells, int rounds, const void *in, void *out,
                       void *stream);

/* ---------------- utilities ---------------- */
/* FP64 <-> FP32 vector conversion */
int sf_convert(long long n, int from_prec, const void *x, int to_prec, void *y, void *stream);
/* deterministic FP64 dot product of two vectors of precision prec; the result
 * is written to a device double (result_dev) -- no host synchronisation */
int sf_dot(long long n, int prec, const void *x, const void *y, double *result_dev,
           void *stream);
/* shape tables used by the kernels (FP64, for inspection and tests):
 * S[q*n+i], D[q*n+j], weights[n]; n = degree+1 */
int sf_shape_tables(int degree, int basis, double *S_host, double *D_host,
                    double *points_host, double *weights_host);

#ifdef __cplusplus
}
#endif
#endif
