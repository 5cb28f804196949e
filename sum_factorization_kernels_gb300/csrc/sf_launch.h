// sf_launch.h -- host launchers of the device kernels (one per .cu file).
#pragma once

#include <cuda_runtime.h>

#include "sf_internal.h"

namespace sf {

// sf_laplace.cu
int launch_cont_vmult(const sf_op *op, int prec, const void *x, void *y, cudaStream_t st);
int launch_cont_kappa_grad(const sf_op *op, int prec, const void *u, const void *lam, void *dk,
                           cudaStream_t st);
int launch_geometry(const sf_op *op, double *G, cudaStream_t st);
int launch_cont_diagonal(const sf_op *op, int prec, void *diag, cudaStream_t st);

// sf_cont_kron.cu: continuous Laplacian (affine, no coefficient), mass and
// convection forms on structured meshes as Kronecker products of assembled
// 1D matrices (a z pass and an x-y tile pass over the node grid)
bool kron_eligible(const sf_op *op);
int kron_work_vectors(const sf_op *op); // work vectors of n_dofs entries the passes need
bool kron_selected(const sf_op *op, int prec); // the default apply of this precision uses them
int launch_cont_kron(const sf_op *op, int prec, const void *x, void *y, cudaStream_t st);

// sf_laplace_line.cu (all degrees, FP64 and FP32)
int launch_cont_vmult_line(const sf_op *op, int prec, const void *x, void *y, cudaStream_t st);
// walk-ordered copy of the FP64 geometry for the line kernel (geoLine64 / geoLine32)
int pack_line_geometry(sf_op *op, int prec);

// sf_dg.cu
int launch_dg_vmult(const sf_op *op, int prec, int nrhs, bool transpose, const void *x, void *y,
                    const void *cheb_b, const void *cheb_dinv, void *cheb_t, double c_np,
                    double c_tm, cudaStream_t st);
int launch_dg_inverse_mass(const sf_op *op, int prec, int nrhs, const void *x, void *y,
                           cudaStream_t st);
// fused advection Runge-Kutta stage: r = M^-1 A src, vec_np = upd + c_np r,
// vec_tm = vec_np + c_tm r (when c_tm != 0)
int launch_dg_rk_stage(const sf_op *op, int prec, int nrhs, const void *src, const void *upd, void *vec_np,
                       void *vec_tm, double c_np, double c_tm, cudaStream_t st);
int launch_dg_diagonal(const sf_op *op, int prec, void *diag, cudaStream_t st);

// sf_dg_precomputed.cu: tensor-product SIPG with precomputed 1D matrices
int launch_dg_precomputed(const sf_op *op, int prec, int nrhs, const void *x, void *y, const void *cheb_b,
                          const void *cheb_dinv, void *cheb_t, double c_np, double c_tm, cudaStream_t st);
int launch_dg_precomputed_diagonal(const sf_op *op, int prec, void *diag, cudaStream_t st);

// sf_dg_advect_tensor.cu: DG advection as a sum of 1D line operators; the
// inverse-mass apply (forward with inverse_mass), otherwise the mass form;
// rk_np non-null: fused Runge-Kutta stage (as launch_dg_rk_stage)
int launch_dg_advect_tensor(const sf_op *op, int prec, int nrhs, bool transpose, const void *x, void *y,
                            const void *cheb_b, const void *cheb_dinv, void *cheb_t, double c_np, double c_tm,
                            const void *rk_upd, void *rk_np, void *rk_tm, cudaStream_t st);
// the DO_FACES operators in the same form: sum_f L_f (x) M1 (x) M1 (plus, for
// the Laplacian, a rank-one face term per direction)
int launch_faces_tensor(const sf_op *op, int prec, int nrhs, const void *x, void *y, cudaStream_t st);

// sf_cell_faces.cu: the DO_FACES cell operators (block diagonal, cell-major)
int launch_cell_faces(const sf_op *op, int prec, int nrhs, const void *x, void *y, cudaStream_t st);

// SM count of the current device (cached per device ordinal)
int device_sm_count();
// grid of a grid-stride kernel over n items: one block per `threads` items,
// at most per_sm blocks per SM
int stream_grid(long long n, int threads, int per_sm);

// blocks of a kernel that fit on one SM with the maximum shared-memory
// carveout: the occupancy calculator does not account for the carveout
// preference, so persistent grids size themselves from the limits directly
int resident_blocks_per_sm(const void *kernel, int threads, size_t dyn_smem, int *blocks);

#define SF_RET_IF(x)                                                           \
  do {                                                                         \
    int r_ = (x);                                                              \
    if (r_ != SF_OK) return r_;                                                \
  } while (0)

// sf_vector.cu
int launch_convert(long long n, int from, const void *x, int to, void *y, cudaStream_t st);
int launch_vector_update(long long n, int prec, const void *ax, const void *b, const void *dinv,
                         const void *x_old, void *x_new, void *t, double c_np, double c_tm,
                         cudaStream_t st);
// partial sums for a deterministic dot product: needs dot_scratch_doubles()
int launch_dot(long long n, int prec, const void *x, const void *y, double *scratch,
               double *result, cudaStream_t st);
constexpr int kDotBlocks = 1024;

} // namespace sf
