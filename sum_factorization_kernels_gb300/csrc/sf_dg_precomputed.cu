// sf_dg_precomputed.cu -- DG SIPG Laplacian in tensor-product form with
// precomputed 1D matrices (the reference's PrecomputedDGLaplacian,
// precomputed_dg_laplacian.h:96-377), Hermite-like basis, periodic
// Cartesian mesh:
//
//   A = sum_d c_d (L + couplings)_d (x) M (x) M,   c_d = hx hy hz / h_d^2,
//
// M the 1D mass matrix, L the 1D stiffness matrix with the own-face SIPG
// terms (penalty p(p+1), reference coordinates), and two coefficients iv0,
// iv1 coupling the end nodes with the neighbour's two nearest node layers
// (a Hermite-like end value and normal derivative live on two layers).  On
// unit cells c_d = 1 and A is the reference's operator; the reference
// evaluates iv0 and iv1 at swapped face points (which makes them vanish),
// this library uses the couplings of the SIPG bilinear form.
//
// The general SIPG operator of SF_OP_DG_SIPG (sf_dg.cu, the reference's
// EvaluationDGLaplacian with tau = penalty (p+1)^2 / h_d) is the same
// Kronecker sum on these Cartesian meshes: its cell and face integrals are
// exact in the tangential directions (Gauss quadrature with n points on
// degree-p products), so they factor into 1D stiffness-plus-face matrices
// and 1D mass matrices, with the 1D penalty penalty (p+1)^2 instead of
// p(p+1).  SF_OP_DG_SIPG handles evaluate it with this kernel by default
// (SF_KERNEL_AUTO); SF_KERNEL_GENERIC selects the cell-and-face kernel.
//
// GPU mapping as in sf_dg.cu: CPB consecutive cells per block, n^2 threads
// per cell, z columns read and written straight from the cell-major vector,
// three padded slabs per cell.  Five phases, four block barriers:
//   z:  X = x;  Az = c_z (L_z x + z couplings)
//   x:  B  = c_x (L_x x + x couplings);        Az = M_x Az
//   y:  B  = M_y B;  Az = M_y Az;   X = c_y (L_y x + y couplings)
//   x:  B += M_x X
//   z:  y = M_z B + Az                       (or the fused Chebyshev step,
//                                             whose b and t arrive by
//                                             asynchronous copies during the
//                                             last two phases)
#include "sf_device.cuh"
#include "sf_dg_common.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"

namespace sf {

namespace {

template <int N, typename T>
struct PDGArgs {
  EOMat<N, T> M, L;        // symmetric and centro-symmetric 1D matrices
  T iv0, iv1;              // neighbour couplings
  T c[3];                  // hx hy hz / h_d^2
  const T *__restrict__ x;
  T *__restrict__ y;
  const T *__restrict__ cb;      // Chebyshev: rhs
  const T *__restrict__ cdinv;   // Chebyshev: inverse diagonal
  T *__restrict__ ct;            // Chebyshev: t
  T c_np, c_tm;
  int nc[3];
  FastDiv div_nx, div_ny;
  long long n_cells, n_dofs;
};

// Slabs X, Az, B of a block's cells: entry (x, y, z) of cell cs at
// BASE + cs RS + SX x + SY y + SZ z.  FP32 degrees 3 and 5: three regions
// with strides from the bank-conflict model (X: 1 z, 2 x, 2 y accesses per
// step; Az: 2, 2, 2; B: 1, 3, 2); otherwise dg_layout's padded layout with
// the three slabs of a cell side by side.
struct PDGSlab {
  int SX, SY, SZ, RS, BASE;
};
struct PDGSlabs {
  PDGSlab X, Az, B;
};

constexpr PDGSlabs pdg_slabs(int n, int elem, int cpb)
{
  if (elem == 4 && n == 4)
    return PDGSlabs{{1, 5, 20, 80, 0}, {1, 4, 19, 80, 8 * 80}, {1, 5, 20, 80, 16 * 80}};
  if (elem == 4 && n == 6)
    return PDGSlabs{{1, 49, 6, 292, 0}, {37, 1, 6, 228, 7 * 292}, {1, 49, 6, 292, 7 * (292 + 228)}};
  const DGLayout L = dg_layout(n, elem);
  const int slab = L.P2 * n, rs = 3 * slab + L.SKEW;
  (void)cpb;
  return PDGSlabs{{1, L.P1, L.P2, rs, 0}, {1, L.P1, L.P2, rs, slab}, {1, L.P1, L.P2, rs, 2 * slab}};
}

constexpr int pdg_slab_end(int n, int cpb, PDGSlab S)
{
  return S.BASE + (cpb - 1) * S.RS + (n - 1) * (S.SX + S.SY + S.SZ) + 1;
}

template <int N, typename T>
struct PDGCfg {
  static constexpr int CPB = DGCells<N>::value;
  static constexpr PDGSlabs S = pdg_slabs(N, (int)sizeof(T), CPB);
  static constexpr int E0 = pdg_slab_end(N, CPB, S.X), E1 = pdg_slab_end(N, CPB, S.Az),
                       E2 = pdg_slab_end(N, CPB, S.B);
  static constexpr int WORDS = E0 > E1 ? (E0 > E2 ? E0 : E2) : (E1 > E2 ? E1 : E2);
  static constexpr size_t SMEM = size_t(WORDS) * sizeof(T);
  // fused Chebyshev step: the b and t entries of each thread's column are
  // staged by asynchronous copies during the last two phases (FP32; at n = 8
  // and in FP64 the extra shared memory costs more residency than the hidden
  // latency gains: measured 186 vs 182 us at p = 7, 2512 vs 2493 us for FP64
  // p = 5, against 174 vs 224 us for FP32 p = 5)
  static constexpr int THREADS = CPB * N * N;
  static constexpr int STAGED = (sizeof(T) == 4 && N != 8) ? 2 : 0;
  static constexpr int STAGE0 = (WORDS + 3) / 4 * 4;
  static constexpr size_t SMEM_CHEB = (size_t(STAGE0) + STAGED * size_t(N) * THREADS) * sizeof(T);
};

template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst, const T *src)
{
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src),
               "n"((int)sizeof(T))
               : "memory");
}

// line residual of the 1D operator L plus the couplings with the two
// neighbours' end layers: lo1, lo2 = left neighbour's nodes n-1, n-2 of this
// line, hi1, hi2 = right neighbour's nodes 0, 1
template <int N, typename T>
__device__ __forceinline__ void stiffness_line(const PDGArgs<N, T> &A, const T (&v)[N], T lo1, T lo2, T hi1,
                                               T hi2, T scale, T (&r)[N])
{
  eo_apply<N, 1>(A.L, v, r);
  r[0] += A.iv0 * lo1 + A.iv1 * lo2;
  r[1] += A.iv1 * lo1;
  r[N - 1] += A.iv0 * hi1 + A.iv1 * hi2;
  r[N - 2] += A.iv1 * hi1;
#pragma unroll
  for (int m = 0; m < N; ++m) r[m] *= scale;
}

template <int N, typename T, bool CHEB>
__global__ void __launch_bounds__(DGCells<N>::value *N *N)
    dg_precomputed_kernel(const __grid_constant__ PDGArgs<N, T> A)
{
  using Cfg = PDGCfg<N, T>;
  constexpr int N2 = N * N, N3 = N * N * N;
  constexpr int CPB = Cfg::CPB;
  constexpr PDGSlab LX = Cfg::S.X, LA = Cfg::S.Az, LB = Cfg::S.B;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *smem = reinterpret_cast<T *>(smem_raw);
  const int tid = threadIdx.x;
  const int cs = tid / N2;
  const int t = tid - cs * N2;
  const int a = t % N, b = t / N;
  const long long cell = (long long)blockIdx.x * CPB + cs;
  const bool valid = cell < A.n_cells;
  T *X = smem + LX.BASE + cs * LX.RS;
  T *Az = smem + LA.BASE + cs * LA.RS;
  T *B = smem + LB.BASE + cs * LB.RS;
  // z column (a, b), x line (y=a, z=b), y line (x=a, z=b) in each slab
  const int zcX = LX.SX * a + LX.SY * b, xlX = LX.SY * a + LX.SZ * b, ylX = LX.SX * a + LX.SZ * b;
  const int zcA = LA.SX * a + LA.SY * b, xlA = LA.SY * a + LA.SZ * b, ylA = LA.SX * a + LA.SZ * b;
  const int zcB = LB.SX * a + LB.SY * b, xlB = LB.SY * a + LB.SZ * b, ylB = LB.SX * a + LB.SZ * b;
  const long long col = cell * N3 + t;
  const long long roff = (long long)blockIdx.y * A.n_dofs; // right-hand side offset
  const T *__restrict__ x = A.x + roff;

  // neighbour cells (periodic) in the three directions
  long long nb[3][2] = {{cell, cell}, {cell, cell}, {cell, cell}};
  if (valid) {
    const unsigned uc = (unsigned)cell;
    const unsigned q = fast_div(uc, A.div_nx);
    const unsigned iz = fast_div(q, A.div_ny);
    const int ix = int(uc - q * (unsigned)A.nc[0]), iy = int(q - iz * (unsigned)A.nc[1]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      nb[d][0] = periodic_neighbour(A.nc, ix, iy, int(iz), d, 0);
      nb[d][1] = periodic_neighbour(A.nc, ix, iy, int(iz), d, 1);
    }
  }
  T v[N], r[N];
  // ---- z: the z column of x; z stiffness with couplings ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = valid ? __ldg(x + col + N2 * m) : T(0);
#pragma unroll
  for (int m = 0; m < N; ++m) X[zcX + LX.SZ * m] = v[m];
  {
    T lo1 = T(0), lo2 = T(0), hi1 = T(0), hi2 = T(0);
    if (valid) {
      const T *xl_ = x + nb[2][0] * N3 + t, *xr_ = x + nb[2][1] * N3 + t;
      lo1 = __ldg(xl_ + N2 * (N - 1));
      lo2 = __ldg(xl_ + N2 * (N - 2));
      hi1 = __ldg(xr_);
      hi2 = __ldg(xr_ + N2);
    }
    stiffness_line<N, T>(A, v, lo1, lo2, hi1, hi2, A.c[2], r);
  }
#pragma unroll
  for (int m = 0; m < N; ++m) Az[zcA + LA.SZ * m] = r[m];
  __syncthreads();
  // ---- x: x stiffness with couplings into B; mass along x of Az ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = X[xlX + LX.SX * m];
  {
    // x line (y=a, z=b): node (m, a, b) at m + N a + N2 b
    T lo1 = T(0), lo2 = T(0), hi1 = T(0), hi2 = T(0);
    if (valid) {
      const T *xl_ = x + nb[0][0] * N3 + N * a + N2 * b, *xr_ = x + nb[0][1] * N3 + N * a + N2 * b;
      lo1 = __ldg(xl_ + (N - 1));
      lo2 = __ldg(xl_ + (N - 2));
      hi1 = __ldg(xr_);
      hi2 = __ldg(xr_ + 1);
    }
    stiffness_line<N, T>(A, v, lo1, lo2, hi1, hi2, A.c[0], r);
  }
#pragma unroll
  for (int m = 0; m < N; ++m) B[xlB + LB.SX * m] = r[m];
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = Az[xlA + LA.SX * m];
  eo_apply<N, 1>(A.M, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) Az[xlA + LA.SX * m] = v[m];
  __syncthreads();
  // ---- y: mass along y of B and Az; y stiffness with couplings into X ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B[ylB + LB.SY * m];
  eo_apply<N, 1>(A.M, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) B[ylB + LB.SY * m] = v[m];
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = Az[ylA + LA.SY * m];
  eo_apply<N, 1>(A.M, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) Az[ylA + LA.SY * m] = v[m];
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = X[ylX + LX.SY * m];
  {
    // y line (x=a, z=b): node (a, m, b) at a + N m + N2 b
    T lo1 = T(0), lo2 = T(0), hi1 = T(0), hi2 = T(0);
    if (valid) {
      const T *xl_ = x + nb[1][0] * N3 + a + N2 * b, *xr_ = x + nb[1][1] * N3 + a + N2 * b;
      lo1 = __ldg(xl_ + N * (N - 1));
      lo2 = __ldg(xl_ + N * (N - 2));
      hi1 = __ldg(xr_);
      hi2 = __ldg(xr_ + N);
    }
    stiffness_line<N, T>(A, v, lo1, lo2, hi1, hi2, A.c[1], r);
  }
#pragma unroll
  for (int m = 0; m < N; ++m) X[ylX + LX.SY * m] = r[m];
  __syncthreads();
  T *stage = smem + Cfg::STAGE0 + tid;
  if (CHEB && Cfg::STAGED && valid) {
    // b and t of the epilogue, in flight during the last two phases
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const long long e = col + N2 * m;
      cp_async_elem(stage + (0 * N + m) * Cfg::THREADS, A.cb + e);
      cp_async_elem(stage + (1 * N + m) * Cfg::THREADS, A.ct + e);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  // ---- x: B += M_x X ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = X[xlX + LX.SX * m];
  eo_apply<N, 1>(A.M, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) B[xlB + LB.SX * m] += v[m];
  __syncthreads();
  // ---- z: y = M_z B + Az ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B[zcB + LB.SZ * m];
  eo_apply<N, 1>(A.M, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] += Az[zcA + LA.SZ * m];
  if (valid) {
    T *dst = A.y + roff + col;
    if (CHEB) {
      if (Cfg::STAGED) asm volatile("cp.async.wait_group 0;" ::: "memory");
#pragma unroll
      for (int m = 0; m < N; ++m) {
        const long long e = col + N2 * m;
        const T vb = Cfg::STAGED ? stage[(0 * N + m) * Cfg::THREADS] : A.cb[e];
        const T vt = Cfg::STAGED ? stage[(1 * N + m) * Cfg::THREADS] : A.ct[e];
        const T res = v[m] - vb;
        const T tn = A.c_tm * vt + A.c_np * __ldg(A.cdinv + e) * res;
        A.ct[e] = tn;
        dst[N2 * m] = __ldg(x + e) - tn;
      }
    } else {
#pragma unroll
      for (int m = 0; m < N; ++m) dst[N2 * m] = v[m];
    }
  }
}

// fill a vector with a per-cell pattern of n^3 values
template <typename T>
__global__ void precomputed_pattern_kernel(long long n, int n3, const T *__restrict__ pat, T *__restrict__ y)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = pat[i % n3];
}

// 1D matrices in FP64 from the Hermite-like tables: values and collocation
// derivatives at the Gauss points, Gauss-Lagrange extrapolation to the faces
// (exact for the degree-p basis); fill_shape_values of
// precomputed_dg_laplacian.h:307-377 with the SIPG couplings
struct Matrices1D {
  double M[kMaxN][kMaxN], L[kMaxN][kMaxN], iv0, iv1;
};

Matrices1D precomputed_matrices(const Shape1D &s, double pen)
{
  const int n = s.n;
  Matrices1D R{};
  double v0[kMaxN], v1[kMaxN], d0[kMaxN], d1[kMaxN], dq[kMaxN][kMaxN];
  for (int i = 0; i < n; ++i) {
    v0[i] = v1[i] = d0[i] = d1[i] = 0.0;
    for (int q = 0; q < n; ++q) {
      v0[i] += s.fv[0][q] * s.S[q][i];
      v1[i] += s.fv[1][q] * s.S[q][i];
      d0[i] += s.fd[0][q] * s.S[q][i];
      d1[i] += s.fd[1][q] * s.S[q][i];
      double t = 0.0;
      for (int j = 0; j < n; ++j) t += s.D[q][j] * s.S[j][i];
      dq[q][i] = t;
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double m = 0.0, l = 0.0;
      for (int q = 0; q < n; ++q) {
        m += s.wq[q] * s.S[q][i] * s.S[q][j];
        l += s.wq[q] * dq[q][i] * dq[q][j];
      }
      l += pen * v0[i] * v0[j] + 0.5 * d0[i] * v0[j] + 0.5 * d0[j] * v0[i];
      l += pen * v1[i] * v1[j] - 0.5 * d1[i] * v1[j] - 0.5 * d1[j] * v1[i];
      R.M[i][j] = m;
      R.L[i][j] = l;
    }
  R.iv0 = -pen * v0[0] * v1[n - 1] - 0.5 * d0[0] * v1[n - 1] + 0.5 * d1[n - 1] * v0[0];
  R.iv1 = -pen * v0[0] * v1[n - 2] - 0.5 * d0[0] * v1[n - 2] + 0.5 * d1[n - 2] * v0[0];
  return R;
}

// 1D penalty in reference coordinates: p(p+1) for the reference's
// PrecomputedDGLaplacian, penalty (p+1)^2 for the SIPG operator
double tensor_penalty(const sf_op *op)
{
  const double p = op->desc.degree;
  if (op->desc.kind == SF_OP_DG_SIPG) return op->desc.penalty * (p + 1) * (p + 1);
  return p * (p + 1);
}

template <int N, typename T>
int precomputed_impl(const sf_op *op, int nrhs, const T *x, T *y, const T *cb, const T *cdinv, T *ct,
                     double c_np, double c_tm, cudaStream_t st)
{
  using Cfg = PDGCfg<N, T>;
  const Matrices1D mats = precomputed_matrices(op->shape, tensor_penalty(op));
  PDGArgs<N, T> A{};
  A.M = make_eo<N, T>([&](int i, int j) { return mats.M[i][j]; });
  A.L = make_eo<N, T>([&](int i, int j) { return mats.L[i][j]; });
  A.iv0 = T(mats.iv0);
  A.iv1 = T(mats.iv1);
  const double vol = op->h[0] * op->h[1] * op->h[2];
  for (int d = 0; d < 3; ++d) {
    A.c[d] = T(vol / (op->h[d] * op->h[d]));
    A.nc[d] = op->desc.n_cells[d];
  }
  A.div_nx = make_fast_div((unsigned)A.nc[0]);
  A.div_ny = make_fast_div((unsigned)A.nc[1]);
  A.n_cells = op->n_cells;
  A.n_dofs = op->n_dofs;
  A.x = x;
  A.y = y;
  A.cb = cb;
  A.cdinv = cdinv;
  A.ct = ct;
  A.c_np = T(c_np);
  A.c_tm = T(c_tm);
  void (*kern)(const PDGArgs<N, T>) = cb ? dg_precomputed_kernel<N, T, true> : dg_precomputed_kernel<N, T, false>;
  const size_t smem = cb ? Cfg::SMEM_CHEB : Cfg::SMEM;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  const long long blocks = (op->n_cells + Cfg::CPB - 1) / Cfg::CPB;
  kern<<<dim3((unsigned)blocks, (unsigned)nrhs), dim3(Cfg::CPB * N * N), smem, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N>
int precomputed_n(const sf_op *op, int prec, int nrhs, const void *x, void *y, const void *cb, const void *cd,
                  void *ct, double c_np, double c_tm, cudaStream_t st)
{
  if (prec == SF_FP64)
    return precomputed_impl<N, double>(op, nrhs, (const double *)x, (double *)y, (const double *)cb,
                                       (const double *)cd, (double *)ct, c_np, c_tm, st);
  return precomputed_impl<N, float>(op, nrhs, (const float *)x, (float *)y, (const float *)cb,
                                    (const float *)cd, (float *)ct, c_np, c_tm, st);
}

} // namespace

int launch_dg_precomputed(const sf_op *op, int prec, int nrhs, const void *x, void *y, const void *cb,
                          const void *cdinv, void *ct, double c_np, double c_tm, cudaStream_t st)
{
  switch (op->n) {
  case 2: return precomputed_n<2>(op, prec, nrhs, x, y, cb, cdinv, ct, c_np, c_tm, st);
  case 3: return precomputed_n<3>(op, prec, nrhs, x, y, cb, cdinv, ct, c_np, c_tm, st);
  case 4: return precomputed_n<4>(op, prec, nrhs, x, y, cb, cdinv, ct, c_np, c_tm, st);
  case 5: return precomputed_n<5>(op, prec, nrhs, x, y, cb, cdinv, ct, c_np, c_tm, st);
  case 6: return precomputed_n<6>(op, prec, nrhs, x, y, cb, cdinv, ct, c_np, c_tm, st);
  case 7: return precomputed_n<7>(op, prec, nrhs, x, y, cb, cdinv, ct, c_np, c_tm, st);
  case 8: return precomputed_n<8>(op, prec, nrhs, x, y, cb, cdinv, ct, c_np, c_tm, st);
  case 9: return precomputed_n<9>(op, prec, nrhs, x, y, cb, cdinv, ct, c_np, c_tm, st);
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;
  }
}

// diagonal: sum_d c_d L_ii (x) M_jj (x) M_kk per cell (the couplings are off
// the diagonal), computed in FP64 on the host and broadcast to all cells
int launch_dg_precomputed_diagonal(const sf_op *op, int prec, void *diag, cudaStream_t st)
{
  const Matrices1D m = precomputed_matrices(op->shape, tensor_penalty(op));
  const int n = op->n, n3 = n * n * n;
  const double vol = op->h[0] * op->h[1] * op->h[2];
  double c[3];
  for (int d = 0; d < 3; ++d) c[d] = vol / (op->h[d] * op->h[d]);
  // 1D diagonals; a direction one cell thick is its own periodic neighbour,
  // and at n = 2 the couplings with the neighbour's end layers then land on
  // the diagonal (targets 0, 1, n-2, n-1 of the coupling terms)
  double ld[3][kMaxN];
  for (int d = 0; d < 3; ++d) {
    for (int i = 0; i < n; ++i) ld[d][i] = m.L[i][i];
    if (op->desc.n_cells[d] != 1) continue;
    const struct {
      int target, source;
      double coef;
    } cpl[6] = {{0, n - 1, m.iv0}, {0, n - 2, m.iv1}, {1, n - 1, m.iv1},
                {n - 1, 0, m.iv0}, {n - 1, 1, m.iv1}, {n - 2, 0, m.iv1}};
    for (const auto &e : cpl)
      if (e.target == e.source) ld[d][e.target] += e.coef;
  }
  double pat[kMaxN * kMaxN * kMaxN];
  float patf[kMaxN * kMaxN * kMaxN];
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double v = c[0] * ld[0][i] * m.M[j][j] * m.M[k][k] + c[1] * m.M[i][i] * ld[1][j] * m.M[k][k] +
                         c[2] * m.M[i][i] * m.M[j][j] * ld[2][k];
        pat[(k * n + j) * n + i] = v;
        patf[(k * n + j) * n + i] = float(v);
      }
  DevBuf buf;
  const size_t es = prec == SF_FP64 ? sizeof(double) : sizeof(float);
  int r = buf.alloc(n3 * es);
  if (r) return r;
  SF_CUDA_TRY(cudaMemcpyAsync(buf.ptr, prec == SF_FP64 ? (const void *)pat : (const void *)patf, n3 * es,
                              cudaMemcpyHostToDevice, st));
  if (prec == SF_FP64)
    precomputed_pattern_kernel<double><<<device_sm_count() * 8, 256, 0, st>>>(op->n_dofs, n3, (const double *)buf.ptr,
                                                               (double *)diag);
  else
    precomputed_pattern_kernel<float><<<device_sm_count() * 8, 256, 0, st>>>(op->n_dofs, n3, (const float *)buf.ptr,
                                                              (float *)diag);
  SF_CUDA_TRY(cudaGetLastError());
  // the staging buffer is released when buf goes out of scope
  SF_CUDA_TRY(cudaStreamSynchronize(st));
  return SF_OK;
}

} // namespace sf
