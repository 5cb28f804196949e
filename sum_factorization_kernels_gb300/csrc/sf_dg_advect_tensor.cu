// sf_dg_advect_tensor.cu -- DG upwind advection on periodic Cartesian meshes
// with a constant velocity, as a sum of one-dimensional operators.
//
// The cell operator of evaluation_dg_advect.h:286-676 (GLL nodal basis,
// Gauss points, upwind flux (a.n) u_upwind) on a uniform Cartesian mesh
// separates by direction: with S the GLL-to-Gauss values, W the Gauss
// weights and R_d the Gauss-point residual of direction d (volume term
// D^T diag(c_d w) for the forward operator, diag(c_d w) D for the
// transpose, plus the face terms through the face-extrapolation rows),
//   A   = sum_d  (S^T R_d S) (x) M1 (x) M1,     M1 = S^T W S,
// the tangential directions contributing only the 1D mass matrix.  The
// neighbour across a face of direction d enters through its nodal end layer
// (its face value: a GLL node sits on the face), again times M1 (x) M1
// tangentially.  Hence, with B_d = (S^T W S)^-1 S^T R_d S = S^-1 W^-1 R_d S,
//   M^-1 A = sum_d B_d (x) I (x) I   (+ neighbour end-layer couplings)
//   A      = M (sum_d B_d (x) I (x) I)
// so the inverse-mass apply (the Runge-Kutta stage operator) is three
// line operators per cell and the plain apply and the transpose add three
// mass sweeps.  The 1D matrices are formed on the host in FP64 from the
// same tables as the cell-and-face kernel (sf_dg.cu), which remains
// selectable (SF_KERNEL_GENERIC) and agrees to rounding.
//
// GPU mapping as in the tensor-form SIPG kernel: a block holds CPB
// consecutive cells with n^2 threads each; the thread of z column (a, b)
// reads and writes that column of the cell-major vector (runs of n^2
// consecutive entries per warp instruction) and owns x line (y, z) = (a, b)
// and y line (x, z) = (a, b) of the shared-memory copy.  The x and y line
// results go to two slabs of their own, so one barrier separates the line
// phase from the column sum.
#include <cmath>

#include "sf_device.cuh"
#include "sf_dg_common.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"

namespace sf {

namespace {

enum { TA_STORE = 0, TA_CHEB = 1, TA_RK = 2 };

template <int N, typename T>
struct TAArgs {
  T B[3][N][N];        // line operator of direction d: r_i = sum_m B[d][i][m] u_m
  T cl[3][N], cr[3][N]; // couplings with the left neighbour's node n-1 / the right neighbour's node 0
  int nbmask;          // bit 2 d + side: the coupling of that side is nonzero
  EOMat<N, T> M;       // 1D mass matrix (plain apply and transpose)
  const T *__restrict__ x;
  T *__restrict__ y;
  const T *__restrict__ cb;    // Chebyshev: rhs
  const T *__restrict__ cdinv; // Chebyshev: inverse diagonal
  T *__restrict__ ct;          // Chebyshev: t
  T c_np, c_tm;
  // Runge-Kutta stage: vec_np = upd + c_np r, vec_tm = vec_np + c_tm r; upd
  // may alias vec_np or vec_tm (read before written, element by element)
  const T *rk_upd;
  T *rk_np, *rk_tm;
  int nc[3], nrhs;
  FastDiv div_nx, div_ny;
  long long n_cells, n_dofs;
};

// slabs X (input copy, and the mass sweeps), R1 (x line results), R2 (y line
// results): entry (x, y, z) of cell cs at BASE + cs RS + SX x + SY y + SZ z,
// the padded layout of dg_layout with the three slabs of a cell side by side
struct TASlab {
  int SX, SY, SZ, RS, BASE;
};

template <int N, typename T>
struct TACfg {
  static constexpr int CPB = DGCells<N>::value;
  static constexpr DGLayout L = dg_layout(N, (int)sizeof(T));
  static constexpr int SLAB = L.P2 * N;
  static constexpr int RS = 3 * SLAB + L.SKEW;
  static constexpr TASlab X{1, L.P1, L.P2, RS, 0}, R1{1, L.P1, L.P2, RS, SLAB}, R2{1, L.P1, L.P2, RS, 2 * SLAB};
  static constexpr size_t SMEM = size_t(CPB) * RS * sizeof(T); // per right-hand side
};

// every entry of the three slabs of a cell has its own word inside RS
constexpr bool ta_slabs_fit(int n, DGLayout L)
{
  bool seen[8192] = {};
  const int slab = L.P2 * n, rs = 3 * slab + L.SKEW;
  if (rs > 8192) return false;
  for (int s = 0; s < 3; ++s)
    for (int z = 0; z < n; ++z)
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
          const int i = s * slab + x + L.P1 * y + L.P2 * z;
          if (i >= rs || seen[i]) return false;
          seen[i] = true;
        }
  return true;
}
static_assert(ta_slabs_fit(2, dg_layout(2, 4)) && ta_slabs_fit(3, dg_layout(3, 4)) && ta_slabs_fit(4, dg_layout(4, 4)) &&
                  ta_slabs_fit(5, dg_layout(5, 4)) && ta_slabs_fit(6, dg_layout(6, 4)) &&
                  ta_slabs_fit(7, dg_layout(7, 4)) && ta_slabs_fit(8, dg_layout(8, 4)) &&
                  ta_slabs_fit(9, dg_layout(9, 4)),
              "FP32 slab entries overlap");
static_assert(ta_slabs_fit(2, dg_layout(2, 8)) && ta_slabs_fit(3, dg_layout(3, 8)) && ta_slabs_fit(4, dg_layout(4, 8)) &&
                  ta_slabs_fit(5, dg_layout(5, 8)) && ta_slabs_fit(6, dg_layout(6, 8)) &&
                  ta_slabs_fit(7, dg_layout(7, 8)) && ta_slabs_fit(8, dg_layout(8, 8)) &&
                  ta_slabs_fit(9, dg_layout(9, 8)),
              "FP64 slab entries overlap");

// r = B_d u + cl_d lo + cr_d hi
template <int N, typename T>
__device__ __forceinline__ void line_op(const TAArgs<N, T> &A, int d, const T (&u)[N], T lo, T hi, T (&r)[N])
{
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T s = fma(A.cl[d][i], lo, A.cr[d][i] * hi);
#pragma unroll
    for (int m = 0; m < N; ++m) s = fma(A.B[d][i][m], u[m], s);
    r[i] = s;
  }
}

// R right-hand sides per thread (blockIdx.y covers R of them): the cell's
// neighbour and address arithmetic is shared and R times as many loads are in
// flight; each right-hand side has slabs of its own
template <int N, typename T, bool MASS, int EPI, int R>
__global__ void __launch_bounds__(DGCells<N>::value *N *N)
    dg_advect_tensor_kernel(const __grid_constant__ TAArgs<N, T> A)
{
  using Cfg = TACfg<N, T>;
  constexpr int N2 = N * N, N3 = N * N * N;
  constexpr int CPB = Cfg::CPB;
  constexpr TASlab LX = Cfg::X, L1 = Cfg::R1, L2 = Cfg::R2;
  constexpr int RSTRIDE = CPB * Cfg::RS; // slab words of one right-hand side
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *smem = reinterpret_cast<T *>(smem_raw);
  const int tid = threadIdx.x;
  const int cs = tid / N2;
  const int t = tid - cs * N2;
  const int a = t % N, b = t / N;
  const long long cell = (long long)blockIdx.x * CPB + cs;
  const bool valid = cell < A.n_cells;
  T *X = smem + LX.BASE + cs * LX.RS;
  T *R1 = smem + L1.BASE + cs * L1.RS;
  T *R2 = smem + L2.BASE + cs * L2.RS;
  // z column (a, b), x line (y, z) = (a, b), y line (x, z) = (a, b)
  const int zcX = LX.SX * a + LX.SY * b, xlX = LX.SY * a + LX.SZ * b, ylX = LX.SX * a + LX.SZ * b;
  const int zc1 = L1.SX * a + L1.SY * b, xl1 = L1.SY * a + L1.SZ * b;
  const int zc2 = L2.SX * a + L2.SY * b, yl2 = L2.SX * a + L2.SZ * b;
  const long long col = cell * N3 + t;
  const int r0 = (int)blockIdx.y * R;
  bool on[R];
#pragma unroll
  for (int k = 0; k < R; ++k) on[k] = valid && r0 + k < A.nrhs;

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
  // neighbour end values of this thread's z column, x line and y line:
  // (a, b, n-1) / (a, b, 0), (n-1, a, b) / (0, a, b), (a, n-1, b) / (a, 0, b)
  const long long off[3][2] = {{nb[0][0] * N3 + (N - 1) + N * a + N2 * b, nb[0][1] * N3 + N * a + N2 * b},
                               {nb[1][0] * N3 + a + N * (N - 1) + N2 * b, nb[1][1] * N3 + a + N2 * b},
                               {nb[2][0] * N3 + t + N2 * (N - 1), nb[2][1] * N3 + t}};
  const bool use[3][2] = {{(A.nbmask & 1) != 0, (A.nbmask & 2) != 0},
                          {(A.nbmask & 4) != 0, (A.nbmask & 8) != 0},
                          {(A.nbmask & 16) != 0, (A.nbmask & 32) != 0}};

  // ---- every global read up front: the z columns, the neighbour end
  // values and the Runge-Kutta updates of the column ----
  T v[R][N], rz[R][N], nbv[R][3][2];
  T upd[R][EPI == TA_RK ? N : 1];
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const T *__restrict__ x = A.x + (long long)(r0 + k) * A.n_dofs;
#pragma unroll
    for (int m = 0; m < N; ++m) v[k][m] = on[k] ? __ldg(x + col + N2 * m) : T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int sd = 0; sd < 2; ++sd) nbv[k][d][sd] = on[k] && use[d][sd] ? __ldg(x + off[d][sd]) : T(0);
    if (EPI == TA_RK) {
#pragma unroll
      for (int m = 0; m < N; ++m)
        upd[k][m] = on[k] ? A.rk_upd[(long long)(r0 + k) * A.n_dofs + col + N2 * m] : T(0);
    }
  }
  // ---- z columns: copy to X, z line operator in registers ----
#pragma unroll
  for (int k = 0; k < R; ++k) {
#pragma unroll
    for (int m = 0; m < N; ++m) X[k * RSTRIDE + zcX + LX.SZ * m] = v[k][m];
    line_op<N, T>(A, 2, v[k], nbv[k][2][0], nbv[k][2][1], rz[k]);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < R; ++k) {
    T u[N], r[N];
    // ---- x line (y, z) = (a, b): node (m, a, b) at m + N a + N2 b ----
#pragma unroll
    for (int m = 0; m < N; ++m) u[m] = X[k * RSTRIDE + xlX + LX.SX * m];
    line_op<N, T>(A, 0, u, nbv[k][0][0], nbv[k][0][1], r);
#pragma unroll
    for (int m = 0; m < N; ++m) R1[k * RSTRIDE + xl1 + L1.SX * m] = r[m];
    // ---- y line (x, z) = (a, b): node (a, m, b) at a + N m + N2 b ----
#pragma unroll
    for (int m = 0; m < N; ++m) u[m] = X[k * RSTRIDE + ylX + LX.SY * m];
    line_op<N, T>(A, 1, u, nbv[k][1][0], nbv[k][1][1], r);
#pragma unroll
    for (int m = 0; m < N; ++m) R2[k * RSTRIDE + yl2 + L2.SY * m] = r[m];
  }
  __syncthreads();
  // ---- column sums of the three directions ----
#pragma unroll
  for (int k = 0; k < R; ++k)
#pragma unroll
    for (int m = 0; m < N; ++m)
      v[k][m] = rz[k][m] + R1[k * RSTRIDE + zc1 + L1.SZ * m] + R2[k * RSTRIDE + zc2 + L2.SZ * m];
  if (MASS) {
    // M = M1 (x) M1 (x) M1: z in registers, then x and y lines in X (its
    // line reads ended at the barrier above)
#pragma unroll
    for (int k = 0; k < R; ++k) {
      eo_apply<N, 1>(A.M, v[k], v[k]);
#pragma unroll
      for (int m = 0; m < N; ++m) X[k * RSTRIDE + zcX + LX.SZ * m] = v[k][m];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < R; ++k) {
      T u[N];
#pragma unroll
      for (int m = 0; m < N; ++m) u[m] = X[k * RSTRIDE + xlX + LX.SX * m];
      eo_apply<N, 1>(A.M, u, u);
#pragma unroll
      for (int m = 0; m < N; ++m) X[k * RSTRIDE + xlX + LX.SX * m] = u[m];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < R; ++k) {
      T u[N];
#pragma unroll
      for (int m = 0; m < N; ++m) u[m] = X[k * RSTRIDE + ylX + LX.SY * m];
      eo_apply<N, 1>(A.M, u, u);
#pragma unroll
      for (int m = 0; m < N; ++m) X[k * RSTRIDE + ylX + LX.SY * m] = u[m];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < R; ++k)
#pragma unroll
      for (int m = 0; m < N; ++m) v[k][m] = X[k * RSTRIDE + zcX + LX.SZ * m];
  }
  // ---- store the z columns (plain, fused Chebyshev or Runge-Kutta update) ----
#pragma unroll
  for (int k = 0; k < R; ++k) {
    if (!on[k]) continue;
    const long long o = (long long)(r0 + k) * A.n_dofs + col;
    if (EPI == TA_RK) {
#pragma unroll
      for (int m = 0; m < N; ++m) {
        const long long e = o + N2 * m;
        const T np = upd[k][m] + A.c_np * v[k][m];
        A.rk_np[e] = np;
        if (A.c_tm != T(0)) A.rk_tm[e] = np + A.c_tm * v[k][m];
      }
    } else if (EPI == TA_CHEB) {
      // one right-hand side (the Chebyshev step of a single vector)
#pragma unroll
      for (int m = 0; m < N; ++m) {
        const long long e = col + N2 * m;
        const T res = v[k][m] - A.cb[e];
        const T tn = A.c_tm * A.ct[e] + A.c_np * A.cdinv[e] * res;
        A.ct[e] = tn;
        A.y[e] = __ldg(A.x + e) - tn;
      }
    } else {
#pragma unroll
      for (int m = 0; m < N; ++m) A.y[o + N2 * m] = v[k][m];
    }
  }
}

// The 1D operators in FP64.  Direction d, inverse size ij, cell volume jxw,
// face area jf = jxw ij, velocity a_d; Gauss-point residual per unit
// tangential weight (the line residual of the cell-and-face kernel):
//   forward:   R = D^T diag(c w) + sum_s fv_s (fa_s + fb_s) fv_s^T,
//              neighbour term fv_s (fa_s - fb_s) u_nb
//   transpose: R = diag(c w) D + sum_s fv_s fa_s fv_s^T,
//              neighbour term -fv_s fa_s u_nb
// with c = a_d ij jxw, fa, fb as in make_dg_args.  B = P R S, couplings
// P (neighbour term), P = S^-1 W^-1 / jxw with the inverse mass and
// S^-1 W^-1 otherwise (the mass sweeps then use M1 = S^T W S without jxw).
struct Tensor1D {
  double B[3][kMaxN][kMaxN], cl[3][kMaxN], cr[3][kMaxN], M1[kMaxN][kMaxN];
};

Tensor1D advect_tensor_1d(const sf_op *op, bool transpose, bool invmass)
{
  const Shape1D &s = op->shape;
  const int n = s.n;
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  Tensor1D R{};
  double P[kMaxN][kMaxN];
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q) P[i][q] = s.Sinv[i][q] / s.wq[q] / (invmass ? jxw : 1.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double m = 0.0;
      for (int q = 0; q < n; ++q) m += s.S[q][i] * s.wq[q] * s.S[q][j];
      R.M1[i][j] = m;
    }
  for (int d = 0; d < 3; ++d) {
    const double ij = 1.0 / op->h[d], jf = jxw * ij, ad = op->desc.velocity[d];
    const double c = ad * ij * jxw;
    double fa[2], fb[2];
    for (int side = 0; side < 2; ++side) {
      const double an = side ? ad : -ad;
      fa[side] = -0.5 * (transpose ? an + std::fabs(an) : an) * jf;
      fb[side] = -0.5 * std::fabs(an) * jf;
    }
    // Gauss-point residual matrix Rq[q][k] (acting on Gauss values u_k) and
    // the neighbour vectors nbq[side][q]
    double Rq[kMaxN][kMaxN], nbq[2][kMaxN];
    for (int q = 0; q < n; ++q) {
      for (int k = 0; k < n; ++k)
        Rq[q][k] = transpose ? c * s.wq[q] * s.D[q][k] : s.D[k][q] * c * s.wq[k];
      for (int side = 0; side < 2; ++side) {
        const double f = transpose ? fa[side] : fa[side] + fb[side];
        for (int k = 0; k < n; ++k) Rq[q][k] += s.fv[side][q] * f * s.fv[side][k];
        nbq[side][q] = s.fv[side][q] * (transpose ? -fa[side] : fa[side] - fb[side]);
      }
    }
    for (int i = 0; i < n; ++i) {
      for (int m = 0; m < n; ++m) {
        double acc = 0.0;
        for (int q = 0; q < n; ++q) {
          double rs = 0.0;
          for (int k = 0; k < n; ++k) rs += Rq[q][k] * s.S[k][m];
          acc += P[i][q] * rs;
        }
        R.B[d][i][m] = acc;
      }
      double al = 0.0, ar = 0.0;
      for (int q = 0; q < n; ++q) {
        al += P[i][q] * nbq[0][q];
        ar += P[i][q] * nbq[1][q];
      }
      R.cl[d][i] = al;
      R.cr[d][i] = ar;
    }
  }
  return R;
}

template <int N, typename T>
int advect_tensor_impl(const sf_op *op, int nrhs, bool transpose, const T *x, T *y, const T *cb,
                       const T *cdinv, T *ct, double c_np, double c_tm, const T *rk_upd, T *rk_np, T *rk_tm,
                       cudaStream_t st)
{
  using Cfg = TACfg<N, T>;
  const bool invmass = !transpose && op->desc.inverse_mass;
  const Tensor1D R = advect_tensor_1d(op, transpose, invmass);
  TAArgs<N, T> A{};
  A.nbmask = 0;
  for (int d = 0; d < 3; ++d) {
    bool lnz = false, rnz = false;
    for (int i = 0; i < N; ++i) {
      for (int m = 0; m < N; ++m) A.B[d][i][m] = T(R.B[d][i][m]);
      A.cl[d][i] = T(R.cl[d][i]);
      A.cr[d][i] = T(R.cr[d][i]);
      lnz |= R.cl[d][i] != 0.0;
      rnz |= R.cr[d][i] != 0.0;
    }
    A.nbmask |= (lnz ? 1 : 0) << (2 * d);
    A.nbmask |= (rnz ? 2 : 0) << (2 * d);
    A.nc[d] = op->desc.n_cells[d];
  }
  A.M = make_eo<N, T>([&](int i, int j) { return R.M1[i][j]; });
  A.x = x;
  A.y = y;
  A.cb = cb;
  A.cdinv = cdinv;
  A.ct = ct;
  A.c_np = T(c_np);
  A.c_tm = T(c_tm);
  A.rk_upd = rk_upd;
  A.rk_np = rk_np;
  A.rk_tm = rk_tm;
  A.div_nx = make_fast_div((unsigned)A.nc[0]);
  A.div_ny = make_fast_div((unsigned)A.nc[1]);
  A.n_cells = op->n_cells;
  A.n_dofs = op->n_dofs;
  A.nrhs = nrhs;
  const bool rk = rk_np != nullptr, cheb = cb != nullptr;
  // two right-hand sides per thread for batched FP32 applies (p = 4, 48^3,
  // 8 right-hand sides: 258 against 301 us); not for the Runge-Kutta stage,
  // whose prefetched updates make the pairs cost residency (1949 against
  // 1737 us per LSRK step), nor in FP64, bound by the FP64 pipe
  const int rps = (nrhs > 1 && sizeof(T) == 4 && !rk) ? 2 : 1;
  void (*kern)(const TAArgs<N, T>);
  if (rps == 2)
    kern = invmass ? dg_advect_tensor_kernel<N, T, false, TA_STORE, 2> : dg_advect_tensor_kernel<N, T, true, TA_STORE, 2>;
  else if (invmass)
    kern = rk ? dg_advect_tensor_kernel<N, T, false, TA_RK, 1>
         : cheb ? dg_advect_tensor_kernel<N, T, false, TA_CHEB, 1> : dg_advect_tensor_kernel<N, T, false, TA_STORE, 1>;
  else
    kern = rk ? dg_advect_tensor_kernel<N, T, true, TA_RK, 1>
         : cheb ? dg_advect_tensor_kernel<N, T, true, TA_CHEB, 1> : dg_advect_tensor_kernel<N, T, true, TA_STORE, 1>;
  const size_t smem = Cfg::SMEM * rps;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  const long long blocks = (op->n_cells + Cfg::CPB - 1) / Cfg::CPB;
  kern<<<dim3((unsigned)blocks, (unsigned)((nrhs + rps - 1) / rps)), dim3(Cfg::CPB * N * N), smem, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N>
int advect_tensor_n(const sf_op *op, int prec, int nrhs, bool tr, const void *x, void *y, const void *cb,
                    const void *cd, void *ct, double c_np, double c_tm, const void *upd, void *vnp, void *vtm,
                    cudaStream_t st)
{
  if (prec == SF_FP64)
    return advect_tensor_impl<N, double>(op, nrhs, tr, (const double *)x, (double *)y, (const double *)cb,
                                         (const double *)cd, (double *)ct, c_np, c_tm, (const double *)upd,
                                         (double *)vnp, (double *)vtm, st);
  return advect_tensor_impl<N, float>(op, nrhs, tr, (const float *)x, (float *)y, (const float *)cb,
                                      (const float *)cd, (float *)ct, c_np, c_tm, (const float *)upd,
                                      (float *)vnp, (float *)vtm, st);
}

} // namespace

int launch_dg_advect_tensor(const sf_op *op, int prec, int nrhs, bool transpose, const void *x, void *y,
                            const void *cheb_b, const void *cheb_dinv, void *cheb_t, double c_np, double c_tm,
                            const void *rk_upd, void *rk_np, void *rk_tm, cudaStream_t st)
{
  if (op->desc.kind != SF_OP_DG_ADVECT) return SF_ERR_STATE;
  switch (op->desc.degree) {
  case 1: return advect_tensor_n<2>(op, prec, nrhs, transpose, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np, rk_tm, st);
  case 2: return advect_tensor_n<3>(op, prec, nrhs, transpose, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np, rk_tm, st);
  case 3: return advect_tensor_n<4>(op, prec, nrhs, transpose, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np, rk_tm, st);
  case 4: return advect_tensor_n<5>(op, prec, nrhs, transpose, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np, rk_tm, st);
  case 5: return advect_tensor_n<6>(op, prec, nrhs, transpose, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np, rk_tm, st);
  case 6: return advect_tensor_n<7>(op, prec, nrhs, transpose, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np, rk_tm, st);
  case 7: return advect_tensor_n<8>(op, prec, nrhs, transpose, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np, rk_tm, st);
  case 8: return advect_tensor_n<9>(op, prec, nrhs, transpose, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np, rk_tm, st);
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;
  }
}

} // namespace sf
