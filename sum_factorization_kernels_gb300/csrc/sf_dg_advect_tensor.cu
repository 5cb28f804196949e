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
// The same kernel evaluates the DO_FACES cell operators of
// evaluation_cell_laplacian.h:505-797 (each Cartesian cell's own faces at 0
// and 1 as the two sides of one face): convection as sum_f L_f (x) M1 (x) M1
// with B_f = M1^-1 L_f and no neighbour coupling, the Laplacian the same way
// plus a rank-one face term per direction (faces_laplace_1d below), and the
// transpose with the inverse mass, A^T M^-1, with couplings through whole
// neighbour lines (advect_transpose_invmass_1d).
//
// GPU mapping as in the tensor-form SIPG kernel: a block holds CPB
// consecutive cells with n^2 threads each; the thread of z column (a, b)
// reads and writes that column of the cell-major vector (runs of n^2
// consecutive entries per warp instruction) and owns x line (y, z) = (a, b)
// and y line (x, z) = (a, b) of the shared-memory copy.  The x and y line
// results go to two slabs of their own, so one barrier separates the line
// phase from the column sum.
#include <cmath>
#include <utility>

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
  // DO_FACES Laplacian: sum_f F2_f (x) Tp (x) Tp with F2_f = f2c[f] (e_p + e_0)^T
  EOMat<N, T> Tp;
  T f2c[3][N];
  // neighbour-line couplings (transpose with the inverse mass): the value of
  // side s is sum_m wnb[s][m] u_m over the neighbour's whole line
  T wnb[2][N];
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
// results), each in a region of its own: entry (x, y, z) of cell cs at
// BASE + cs RS + SX x + SY y + SZ z.  FP32: strides from the bank-conflict
// model of the kernel's accesses over the lanes of each warp (X: z column
// stores, x and y line loads; R1: x line stores, z column loads; R2: y line
// stores, z column loads; p = 4: 190 weighted wavefronts per cell group
// against 220 for the padded layout); FP64: the padded layout of dg_layout.
struct TASlab {
  int SX, SY, SZ, RS, BASE;
};
struct TASlabs {
  TASlab X, R1, R2;
};

constexpr TASlabs ta_slabs3(TASlab x, TASlab r1, TASlab r2, int cpb)
{
  return TASlabs{{x.SX, x.SY, x.SZ, x.RS, 0}, {r1.SX, r1.SY, r1.SZ, r1.RS, cpb * x.RS},
                 {r2.SX, r2.SY, r2.SZ, r2.RS, cpb * (x.RS + r1.RS)}};
}

constexpr TASlabs ta_slabs(int n, int elem, int cpb)
{
  if (elem == 4) {
    switch (n) {
    case 2: return ta_slabs3({5, 1, 2, 12, 0}, {5, 2, 1, 12, 0}, {2, 5, 1, 12, 0}, cpb);
    case 3: return ta_slabs3({3, 1, 9, 27, 0}, {3, 9, 1, 27, 0}, {11, 33, 1, 99, 0}, cpb);
    case 4: return ta_slabs3({19, 4, 1, 80, 0}, {17, 4, 1, 80, 0}, {4, 1, 17, 80, 0}, cpb);
    case 5: return ta_slabs3({26, 1, 5, 153, 0}, {26, 1, 5, 153, 0}, {1, 5, 37, 185, 0}, cpb);
    case 6: return ta_slabs3({37, 1, 6, 228, 0}, {37, 1, 6, 228, 0}, {1, 6, 38, 228, 0}, cpb);
    case 7: return ta_slabs3({1, 52, 7, 369, 0}, {1, 7, 49, 343, 0}, {7, 49, 1, 343, 0}, cpb);
    case 8: return ta_slabs3({67, 1, 8, 533, 0}, {68, 1, 8, 540, 0}, {1, 72, 8, 568, 0}, cpb);
    case 9: return ta_slabs3({1, 9, 81, 729, 0}, {1, 9, 81, 729, 0}, {1, 9, 105, 945, 0}, cpb);
    default: break;
    }
  }
  const DGLayout L = dg_layout(n, elem);
  const int slab = L.P2 * n, rs = 3 * slab + L.SKEW;
  return TASlabs{{1, L.P1, L.P2, rs, 0}, {1, L.P1, L.P2, rs, slab}, {1, L.P1, L.P2, rs, 2 * slab}};
}

constexpr int ta_slab_end(int n, int cpb, TASlab S)
{
  return S.BASE + (cpb - 1) * S.RS + (n - 1) * (S.SX + S.SY + S.SZ) + 1;
}

template <int N, typename T>
struct TACfg {
  static constexpr int CPB = DGCells<N>::value;
  static constexpr TASlabs S = ta_slabs(N, (int)sizeof(T), CPB);
  static constexpr TASlab X = S.X, R1 = S.R1, R2 = S.R2;
  static constexpr int E0 = ta_slab_end(N, CPB, X), E1 = ta_slab_end(N, CPB, R1), E2 = ta_slab_end(N, CPB, R2);
  static constexpr int WORDS = E0 > E1 ? (E0 > E2 ? E0 : E2) : (E1 > E2 ? E1 : E2); // slabs of one right-hand side
  static constexpr size_t SMEM = size_t(WORDS) * sizeof(T);                        // per right-hand side
  // DO_FACES Laplacian: three n x n face arrays per cell after the slabs
  static constexpr int FW = 3 * N * N;
  static constexpr size_t SMEM_F2 = (size_t(WORDS) + size_t(CPB) * FW) * sizeof(T);
};

// every entry of the three slabs of every cell of a block has its own word
constexpr bool ta_slabs_fit(int n, int cpb, TASlabs S)
{
  bool seen[16384] = {};
  const TASlab L[3] = {S.X, S.R1, S.R2};
  for (int s = 0; s < 3; ++s)
    for (int c = 0; c < cpb; ++c)
      for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
          for (int x = 0; x < n; ++x) {
            const int i = L[s].BASE + c * L[s].RS + L[s].SX * x + L[s].SY * y + L[s].SZ * z;
            if (i < 0 || i >= 16384 || seen[i]) return false;
            seen[i] = true;
          }
  return true;
}
static_assert(ta_slabs_fit(2, DGCells<2>::value, ta_slabs(2, 4, DGCells<2>::value)) &&
                  ta_slabs_fit(3, DGCells<3>::value, ta_slabs(3, 4, DGCells<3>::value)) &&
                  ta_slabs_fit(4, DGCells<4>::value, ta_slabs(4, 4, DGCells<4>::value)) &&
                  ta_slabs_fit(5, DGCells<5>::value, ta_slabs(5, 4, DGCells<5>::value)) &&
                  ta_slabs_fit(6, DGCells<6>::value, ta_slabs(6, 4, DGCells<6>::value)) &&
                  ta_slabs_fit(7, DGCells<7>::value, ta_slabs(7, 4, DGCells<7>::value)) &&
                  ta_slabs_fit(8, DGCells<8>::value, ta_slabs(8, 4, DGCells<8>::value)) &&
                  ta_slabs_fit(9, DGCells<9>::value, ta_slabs(9, 4, DGCells<9>::value)),
              "FP32 slab entries overlap");
static_assert(ta_slabs_fit(2, DGCells<2>::value, ta_slabs(2, 8, DGCells<2>::value)) &&
                  ta_slabs_fit(3, DGCells<3>::value, ta_slabs(3, 8, DGCells<3>::value)) &&
                  ta_slabs_fit(4, DGCells<4>::value, ta_slabs(4, 8, DGCells<4>::value)) &&
                  ta_slabs_fit(5, DGCells<5>::value, ta_slabs(5, 8, DGCells<5>::value)) &&
                  ta_slabs_fit(6, DGCells<6>::value, ta_slabs(6, 8, DGCells<6>::value)) &&
                  ta_slabs_fit(7, DGCells<7>::value, ta_slabs(7, 8, DGCells<7>::value)) &&
                  ta_slabs_fit(8, DGCells<8>::value, ta_slabs(8, 8, DGCells<8>::value)) &&
                  ta_slabs_fit(9, DGCells<9>::value, ta_slabs(9, 8, DGCells<9>::value)),
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
template <int N, typename T, bool MASS, int EPI, int R, bool F2 = false, bool NBL = false>
__global__ void __launch_bounds__(DGCells<N>::value *N *N)
    dg_advect_tensor_kernel(const __grid_constant__ TAArgs<N, T> A)
{
  static_assert(!F2 || (MASS && EPI == TA_STORE), "face term: mass form, plain store");
  static_assert(!NBL || (!MASS && EPI == TA_STORE), "neighbour lines: line form, plain store");
  using Cfg = TACfg<N, T>;
  constexpr int N2 = N * N, N3 = N * N * N;
  constexpr int CPB = Cfg::CPB;
  constexpr TASlab LX = Cfg::X, L1 = Cfg::R1, L2 = Cfg::R2;
  // slab (and face array) words of one right-hand side
  constexpr int RSTRIDE = Cfg::WORDS + (F2 ? CPB * Cfg::FW : 0);
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
  // face arrays of the F2 term: Fx over (y, z), Fy over (x, z), Fz over (x, y),
  // entry (i, j) at i + N j
  T *Fx = smem + Cfg::WORDS + cs * Cfg::FW, *Fy = Fx + N * N, *Fz = Fy + N * N;
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
  // (NBL: the start of the neighbour's line through the same face point,
  // node stride 1, N, N^2 for x, y, z)
  const long long off[3][2] =
      {{nb[0][0] * N3 + (NBL ? 0 : N - 1) + N * a + N2 * b, nb[0][1] * N3 + N * a + N2 * b},
       {nb[1][0] * N3 + a + (NBL ? 0 : N * (N - 1)) + N2 * b, nb[1][1] * N3 + a + N2 * b},
       {nb[2][0] * N3 + t + (NBL ? 0 : N2 * (N - 1)), nb[2][1] * N3 + t}};
  constexpr int lstride[3] = {1, N, N2};
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
      for (int sd = 0; sd < 2; ++sd) {
        if (NBL) {
          T acc = T(0);
          if (on[k] && use[d][sd]) {
#pragma unroll
            for (int m = 0; m < N; ++m) acc = fma(A.wnb[sd][m], __ldg(x + off[d][sd] + lstride[d] * m), acc);
          }
          nbv[k][d][sd] = acc;
        } else {
          nbv[k][d][sd] = on[k] && use[d][sd] ? __ldg(x + off[d][sd]) : T(0);
        }
      }
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
    if (F2) Fz[k * RSTRIDE + a + N * b] = v[k][0] + v[k][N - 1];
    line_op<N, T>(A, 2, v[k], nbv[k][2][0], nbv[k][2][1], rz[k]);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < R; ++k) {
    T u[N], r[N];
    // ---- x line (y, z) = (a, b): node (m, a, b) at m + N a + N2 b ----
#pragma unroll
    for (int m = 0; m < N; ++m) u[m] = X[k * RSTRIDE + xlX + LX.SX * m];
    if (F2) Fx[k * RSTRIDE + a + N * b] = u[0] + u[N - 1];
    line_op<N, T>(A, 0, u, nbv[k][0][0], nbv[k][0][1], r);
#pragma unroll
    for (int m = 0; m < N; ++m) R1[k * RSTRIDE + xl1 + L1.SX * m] = r[m];
    // ---- y line (x, z) = (a, b): node (a, m, b) at a + N m + N2 b ----
#pragma unroll
    for (int m = 0; m < N; ++m) u[m] = X[k * RSTRIDE + ylX + LX.SY * m];
    if (F2) Fy[k * RSTRIDE + a + N * b] = u[0] + u[N - 1];
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
    // line reads ended at the barrier above); with F2 the face arrays get
    // Tp along their first and second coordinate in the same phases (3 n
    // face lines per cell over its n^2 threads)
#pragma unroll
    for (int k = 0; k < R; ++k) {
      eo_apply<N, 1>(A.M, v[k], v[k]);
#pragma unroll
      for (int m = 0; m < N; ++m) X[k * RSTRIDE + zcX + LX.SZ * m] = v[k][m];
    }
    for (int task = t; F2 && task < 3 * N; task += N * N) {
      const int arr = task / N, j = task - arr * N;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        T u[N];
        T *Fa = Fx + k * RSTRIDE + arr * N * N + N * j;
#pragma unroll
        for (int i = 0; i < N; ++i) u[i] = Fa[i];
        eo_apply<N, 1>(A.Tp, u, u);
#pragma unroll
        for (int i = 0; i < N; ++i) Fa[i] = u[i];
      }
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
    for (int task = t; F2 && task < 3 * N; task += N * N) {
      const int arr = task / N, i = task - arr * N;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        T u[N];
        T *Fa = Fx + k * RSTRIDE + arr * N * N + i;
#pragma unroll
        for (int j = 0; j < N; ++j) u[j] = Fa[N * j];
        eo_apply<N, 1>(A.Tp, u, u);
#pragma unroll
        for (int j = 0; j < N; ++j) Fa[N * j] = u[j];
      }
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
    if (F2) {
      // node (a, b, m): the z face term at layer m, the x face term at layer
      // a (face point (y, z) = (b, m)), the y face term at layer b ((x, z) = (a, m))
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const T tz = Fz[k * RSTRIDE + a + N * b];
        const T cx = A.f2c[0][a], cy = A.f2c[1][b];
#pragma unroll
        for (int m = 0; m < N; ++m) {
          T acc = fma(A.f2c[2][m], tz, v[k][m]);
          acc = fma(cx, Fx[k * RSTRIDE + b + N * m], acc);
          v[k][m] = fma(cy, Fy[k * RSTRIDE + a + N * m], acc);
        }
      }
    }
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
  bool f2;                                    // DO_FACES Laplacian face term
  double Tp[kMaxN][kMaxN], f2c[3][kMaxN];
  bool nbline;                                // couplings through whole neighbour lines
  double wnb[2][kMaxN];
};

// M1 = S^T W S
void mass_1d(const Shape1D &s, double (&M1)[kMaxN][kMaxN])
{
  for (int i = 0; i < s.n; ++i)
    for (int j = 0; j < s.n; ++j) {
      double m = 0.0;
      for (int q = 0; q < s.n; ++q) m += s.S[q][i] * s.wq[q] * s.S[q][j];
      M1[i][j] = m;
    }
}

// B = M1^-1 L by Gaussian elimination with partial pivoting (L is overwritten)
void solve_mass(int n, const double (&M1)[kMaxN][kMaxN], double (&L)[kMaxN][kMaxN], double (&B)[kMaxN][kMaxN])
{
  double Mw[kMaxN][kMaxN];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Mw[i][j] = M1[i][j];
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(Mw[r][c]) > std::fabs(Mw[piv][c])) piv = r;
    for (int j = 0; j < n; ++j) {
      std::swap(Mw[c][j], Mw[piv][j]);
      std::swap(L[c][j], L[piv][j]);
    }
    for (int r = c + 1; r < n; ++r) {
      const double fct = Mw[r][c] / Mw[c][c];
      for (int j = 0; j < n; ++j) {
        Mw[r][j] -= fct * Mw[c][j];
        L[r][j] -= fct * L[c][j];
      }
    }
  }
  for (int c = n - 1; c >= 0; --c)
    for (int j = 0; j < n; ++j) {
      double v = L[c][j];
      for (int k = c + 1; k < n; ++k) v -= Mw[c][k] * B[k][j];
      B[c][j] = v / Mw[c][c];
    }
}

Tensor1D advect_tensor_1d(const sf_op *op, bool transpose, bool invmass)
{
  const Shape1D &s = op->shape;
  const int n = s.n;
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  Tensor1D R{};
  double P[kMaxN][kMaxN];
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q) P[i][q] = s.Sinv[i][q] / s.wq[q] / (invmass ? jxw : 1.0);
  mass_1d(s, R.M1);
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

// The DO_FACES convection operator (cell-major, Hermite-like basis, each
// cell's own faces at 0 and 1 as the two sides of one face,
// evaluation_cell_laplacian.h:505-797) on Cartesian cells is
// sum_f L_f (x) M1 (x) M1 with M1 = S^T W S and
//   L_f = b_f ij_f jxw S^T D^T W S - jf (e_p - e_0) flux^T,
//   flux = (b_f (e_p + e_0) + |b_f| (e_p - e_0)) / 2,
// jf = jxw ij_f the face area (the value of the Hermite-like basis at a face
// is its end coefficient).  Evaluated in the mass form with B_f = M1^-1 L_f
// and no neighbour couplings.
Tensor1D faces_convection_1d(const sf_op *op)
{
  const Shape1D &s = op->shape;
  const int n = s.n, p = n - 1;
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  Tensor1D R{};
  mass_1d(s, R.M1);
  for (int f = 0; f < 3; ++f) {
    const double ij = 1.0 / op->h[f], jf = jxw * ij, bf = op->desc.velocity[f];
    // L_f = b_f ij jxw S^T D^T W S, (D^T W S)[q][j] = sum_k D[k][q] w_k S[k][j]
    double L[kMaxN][kMaxN];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double acc = 0.0;
        for (int q = 0; q < n; ++q) {
          double ds = 0.0;
          for (int k = 0; k < n; ++k) ds += s.D[k][q] * s.wq[k] * s.S[k][j];
          acc += s.S[q][i] * ds;
        }
        L[i][j] = bf * ij * jxw * acc;
      }
    double flux[kMaxN] = {};
    flux[p] += 0.5 * (bf + std::fabs(bf));
    flux[0] += 0.5 * (bf - std::fabs(bf));
    for (int j = 0; j < n; ++j) {
      L[p][j] -= jf * flux[j];
      L[0][j] += jf * flux[j];
    }
    solve_mass(n, R.M1, L, R.B[f]);
  }
  return R;
}

// The DO_FACES Laplacian (same source) on Cartesian cells is
//   sum_f (K_f + F1_f) (x) M1 (x) M1 + sum_f F2_f (x) Tp (x) Tp,
// K_f = jxw ij_f^2 (D S)^T W (D S), Tp = S W S (the reference interpolates
// the derivative-test term of the face with S, not S^T), and with e_i the
// unit vectors, sigma = n^2 ij_f, hd = phi_0'(0), jf = jxw ij_f:
//   F1_f = jf (e_p - e_0) (sigma (e_p + e_0) - ij_f hd (e_{p-1} - e_p + e_1 - e_0) / 2)^T
//   F2_f = -jf ij_f hd (-e_p + e_{p-1} - e_0 + e_1) (e_p + e_0)^T / 2.
// The first sum runs in the mass form with B_f = M1^-1 (K_f + F1_f); the
// second is rank one per direction: the sum of the two end layers, Tp along
// both face directions, injected into layers 0, 1, p-1, p.
Tensor1D faces_laplace_1d(const sf_op *op)
{
  const Shape1D &s = op->shape;
  const int n = s.n, p = n - 1;
  const double jxw = op->h[0] * op->h[1] * op->h[2], hd = s.hermite_d0;
  Tensor1D R{};
  R.f2 = true;
  mass_1d(s, R.M1);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double m = 0.0;
      for (int q = 0; q < n; ++q) m += s.S[i][q] * s.wq[q] * s.S[q][j];
      R.Tp[i][j] = m;
    }
  double DS[kMaxN][kMaxN];
  for (int q = 0; q < n; ++q)
    for (int j = 0; j < n; ++j) {
      double v = 0.0;
      for (int k = 0; k < n; ++k) v += s.D[q][k] * s.S[k][j];
      DS[q][j] = v;
    }
  for (int f = 0; f < 3; ++f) {
    const double ij = 1.0 / op->h[f], jf = jxw * ij, sigma = double(n * n) * ij;
    double L[kMaxN][kMaxN];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double acc = 0.0;
        for (int q = 0; q < n; ++q) acc += DS[q][i] * s.wq[q] * DS[q][j];
        L[i][j] = jxw * ij * ij * acc;
      }
    double rowv[kMaxN] = {}, g[kMaxN] = {};
    rowv[p] += sigma;
    rowv[0] += sigma;
    rowv[p - 1] -= 0.5 * ij * hd;
    rowv[p] += 0.5 * ij * hd;
    rowv[1] -= 0.5 * ij * hd;
    rowv[0] += 0.5 * ij * hd;
    for (int j = 0; j < n; ++j) {
      L[p][j] += jf * rowv[j];
      L[0][j] -= jf * rowv[j];
    }
    solve_mass(n, R.M1, L, R.B[f]);
    g[p] -= 1.0;
    g[p - 1] += 1.0;
    g[0] -= 1.0;
    g[1] += 1.0;
    for (int i = 0; i < n; ++i) R.f2c[f][i] = -0.5 * jf * ij * hd * g[i];
  }
  return R;
}

// The transpose with the inverse mass, A^T M^-1.  With A^T = M1^{x3}
// (sum_d B'_d (x) I (x) I + couplings) from advect_tensor_1d(transpose, no
// inverse mass) and M^-1 = (M1^-1)^{x3} / jxw, the tangential M1 and M1^-1
// cancel:
//   A^T M^-1 = sum_d C_d (x) I (x) I / jxw,  C_d = M1 B'_d M1^-1,
// and the coupling of side s becomes (M1 c_s) times the dot product of row
// n-1 (left neighbour) or row 0 (right neighbour) of M1^-1 with the
// neighbour's whole line: one launch instead of an inverse-mass pass and the
// transposed apply.
Tensor1D advect_transpose_invmass_1d(const sf_op *op)
{
  const int n = op->shape.n;
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  const Tensor1D T0 = advect_tensor_1d(op, true, false);
  Tensor1D R{};
  R.nbline = true;
  double Minv[kMaxN][kMaxN], I[kMaxN][kMaxN] = {};
  for (int i = 0; i < n; ++i) I[i][i] = 1.0;
  solve_mass(n, T0.M1, I, Minv);
  for (int m = 0; m < n; ++m) {
    R.wnb[0][m] = Minv[n - 1][m];
    R.wnb[1][m] = Minv[0][m];
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) R.M1[i][j] = T0.M1[i][j];
  for (int d = 0; d < 3; ++d) {
    double MB[kMaxN][kMaxN];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double v = 0.0;
        for (int k = 0; k < n; ++k) v += T0.M1[i][k] * T0.B[d][k][j];
        MB[i][j] = v;
      }
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) {
        double v = 0.0;
        for (int k = 0; k < n; ++k) v += MB[i][k] * Minv[k][j];
        R.B[d][i][j] = v / jxw;
      }
      double l = 0.0, r = 0.0;
      for (int k = 0; k < n; ++k) {
        l += T0.M1[i][k] * T0.cl[d][k];
        r += T0.M1[i][k] * T0.cr[d][k];
      }
      R.cl[d][i] = l / jxw;
      R.cr[d][i] = r / jxw;
    }
  }
  return R;
}

template <int N, typename T>
int line_sum_impl(const sf_op *op, const Tensor1D &R, bool invmass, int nrhs, const T *x, T *y, const T *cb,
                  const T *cdinv, T *ct, double c_np, double c_tm, const T *rk_upd, T *rk_np, T *rk_tm,
                  cudaStream_t st)
{
  using Cfg = TACfg<N, T>;
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
  A.Tp = make_eo<N, T>([&](int i, int j) { return R.Tp[i][j]; });
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < N; ++i) A.f2c[d][i] = T(R.f2c[d][i]);
  for (int sd = 0; sd < 2; ++sd)
    for (int i = 0; i < N; ++i) A.wnb[sd][i] = T(R.wnb[sd][i]);
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
  if (R.f2)
    kern = rps == 2 ? dg_advect_tensor_kernel<N, T, true, TA_STORE, 2, true>
                    : dg_advect_tensor_kernel<N, T, true, TA_STORE, 1, true>;
  else if (R.nbline)
    kern = rps == 2 ? dg_advect_tensor_kernel<N, T, false, TA_STORE, 2, false, true>
                    : dg_advect_tensor_kernel<N, T, false, TA_STORE, 1, false, true>;
  else if (rps == 2)
    kern = invmass ? dg_advect_tensor_kernel<N, T, false, TA_STORE, 2> : dg_advect_tensor_kernel<N, T, true, TA_STORE, 2>;
  else if (invmass)
    kern = rk ? dg_advect_tensor_kernel<N, T, false, TA_RK, 1>
         : cheb ? dg_advect_tensor_kernel<N, T, false, TA_CHEB, 1> : dg_advect_tensor_kernel<N, T, false, TA_STORE, 1>;
  else
    kern = rk ? dg_advect_tensor_kernel<N, T, true, TA_RK, 1>
         : cheb ? dg_advect_tensor_kernel<N, T, true, TA_CHEB, 1> : dg_advect_tensor_kernel<N, T, true, TA_STORE, 1>;
  const size_t smem = (R.f2 ? Cfg::SMEM_F2 : Cfg::SMEM) * rps;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  const long long blocks = (op->n_cells + Cfg::CPB - 1) / Cfg::CPB;
  kern<<<dim3((unsigned)blocks, (unsigned)((nrhs + rps - 1) / rps)), dim3(Cfg::CPB * N * N), smem, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N>
int line_sum_n(const sf_op *op, const Tensor1D &R, bool invmass, int prec, int nrhs, const void *x, void *y,
               const void *cb, const void *cd, void *ct, double c_np, double c_tm, const void *upd, void *vnp,
               void *vtm, cudaStream_t st)
{
  if (prec == SF_FP64)
    return line_sum_impl<N, double>(op, R, invmass, nrhs, (const double *)x, (double *)y, (const double *)cb,
                                    (const double *)cd, (double *)ct, c_np, c_tm, (const double *)upd,
                                    (double *)vnp, (double *)vtm, st);
  return line_sum_impl<N, float>(op, R, invmass, nrhs, (const float *)x, (float *)y, (const float *)cb,
                                 (const float *)cd, (float *)ct, c_np, c_tm, (const float *)upd, (float *)vnp,
                                 (float *)vtm, st);
}

int line_sum_dispatch(const sf_op *op, const Tensor1D &R, bool invmass, int prec, int nrhs, const void *x,
                      void *y, const void *cb, const void *cd, void *ct, double c_np, double c_tm, const void *upd,
                      void *vnp, void *vtm, cudaStream_t st)
{
  switch (op->desc.degree) {
  case 1: return line_sum_n<2>(op, R, invmass, prec, nrhs, x, y, cb, cd, ct, c_np, c_tm, upd, vnp, vtm, st);
  case 2: return line_sum_n<3>(op, R, invmass, prec, nrhs, x, y, cb, cd, ct, c_np, c_tm, upd, vnp, vtm, st);
  case 3: return line_sum_n<4>(op, R, invmass, prec, nrhs, x, y, cb, cd, ct, c_np, c_tm, upd, vnp, vtm, st);
  case 4: return line_sum_n<5>(op, R, invmass, prec, nrhs, x, y, cb, cd, ct, c_np, c_tm, upd, vnp, vtm, st);
  case 5: return line_sum_n<6>(op, R, invmass, prec, nrhs, x, y, cb, cd, ct, c_np, c_tm, upd, vnp, vtm, st);
  case 6: return line_sum_n<7>(op, R, invmass, prec, nrhs, x, y, cb, cd, ct, c_np, c_tm, upd, vnp, vtm, st);
  case 7: return line_sum_n<8>(op, R, invmass, prec, nrhs, x, y, cb, cd, ct, c_np, c_tm, upd, vnp, vtm, st);
  case 8: return line_sum_n<9>(op, R, invmass, prec, nrhs, x, y, cb, cd, ct, c_np, c_tm, upd, vnp, vtm, st);
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;
  }
}

} // namespace

int launch_dg_advect_tensor(const sf_op *op, int prec, int nrhs, bool transpose, const void *x, void *y,
                            const void *cheb_b, const void *cheb_dinv, void *cheb_t, double c_np, double c_tm,
                            const void *rk_upd, void *rk_np, void *rk_tm, cudaStream_t st)
{
  if (op->desc.kind != SF_OP_DG_ADVECT) return SF_ERR_STATE;
  if (transpose && op->desc.inverse_mass) {
    // A^T M^-1 in one launch (no Chebyshev or Runge-Kutta epilogue here)
    if (cheb_b || rk_np) return SF_ERR_STATE;
    const Tensor1D R = advect_transpose_invmass_1d(op);
    return line_sum_dispatch(op, R, true, prec, nrhs, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, nullptr, nullptr,
                             nullptr, st);
  }
  const bool invmass = !transpose && op->desc.inverse_mass;
  const Tensor1D R = advect_tensor_1d(op, transpose, invmass);
  return line_sum_dispatch(op, R, invmass, prec, nrhs, x, y, cheb_b, cheb_dinv, cheb_t, c_np, c_tm, rk_upd, rk_np,
                           rk_tm, st);
}

int launch_faces_tensor(const sf_op *op, int prec, int nrhs, const void *x, void *y, cudaStream_t st)
{
  if (op->desc.kind != SF_OP_CONVECTION_FACES && op->desc.kind != SF_OP_LAPLACE_FACES) return SF_ERR_STATE;
  const Tensor1D R = op->desc.kind == SF_OP_LAPLACE_FACES ? faces_laplace_1d(op) : faces_convection_1d(op);
  return line_sum_dispatch(op, R, false, prec, nrhs, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, nullptr, nullptr,
                           nullptr, st);
}

} // namespace sf
