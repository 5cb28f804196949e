// sf_cont_kron.cu -- continuous operators on affine Cartesian meshes with
// constant coefficients as Kronecker products of assembled 1D matrices.
//
// On a structured mesh of congruent box cells the global node numbering is a
// tensor product of 1D numberings (node X = i p + a along x, likewise y, z),
// and every cell matrix of the Laplacian, mass and convection forms of
// evaluation_cell_laplacian.h:216-503 (DO_MASS_MATRIX / DO_CONVECTION
// variants :299-354) is a tensor product of (p+1)x(p+1) matrices.  Assembly
// therefore factorises:
//   mass        jxw M1 (x) M1 (x) M1               -> M_z (x) M_y (x) M_x
//   Laplacian   sum_d jxw/h_d^2 K1_d (x) M1 (x) M1 -> K_x M_y M_z + M_x K_y M_z + M_x M_y K_z
//   convection  sum_d b_d/h_d jxw C1_d (x) ...     -> the same with C in place of K
// with the assembled banded 1D matrices M_d = assembly of h_d M1, K_d of
// K1 / h_d (K1 = (D S)^T W (D S)) and C_d of b_d C1 (C1 = S^T D^T W S).
// Homogeneous Dirichlet conditions keep the structure: the projection on the
// interior nodes is P_x (x) P_y (x) P_z, so each 1D matrix loses its boundary
// rows and columns, and the boundary rows of the result are y = x.
//
// Evaluation in two kernels.  The z pass streams along z: a thread owns G
// consecutive cell segments of a z line (a segment is the p nodes from its
// first vertex on; the last segment of a line is the final vertex alone),
// loads the (G+1)p+1 nodes around them once and applies the cell-local 1D
// matrices (a vertex sums the last row of the left cell and the first row of
// the right cell); consecutive threads hold consecutive x, so every access
// is coalesced.  The x-y pass stages a tile of each z-plane with its halo in
// shared memory and runs the x and y sweeps there.  The Laplacian and
// convection forms:
//   z: a = M_z x, b = K_z x;   x-y: y = M_y (K_x a + M_x b) + K_y (M_x a)
// (6 vector transfers); the mass matrix: a = M_z x, y = M_y M_x a (4).
// Each cell-local product runs in the even-odd form of the 1D kernels (the
// cell matrices are centro- or anti-centro-symmetric), in FP64 below n = 7
// as dense rows.  Compared with the cell-by-cell apply there is no
// colouring, no gather and no scatter; the work vectors are allocated with
// the handle.
#include "sf_device.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"

namespace sf {

namespace {

template <int N, typename T>
struct KronArgs {
  // cell-local 1D matrices of this pass: out_o = sum_i A[o][i] in_i, A[o][i]
  // = mat[sel[o][i] - 1] (sel 0: no term)
  T mat[4][N][N];      // z pass: mat[0..1]; x-y tile: M_x, K_x, M_y, K_y
  EOMat<N, T> eo[4];   // the same matrices in even-odd form (M and the Laplacian's
                       // K centro-symmetric, the convection C anti-centro-symmetric)
  const T *in0, *in1;
  T *out0, *out1;
  const T *x;          // last pass: the Dirichlet rows y = x
  int nn[3];           // nodes per direction
  int nc[3];           // cells per direction
  int dirichlet;
  long long tasks;     // z pass: segment chunks x nodes of a plane
  FastDiv div_a;       // z pass: division by the nodes of a plane
};

// row p of a cell matrix times the left cell's nodes (the left cell's share
// of the segment's vertex)
template <int N, typename T, typename U>
__device__ __forceinline__ T last_row(const T (&M)[N][N], const U &u, int off)
{
  T v = T(0);
#pragma unroll
  for (int j = 0; j < N; ++j) v = fma(M[N - 1][j], u[off + j], v);
  return v;
}

// all rows of a cell matrix times the right cell's nodes u[off .. off + p]:
// the even-odd form (symmetry SIGN), or the dense rows for FP64 below n = 7,
// where the even-odd form's additions (on the same FP64 pipe) cost more than
// its saved products (measured: p = 2 Laplacian 162 vs 213 us, p = 4 1.67 vs
// 1.80 ms; p = 8 3.06 vs 3.77 ms the other way)
// (ROWS: the rows the caller uses; the dense form computes only those)
template <int N, int SIGN, typename T, typename U, int ROWS = N>
__device__ __forceinline__ void cell_rows(const EOMat<N, T> &E, const T (&M)[N][N], const U &u, int off,
                                          T (&out)[N])
{
  T in[N];
#pragma unroll
  for (int j = 0; j < N; ++j) in[j] = u[off + j];
  if constexpr (sizeof(T) == 8 && N < 7) {
#pragma unroll
    for (int i = 0; i < N; ++i) out[i] = T(0);
#pragma unroll
    for (int i = 0; i < ROWS; ++i) {
      T v = M[i][0] * in[0];
#pragma unroll
      for (int j = 1; j < N; ++j) v = fma(M[i][j], in[j], v);
      out[i] = v;
    }
  } else {
    eo_apply<N, SIGN>(E, in, out);
  }
}

// segments per thread: a thread walks G consecutive cell segments of its
// line and loads each node once ((G + 1) p + 1 inputs per G p outputs)
template <int N>
struct KronG {
  static constexpr int value = N <= 5 ? 4 : 2;
};

// the z pass: out_o = sum_i A[o][i] in_i along the z lines, SEL[o][i] in
// {0, 1, 2} picking no term / mat[0] / mat[1]
template <int N, typename T, int NIN, int NOUT, int S00, int S01, int S10, int S11, int KS>
__global__ void __launch_bounds__(256) kron_pass(const __grid_constant__ KronArgs<N, T> A)
{
  constexpr int DIR = 2;
  constexpr int P = N - 1;
  // dense rows for FP64 below n = 7 (see cell_rows), even-odd otherwise
  constexpr bool DENSE = sizeof(T) == 8 && N < 7;
  constexpr int G = KronG<N>::value;
  constexpr int W = (G + 1) * P + 1; // window: nodes s0 p - p .. (s0 + G) p
  constexpr int SEL[2][2] = {{S00, S01}, {S10, S11}};
  const long long plane = (long long)A.nn[0] * A.nn[1];
  const long long stride = plane;
  const int nc = A.nc[DIR];
  const int nd = A.nn[DIR];
  for (long long task = blockIdx.x * (long long)blockDim.x + threadIdx.x; task < A.tasks;
       task += (long long)gridDim.x * blockDim.x) {
    // task = (X, Y, chunk): consecutive threads hold consecutive nodes of a
    // plane, so every load and store is coalesced
    const unsigned q = fast_div((unsigned)task, A.div_a); // task / plane
    const int ch = int(q);
    const long long base = task - (long long)q * plane;  // X + nx Y
    const int s0 = ch * G;
    const long long w0 = (long long)s0 * P - P; // window start along DIR
    // the chunk reaches a line end (or a Dirichlet boundary node): checked loads
    const bool edge = s0 < 2 || s0 + G > nc - 1;
    T u[NIN][W];
#pragma unroll
    for (int i = 0; i < NIN; ++i) {
      const T *src = i == 0 ? A.in0 : A.in1;
      if (!edge) {
        // w0 >= p here: the window lies inside the line
        const T *w = src + base + w0 * stride;
#pragma unroll
        for (int k = 0; k < W; ++k) u[i][k] = __ldg(w + k * stride);
      } else {
#pragma unroll
        for (int k = 0; k < W; ++k) {
          const long long pos = w0 + k;
          const bool ok = pos >= 0 && pos < nd && !(A.dirichlet && (pos == 0 || pos == nd - 1));
          u[i][k] = ok ? __ldg(src + (base + pos * stride)) : T(0);
        }
      }
    }
    // segment g's left cell is segment g - 1's right cell: in the even-odd
    // form its last row is carried along the chain (computed directly for
    // the first segment); the dense form (FP64 below n = 7) takes the left
    // cell's last row and the right cell's rows 0 .. p - 1 directly
    T carry[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; ++o) carry[o] = T(0);
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int s = s0 + g;
      if (s > nc) break;
      const bool left = s > 0, right = s < nc;
      // window offsets: left cell g p .. g p + p, right cell g p + p .. g p + 2p
      T r[NOUT][P];
#pragma unroll
      for (int o = 0; o < NOUT; ++o) {
#pragma unroll
        for (int q = 0; q < P; ++q) r[o][q] = T(0);
        if constexpr (DENSE) {
#pragma unroll
          for (int i = 0; i < NIN; ++i) {
            if (SEL[o][i] == 0) continue;
            const T(&M)[N][N] = A.mat[SEL[o][i] - 1];
            T v = r[o][0];
            if (left) {
#pragma unroll
              for (int j = 0; j < N; ++j) v = fma(M[P][j], u[i][g * P + j], v);
            }
            if (right) {
#pragma unroll
              for (int j = 0; j < N; ++j) v = fma(M[0][j], u[i][g * P + P + j], v);
#pragma unroll
              for (int q = 1; q < P; ++q) {
                T w = r[o][q];
#pragma unroll
                for (int j = 0; j < N; ++j) w = fma(M[q][j], u[i][g * P + P + j], w);
                r[o][q] = w;
              }
            }
            r[o][0] = v;
          }
        } else {
          T v = g > 0 ? carry[o] : T(0), next = T(0);
#pragma unroll
          for (int i = 0; i < NIN; ++i) {
            if (SEL[o][i] == 0) continue;
            const int k = SEL[o][i] - 1;
            if (g == 0 && left) v += last_row<N, T>(A.mat[k], u[i], 0);
            if (right) {
              T pr[N];
              if (k == 0) cell_rows<N, 1, T>(A.eo[0], A.mat[0], u[i], g * P + P, pr);
              else cell_rows<N, KS, T>(A.eo[1], A.mat[1], u[i], g * P + P, pr);
#pragma unroll
              for (int q = 0; q < P; ++q) r[o][q] += pr[q];
              next += pr[P];
            }
          }
          r[o][0] += left ? v : T(0);
          carry[o] = next;
        }
      }
      // store nodes s p .. s p + p - 1 (the final vertex alone), projected
      // on the z boundary
      const int cnt = right ? P : 1;
#pragma unroll
      for (int q = 0; q < P; ++q) {
        if (q >= cnt) break;
        const long long pos = (long long)s * P + q;
        const long long node = base + pos * stride;
        const bool bnd = A.dirichlet && (pos == 0 || pos == nd - 1);
#pragma unroll
        for (int o = 0; o < NOUT; ++o) (o == 0 ? A.out0 : A.out1)[node] = bnd ? T(0) : r[o][q];
      }
    }
  }
}

// x-y tile of the two passes along x and y: per z-plane Z = blockIdx.z and
// tile (blockIdx.x, blockIdx.y) of CX x CY cells, the input nodes
// X0 - p .. X0 + TX + p, Y0 - p .. Y0 + TY + p are staged in shared memory
// (coalesced along x), the x sweep runs on every staged row, the y sweep on
// the owned columns, and the results are stored coalesced.  Terms (with the
// z pass's a, b):
//   NIN = 1 (mass):  y = M_y (M_x a)
//   NIN = 2:         y = M_y (K_x a + M_x b) + K_y (M_x a)
// Owned nodes: X0 .. X0 + TX - 1 (and the final vertex Nx - 1 in the last
// tile), likewise in y.  The z pass has already applied P_z; the tile
// applies P_x and P_y to its inputs and outputs and writes y = x on every
// boundary node.
template <int N>
struct KronTile {
  static constexpr int P = N - 1;
  static constexpr int CX = (64 + P - 1) / P;        // cells along x: about 64 nodes
  // about 32 rows (measured against 16 and 48 rows: p = 4 Laplacian 148 vs
  // 158 / 178 us FP32; fewer halo rows per owned row than 16, more resident
  // blocks than 48)
  static constexpr int CY = (32 + P - 1) / P;
  static constexpr int TX = CX * P, TY = CY * P;
  static constexpr int IC = TX + 2 * P + 1;          // staged columns
  static constexpr int IR = TY + 2 * P + 1;          // staged rows
  static constexpr int OC = TX + 1;                  // x-sweep result columns
  static constexpr int THREADS = 256;
};

template <int N, typename T, int NIN, int KS>
__global__ void __launch_bounds__(KronTile<N>::THREADS) kron_xy(const __grid_constant__ KronArgs<N, T> A)
{
  using TL = KronTile<N>;
  constexpr int P = N - 1, CX = TL::CX, CY = TL::CY, TX = TL::TX;
  constexpr int IC = TL::IC, IR = TL::IR, OC = TL::OC;
  constexpr int NQ = NIN == 1 ? 1 : 2; // x-sweep results per node
  constexpr bool DENSE = sizeof(T) == 8 && N < 7; // dense rows (see cell_rows)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *in = reinterpret_cast<T *>(smem_raw);   // [NIN][IR][IC]
  T *qx = in + NIN * IR * IC;                // [NQ][IR][OC]
  const int nx = A.nn[0], ny = A.nn[1], nz = A.nn[2];
  const long long plane = (long long)nx * ny;
  const int Z = blockIdx.z;
  const int cx0 = blockIdx.x * CX, cy0 = blockIdx.y * CY;
  const int X0 = cx0 * P, Y0 = cy0 * P;
  const bool dir = A.dirichlet != 0;
  const long long zoff = (long long)Z * plane;
  // ---- stage the inputs (zero outside the mesh and at x / y boundary nodes):
  // warps on rows, lanes on columns (the column tests once per lane); each
  // warp issues all loads of its rows before its first store ----
  constexpr int WARPS = TL::THREADS / 32, CW = (IC + 31) / 32, RW = (IR + WARPS - 1) / WARPS;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool cok[CW];
#pragma unroll
  for (int j = 0; j < CW; ++j) {
    const int c = lane + 32 * j, X = X0 - P + c;
    cok[j] = c < IC && X >= 0 && X < nx && !(dir && (X == 0 || X == nx - 1));
  }
#pragma unroll
  for (int i = 0; i < NIN; ++i) {
    const T *src = i == 0 ? A.in0 : A.in1;
    T stage[RW][CW];
#pragma unroll
    for (int k = 0; k < RW; ++k) {
      const int r = warp + WARPS * k, Y = Y0 - P + r;
      const bool rok = r < IR && Y >= 0 && Y < ny && !(dir && (Y == 0 || Y == ny - 1));
      // node (X0 - p + c, Y) of plane Z, formed only for loaded (in-mesh) nodes
      const long long row = zoff + (long long)Y * nx + (X0 - P);
#pragma unroll
      for (int j = 0; j < CW; ++j) stage[k][j] = (rok && cok[j]) ? __ldg(src + (row + lane + 32 * j)) : T(0);
    }
#pragma unroll
    for (int k = 0; k < RW; ++k) {
      const int r = warp + WARPS * k;
#pragma unroll
      for (int j = 0; j < CW; ++j) {
        const int c = lane + 32 * j;
        if (r < IR && c < IC) in[(i * IR + r) * IC + c] = stage[k][j];
      }
    }
  }
  __syncthreads();
  // ---- x sweep: every staged row, the owned segments (lanes on rows) ----
  const T(&Mx)[N][N] = A.mat[0];
  const T(&Kx)[N][N] = A.mat[1];
  for (int task = threadIdx.x; task < IR * (CX + 1); task += blockDim.x) {
    const int r = task % IR, sl = task / IR;
    const int s = cx0 + sl;              // global segment
    const bool mine = sl < CX ? s <= A.nc[0] : s == A.nc[0];
    if (!mine) continue;
    const bool left = s > 0, right = s < A.nc[0];
    T u[NIN][2 * P + 1];
#pragma unroll
    for (int i = 0; i < NIN; ++i)
#pragma unroll
      for (int k = 0; k < 2 * P + 1; ++k) u[i][k] = in[(i * IR + r) * IC + sl * P + k];
    // q0 = (K_x a + M_x b) or M_x a (NIN = 1), q1 = M_x a
    T q0[P], q1[P];
    if constexpr (DENSE) {
#pragma unroll
      for (int q = 0; q < P; ++q) q0[q] = q1[q] = T(0);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const T a_l = u[0][j], a_r = u[0][P + j];
        if (NIN == 1) {
          if (left) q0[0] = fma(Mx[P][j], a_l, q0[0]);
          if (right) {
#pragma unroll
            for (int q = 0; q < P; ++q) q0[q] = fma(Mx[q][j], a_r, q0[q]);
          }
        } else {
          const T b_l = u[NIN - 1][j], b_r = u[NIN - 1][P + j];
          if (left) {
            q0[0] = fma(Kx[P][j], a_l, fma(Mx[P][j], b_l, q0[0]));
            q1[0] = fma(Mx[P][j], a_l, q1[0]);
          }
          if (right) {
#pragma unroll
            for (int q = 0; q < P; ++q) {
              q0[q] = fma(Kx[q][j], a_r, fma(Mx[q][j], b_r, q0[q]));
              q1[q] = fma(Mx[q][j], a_r, q1[q]);
            }
          }
        }
      }
    } else {
      // the right cell's rows by even-odd products, the vertex's left-cell
      // row directly
    {
      const T(&ua)[2 * P + 1] = u[0];
      const T(&ub)[2 * P + 1] = u[NIN - 1];
      T la = T(0), lb = T(0);
      if (left) {
        la = last_row<N, T>(NIN == 1 ? Mx : Kx, ua, 0);
        if (NIN == 2) {
          la += last_row<N, T>(Mx, ub, 0);
          lb = last_row<N, T>(Mx, ua, 0);
        }
      }
#pragma unroll
      for (int q = 0; q < P; ++q) q0[q] = q1[q] = T(0);
      if (right) {
        T pr[N];
        if (NIN == 1) {
          cell_rows<N, 1, T, decltype(ua), N - 1>(A.eo[0], Mx, ua, P, pr);
#pragma unroll
          for (int q = 0; q < P; ++q) q0[q] = pr[q];
        } else {
          cell_rows<N, KS, T, decltype(ua), N - 1>(A.eo[1], Kx, ua, P, pr);
#pragma unroll
          for (int q = 0; q < P; ++q) q0[q] = pr[q];
          cell_rows<N, 1, T, decltype(ub), N - 1>(A.eo[0], Mx, ub, P, pr);
#pragma unroll
          for (int q = 0; q < P; ++q) q0[q] += pr[q];
          cell_rows<N, 1, T, decltype(ua), N - 1>(A.eo[0], Mx, ua, P, pr);
#pragma unroll
          for (int q = 0; q < P; ++q) q1[q] = pr[q];
        }
      }
      q0[0] += la;
      q1[0] += lb;
    }
    }
    const int cnt = right ? P : 1;
#pragma unroll
    for (int q = 0; q < P; ++q) {
      if (q >= cnt) break;
      const int X = s * P + q;
      const bool xb = dir && (X == 0 || X == nx - 1);
      qx[r * OC + sl * P + q] = xb ? T(0) : q0[q];
      if (NQ == 2) qx[(IR + r) * OC + sl * P + q] = xb ? T(0) : q1[q];
    }
  }
  __syncthreads();
  // ---- y sweep: owned columns (lanes on columns), owned y segments; store ----
  const T(&My)[N][N] = A.mat[2];
  const T(&Ky)[N][N] = A.mat[3];
  for (int task = threadIdx.x; task < OC * (CY + 1); task += blockDim.x) {
    const int c = task % OC, tl = task / OC;
    const int X = X0 + c;
    const bool xmine = c < TX ? X < nx : X == nx - 1;
    const int t = cy0 + tl;
    const bool ymine = tl < CY ? t <= A.nc[1] : t == A.nc[1];
    if (!xmine || !ymine) continue;
    const bool left = t > 0, right = t < A.nc[1];
    // staged rows of segment t: local rows tl p .. tl p + 2p (y sweep inputs,
    // projected on the y boundary)
    T v[NQ][2 * P + 1];
#pragma unroll
    for (int k = 0; k < 2 * P + 1; ++k) {
      const int Y = t * P - P + k;
      const bool yb = dir && (Y == 0 || Y == ny - 1);
#pragma unroll
      for (int o = 0; o < NQ; ++o) v[o][k] = yb ? T(0) : qx[(o * IR + tl * P + k) * OC + c];
    }
    // y = M_y q0 (+ K_y q1)
    T y[P];
#pragma unroll
    for (int q = 0; q < P; ++q) y[q] = T(0);
    if constexpr (DENSE) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        if (left) {
          y[0] = fma(My[P][j], v[0][j], y[0]);
          if (NQ == 2) y[0] = fma(Ky[P][j], v[1][j], y[0]);
        }
        if (right) {
#pragma unroll
          for (int q = 0; q < P; ++q) {
            y[q] = fma(My[q][j], v[0][P + j], y[q]);
            if (NQ == 2) y[q] = fma(Ky[q][j], v[1][P + j], y[q]);
          }
        }
      }
    } else {
      // right cell by even-odd products, the vertex's left-cell row directly
    if (right) {
      T pr[N];
      cell_rows<N, 1, T, decltype(v[0]), N - 1>(A.eo[2], My, v[0], P, pr);
#pragma unroll
      for (int q = 0; q < P; ++q) y[q] = pr[q];
      if (NQ == 2) {
        cell_rows<N, KS, T, decltype(v[NQ - 1]), N - 1>(A.eo[3], Ky, v[NQ - 1], P, pr);
#pragma unroll
        for (int q = 0; q < P; ++q) y[q] += pr[q];
      }
    }
    if (left) {
      y[0] += last_row<N, T>(My, v[0], 0);
      if (NQ == 2) y[0] += last_row<N, T>(Ky, v[NQ - 1], 0);
    }
    }
    const int cnt = right ? P : 1;
    const bool xzb = dir && (X == 0 || X == nx - 1 || Z == 0 || Z == nz - 1);
#pragma unroll
    for (int q = 0; q < P; ++q) {
      if (q >= cnt) break;
      const int Y = t * P + q;
      const long long node = zoff + (long long)Y * nx + X;
      const bool bnd = xzb || (dir && (Y == 0 || Y == ny - 1));
      A.out0[node] = bnd ? __ldg(A.x + node) : y[q];
    }
  }
}

// cell-local 1D matrices (FP64): mass h M1, stiffness K1 / h, convection b C1
void kron_mats(const sf_op *op, int d, double (&M)[kMaxN][kMaxN], double (&K)[kMaxN][kMaxN])
{
  const Shape1D &s = op->shape;
  const int n = s.n;
  double DS[kMaxN][kMaxN];
  for (int q = 0; q < n; ++q)
    for (int j = 0; j < n; ++j) {
      double v = 0.0;
      for (int k = 0; k < n; ++k) v += s.D[q][k] * s.S[k][j];
      DS[q][j] = v;
    }
  const double h = op->h[d];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double m = 0.0, k = 0.0, c = 0.0;
      for (int q = 0; q < n; ++q) {
        m += s.S[q][i] * s.wq[q] * s.S[q][j];
        k += DS[q][i] * s.wq[q] * DS[q][j];
        c += DS[q][i] * s.wq[q] * s.S[q][j]; // (S^T D^T W S)[i][j] = sum_q (D S)[q][i] w_q S[q][j]
      }
      M[i][j] = h * m;
      K[i][j] = op->desc.kind == SF_OP_CONVECTION ? op->desc.velocity[d] * c : k / h;
    }
}

template <int N, typename T, int NIN, int NOUT, int S00, int S01, int S10, int S11, int KS>
int launch_zpass(const sf_op *op, const T *in0, T *out0, T *out1, cudaStream_t st)
{
  KronArgs<N, T> A{};
  double M[kMaxN][kMaxN], K[kMaxN][kMaxN];
  kron_mats(op, 2, M, K);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      A.mat[0][i][j] = T(M[i][j]);
      A.mat[1][i][j] = T(K[i][j]);
    }
  A.eo[0] = make_eo<N, T>([&](int i, int j) { return M[i][j]; });
  A.eo[1] = make_eo<N, T>([&](int i, int j) { return K[i][j]; });
  for (int d = 0; d < 3; ++d) {
    A.nc[d] = op->desc.n_cells[d];
    A.nn[d] = (N - 1) * A.nc[d] + 1;
  }
  A.in0 = in0;
  A.out0 = out0;
  A.out1 = out1;
  A.dirichlet = op->desc.dirichlet;
  const long long plane = (long long)A.nn[0] * A.nn[1];
  constexpr int G = KronG<N>::value;
  const long long nchunk = (A.nc[2] + 1 + G - 1) / G;
  A.tasks = nchunk * plane;
  if (A.tasks >= (1LL << 32)) {
    set_error("node grid too large for the Kronecker passes");
    return SF_ERR_UNSUPPORTED;
  }
  A.div_a = make_fast_div((unsigned)plane);
  const int threads = 256;
  const long long want = (A.tasks + threads - 1) / threads;
  const long long cap = (long long)device_sm_count() * 16;
  kron_pass<N, T, NIN, NOUT, S00, S01, S10, S11, KS><<<(unsigned)(want < cap ? want : cap), threads, 0, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N, typename T, int NIN, int KS>
int launch_xy(const sf_op *op, const T *a, const T *b, T *y, const T *x, cudaStream_t st)
{
  using TL = KronTile<N>;
  KronArgs<N, T> A{};
  for (int d = 0; d < 2; ++d) {
    double M[kMaxN][kMaxN], K[kMaxN][kMaxN];
    kron_mats(op, d, M, K);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        A.mat[2 * d][i][j] = T(M[i][j]);
        A.mat[2 * d + 1][i][j] = T(K[i][j]);
      }
    A.eo[2 * d] = make_eo<N, T>([&](int i, int j) { return M[i][j]; });
    A.eo[2 * d + 1] = make_eo<N, T>([&](int i, int j) { return K[i][j]; });
  }
  for (int d = 0; d < 3; ++d) {
    A.nc[d] = op->desc.n_cells[d];
    A.nn[d] = (N - 1) * A.nc[d] + 1;
  }
  A.in0 = a;
  A.in1 = b;
  A.out0 = y;
  A.x = x;
  A.dirichlet = op->desc.dirichlet;
  constexpr int NQ = NIN == 1 ? 1 : 2;
  const size_t smem = size_t(NIN * TL::IR * TL::IC + NQ * TL::IR * TL::OC) * sizeof(T);
  SF_CUDA_TRY(cudaFuncSetAttribute(kron_xy<N, T, NIN, KS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const dim3 grid((unsigned)((A.nc[0] + TL::CX - 1) / TL::CX), (unsigned)((A.nc[1] + TL::CY - 1) / TL::CY),
                  (unsigned)A.nn[2]);
  if (A.nn[2] > 65535) {
    set_error("Kronecker passes: more than 65535 node planes");
    return SF_ERR_UNSUPPORTED;
  }
  kron_xy<N, T, NIN, KS><<<grid, TL::THREADS, smem, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N, typename T>
int kron_impl(const sf_op *op, const T *x, T *y, cudaStream_t st)
{
  const long long n = op->n_dofs;
  T *w = (T *)op->kron.ptr;
  if (!w || op->kron.bytes < size_t(kron_work_vectors(op)) * size_t(n) * sizeof(T)) {
    set_error("Kronecker passes: work vectors missing");
    return SF_ERR_STATE;
  }
  if (op->desc.kind == SF_OP_MASS) {
    // a = M_z x; y = M_y M_x a
    SF_RET_IF((launch_zpass<N, T, 1, 1, 1, 0, 0, 0, 1>(op, x, w, nullptr, st)));
    return launch_xy<N, T, 1, 1>(op, w, nullptr, y, x, st);
  }
  // a = M_z x, b = K_z x; y = M_y (K_x a + M_x b) + K_y (M_x a)
  T *a = w, *b = w + n;
  // K: the Laplacian's stiffness is centro-symmetric, the convection matrix
  // anti-centro-symmetric
  if (op->desc.kind == SF_OP_CONVECTION) {
    SF_RET_IF((launch_zpass<N, T, 1, 2, 1, 0, 2, 0, -1>(op, x, a, b, st)));
    return launch_xy<N, T, 2, -1>(op, a, b, y, x, st);
  }
  SF_RET_IF((launch_zpass<N, T, 1, 2, 1, 0, 2, 0, 1>(op, x, a, b, st)));
  return launch_xy<N, T, 2, 1>(op, a, b, y, x, st);
}

template <int N>
int kron_n(const sf_op *op, int prec, const void *x, void *y, cudaStream_t st)
{
  if (prec == SF_FP64) return kron_impl<N, double>(op, (const double *)x, (double *)y, st);
  return kron_impl<N, float>(op, (const float *)x, (float *)y, st);
}

} // namespace

// affine operators whose node grid fits the launch shapes of both passes:
// one x-y block per tile and node plane (grid y and z at most 65535) and the
// z pass's 32-bit task index.  Larger meshes keep the line-ownership kernel.
bool kron_eligible(const sf_op *op)
{
  const int k = op->desc.kind;
  if (!((k == SF_OP_LAPLACE || k == SF_OP_MASS || k == SF_OP_CONVECTION) && !op->deformed && !op->has_kappa))
    return false;
  const long long p = op->desc.degree;
  if (p < 1 || p > kMaxN - 1) return false;
  long long nc[3], nn[3];
  for (int d = 0; d < 3; ++d) {
    nc[d] = op->desc.n_cells[d];
    nn[d] = p * nc[d] + 1;
  }
  static_assert(KronG<5>::value == 4 && KronG<6>::value == 2, "G below restates KronG");
  static_assert(KronTile<2>::CY == 32 && KronTile<5>::CY == 8 && KronTile<9>::CY == 4,
                "cy below restates KronTile::CY");
  const long long G = p + 1 <= 5 ? 4 : 2;
  const long long cy = (32 + p - 1) / p;
  const long long tasks = (nc[2] + G) / G * nn[0] * nn[1];
  return nn[2] <= 65535 && (nc[1] + cy - 1) / cy <= 65535 && tasks < (1LL << 32);
}

int kron_work_vectors(const sf_op *op) { return op->desc.kind == SF_OP_MASS ? 1 : 2; }

// FP64: always (1.3-2.4x the line kernel at p = 2..8; convection at p = 7
// within 3 %).  FP32: where measured faster than the line kernel (64^3 at
// p = 4, 48^3, 40^3, 36^3, 32^3 at p = 5..8): the Laplacian and the mass
// matrix at every degree (p = 4 Laplacian 148 vs 197 us, mass 94 vs 153;
// p = 8 187 vs 230 and 100 vs 143 us), convection up to p = 5 (141 vs 179
// us at p = 4); convection from p = 6 on stays with the line kernel (136 vs
// 139 us at p = 6, 165 vs 180 at p = 7).
bool kron_selected(const sf_op *op, int prec)
{
  if (!kron_eligible(op) || op->kernel_variant == SF_KERNEL_GENERIC || !op->kron.ptr) return false;
  if (prec == SF_FP64) return true;
  return op->desc.kind != SF_OP_CONVECTION || op->desc.degree <= 5;
}

int launch_cont_kron(const sf_op *op, int prec, const void *x, void *y, cudaStream_t st)
{
  switch (op->desc.degree) {
  case 1: return kron_n<2>(op, prec, x, y, st);
  case 2: return kron_n<3>(op, prec, x, y, st);
  case 3: return kron_n<4>(op, prec, x, y, st);
  case 4: return kron_n<5>(op, prec, x, y, st);
  case 5: return kron_n<6>(op, prec, x, y, st);
  case 6: return kron_n<7>(op, prec, x, y, st);
  case 7: return kron_n<8>(op, prec, x, y, st);
  case 8: return kron_n<9>(op, prec, x, y, st);
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;
  }
}

} // namespace sf
