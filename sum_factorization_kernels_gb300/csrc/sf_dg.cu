// sf_dg.cu -- DG operators on periodic Cartesian meshes: symmetric interior
// penalty Laplacian (Hermite-like basis) and upwind advection (GLL basis,
// optional inverse mass matrix), forward and transpose, several right-hand
// sides per launch, fused Chebyshev epilogue.
//
// Mathematics of evaluation_dg_laplacian.h:130-510 and
// evaluation_dg_advect.h:286-676: values and collocation gradients at Gauss
// points, face values/normal derivatives of the own cell extrapolated from
// the Gauss-point values, those of the neighbour read from one node layer
// (value) and two node layers (normal derivative, Hermite-like basis), SIPG
// flux -{du/dn}[v] - [u]{dv/dn} + tau [u][v] with tau = penalty (p+1)^2 / h,
// upwind flux (a.n) u_upwind, integration with the transposed matrices and
// face injection.  Corrections relative to the reference: periodic x
// neighbour index, transposed values in the last SIPG sweep.
//
// GPU mapping: a block holds CPB consecutive cells (n^2 threads each); a
// thread reads and writes one z column of its cell straight from and to the
// cell-major vector (each warp instruction covers runs of n^2 consecutive
// entries), the x and y sweeps are line-local in three padded shared-memory
// slabs per cell; each thread also owns one point of each face pair of its
// line, so the face fluxes are computed in the thread that holds the
// matching line.
#include <cmath>

#include "sf_device.cuh"
#include "sf_dg_common.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"

namespace sf {

namespace {

enum { K_SIPG = 0, K_ADVECT = 1 };
// epilogue of the apply: plain store, fused Chebyshev step, fused
// Runge-Kutta stage
enum { EPI_STORE = 0, EPI_CHEB = 1, EPI_RK = 2 };

template <int N, typename T>
struct DGArgs {
  EOMat<N, T> S, ST, D, DT, P;   // P = Sinv (Gauss values -> GLL nodes)
  EOMat<N, T> PW, PWJ;           // P W^-1 and P W^-1 / JxW (inverse mass sweeps)
  T fv0[N], fv1[N], fd0[N], fd1[N];
  T w[N];
  T iw[N];        // 1 / w
  T ij[3];        // inverse cell sizes
  T jxw;          // cell volume
  T ijxw;         // 1 / jxw
  T jface[3];     // face area elements jxw * ij_d
  T tau[3];       // SIPG penalty per direction
  T cw[3][N];     // c_d w_m, c_d = ij_d^2 jxw (SIPG), a_d ij_d jxw (advection)
  // advection flux coefficients per direction and side: fa, fb =
  // -(a.n) jface / 2, -|a.n| jface / 2 (forward), fa = -((a.n) + |a.n|)
  // jface / 2 (transpose)
  T fa[3][2], fb[3][2];
  T hd0;          // derivative of the first Hermite-like function at 0
  const T *__restrict__ x;
  T *__restrict__ y;
  const T *__restrict__ cb;      // Chebyshev: rhs
  const T *__restrict__ cdinv;   // Chebyshev: inverse diagonal
  T *__restrict__ ct;            // Chebyshev: t
  T c_np, c_tm;
  // Runge-Kutta stage: vec_np = upd + c_np r, vec_tm = vec_np + c_tm r;
  // upd may alias vec_np or vec_tm (read before written, element by element)
  const T *rk_upd;
  T *rk_np, *rk_tm;
  int nc[3];
  FastDiv div_nx, div_ny;        // division by nc[0], nc[1]
  long long n_cells, n_dofs;
};


template <int N, typename T>
__device__ __forceinline__ long long neighbour(const DGArgs<N, T> &A, int ix, int iy, int iz, int dir, int side)
{
  return periodic_neighbour(A.nc, ix, iy, iz, dir, side);
}

// face flux at one face point.  side 0: face at coordinate 0 (outer normal
// -e_d), side 1: at 1 (+e_d).  um/dm: own value and reference-coordinate
// derivative, up/dp: neighbour's.  Returns the value-test coefficient in fv
// and the derivative-test coefficient in fd (SIPG).
template <int KIND, bool TRANSPOSE, int N, typename T>
__device__ __forceinline__ void face_flux(const DGArgs<N, T> &A, int d, int side, T um, T dm, T up,
                                          T dp, T wf, T &fv, T &fd)
{
  const T jump = um - up;
  if (KIND == K_SIPG) {
    // (-{du/dn} + tau [u]) jface w and -[u] {dv/dn} jface w (the same
    // arithmetic with precomputed coefficients takes 8 more registers)
    const T sgn = side ? T(-1) : T(1);
    const T avg = sgn * T(0.5) * A.ij[d] * (dm + dp);
    fv = (avg + jump * A.tau[d]) * A.jface[d] * wf;
    fd = sgn * (T(0.5) * A.ij[d] * A.jface[d]) * jump * wf;
  } else {
    // fv = -(a.n) u_upwind jface w with (a.n) u_upwind = (a.n) {u} + |a.n| [u] / 2
    if (TRANSPOSE)
      fv = jump * A.fa[d][side] * wf;
    else
      fv = fma(um + up, A.fa[d][side], jump * A.fb[d][side]) * wf;
    fd = T(0);
  }
}

// Face arrays of a cell: NF arrays of n^2 face points, array (d, side,
// value/derivative) at index 4 d + 2 side + deriv for SIPG (12 arrays) and
// 2 d + side for advection (6 value arrays).  Arrays are FA apart, cells
// NF FA + SKEW apart; the tangential sweeps give lane `task` the line of
// array task / n (arr-major) or task % NF (line-major).  FA, SKEW and the
// map come from a bank-conflict model of the face writes, the two sweeps
// and the residual reads over the lanes of each warp.
struct DGFaceLayout {
  int FA, SKEW, LINE_MAJOR;
};

constexpr DGFaceLayout dg_face_layout(int n, bool sipg)
{
  return sipg ? (n == 2   ? DGFaceLayout{5, 0, 1}
                 : n == 3 ? DGFaceLayout{9, 5, 1}
                 : n == 4 ? DGFaceLayout{19, 12, 0}
                 : n == 5 ? DGFaceLayout{30, 17, 1}
                 : n == 6 ? DGFaceLayout{37, 8, 1}
                 : n == 7 ? DGFaceLayout{56, 17, 0}
                 : n == 8 ? DGFaceLayout{67, 0, 1}
                          : DGFaceLayout{81, 5, 0})
              : (n == 2   ? DGFaceLayout{5, 6, 1}
                 : n == 3 ? DGFaceLayout{9, 5, 0}
                 : n == 4 ? DGFaceLayout{21, 18, 0}
                 : n == 5 ? DGFaceLayout{25, 3, 0}
                 : n == 6 ? DGFaceLayout{37, 6, 1}
                 : n == 7 ? DGFaceLayout{56, 1, 0}
                 : n == 8 ? DGFaceLayout{67, 0, 1}
                          : DGFaceLayout{81, 11, 0});
}

template <int KIND>
__host__ __device__ constexpr int face_arrays()
{
  return KIND == K_SIPG ? 12 : 6;
}

// array index of (direction, side, value = 0 / derivative = 1)
template <int KIND>
__device__ __forceinline__ constexpr int face_index(int d, int side, int deriv)
{
  return KIND == K_SIPG ? 4 * d + 2 * side + deriv : 2 * d + side;
}

// Everything for one line of direction d held by this thread: values at Gauss
// points u[], neighbour face data at index fi, produce the line residual r[]
// (collocation space) = cell term + face injections.
template <int KIND, bool TRANSPOSE, int N, typename T>
__device__ __forceinline__ void line_residual(const DGArgs<N, T> &A, int d, const T (&u)[N], T wt,
                                              const T *F, int fi, T (&r)[N])
{
  // own face values/derivatives (reference coordinates)
  const T vm = dot_row<N, T>(A.fv0, u), vp = dot_row<N, T>(A.fv1, u);
  T dm = T(0), dp = T(0);
  if (KIND == K_SIPG) {
    dm = dot_row<N, T>(A.fd0, u);
    dp = dot_row<N, T>(A.fd1, u);
  }
  constexpr int FA = dg_face_layout(N, KIND == K_SIPG).FA;
  const T *Fm = F + face_index<KIND>(d, 0, 0) * FA, *Fp = F + face_index<KIND>(d, 1, 0) * FA;
  T fvm, fdm, fvp, fdp;
  // the derivative array follows the value array of the same face (SIPG)
  face_flux<KIND, TRANSPOSE, N, T>(A, d, 0, vm, dm, Fm[fi], KIND == K_SIPG ? Fm[FA + fi] : T(0), wt,
                                   fvm, fdm);
  face_flux<KIND, TRANSPOSE, N, T>(A, d, 1, vp, dp, Fp[fi], KIND == K_SIPG ? Fp[FA + fi] : T(0), wt,
                                   fvp, fdp);
  T g[N];
  if (KIND == K_SIPG) {
    eo_apply<N, -1>(A.D, u, g);
#pragma unroll
    for (int m = 0; m < N; ++m) g[m] *= A.cw[d][m] * wt;
    eo_apply<N, -1>(A.DT, g, r);
  } else if (!TRANSPOSE) {
#pragma unroll
    for (int m = 0; m < N; ++m) g[m] = A.cw[d][m] * wt * u[m];
    eo_apply<N, -1>(A.DT, g, r);
  } else {
    eo_apply<N, -1>(A.D, u, g);
#pragma unroll
    for (int m = 0; m < N; ++m) r[m] = A.cw[d][m] * wt * g[m];
  }
#pragma unroll
  for (int m = 0; m < N; ++m) {
    r[m] = fma(A.fv0[m], fvm, r[m]);
    r[m] = fma(A.fv1[m], fvp, r[m]);
    if (KIND == K_SIPG) {
      r[m] = fma(A.fd0[m], fdm, r[m]);
      r[m] = fma(A.fd1[m], fdp, r[m]);
    }
  }
}

// Shared-memory layout of one of the three slabs of dg_kernel: entry
// (x, y, z) of the block's cell cs at BASE + cs RS + SX x + SY y + SZ z.
struct DGSlab {
  int SX, SY, SZ, RS, BASE;
};

// The slabs and the lines the threads own in the x and y sweeps: the thread
// of z column (a, b) owns the x line (y, z) = (a, b), or (b, a) with XS, and
// the y line (x, z) = (a, b), or (b, a) with YS.  Either the padded layout
// of dg_layout with the three slabs of a cell side by side, or (FP32) three
// regions with strides from a bank-conflict model of the kernel's access
// patterns over the lanes of each warp.
struct DGSlabs {
  int XS, YS;
  DGSlab B0, B1, B2;
};

constexpr DGSlabs dg_slabs(int n, int elem)
{
  if (elem == 4 && n == 5)
    return DGSlabs{0, 0, {26, 1, 5, 153, 0}, {26, 1, 5, 153, 5 * 153}, {1, 5, 37, 185, 10 * 153}};
  if (elem == 4 && n == 6)
    return DGSlabs{1, 0, {1, 6, 49, 292, 0}, {37, 6, 1, 228, 7 * 292}, {1, 6, 38, 228, 7 * 292 + 7 * 228}};
  if (elem == 4 && n == 2)
    return DGSlabs{0, 0, {1, 2, 5, 12, 0}, {1, 2, 5, 12, 32 * 12}, {1, 2, 6, 12, 64 * 12}};
  if (elem == 4 && n == 4)
    return DGSlabs{0, 0, {1, 4, 19, 80, 0}, {1, 4, 19, 80, 8 * 80}, {1, 4, 20, 80, 16 * 80}};
  if (elem == 4 && n == 7)
    return DGSlabs{1, 1, {52, 7, 1, 369, 0}, {1, 7, 52, 369, 5 * 369}, {7, 49, 1, 343, 10 * 369}};
  if (elem == 4 && n == 8)
    return DGSlabs{1, 0, {67, 8, 1, 533, 0}, {67, 8, 1, 533, 2 * 533}, {1, 8, 72, 568, 4 * 533}};
  if (elem == 4 && n == 9)
    return DGSlabs{0, 0, {1, 9, 81, 729, 0}, {1, 9, 81, 729, 3 * 729}, {1, 9, 105, 945, 6 * 729}};
  const DGLayout L = dg_layout(n, elem);
  const int slab = L.P2 * n, rs = 3 * slab + L.SKEW;
  return DGSlabs{0, 0, {1, L.P1, L.P2, rs, 0}, {1, L.P1, L.P2, rs, slab}, {1, L.P1, L.P2, rs, 2 * slab}};
}

// words from the start of the slabs to the end of slab S of the last cell
constexpr int dg_slab_end(int n, int cpb, DGSlab S)
{
  return S.BASE + (cpb - 1) * S.RS + (n - 1) * (S.SX + S.SY + S.SZ) + 1;
}

constexpr int imax3(int a, int b, int c) { return a > b ? (a > c ? a : c) : (b > c ? b : c); }

// every entry of the first ns slabs has its own word and the slabs of the
// block's cells do not overlap
constexpr bool dg_slabs_fit(int n, int cpb, DGSlabs S, int ns = 3)
{
  bool seen[8192] = {};
  const DGSlab L[3] = {S.B0, S.B1, S.B2};
  for (int s = 0; s < ns; ++s)
    for (int c = 0; c < cpb; ++c)
      for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
          for (int x = 0; x < n; ++x) {
            const int i = L[s].BASE + c * L[s].RS + L[s].SX * x + L[s].SY * y + L[s].SZ * z;
            if (i < 0 || i >= 8192 || seen[i]) return false;
            seen[i] = true;
          }
  return true;
}

template <int N, typename T>
struct DGCfg {
  static constexpr int CPB = DGCells<N>::value;
  static constexpr DGSlabs S = dg_slabs(N, (int)sizeof(T));
  // slab words of a block
  static constexpr int SLABS = imax3(dg_slab_end(N, CPB, S.B0), dg_slab_end(N, CPB, S.B1), dg_slab_end(N, CPB, S.B2));
  static_assert(SLABS > 8192 || dg_slabs_fit(N, CPB, S), "slab entries overlap");
  // face region per cell of an operator kind
  static constexpr int face_stride(bool sipg)
  {
    return (sipg ? 12 : 6) * dg_face_layout(N, sipg).FA + dg_face_layout(N, sipg).SKEW;
  }
  static constexpr size_t smem(bool sipg)
  {
    return (size_t(SLABS) + size_t(CPB) * face_stride(sipg)) * sizeof(T);
  }
};

template <int N, typename T, int KIND, bool TRANSPOSE, bool INVMASS, int EPI>
__global__ void __launch_bounds__(DGCells<N>::value *N *N)
    dg_kernel(const __grid_constant__ DGArgs<N, T> A)
{
  using Cfg = DGCfg<N, T>;
  constexpr int N2 = N * N, N3 = N * N * N;
  constexpr int CPB = Cfg::CPB;
  constexpr DGSlab L0 = Cfg::S.B0, L1 = Cfg::S.B1, L2 = Cfg::S.B2;
  constexpr int NF = face_arrays<KIND>(); // face arrays per cell
  constexpr DGFaceLayout FL = dg_face_layout(N, KIND == K_SIPG);
  constexpr int FA = FL.FA;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *smem = reinterpret_cast<T *>(smem_raw);
  const int tid = threadIdx.x;
  const int cs = tid / N2;
  const int t = tid - cs * N2;
  const int a = t % N, b = t / N;
  const long long cell0 = (long long)blockIdx.x * CPB;
  const long long cell = cell0 + cs;
  const bool valid = cell < A.n_cells;
  const long long roff = (long long)blockIdx.y * A.n_dofs; // right-hand side offset
  const T *__restrict__ x = A.x + roff;
  T *B0 = smem + L0.BASE + cs * L0.RS;
  T *B1 = smem + L1.BASE + cs * L1.RS;
  T *B2 = smem + L2.BASE + cs * L2.RS;
  // face arrays: [dir][side][value, derivative][n^2]  (SIPG), values only (advection)
  T *F = smem + Cfg::SLABS + cs * Cfg::face_stride(KIND == K_SIPG);
  // the lines of this thread: z column (a, b), x line (y, z) = (xy, xz),
  // y line (x, z) = (yx, yz); their bases in each slab
  const int xy = Cfg::S.XS ? b : a, xz = Cfg::S.XS ? a : b;
  const int yx = Cfg::S.YS ? b : a, yz = Cfg::S.YS ? a : b;
  const int zc0 = L0.SX * a + L0.SY * b, xl0 = L0.SY * xy + L0.SZ * xz, yl0 = L0.SX * yx + L0.SZ * yz;
  const int zc1 = L1.SX * a + L1.SY * b, xl1 = L1.SY * xy + L1.SZ * xz, yl1 = L1.SX * yx + L1.SZ * yz;
  const int zc2 = L2.SX * a + L2.SY * b, yl2 = L2.SX * yx + L2.SZ * yz;
  // face point index of the x line on the x faces, of the y line on the y faces
  const int fx = xy + N * xz, fy = yx + N * yz;
  // this thread's z column in the cell-major vector: runs of n^2 consecutive
  // entries per warp instruction (coalesced)
  const long long col = cell * N3 + t;

  T v[N], r[N];
  // ---- z column of the input, z sweep ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = valid ? __ldg(x + col + N2 * m) : T(0);
  eo_apply<N, 1>(A.S, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) B0[zc0 + L0.SZ * m] = v[m];
  // ---- neighbour face layers ----
  if (valid) {
    const unsigned uc = (unsigned)cell;
    const unsigned q = fast_div(uc, A.div_nx);
    const unsigned iz = fast_div(q, A.div_ny);
    const int ix = int(uc - q * (unsigned)A.nc[0]), iy = int(q - iz * (unsigned)A.nc[1]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      // face-local index t: x faces (b,c) = (t%N, t/N), y faces (a,c), z faces (a,b)
      const int f0 = t % N, f1 = t / N;
      long long base_in[2];
      int stride_n;
      // offset of the face point inside a cell, without the normal coordinate
      int off;
      if (d == 0) { off = N * f0 + N2 * f1; stride_n = 1; }
      else if (d == 1) { off = f0 + N2 * f1; stride_n = N; }
      else { off = f0 + N * f1; stride_n = N2; }
      base_in[0] = neighbour(A, ix, iy, int(iz), d, 0) * N3 + off;
      base_in[1] = neighbour(A, ix, iy, int(iz), d, 1) * N3 + off;
      // side 0 (face at 0): neighbour's layer p (value) and p-1; side 1: layers 0 and 1
      const T v0 = __ldg(x + base_in[0] + (N - 1) * stride_n);
      const T v1 = __ldg(x + base_in[1]);
      F[face_index<KIND>(d, 0, 0) * FA + t] = v0;
      F[face_index<KIND>(d, 1, 0) * FA + t] = v1;
      if (KIND == K_SIPG) {
        const T u0 = __ldg(x + base_in[0] + (N - 2) * stride_n);
        const T u1 = __ldg(x + base_in[1] + stride_n);
        F[face_index<KIND>(d, 0, 1) * FA + t] = A.hd0 * (u0 - v0);
        F[face_index<KIND>(d, 1, 1) * FA + t] = -A.hd0 * (u1 - v1);
      }
    }
  }
  __syncthreads();
  // ---- first tangential direction of the faces ----
  for (int task = t; task < NF * N; task += N2) {
    const int arr = FL.LINE_MAJOR ? task % NF : task / N, line = FL.LINE_MAJOR ? task / NF : task % N;
    T *Fa = F + arr * FA + line * N;
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Fa[m];
    eo_apply<N, 1>(A.S, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m) Fa[m] = v[m];
  }
  __syncthreads();
  // ---- x sweep, second tangential direction of the faces ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B0[xl0 + L0.SX * m];
  eo_apply<N, 1>(A.S, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) B0[xl0 + L0.SX * m] = v[m];
  for (int task = t; task < NF * N; task += N2) {
    const int arr = FL.LINE_MAJOR ? task % NF : task / N, line = FL.LINE_MAJOR ? task / NF : task % N;
    T *Fa = F + arr * FA + line;
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Fa[N * m];
    eo_apply<N, 1>(A.S, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m) Fa[N * m] = v[m];
  }
  __syncthreads();
  // ---- y lines: Gauss-point values, y residual ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B0[yl0 + L0.SY * m];
  eo_apply<N, 1>(A.S, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) B1[yl1 + L1.SY * m] = v[m];
  // y line (x, z): face point (x, z) has weight w_x w_z
  line_residual<KIND, TRANSPOSE, N, T>(A, 1, v, A.w[a] * A.w[b], F, fy, r);
#pragma unroll
  for (int m = 0; m < N; ++m) B2[yl2 + L2.SY * m] = r[m];
  __syncthreads();
  // ---- x lines and z lines ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B1[xl1 + L1.SX * m];
  // x line (y, z)
  line_residual<KIND, TRANSPOSE, N, T>(A, 0, v, A.w[a] * A.w[b], F, fx, r);
#pragma unroll
  for (int m = 0; m < N; ++m) B0[xl0 + L0.SX * m] = r[m];
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B1[zc1 + L1.SZ * m];
  T rz[N];
  line_residual<KIND, TRANSPOSE, N, T>(A, 2, v, A.w[a] * A.w[b], F, t, rz);
  __syncthreads();
  // ---- sum; integrate / apply the inverse mass along x, y, then z ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = rz[m] + B0[zc0 + L0.SZ * m] + B2[zc2 + L2.SZ * m];
  // with the inverse mass, the scaling 1 / (JxW w_x w_y w_z) at the Gauss
  // points sits in the tables of the three P sweeps (PW, PW, PWJ)
#pragma unroll
  for (int m = 0; m < N; ++m) B1[zc1 + L1.SZ * m] = v[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B1[xl1 + L1.SX * m];
  if (INVMASS) eo_apply<N, 1>(A.PW, v, v);
  else eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) B1[xl1 + L1.SX * m] = v[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B1[yl1 + L1.SY * m];
  if (INVMASS) eo_apply<N, 1>(A.PW, v, v);
  else eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) B1[yl1 + L1.SY * m] = v[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = B1[zc1 + L1.SZ * m];
  if (INVMASS) eo_apply<N, 1>(A.PWJ, v, v);
  else eo_apply<N, 1>(A.ST, v, v);
  // ---- store the z column (plain, fused Chebyshev or Runge-Kutta update) ----
  if (valid) {
    T *dst = A.y + roff + col;
    if (EPI == EPI_RK) {
      const long long o = roff + col;
#pragma unroll
      for (int m = 0; m < N; ++m) {
        const long long e = o + N2 * m;
        const T np = A.rk_upd[e] + A.c_np * v[m];
        A.rk_np[e] = np;
        if (A.c_tm != T(0)) A.rk_tm[e] = np + A.c_tm * v[m];
      }
    } else if (EPI == EPI_CHEB) {
      const long long o = col;
#pragma unroll
      for (int m = 0; m < N; ++m) {
        const long long e = o + N2 * m;
        const T res = v[m] - A.cb[e];
        const T tn = A.c_tm * A.ct[e] + A.c_np * A.cdinv[e] * res;
        A.ct[e] = tn;
        dst[N2 * m] = __ldg(x + e) - tn;
      }
    } else {
#pragma unroll
      for (int m = 0; m < N; ++m) dst[N2 * m] = v[m];
    }
  }
}

// Slabs of the inverse mass kernel: region ZX (written along z columns, read
// along x lines and the reverse) and region XY (x and y lines), x lines
// (y, z) = (b, a) with XS, y lines (x, z) = (b, a) with YS.  FP32: layouts
// from the bank-conflict model (both regions conflict-free for their two
// patterns at degrees 1 and 3-5, 7, 8); FP64: the padded layout of
// dg_layout in both regions.
struct DGInvLayout {
  int XS, YS;
  DGSlab ZX, XY;
};

constexpr DGInvLayout dg_inv_layout(int n, int elem, int cpb)
{
  if (elem == 4) {
    switch (n) {
    case 2: return DGInvLayout{0, 0, {1, 2, 5, 12, 0}, {1, 3, 6, 12, 32 * 12}};
    case 3: return DGInvLayout{1, 1, {3, 9, 1, 27, 0}, {1, 33, 11, 99, 14 * 27}};
    case 4: return DGInvLayout{0, 0, {1, 4, 17, 80, 0}, {1, 5, 20, 80, 8 * 80}};
    case 5: return DGInvLayout{1, 1, {1, 5, 33, 185, 0}, {5, 37, 1, 185, 5 * 185}};
    case 6: return DGInvLayout{1, 1, {1, 6, 49, 292, 0}, {6, 38, 1, 228, 7 * 292}};
    case 7: return DGInvLayout{0, 0, {1, 7, 49, 343, 0}, {1, 65, 7, 465, 5 * 343}};
    case 8: return DGInvLayout{0, 0, {68, 1, 8, 540, 0}, {1, 65, 8, 519, 2 * 540}};
    case 9: return DGInvLayout{1, 1, {1, 9, 97, 881, 0}, {9, 105, 1, 945, 3 * 881}};
    default: break;
    }
  }
  const DGLayout L = dg_layout(n, elem);
  const int rs = L.P2 * n + L.SKEW;
  return DGInvLayout{0, 0, {1, L.P1, L.P2, rs, 0}, {1, L.P1, L.P2, rs, cpb * rs}};
}

template <int N, typename T>
struct DGInvCfg {
  static constexpr int CPB = DGCells<N>::value;
  static constexpr DGInvLayout L = dg_inv_layout(N, (int)sizeof(T), CPB);
  static constexpr int WORDS = dg_slab_end(N, CPB, L.ZX) > dg_slab_end(N, CPB, L.XY) ? dg_slab_end(N, CPB, L.ZX)
                                                                                       : dg_slab_end(N, CPB, L.XY);
  static_assert(WORDS > 8192 || dg_slabs_fit(N, CPB, DGSlabs{0, 0, L.ZX, L.XY, L.XY}, 2), "slab entries overlap");
};

// cell-local inverse mass matrix M^-1 = P W^-1 P^T (GLL basis, Gauss points)
template <int N, typename T>
__global__ void __launch_bounds__(DGCells<N>::value *N *N)
    dg_inverse_mass_kernel(const __grid_constant__ DGArgs<N, T> A)
{
  // z columns read and written straight from the cell-major vectors: P^T
  // along z (registers), x, y; scale by 1/(JxW w) at the Gauss points (the
  // 1/w of the y direction sits in the table, slot D = W^-1 P^T); P along y,
  // x, z (registers).  Slot ST holds P^T.
  using Cfg = DGInvCfg<N, T>;
  constexpr int N2 = N * N, N3 = N * N * N;
  constexpr int CPB = Cfg::CPB;
  constexpr DGSlab ZX = Cfg::L.ZX, XY = Cfg::L.XY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *smem = reinterpret_cast<T *>(smem_raw);
  const int tid = threadIdx.x;
  const int cs = tid / N2;
  const int t = tid - cs * N2;
  const int a = t % N, b = t / N;
  const int xy = Cfg::L.XS ? b : a, xz = Cfg::L.XS ? a : b; // x line (y, z)
  const int yx = Cfg::L.YS ? b : a, yz = Cfg::L.YS ? a : b; // y line (x, z)
  const long long cell = (long long)blockIdx.x * CPB + cs;
  const bool valid = cell < A.n_cells;
  const long long col = (long long)blockIdx.y * A.n_dofs + cell * N3 + t;
  T *Z = smem + ZX.BASE + cs * ZX.RS;
  T *X = smem + XY.BASE + cs * XY.RS;
  const int zc = ZX.SX * a + ZX.SY * b, xlz = ZX.SY * xy + ZX.SZ * xz;
  const int xlx = XY.SY * xy + XY.SZ * xz, ylx = XY.SX * yx + XY.SZ * yz;
  T v[N];
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = valid ? __ldg(A.x + col + N2 * m) : T(0);
  eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) Z[zc + ZX.SZ * m] = v[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = Z[xlz + ZX.SX * m];
  eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) X[xlx + XY.SX * m] = v[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = X[ylx + XY.SY * m];
  eo_apply<N, 1>(A.D, v, v);
  // Gauss point (yx, m, yz): the remaining 1 / (JxW w_x w_z)
  const T iwab = A.ijxw * A.iw[yx] * A.iw[yz];
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] *= iwab;
  eo_apply<N, 1>(A.P, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) X[ylx + XY.SY * m] = v[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = X[xlx + XY.SX * m];
  eo_apply<N, 1>(A.P, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) Z[xlz + ZX.SX * m] = v[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = Z[zc + ZX.SZ * m];
  eo_apply<N, 1>(A.P, v, v);
  if (valid) {
#pragma unroll
    for (int m = 0; m < N; ++m) A.y[col + N2 * m] = v[m];
  }
}

// fill a vector with a per-cell pattern of n^3 values (uniform Cartesian mesh)
template <typename T>
__global__ void pattern_kernel(long long n, int n3, const T *__restrict__ pat, T *__restrict__ y)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = pat[i % n3];
}

template <int N, typename T>
DGArgs<N, T> make_dg_args(const sf_op *op, bool transpose = false)
{
  DGArgs<N, T> A{};
  const Shape1D &s = op->shape;
  A.S = eo_of<N, T>(s.S, false);
  A.ST = eo_of<N, T>(s.S, true);
  A.D = eo_of<N, T>(s.D, false);
  A.DT = eo_of<N, T>(s.D, true);
  A.P = eo_of<N, T>(s.Sinv, false);
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  A.PW = make_eo<N, T>([&](int i, int j) { return s.Sinv[i][j] / s.wq[j]; });
  A.PWJ = make_eo<N, T>([&](int i, int j) { return s.Sinv[i][j] / (s.wq[j] * jxw); });
  for (int i = 0; i < N; ++i) {
    A.fv0[i] = T(s.fv[0][i]);
    A.fv1[i] = T(s.fv[1][i]);
    A.fd0[i] = T(s.fd[0][i]);
    A.fd1[i] = T(s.fd[1][i]);
    A.w[i] = T(s.wq[i]);
    A.iw[i] = T(1.0 / s.wq[i]);
  }
  A.jxw = T(jxw);
  A.ijxw = T(1.0 / jxw);
  for (int d = 0; d < 3; ++d) {
    const double ij = 1.0 / op->h[d];
    A.ij[d] = T(ij);
    A.jface[d] = T(jxw * ij);
    A.tau[d] = T((N) * (N) * op->desc.penalty * ij);
    const double cdir = op->desc.kind == SF_OP_DG_SIPG ? ij * ij * jxw : op->desc.velocity[d] * ij * jxw;
    for (int m = 0; m < N; ++m) A.cw[d][m] = T(cdir * s.wq[m]);
    const double jf = jxw * ij;
    for (int side = 0; side < 2; ++side) {
      const double an = side ? op->desc.velocity[d] : -op->desc.velocity[d];
      A.fa[d][side] = T(-0.5 * (transpose ? an + std::fabs(an) : an) * jf);
      A.fb[d][side] = T(-0.5 * std::fabs(an) * jf);
    }
    A.nc[d] = op->desc.n_cells[d];
  }
  A.div_nx = make_fast_div((unsigned)A.nc[0]);
  A.div_ny = make_fast_div((unsigned)A.nc[1]);
  A.hd0 = T(s.hermite_d0);
  A.n_cells = op->n_cells;
  A.n_dofs = op->n_dofs;
  return A;
}

template <int N, typename T>
int dg_vmult_impl(const sf_op *op, int nrhs, bool transpose, const T *x, T *y, const T *cb,
                  const T *cdinv, T *ct, double c_np, double c_tm, const T *rk_upd, T *rk_np, T *rk_tm,
                  cudaStream_t st)
{
  constexpr int CPB = DGCells<N>::value;
  DGArgs<N, T> A = make_dg_args<N, T>(op, transpose);
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
  const bool sipg = op->desc.kind == SF_OP_DG_SIPG;
  const bool cheb = cb != nullptr, rk = rk_np != nullptr;
  const bool invm = !sipg && !transpose && op->desc.inverse_mass;
  void (*kern)(const DGArgs<N, T>);
  if (sipg)
    kern = cheb ? dg_kernel<N, T, K_SIPG, false, false, EPI_CHEB> : dg_kernel<N, T, K_SIPG, false, false, EPI_STORE>;
  else if (transpose)
    kern = dg_kernel<N, T, K_ADVECT, true, false, EPI_STORE>;
  else if (invm)
    kern = rk ? dg_kernel<N, T, K_ADVECT, false, true, EPI_RK>
         : cheb ? dg_kernel<N, T, K_ADVECT, false, true, EPI_CHEB> : dg_kernel<N, T, K_ADVECT, false, true, EPI_STORE>;
  else
    kern = rk ? dg_kernel<N, T, K_ADVECT, false, false, EPI_RK>
         : cheb ? dg_kernel<N, T, K_ADVECT, false, false, EPI_CHEB>
                : dg_kernel<N, T, K_ADVECT, false, false, EPI_STORE>;
  const size_t smem = DGCfg<N, T>::smem(sipg);
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  const long long blocks = (op->n_cells + CPB - 1) / CPB;
  kern<<<dim3((unsigned)blocks, (unsigned)nrhs), dim3(CPB * N * N), smem, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N, typename T>
int dg_invmass_impl(const sf_op *op, int nrhs, const T *x, T *y, cudaStream_t st)
{
  constexpr int CPB = DGCells<N>::value;
  DGArgs<N, T> A = make_dg_args<N, T>(op);
  // P^T in the ST slot, W^-1 P^T (Gauss weights along the row) in the D slot
  const Shape1D &sh = op->shape;
  A.ST = eo_of<N, T>(sh.Sinv, true);
  A.D = make_eo<N, T>([&](int i, int j) { return sh.Sinv[j][i] / sh.wq[i]; });
  A.x = x;
  A.y = y;
  const size_t smem = size_t(DGInvCfg<N, T>::WORDS) * sizeof(T);
  SF_CUDA_TRY(cudaFuncSetAttribute(dg_inverse_mass_kernel<N, T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long blocks = (op->n_cells + CPB - 1) / CPB;
  dg_inverse_mass_kernel<N, T><<<dim3((unsigned)blocks, (unsigned)nrhs), dim3(CPB * N * N), smem, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N>
int dg_vmult_n(const sf_op *op, int prec, int nrhs, bool tr, const void *x, void *y, const void *cb,
               const void *cd, void *ct, double c_np, double c_tm, const void *upd, void *vnp, void *vtm,
               cudaStream_t st)
{
  if (prec == SF_FP64)
    return dg_vmult_impl<N, double>(op, nrhs, tr, (const double *)x, (double *)y, (const double *)cb,
                                    (const double *)cd, (double *)ct, c_np, c_tm, (const double *)upd,
                                    (double *)vnp, (double *)vtm, st);
  return dg_vmult_impl<N, float>(op, nrhs, tr, (const float *)x, (float *)y, (const float *)cb,
                                 (const float *)cd, (float *)ct, c_np, c_tm, (const float *)upd, (float *)vnp,
                                 (float *)vtm, st);
}

template <int N>
int dg_invmass_n(const sf_op *op, int prec, int nrhs, const void *x, void *y, cudaStream_t st)
{
  if (prec == SF_FP64) return dg_invmass_impl<N, double>(op, nrhs, (const double *)x, (double *)y, st);
  return dg_invmass_impl<N, float>(op, nrhs, (const float *)x, (float *)y, st);
}

} // namespace

#define SF_DEG_DISPATCH(DEG, FN, ...)                                          \
  switch (DEG) {                                                               \
  case 1: return FN<2>(__VA_ARGS__);                                           \
  case 2: return FN<3>(__VA_ARGS__);                                           \
  case 3: return FN<4>(__VA_ARGS__);                                           \
  case 4: return FN<5>(__VA_ARGS__);                                           \
  case 5: return FN<6>(__VA_ARGS__);                                           \
  case 6: return FN<7>(__VA_ARGS__);                                           \
  case 7: return FN<8>(__VA_ARGS__);                                           \
  case 8: return FN<9>(__VA_ARGS__);                                           \
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;         \
  }

int launch_dg_vmult(const sf_op *op, int prec, int nrhs, bool transpose, const void *x, void *y,
                    const void *cb, const void *cdinv, void *ct, double c_np, double c_tm,
                    cudaStream_t st)
{
  if (op->desc.n_cells[0] < 1) return SF_ERR_INVALID;
  SF_DEG_DISPATCH(op->desc.degree, dg_vmult_n, op, prec, nrhs, transpose, x, y, cb, cdinv, ct, c_np,
                  c_tm, nullptr, nullptr, nullptr, st)
}

int launch_dg_rk_stage(const sf_op *op, int prec, int nrhs, const void *src, const void *upd, void *vec_np,
                       void *vec_tm, double c_np, double c_tm, cudaStream_t st)
{
  if (op->desc.kind != SF_OP_DG_ADVECT) return SF_ERR_STATE;
  SF_DEG_DISPATCH(op->desc.degree, dg_vmult_n, op, prec, nrhs, false, src, vec_np, nullptr, nullptr, nullptr,
                  c_np, c_tm, upd, vec_np, vec_tm, st)
}

int launch_dg_inverse_mass(const sf_op *op, int prec, int nrhs, const void *x, void *y,
                           cudaStream_t st)
{
  SF_DEG_DISPATCH(op->desc.degree, dg_invmass_n, op, prec, nrhs, x, y, st)
}

// Diagonal of the SIPG operator on a uniform periodic Cartesian mesh.  The
// operator is sum_d (1D SIPG along d) x (1D mass) x (1D mass); its diagonal
// entry for local node (a,b,c) is
//   sum_d K_d[i_d] prod_{e != d} M[i_e]
// with M[i] = sum_q w_q phi_i(x_q)^2 and, for direction d with inverse size
// ij, volume jxw, face area jf = jxw ij and tau = pen (p+1)^2 ij,
//   K_d[i] = ij^2 jxw sum_q w_q phi_i'(x_q)^2
//          + jf (ij phi_i'(0) phi_i(0) + tau phi_i(0)^2
//                - ij phi_i'(1) phi_i(1) + tau phi_i(1)^2)
// (the own-cell part of the face terms; neighbour couplings are off the
// diagonal except along a direction one cell thick).  Computed on the host in FP64 and broadcast to all cells.
// Advection has no diagonal preconditioner use; it gets the same formula's
// analogue: sum_d of the cell-diagonal of M^-1 K along d is not provided.
int launch_dg_diagonal(const sf_op *op, int prec, void *diag, cudaStream_t st)
{
  if (op->desc.kind != SF_OP_DG_SIPG) {
    set_error("diagonal only for SF_OP_DG_SIPG and SF_OP_LAPLACE");
    return SF_ERR_STATE;
  }
  const Shape1D &s = op->shape;
  const int n = s.n, n3 = n * n * n;
  // 1D basis values / derivatives at Gauss points and faces, through the
  // Gauss-Lagrange interpolant of the Gauss-point values (exact)
  double M[kMaxN], K[3][kMaxN];
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  for (int i = 0; i < n; ++i) {
    double m = 0, k = 0, v0 = 0, v1 = 0, d0 = 0, d1 = 0;
    double dq[kMaxN];
    for (int q = 0; q < n; ++q) {
      double dd = 0;
      for (int j = 0; j < n; ++j) dd += s.D[q][j] * s.S[j][i];
      dq[q] = dd;
    }
    for (int q = 0; q < n; ++q) {
      m += s.wq[q] * s.S[q][i] * s.S[q][i];
      k += s.wq[q] * dq[q] * dq[q];
      v0 += s.fv[0][q] * s.S[q][i];
      v1 += s.fv[1][q] * s.S[q][i];
      d0 += s.fd[0][q] * s.S[q][i];
      d1 += s.fd[1][q] * s.S[q][i];
    }
    M[i] = m;
    for (int d = 0; d < 3; ++d) {
      const double ij = 1.0 / op->h[d], jf = jxw * ij;
      const double tau = op->desc.penalty * n * n * ij;
      K[d][i] = ij * ij * jxw * k + jf * (ij * d0 * v0 + tau * v0 * v0 - ij * d1 * v1 + tau * v1 * v1);
      // a direction one cell thick is its own periodic neighbour on both
      // faces: the couplings with the neighbour's end values (left: trial at
      // 1, test at 0; right: the mirror) then contribute to the diagonal
      if (op->desc.n_cells[d] == 1) K[d][i] += jf * (-2.0 * tau * v0 * v1 - ij * d0 * v1 + ij * v0 * d1);
    }
  }
  double pat[kMaxN * kMaxN * kMaxN];
  for (int c = 0; c < n; ++c)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a)
        pat[(c * n + b) * n + a] = K[0][a] * M[b] * M[c] + M[a] * K[1][b] * M[c] + M[a] * M[b] * K[2][c];
  DevBuf buf;
  if (prec == SF_FP64) {
    int r = buf.alloc(n3 * sizeof(double));
    if (r) return r;
    SF_CUDA_TRY(cudaMemcpyAsync(buf.ptr, pat, n3 * sizeof(double), cudaMemcpyHostToDevice, st));
    pattern_kernel<double><<<device_sm_count() * 8, 256, 0, st>>>(op->n_dofs, n3, (const double *)buf.ptr, (double *)diag);
  } else {
    float pf[kMaxN * kMaxN * kMaxN];
    for (int i = 0; i < n3; ++i) pf[i] = float(pat[i]);
    int r = buf.alloc(n3 * sizeof(float));
    if (r) return r;
    SF_CUDA_TRY(cudaMemcpyAsync(buf.ptr, pf, n3 * sizeof(float), cudaMemcpyHostToDevice, st));
    pattern_kernel<float><<<device_sm_count() * 8, 256, 0, st>>>(op->n_dofs, n3, (const float *)buf.ptr, (float *)diag);
  }
  SF_CUDA_TRY(cudaGetLastError());
  // the staging buffer is released when buf goes out of scope; wait for the
  // kernel that reads it
  SF_CUDA_TRY(cudaStreamSynchronize(st));
  return SF_OK;
}

} // namespace sf
