// sf_laplace_line.cu -- continuous Laplacian, line ownership, all degrees and
// both precisions: the default apply.
//
// A cell group of W warps processes K cells of one colour class at a time:
// lane t works on cell t / n^2 and owns line l = t % n^2 of it (x line, y
// line and z column (a, b) with l = a + n b), so K n^2 of the 32 W lanes do
// useful work (5 cells in 4 warps at n = 5, 8 cells in one warp at n = 2).
// Per cell, 12 line sweeps go through three padded shared-memory slabs; the
// z sweeps run in registers on the column the thread also gathers and
// scatters.  The group synchronises with a named barrier (or __syncwarp),
// so the groups of one block run independently.
//
// The grid is persistent: a group walks a strided list of the colour's
// cells, K consecutive ordinals per step.  The geometry is stored in the
// order of that walk (a copy of the natural [cell][6][n^3] tensors made at
// setup): per colour class, blocks of K ordinals, each block
// [n][3][K n^2][2] (point, component pair, lane, pair member) so that lane
// t reads three 2-wide words per point (consecutive lanes, consecutive
// pairs: no bank conflicts).  The next step's block is
// fetched by one TMA bulk copy right after the quadrature-point operation
// of the current step (one mbarrier per group, bounded wait).  Summation: 8
// colour launches, first-touch store / add, programmatic dependent launch
// for colours 1..7 (see sf_cont_column.cuh).
//
// The lane-to-cell map, the line each lane owns in the x and y sweeps and
// the strides of the three slabs come from a search of the shared-memory
// bank conflicts of the access patterns for each (n, W, K); slab B2, read
// and written only along y lines and z columns, has a layout of its own.
#include <type_traits>

#include "sf_cont_column.cuh"
#include "sf_device.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"
#include "sf_tma.cuh"

namespace sf {

namespace {

// Shared-memory layout of one slab: entry (x, y, z) of cell k at
// k RS + SX x + SY y + SZ z.
struct SlabLayout {
  int SX, SY, SZ, RS;
};

// W warps per group, K cells per group, GROUPS groups per block, MINB the
// resident-block target handed to the register allocator.  INTER: lane t
// works on cell t % K, line t / K (else cell t / n^2, line t % n^2).  The
// lane with line l = a + n b owns z column (a, b), in the x sweeps the x
// line (y, z) = (a, b), or (b, a) with XS, in the y sweeps the y line
// (x, z) = (a, b), or (b, a) with YS.  Slabs B0 and B1 see x, y and z
// patterns, B2 y and z patterns; each lives in a region of its own.
struct PackParams {
  int W, K, GROUPS, MINB, INTER, XS, YS;
  SlabLayout B0, B1, B2;
};

constexpr PackParams pack_params(int n, int elem)
{
  return elem == 4 ? (n == 2   ? PackParams{1, 8, 4, 1, 0, 0, 0, {1, 2, 5, 20}, {1, 2, 5, 20}, {1, 2, 6, 12}}
                      : n == 3 ? PackParams{2, 7, 2, 1, 0, 0, 0, {1, 3, 9, 59}, {1, 3, 9, 59}, {1, 3, 11, 41}}
                      : n == 4 ? PackParams{1, 2, 4, 1, 0, 0, 0, {1, 4, 19, 176}, {1, 4, 19, 176}, {1, 4, 20, 80}}
                      : n == 5 ? PackParams{4, 5, 1, 7, 1, 1, 0, {1, 5, 33, 173}, {1, 5, 33, 173}, {1, 5, 37, 173}}
                      : n == 6 ? PackParams{7, 6, 1, 1, 0, 0, 0, {1, 7, 42, 508}, {1, 7, 42, 508}, {1, 6, 38, 228}}
                      : n == 7 ? PackParams{5, 3, 1, 1, 1, 1, 0, {1, 7, 65, 459}, {1, 7, 65, 459}, {1, 7, 49, 363}}
                      : n == 8 ? PackParams{2, 1, 2, 1, 0, 1, 0, {67, 8, 1, 533}, {67, 8, 1, 533}, {1, 8, 72, 568}}
                               : PackParams{8, 3, 1, 1, 1, 1, 0, {1, 9, 97, 875}, {1, 9, 97, 875}, {1, 9, 105, 939}})
                   : (n == 2   ? PackParams{1, 8, 4, 1, 0, 0, 0, {1, 2, 5, 20}, {1, 2, 5, 20}, {1, 2, 6, 12}}
                      : n == 3 ? PackParams{2, 7, 2, 1, 0, 0, 0, {1, 3, 18, 121}, {1, 3, 18, 121}, {1, 3, 19, 57}}
                      : n == 4 ? PackParams{1, 2, 4, 1, 0, 0, 0, {1, 4, 19, 152}, {1, 4, 19, 152}, {1, 4, 20, 80}}
                      : n == 5 ? PackParams{4, 5, 1, 1, 0, 0, 0, {1, 5, 25, 253}, {1, 5, 25, 253}, {1, 5, 37, 185}}
                      : n == 6 ? PackParams{7, 6, 1, 1, 0, 0, 0, {1, 7, 42, 508}, {1, 7, 42, 508}, {1, 6, 38, 228}}
                      : n == 7 ? PackParams{5, 3, 1, 1, 0, 0, 0, {1, 7, 49, 695}, {1, 7, 49, 695}, {1, 7, 55, 385}}
                      : n == 8 ? PackParams{2, 1, 2, 1, 0, 0, 0, {1, 9, 72, 1152}, {1, 9, 72, 1152}, {1, 8, 72, 576}}
                               : PackParams{3, 1, 2, 1, 0, 0, 0, {1, 9, 81, 1458}, {1, 9, 81, 1458}, {1, 9, 89, 801}});
}

// every entry of an n^3 slab lands on its own word inside RS
constexpr bool slab_fits(int n, SlabLayout L)
{
  bool seen[4096] = {};
  if (L.RS > 4096) return false;
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        const int i = L.SX * x + L.SY * y + L.SZ * z;
        if (i < 0 || i >= L.RS || seen[i]) return false;
        seen[i] = true;
      }
  return true;
}

template <int N, typename T>
struct LineCfg {
  static constexpr PackParams PP = pack_params(N, (int)sizeof(T));
  static constexpr int W = PP.W, K = PP.K, GROUPS = PP.GROUPS;
  static constexpr int N2 = N * N, N3 = N * N * N;
  static constexpr SlabLayout L0 = PP.B0, L1 = PP.B1, L2 = PP.B2;
  static constexpr int RS = L0.RS + L1.RS + L2.RS; // slab words per cell
  static constexpr int AL = 16 / (int)sizeof(T);   // elements per 16 bytes
  static constexpr int KN2 = K * N2;               // lanes that own a line
  static constexpr int GB = (6 * N * KN2 + AL - 1) / AL * AL; // geometry block of K cells
  static constexpr int GT = 32 * W;                // threads per group
  static constexpr long long GROUP_BYTES =
      ((long long)(GB + K * RS) * (long long)sizeof(T) + 127) / 128 * 128;
  static_assert(KN2 <= GT, "cells do not fit the group");
  static_assert(slab_fits(N, L0) && slab_fits(N, L1) && slab_fits(N, L2), "slab entries overlap");
  static_assert(GB * sizeof(T) < (1u << 20), "geometry block exceeds the mbarrier transaction count");
};

// number of cells of colour `color` and the offset of its first geometry
// block in the walk-ordered layout (elements)
template <int N, typename T>
long long line_color_geometry(const int (&nc)[3], int color, long long *count)
{
  using Cfg = LineCfg<N, T>;
  long long base = 0;
  for (int c = 0;; ++c) {
    const long long cnt = (long long)((nc[0] - (c & 1) + 1) / 2) * ((nc[1] - ((c >> 1) & 1) + 1) / 2) *
                          ((nc[2] - ((c >> 2) & 1) + 1) / 2);
    if (c == color) {
      *count = cnt;
      return base;
    }
    base += (cnt + Cfg::K - 1) / Cfg::K * Cfg::GB;
  }
}

template <int N, typename T>
struct LineArgs {
  EOMat<N, T> S, ST, D, DT;
  // the same tables as (e, o) pairs for packed FP32x2 arithmetic: S, ST, D, DT
  struct {
    float2 eo[N / 2 > 0 ? N / 2 : 1][N / 2 > 0 ? N / 2 : 1];
  } P2[4];
  T w[N];
  const T *__restrict__ x;
  T *__restrict__ y;
  const T *__restrict__ geo;    // this colour's walk-ordered geometry blocks (GB elements each)
  const T *__restrict__ kappa;  // [cell][n^3] or null
  int nc[3];
  int Nx, plane;                // nodes per x line, per z plane
  T aff[3];
  T jxw;                        // mass / convection: cell volume (affine)
  // unstructured meshes: node (x, y, z) of cell e at idx[e n^3 + (z n + y) n + x],
  // umask[e n^2 + column]: keep bits 0..n-1, add bits 16..16+n-1, ucells: the
  // colour's cells in walk order
  const int *__restrict__ idx;
  const unsigned *__restrict__ umask;
  const int *__restrict__ ucells;
  T conv[3];                    // convection: b_d / h_d
  int dirichlet;
  int color, cx, cy, cz, mx, my;
  long long count;              // cells of this colour
  int *err;
  // stride of the walk (K x groups in the grid) decomposed in the colour's
  // (mi, mj, mk) index space: no division inside the loop
  int step_i, step_j, step_k;
};

// out = M in.  In FP32 the even and odd products of output pair i,
// (e[i][j] u+_j, o[i][j] u-_j), run as one packed FP32x2 FMA with the pair
// table P2[WHICH]; the sums and the middle row stay scalar.  FP64 uses the
// scalar even-odd contraction.
template <int N, int SIGN, int WHICH, typename T, typename ARGS>
__device__ __forceinline__ void eo_line(const ARGS &A, const EOMat<N, T> &M, const T (&in)[N], T (&out)[N])
{
  if constexpr (std::is_same<T, float>::value && N >= 2) {
    constexpr int H = N / 2;
    float up[H], um[H];
#pragma unroll
    for (int j = 0; j < H; ++j) {
      up[j] = in[j] + in[N - 1 - j];
      um[j] = in[j] - in[N - 1 - j];
    }
    float2 acc[H];
#pragma unroll
    for (int i = 0; i < H; ++i) acc[i] = make_float2((N % 2 == 1) ? M.mc[i] * in[H] : 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < H; ++j) {
      const float2 u = make_float2(up[j], um[j]);
#pragma unroll
      for (int i = 0; i < H; ++i) acc[i] = __ffma2_rn(A.P2[WHICH].eo[i][j], u, acc[i]);
    }
    float res[N];
#pragma unroll
    for (int i = 0; i < H; ++i) {
      res[i] = acc[i].x + acc[i].y;
      res[N - 1 - i] = SIGN > 0 ? acc[i].x - acc[i].y : acc[i].y - acc[i].x;
    }
    if (N % 2 == 1) {
      float m = SIGN > 0 ? M.mm * in[H] : 0.f;
#pragma unroll
      for (int j = 0; j < H; ++j) m = fmaf(M.mr[j], SIGN > 0 ? up[j] : um[j], m);
      res[H] = m;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) out[i] = res[i];
  } else {
    eo_apply<N, SIGN>(M, in, out);
  }
}

// cell operator of the apply: the Laplacian (div(kappa grad)), the mass
// matrix or the convection form (u, b . grad v); the last two on affine
// meshes (the reference's DO_MASS_MATRIX / DO_CONVECTION variants of the
// cell Laplacian, evaluation_cell_laplacian.h:299-354)
enum { OP_LAPLACE = 0, OP_MASS = 1, OP_CONVECTION = 2 };

// column of an unstructured cell: its node indices and masks
template <int N, typename T>
__device__ __forceinline__ void unstr_column(const LineArgs<N, T> &A, bool valid, long long o, int l, int (&nd)[N],
                                             ColumnMask &m)
{
  constexpr int N2 = N * N, N3 = N * N * N;
  const long long cell = valid ? (long long)__ldg(A.ucells + o) : 0;
  const unsigned u = valid ? __ldg(A.umask + cell * N2 + l) : 0u;
  m.keep = u & 0xffffu;
  m.add = u >> 16;
#pragma unroll
  for (int c = 0; c < N; ++c) nd[c] = valid ? __ldg(A.idx + cell * N3 + c * N2 + l) : 0;
}

template <int N, typename T>
__device__ __forceinline__ void gather_nodes(const T *__restrict__ x, const int (&nd)[N], unsigned keep, T (&v)[N])
{
#pragma unroll
  for (int c = 0; c < N; ++c) v[c] = ((keep >> c) & 1u) ? __ldg(x + nd[c]) : T(0);
}

template <int N, typename T, bool DEFORMED, bool KAPPA, int OPK = OP_LAPLACE, bool UNSTR = false>
__global__ void __launch_bounds__(LineCfg<N, T>::GT * LineCfg<N, T>::GROUPS,
                                  UNSTR && LineCfg<N, T>::PP.MINB > 1 ? LineCfg<N, T>::PP.MINB - 1
                                                                     : LineCfg<N, T>::PP.MINB)
    line_vmult_kernel(const __grid_constant__ LineArgs<N, T> A)
{
  static_assert(!UNSTR || (DEFORMED && !KAPPA && OPK == OP_LAPLACE), "unstructured: deformed Laplacian only");
  using Cfg = LineCfg<N, T>;
  constexpr int N2 = Cfg::N2, N3 = Cfg::N3, K = Cfg::K, W = Cfg::W, GT = Cfg::GT;
  constexpr SlabLayout L0 = Cfg::L0, L1 = Cfg::L1, L2 = Cfg::L2;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw);
  const int grp = threadIdx.x / GT, t = threadIdx.x % GT;
  unsigned char *gbase = smem_raw + 128 + grp * Cfg::GROUP_BYTES;
  uint64_t *bar = bars + grp;

  // Lanes beyond K n^2 repeat the last used lane's line with every store
  // predicated off, so the sweeps carry no divergent branches and their
  // shared-memory addresses coincide with a lane of the same warp (a
  // broadcast, no extra bank conflict).
  const bool used = t < K * N2;
  const int tt = used ? t : K * N2 - 1;
  const int k = Cfg::PP.INTER ? tt % K : tt / N2, l = Cfg::PP.INTER ? tt / K : tt % N2;
  const int a = l % N, b = l / N; // z column (a, b)
  const int xy = Cfg::PP.XS ? b : a, xz = Cfg::PP.XS ? a : b; // x line (y, z)
  const int yx = Cfg::PP.YS ? b : a, yz = Cfg::PP.YS ? a : b; // y line (x, z)
  T *geo_s = reinterpret_cast<T *>(gbase);
  T *B0 = reinterpret_cast<T *>(gbase) + Cfg::GB + k * L0.RS;
  T *B1 = reinterpret_cast<T *>(gbase) + Cfg::GB + K * L0.RS + k * L1.RS;
  T *B2 = reinterpret_cast<T *>(gbase) + Cfg::GB + K * (L0.RS + L1.RS) + k * L2.RS;
  // line bases in each slab (z column stride SZ, x line stride SX, y line stride SY)
  const int zc0 = L0.SX * a + L0.SY * b, xl0 = L0.SY * xy + L0.SZ * xz, yl0 = L0.SX * yx + L0.SZ * yz;
  const int zc1 = L1.SX * a + L1.SY * b, xl1 = L1.SY * xy + L1.SZ * xz, yl1 = L1.SX * yx + L1.SZ * yz;
  const int zc2 = L2.SX * a + L2.SY * b, yl2 = L2.SX * yx + L2.SZ * yz;
  const int plane = A.plane;
  const int toff = b * A.Nx + a;  // node (a, b, 0) relative to the cell's node (0, 0, 0)

  const long long ng = (long long)gridDim.x * Cfg::GROUPS;
  const long long gid = (long long)blockIdx.x * Cfg::GROUPS + grp;
  const long long step = ng * K;
  constexpr uint32_t geo_bytes = (uint32_t)(Cfg::GB * sizeof(T));
  long long blk = gid; // geometry block of the current step (ordinal / K)

  // position (mi, mj, mk) of this lane's first cell in the colour's index
  // space; later cells follow by a division-free strided walk
  long long o = gid * K + k;
  int mi = 0, mj = 0, mk = 0;
  if (!UNSTR && o < A.count) {
    const unsigned uo = (unsigned)o, umx = (unsigned)A.mx, umy = (unsigned)A.my;
    const unsigned q = uo / umx;
    mi = int(uo - q * umx);
    mk = int(q / umy);
    mj = int(q - unsigned(mk) * umy);
  }
  const bool dir = A.dirichlet != 0;
  uint64_t pol = 0;
  if (DEFORMED) {
    pol = l2_policy_evict_first();
    if (t == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
      if (gid * K < A.count) {
        mbar_arrive_expect_tx(bar, geo_bytes);
        tma_load_1d_hint(geo_s, A.geo + blk * Cfg::GB, geo_bytes, bar, pol);
      }
    }
    cell_group_sync<W, Cfg::GROUPS>(grp);
  }
  pdl_trigger();
  uint32_t parity = 0;
  bool y_ready = false;

  // the current cell's column: bookkeeping, node base, gathered x; the next
  // cell's column is fetched during the current cell's integration sweeps
  bool valid = used && o < A.count;
  ColumnMask msk;
  long long nb = 0;
  int cn[N]; // unstructured: the column's node indices
  T xv[N];
  if constexpr (UNSTR) {
    unstr_column<N, T>(A, valid, o, l, cn, msk);
    gather_nodes<N, T>(A.x, cn, msk.keep, xv);
  } else {
    msk = column_mask<N>(a, b, 2 * mi + A.cx, 2 * mj + A.cy, 2 * mk + A.cz, A.nc, A.color, dir, valid);
    nb = cell_node_base<N>(2 * mi + A.cx, 2 * mj + A.cy, 2 * mk + A.cz, A.Nx, plane) + toff;
    gather_column<N, T>(A.x + nb, plane, msk.keep, xv);
  }

  for (long long o0 = gid * K; o0 < A.count; o0 += step, o += step) {
    const int ci = 2 * mi + A.cx, cj = 2 * mj + A.cy, ck = 2 * mk + A.cz;
    // this lane's next cell
    int ni = mi + A.step_i, nj = mj + A.step_j, nk = mk + A.step_k;
    if (ni >= A.mx) {
      ni -= A.mx;
      ++nj;
    }
    if (nj >= A.my) {
      nj -= A.my;
      ++nk;
    }
    T v[N], g[N], gz[N];
    ColumnMask nmsk;
    long long nnb = 0;
    int nn[N];
    if constexpr (UNSTR) {
      // the next cell's node indices and masks arrive during this step's
      // sweeps; its x column is gathered after the quadrature-point operation
      unstr_column<N, T>(A, used && o + step < A.count, o + step, l, nn, nmsk);
    }
    // ---- sweeps S_z (gathered column), S_x, S_y and D_y ----
    eo_line<N, 1, 0>(A, A.S, xv, v);
#pragma unroll
    for (int c = 0; c < N; ++c)
      if (used) B0[zc0 + L0.SZ * c] = v[c];
    cell_group_sync<W, Cfg::GROUPS>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[xl0 + L0.SX * m];
    eo_line<N, 1, 0>(A, A.S, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (used) B0[xl0 + L0.SX * m] = v[m];
    cell_group_sync<W, Cfg::GROUPS>(grp);
    if constexpr (OPK != OP_LAPLACE) {
      // ---- y lines: S_y, the weights JxW w at the Gauss points ----
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B0[yl0 + L0.SY * m];
      eo_line<N, 1, 0>(A, A.S, v, v);
      const T wxz = A.jxw * A.w[yx] * A.w[yz];
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] *= wxz * A.w[m];
      if constexpr (OPK == OP_MASS) {
        eo_line<N, 1, 1>(A, A.ST, v, v);
#pragma unroll
        for (int m = 0; m < N; ++m)
          if (used) B1[yl1 + L1.SY * m] = v[m];
      } else {
        // convection: r = u JxW w stays in B0 for the x and z lines; the y
        // term b_y / h_y D^T r goes to B1
        eo_line<N, -1, 3>(A, A.DT, v, g);
#pragma unroll
        for (int m = 0; m < N; ++m) {
          if (used) B0[yl0 + L0.SY * m] = v[m];
          if (used) B1[yl1 + L1.SY * m] = A.conv[1] * g[m];
        }
      }
      cell_group_sync<W, Cfg::GROUPS>(grp);
      if constexpr (OPK == OP_CONVECTION) {
        // ---- x lines: + b_x / h_x D^T r ----
#pragma unroll
        for (int m = 0; m < N; ++m) v[m] = B0[xl0 + L0.SX * m];
        eo_line<N, -1, 3>(A, A.DT, v, g);
#pragma unroll
        for (int m = 0; m < N; ++m) {
          const T s = fma(A.conv[0], g[m], B1[xl1 + L1.SX * m]);
          if (used) B1[xl1 + L1.SX * m] = s;
        }
        cell_group_sync<W, Cfg::GROUPS>(grp);
      }
      // loads overlapped with the remaining sweeps: the y values this column
      // adds to, and the next cell's x column
      const bool nvalid = used && o + step < A.count;
      if (!y_ready) {
        pdl_wait();
        y_ready = true;
      }
      T yo[N];
      load_column_sums<N, T>(A.y + nb, plane, msk.add, yo);
      const ColumnMask nmsk =
          column_mask<N>(a, b, 2 * ni + A.cx, 2 * nj + A.cy, 2 * nk + A.cz, A.nc, A.color, dir, nvalid);
      const long long nnb = cell_node_base<N>(2 * ni + A.cx, 2 * nj + A.cy, 2 * nk + A.cz, A.Nx, plane) + toff;
      gather_column<N, T>(A.x + nnb, plane, nmsk.keep, xv);
      if constexpr (OPK == OP_CONVECTION) {
        // ---- z columns: + b_z / h_z D^T r, then S_z^T ----
#pragma unroll
        for (int m = 0; m < N; ++m) v[m] = B0[zc0 + L0.SZ * m];
        eo_line<N, -1, 3>(A, A.DT, v, g);
#pragma unroll
        for (int m = 0; m < N; ++m) v[m] = fma(A.conv[2], g[m], B1[zc1 + L1.SZ * m]);
        eo_line<N, 1, 1>(A, A.ST, v, v);
#pragma unroll
        for (int m = 0; m < N; ++m)
          if (used) B1[zc1 + L1.SZ * m] = v[m];
        cell_group_sync<W, Cfg::GROUPS>(grp);
#pragma unroll
        for (int m = 0; m < N; ++m) v[m] = B1[yl1 + L1.SY * m];
        eo_line<N, 1, 1>(A, A.ST, v, v);
#pragma unroll
        for (int m = 0; m < N; ++m)
          if (used) B1[yl1 + L1.SY * m] = v[m];
        cell_group_sync<W, Cfg::GROUPS>(grp);
      }
      // ---- x lines: S_x^T ----
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B1[xl1 + L1.SX * m];
      eo_line<N, 1, 1>(A, A.ST, v, v);
#pragma unroll
      for (int m = 0; m < N; ++m)
        if (used) B1[xl1 + L1.SX * m] = v[m];
      cell_group_sync<W, Cfg::GROUPS>(grp);
      // ---- z column: S_z^T (mass), scatter ----
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B1[zc1 + L1.SZ * m];
      if constexpr (OPK == OP_MASS) eo_line<N, 1, 1>(A, A.ST, v, v);
      if (valid) store_column<N, T>(A.y + nb, A.x + nb, plane, msk.keep, v, yo);
      msk = nmsk;
      nb = nnb;
      valid = nvalid;
      mi = ni;
      mj = nj;
      mk = nk;
      continue;
    } else {
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[yl0 + L0.SY * m];
    eo_line<N, 1, 0>(A, A.S, v, v);
    eo_line<N, -1, 2>(A, A.D, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (used) B1[yl1 + L1.SY * m] = v[m];
      if (used) B2[yl2 + L2.SY * m] = g[m];
    }
    cell_group_sync<W, Cfg::GROUPS>(grp);
    // ---- D_x into B0; D_z stays in registers (same thread, same column) ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[xl1 + L1.SX * m];
    eo_line<N, -1, 2>(A, A.D, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (used) B0[xl0 + L0.SX * m] = g[m];
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[zc1 + L1.SZ * m];
    eo_line<N, -1, 2>(A, A.D, v, gz);
    cell_group_sync<W, Cfg::GROUPS>(grp);
    // ---- quadrature points of column (a,b) ----
    const bool more = o0 + step < A.count;
    if (DEFORMED) {
      mbar_wait(bar, parity, A.err);
      parity ^= 1;
      // the next step's copies are issued after the group barrier below;
      // announce their bytes now (the barrier is already in its next phase)
      if (t == 0 && more) mbar_arrive_expect_tx(bar, geo_bytes);
    }
    T tz[N];
    {
      const T wab = A.w[a] * A.w[b];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const int s = zc0 + L0.SZ * c;
        const T gx = B0[s], gy = B2[zc2 + L2.SZ * c];
        T tx, ty, tzc;
        if (DEFORMED) {
          // component pairs (xx, yy), (zz, xy), (xz, yz) of point c of lane tt:
          // three 2-wide loads, consecutive lanes on consecutive pairs
          using T2 = typename std::conditional<sizeof(T) == 8, double2, float2>::type;
          const T2 *Gq = reinterpret_cast<const T2 *>(geo_s) + c * 3 * Cfg::KN2 + tt;
          const T2 p0 = Gq[0], p1 = Gq[Cfg::KN2], p2 = Gq[2 * Cfg::KN2];
          const T g0 = p0.x, g1 = p0.y, g2 = p1.x, g3 = p1.y, g4 = p2.x, g5 = p2.y;
          tx = gx * g0 + gy * g3 + gz[c] * g4;
          ty = gx * g3 + gy * g1 + gz[c] * g5;
          tzc = gx * g4 + gy * g5 + gz[c] * g2;
        } else {
          const T wq = wab * A.w[c];
          tx = gx * (A.aff[0] * wq);
          ty = gy * (A.aff[1] * wq);
          tzc = gz[c] * (A.aff[2] * wq);
        }
        if (KAPPA) {
          const long long cell = ((long long)ck * A.nc[1] + cj) * A.nc[0] + ci;
          const T kq = valid ? __ldg(A.kappa + cell * N3 + c * N2 + l) : T(0);
          tx *= kq;
          ty *= kq;
          tzc *= kq;
        }
        if (used) B0[s] = tx;
        if (used) B2[zc2 + L2.SZ * c] = ty;
        tz[c] = tzc;
      }
      eo_line<N, -1, 3>(A, A.DT, tz, g);
#pragma unroll
      for (int c = 0; c < N; ++c)
        if (used) B1[zc1 + L1.SZ * c] = g[c];
    }
    if (DEFORMED) fence_proxy_async_smem();
    cell_group_sync<W, Cfg::GROUPS>(grp);
    // geometry buffers free: fetch the next step's blocks
    const bool nvalid = used && o + step < A.count;
    blk += ng;
    if (DEFORMED && more && t == 0) tma_load_1d_hint(geo_s, A.geo + blk * Cfg::GB, geo_bytes, bar, pol);
    // loads overlapped with the integration sweeps: the y values this
    // column adds to, and the next cell's x column
    if (!y_ready) {
      pdl_wait();
      y_ready = true;
    }
    T yo[N];
    if constexpr (UNSTR) {
#pragma unroll
      for (int c = 0; c < N; ++c) yo[c] = ((msk.add >> c) & 1u) ? A.y[cn[c]] : T(0);
      gather_nodes<N, T>(A.x, nn, nmsk.keep, xv);
    } else {
      load_column_sums<N, T>(A.y + nb, plane, msk.add, yo);
      nmsk = column_mask<N>(a, b, 2 * ni + A.cx, 2 * nj + A.cy, 2 * nk + A.cz, A.nc, A.color, dir, nvalid);
      nnb = cell_node_base<N>(2 * ni + A.cx, 2 * nj + A.cy, 2 * nk + A.cz, A.Nx, plane) + toff;
      gather_column<N, T>(A.x + nnb, plane, nmsk.keep, xv);
    }
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[xl0 + L0.SX * m];
    eo_line<N, -1, 3>(A, A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const T s = B1[xl1 + L1.SX * m] + g[m];
      if (used) B1[xl1 + L1.SX * m] = s;
    }
    cell_group_sync<W, Cfg::GROUPS>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B2[yl2 + L2.SY * m];
    eo_line<N, -1, 3>(A, A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) g[m] += B1[yl1 + L1.SY * m];
    eo_line<N, 1, 1>(A, A.ST, g, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (used) B1[yl1 + L1.SY * m] = v[m];
    cell_group_sync<W, Cfg::GROUPS>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[xl1 + L1.SX * m];
    eo_line<N, 1, 1>(A, A.ST, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (used) B1[xl1 + L1.SX * m] = v[m];
    cell_group_sync<W, Cfg::GROUPS>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[zc1 + L1.SZ * m];
    eo_line<N, 1, 1>(A, A.ST, v, v);
    // ---- scatter the z column: first colour stores, later ones add ----
    if constexpr (UNSTR) {
      if (valid) {
#pragma unroll
        for (int c = 0; c < N; ++c) A.y[cn[c]] = ((msk.keep >> c) & 1u) ? v[c] + yo[c] : __ldg(A.x + cn[c]);
      }
#pragma unroll
      for (int c = 0; c < N; ++c) cn[c] = nn[c];
    } else {
      if (valid) store_column<N, T>(A.y + nb, A.x + nb, plane, msk.keep, v, yo);
    }
    msk = nmsk;
    nb = nnb;
    valid = nvalid;
    mi = ni;
    mj = nj;
    mk = nk;
    }
  }
  if (!y_ready) pdl_wait();
}

// walk-ordered copy of one colour's geometry: entry (blk, c, pr, t, h) =
// component e = 2 pr + h at point (l, c) of the colour's cell with ordinal
// blk K + k, (k, l) the cell and line of lane t; zero past the colour's
// last cell and in the block padding
template <int N, typename T>
__global__ void line_pack_geometry_kernel(const double *__restrict__ G, long long gstride, T *__restrict__ out,
                                          long long total, long long count, int nc0, int nc1, int cx, int cy,
                                          int cz, int mx, int my, const int *__restrict__ cells)
{
  using Cfg = LineCfg<N, T>;
  constexpr int KN2 = Cfg::KN2, N2 = Cfg::N2;
  const long long str = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += str) {
    const long long blk = i / Cfg::GB;
    const int r = int(i - blk * Cfg::GB);
    T v = T(0);
    if (r < 6 * N * KN2) {
      // r = ((c 3 + pr) KN2 + tl) 2 + h holds component e = 2 pr + h
      const int h = r & 1, tl = (r >> 1) % KN2, cp = (r >> 1) / KN2;
      const int c = cp / 3, e = 2 * (cp - 3 * c) + h;
      const int k = Cfg::PP.INTER ? tl % Cfg::K : tl / N2, l = Cfg::PP.INTER ? tl / Cfg::K : tl % N2;
      const long long o = blk * Cfg::K + k;
      if (o < count) {
        long long cell;
        if (cells) {
          cell = cells[o];
        } else {
          const long long q = o / mx, mk = q / my;
          const long long mi = o - q * mx, mj = q - mk * my;
          cell = ((2 * mk + cz) * nc1 + (2 * mj + cy)) * nc0 + (2 * mi + cx);
        }
        v = T(G[cell * gstride + (long long)e * Cfg::N3 + c * N2 + l]);
      }
    }
    out[i] = v;
  }
}

template <int N, typename T>
int line_pack_impl(sf_op *op, DevBuf &buf)
{
  using Cfg = LineCfg<N, T>;
  int nc[3];
  for (int d = 0; d < 3; ++d) nc[d] = op->desc.n_cells[d];
  long long cnt7 = 0;
  const long long total = line_color_geometry<N, T>(nc, 7, &cnt7) + (cnt7 + Cfg::K - 1) / Cfg::K * Cfg::GB;
  const size_t bytes = (size_t)total * sizeof(T);
  if (buf.bytes != bytes) {
    const int e = buf.alloc(bytes);
    if (e != SF_OK) return e;
  }
  for (int color = 0; color < 8; ++color) {
    long long count = 0;
    const long long base = line_color_geometry<N, T>(nc, color, &count);
    const long long n = (count + Cfg::K - 1) / Cfg::K * Cfg::GB;
    if (n == 0) continue;
    const int cx = color & 1, cy = (color >> 1) & 1, cz = (color >> 2) & 1;
    const int mx = (nc[0] - cx + 1) / 2, my = (nc[1] - cy + 1) / 2;
    const long long blocks = stream_grid(n, 256, 32);
    line_pack_geometry_kernel<N, T><<<(unsigned)blocks, 256>>>((const double *)op->geo64.ptr, op->geo_stride,
                                                              (T *)buf.ptr + base, n, count, nc[0], nc[1], cx,
                                                              cy, cz, mx, my, nullptr);
    SF_CUDA_TRY(cudaGetLastError());
  }
  return SF_OK;
}

// unstructured meshes: the geometry of each colour's cells in walk order
template <int N, typename T>
int line_unstr_pack_impl(sf_op *op, DevBuf &buf)
{
  using Cfg = LineCfg<N, T>;
  const sf_unstructured &M = *op->unstr;
  long long total = 0;
  for (size_t c = 0; c + 1 < M.color_start.size(); ++c)
    total += (M.color_start[c + 1] - M.color_start[c] + Cfg::K - 1) / Cfg::K * Cfg::GB;
  const size_t bytes = (size_t)total * sizeof(T);
  if (buf.bytes != bytes) {
    const int e = buf.alloc(bytes);
    if (e != SF_OK) return e;
  }
  long long base = 0;
  for (size_t c = 0; c + 1 < M.color_start.size(); ++c) {
    const long long count = M.color_start[c + 1] - M.color_start[c];
    const long long n = (count + Cfg::K - 1) / Cfg::K * Cfg::GB;
    if (n == 0) continue;
    const long long blocks = stream_grid(n, 256, 32);
    line_pack_geometry_kernel<N, T><<<(unsigned)blocks, 256>>>(
        (const double *)op->geo64.ptr, op->geo_stride, (T *)buf.ptr + base, n, count, 1, 1, 0, 0, 0, 1, 1,
        (const int *)M.cells.ptr + M.color_start[c]);
    SF_CUDA_TRY(cudaGetLastError());
    base += n;
  }
  return SF_OK;
}

// the (e, o) pair tables of the FP32 contractions
template <int N, typename T>
void fill_pairs(LineArgs<N, T> &A)
{
  const EOMat<N, T> *ms[4] = {&A.S, &A.ST, &A.D, &A.DT};
  for (int w = 0; w < 4; ++w)
    for (int i = 0; i < N / 2; ++i)
      for (int j = 0; j < N / 2; ++j) A.P2[w].eo[i][j] = make_float2(float(ms[w]->e[i][j]), float(ms[w]->o[i][j]));
}

template <int N, typename T>
int line_unstr_vmult_impl(const sf_op *op, const T *x, T *y, cudaStream_t st)
{
  using Cfg = LineCfg<N, T>;
  const sf_unstructured &M = *op->unstr;
  LineArgs<N, T> A{};
  const Shape1D &s = op->shape;
  A.S = eo_of<N, T>(s.S, false);
  A.ST = eo_of<N, T>(s.S, true);
  A.D = eo_of<N, T>(s.D, false);
  A.DT = eo_of<N, T>(s.D, true);
  fill_pairs<N, T>(A);
  for (int i = 0; i < N; ++i) A.w[i] = T(s.wq[i]);
  A.x = x;
  A.y = y;
  A.err = (int *)op->dev_err.ptr;
  A.idx = (const int *)M.idx.ptr;
  A.umask = (const unsigned *)M.masks.ptr;
  A.mx = A.my = 1;
  const T *geo = (const T *)(sizeof(T) == 8 ? op->geoLine64.ptr : op->geoLine32.ptr);
  if (!geo) {
    set_error("line kernel: walk-ordered geometry missing");
    return SF_ERR_STATE;
  }
  void (*kern)(const LineArgs<N, T>) = line_vmult_kernel<N, T, true, false, OP_LAPLACE, true>;
  const size_t smem = 128 + size_t(Cfg::GROUPS) * Cfg::GROUP_BYTES;
  const int threads = Cfg::GT * Cfg::GROUPS;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  int per_sm = 0;
  SF_RET_IF(resident_blocks_per_sm((const void *)kern, threads, smem, &per_sm));
  int n_sm = 0, dev = 0;
  SF_CUDA_TRY(cudaGetDevice(&dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  long long base = 0;
  for (size_t c = 0; c + 1 < M.color_start.size(); ++c) {
    A.count = M.color_start[c + 1] - M.color_start[c];
    if (A.count == 0) continue;
    A.ucells = (const int *)M.cells.ptr + M.color_start[c];
    A.geo = geo + base;
    base += (A.count + Cfg::K - 1) / Cfg::K * Cfg::GB;
    A.color = (int)c;
    const long long steps = (A.count + Cfg::K - 1) / Cfg::K;
    const long long blocks =
        std::min<long long>((steps + Cfg::GROUPS - 1) / Cfg::GROUPS, (long long)per_sm * n_sm);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = c > 0 ? 1 : 0; // colour 0 reads x behind its producer
    SF_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, A));
  }
  return SF_OK;
}

template <int N, typename T>
int line_vmult_impl(const sf_op *op, const T *x, T *y, cudaStream_t st)
{
  if (op->desc.kind == SF_OP_LAPLACE_UNSTRUCTURED) return line_unstr_vmult_impl<N, T>(op, x, y, st);
  using Cfg = LineCfg<N, T>;
  LineArgs<N, T> A{};
  const Shape1D &s = op->shape;
  A.S = eo_of<N, T>(s.S, false);
  A.ST = eo_of<N, T>(s.S, true);
  A.D = eo_of<N, T>(s.D, false);
  A.DT = eo_of<N, T>(s.D, true);
  fill_pairs<N, T>(A);
  for (int i = 0; i < N; ++i) A.w[i] = T(s.wq[i]);
  for (int d = 0; d < 3; ++d) A.nc[d] = op->desc.n_cells[d];
  A.Nx = (N - 1) * A.nc[0] + 1;
  A.plane = A.Nx * ((N - 1) * A.nc[1] + 1);
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  for (int d = 0; d < 3; ++d) A.aff[d] = T(jxw / (op->h[d] * op->h[d]));
  A.jxw = T(jxw);
  for (int d = 0; d < 3; ++d) A.conv[d] = T(op->desc.velocity[d] / op->h[d]);
  A.dirichlet = op->desc.dirichlet;
  A.x = x;
  A.y = y;
  A.err = (int *)op->dev_err.ptr;
  const bool deformed = op->deformed, kap = op->has_kappa;
  const T *geo = (const T *)(sizeof(T) == 8 ? op->geoLine64.ptr : op->geoLine32.ptr);
  A.kappa = (const T *)(sizeof(T) == 8 ? op->kap64.ptr : op->kap32.ptr);
  if (deformed && !geo) {
    set_error("line kernel: walk-ordered geometry missing");
    return SF_ERR_STATE;
  }
  if (kap && !A.kappa) {
    set_error("line kernel: coefficient missing");
    return SF_ERR_STATE;
  }
  const int kind = op->desc.kind;
  if ((kind == SF_OP_MASS || kind == SF_OP_CONVECTION) && (deformed || kap)) {
    set_error("mass and convection operators: affine meshes without a coefficient only");
    return SF_ERR_UNSUPPORTED;
  }
  void (*kern)(const LineArgs<N, T>) =
      kind == SF_OP_MASS         ? line_vmult_kernel<N, T, false, false, OP_MASS>
      : kind == SF_OP_CONVECTION ? line_vmult_kernel<N, T, false, false, OP_CONVECTION>
      : deformed ? (kap ? line_vmult_kernel<N, T, true, true> : line_vmult_kernel<N, T, true, false>)
                 : (kap ? line_vmult_kernel<N, T, false, true> : line_vmult_kernel<N, T, false, false>);
  const size_t smem = 128 + size_t(Cfg::GROUPS) * Cfg::GROUP_BYTES;
  const int threads = Cfg::GT * Cfg::GROUPS;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  int per_sm = 0;
  SF_RET_IF(resident_blocks_per_sm((const void *)kern, threads, smem, &per_sm));
  int n_sm = 0, dev = 0;
  SF_CUDA_TRY(cudaGetDevice(&dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  for (int color = 0; color < 8; ++color) {
    A.color = color;
    A.cx = color & 1;
    A.cy = (color >> 1) & 1;
    A.cz = (color >> 2) & 1;
    A.mx = (A.nc[0] - A.cx + 1) / 2;
    A.my = (A.nc[1] - A.cy + 1) / 2;
    const long long gbase = line_color_geometry<N, T>(A.nc, color, &A.count);
    A.geo = deformed ? geo + gbase : nullptr;
    if (A.count == 0) continue;
    const long long steps = (A.count + Cfg::K - 1) / Cfg::K;
    const long long blocks =
        std::min<long long>((steps + Cfg::GROUPS - 1) / Cfg::GROUPS, (long long)per_sm * n_sm);
    const long long stride = blocks * Cfg::GROUPS * Cfg::K;
    A.step_i = int(stride % A.mx);
    A.step_j = int((stride / A.mx) % A.my);
    A.step_k = int(stride / ((long long)A.mx * A.my));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = color > 0 ? 1 : 0; // colour 0 reads x behind its producer
    SF_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, A));
  }
  return SF_OK;
}

template <int N>
int line_vmult_n(const sf_op *op, int prec, const void *x, void *y, cudaStream_t st)
{
  if (prec == SF_FP64) return line_vmult_impl<N, double>(op, (const double *)x, (double *)y, st);
  return line_vmult_impl<N, float>(op, (const float *)x, (float *)y, st);
}

template <int N>
int line_pack_n(sf_op *op, int prec)
{
  if (op->unstr) {
    if (prec == SF_FP64) return line_unstr_pack_impl<N, double>(op, op->geoLine64);
    return line_unstr_pack_impl<N, float>(op, op->geoLine32);
  }
  if (prec == SF_FP64) return line_pack_impl<N, double>(op, op->geoLine64);
  return line_pack_impl<N, float>(op, op->geoLine32);
}

} // namespace

int pack_line_geometry(sf_op *op, int prec)
{
  switch (op->n) {
  case 2: return line_pack_n<2>(op, prec);
  case 3: return line_pack_n<3>(op, prec);
  case 4: return line_pack_n<4>(op, prec);
  case 5: return line_pack_n<5>(op, prec);
  case 6: return line_pack_n<6>(op, prec);
  case 7: return line_pack_n<7>(op, prec);
  case 8: return line_pack_n<8>(op, prec);
  case 9: return line_pack_n<9>(op, prec);
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;
  }
}

int launch_cont_vmult_line(const sf_op *op, int prec, const void *x, void *y, cudaStream_t st)
{
  switch (op->n) {
  case 2: return line_vmult_n<2>(op, prec, x, y, st);
  case 3: return line_vmult_n<3>(op, prec, x, y, st);
  case 4: return line_vmult_n<4>(op, prec, x, y, st);
  case 5: return line_vmult_n<5>(op, prec, x, y, st);
  case 6: return line_vmult_n<6>(op, prec, x, y, st);
  case 7: return line_vmult_n<7>(op, prec, x, y, st);
  case 8: return line_vmult_n<8>(op, prec, x, y, st);
  case 9: return line_vmult_n<9>(op, prec, x, y, st);
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;
  }
}

} // namespace sf
