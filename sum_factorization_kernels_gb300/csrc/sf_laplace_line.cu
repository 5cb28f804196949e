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
// cells, K consecutive ordinals per step.  The next step's K geometry blocks
// are fetched by TMA bulk copies right after the quadrature-point operation
// of the current step (one mbarrier per group, bounded wait).  Summation: 8
// colour launches, first-touch store / add, programmatic dependent launch
// for colours 1..7 (see sf_cont_column.cuh).
//
// The slab paddings (P1, P2, Q1, Q2, per-cell skews) come from a search of
// the shared-memory bank conflicts of the access patterns for each (n, W,
// K); slab B2, read and written only along y lines and z columns, lives in
// its own region with a layout that is conflict-free for those two patterns.
#include "sf_cont_column.cuh"
#include "sf_device.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"
#include "sf_tma.cuh"

namespace sf {

namespace {

// W warps per group, K cells per group, GROUPS groups per block; slab
// index (a, b, c) = a + P1 b + P2 c for slabs B0 and B1 (which see x, y and
// z line patterns), SKEW pads their per-cell region; slab B2 (y and z
// patterns only) has its own layout a + Q1 b + Q2 c and per-cell skew SKEW2
// in a separate region; GPAD pads the per-cell geometry block in shared
// memory (elements); MINB is the resident-block target handed to the
// register allocator.
struct PackParams {
  int W, K, GROUPS, P1, P2, SKEW, GPAD, MINB, Q1, Q2, SKEW2;
};

constexpr PackParams pack_params(int n, int elem)
{
  return elem == 4 ? (n == 2   ? PackParams{1, 8, 4, 2, 5, 0, 4, 1, 2, 6, 0}
                      : n == 3 ? PackParams{2, 7, 2, 3, 9, 5, 4, 1, 3, 11, 8}
                      : n == 4 ? PackParams{1, 2, 4, 4, 19, 24, 16, 1, 4, 20, 0}
                      : n == 5 ? PackParams{4, 5, 2, 5, 25, 3, 12, 4, 5, 37, 0}
                      : n == 6 ? PackParams{7, 6, 1, 7, 42, 4, 20, 1, 6, 38, 0}
                      : n == 7 ? PackParams{5, 3, 1, 7, 56, 1, 0, 1, 7, 52, 5}
                      : n == 8 ? PackParams{2, 1, 2, 9, 72, 0, 0, 1, 8, 72, 0}
                               : PackParams{8, 3, 1, 9, 81, 7, 0, 1, 9, 85, 20})
                   : (n == 2   ? PackParams{1, 8, 4, 2, 5, 0, 4, 1, 2, 6, 0}
                      : n == 3 ? PackParams{2, 7, 2, 3, 18, 13, 8, 1, 3, 19, 0}
                      : n == 4 ? PackParams{1, 2, 4, 4, 19, 0, 0, 1, 4, 20, 0}
                      : n == 5 ? PackParams{4, 5, 1, 5, 25, 3, 0, 1, 5, 37, 0}
                      : n == 6 ? PackParams{7, 6, 1, 7, 42, 4, 4, 1, 6, 38, 0}
                      : n == 7 ? PackParams{5, 3, 1, 7, 49, 9, 0, 1, 7, 55, 0}
                      : n == 8 ? PackParams{2, 1, 2, 9, 72, 0, 0, 1, 8, 72, 0}
                               : PackParams{3, 1, 2, 9, 81, 0, 0, 1, 9, 89, 0});
}

template <int N, typename T>
struct LineCfg {
  static constexpr PackParams PP = pack_params(N, (int)sizeof(T));
  static constexpr int W = PP.W, K = PP.K, GROUPS = PP.GROUPS, P1 = PP.P1, P2 = PP.P2;
  static constexpr int N2 = N * N, N3 = N * N * N;
  static constexpr int Q1 = PP.Q1, Q2 = PP.Q2;
  static constexpr int SLAB = P2 * N;              // elements per slab B0, B1
  static constexpr int RS = 2 * SLAB + PP.SKEW;    // B0 + B1 region per cell
  static constexpr int RS2 = Q2 * N + PP.SKEW2;    // B2 region per cell
  static constexpr int AL = 16 / (int)sizeof(T);   // elements per 16 bytes
  static constexpr int GEO = (6 * N3 + 3) / 4 * 4; // geometry block in global memory
  static constexpr int GS = GEO + PP.GPAD;         // geometry block in shared memory
  static constexpr int GT = 32 * W;                // threads per group
  static constexpr long long GROUP_BYTES =
      ((long long)K * (GS + RS + RS2) * (long long)sizeof(T) + 127) / 128 * 128;
  static_assert(K * N2 <= GT, "cells do not fit the group");
  static_assert((P1 + 1) * (N - 1) < P2, "slab padding overlaps");
  static_assert((Q1 + 1) * (N - 1) < Q2 && Q1 >= N, "B2 slab padding overlaps");
  static_assert(GS % AL == 0, "geometry blocks must stay 16-byte aligned");
};

template <int N, typename T>
struct LineArgs {
  EOMat<N, T> S, ST, D, DT;
  T w[N];
  const T *__restrict__ x;
  T *__restrict__ y;
  const T *__restrict__ geo;    // natural layout [cell][6][n^3], block GEO elements
  const T *__restrict__ kappa;  // [cell][n^3] or null
  int nc[3];
  int Nx, plane;                // nodes per x line, per z plane
  T aff[3];
  int dirichlet;
  int color, cx, cy, cz, mx, my;
  long long count;              // cells of this colour
  int *err;
  // stride of the walk (K x groups in the grid) decomposed in the colour's
  // (mi, mj, mk) index space: no division inside the loop
  int step_i, step_j, step_k;
};

template <int N, typename T, bool DEFORMED, bool KAPPA>
__global__ void __launch_bounds__(LineCfg<N, T>::GT * LineCfg<N, T>::GROUPS, LineCfg<N, T>::PP.MINB)
    line_vmult_kernel(const __grid_constant__ LineArgs<N, T> A)
{
  using Cfg = LineCfg<N, T>;
  constexpr int N2 = Cfg::N2, N3 = Cfg::N3, K = Cfg::K, W = Cfg::W, GT = Cfg::GT;
  constexpr int P1 = Cfg::P1, P2 = Cfg::P2, SLAB = Cfg::SLAB, Q1 = Cfg::Q1, Q2 = Cfg::Q2;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw);
  const int grp = threadIdx.x / GT, t = threadIdx.x % GT;
  unsigned char *gbase = smem_raw + 128 + grp * Cfg::GROUP_BYTES;
  uint64_t *bar = bars + grp;

  // Lanes beyond K n^2 run line 0 of cell 0 with every store predicated
  // off, so the sweeps carry no divergent branches.
  const bool used = t < K * N2;
  const int tt = used ? t : 0;
  const int k = tt / N2, l = tt % N2;
  const int a = l % N, b = l / N; // z column (a,b) / y line (a,c=b) / x line (b'=a, c'=b)
  T *geo_s = reinterpret_cast<T *>(gbase) + k * Cfg::GS;
  T *B0 = reinterpret_cast<T *>(gbase) + K * Cfg::GS + k * Cfg::RS;
  T *B1 = B0 + SLAB;
  T *B2 = reinterpret_cast<T *>(gbase) + K * (Cfg::GS + Cfg::RS) + k * Cfg::RS2;
  const int zc = a + P1 * b;      // z column base
  const int xl = P1 * a + P2 * b; // x line (b'=a, c'=b) base, stride 1
  const int yl = a + P2 * b;      // y line (a, c=b) base, stride P1
  const int zc2 = a + Q1 * b;     // the same z column in B2, stride Q2
  const int yl2 = a + Q2 * b;     // the same y line in B2, stride Q1
  const int plane = A.plane;
  const int toff = b * A.Nx + a;  // node (a, b, 0) relative to the cell's node (0, 0, 0)

  const long long ng = (long long)gridDim.x * Cfg::GROUPS;
  const long long gid = (long long)blockIdx.x * Cfg::GROUPS + grp;
  const long long step = ng * K;
  constexpr uint32_t geo_bytes = (uint32_t)(Cfg::GEO * sizeof(T));

  // position (mi, mj, mk) of this lane's first cell in the colour's index
  // space; later cells follow by a division-free strided walk
  long long o = gid * K + k;
  int mi = 0, mj = 0, mk = 0;
  if (o < A.count) {
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
      if (gid * K < A.count)
        mbar_arrive_expect_tx(bar, geo_bytes * (uint32_t)min((long long)K, A.count - gid * K));
      fence_mbar_init();
    }
    cell_group_sync<W>(grp);
    if (used && l == 0 && o < A.count) {
      const long long cell = ((long long)(2 * mk + A.cz) * A.nc[1] + (2 * mj + A.cy)) * A.nc[0] + (2 * mi + A.cx);
      tma_load_1d_hint(geo_s, A.geo + cell * Cfg::GEO, geo_bytes, bar, pol);
    }
  }
  pdl_trigger();
  uint32_t parity = 0;
  bool y_ready = false;

  // the current cell's column: bookkeeping, node base, gathered x; the next
  // cell's column is fetched during the current cell's integration sweeps
  bool valid = used && o < A.count;
  ColumnMask msk = column_mask<N>(a, b, 2 * mi + A.cx, 2 * mj + A.cy, 2 * mk + A.cz, A.nc, A.color, dir, valid);
  long long nb = cell_node_base<N>(2 * mi + A.cx, 2 * mj + A.cy, 2 * mk + A.cz, A.Nx, plane) + toff;
  T xv[N];
  gather_column<N, T>(A.x + nb, plane, msk.keep, xv);

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
    // ---- sweeps S_z (gathered column), S_x, S_y and D_y ----
    eo_apply<N, 1>(A.S, xv, v);
#pragma unroll
    for (int c = 0; c < N; ++c)
      if (used) B0[zc + P2 * c] = v[c];
    cell_group_sync<W>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[xl + m];
    eo_apply<N, 1>(A.S, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (used) B0[xl + m] = v[m];
    cell_group_sync<W>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[yl + P1 * m];
    eo_apply<N, 1>(A.S, v, v);
    eo_apply<N, -1>(A.D, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (used) B1[yl + P1 * m] = v[m];
      if (used) B2[yl2 + Q1 * m] = g[m];
    }
    cell_group_sync<W>(grp);
    // ---- D_x into B0; D_z stays in registers (same thread, same column) ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[xl + m];
    eo_apply<N, -1>(A.D, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (used) B0[xl + m] = g[m];
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[zc + P2 * m];
    eo_apply<N, -1>(A.D, v, gz);
    cell_group_sync<W>(grp);
    // ---- quadrature points of column (a,b) ----
    const bool more = o0 + step < A.count;
    if (DEFORMED) {
      mbar_wait(bar, parity, A.err);
      parity ^= 1;
      // the next step's copies are issued after the group barrier below;
      // announce their bytes now (the barrier is already in its next phase)
      if (t == 0 && more)
        mbar_arrive_expect_tx(bar, geo_bytes * (uint32_t)min((long long)K, A.count - (o0 + step)));
    }
    T tz[N];
    {
      const T wab = A.w[a] * A.w[b];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const int s = zc + P2 * c;
        const T gx = B0[s], gy = B2[zc2 + Q2 * c];
        T tx, ty, tzc;
        if (DEFORMED) {
          const T *Gq = geo_s + c * N2 + l;
          const T g0 = Gq[0], g1 = Gq[N3], g2 = Gq[2 * N3], g3 = Gq[3 * N3], g4 = Gq[4 * N3], g5 = Gq[5 * N3];
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
        if (used) B2[zc2 + Q2 * c] = ty;
        tz[c] = tzc;
      }
      eo_apply<N, -1>(A.DT, tz, g);
#pragma unroll
      for (int c = 0; c < N; ++c)
        if (used) B1[zc + P2 * c] = g[c];
    }
    if (DEFORMED) fence_proxy_async_smem();
    cell_group_sync<W>(grp);
    // geometry buffers free: fetch the next step's blocks
    const bool nvalid = used && o + step < A.count;
    if (DEFORMED && more && nvalid && l == 0) {
      const long long cell = ((long long)(2 * nk + A.cz) * A.nc[1] + (2 * nj + A.cy)) * A.nc[0] + (2 * ni + A.cx);
      tma_load_1d_hint(geo_s, A.geo + cell * Cfg::GEO, geo_bytes, bar, pol);
    }
    // loads overlapped with the integration sweeps: the y values this
    // column adds to, and the next cell's x column
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
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[xl + m];
    eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const T s = B1[xl + m] + g[m];
      if (used) B1[xl + m] = s;
    }
    cell_group_sync<W>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B2[yl2 + Q1 * m];
    eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) g[m] += B1[yl + P1 * m];
    eo_apply<N, 1>(A.ST, g, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (used) B1[yl + P1 * m] = v[m];
    cell_group_sync<W>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[xl + m];
    eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (used) B1[xl + m] = v[m];
    cell_group_sync<W>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[zc + P2 * m];
    eo_apply<N, 1>(A.ST, v, v);
    // ---- scatter the z column: first colour stores, later ones add ----
    if (valid) store_column<N, T>(A.y + nb, A.x + nb, plane, msk.keep, v, yo);
    msk = nmsk;
    nb = nnb;
    valid = nvalid;
    mi = ni;
    mj = nj;
    mk = nk;
  }
  if (!y_ready) pdl_wait();
}

template <int N, typename T>
int line_vmult_impl(const sf_op *op, const T *x, T *y, cudaStream_t st)
{
  using Cfg = LineCfg<N, T>;
  LineArgs<N, T> A{};
  const Shape1D &s = op->shape;
  A.S = eo_of<N, T>(s.S, false);
  A.ST = eo_of<N, T>(s.S, true);
  A.D = eo_of<N, T>(s.D, false);
  A.DT = eo_of<N, T>(s.D, true);
  for (int i = 0; i < N; ++i) A.w[i] = T(s.wq[i]);
  for (int d = 0; d < 3; ++d) A.nc[d] = op->desc.n_cells[d];
  A.Nx = (N - 1) * A.nc[0] + 1;
  A.plane = A.Nx * ((N - 1) * A.nc[1] + 1);
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  for (int d = 0; d < 3; ++d) A.aff[d] = T(jxw / (op->h[d] * op->h[d]));
  A.dirichlet = op->desc.dirichlet;
  A.x = x;
  A.y = y;
  A.err = (int *)op->dev_err.ptr;
  const bool deformed = op->deformed, kap = op->has_kappa;
  A.geo = (const T *)(sizeof(T) == 8 ? op->geo64.ptr : op->geo32.ptr);
  A.kappa = (const T *)(sizeof(T) == 8 ? op->kap64.ptr : op->kap32.ptr);
  if (deformed && (!A.geo || op->geo_stride != Cfg::GEO)) {
    set_error("line kernel: geometry missing or with an unexpected block size");
    return SF_ERR_STATE;
  }
  if (kap && !A.kappa) {
    set_error("line kernel: coefficient missing");
    return SF_ERR_STATE;
  }
  void (*kern)(const LineArgs<N, T>) =
      deformed ? (kap ? line_vmult_kernel<N, T, true, true> : line_vmult_kernel<N, T, true, false>)
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
    const int mz = (A.nc[2] - A.cz + 1) / 2;
    A.count = (long long)A.mx * A.my * mz;
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

} // namespace

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
