// sf_laplace_line.cu -- continuous Laplacian with line ownership for all
// degrees and both precisions (the FP32 path of degrees 5..8 and the FP64
// path): one warp group of ceil(n^2/32) warps per cell, one thread per line.
//
// Per cell, 12 line sweeps through a padded shared-memory slab (x lines
// (b,c), y lines (a,c), z columns (a,b)); the group synchronises with a
// named barrier, so groups of one block run independently.  The grid is
// persistent: each group walks a strided list of the cells of one colour
// class and prefetches the next cell's geometry block with one TMA bulk copy
// right after the quadrature-point operation of the current cell (bounded
// mbarrier wait).  Summation and colour launches as in sf_laplace_plane.cu:
// first-touch store / add, programmatic dependent launch for colours 1..7.
#include "sf_device.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"
#include "sf_tma.cuh"

namespace sf {

namespace {

template <int N, typename T>
struct LineCfg {
  static constexpr int G = (N * N + 31) / 32;  // warps per cell group
  // padded slab layout idx(a,b,c) = a + P1 b + P2 c (few bank conflicts)
  static constexpr int P1 = N == 8 ? 9 : N;
  static constexpr int P2 = N == 7 ? 52 : N == 8 ? 72 : N * N;
  static constexpr int SLAB = P2 * N;
  // groups per block
  static constexpr int GROUPS = G == 1 ? 4 : (G == 2 ? 3 : 2);
};

template <int N, typename T>
struct LineArgs {
  EOMat<N, T> S, ST, D, DT;
  T w[N];
  const T *__restrict__ x;
  T *__restrict__ y;
  const T *__restrict__ geo;    // natural layout [cell][6][n^3], stride geo_stride
  const T *__restrict__ kappa;  // [cell][n^3] or null
  long long geo_stride;
  int nc[3];
  long long Nx, Ny, Nz;
  T aff[3];
  int dirichlet;
  int color, cx, cy, cz, mx, my;
  long long count;
  int *err;
  // stride of the cell walk (number of groups in the grid) decomposed in
  // the colour's (mi, mj, mk) index space: no division inside the loop
  int step_i, step_j, step_k;
};

template <int N, typename T, bool DEFORMED, bool KAPPA>
__global__ void __launch_bounds__(32 * LineCfg<N, T>::G * LineCfg<N, T>::GROUPS)
    line_vmult_kernel(const __grid_constant__ LineArgs<N, T> A)
{
  using Cfg = LineCfg<N, T>;
  constexpr int P = N - 1, N2 = N * N, N3 = N * N * N;
  constexpr int G = Cfg::G, GROUPS = Cfg::GROUPS, P1 = Cfg::P1, P2 = Cfg::P2, SLAB = Cfg::SLAB;
  constexpr int GT = 32 * G; // threads per group
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw);
  const int grp = threadIdx.x / GT, t = threadIdx.x % GT;
  const long long geo_e = DEFORMED ? A.geo_stride : 0;
  const long long region = (geo_e * sizeof(T) + 4 * SLAB * sizeof(T) + 127) / 128 * 128; // bytes
  unsigned char *gbase = smem_raw + 128 + grp * region;
  T *geo_s = reinterpret_cast<T *>(gbase);
  T *B0 = reinterpret_cast<T *>(gbase + geo_e * sizeof(T));
  T *B1 = B0 + SLAB, *B2 = B1 + SLAB, *B3 = B2 + SLAB;
  uint64_t *bar = bars + grp;

  const bool active = t < N2;
  const int tt = active ? t : 0;
  const int a = tt % N, b = tt / N;  // z column (a,b) / y line (a,c=b) / x line (b'=a, c'=b)
  const int zc = a + P1 * b;                 // z column base
  const int xl = P1 * a + P2 * b;            // x line (b'=a, c'=b) base, stride 1
  const int yl = a + P2 * b;                 // y line (a, c=b) base, stride P1

  const long long ng = (long long)gridDim.x * GROUPS;
  const long long gid = (long long)blockIdx.x * GROUPS + grp;

  // position (mi, mj, mk) of ordinal o in the colour's index space
  auto decode = [&](long long o, int &mi, int &mj, int &mk) {
    const unsigned uo = (unsigned)o, umx = (unsigned)A.mx, umy = (unsigned)A.my;
    const unsigned q = uo / umx;
    mi = int(uo - q * umx);
    mk = int(q / umy);
    mj = int(q - unsigned(mk) * umy);
  };
  auto advance = [&](int &mi, int &mj, int &mk) {
    mi += A.step_i;
    int carry = 0;
    if (mi >= A.mx) { mi -= A.mx; carry = 1; }
    mj += A.step_j + carry;
    carry = 0;
    if (mj >= A.my) { mj -= A.my; carry = 1; }
    mk += A.step_k + carry;
  };
  auto issue = [&](int mi, int mj, int mk) {
    const long long cell = ((long long)(2 * mk + A.cz) * A.nc[1] + (2 * mj + A.cy)) * A.nc[0] + (2 * mi + A.cx);
    const uint32_t bytes = (uint32_t)(A.geo_stride * sizeof(T));
    mbar_arrive_expect_tx(bar, bytes);
    tma_load_1d(geo_s, A.geo + cell * A.geo_stride, bytes, bar);
  };
  int mi = 0, mj = 0, mk = 0;
  if (gid < A.count) decode(gid, mi, mj, mk);
  if (DEFORMED) {
    if (t == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    cell_group_sync<G>(grp);
    if (t == 0 && gid < A.count) issue(mi, mj, mk);
  }
  pdl_trigger();
  uint32_t parity = 0;
  bool y_ready = false;

  for (long long o = gid; o < A.count; o += ng) {
    const int ci = 2 * mi + A.cx, cj = 2 * mj + A.cy, ck = 2 * mk + A.cz;
    int ni = mi, nj = mj, nk = mk; // next cell of this group
    advance(ni, nj, nk);
    const long long cell = ((long long)ck * A.nc[1] + cj) * A.nc[0] + ci;
    const bool dir = A.dirichlet != 0;
    const long long X = (long long)ci * P + a, Y = (long long)cj * P + b, Z0 = (long long)ck * P;
    const long long plane = A.Nx * A.Ny;
    const long long gb = (Z0 * A.Ny + Y) * A.Nx + X;
    const bool side = dir && (X == 0 || X == A.Nx - 1 || Y == 0 || Y == A.Ny - 1);
    const bool zlo = dir && ck == 0, zhi = dir && ck == A.nc[2] - 1;
    T v[N], g[N];
    // ---- gather the z column (a,b) ----
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const bool bnd = side || (c == 0 && zlo) || (c == P && zhi);
      v[c] = (active && !bnd) ? __ldg(A.x + gb + c * plane) : T(0);
    }
    eo_apply<N, 1>(A.S, v, v);
    if (active) {
#pragma unroll
      for (int c = 0; c < N; ++c) B0[zc + P2 * c] = v[c];
    }
    cell_group_sync<G>(grp);
    if (active) {
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B0[xl + m];
      eo_apply<N, 1>(A.S, v, v);
#pragma unroll
      for (int m = 0; m < N; ++m) B0[xl + m] = v[m];
    }
    cell_group_sync<G>(grp);
    if (active) {
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B0[yl + P1 * m];
      eo_apply<N, 1>(A.S, v, v);
      eo_apply<N, -1>(A.D, v, g);
#pragma unroll
      for (int m = 0; m < N; ++m) {
        B1[yl + P1 * m] = v[m];
        B2[yl + P1 * m] = g[m];
      }
    }
    cell_group_sync<G>(grp);
    if (active) {
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B1[xl + m];
      eo_apply<N, -1>(A.D, v, g);
#pragma unroll
      for (int m = 0; m < N; ++m) B0[xl + m] = g[m];
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B1[zc + P2 * m];
      eo_apply<N, -1>(A.D, v, g);
#pragma unroll
      for (int m = 0; m < N; ++m) B3[zc + P2 * m] = g[m];
    }
    cell_group_sync<G>(grp);
    // ---- quadrature points of column (a,b) ----
    T tz[N];
    if (DEFORMED) {
      mbar_wait(bar, parity, A.err);
      parity ^= 1;
    }
    if (active) {
      const T wab = A.w[a] * A.w[b];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const int s = zc + P2 * c;
        const T gx = B0[s], gy = B2[s], gz = B3[s];
        T tx, ty, tzc;
        if (DEFORMED) {
          const T *Gq = geo_s + c * N2 + tt;
          const T g0 = Gq[0], g1 = Gq[N3], g2 = Gq[2 * N3], g3 = Gq[3 * N3], g4 = Gq[4 * N3], g5 = Gq[5 * N3];
          tx = gx * g0 + gy * g3 + gz * g4;
          ty = gx * g3 + gy * g1 + gz * g5;
          tzc = gx * g4 + gy * g5 + gz * g2;
        } else {
          const T wq = wab * A.w[c];
          tx = gx * (A.aff[0] * wq);
          ty = gy * (A.aff[1] * wq);
          tzc = gz * (A.aff[2] * wq);
        }
        if (KAPPA) {
          const T kq = __ldg(A.kappa + cell * N3 + c * N2 + tt);
          tx *= kq;
          ty *= kq;
          tzc *= kq;
        }
        B0[s] = tx;
        B2[s] = ty;
        tz[c] = tzc;
      }
      eo_apply<N, -1>(A.DT, tz, g);
#pragma unroll
      for (int c = 0; c < N; ++c) B1[zc + P2 * c] = g[c];
    }
    if (DEFORMED) fence_proxy_async_smem();
    cell_group_sync<G>(grp);
    // geometry buffer free: fetch the next cell's block
    if (DEFORMED && t == 0 && o + ng < A.count) issue(ni, nj, nk);
    if (active) {
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B0[xl + m];
      eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
      for (int m = 0; m < N; ++m) B1[xl + m] += g[m];
    }
    cell_group_sync<G>(grp);
    if (active) {
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B2[yl + P1 * m];
      eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
      for (int m = 0; m < N; ++m) g[m] += B1[yl + P1 * m];
      eo_apply<N, 1>(A.ST, g, v);
#pragma unroll
      for (int m = 0; m < N; ++m) B1[yl + P1 * m] = v[m];
    }
    cell_group_sync<G>(grp);
    if (active) {
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B1[xl + m];
      eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
      for (int m = 0; m < N; ++m) B1[xl + m] = v[m];
    }
    cell_group_sync<G>(grp);
    if (active) {
#pragma unroll
      for (int m = 0; m < N; ++m) v[m] = B1[zc + P2 * m];
      eo_apply<N, 1>(A.ST, v, v);
    }
    // ---- scatter the z column: first colour stores, later ones add ----
    if (!y_ready) {
      pdl_wait();
      y_ready = true;
    }
    if (active) {
      const int mxy = ((a == 0 && ci > 0) || (a == P && ci < A.nc[0] - 1) ? 1 : 0) |
                      ((b == 0 && cj > 0) || (b == P && cj < A.nc[1] - 1) ? 2 : 0);
      const bool zl = ck > 0, zh = ck < A.nc[2] - 1;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const bool bnd = side || (c == 0 && zlo) || (c == P && zhi);
        const int mz = ((c == 0 && zl) || (c == P && zh)) ? 4 : 0;
        T *dst = A.y + gb + c * plane;
        if (bnd) *dst = __ldg(A.x + gb + c * plane);
        else if (A.color & (mxy | mz)) *dst += v[c];
        else *dst = v[c];
      }
    }
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
  A.Nx = (long long)(N - 1) * A.nc[0] + 1;
  A.Ny = (long long)(N - 1) * A.nc[1] + 1;
  A.Nz = (long long)(N - 1) * A.nc[2] + 1;
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  for (int d = 0; d < 3; ++d) A.aff[d] = T(jxw / (op->h[d] * op->h[d]));
  A.dirichlet = op->desc.dirichlet;
  A.x = x;
  A.y = y;
  A.err = (int *)op->dev_err.ptr;
  const bool deformed = op->deformed, kap = op->has_kappa;
  A.geo = (const T *)(sizeof(T) == 8 ? op->geo64.ptr : op->geo32.ptr);
  A.kappa = (const T *)(sizeof(T) == 8 ? op->kap64.ptr : op->kap32.ptr);
  A.geo_stride = op->geo_stride;
  void (*kern)(const LineArgs<N, T>) =
      deformed ? (kap ? line_vmult_kernel<N, T, true, true> : line_vmult_kernel<N, T, true, false>)
               : (kap ? line_vmult_kernel<N, T, false, true> : line_vmult_kernel<N, T, false, false>);
  const long long geo_e = deformed ? A.geo_stride : 0;
  const long long region = (geo_e * (long long)sizeof(T) + 4LL * Cfg::SLAB * sizeof(T) + 127) / 128 * 128;
  const size_t smem = 128 + size_t(Cfg::GROUPS) * region;
  const int threads = 32 * Cfg::G * Cfg::GROUPS;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  int per_sm = 0;
  SF_RET_IF(resident_blocks_per_sm((const void *)kern, threads, smem, &per_sm));
  if (per_sm < 1) {
    set_error("line kernel does not fit on an SM");
    return SF_ERR_UNSUPPORTED;
  }
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
    const long long blocks =
        std::min<long long>((A.count + Cfg::GROUPS - 1) / Cfg::GROUPS, (long long)per_sm * n_sm);
    const long long ng = blocks * Cfg::GROUPS;
    A.step_i = int(ng % A.mx);
    A.step_j = int((ng / A.mx) % A.my);
    A.step_k = int(ng / ((long long)A.mx * A.my));
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
