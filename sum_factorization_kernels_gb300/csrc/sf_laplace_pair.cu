// sf_laplace_pair.cu -- FP32 continuous Laplacian, all degrees, two cells
// per warp group processed together in packed FP32x2 arithmetic.
//
// Every thread owns one line (x line, y line or z column, as in
// sf_laplace_line.cu) of TWO cells of the same colour class; values are held
// as float2 (cell A, cell B) and contracted with the sm_100 packed
// instructions __ffma2_rn / __fadd2_rn / __fmul2_rn against duplicated
// even-odd coefficients, so one instruction does the work of two.  The
// shared-memory slab holds float2 pairs (64-bit accesses), and the geometry
// is stored pair-interleaved ([pair][component][point][2], colour-major) so
// one TMA bulk copy brings both cells' tensors.  Lanes beyond n^2 work on
// line 0 of the slab with their stores predicated off, so the sweeps need no
// divergent branches.  Summation, colours and PDL as in the other kernels.
#include "sf_cont_column.cuh"
#include "sf_device.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"
#include "sf_tma.cuh"

namespace sf {

namespace {

template <int N>
struct PairCfg {
  static constexpr int G = (N * N + 31) / 32;  // warps per group
  static constexpr int P1 = N == 8 ? 9 : N;
  static constexpr int P2 = N == 7 ? 52 : N == 8 ? 72 : N * N;
  static constexpr int SLAB = P2 * N;          // float2 entries
  static constexpr int NSLAB = 3;              // slabs per group
  static constexpr int GROUPS = G == 1 ? 4 : (G == 2 ? 3 : 2);
};

// geometry stride of one pair block (floats, multiple of 4)
inline long long pair_geo_stride(int n, int ncomp) { return ((long long)2 * ncomp * n * n * n + 3) / 4 * 4; }

template <int N>
struct EO2 {
  static constexpr int H = N / 2;
  static constexpr int HH = H > 0 ? H : 1;
  float2 e[HH][HH], o[HH][HH], mc[HH], mr[HH], mm;
};

template <int N>
EO2<N> eo2_of(const double (&M)[kMaxN][kMaxN], bool transpose)
{
  const EOMat<N, float> f = eo_of<N, float>(M, transpose);
  EO2<N> r{};
  constexpr int HH = EO2<N>::HH;
  for (int i = 0; i < HH; ++i) {
    for (int j = 0; j < HH; ++j) {
      r.e[i][j] = make_float2(f.e[i][j], f.e[i][j]);
      r.o[i][j] = make_float2(f.o[i][j], f.o[i][j]);
    }
    r.mc[i] = make_float2(f.mc[i], f.mc[i]);
    r.mr[i] = make_float2(f.mr[i], f.mr[i]);
  }
  r.mm = make_float2(f.mm, f.mm);
  return r;
}

__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
// a - b as one packed FMA
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// out = M in on packed pairs (see sf_device.cuh for the even-odd scheme)
template <int N, int SIGN>
__device__ __forceinline__ void eo2(const EO2<N> &M, const float2 (&in)[N], float2 (&out)[N])
{
  constexpr int H = N / 2;
  constexpr int HH = H > 0 ? H : 1;
  float2 up[HH], um[HH];
#pragma unroll
  for (int j = 0; j < H; ++j) {
    up[j] = f2add(in[j], in[N - 1 - j]);
    um[j] = f2sub(in[j], in[N - 1 - j]);
  }
  float2 res[N];
#pragma unroll
  for (int i = 0; i < H; ++i) {
    float2 a = (N % 2 == 1) ? f2fma(M.e[i][0], up[0], f2mul(M.mc[i], in[H])) : f2mul(M.e[i][0], up[0]);
#pragma unroll
    for (int j = 1; j < H; ++j) a = f2fma(M.e[i][j], up[j], a);
    float2 b = f2mul(M.o[i][0], um[0]);
#pragma unroll
    for (int j = 1; j < H; ++j) b = f2fma(M.o[i][j], um[j], b);
    res[i] = f2add(a, b);
    res[N - 1 - i] = SIGN > 0 ? f2sub(a, b) : f2sub(b, a);
  }
  if (N % 2 == 1) {
    if (H == 0) {
      res[0] = f2mul(M.mm, in[0]);
    } else if (SIGN > 0) {
      float2 m = f2fma(M.mr[0], up[0], f2mul(M.mm, in[H]));
#pragma unroll
      for (int j = 1; j < H; ++j) m = f2fma(M.mr[j], up[j], m);
      res[H] = m;
    } else {
      float2 m = f2mul(M.mr[0], um[0]);
#pragma unroll
      for (int j = 1; j < H; ++j) m = f2fma(M.mr[j], um[j], m);
      res[H] = m;
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) out[i] = res[i];
}

template <int N>
struct PairArgs {
  EO2<N> S, ST, D, DT;
  float w[N];
  const float *__restrict__ x;
  float *__restrict__ y;
  const float *__restrict__ geo;   // pair blocks, colour-major
  long long gstride;               // floats per pair block
  long long pair_base;             // first pair of this colour in the geometry
  int nc[3];
  int Nx, plane;                   // nodes per x line, per z plane
  float aff[3];
  int dirichlet;
  int color, cx, cy, cz, mx, my;
  long long count;                 // cells of this colour
  int *err;
  int step_i, step_j, step_k;      // walk stride (2 x groups) in (mi, mj, mk)
};

template <int N, bool DEFORMED, bool KAPPA>
__global__ void __launch_bounds__(32 * PairCfg<N>::G * PairCfg<N>::GROUPS)
    pair_vmult_kernel(const __grid_constant__ PairArgs<N> A)
{
  using Cfg = PairCfg<N>;
  constexpr int N2 = N * N, N3 = N * N * N;
  constexpr int G = Cfg::G, GROUPS = Cfg::GROUPS, P1 = Cfg::P1, P2 = Cfg::P2;
  constexpr int GT = 32 * G;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw);
  const int grp = threadIdx.x / GT, t = threadIdx.x % GT;
  const long long geo_f = DEFORMED ? A.gstride : 0;
  const long long region = (geo_f * 4 + 8LL * Cfg::NSLAB * Cfg::SLAB + 127) / 128 * 128;
  unsigned char *gbase = smem_raw + 128 + grp * region;
  float *geo_s = reinterpret_cast<float *>(gbase);
  float2 *B0 = reinterpret_cast<float2 *>(gbase + geo_f * 4);
  float2 *B1 = B0 + Cfg::SLAB, *B2 = B1 + Cfg::SLAB;
  uint64_t *bar = bars + grp;

  // idle lanes (t >= n^2) run line 0 with their shared stores predicated
  // off, so the sweeps carry no divergent branches
  const bool active = t < N2;
  const int ta = active ? t : 0;
  const int a = ta % N, b = ta / N;
  const int zc = a + P1 * b;
  const int xl = P1 * a + P2 * b;
  const int yl = a + P2 * b;
  const int plane = A.plane;
  const int toff = b * A.Nx + a;

  const long long npairs = (A.count + 1) / 2;
  const long long ng = (long long)gridDim.x * GROUPS;
  const long long gid = (long long)blockIdx.x * GROUPS + grp;

  auto issue = [&](long long pr) {
    const uint32_t bytes = (uint32_t)(A.gstride * 4);
    mbar_arrive_expect_tx(bar, bytes);
    tma_load_1d(geo_s, A.geo + (A.pair_base + pr) * A.gstride, bytes, bar);
  };
  // (mi, mj, mk) of the first cell (ordinal 2 * pair) of this group's pair
  int mi = 0, mj = 0, mk = 0;
  if (gid < npairs) {
    const unsigned uo = (unsigned)(2 * gid), umx = (unsigned)A.mx, umy = (unsigned)A.my;
    const unsigned q = uo / umx;
    mi = int(uo - q * umx);
    mk = int(q / umy);
    mj = int(q - unsigned(mk) * umy);
  }
  if (DEFORMED) {
    if (t == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    cell_group_sync<G>(grp);
    if (t == 0 && gid < npairs) issue(gid);
  }
  pdl_trigger();
  uint32_t parity = 0;
  bool y_ready = false;

  for (long long pr = gid; pr < npairs; pr += ng) {
    // the two cells: ordinals 2 pr and 2 pr + 1
    int bi = mi + 1, bj = mj, bk = mk;
    if (bi >= A.mx) {
      bi = 0;
      if (++bj >= A.my) {
        bj = 0;
        ++bk;
      }
    }
    const bool hasB = 2 * pr + 1 < A.count;
    const int ai = 2 * mi + A.cx, aj = 2 * mj + A.cy, ak = 2 * mk + A.cz;
    const int ei = 2 * bi + A.cx, ej = 2 * bj + A.cy, ek = 2 * bk + A.cz;
    const bool dir = A.dirichlet != 0;
    const ColumnMask mA = column_mask<N>(a, b, ai, aj, ak, A.nc, A.color, dir, active);
    const ColumnMask mB = column_mask<N>(a, b, ei, ej, ek, A.nc, A.color, dir, active && hasB);
    const long long nbA = cell_node_base<N>(ai, aj, ak, A.Nx, plane) + toff;
    const long long nbB = cell_node_base<N>(ei, ej, ek, A.Nx, plane) + toff;
    float2 v[N], g[N], gz[N];
    {
      float va[N], vb[N];
      gather_column<N, float>(A.x + nbA, plane, mA.keep, va);
      gather_column<N, float>(A.x + nbB, plane, mB.keep, vb);
#pragma unroll
      for (int c = 0; c < N; ++c) v[c] = make_float2(va[c], vb[c]);
    }
    eo2<N, 1>(A.S, v, v);
#pragma unroll
    for (int c = 0; c < N; ++c)
      if (active) B0[zc + P2 * c] = v[c];
    cell_group_sync<G>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[xl + m];
    eo2<N, 1>(A.S, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (active) B0[xl + m] = v[m];
    cell_group_sync<G>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[yl + P1 * m];
    eo2<N, 1>(A.S, v, v);
    eo2<N, -1>(A.D, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (active) B1[yl + P1 * m] = v[m];
      if (active) B2[yl + P1 * m] = g[m];
    }
    cell_group_sync<G>(grp);
    // D_x into B0; D_z stays in registers (same thread, same column)
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[xl + m];
    eo2<N, -1>(A.D, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (active) B0[xl + m] = g[m];
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[zc + P2 * m];
    eo2<N, -1>(A.D, v, gz);
    cell_group_sync<G>(grp);
    // ---- quadrature points of column (a,b), both cells ----
    float2 tz[N];
    if (DEFORMED) {
      mbar_wait(bar, parity, A.err);
      parity ^= 1;
    }
    {
      const float wab = A.w[a] * A.w[b];
      const int q0 = a + N * b;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const int s = zc + P2 * c;
        const float2 gx = B0[s], gy = B2[s];
        float2 tx, ty, tzc;
        if (DEFORMED) {
          const float2 *Gq = reinterpret_cast<const float2 *>(geo_s) + c * N2 + q0;
          const float2 g0 = Gq[0], g1 = Gq[N3], g2 = Gq[2 * N3], g3 = Gq[3 * N3], g4 = Gq[4 * N3],
                       g5 = Gq[5 * N3];
          tx = f2fma(gz[c], g4, f2fma(gy, g3, f2mul(gx, g0)));
          ty = f2fma(gz[c], g5, f2fma(gy, g1, f2mul(gx, g3)));
          tzc = f2fma(gz[c], g2, f2fma(gy, g5, f2mul(gx, g4)));
          if (KAPPA) {
            const float2 kq = Gq[6 * N3];
            tx = f2mul(tx, kq);
            ty = f2mul(ty, kq);
            tzc = f2mul(tzc, kq);
          }
        } else {
          const float wq = wab * A.w[c];
          tx = f2mul(gx, make_float2(A.aff[0] * wq, A.aff[0] * wq));
          ty = f2mul(gy, make_float2(A.aff[1] * wq, A.aff[1] * wq));
          tzc = f2mul(gz[c], make_float2(A.aff[2] * wq, A.aff[2] * wq));
        }
        if (active) B0[s] = tx;
        if (active) B2[s] = ty;
        tz[c] = tzc;
      }
    }
    eo2<N, -1>(A.DT, tz, g);
#pragma unroll
    for (int c = 0; c < N; ++c)
      if (active) B1[zc + P2 * c] = g[c];
    if (DEFORMED) fence_proxy_async_smem();
    cell_group_sync<G>(grp);
    if (DEFORMED && t == 0 && pr + ng < npairs) issue(pr + ng);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B0[xl + m];
    eo2<N, -1>(A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const float2 s = f2add(B1[xl + m], g[m]);
      if (active) B1[xl + m] = s;
    }
    cell_group_sync<G>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B2[yl + P1 * m];
    eo2<N, -1>(A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) g[m] = f2add(g[m], B1[yl + P1 * m]);
    eo2<N, 1>(A.ST, g, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (active) B1[yl + P1 * m] = v[m];
    cell_group_sync<G>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[xl + m];
    eo2<N, 1>(A.ST, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (active) B1[xl + m] = v[m];
    cell_group_sync<G>(grp);
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = B1[zc + P2 * m];
    eo2<N, 1>(A.ST, v, v);
    // ---- scatter both columns ----
    if (!y_ready) {
      pdl_wait();
      y_ready = true;
    }
    {
      float va[N], vb[N];
#pragma unroll
      for (int c = 0; c < N; ++c) {
        va[c] = v[c].x;
        vb[c] = v[c].y;
      }
      if (active) scatter_column<N, float>(A.y + nbA, A.x + nbA, plane, mA, va);
      if (active && hasB) scatter_column<N, float>(A.y + nbB, A.x + nbB, plane, mB, vb);
    }
    // advance the pair walk by 2 * ng ordinals
    mi += A.step_i;
    int carry = 0;
    if (mi >= A.mx) { mi -= A.mx; carry = 1; }
    mj += A.step_j + carry;
    carry = 0;
    if (mj >= A.my) { mj -= A.my; carry = 1; }
    mk += A.step_k + carry;
  }
  if (!y_ready) pdl_wait();
}

// natural FP64 geometry (+kappa) -> pair-interleaved colour-major FP32
template <int N>
__global__ void pair_repack_kernel(const double *__restrict__ G, long long s64, const double *__restrict__ kap,
                                   float *__restrict__ out, long long gstride, int ncomp, int nx, int ny, int nz,
                                   const long long *__restrict__ pbase)
{
  constexpr int N3 = N * N * N;
  const long long C = (long long)nx * ny * nz;
  const long long total = C * ncomp * N3;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < total;
       s += (long long)gridDim.x * blockDim.x) {
    const long long cell = s / (ncomp * N3);
    const int rem = int(s - cell * ncomp * N3);
    const int e = rem / N3, q = rem % N3;
    const int i = int(cell % nx), j = int((cell / nx) % ny), k = int(cell / ((long long)nx * ny));
    const int color = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2);
    const int mx = (nx - (i & 1) + 1) / 2, my = (ny - (j & 1) + 1) / 2;
    const long long ord = (i >> 1) + (long long)mx * ((j >> 1) + (long long)my * (k >> 1));
    const long long pair = pbase[color] + ord / 2;
    const double v = e < 6 ? G[cell * s64 + e * N3 + q] : kap[cell * N3 + q];
    out[pair * gstride + ((long long)e * N3 + q) * 2 + (ord & 1)] = float(v);
  }
}

template <int N>
int pair_vmult_impl(const sf_op *op, const float *x, float *y, cudaStream_t st)
{
  using Cfg = PairCfg<N>;
  PairArgs<N> A{};
  const Shape1D &s = op->shape;
  A.S = eo2_of<N>(s.S, false);
  A.ST = eo2_of<N>(s.S, true);
  A.D = eo2_of<N>(s.D, false);
  A.DT = eo2_of<N>(s.D, true);
  for (int i = 0; i < N; ++i) A.w[i] = float(s.wq[i]);
  for (int d = 0; d < 3; ++d) A.nc[d] = op->desc.n_cells[d];
  A.Nx = (N - 1) * A.nc[0] + 1;
  A.plane = A.Nx * ((N - 1) * A.nc[1] + 1);
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  for (int d = 0; d < 3; ++d) A.aff[d] = float(jxw / (op->h[d] * op->h[d]));
  A.dirichlet = op->desc.dirichlet;
  A.x = x;
  A.y = y;
  A.err = (int *)op->dev_err.ptr;
  const bool deformed = op->deformed, kap = op->has_kappa;
  if (!deformed && kap) {
    set_error("kappa on an affine mesh needs the geometry path");
    return SF_ERR_STATE;
  }
  A.geo = (const float *)op->geoPair.ptr;
  A.gstride = op->geoPair_stride;
  if (deformed && !A.geo) {
    set_error("pair kernel geometry missing");
    return SF_ERR_STATE;
  }
  void (*kern)(const PairArgs<N>) =
      deformed ? (kap ? pair_vmult_kernel<N, true, true> : pair_vmult_kernel<N, true, false>)
               : pair_vmult_kernel<N, false, false>;
  const long long geo_f = deformed ? A.gstride : 0;
  const long long region = (geo_f * 4 + 8LL * Cfg::NSLAB * Cfg::SLAB + 127) / 128 * 128;
  const size_t smem = 128 + size_t(Cfg::GROUPS) * region;
  const int threads = 32 * Cfg::G * Cfg::GROUPS;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  int per_sm = 0;
  SF_RET_IF(resident_blocks_per_sm((const void *)kern, threads, smem, &per_sm));
  int n_sm = 0, dev = 0;
  SF_CUDA_TRY(cudaGetDevice(&dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  long long pbase = 0;
  for (int color = 0; color < 8; ++color) {
    A.color = color;
    A.cx = color & 1;
    A.cy = (color >> 1) & 1;
    A.cz = (color >> 2) & 1;
    A.mx = (A.nc[0] - A.cx + 1) / 2;
    A.my = (A.nc[1] - A.cy + 1) / 2;
    const int mz = (A.nc[2] - A.cz + 1) / 2;
    A.count = (long long)A.mx * A.my * mz;
    A.pair_base = pbase;
    pbase += (A.count + 1) / 2;
    if (A.count == 0) continue;
    const long long npairs = (A.count + 1) / 2;
    const long long blocks = std::min<long long>((npairs + Cfg::GROUPS - 1) / Cfg::GROUPS, (long long)per_sm * n_sm);
    const long long stride = 2 * blocks * Cfg::GROUPS;
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
    cfg.numAttrs = color > 0 ? 1 : 0;
    SF_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, A));
  }
  return SF_OK;
}

template <int N>
int pair_repack_impl(sf_op *op, const double *G64, long long s64, const double *kap64, cudaStream_t st)
{
  const int ncomp = kap64 ? 7 : 6;
  const long long gs = pair_geo_stride(N, ncomp);
  const int nx = op->desc.n_cells[0], ny = op->desc.n_cells[1], nz = op->desc.n_cells[2];
  long long pb[8], acc = 0;
  for (int color = 0; color < 8; ++color) {
    const int cx = color & 1, cy = (color >> 1) & 1, cz = (color >> 2) & 1;
    pb[color] = acc;
    acc += ((long long)((nx - cx + 1) / 2) * ((ny - cy + 1) / 2) * ((nz - cz + 1) / 2) + 1) / 2;
  }
  const size_t bytes = (size_t)acc * gs * sizeof(float);
  if (op->geoPair.bytes != bytes) {
    int e = op->geoPair.alloc(bytes);
    if (e) return e;
  }
  SF_CUDA_TRY(cudaMemsetAsync(op->geoPair.ptr, 0, bytes, st)); // absent partner cells stay zero
  op->geoPair_stride = gs;
  DevBuf pbd;
  int e = pbd.alloc(sizeof(pb));
  if (e) return e;
  SF_CUDA_TRY(cudaMemcpyAsync(pbd.ptr, pb, sizeof(pb), cudaMemcpyHostToDevice, st));
  pair_repack_kernel<N><<<152 * 16, 256, 0, st>>>(G64, s64, kap64, (float *)op->geoPair.ptr, gs, ncomp, nx, ny,
                                                  nz, (const long long *)pbd.ptr);
  SF_CUDA_TRY(cudaGetLastError());
  SF_CUDA_TRY(cudaStreamSynchronize(st));
  return SF_OK;
}

} // namespace

bool pair_path(const sf_op *op, int prec)
{
  return op->kernel_variant == SF_KERNEL_PAIR && prec == SF_FP32 && op->desc.kind == SF_OP_LAPLACE &&
         (op->deformed || !op->has_kappa);
}

int launch_cont_vmult_pair(const sf_op *op, const float *x, float *y, cudaStream_t st)
{
  switch (op->n) {
  case 2: return pair_vmult_impl<2>(op, x, y, st);
  case 3: return pair_vmult_impl<3>(op, x, y, st);
  case 4: return pair_vmult_impl<4>(op, x, y, st);
  case 5: return pair_vmult_impl<5>(op, x, y, st);
  case 6: return pair_vmult_impl<6>(op, x, y, st);
  case 7: return pair_vmult_impl<7>(op, x, y, st);
  case 8: return pair_vmult_impl<8>(op, x, y, st);
  case 9: return pair_vmult_impl<9>(op, x, y, st);
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;
  }
}

int repack_pair_geometry(sf_op *op, const double *G64, long long s64, const double *kap64, cudaStream_t st)
{
  switch (op->n) {
  case 2: return pair_repack_impl<2>(op, G64, s64, kap64, st);
  case 3: return pair_repack_impl<3>(op, G64, s64, kap64, st);
  case 4: return pair_repack_impl<4>(op, G64, s64, kap64, st);
  case 5: return pair_repack_impl<5>(op, G64, s64, kap64, st);
  case 6: return pair_repack_impl<6>(op, G64, s64, kap64, st);
  case 7: return pair_repack_impl<7>(op, G64, s64, kap64, st);
  case 8: return pair_repack_impl<8>(op, G64, s64, kap64, st);
  case 9: return pair_repack_impl<9>(op, G64, s64, kap64, st);
  default: return SF_ERR_UNSUPPORTED;
  }
}

} // namespace sf
