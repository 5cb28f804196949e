// sf_laplace_plane.cu -- FP32 continuous Laplacian for degrees 1..4 with
// plane ownership: one warp processes 32/n cells at once, one thread per
// xy-plane of a cell.
//
// Data flow of one cell (thread r owns plane r; "XY" = xy-plane c=r held as
// u[b][a], "XZ" = xz-plane b=r held as w[c][a]):
//   gather XY -> S_x, S_y in registers -> XY->XZ transpose -> S_z, D_x, D_z
//   -> uq XZ->XY, D_y, gy XY->XZ -> quadrature-point operation with the
//   geometry staged by TMA -> D_x^T + D_z^T in XZ, (t_y, r) XZ->XY, D_y^T,
//   S_y^T, S_x^T -> XY->XZ, S_z^T -> scatter.
// Five shared-memory transposes (x2 arrays for one of them) per cell instead
// of a round trip per 1D sweep; only __syncwarp() between phases because a
// cell never leaves its warp.
//
// Geometry: the merged 6-entry tensor (7th entry kappa when a coefficient is
// set) is stored in colour-major cell order, each cell block ordered
// [component][b][c][a], so the 32/n cells a warp needs are one contiguous
// range: one cp.async.bulk per warp and batch, issued one batch ahead into
// shared memory and completed on an mbarrier (bounded wait).
//
// Summation: 8 colour classes (parity of i, j, k), launched in colour order.
// A node is stored by the first colour that touches it and added to by the
// later ones: with M the set of directions in which a neighbouring cell of
// the mesh shares the node, an earlier-colour cell shares it iff
// (colour & M) != 0.  No zeroing pass and no atomics; Dirichlet rows are
// written as y_b = x_b by every cell touching them.  Successive colour
// launches overlap through programmatic dependent launch: a kernel's
// geometry prefetch and gather run before griddepcontrol.wait, which guards
// the first access of y.
#include "sf_device.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"
#include "sf_tma.cuh"

namespace sf {

template <int N>
struct PlaneCfg {
  static constexpr int CPW = 32 / N;                       // cells per warp
  static constexpr int PS = (N * N + 3) / 4 * 4;           // plane stride (floats)
  // cell stride of the transposition buffers, chosen for few bank conflicts
  static constexpr int CS = N == 2 ? 9 : N == 3 ? 41 : N == 4 ? 65 : 153;
  static constexpr int WARPS = 4;                          // warps per block
};

// geometry cell stride (floats, multiple of 4) for ncomp = 6 or 7 components
inline long long plane_geo_stride(int n, int ncomp)
{
  static const int s6[6] = {0, 0, 52, 164, 388, 756};
  static const int s7[6] = {0, 0, 56, 196, 452, 876};
  return ncomp == 6 ? s6[n] : s7[n];
}

namespace {

template <int N>
struct PlaneArgs {
  EOMat<N, float> S, ST, D, DT;
  float w[N];
  const float *__restrict__ x;
  float *__restrict__ y;
  const float *__restrict__ geo;
  long long gstride;
  long long color_base;
  int nc[3];
  long long Nx, Ny, Nz;
  float aff[3];
  int dirichlet;
  int color, cx, cy, cz, mx, my;
  long long count;
  int *err;
  // ordinal stride of a warp's walk (warps x cells per warp), decomposed
  // in the colour's (mi, mj, mk) index space
  int step_i, step_j, step_k;
};

template <int N, int SIGN>
__device__ __forceinline__ void sweep_cols(const EOMat<N, float> &M, float (&u)[N][N])
{
#pragma unroll
  for (int a = 0; a < N; ++a) {
    float col[N];
#pragma unroll
    for (int m = 0; m < N; ++m) col[m] = u[m][a];
    eo_apply<N, SIGN>(M, col, col);
#pragma unroll
    for (int m = 0; m < N; ++m) u[m][a] = col[m];
  }
}

template <int N, int SIGN>
__device__ __forceinline__ void sweep_cols_to(const EOMat<N, float> &M, const float (&u)[N][N],
                                              float (&o)[N][N])
{
#pragma unroll
  for (int a = 0; a < N; ++a) {
    float col[N];
#pragma unroll
    for (int m = 0; m < N; ++m) col[m] = u[m][a];
    eo_apply<N, SIGN>(M, col, col);
#pragma unroll
    for (int m = 0; m < N; ++m) o[m][a] = col[m];
  }
}

template <int N, bool AFFINE, bool KAPPA>
__global__ void __launch_bounds__(32 * PlaneCfg<N>::WARPS)
    plane_vmult_kernel(const __grid_constant__ PlaneArgs<N> A)
{
  using Cfg = PlaneCfg<N>;
  constexpr int P = N - 1, N2 = N * N, N3 = N * N * N;
  constexpr int CPW = Cfg::CPW, PS = Cfg::PS, CS = Cfg::CS, WARPS = Cfg::WARPS;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long geo_f = AFFINE ? 0 : CPW * A.gstride;
  const long long region = (geo_f + 2 * CPW * CS + 31) / 32 * 32;
  float *base = reinterpret_cast<float *>(smem_raw + 128) + warp * region;
  float *geo_s = base;
  float *As = base + geo_f, *Bs = As + CPW * CS;
  uint64_t *bar = bars + warp;

  const bool active = lane < CPW * N;
  const int k = active ? lane / N : 0;
  const int r = active ? lane % N : 0;
  float *Ak = As + k * CS, *Bk = Bs + k * CS;

  const long long nbatch = (A.count + CPW - 1) / CPW;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  const long long nw = (long long)gridDim.x * WARPS;

  if (!AFFINE) {
    if (lane == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    __syncwarp();
    if (lane == 0 && gw < nbatch) {
      const long long o0 = gw * CPW;
      const int nv = (int)min((long long)CPW, A.count - o0);
      const uint32_t bytes = (uint32_t)(nv * A.gstride * 4);
      mbar_arrive_expect_tx(bar, bytes);
      tma_load_1d(geo_s, A.geo + (A.color_base + o0) * A.gstride, bytes, bar);
    }
  }
  pdl_trigger();
  uint32_t parity = 0;
  bool y_ready = false;
  // (mi, mj, mk) of this lane's cell; advanced by the walk stride each batch
  int mi, mj, mk;
  {
    const unsigned uo = (unsigned)(gw * CPW + k), umx = (unsigned)A.mx, umy = (unsigned)A.my;
    const unsigned q = uo / umx;
    mi = int(uo - q * umx);
    mk = int(q / umy);
    mj = int(q - unsigned(mk) * umy);
  }

  for (long long batch = gw; batch < nbatch; batch += nw) {
    __syncwarp();
    const long long o = batch * CPW + k;
    const bool valid = active && o < A.count;
    const int ci = 2 * mi + A.cx, cj = 2 * mj + A.cy, ck = 2 * mk + A.cz;
    const long long X0 = (long long)ci * P;
    const bool dir = A.dirichlet != 0;
    const bool xl = dir && ci == 0, xr = dir && ci == A.nc[0] - 1;

    // ---- gather the xy-plane c = r ----
    float u[N][N];
    {
      const long long Z = (long long)ck * P + r;
      const bool zb = dir && (Z == 0 || Z == A.Nz - 1);
#pragma unroll
      for (int b = 0; b < N; ++b) {
        const long long Y = (long long)cj * P + b;
        const bool yb = zb || (dir && (Y == 0 || Y == A.Ny - 1));
        const float *src = A.x + (Z * A.Ny + Y) * A.Nx + X0;
#pragma unroll
        for (int a = 0; a < N; ++a) {
          const bool bnd = yb || (a == 0 && xl) || (a == P && xr);
          u[b][a] = (valid && !bnd) ? __ldg(src + a) : 0.f;
        }
      }
    }
    // ---- S_x, S_y in registers ----
#pragma unroll
    for (int b = 0; b < N; ++b) eo_apply<N, 1>(A.S, u[b], u[b]);
    sweep_cols<N, 1>(A.S, u);
    // ---- XY -> XZ ----
    if (active) {
#pragma unroll
      for (int b = 0; b < N; ++b)
#pragma unroll
        for (int a = 0; a < N; ++a) Ak[r * PS + b * N + a] = u[b][a];
    }
    __syncwarp();
    float w[N][N];
#pragma unroll
    for (int c = 0; c < N; ++c)
#pragma unroll
      for (int a = 0; a < N; ++a) w[c][a] = Ak[c * PS + r * N + a];
    // ---- S_z; D_x, D_z ----
    sweep_cols<N, 1>(A.S, w);
    float gx[N][N], gz[N][N];
#pragma unroll
    for (int c = 0; c < N; ++c) eo_apply<N, -1>(A.D, w[c], gx[c]);
    sweep_cols_to<N, -1>(A.D, w, gz);
    // ---- D_y via XZ -> XY -> XZ ----
    if (active) {
#pragma unroll
      for (int c = 0; c < N; ++c)
#pragma unroll
        for (int a = 0; a < N; ++a) Ak[c * PS + r * N + a] = w[c][a];
    }
    __syncwarp();
#pragma unroll
    for (int b = 0; b < N; ++b)
#pragma unroll
      for (int a = 0; a < N; ++a) u[b][a] = Ak[r * PS + b * N + a];
    sweep_cols<N, -1>(A.D, u);
    if (active) {
#pragma unroll
      for (int b = 0; b < N; ++b)
#pragma unroll
        for (int a = 0; a < N; ++a) Bk[r * PS + b * N + a] = u[b][a];
    }
    __syncwarp();
    float gy[N][N];
#pragma unroll
    for (int c = 0; c < N; ++c)
#pragma unroll
      for (int a = 0; a < N; ++a) gy[c][a] = Bk[c * PS + r * N + a];
    // ---- quadrature points (a, b=r, c) ----
    if (!AFFINE) {
      mbar_wait(bar, parity, A.err);
      parity ^= 1;
      const float *G = geo_s + k * A.gstride + r * N2;
#pragma unroll
      for (int c = 0; c < N; ++c)
#pragma unroll
        for (int a = 0; a < N; ++a) {
          const int q = c * N + a;
          const float g0 = G[q], g1 = G[N3 + q], g2 = G[2 * N3 + q], g3 = G[3 * N3 + q],
                      g4 = G[4 * N3 + q], g5 = G[5 * N3 + q];
          const float vx = gx[c][a], vy = gy[c][a], vz = gz[c][a];
          float tx = vx * g0 + vy * g3 + vz * g4;
          float ty = vx * g3 + vy * g1 + vz * g5;
          float tz = vx * g4 + vy * g5 + vz * g2;
          if (KAPPA) {
            const float kq = G[6 * N3 + q];
            tx *= kq;
            ty *= kq;
            tz *= kq;
          }
          gx[c][a] = tx;
          gy[c][a] = ty;
          gz[c][a] = tz;
        }
      fence_proxy_async_smem();
      __syncwarp();
      const long long next = batch + nw;
      if (lane == 0 && next < nbatch) {
        const long long o0 = next * CPW;
        const int nv = (int)min((long long)CPW, A.count - o0);
        const uint32_t bytes = (uint32_t)(nv * A.gstride * 4);
        mbar_arrive_expect_tx(bar, bytes);
        tma_load_1d(geo_s, A.geo + (A.color_base + o0) * A.gstride, bytes, bar);
      }
    } else {
      const float wr = A.w[r];
#pragma unroll
      for (int c = 0; c < N; ++c)
#pragma unroll
        for (int a = 0; a < N; ++a) {
          const float wq = A.w[a] * wr * A.w[c];
          gx[c][a] *= A.aff[0] * wq;
          gy[c][a] *= A.aff[1] * wq;
          gz[c][a] *= A.aff[2] * wq;
        }
    }
    // ---- D_x^T t_x + D_z^T t_z (XZ); t_y and that sum to XY ----
    float r1[N][N];
#pragma unroll
    for (int c = 0; c < N; ++c) eo_apply<N, -1>(A.DT, gx[c], r1[c]);
    sweep_cols<N, -1>(A.DT, gz);
#pragma unroll
    for (int c = 0; c < N; ++c)
#pragma unroll
      for (int a = 0; a < N; ++a) r1[c][a] += gz[c][a];
    if (active) {
#pragma unroll
      for (int c = 0; c < N; ++c)
#pragma unroll
        for (int a = 0; a < N; ++a) {
          Ak[c * PS + r * N + a] = gy[c][a];
          Bk[c * PS + r * N + a] = r1[c][a];
        }
    }
    __syncwarp();
#pragma unroll
    for (int b = 0; b < N; ++b)
#pragma unroll
      for (int a = 0; a < N; ++a) {
        u[b][a] = Ak[r * PS + b * N + a];
        gx[b][a] = Bk[r * PS + b * N + a];
      }
    sweep_cols<N, -1>(A.DT, u);
#pragma unroll
    for (int b = 0; b < N; ++b)
#pragma unroll
      for (int a = 0; a < N; ++a) u[b][a] += gx[b][a];
    sweep_cols<N, 1>(A.ST, u);
#pragma unroll
    for (int b = 0; b < N; ++b) eo_apply<N, 1>(A.ST, u[b], u[b]);
    // ---- XY -> XZ, S_z^T ----
    if (active) {
#pragma unroll
      for (int b = 0; b < N; ++b)
#pragma unroll
        for (int a = 0; a < N; ++a) Ak[r * PS + b * N + a] = u[b][a];
    }
    __syncwarp();
#pragma unroll
    for (int c = 0; c < N; ++c)
#pragma unroll
      for (int a = 0; a < N; ++a) w[c][a] = Ak[c * PS + r * N + a];
    sweep_cols<N, 1>(A.ST, w);

    // ---- scatter the xz-plane b = r: first colour stores, later ones add ----
    if (!y_ready) {
      pdl_wait();
      y_ready = true;
    }
    if (valid) {
      const long long Y = (long long)cj * P + r;
      const bool yb = dir && (Y == 0 || Y == A.Ny - 1);
      const int my = ((r == 0 && cj > 0) || (r == P && cj < A.nc[1] - 1)) ? 2 : 0;
      const int mxl = ci > 0 ? 1 : 0, mxr = ci < A.nc[0] - 1 ? 1 : 0;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const long long Z = (long long)ck * P + c;
        const bool zb = yb || (dir && (Z == 0 || Z == A.Nz - 1));
        const int mz = ((c == 0 && ck > 0) || (c == P && ck < A.nc[2] - 1)) ? 4 : 0;
        const long long row = (Z * A.Ny + Y) * A.Nx + X0;
        float *dst = A.y + row;
#pragma unroll
        for (int a = 0; a < N; ++a) {
          const bool bnd = zb || (a == 0 && xl) || (a == P && xr);
          const int mx = a == 0 ? mxl : (a == P ? mxr : 0);
          if (bnd) {
            dst[a] = __ldg(A.x + row + a);
          } else if (A.color & (mx | my | mz)) {
            dst[a] += w[c][a];
          } else {
            dst[a] = w[c][a];
          }
        }
      }
    }
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

// natural geometry (FP64 [cell][6][n^3] with stride s64, points a + n b +
// n^2 c) and optional kappa -> colour-major FP32 plane layout
template <int N>
__global__ void plane_repack_kernel(const double *__restrict__ G, long long s64,
                                    const double *__restrict__ kap, float *__restrict__ out,
                                    long long gstride, int ncomp, int nx, int ny, int nz,
                                    const long long *__restrict__ cbase)
{
  constexpr int N2 = N * N, N3 = N * N * N;
  const long long C = (long long)nx * ny * nz;
  const long long total = C * ncomp * N3;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < total;
       s += (long long)gridDim.x * blockDim.x) {
    const long long cell = s / (ncomp * N3);
    const int rem = int(s - cell * ncomp * N3);
    const int e = rem / N3, q = rem % N3; // q = a + N b + N^2 c (natural)
    const int a = q % N, b = (q / N) % N, c = q / N2;
    const int i = int(cell % nx), j = int((cell / nx) % ny), k = int(cell / ((long long)nx * ny));
    const int color = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2);
    const int mx = (nx - (i & 1) + 1) / 2, my = (ny - (j & 1) + 1) / 2;
    const long long ord = cbase[color] + (i >> 1) + (long long)mx * ((j >> 1) + (long long)my * (k >> 1));
    const double v = e < 6 ? G[cell * s64 + e * N3 + q] : kap[cell * N3 + q];
    out[ord * gstride + e * N3 + b * N2 + c * N + a] = float(v);
  }
}

template <int N>
int plane_vmult_impl(const sf_op *op, const float *x, float *y, cudaStream_t st)
{
  using Cfg = PlaneCfg<N>;
  PlaneArgs<N> A{};
  const Shape1D &s = op->shape;
  A.S = eo_of<N, float>(s.S, false);
  A.ST = eo_of<N, float>(s.S, true);
  A.D = eo_of<N, float>(s.D, false);
  A.DT = eo_of<N, float>(s.D, true);
  for (int i = 0; i < N; ++i) A.w[i] = float(s.wq[i]);
  for (int d = 0; d < 3; ++d) A.nc[d] = op->desc.n_cells[d];
  A.Nx = (long long)(N - 1) * A.nc[0] + 1;
  A.Ny = (long long)(N - 1) * A.nc[1] + 1;
  A.Nz = (long long)(N - 1) * A.nc[2] + 1;
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  for (int d = 0; d < 3; ++d) A.aff[d] = float(jxw / (op->h[d] * op->h[d]));
  A.dirichlet = op->desc.dirichlet;
  A.x = x;
  A.y = y;
  A.err = (int *)op->dev_err.ptr;
  const bool affine = !op->deformed;
  const bool kap = op->has_kappa;
  A.geo = (const float *)op->geoP.ptr;
  A.gstride = op->geoP_stride;
  if (op->deformed && !A.geo) {
    set_error("plane kernel geometry missing");
    return SF_ERR_STATE;
  }
  void (*kern)(const PlaneArgs<N>);
  if (affine) {
    if (kap) {
      set_error("kappa on an affine mesh needs the geometry path");
      return SF_ERR_STATE;
    }
    kern = plane_vmult_kernel<N, true, false>;
  } else {
    kern = kap ? plane_vmult_kernel<N, false, true> : plane_vmult_kernel<N, false, false>;
  }
  const long long geo_f = affine ? 0 : Cfg::CPW * A.gstride;
  const long long region = (geo_f + 2 * Cfg::CPW * Cfg::CS + 31) / 32 * 32;
  const size_t smem = 128 + size_t(Cfg::WARPS) * region * sizeof(float);
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
  int per_sm = 0;
  SF_RET_IF(resident_blocks_per_sm((const void *)kern, 32 * Cfg::WARPS, smem, &per_sm));
  if (per_sm < 1) per_sm = 1;
  int n_sm = 0, dev = 0;
  SF_CUDA_TRY(cudaGetDevice(&dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  long long cbase = 0;
  for (int color = 0; color < 8; ++color) {
    A.color = color;
    A.cx = color & 1;
    A.cy = (color >> 1) & 1;
    A.cz = (color >> 2) & 1;
    A.mx = (A.nc[0] - A.cx + 1) / 2;
    A.my = (A.nc[1] - A.cy + 1) / 2;
    const int mz = (A.nc[2] - A.cz + 1) / 2;
    A.count = (long long)A.mx * A.my * mz;
    A.color_base = cbase;
    cbase += A.count;
    if (A.count == 0) continue;
    const long long nbatch = (A.count + Cfg::CPW - 1) / Cfg::CPW;
    long long blocks = std::min<long long>((nbatch + Cfg::WARPS - 1) / Cfg::WARPS, (long long)per_sm * n_sm);
    const long long stride = blocks * Cfg::WARPS * Cfg::CPW;
    A.step_i = int(stride % A.mx);
    A.step_j = int((stride / A.mx) % A.my);
    A.step_k = int(stride / ((long long)A.mx * A.my));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(32 * Cfg::WARPS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    // colours 1..7 overlap with their predecessor (they read x and the
    // geometry before griddepcontrol.wait and touch y only after it); the
    // first colour is ordered normally behind whatever produced x
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
int plane_repack_impl(sf_op *op, const double *G64, long long s64, const double *kap64, cudaStream_t st)
{
  const int ncomp = kap64 ? 7 : 6;
  const long long gs = plane_geo_stride(N, ncomp);
  const size_t bytes = (size_t)op->n_cells * gs * sizeof(float);
  if (op->geoP.bytes != bytes) {
    int e = op->geoP.alloc(bytes);
    if (e) return e;
  }
  SF_CUDA_TRY(cudaMemsetAsync(op->geoP.ptr, 0, bytes, st)); // padding words defined
  op->geoP_stride = gs;
  long long cb[8], acc = 0;
  const int nx = op->desc.n_cells[0], ny = op->desc.n_cells[1], nz = op->desc.n_cells[2];
  for (int color = 0; color < 8; ++color) {
    const int cx = color & 1, cy = (color >> 1) & 1, cz = (color >> 2) & 1;
    cb[color] = acc;
    acc += (long long)((nx - cx + 1) / 2) * ((ny - cy + 1) / 2) * ((nz - cz + 1) / 2);
  }
  DevBuf cbd;
  int e = cbd.alloc(sizeof(cb));
  if (e) return e;
  SF_CUDA_TRY(cudaMemcpyAsync(cbd.ptr, cb, sizeof(cb), cudaMemcpyHostToDevice, st));
  plane_repack_kernel<N><<<152 * 16, 256, 0, st>>>(G64, s64, kap64, (float *)op->geoP.ptr, gs, ncomp, nx, ny,
                                                   nz, (const long long *)cbd.ptr);
  SF_CUDA_TRY(cudaGetLastError());
  SF_CUDA_TRY(cudaStreamSynchronize(st));
  return SF_OK;
}

} // namespace

bool plane_path(const sf_op *op, int prec)
{
  return op->kernel_variant == SF_KERNEL_PLANE && prec == SF_FP32 && op->desc.kind == SF_OP_LAPLACE &&
         op->n <= 5 && (op->deformed || !op->has_kappa);
}

int launch_cont_vmult_plane(const sf_op *op, const float *x, float *y, cudaStream_t st)
{
  switch (op->n) {
  case 2: return plane_vmult_impl<2>(op, x, y, st);
  case 3: return plane_vmult_impl<3>(op, x, y, st);
  case 4: return plane_vmult_impl<4>(op, x, y, st);
  case 5: return plane_vmult_impl<5>(op, x, y, st);
  default: set_error("plane kernel covers degrees 1..4"); return SF_ERR_UNSUPPORTED;
  }
}

int repack_plane_geometry(sf_op *op, const double *G64, long long s64, const double *kap64, cudaStream_t st)
{
  switch (op->n) {
  case 2: return plane_repack_impl<2>(op, G64, s64, kap64, st);
  case 3: return plane_repack_impl<3>(op, G64, s64, kap64, st);
  case 4: return plane_repack_impl<4>(op, G64, s64, kap64, st);
  case 5: return plane_repack_impl<5>(op, G64, s64, kap64, st);
  default: return SF_OK;
  }
}

} // namespace sf
