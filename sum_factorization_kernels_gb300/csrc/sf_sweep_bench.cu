// sf_sweep_bench.cu -- the shared-memory slab sweeps of the operator
// kernels, timed in isolation with three arithmetic paths, to decide
// between CUDA cores and tensor cores for the 1D contractions
// (matrix_vector_kernel.h:30-185 applied along x and y lines):
//   SF_SWEEP_EO_FP32 / SF_SWEEP_EO_FP64: one thread per line, the even-odd
//     contraction with constant-bank coefficients (as in the operators);
//   SF_SWEEP_MMA_TF32X3: one warp per 16 lines, mma.sync m16n8k8 with TF32
//     operands and FP32 accumulation, each operand split into a TF32 high
//     part and a TF32 remainder, D = A_hi B_hi + A_hi B_lo + A_lo B_hi
//     (FP32-level accuracy; three tensor-core products per tile);
//   SF_SWEEP_MMA_TF32: the same with A_hi B_hi only (TF32 accuracy).
// A block holds CPB cells (CPB n^2 <= 128 lines) in two shared slabs; each
// round applies the interpolation matrix S along x (slab 0 -> 1) and along y
// (slab 1 -> 0).  The input cells are read from and the result written back
// to global memory once per launch.
#include <cstring>

#include "sf_device.cuh"
#include "sf_internal.h"
#include "sf_launch.h"
#include "sf_tables.h"

namespace sf {

namespace {

constexpr int kSweepThreads = 128;

template <int N>
struct SweepCfg {
  static constexpr int N2 = N * N, N3 = N * N * N;
  static constexpr int CPB = kSweepThreads / N2 > 0 ? kSweepThreads / N2 : 1;
  static constexpr int LINES = CPB * N2;
  static constexpr int YS = N % 2 == 1 ? N : N + 1; // odd line stride: x lines conflict-free
  static constexpr int ZS = N * YS;
  static constexpr int CS = N * ZS + 1;
  static constexpr int KT = (N + 7) / 8;             // k steps and n tiles of m16n8k8
};

template <int N, typename T>
struct SweepArgs {
  EOMat<N, T> S;
  float bhi[16][16], blo[16][16]; // B[k][j] = S[j][k], split into TF32 high part and remainder
  const T *__restrict__ in;
  T *__restrict__ out;
  long long n_cells;
  int rounds;
};

__device__ __forceinline__ uint32_t to_tf32(float v)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// slab offset of entry m of line l: x lines (dir 0) run along x at (c, z, y),
// y lines (dir 1) along y at (c, z, x); lines are numbered cell-major
template <int N>
__device__ __forceinline__ int line_base(int l, int dir)
{
  using C = SweepCfg<N>;
  const int c = l / C::N2, r = l - c * C::N2, z = r / N, w = r - z * N;
  return c * C::CS + z * C::ZS + (dir == 0 ? w * C::YS : w);
}

template <int N>
__device__ __forceinline__ int line_stride(int dir) { return dir == 0 ? 1 : SweepCfg<N>::YS; }

// one sweep on the CUDA cores: thread t owns line t
template <int N, typename T>
__device__ __forceinline__ void sweep_eo(const SweepArgs<N, T> &A, const T *src, T *dst, int dir)
{
  using C = SweepCfg<N>;
  const int t = threadIdx.x;
  if (t < C::LINES) {
    const int b = line_base<N>(t, dir), s = line_stride<N>(dir);
    T v[N];
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = src[b + s * m];
    eo_apply<N, 1>(A.S, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m) dst[b + s * m] = v[m];
  }
}

// one sweep on the tensor cores: warp w takes the 16-line tiles w, w + 4, ...
template <int N, int PASSES>
__device__ __forceinline__ void sweep_mma(const SweepArgs<N, float> &A, const uint32_t (&bh)[2][2][2],
                                          const uint32_t (&bl)[2][2][2], const float *src, float *dst, int dir)
{
  using C = SweepCfg<N>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, q = lane & 3;
  const int s = line_stride<N>(dir);
  constexpr int TILES = (C::LINES + 15) / 16;
  for (int tile = warp; tile < TILES; tile += kSweepThreads / 32) {
    const int l0 = tile * 16 + g, l1 = l0 + 8;
    const bool v0 = l0 < C::LINES, v1 = l1 < C::LINES;
    const int b0 = v0 ? line_base<N>(l0, dir) : 0, b1 = v1 ? line_base<N>(l1, dir) : 0;
    float d[C::KT][4];
#pragma unroll
    for (int nt = 0; nt < C::KT; ++nt) d[nt][0] = d[nt][1] = d[nt][2] = d[nt][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < C::KT; ++kt) {
      const int k0 = kt * 8 + q, k1 = k0 + 4;
      const float x00 = (v0 && k0 < N) ? src[b0 + s * k0] : 0.f, x10 = (v1 && k0 < N) ? src[b1 + s * k0] : 0.f;
      const float x01 = (v0 && k1 < N) ? src[b0 + s * k1] : 0.f, x11 = (v1 && k1 < N) ? src[b1 + s * k1] : 0.f;
      uint32_t ah[4] = {to_tf32(x00), to_tf32(x10), to_tf32(x01), to_tf32(x11)};
      uint32_t al[4];
      if (PASSES == 3) {
        al[0] = to_tf32(x00 - __uint_as_float(ah[0]));
        al[1] = to_tf32(x10 - __uint_as_float(ah[1]));
        al[2] = to_tf32(x01 - __uint_as_float(ah[2]));
        al[3] = to_tf32(x11 - __uint_as_float(ah[3]));
      }
#pragma unroll
      for (int nt = 0; nt < C::KT; ++nt) {
        if (PASSES == 3) {
          mma_tf32(d[nt], al, bh[kt][nt][0], bh[kt][nt][1]);
          mma_tf32(d[nt], ah, bl[kt][nt][0], bl[kt][nt][1]);
        }
        mma_tf32(d[nt], ah, bh[kt][nt][0], bh[kt][nt][1]);
      }
    }
#pragma unroll
    for (int nt = 0; nt < C::KT; ++nt) {
      const int j0 = nt * 8 + 2 * q, j1 = j0 + 1;
      if (v0 && j0 < N) dst[b0 + s * j0] = d[nt][0];
      if (v0 && j1 < N) dst[b0 + s * j1] = d[nt][1];
      if (v1 && j0 < N) dst[b1 + s * j0] = d[nt][2];
      if (v1 && j1 < N) dst[b1 + s * j1] = d[nt][3];
    }
  }
}

template <int N, typename T, int METHOD>
__global__ void __launch_bounds__(kSweepThreads) sweep_bench_kernel(const __grid_constant__ SweepArgs<N, T> A)
{
  using C = SweepCfg<N>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *s0 = reinterpret_cast<T *>(smem_raw), *s1 = s0 + C::CPB * C::CS;
  const long long cell0 = (long long)blockIdx.x * C::CPB;
  // load the block's cells (cell-major n^3, x fastest)
  for (int i = threadIdx.x; i < C::CPB * C::N3; i += kSweepThreads) {
    const int c = i / C::N3, r = i - c * C::N3, z = r / C::N2, y = (r / N) % N, x = r % N;
    const long long cell = cell0 + c;
    s0[c * C::CS + z * C::ZS + y * C::YS + x] = cell < A.n_cells ? A.in[cell * C::N3 + r] : T(0);
  }
  uint32_t bh[2][2][2] = {}, bl[2][2][2] = {};
  if (METHOD == SF_SWEEP_MMA_TF32X3 || METHOD == SF_SWEEP_MMA_TF32) {
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int kt = 0; kt < C::KT; ++kt)
#pragma unroll
      for (int nt = 0; nt < C::KT; ++nt) {
        bh[kt][nt][0] = __float_as_uint(A.bhi[kt * 8 + q][nt * 8 + g]);
        bh[kt][nt][1] = __float_as_uint(A.bhi[kt * 8 + q + 4][nt * 8 + g]);
        bl[kt][nt][0] = __float_as_uint(A.blo[kt * 8 + q][nt * 8 + g]);
        bl[kt][nt][1] = __float_as_uint(A.blo[kt * 8 + q + 4][nt * 8 + g]);
      }
  }
  __syncthreads();
  for (int r = 0; r < A.rounds; ++r) {
    for (int dir = 0; dir < 2; ++dir) {
      const T *src = dir == 0 ? s0 : s1;
      T *dst = dir == 0 ? s1 : s0;
      if constexpr (METHOD == SF_SWEEP_EO_FP32 || METHOD == SF_SWEEP_EO_FP64) {
        sweep_eo<N, T>(A, src, dst, dir);
      } else if constexpr (METHOD == SF_SWEEP_MMA_TF32X3) {
        sweep_mma<N, 3>(A, bh, bl, src, dst, dir);
      } else {
        sweep_mma<N, 1>(A, bh, bl, src, dst, dir);
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < C::CPB * C::N3; i += kSweepThreads) {
    const int c = i / C::N3, r = i - c * C::N3, z = r / C::N2, y = (r / N) % N, x = r % N;
    const long long cell = cell0 + c;
    if (cell < A.n_cells) A.out[cell * C::N3 + r] = s0[c * C::CS + z * C::ZS + y * C::YS + x];
  }
}

template <int N, typename T, int METHOD>
int sweep_bench_impl(const Shape1D &sh, long long n_cells, int rounds, const void *in, void *out, cudaStream_t st)
{
  using C = SweepCfg<N>;
  SweepArgs<N, T> A{};
  A.S = eo_of<N, T>(sh.S, false);
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j) {
      const float v = float(sh.S[j][k]);
      // TF32 high part: round the mantissa to 10 bits (nearest, ties away)
      uint32_t u;
      std::memcpy(&u, &v, 4);
      u = (u + 0x1000u) & 0xffffe000u;
      float hi;
      std::memcpy(&hi, &u, 4);
      A.bhi[k][j] = hi;
      float lo = float(double(sh.S[j][k]) - double(hi));
      std::memcpy(&u, &lo, 4);
      u = (u + 0x1000u) & 0xffffe000u;
      std::memcpy(&lo, &u, 4);
      A.blo[k][j] = lo;
    }
  A.in = (const T *)in;
  A.out = (T *)out;
  A.n_cells = n_cells;
  A.rounds = rounds;
  const size_t smem = 2 * size_t(C::CPB) * C::CS * sizeof(T);
  auto kern = sweep_bench_kernel<N, T, METHOD>;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long blocks = (n_cells + C::CPB - 1) / C::CPB;
  kern<<<(unsigned)blocks, kSweepThreads, smem, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N>
int sweep_bench_n(const Shape1D &sh, int method, long long n_cells, int rounds, const void *in, void *out,
                  cudaStream_t st)
{
  switch (method) {
  case SF_SWEEP_EO_FP32: return sweep_bench_impl<N, float, SF_SWEEP_EO_FP32>(sh, n_cells, rounds, in, out, st);
  case SF_SWEEP_MMA_TF32X3:
    return sweep_bench_impl<N, float, SF_SWEEP_MMA_TF32X3>(sh, n_cells, rounds, in, out, st);
  case SF_SWEEP_MMA_TF32: return sweep_bench_impl<N, float, SF_SWEEP_MMA_TF32>(sh, n_cells, rounds, in, out, st);
  default: return sweep_bench_impl<N, double, SF_SWEEP_EO_FP64>(sh, n_cells, rounds, in, out, st);
  }
}

} // namespace
} // namespace sf

extern "C" int sf_sweep_benchmark(int degree, int method, long long n_cells, int rounds, const void *in, void *out,
                                  void *stream)
{
  using namespace sf;
  if (!in || !out) {
    set_error("in/out is NULL");
    return SF_ERR_NULL;
  }
  if (degree < 1 || degree > kMaxDegree) {
    set_error("degree must be 1..8");
    return SF_ERR_UNSUPPORTED;
  }
  if (method < SF_SWEEP_EO_FP32 || method > SF_SWEEP_EO_FP64 || n_cells < 1 || n_cells >= (1LL << 31) ||
      rounds < 1 || rounds > 1024 || in == out) {
    set_error("invalid sweep benchmark arguments");
    return SF_ERR_INVALID;
  }
  const size_t es = method == SF_SWEEP_EO_FP64 ? sizeof(double) : sizeof(float);
  if (reinterpret_cast<uintptr_t>(in) % es || reinterpret_cast<uintptr_t>(out) % es) {
    set_error("in/out not aligned to the element size");
    return SF_ERR_ALIGN;
  }
  Shape1D sh;
  fill_shape(degree, SF_BASIS_GLL, sh);
  cudaStream_t st = (cudaStream_t)stream;
  switch (degree + 1) {
  case 2: return sweep_bench_n<2>(sh, method, n_cells, rounds, in, out, st);
  case 3: return sweep_bench_n<3>(sh, method, n_cells, rounds, in, out, st);
  case 4: return sweep_bench_n<4>(sh, method, n_cells, rounds, in, out, st);
  case 5: return sweep_bench_n<5>(sh, method, n_cells, rounds, in, out, st);
  case 6: return sweep_bench_n<6>(sh, method, n_cells, rounds, in, out, st);
  case 7: return sweep_bench_n<7>(sh, method, n_cells, rounds, in, out, st);
  case 8: return sweep_bench_n<8>(sh, method, n_cells, rounds, in, out, st);
  default: return sweep_bench_n<9>(sh, method, n_cells, rounds, in, out, st);
  }
}
