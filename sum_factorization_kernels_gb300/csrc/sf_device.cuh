// sf_device.cuh -- device building blocks shared by the operator kernels.
//
// The 1D contraction is the even-odd decomposition of an n x n matrix M that
// is centro-symmetric (M[n-1-i][n-1-j] = M[i][j], interpolation matrices) or
// anti-centro-symmetric (= -M[i][j], collocation derivatives).  With
// u+_j = u_j + u_{n-1-j}, u-_j = u_j - u_{n-1-j} (j < h = n/2):
//   A_i = sum_j E[i][j] u+_j + M[i][mid] u_mid     (n odd)
//   B_i = sum_j O[i][j] u-_j
//   out_i = A_i + B_i,  out_{n-1-i} = s (A_i - B_i)            (i < h)
//   out_mid = sum_j M[mid][j] u+_j + M[mid][mid] u_mid         (s = +1)
//           = sum_j M[mid][j] u-_j                              (s = -1)
// with E = (M[i][j] + M[i][n-1-j]) / 2, O = (M[i][j] - M[i][n-1-j]) / 2.
// This halves the multiplications of the plain n x n product, the same
// saving as the reference's apply_1d_matvec_kernel
// (matrix_vector_kernel.h:30-185), in a formulation that treats forward and
// transposed contractions alike (the transpose gets its own tables).
//
// All tables live in the kernel parameter block (constant bank) and are read
// with compile-time indices only, so every coefficient is a constant operand
// of an FMA; the per-thread data lives in registers.
#pragma once

#include <cuda_runtime.h>

namespace sf {

template <int N, typename T>
struct EOMat {
  static constexpr int H = N / 2;
  static constexpr int HH = H > 0 ? H : 1;
  T e[HH][HH];
  T o[HH][HH];
  T mc[HH]; // M[i][mid], i < H   (n odd)
  T mr[HH]; // M[mid][j], j < H   (n odd)
  T mm;     // M[mid][mid]
};

// out = M in  (in and out may alias)
template <int N, int SIGN, typename T>
__device__ __forceinline__ void eo_apply(const EOMat<N, T> &M, const T (&in)[N], T (&out)[N])
{
  constexpr int H = N / 2;
  constexpr int HH = H > 0 ? H : 1;
  T up[HH], um[HH];
#pragma unroll
  for (int j = 0; j < H; ++j) {
    up[j] = in[j] + in[N - 1 - j];
    um[j] = in[j] - in[N - 1 - j];
  }
  T res[N];
#pragma unroll
  for (int i = 0; i < H; ++i) {
    T a = (N % 2 == 1) ? M.mc[i] * in[H] : T(0);
#pragma unroll
    for (int j = 0; j < H; ++j) a = fma(M.e[i][j], up[j], a);
    T b = T(0);
#pragma unroll
    for (int j = 0; j < H; ++j) b = fma(M.o[i][j], um[j], b);
    res[i] = a + b;
    res[N - 1 - i] = SIGN > 0 ? a - b : b - a;
  }
  if (N % 2 == 1) {
    T m = SIGN > 0 ? M.mm * in[H] : T(0);
#pragma unroll
    for (int j = 0; j < H; ++j) m = fma(M.mr[j], SIGN > 0 ? up[j] : um[j], m);
    res[H] = m;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) out[i] = res[i];
}

// plain dot of a table row with a register line (face evaluation)
template <int N, typename T>
__device__ __forceinline__ T dot_row(const T (&row)[N], const T (&v)[N])
{
  T s = row[0] * v[0];
#pragma unroll
  for (int i = 1; i < N; ++i) s = fma(row[i], v[i], s);
  return s;
}

// Synchronise the threads of one cell group of G warps (NGROUPS groups per
// block).  A one-warp group uses __syncwarp (no hardware barrier); larger
// groups use named barriers 1..4 with compile-time ids, so a block reserves
// only NGROUPS + 1 of the SM's barriers (a register id would reserve all 16
// and cap residency); a block of one group needs no branch on the group.
template <int G, int NGROUPS = 4>
__device__ __forceinline__ void cell_group_sync(int grp)
{
  if (G == 1) {
    __syncwarp();
  } else if (NGROUPS == 1) {
    asm volatile("bar.sync 1, %0;" ::"n"(32 * G) : "memory");
  } else {
    constexpr int NT = 32 * G;
    if (grp == 0) asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
    else if (grp == 1) asm volatile("bar.sync 2, %0;" ::"n"(NT) : "memory");
    else if (grp == 2) asm volatile("bar.sync 3, %0;" ::"n"(NT) : "memory");
    else asm volatile("bar.sync 4, %0;" ::"n"(NT) : "memory");
  }
}

// Division of 32-bit unsigned integers by a runtime constant d >= 1 with one
// 64-bit high multiply: q = floor(m n / 2^64) with m = floor((2^64 - 1) / d)
// + 1 is exact for every n < 2^32 (Lemire, Kaser and Kurz, "Faster
// remainder by direct computation", Software: Practice and Experience
// 49(6), 2019).  d = 1 (m would be 2^64) is flagged by m = 0.
struct FastDiv {
  unsigned long long m;
};

__host__ __device__ inline FastDiv make_fast_div(unsigned d)
{
  return FastDiv{d == 1u ? 0ull : ~0ull / d + 1ull};
}

__device__ __forceinline__ unsigned fast_div(unsigned n, FastDiv f)
{
  return f.m == 0ull ? n : (unsigned)__umul64hi(f.m, (unsigned long long)n);
}

// cells per thread block for n^2 threads per cell (about 128-256 threads)
template <int N>
struct CellsPerBlock {
  static constexpr int value = N == 2 ? 32 : N == 3 ? 14 : N == 4 ? 8 : N == 5 ? 5
                               : N == 6 ? 7 : N == 7 ? 5 : N == 8 ? 2 : 3;
};

} // namespace sf
