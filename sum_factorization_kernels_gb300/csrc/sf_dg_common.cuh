// sf_dg_common.cuh -- block shape and shared-memory layout shared by the DG
// kernels (cell-major periodic Cartesian meshes, n^3 values per cell).
#pragma once

#include <cuda_runtime.h>

namespace sf {

template <int N>
struct DGCells {
  // cells per block, about 128-256 threads
  static constexpr int value = N == 2 ? 32 : N == 3 ? 14 : N == 4 ? 8 : N == 5 ? 5 : N == 6 ? 7
                               : N == 7 ? 5 : N == 8 ? 2 : 3;
};

// Shared-memory layout of the DG kernels: per cell three slabs with index
// (a, b, c) = a + P1 b + P2 c and a per-cell skew, chosen from a
// bank-conflict model of the three sweep patterns over the lanes of each
// warp (a block holds CPB consecutive cells, cell-major lanes).
struct DGLayout {
  int P1, P2, SKEW;
};

constexpr DGLayout dg_layout(int n, int elem)
{
  return elem == 4 ? (n == 2   ? DGLayout{2, 5, 6}
                      : n == 3 ? DGLayout{3, 9, 10}
                      : n == 4 ? DGLayout{4, 19, 12}
                      : n == 5 ? DGLayout{5, 25, 2}
                      : n == 6 ? DGLayout{7, 42, 8}
                      : n == 7 ? DGLayout{7, 56, 25}
                      : n == 8 ? DGLayout{9, 72, 0}
                               : DGLayout{9, 81, 6})
                   : (n == 2   ? DGLayout{2, 5, 6}
                      : n == 3 ? DGLayout{3, 18, 7}
                      : n == 4 ? DGLayout{4, 19, 0}
                      : n == 5 ? DGLayout{5, 25, 2}
                      : n == 6 ? DGLayout{9, 54, 8}
                      : n == 7 ? DGLayout{7, 49, 12}
                      : n == 8 ? DGLayout{9, 72, 0}
                               : DGLayout{9, 81, 6});
}

// periodic neighbour of the cell (ix, iy, iz) across face `side` of
// direction `dir` (no division: a +-1 step with wrap-around)
__device__ __forceinline__ long long periodic_neighbour(const int (&nc)[3], int ix, int iy, int iz, int dir,
                                                        int side)
{
  if (dir == 0) ix = side ? (ix + 1 == nc[0] ? 0 : ix + 1) : (ix == 0 ? nc[0] - 1 : ix - 1);
  if (dir == 1) iy = side ? (iy + 1 == nc[1] ? 0 : iy + 1) : (iy == 0 ? nc[1] - 1 : iy - 1);
  if (dir == 2) iz = side ? (iz + 1 == nc[2] ? 0 : iz + 1) : (iz == 0 ? nc[2] - 1 : iz - 1);
  return ((long long)iz * nc[1] + iy) * nc[0] + ix;
}

} // namespace sf
