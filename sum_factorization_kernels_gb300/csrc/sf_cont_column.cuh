// sf_cont_column.cuh -- node bookkeeping of one z column of a cell in the
// continuous (lexicographic) numbering, shared by the line-ownership and
// paired Laplacian kernels.
//
// Node (X, Y, Z) of the (p nx + 1) x (p ny + 1) x (p nz + 1) node grid has
// index (Z Ny + Y) Nx + X.  The thread that owns the z column (a, b) of cell
// (ci, cj, ck) touches the nodes X = ci p + a, Y = cj p + b, Z = ck p + c,
// c = 0..p: a base pointer plus c times the node-plane size, a 32-bit offset
// (the plane size times p + 1 is limited to 2^31 at operator creation).
//
// Two bit masks over c describe what the column does with its nodes:
//   keep: the node is free.  Homogeneous Dirichlet nodes (on the domain
//         boundary when Dirichlet conditions are on) read as zero and are
//         written as y = x: identity rows and columns of the constrained
//         operator.  (The reference applies cell operators only; the global
//         numbering and the constraint treatment are this library's.)
//   add:  the node is shared with a cell of a lower colour.  Cells of colour
//         (ci & 1) | (cj & 1) << 1 | (ck & 1) << 2 run in colour order; the
//         first cell to touch a node stores, later ones add.  A node on the
//         x (y, z) face of the cell with a neighbour across that face is
//         shared with the neighbour, whose colour differs in bit 0 (1, 2),
//         and that neighbour ran first when this colour has the bit set.
#pragma once

#include <cuda_runtime.h>

namespace sf {

struct ColumnMask {
  unsigned keep, add;
};

template <int N>
__device__ __forceinline__ ColumnMask column_mask(int a, int b, int ci, int cj, int ck, const int (&nc)[3],
                                                  int color, bool dirichlet, bool valid)
{
  constexpr int P = N - 1;
  constexpr unsigned FULL = (1u << N) - 1;
  unsigned keep = valid ? FULL : 0u;
  if (dirichlet) {
    const bool side = (a == 0 && ci == 0) || (a == P && ci == nc[0] - 1) || (b == 0 && cj == 0) ||
                      (b == P && cj == nc[1] - 1);
    if (side) keep = 0u;
    keep &= ~((ck == 0 ? 1u : 0u) | (ck == nc[2] - 1 ? (1u << P) : 0u));
  }
  const int mxy = ((a == 0 && ci > 0) || (a == P && ci < nc[0] - 1) ? 1 : 0) |
                  ((b == 0 && cj > 0) || (b == P && cj < nc[1] - 1) ? 2 : 0);
  unsigned add = (color & mxy) ? FULL : 0u;
  if (color & 4) add |= (ck > 0 ? 1u : 0u) | (ck < nc[2] - 1 ? (1u << P) : 0u);
  return ColumnMask{keep, valid ? add : 0u};
}

// offset of node (0, 0, 0) of cell (ci, cj, ck)
template <int N>
__device__ __forceinline__ long long cell_node_base(int ci, int cj, int ck, int nx_nodes, int plane)
{
  constexpr int P = N - 1;
  return (long long)(ck * P) * plane + (cj * P) * nx_nodes + ci * P;
}

// v[c] = x of node c of the column, zero for fixed and absent nodes
template <int N, typename T>
__device__ __forceinline__ void gather_column(const T *__restrict__ xc, int plane, unsigned keep, T (&v)[N])
{
#pragma unroll
  for (int c = 0; c < N; ++c) v[c] = ((keep >> c) & 1u) ? __ldg(xc + c * plane) : T(0);
}

// store or add the column's results; fixed nodes get y = x
template <int N, typename T>
__device__ __forceinline__ void scatter_column(T *yc, const T *__restrict__ xc, int plane, ColumnMask m,
                                               const T (&v)[N])
{
#pragma unroll
  for (int c = 0; c < N; ++c) {
    T *p = yc + c * plane;
    T val = v[c];
    if ((m.add >> c) & 1u) val += *p;
    if (!((m.keep >> c) & 1u)) val = __ldg(xc + c * plane);
    *p = val;
  }
}

// y values the column adds to (zero where it stores first or is absent)
template <int N, typename T>
__device__ __forceinline__ void load_column_sums(const T *yc, int plane, unsigned add, T (&yo)[N])
{
#pragma unroll
  for (int c = 0; c < N; ++c) yo[c] = ((add >> c) & 1u) ? yc[c * plane] : T(0);
}

// write the column's results given the prefetched sums; fixed nodes get y = x
template <int N, typename T>
__device__ __forceinline__ void store_column(T *yc, const T *__restrict__ xc, int plane, unsigned keep,
                                             const T (&v)[N], const T (&yo)[N])
{
#pragma unroll
  for (int c = 0; c < N; ++c) {
    T val = v[c] + yo[c];
    if (!((keep >> c) & 1u)) val = __ldg(xc + c * plane);
    yc[c * plane] = val;
  }
}

} // namespace sf
