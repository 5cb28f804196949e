// sf_internal.h -- shared declarations of the sfgpu library (host side).
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/sfgpu.h"

struct sf_op;

namespace sf {

constexpr int kMaxDegree = 8;
constexpr int kMaxN = kMaxDegree + 1;

// FP64 1D tables of one degree and basis (see sf_basis.cpp)
struct Shape1D {
  int degree, n, basis;
  double xq[kMaxN], wq[kMaxN], xgll[kMaxN];
  double S[kMaxN][kMaxN];    // S[q][i]    = phi_i(xq_q)
  double D[kMaxN][kMaxN];    // D[q][j]    = l_j'(xq_q)   (Gauss-Lagrange)
  double Sinv[kMaxN][kMaxN]; // Sinv[i][q] = l_q(xgll_i)
  double fv[2][kMaxN];       // l_j(0), l_j(1)
  double fd[2][kMaxN];       // l_j'(0), l_j'(1)
  double hermite_d0;         // phi_0'(0) of the Hermite-like basis
};

void gauss_points(int n, double *x, double *w);
void gll_points(int n, double *x);
int fill_shape(int degree, int basis, Shape1D &s);

// thread-local error text for sf_last_error()
void set_error(const std::string &msg);

// the byte ranges [a, a + bytes) and [b, b + bytes) share an address: an
// output that overlaps an input of an apply is read by other threads after
// they wrote it (neighbour values, the fused epilogues), so it is rejected
inline bool ranges_overlap(const void *a, const void *b, size_t bytes)
{
  const uintptr_t pa = reinterpret_cast<uintptr_t>(a), pb = reinterpret_cast<uintptr_t>(b);
  return pa < pb + bytes && pb < pa + bytes;
}

// drops the cached preconditioner state of a handle (sf_solver.cu)
void release_solver_cache(sf_op *op);

// device buffer owned by a handle
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  int alloc(size_t b);
  void release();
  ~DevBuf() { release(); }
};

// NVTX range around one library call, named after the LIKWID region the
// reference's drivers put around the same operation
// (legacy/src/test_program.cc:107-109: cell_laplacian_deg_<p>;
// legacy/include/evaluation_dg_laplacian.h:525-529:
// real_dg_laplacian_3d_deg_<p>{mv,ch}; legacy/include/evaluation_dg_advect.h:
// 693-695: dg_advect_3d_deg_<p>{mv,rk})
struct Region {
  explicit Region(const char *name) { nvtxRangePushA(name); }
  ~Region() { nvtxRangePop(); }
  Region(const Region &) = delete;
  Region &operator=(const Region &) = delete;
};

} // namespace sf

// unstructured-mesh data of a SF_OP_LAPLACE_UNSTRUCTURED handle
struct sf_unstructured {
  sf::DevBuf idx;                     // [cell][n^3] node indices (int32)
  sf::DevBuf masks;                   // [cell][n^2] keep / add bits (uint32)
  sf::DevBuf cells;                   // cells grouped by colour (int32)
  std::vector<long long> color_start; // colour c: cells[color_start[c] .. color_start[c+1])
  long long n_nodes = 0;
};

// the opaque handle
struct sf_op {
  sf_desc desc;
  sf::Shape1D shape;
  long long n_dofs = 0, n_cells = 0;
  int n = 0;                    // degree + 1
  long long geo_stride = 0;     // entries per cell in the geometry arrays
  bool deformed = false;
  sf::DevBuf geo64, geo32;      // [cell][6][n^3] (+pad) merged tensors
  sf::DevBuf kap64, kap32;      // [cell][n^3] coefficient
  bool has_kappa = false;
  sf::DevBuf scratch;           // operator-private scratch (transpose, M^-1)
  sf::DevBuf kron;              // work vectors of the Kronecker passes (affine continuous operators)
  sf::DevBuf geoLine64, geoLine32; // geometry in the line kernel's walk order
  std::unique_ptr<sf_unstructured> unstr; // SF_OP_LAPLACE_UNSTRUCTURED only
  sf::DevBuf dev_err;           // device error flags (bounded waits)
  int kernel_variant = 0;       // sf_kernel_variant
  char region_mv[48] = {};      // NVTX names of the apply and of the smoother /
  char region_ch[48] = {};      // Runge-Kutta step (sf::Region)
  double h[3];
};

#define SF_CUDA_TRY(call)                                                     \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      sf::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
      return SF_ERR_CUDA;                                                     \
    }                                                                         \
  } while (0)
