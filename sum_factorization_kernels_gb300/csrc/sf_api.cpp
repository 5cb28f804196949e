// sf_api.cpp -- the C ABI (include/sfgpu.h): argument validation, handle
// state, dispatch to the kernel launchers.  No exception leaves this file.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include <algorithm>
#include <memory>
#include <vector>

#include "sf_internal.h"
#include "sf_launch.h"

namespace sf {

static thread_local std::string g_error;

void set_error(const std::string &msg) { g_error = msg; }

int DevBuf::alloc(size_t b)
{
  release();
  if (b == 0) return SF_OK;
  cudaError_t e = cudaMalloc(&ptr, b);
  if (e != cudaSuccess) {
    ptr = nullptr;
    (void)cudaGetLastError();
    set_error(std::string("cudaMalloc(") + std::to_string(b) + " bytes): " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SF_ERR_OOM : SF_ERR_CUDA;
  }
  bytes = b;
  return SF_OK;
}

void DevBuf::release()
{
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

} // namespace sf

using namespace sf;

namespace {

int fail(int code, const std::string &msg)
{
  set_error(msg);
  return code;
}

size_t elem_size(int prec) { return prec == SF_FP64 ? sizeof(double) : sizeof(float); }

int check_prec(const sf_op *op, int prec)
{
  if (prec != SF_FP64 && prec != SF_FP32) return fail(SF_ERR_INVALID, "precision must be SF_FP64 or SF_FP32");
  const int bit = prec == SF_FP64 ? 1 : 2;
  if (op && !(op->desc.precisions & bit))
    return fail(SF_ERR_STATE, "precision not prepared by sf_create (desc.precisions)");
  return SF_OK;
}

bool is_cell_faces(int kind) { return kind == SF_OP_LAPLACE_FACES || kind == SF_OP_CONVECTION_FACES; }

// operators evaluated by the tensor-product kernel: the precomputed SIPG
// form, and the SIPG operator itself unless the cell-and-face kernel is
// selected (the two are the same Kronecker sum on Cartesian meshes)
bool tensor_form(const sf_op *op)
{
  return op->desc.kind == SF_OP_DG_PRECOMPUTED ||
         (op->desc.kind == SF_OP_DG_SIPG && op->kernel_variant != SF_KERNEL_GENERIC);
}

// DG advection as a sum of one-dimensional line operators (constant
// velocity, Cartesian cells) unless the cell-and-face kernel is selected
bool advect_tensor(const sf_op *op)
{
  return op->desc.kind == SF_OP_DG_ADVECT && op->kernel_variant != SF_KERNEL_GENERIC;
}

bool is_continuous(int kind)
{
  return kind == SF_OP_LAPLACE || kind == SF_OP_MASS || kind == SF_OP_CONVECTION ||
         kind == SF_OP_LAPLACE_UNSTRUCTURED;
}

int check_ptr(const void *p, int prec, const char *name)
{
  if (!p) return fail(SF_ERR_NULL, std::string(name) + " is NULL");
  if (reinterpret_cast<uintptr_t>(p) % elem_size(prec) != 0)
    return fail(SF_ERR_ALIGN, std::string(name) + " is not aligned to its element size");
  return SF_OK;
}

// NVTX names of a handle's calls, after the reference's LIKWID regions
void name_regions(sf_op *op)
{
  const int p = op->desc.degree;
  const int k = op->desc.kind;
  if (k == SF_OP_DG_SIPG || k == SF_OP_DG_PRECOMPUTED) {
    std::snprintf(op->region_mv, sizeof op->region_mv, "real_dg_laplacian_3d_deg_%dmv", p);
    std::snprintf(op->region_ch, sizeof op->region_ch, "real_dg_laplacian_3d_deg_%dch", p);
  } else if (k == SF_OP_DG_ADVECT) {
    std::snprintf(op->region_mv, sizeof op->region_mv, "dg_advect_3d_deg_%dmv", p);
    std::snprintf(op->region_ch, sizeof op->region_ch, "dg_advect_3d_deg_%drk", p);
  } else {
    std::snprintf(op->region_mv, sizeof op->region_mv, "cell_laplacian_deg_%d", p);
    std::snprintf(op->region_ch, sizeof op->region_ch, "cell_laplacian_deg_%d_cheby", p);
  }
}

#define SF_RET(x)                                                              \
  do {                                                                         \
    int r_ = (x);                                                              \
    if (r_ != SF_OK) return r_;                                                \
  } while (0)

// derived copies of the FP64 geometry: the walk-ordered blocks of the line
// kernel (each prepared precision) and the natural FP32 copy (diagonal,
// kappa gradient)
int derive_fp32_geometry(sf_op *op)
{
  if (!op->deformed) return SF_OK;
  if (op->desc.precisions & 1) SF_RET(pack_line_geometry(op, SF_FP64));
  if (!(op->desc.precisions & 2)) {
    SF_CUDA_TRY(cudaDeviceSynchronize());
    return SF_OK;
  }
  SF_RET(pack_line_geometry(op, SF_FP32));
  const size_t entries = (size_t)op->n_cells * op->geo_stride;
  if (op->geo32.bytes != entries * sizeof(float)) SF_RET(op->geo32.alloc(entries * sizeof(float)));
  SF_RET(launch_convert((long long)entries, SF_FP64, op->geo64.ptr, SF_FP32, op->geo32.ptr, 0));
  SF_CUDA_TRY(cudaDeviceSynchronize());
  return SF_OK;
}

// the FP64 geometry is always kept (it is the source of the FP32 copies)
int prepare_geometry(sf_op *op)
{
  const long long n3 = (long long)op->n * op->n * op->n;
  op->geo_stride = (6 * n3 + 3) / 4 * 4; // 16-byte aligned cell blocks in FP32
  const size_t entries = (size_t)op->n_cells * op->geo_stride;
  SF_RET(op->geo64.alloc(entries * sizeof(double)));
  SF_RET(launch_geometry(op, (double *)op->geo64.ptr, 0));
  SF_CUDA_TRY(cudaDeviceSynchronize());
  return derive_fp32_geometry(op);
}

} // namespace

extern "C" {

const char *sf_last_error(void) { return g_error.c_str(); }

const char *sf_version(void) { return "sfgpu 0.1 (sm_103a)"; }

int sf_create(const sf_desc *desc, sf_op **out)
{
  if (!desc || !out) return fail(SF_ERR_NULL, "desc/op is NULL");
  *out = nullptr;
  const sf_desc &d = *desc;
  if (d.kind < SF_OP_LAPLACE || d.kind > SF_OP_CONVECTION_FACES) return fail(SF_ERR_INVALID, "unknown operator kind");
  if (d.kind == SF_OP_LAPLACE_UNSTRUCTURED) return fail(SF_ERR_INVALID, "unstructured meshes: sf_create_unstructured");
  const bool cont = is_continuous(d.kind);
  if (d.degree < 1 || d.degree > kMaxDegree) return fail(SF_ERR_UNSUPPORTED, "degree must be 1..8");
  for (int k = 0; k < 3; ++k) {
    if (d.n_cells[k] < 1 || d.n_cells[k] > (1 << 20)) return fail(SF_ERR_INVALID, "n_cells out of range");
    if (!(d.length[k] > 0.0)) return fail(SF_ERR_INVALID, "length must be positive");
  }
  if ((d.precisions & 3) == 0) return fail(SF_ERR_INVALID, "precisions must select FP64 and/or FP32");
  if (cont && d.basis != SF_BASIS_GLL && d.basis != SF_BASIS_HERMITE) return fail(SF_ERR_INVALID, "unknown basis");
  if ((d.kind == SF_OP_MASS || d.kind == SF_OP_CONVECTION) && d.deform != 0.0)
    return fail(SF_ERR_UNSUPPORTED, "mass and convection operators: affine meshes only (deform = 0)");
  if (d.kind == SF_OP_DG_SIPG && !(d.penalty > 0.0)) return fail(SF_ERR_INVALID, "penalty must be positive");
  if (d.kind == SF_OP_LAPLACE && !(d.deform >= 0.0 && d.deform < 0.15))
    return fail(SF_ERR_INVALID, "deform amplitude must be in [0, 0.15) to keep the mapping invertible");
  sf_op *op = new (std::nothrow) sf_op();
  if (!op) return fail(SF_ERR_OOM, "host allocation failed");
  op->desc = d;
  const int basis = cont ? d.basis : (d.kind == SF_OP_DG_ADVECT ? SF_BASIS_GLL : SF_BASIS_HERMITE);
  op->desc.basis = basis;
  fill_shape(d.degree, basis, op->shape);
  op->n = d.degree + 1;
  name_regions(op);
  for (int k = 0; k < 3; ++k) op->h[k] = d.length[k] / d.n_cells[k];
  op->n_cells = (long long)d.n_cells[0] * d.n_cells[1] * d.n_cells[2];
  if (op->n_cells >= (1LL << 31)) {
    delete op;
    return fail(SF_ERR_INVALID, "more than 2^31 - 1 cells");
  }
  const long long n3 = (long long)op->n * op->n * op->n;
  if (cont)
    op->n_dofs = ((long long)d.degree * d.n_cells[0] + 1) * ((long long)d.degree * d.n_cells[1] + 1) *
                 ((long long)d.degree * d.n_cells[2] + 1);
  else
    op->n_dofs = op->n_cells * n3;
  if (op->n_dofs >= (1LL << 40)) {
    delete op;
    return fail(SF_ERR_INVALID, "problem too large");
  }
  // the Laplacian kernels address the nodes of a cell by 32-bit offsets
  // within the degree + 1 node planes that the cell spans
  if (cont &&
      ((long long)d.degree * d.n_cells[0] + 1) * ((long long)d.degree * d.n_cells[1] + 1) * (d.degree + 1) >=
          (1LL << 31)) {
    delete op;
    return fail(SF_ERR_INVALID, "node plane too large: (p nx + 1)(p ny + 1)(p + 1) must stay below 2^31");
  }
  {
    int r = op->dev_err.alloc(sizeof(int));
    if (r == SF_OK && cudaMemset(op->dev_err.ptr, 0, sizeof(int)) != cudaSuccess) r = SF_ERR_CUDA;
    if (r != SF_OK) {
      delete op;
      return r;
    }
  }
  if (d.kind == SF_OP_LAPLACE && d.deform > 0.0) {
    op->deformed = true;
    int r = prepare_geometry(op);
    if (r != SF_OK) {
      delete op;
      return r;
    }
  }
  if (kron_eligible(op)) {
    // work vectors of the Kronecker passes, for the wider prepared precision
    const size_t es = (d.precisions & 1) ? sizeof(double) : sizeof(float);
    int r = op->kron.alloc(size_t(kron_work_vectors(op)) * size_t(op->n_dofs) * es);
    if (r != SF_OK) {
      delete op;
      return r;
    }
  }
  *out = op;
  return SF_OK;
}

int sf_create_unstructured(int degree, int basis, long long n_cells, long long n_nodes, const int *cell_nodes,
                           const double *merged6, const unsigned char *dirichlet, int precisions, sf_op **out)
{
  if (!out || !cell_nodes || !merged6) return fail(SF_ERR_NULL, "op/cell_nodes/merged6 is NULL");
  *out = nullptr;
  if (degree < 1 || degree > kMaxDegree) return fail(SF_ERR_UNSUPPORTED, "degree must be 1..8");
  if (basis != SF_BASIS_GLL && basis != SF_BASIS_HERMITE) return fail(SF_ERR_INVALID, "unknown basis");
  if (n_cells < 1 || n_cells >= (1LL << 31) || n_nodes < 1 || n_nodes >= (1LL << 31))
    return fail(SF_ERR_INVALID, "n_cells and n_nodes must be in [1, 2^31)");
  if ((precisions & 3) == 0) return fail(SF_ERR_INVALID, "precisions must select FP64 and/or FP32");
  const int n = degree + 1, n2 = n * n, n3 = n * n * n;
  const long long ne = n_cells * n3;
  for (long long i = 0; i < ne; ++i)
    if (cell_nodes[i] < 0 || cell_nodes[i] >= n_nodes) return fail(SF_ERR_INVALID, "cell_nodes entry out of range");
  // a cell's columns write its nodes from different threads with one
  // store-or-add decision per node: a node listed twice would be written twice
  {
    std::vector<int> seen((size_t)n_nodes, -1);
    for (long long e = 0; e < n_cells; ++e)
      for (int q = 0; q < n3; ++q) {
        int &s = seen[(size_t)cell_nodes[e * n3 + q]];
        if (s == (int)e) return fail(SF_ERR_INVALID, "a cell lists the same node twice");
        s = (int)e;
      }
  }
  // greedy colouring: a cell takes the smallest colour no cell sharing one of
  // its nodes has; node -> cells in compressed rows
  std::vector<long long> start((size_t)n_nodes + 1, 0);
  for (long long i = 0; i < ne; ++i) ++start[(size_t)cell_nodes[i] + 1];
  for (long long v = 0; v < n_nodes; ++v) start[(size_t)v + 1] += start[(size_t)v];
  std::vector<int> node_cells((size_t)ne);
  {
    std::vector<long long> fill(start.begin(), start.end() - 1);
    for (long long e = 0; e < n_cells; ++e)
      for (int q = 0; q < n3; ++q) node_cells[(size_t)fill[(size_t)cell_nodes[e * n3 + q]]++] = (int)e;
  }
  std::vector<int> color((size_t)n_cells, -1), stamp(1024, -1);
  int n_colors = 0;
  for (long long e = 0; e < n_cells; ++e) {
    for (int q = 0; q < n3; ++q) {
      const int v = cell_nodes[e * n3 + q];
      for (long long k = start[(size_t)v]; k < start[(size_t)v + 1]; ++k) {
        const int c = color[(size_t)node_cells[(size_t)k]];
        if (c >= 0) stamp[(size_t)c] = (int)e;
      }
    }
    int c = 0;
    while (c < 1023 && stamp[(size_t)c] == (int)e) ++c;
    if (c >= 1023) return fail(SF_ERR_UNSUPPORTED, "mesh needs more than 1023 colours");
    color[(size_t)e] = c;
    n_colors = std::max(n_colors, c + 1);
  }
  // first colour to touch each node; keep / add bits per cell column
  std::vector<int> first((size_t)n_nodes, 1 << 30);
  for (long long e = 0; e < n_cells; ++e)
    for (int q = 0; q < n3; ++q) {
      int &f = first[(size_t)cell_nodes[e * n3 + q]];
      f = std::min(f, color[(size_t)e]);
    }
  std::vector<unsigned> masks((size_t)(n_cells * n2), 0u);
  for (long long e = 0; e < n_cells; ++e)
    for (int t = 0; t < n2; ++t) {
      unsigned m = 0;
      for (int z = 0; z < n; ++z) {
        const int v = cell_nodes[e * n3 + z * n2 + t];
        if (!(dirichlet && dirichlet[v])) m |= 1u << z;
        if (first[(size_t)v] < color[(size_t)e]) m |= 1u << (16 + z);
      }
      masks[(size_t)(e * n2 + t)] = m;
    }
  std::vector<long long> cstart((size_t)n_colors + 1, 0);
  for (long long e = 0; e < n_cells; ++e) ++cstart[(size_t)color[(size_t)e] + 1];
  for (int c = 0; c < n_colors; ++c) cstart[(size_t)c + 1] += cstart[(size_t)c];
  std::vector<int> cells((size_t)n_cells);
  {
    std::vector<long long> fill(cstart.begin(), cstart.end() - 1);
    for (long long e = 0; e < n_cells; ++e) cells[(size_t)fill[(size_t)color[(size_t)e]]++] = (int)e;
  }

  sf_op *op = new (std::nothrow) sf_op();
  if (!op) return fail(SF_ERR_OOM, "host allocation failed");
  std::unique_ptr<sf_op> guard(op);
  op->desc = sf_desc{};
  op->desc.kind = SF_OP_LAPLACE_UNSTRUCTURED;
  op->desc.degree = degree;
  op->desc.basis = basis;
  op->desc.dirichlet = dirichlet ? 1 : 0;
  op->desc.precisions = precisions;
  for (int k = 0; k < 3; ++k) {
    op->desc.n_cells[k] = 1;
    op->desc.length[k] = 1.0;
    op->h[k] = 1.0;
  }
  fill_shape(degree, basis, op->shape);
  op->n = n;
  name_regions(op);
  op->n_cells = n_cells;
  op->n_dofs = n_nodes;
  op->unstr.reset(new (std::nothrow) sf_unstructured());
  if (!op->unstr) return fail(SF_ERR_OOM, "host allocation failed");
  sf_unstructured &M = *op->unstr;
  M.n_nodes = n_nodes;
  M.color_start = cstart;
  SF_RET(op->dev_err.alloc(sizeof(int)));
  SF_CUDA_TRY(cudaMemset(op->dev_err.ptr, 0, sizeof(int)));
  SF_RET(M.idx.alloc(sizeof(int) * (size_t)ne));
  SF_CUDA_TRY(cudaMemcpy(M.idx.ptr, cell_nodes, sizeof(int) * (size_t)ne, cudaMemcpyHostToDevice));
  SF_RET(M.masks.alloc(sizeof(unsigned) * masks.size()));
  SF_CUDA_TRY(cudaMemcpy(M.masks.ptr, masks.data(), sizeof(unsigned) * masks.size(), cudaMemcpyHostToDevice));
  SF_RET(M.cells.alloc(sizeof(int) * cells.size()));
  SF_CUDA_TRY(cudaMemcpy(M.cells.ptr, cells.data(), sizeof(int) * cells.size(), cudaMemcpyHostToDevice));
  op->geo_stride = 6LL * n3;
  const size_t entries = (size_t)(n_cells * op->geo_stride);
  SF_RET(op->geo64.alloc(entries * sizeof(double)));
  SF_CUDA_TRY(cudaMemcpy(op->geo64.ptr, merged6, entries * sizeof(double), cudaMemcpyHostToDevice));
  if (precisions & 2) {
    SF_RET(op->geo32.alloc(entries * sizeof(float)));
    SF_RET(launch_convert((long long)entries, SF_FP64, op->geo64.ptr, SF_FP32, op->geo32.ptr, 0));
  }
  // the line kernel's walk-ordered geometry, colour by colour
  op->deformed = true;
  if (precisions & 1) SF_RET(pack_line_geometry(op, SF_FP64));
  if (precisions & 2) SF_RET(pack_line_geometry(op, SF_FP32));
  SF_CUDA_TRY(cudaDeviceSynchronize());
  *out = guard.release();
  return SF_OK;
}

int sf_destroy(sf_op *op)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  release_solver_cache(op);
  delete op;
  return SF_OK;
}

int sf_sizes(const sf_op *op, long long *n_dofs, long long *n_cells)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (n_dofs) *n_dofs = op->n_dofs;
  if (n_cells) *n_cells = op->n_cells;
  return SF_OK;
}

int sf_set_geometry(sf_op *op, const double *G)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (op->desc.kind != SF_OP_LAPLACE) return fail(SF_ERR_STATE, "geometry only for SF_OP_LAPLACE");
  SF_RET(check_ptr(G, SF_FP64, "merged6"));
  const long long n3 = (long long)op->n * op->n * op->n;
  op->geo_stride = (6 * n3 + 3) / 4 * 4;
  const size_t entries = (size_t)op->n_cells * op->geo_stride;
  if (op->geo64.bytes != entries * sizeof(double)) SF_RET(op->geo64.alloc(entries * sizeof(double)));
  SF_CUDA_TRY(cudaMemcpy2D(op->geo64.ptr, op->geo_stride * sizeof(double), G, 6 * n3 * sizeof(double),
                           6 * n3 * sizeof(double), (size_t)op->n_cells, cudaMemcpyDeviceToDevice));
  op->deformed = true;
  return derive_fp32_geometry(op);
}

int sf_set_coefficient(sf_op *op, const double *kappa)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (op->desc.kind != SF_OP_LAPLACE) return fail(SF_ERR_STATE, "coefficient only for SF_OP_LAPLACE");
  if (!kappa) {
    op->kap64.release();
    op->kap32.release();
    op->has_kappa = false;
    return derive_fp32_geometry(op);
  }
  SF_RET(check_ptr(kappa, SF_FP64, "kappa"));
  const long long n3 = (long long)op->n * op->n * op->n;
  const size_t entries = (size_t)op->n_cells * n3;
  if (op->kap64.bytes != entries * sizeof(double)) SF_RET(op->kap64.alloc(entries * sizeof(double)));
  SF_CUDA_TRY(cudaMemcpy(op->kap64.ptr, kappa, entries * sizeof(double), cudaMemcpyDeviceToDevice));
  if (op->desc.precisions & 2) {
    if (op->kap32.bytes != entries * sizeof(float)) SF_RET(op->kap32.alloc(entries * sizeof(float)));
    SF_RET(launch_convert((long long)entries, SF_FP64, kappa, SF_FP32, op->kap32.ptr, 0));
  }
  op->has_kappa = true;
  SF_RET(derive_fp32_geometry(op));
  SF_CUDA_TRY(cudaDeviceSynchronize());
  return SF_OK;
}

int sf_set_kernel_variant(sf_op *op, int variant)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (variant < SF_KERNEL_AUTO || variant > SF_KERNEL_GENERIC)
    return fail(SF_ERR_INVALID, "unknown kernel variant");
  op->kernel_variant = variant;
  return SF_OK;
}

int sf_device_status(sf_op *op, int *flags)
{
  if (!op || !flags) return fail(SF_ERR_NULL, "op/flags is NULL");
  SF_CUDA_TRY(cudaMemcpy(flags, op->dev_err.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  return SF_OK;
}

int sf_vmult(sf_op *op, int prec, const void *x, void *y, void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  SF_RET(check_prec(op, prec));
  SF_RET(check_ptr(x, prec, "x"));
  SF_RET(check_ptr(y, prec, "y"));
  if (ranges_overlap(x, y, (size_t)op->n_dofs * elem_size(prec)))
    return fail(SF_ERR_INVALID, "x and y must not overlap");
  cudaStream_t st = (cudaStream_t)stream;
  const Region region(op->region_mv);
  if (is_continuous(op->desc.kind)) return launch_cont_vmult(op, prec, x, y, st);
  if (is_cell_faces(op->desc.kind) && op->kernel_variant != SF_KERNEL_GENERIC)
    return launch_faces_tensor(op, prec, 1, x, y, st);
  if (is_cell_faces(op->desc.kind)) return launch_cell_faces(op, prec, 1, x, y, st);
  if (tensor_form(op))
    return launch_dg_precomputed(op, prec, 1, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, st);
  if (advect_tensor(op))
    return launch_dg_advect_tensor(op, prec, 1, false, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, nullptr,
                                   nullptr, nullptr, st);
  return launch_dg_vmult(op, prec, 1, false, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, st);
}

int sf_vmult_transpose(sf_op *op, int prec, const void *x, void *y, void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (op->desc.kind == SF_OP_CONVECTION || is_cell_faces(op->desc.kind))
    return fail(SF_ERR_UNSUPPORTED, "no transpose of the convection form or of the face-term operators");
  if (op->desc.kind != SF_OP_DG_ADVECT) return sf_vmult(op, prec, x, y, stream);
  return sf_vmult_transpose_batched(op, prec, 1, x, y, stream);
}

int sf_vmult_batched(sf_op *op, int prec, int nrhs, const void *x, void *y, void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  SF_RET(check_prec(op, prec));
  SF_RET(check_ptr(x, prec, "x"));
  SF_RET(check_ptr(y, prec, "y"));
  if (nrhs < 1 || nrhs > 64) return fail(SF_ERR_INVALID, "nrhs must be 1..64");
  if (ranges_overlap(x, y, (size_t)nrhs * (size_t)op->n_dofs * elem_size(prec)))
    return fail(SF_ERR_INVALID, "x and y must not overlap");
  cudaStream_t st = (cudaStream_t)stream;
  const Region region(op->region_mv);
  if (is_continuous(op->desc.kind)) {
    const size_t es = elem_size(prec);
    for (int r = 0; r < nrhs; ++r)
      SF_RET(launch_cont_vmult(op, prec, (const char *)x + r * op->n_dofs * es,
                               (char *)y + r * op->n_dofs * es, st));
    return SF_OK;
  }
  if (is_cell_faces(op->desc.kind) && op->kernel_variant != SF_KERNEL_GENERIC)
    return launch_faces_tensor(op, prec, nrhs, x, y, st);
  if (is_cell_faces(op->desc.kind)) return launch_cell_faces(op, prec, nrhs, x, y, st);
  if (tensor_form(op))
    return launch_dg_precomputed(op, prec, nrhs, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, st);
  if (advect_tensor(op))
    return launch_dg_advect_tensor(op, prec, nrhs, false, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, nullptr,
                                   nullptr, nullptr, st);
  return launch_dg_vmult(op, prec, nrhs, false, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, st);
}

int sf_vmult_transpose_batched(sf_op *op, int prec, int nrhs, const void *x, void *y, void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (op->desc.kind == SF_OP_CONVECTION || is_cell_faces(op->desc.kind))
    return fail(SF_ERR_UNSUPPORTED, "no transpose of the convection form or of the face-term operators");
  if (op->desc.kind != SF_OP_DG_ADVECT) return sf_vmult_batched(op, prec, nrhs, x, y, stream);
  SF_RET(check_prec(op, prec));
  SF_RET(check_ptr(x, prec, "x"));
  SF_RET(check_ptr(y, prec, "y"));
  if (nrhs < 1 || nrhs > 64) return fail(SF_ERR_INVALID, "nrhs must be 1..64");
  if (ranges_overlap(x, y, (size_t)nrhs * (size_t)op->n_dofs * elem_size(prec)))
    return fail(SF_ERR_INVALID, "x and y must not overlap");
  cudaStream_t st = (cudaStream_t)stream;
  const Region region(op->region_mv);
  // line operators: A^T, or A^T M^-1 in one launch
  if (advect_tensor(op))
    return launch_dg_advect_tensor(op, prec, nrhs, true, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, nullptr,
                                   nullptr, nullptr, st);
  const void *src = x;
  if (op->desc.inverse_mass) {
    const size_t bytes = (size_t)nrhs * op->n_dofs * elem_size(prec);
    if (op->scratch.bytes < bytes) SF_RET(op->scratch.alloc(bytes));
    SF_RET(launch_dg_inverse_mass(op, prec, nrhs, x, op->scratch.ptr, st));
    src = op->scratch.ptr;
  }
  return launch_dg_vmult(op, prec, nrhs, true, src, y, nullptr, nullptr, nullptr, 0.0, 0.0, st);
}

int sf_chebyshev_step(sf_op *op, int prec, const void *b, const void *diag_inv, const void *x_old,
                      void *x_new, void *t, double c_np, double c_tm, void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  SF_RET(check_prec(op, prec));
  SF_RET(check_ptr(b, prec, "b"));
  SF_RET(check_ptr(diag_inv, prec, "diag_inv"));
  SF_RET(check_ptr(x_old, prec, "x_old"));
  SF_RET(check_ptr(x_new, prec, "x_new"));
  SF_RET(check_ptr(t, prec, "t"));
  {
    // the outputs x_new and t overlap neither each other nor an input
    const size_t bytes = (size_t)op->n_dofs * elem_size(prec);
    const void *in[3] = {x_old, b, diag_inv};
    const char *in_name[3] = {"x_old", "b", "diag_inv"};
    if (ranges_overlap(x_new, t, bytes)) return fail(SF_ERR_INVALID, "x_new and t must not overlap");
    for (int i = 0; i < 3; ++i) {
      if (ranges_overlap(x_new, in[i], bytes))
        return fail(SF_ERR_INVALID, std::string("x_new and ") + in_name[i] + " must not overlap");
      if (ranges_overlap(t, in[i], bytes))
        return fail(SF_ERR_INVALID, std::string("t and ") + in_name[i] + " must not overlap");
    }
  }
  if (is_cell_faces(op->desc.kind))
    return fail(SF_ERR_UNSUPPORTED, "Chebyshev steps: not for the face-term operators");
  cudaStream_t st = (cudaStream_t)stream;
  const Region region(op->region_ch);
  if (tensor_form(op)) return launch_dg_precomputed(op, prec, 1, x_old, x_new, b, diag_inv, t, c_np, c_tm, st);
  if (advect_tensor(op))
    return launch_dg_advect_tensor(op, prec, 1, false, x_old, x_new, b, diag_inv, t, c_np, c_tm, nullptr, nullptr,
                                   nullptr, st);
  if (op->desc.kind == SF_OP_DG_SIPG || op->desc.kind == SF_OP_DG_ADVECT)
    return launch_dg_vmult(op, prec, 1, false, x_old, x_new, b, diag_inv, t, c_np, c_tm, st);
  // continuous: operator into x_new, then the fused vector update in place
  SF_RET(launch_cont_vmult(op, prec, x_old, x_new, st));
  return launch_vector_update(op->n_dofs, prec, x_new, b, diag_inv, x_old, x_new, t, c_np, c_tm, st);
}

int sf_rk_stage(sf_op *op, int prec, int nrhs, const void *src, const void *upd, void *vec_np, void *vec_tm,
                double c_np, double c_tm, void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (op->desc.kind != SF_OP_DG_ADVECT) return fail(SF_ERR_STATE, "Runge-Kutta stages need SF_OP_DG_ADVECT");
  SF_RET(check_prec(op, prec));
  SF_RET(check_ptr(src, prec, "src"));
  SF_RET(check_ptr(upd, prec, "upd"));
  SF_RET(check_ptr(vec_np, prec, "vec_np"));
  if (c_tm != 0.0) SF_RET(check_ptr(vec_tm, prec, "vec_tm"));
  if (nrhs < 1 || nrhs > 64) return fail(SF_ERR_INVALID, "nrhs must be 1..64");
  {
    // src and the outputs are disjoint; upd is one of the other vectors
    // itself (as in the reference's do_time_step) or disjoint from it
    const size_t bytes = (size_t)nrhs * (size_t)op->n_dofs * elem_size(prec);
    const bool tm = c_tm != 0.0;
    if (ranges_overlap(src, vec_np, bytes) || (tm && ranges_overlap(src, vec_tm, bytes)))
      return fail(SF_ERR_INVALID, "src must not overlap an output vector");
    if (tm && ranges_overlap(vec_np, vec_tm, bytes))
      return fail(SF_ERR_INVALID, "vec_np and vec_tm must not overlap");
    const void *other[3] = {src, vec_np, tm ? vec_tm : nullptr};
    for (const void *v : other)
      if (v && v != upd && ranges_overlap(upd, v, bytes))
        return fail(SF_ERR_INVALID, "upd must be src, vec_np, vec_tm itself or not overlap them");
  }
  const Region region(op->region_ch);
  if (advect_tensor(op))
    return launch_dg_advect_tensor(op, prec, nrhs, false, src, nullptr, nullptr, nullptr, nullptr, c_np, c_tm,
                                   upd, vec_np, c_tm != 0.0 ? vec_tm : nullptr, (cudaStream_t)stream);
  return launch_dg_rk_stage(op, prec, nrhs, src, upd, vec_np, c_tm != 0.0 ? vec_tm : nullptr, c_np, c_tm,
                            (cudaStream_t)stream);
}

// LSRK(5,4) of evaluation_dg_advect.h:192-212: coefficients and the rotation
// of the three registers over the five stages
int sf_lsrk_step(sf_op *op, int prec, int nrhs, void *sol_new, void *sol_old, void *sol_tmp, double dt,
                 void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (!sol_new || !sol_old || !sol_tmp) return fail(SF_ERR_NULL, "sol_new/sol_old/sol_tmp is NULL");
  if (nrhs < 1 || nrhs > 64) return fail(SF_ERR_INVALID, "nrhs must be 1..64");
  SF_RET(check_prec(op, prec));
  {
    const size_t bytes = (size_t)nrhs * (size_t)op->n_dofs * elem_size(prec);
    if (ranges_overlap(sol_new, sol_old, bytes) || ranges_overlap(sol_new, sol_tmp, bytes) ||
        ranges_overlap(sol_old, sol_tmp, bytes))
      return fail(SF_ERR_INVALID, "sol_new, sol_old and sol_tmp must not overlap");
  }
  const double a21 = 970286171893. / 4311952581923.;
  const double a32 = 6584761158862. / 12103376702013.;
  const double a43 = 2251764453980. / 15575788980749.;
  const double a54 = 26877169314380. / 34165994151039.;
  const double b1 = 1153189308089. / 22510343858157.;
  const double b2 = 1772645290293. / 4653164025191.;
  const double b3 = -1672844663538. / 4480602732383.;
  const double b4 = 2114624349019. / 3568978502595.;
  const double b5 = 5198255086312. / 14908931495163.;
  SF_RET(sf_rk_stage(op, prec, nrhs, sol_new, sol_new, sol_old, sol_tmp, a21 * dt, (b1 - a21) * dt, stream));
  SF_RET(sf_rk_stage(op, prec, nrhs, sol_old, sol_tmp, sol_new, sol_tmp, a32 * dt, (b2 - a32) * dt, stream));
  SF_RET(sf_rk_stage(op, prec, nrhs, sol_new, sol_tmp, sol_old, sol_tmp, a43 * dt, (b3 - a43) * dt, stream));
  SF_RET(sf_rk_stage(op, prec, nrhs, sol_old, sol_tmp, sol_tmp, sol_new, a54 * dt, (b4 - a54) * dt, stream));
  return sf_rk_stage(op, prec, nrhs, sol_tmp, sol_new, sol_new, sol_tmp, b5 * dt, 0.0, stream);
}

int sf_vector_update(long long n, int prec, const void *ax, const void *b, const void *diag_inv,
                     const void *x_old, void *x_new, void *t, double c_np, double c_tm, void *stream)
{
  SF_RET(check_prec(nullptr, prec));
  if (n < 0) return fail(SF_ERR_INVALID, "n < 0");
  SF_RET(check_ptr(ax, prec, "ax"));
  SF_RET(check_ptr(b, prec, "b"));
  SF_RET(check_ptr(diag_inv, prec, "diag_inv"));
  SF_RET(check_ptr(x_old, prec, "x_old"));
  SF_RET(check_ptr(x_new, prec, "x_new"));
  SF_RET(check_ptr(t, prec, "t"));
  {
    // the outputs x_new and t overlap neither each other nor an input, except
    // that ax may be x_new itself (the reference's emulation passes sol_new as
    // both; each entry of ax is read before the same entry of x_new is written)
    const size_t bytes = (size_t)n * elem_size(prec);
    const void *in[4] = {ax, b, diag_inv, x_old};
    const char *in_name[4] = {"ax", "b", "diag_inv", "x_old"};
    if (ranges_overlap(x_new, t, bytes)) return fail(SF_ERR_INVALID, "x_new and t must not overlap");
    for (int i = 0; i < 4; ++i) {
      if (ranges_overlap(x_new, in[i], bytes) && !(i == 0 && ax == x_new))
        return fail(SF_ERR_INVALID, std::string("x_new and ") + in_name[i] + " must not overlap");
      if (ranges_overlap(t, in[i], bytes))
        return fail(SF_ERR_INVALID, std::string("t and ") + in_name[i] + " must not overlap");
    }
  }
  if (n == 0) return SF_OK;
  return launch_vector_update(n, prec, ax, b, diag_inv, x_old, x_new, t, c_np, c_tm,
                              (cudaStream_t)stream);
}

int sf_diagonal(sf_op *op, int prec, void *diag, void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  SF_RET(check_prec(op, prec));
  SF_RET(check_ptr(diag, prec, "diag"));
  if (op->desc.kind == SF_OP_MASS || op->desc.kind == SF_OP_CONVECTION ||
      op->desc.kind == SF_OP_LAPLACE_UNSTRUCTURED || is_cell_faces(op->desc.kind))
    return fail(SF_ERR_UNSUPPORTED, "diagonal: structured Laplacian and DG operators only");
  if (op->desc.kind == SF_OP_LAPLACE) return launch_cont_diagonal(op, prec, diag, (cudaStream_t)stream);
  if (tensor_form(op)) return launch_dg_precomputed_diagonal(op, prec, diag, (cudaStream_t)stream);
  return launch_dg_diagonal(op, prec, diag, (cudaStream_t)stream);
}

int sf_kappa_gradient(sf_op *op, int prec, const void *u, const void *lam, void *dkappa, void *stream)
{
  if (!op) return fail(SF_ERR_NULL, "op is NULL");
  if (op->desc.kind != SF_OP_LAPLACE) return fail(SF_ERR_STATE, "kappa gradient only for SF_OP_LAPLACE");
  SF_RET(check_prec(op, prec));
  SF_RET(check_ptr(u, prec, "u"));
  SF_RET(check_ptr(lam, prec, "lam"));
  SF_RET(check_ptr(dkappa, prec, "dkappa"));
  return launch_cont_kappa_grad(op, prec, u, lam, dkappa, (cudaStream_t)stream);
}

int sf_convert(long long n, int from_prec, const void *x, int to_prec, void *y, void *stream)
{
  SF_RET(check_prec(nullptr, from_prec));
  SF_RET(check_prec(nullptr, to_prec));
  SF_RET(check_ptr(x, from_prec, "x"));
  SF_RET(check_ptr(y, to_prec, "y"));
  if (n < 0) return fail(SF_ERR_INVALID, "n < 0");
  if (n == 0) return SF_OK;
  return launch_convert(n, from_prec, x, to_prec, y, (cudaStream_t)stream);
}

int sf_dot(long long n, int prec, const void *x, const void *y, double *result_dev, void *stream)
{
  SF_RET(check_prec(nullptr, prec));
  SF_RET(check_ptr(x, prec, "x"));
  SF_RET(check_ptr(y, prec, "y"));
  SF_RET(check_ptr(result_dev, SF_FP64, "result_dev"));
  if (n < 0) return fail(SF_ERR_INVALID, "n < 0");
  // per-thread scratch for the partial sums (allocated once per thread)
  static thread_local DevBuf scratch;
  if (!scratch.ptr) SF_RET(scratch.alloc(sizeof(double) * kDotBlocks));
  return launch_dot(n, prec, x, y, (double *)scratch.ptr, result_dev, (cudaStream_t)stream);
}

int sf_shape_tables(int degree, int basis, double *S, double *D, double *pts, double *w)
{
  Shape1D s;
  if (fill_shape(degree, basis, s) != 0) return fail(SF_ERR_UNSUPPORTED, "degree must be 1..8");
  const int n = s.n;
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i) {
      if (S) S[q * n + i] = s.S[q][i];
      if (D) D[q * n + i] = s.D[q][i];
    }
  for (int q = 0; q < n; ++q) {
    if (pts) pts[q] = s.xq[q];
    if (w) w[q] = s.wq[q];
  }
  return SF_OK;
}

} // extern "C"
