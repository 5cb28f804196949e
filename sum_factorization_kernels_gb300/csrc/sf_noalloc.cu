// sf_noalloc.cu -- transposed DG advection apply that allocates nothing.
//
// The transpose of the inverse-mass advection operator, (M^-1 K)^T =
// K^T M^-1, runs in two passes in the cell-and-face form and needs an
// intermediate vector between them.  sf_vmult_transpose_batched() with that
// form (SF_KERNEL_GENERIC) keeps the vector in a per-handle device buffer
// that it allocates with cudaMalloc on first use (its default line-operator
// form needs none).  This entry point always runs the two-pass form.  Some
// callers cannot allow that: applications that hand out all device memory
// from their own pool or reserve a fixed budget up front, and must not see
// a foreign allocation appear mid-run, and time-stepping loops where an
// allocation's implicit device synchronisation is not acceptable.  For
// them, sf_vmult_transpose_static() takes the intermediate vector from a
// fixed device array compiled into this library instead.
//
// The array holds kStaticScratchBytes (4 MiB).  Every GPU that loads the
// library reserves it until the process exits.  All calls share it and it
// keeps the previous call's contents; nothing in it has to start at zero
// because the first pass writes every entry that the second pass reads.
// Two calls whose work overlaps on the GPU (different streams, or different
// host threads on the same device) race on the array and corrupt each
// other's results; order them on one stream or synchronise between them.

#include "sf_internal.h"
#include "sf_launch.h"

namespace {

constexpr size_t kStaticScratchBytes = size_t(4) << 20;

// device-resident intermediate vector shared by all calls on a device
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// device address of g_static_scratch in the current context (the name is
// only a host-side stand-in, not a device address).  Looked up on every call
// and never cached: cudaDeviceReset() unloads the library's module, and the
// array can sit at another address once the module is loaded again.
int scratch_address(void **out)
{
  void *p = nullptr;
  SF_CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
  *out = p;
  return SF_OK;
}

} // namespace

extern "C" int sf_vmult_transpose_static(sf_op *op, int prec, int nrhs, const void *x, void *y,
                                         void *stream)
{
  if (!op || !x || !y) {
    sf::set_error("op/x/y is NULL");
    return SF_ERR_NULL;
  }
  if (op->desc.kind != SF_OP_DG_ADVECT) {
    sf::set_error("sf_vmult_transpose_static is for SF_OP_DG_ADVECT handles");
    return SF_ERR_STATE;
  }
  if (prec != SF_FP64 && prec != SF_FP32) {
    sf::set_error("precision must be SF_FP64 or SF_FP32");
    return SF_ERR_INVALID;
  }
  if (!(op->desc.precisions & (prec == SF_FP64 ? 1 : 2))) {
    sf::set_error("precision not prepared by sf_create (desc.precisions)");
    return SF_ERR_STATE;
  }
  const size_t es = prec == SF_FP64 ? sizeof(double) : sizeof(float);
  if (reinterpret_cast<uintptr_t>(x) % es || reinterpret_cast<uintptr_t>(y) % es) {
    sf::set_error("x/y not aligned to the element size");
    return SF_ERR_ALIGN;
  }
  if (nrhs < 1 || nrhs > 64) {
    sf::set_error("nrhs must be 1..64");
    return SF_ERR_INVALID;
  }
  if (sf::ranges_overlap(x, y, (size_t)nrhs * (size_t)op->n_dofs * es)) {
    sf::set_error("x and y must not overlap");
    return SF_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (!op->desc.inverse_mass) // K^T needs no intermediate vector
    return sf::launch_dg_vmult(op, prec, nrhs, true, x, y, nullptr, nullptr, nullptr, 0.0, 0.0, st);
  const size_t need = (size_t)nrhs * (size_t)op->n_dofs * es;
  if (need > kStaticScratchBytes) {
    sf::set_error("sf_vmult_transpose_static: nrhs * n_dofs * element size = " + std::to_string(need) +
                  " bytes exceeds the static scratch of " + std::to_string(kStaticScratchBytes) +
                  " bytes; use sf_vmult_transpose_batched");
    return SF_ERR_INVALID;
  }
  void *scratch = nullptr;
  int e = scratch_address(&scratch);
  if (e != SF_OK) return e;
  e = sf::launch_dg_inverse_mass(op, prec, nrhs, x, scratch, st);
  if (e != SF_OK) return e;
  return sf::launch_dg_vmult(op, prec, nrhs, true, scratch, y, nullptr, nullptr, nullptr, 0.0, 0.0, st);
}
