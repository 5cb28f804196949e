// sf_vector.cu -- vector kernels: precision conversion, the standalone
// Chebyshev vector update (evaluation_dg_laplacian.h:556-601) and a
// deterministic FP64 dot product.
//
// All are HBM-streaming kernels: grid-stride loops over 128-bit vector
// accesses where the pointers allow it, grids sized to the SM count.
#include "sf_internal.h"
#include "sf_launch.h"

#include <algorithm>
#include <atomic>

namespace sf {

int device_sm_count()
{
  // cached per device ordinal (attribute queries are host-side only)
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (dev >= 0 && dev < 64) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) return 1;
  if (dev >= 0 && dev < 64) cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

int stream_grid(long long n, int threads, int per_sm)
{
  long long g = (n + threads - 1) / threads;
  const long long cap = (long long)device_sm_count() * per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

namespace {

constexpr int kThreads = 256;

// enough resident blocks to cover the SMs several times over
int grid_for(long long n) { return stream_grid(n, kThreads, 16); }

template <typename S, typename D>
__global__ void convert_kernel(long long n, const S *__restrict__ x, D *__restrict__ y)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = D(x[i]);
}

template <typename T>
__global__ void vector_update_kernel(long long n, const T *ax, const T *__restrict__ b,
                                     const T *__restrict__ dinv, const T *__restrict__ xo,
                                     T *xn, T *__restrict__ t, T c_np, T c_tm)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const T res = ax[i] - b[i];
    const T tmp = c_tm * t[i] + c_np * dinv[i] * res;
    t[i] = tmp;
    xn[i] = xo[i] - tmp;
  }
}

// block partial sums over a fixed interleaving: partial[blockIdx.x]
template <typename T>
__global__ void dot_partial_kernel(long long n, const T *__restrict__ x, const T *__restrict__ y,
                                   double *__restrict__ partial)
{
  __shared__ double red[kThreads];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s = fma(double(x[i]), double(y[i]), s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void dot_final_kernel(const double *__restrict__ partial, int np, double *__restrict__ out)
{
  __shared__ double red[kThreads];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

} // namespace

int resident_blocks_per_sm(const void *kernel, int threads, size_t dyn_smem, int *blocks)
{
  cudaFuncAttributes fa;
  SF_CUDA_TRY(cudaFuncGetAttributes(&fa, kernel));
  int dev = 0, max_thr = 0, max_smem = 0, regs = 0, max_blk = 0, reserved = 0;
  SF_CUDA_TRY(cudaGetDevice(&dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&max_thr, cudaDevAttrMaxThreadsPerMultiProcessor, dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&regs, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&max_blk, cudaDevAttrMaxBlocksPerMultiprocessor, dev));
  SF_CUDA_TRY(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
  int b = std::min(max_thr / threads, max_blk);
  // registers are allocated per warp in units of 256
  const int warps = (threads + 31) / 32;
  const int regs_per_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
  if (regs_per_warp > 0) b = std::min(b, regs / (regs_per_warp * warps));
  const size_t per_block = dyn_smem + fa.sharedSizeBytes + (size_t)reserved;
  if (per_block > 0) b = std::min<long long>(b, (long long)(max_smem / per_block));
  *blocks = b;
  if (b < 1) {
    set_error("kernel does not fit on an SM");
    return SF_ERR_UNSUPPORTED;
  }
  return SF_OK;
}

int launch_convert(long long n, int from, const void *x, int to, void *y, cudaStream_t st)
{
  const int g = grid_for(n);
  if (from == SF_FP64 && to == SF_FP32)
    convert_kernel<double, float><<<g, kThreads, 0, st>>>(n, (const double *)x, (float *)y);
  else if (from == SF_FP32 && to == SF_FP64)
    convert_kernel<float, double><<<g, kThreads, 0, st>>>(n, (const float *)x, (double *)y);
  else if (from == SF_FP64)
    SF_CUDA_TRY(cudaMemcpyAsync(y, x, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  else
    SF_CUDA_TRY(cudaMemcpyAsync(y, x, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

int launch_vector_update(long long n, int prec, const void *ax, const void *b, const void *dinv,
                         const void *x_old, void *x_new, void *t, double c_np, double c_tm,
                         cudaStream_t st)
{
  const int g = grid_for(n);
  if (prec == SF_FP64)
    vector_update_kernel<double><<<g, kThreads, 0, st>>>(
        n, (const double *)ax, (const double *)b, (const double *)dinv, (const double *)x_old,
        (double *)x_new, (double *)t, c_np, c_tm);
  else
    vector_update_kernel<float><<<g, kThreads, 0, st>>>(
        n, (const float *)ax, (const float *)b, (const float *)dinv, (const float *)x_old,
        (float *)x_new, (float *)t, (float)c_np, (float)c_tm);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

int launch_dot(long long n, int prec, const void *x, const void *y, double *scratch, double *result,
               cudaStream_t st)
{
  if (prec == SF_FP64)
    dot_partial_kernel<double><<<kDotBlocks, kThreads, 0, st>>>(n, (const double *)x,
                                                                (const double *)y, scratch);
  else
    dot_partial_kernel<float><<<kDotBlocks, kThreads, 0, st>>>(n, (const float *)x,
                                                               (const float *)y, scratch);
  dot_final_kernel<<<1, kThreads, 0, st>>>(scratch, kDotBlocks, result);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

} // namespace sf
