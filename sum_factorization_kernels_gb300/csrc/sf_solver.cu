// sf_solver.cu -- conjugate gradients around the operators (no reference
// counterpart: the reference times operator applications only).
//
//  * SF_SOLVE_FP64: preconditioned CG with FP64 vectors and the FP64 operator.
//  * SF_SOLVE_MIXED: FP32 preconditioned CG (FP32 operator, FP32 vectors,
//    FP64 reductions) on the correction A d = r / |r| of an FP64 iterate,
//    with reliable updates (residual replacement): whenever the recursive
//    FP32 residual has dropped by a factor inner_rtol since the last
//    replacement, the correction is added to the FP64 iterate, the true
//    residual b - A x is formed with the FP64 operator and becomes the FP32
//    residual, and the iteration continues with the same search direction.
//    The Krylov space is not restarted, so the FP32 solve needs about as many
//    iterations as the FP64 one.  The solve targets the outer tolerance
//    directly; an FP64 refinement step around it (the true residual, then
//    another FP32 solve) only follows if the FP32 solve stalls.
//  * Preconditioners: none, Jacobi (inverse diagonal) or a Chebyshev
//    polynomial of D^-1 A (the smoother form of the reference's fused
//    Chebyshev step, evaluation_dg_laplacian.h:485-502) with lambda_max from
//    a Lanczos estimate built out of the CG coefficients of a few Jacobi-CG
//    steps, range [lambda_max / range, 1.2 lambda_max].
//  * Scalars (alpha, beta, dot products, the convergence flag) stay on the
//    device.  Reductions are single-pass: fixed-size block partials, summed
//    in block order by the last block to finish (deterministic); FP32
//    vectors are reduced four entries at a time in FP32 and accumulated in
//    FP64.  The host
//    never waits for the iteration it has just queued: it queues iteration
//    k, then reads the scalars of iteration k-1 from pinned memory.  An
//    iteration queued after convergence changes nothing, because the update
//    kernels return when the device flag says the solve is done.
//  * Work vectors and scalars are allocated once per handle and precision
//    and kept with the preconditioner state.
//  * Periodic DG SIPG has the constants as null space: with
//    project_constant the right-hand side and every preconditioned residual
//    are projected to mean zero.
#include <chrono>
#include <cstdint>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "sf_internal.h"
#include "sf_launch.h"

namespace sf {

namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 1024; // fixed reduction grid: deterministic results

struct Scalars {
  double rz, rz_old, pAp, rr, sum;
  double tol2;        // the solve is done once rr <= tol2
  int done;           // convergence or breakdown: update kernels return
  int breakdown;      // non-positive curvature or non-finite residual
  unsigned ticket;    // blocks finished in the running reduction
  int pad;
};

int grid_for(long long n) { return stream_grid(n, kThreads, 16); }

// block sum of two values per thread; the result is in s1[0], s2[0]
__device__ __forceinline__ void block_sum2(double *s1, double *s2, double a, double b)
{
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
}

enum { RED_RZ = 0, RED_PAP = 1, RED_SUM = 2 };

// single-pass reduction.  RED_RZ: rz = (a, b), rr = (a, a), convergence and
// finiteness checks; RED_PAP: pAp = (a, b), curvature check; RED_SUM:
// sum = sum(a).  The last block to finish sums the partials in block order.
template <typename T, int MODE>
__global__ void __launch_bounds__(kThreads) reduce_kernel(long long n, const T *__restrict__ a,
                                                          const T *__restrict__ b, double *__restrict__ part,
                                                          Scalars *sc)
{
  __shared__ double s1[kThreads], s2[kThreads];
  __shared__ bool last;
  double u = 0, v = 0;
  const long long gs = (long long)gridDim.x * blockDim.x;
  long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if constexpr (sizeof(T) == 4) {
    // FP32 vectors: four products and their sum in FP32, accumulated in
    // FP64 once per four entries (the FP64 pipe runs at 1/64 of FP32 rate
    // and would bound a per-entry FP64 accumulation)
    const bool aligned = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0;
    if (aligned) {
      const long long n4 = n / 4;
      const float4 *a4 = reinterpret_cast<const float4 *>(a), *b4 = reinterpret_cast<const float4 *>(b);
      for (long long i = i0; i < n4; i += gs) {
        const float4 x = a4[i];
        if (MODE == RED_SUM) {
          u += double((x.x + x.y) + (x.z + x.w));
        } else {
          const float4 y = b4[i];
          u += double(fmaf(x.w, y.w, fmaf(x.z, y.z, fmaf(x.y, y.y, x.x * y.x))));
          if (MODE == RED_RZ) v += double(fmaf(x.w, x.w, fmaf(x.z, x.z, fmaf(x.y, x.y, x.x * x.x))));
        }
      }
      i0 += 4 * n4;
    }
  }
  for (long long i = i0; i < n; i += gs) {
    const double ai = a[i];
    if (MODE == RED_SUM) {
      u += ai;
    } else {
      u = fma(ai, double(b[i]), u);
      if (MODE == RED_RZ) v = fma(ai, ai, v);
    }
  }
  block_sum2(s1, s2, u, v);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = s2[0];
    __threadfence();
    last = atomicAdd(&sc->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  u = 0;
  v = 0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    u += __ldcg(part + 2 * i);
    v += __ldcg(part + 2 * i + 1);
  }
  block_sum2(s1, s2, u, v);
  if (threadIdx.x == 0) {
    if (MODE == RED_RZ) {
      sc->rz_old = sc->rz;
      sc->rz = s1[0];
      sc->rr = s2[0];
      if (!isfinite(s2[0])) {
        sc->breakdown = 1;
        sc->done = 1;
      } else if (s2[0] <= sc->tol2) {
        sc->done = 1;
      }
    } else if (MODE == RED_PAP) {
      sc->pAp = s1[0];
      if (!(s1[0] > 0.0)) {
        sc->breakdown = 1;
        sc->done = 1;
      }
    } else {
      sc->sum = s1[0];
    }
    sc->ticket = 0;
  }
}

__global__ void begin_solve_kernel(Scalars *sc, double tol2)
{
  sc->tol2 = tol2;
  sc->done = 0;
  sc->breakdown = 0;
  sc->ticket = 0;
}

template <typename T>
__global__ void subtract_mean(long long n, T *__restrict__ x, const Scalars *sc)
{
  const T m = T(sc->sum / double(n));
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] -= m;
}

enum { PC_NONE = 0, PC_JACOBI = 1, PC_CHEB = 2 };

// x += alpha p, r -= alpha Ap (alpha = rz / pAp), then the first step of
// the preconditioner on the new residual: z = D^-1 r (Jacobi) or z = s D^-1 r,
// t = -z (first Chebyshev step from a zero start); nothing when done
template <typename T, int PC>
__global__ void update_xr_precond(long long n, T *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
                                  const T *__restrict__ Ap, const T *__restrict__ dinv, T *__restrict__ z,
                                  T *__restrict__ t, T s, const Scalars *sc)
{
  if (sc->done) return;
  const T a = T(sc->rz / sc->pAp);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    const T ri = r[i] - a * Ap[i];
    r[i] = ri;
    if (PC == PC_JACOBI) z[i] = dinv[i] * ri;
    if (PC == PC_CHEB) {
      const T v = s * dinv[i] * ri;
      z[i] = v;
      t[i] = -v;
    }
  }
}

// p = z + beta p, beta = rz / rz_old; nothing when done
template <typename T>
__global__ void update_p(long long n, T *__restrict__ p, const T *__restrict__ z, const Scalars *sc)
{
  if (sc->done) return;
  const T be = T(sc->rz / sc->rz_old);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = z[i] + be * p[i];
}

// first preconditioner step on a residual (outside the iteration)
template <typename T, int PC>
__global__ void precond_first(long long n, const T *__restrict__ r, const T *__restrict__ dinv, T *__restrict__ z,
                              T *__restrict__ t, T s)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (PC == PC_JACOBI) z[i] = dinv[i] * r[i];
    if (PC == PC_CHEB) {
      const T v = s * dinv[i] * r[i];
      z[i] = v;
      t[i] = -v;
    }
  }
}

template <typename T>
__global__ void inverse_kernel(long long n, T *__restrict__ d)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    d[i] = d[i] != T(0) ? T(1) / d[i] : T(1);
}

template <typename T>
__global__ void sub_kernel(long long n, T *__restrict__ r, const T *__restrict__ b, const T *__restrict__ ax)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    r[i] = b[i] - ax[i];
}

// y = x / |r| in FP32 (the unit right-hand side of an inner solve)
__global__ void to_f32_scaled(long long n, float *__restrict__ y, const double *__restrict__ x, const Scalars *sc)
{
  const double s = 1.0 / sqrt(sc->rr);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = float(x[i] * s);
}

// y = x * s in FP32 (a replaced residual in the scale of the running solve)
__global__ void to_f32_times(long long n, float *__restrict__ y, const double *__restrict__ x, double s)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = float(x[i] * s);
}

// x += scale d (scale = |r| of the outer step)
__global__ void add_f32_scaled(long long n, double *__restrict__ x, const float *__restrict__ d, double scale)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] += scale * double(d[i]);
}

template <typename T>
__global__ void copy_kernel(long long n, T *__restrict__ y, const T *__restrict__ x)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = x[i];
}

template <typename T>
constexpr int prec_of() { return sizeof(T) == 8 ? SF_FP64 : SF_FP32; }

// largest eigenvalue of the symmetric tridiagonal (d, e) by bisection on
// the Sturm sequence count
double tridiag_max_eig(const std::vector<double> &d, const std::vector<double> &e)
{
  const int m = (int)d.size();
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(e[i]) : 0.0);
    lo = std::fmin(lo, d[i] - r);
    hi = std::fmax(hi, d[i] + r);
  }
  auto count_below = [&](double x) {
    int c = 0;
    double q = 1.0;
    for (int i = 0; i < m; ++i) {
      const double ee = i > 0 ? e[i - 1] * e[i - 1] : 0.0;
      q = d[i] - x - (i > 0 ? ee / q : 0.0);
      if (q == 0.0) q = 1e-300;
      if (q < 0) ++c;
    }
    return c;
  };
  for (int it = 0; it < 200 && hi - lo > 1e-12 * std::fabs(hi); ++it) {
    const double mid = 0.5 * (lo + hi);
    if (count_below(mid) >= m) hi = mid;
    else lo = mid;
  }
  return hi;
}

// CG work vectors of one precision
struct Work {
  DevBuf r, p, ap, z;
  template <typename T>
  int ensure(long long n)
  {
    const size_t b = sizeof(T) * (size_t)n;
    int e;
    if (r.bytes == b) return SF_OK;
    if ((e = r.alloc(b)) || (e = p.alloc(b)) || (e = ap.alloc(b)) || (e = z.alloc(b))) return e;
    return SF_OK;
  }
};

// per-precision preconditioner state and work vectors, kept per handle
struct PrecState {
  DevBuf dinv, z2, t;
  Work work;
  double lambda_max = 0.0;
  bool have_diag = false, have_eig = false;
};

// state of the solver kept per handle: preconditioners, work vectors,
// device scalars, pinned host copies of the scalars
struct SolverCache {
  sf_op *op = nullptr;
  PrecState st[2];
  DevBuf part, scal, bcopy, r64, ax64, r32, d32;
  Scalars *host = nullptr; // pinned ring of 2
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~SolverCache()
  {
    if (host) cudaFreeHost(host);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  }
  int init()
  {
    if (host) return SF_OK;
    int r = part.alloc(sizeof(double) * 2 * kBlocks);
    if (r) return r;
    if ((r = scal.alloc(sizeof(Scalars)))) return r;
    SF_CUDA_TRY(cudaMemset(scal.ptr, 0, sizeof(Scalars)));
    for (auto &e : ev) SF_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    SF_CUDA_TRY(cudaMallocHost(&host, 2 * sizeof(Scalars)));
    std::memset(host, 0, 2 * sizeof(Scalars));
    return SF_OK;
  }
};

struct Solver {
  sf_op *op;
  cudaStream_t st;
  long long n;
  SolverCache *cache;
  Scalars *sc = nullptr;
  double *part_d = nullptr;
  int applies = 0;

  void bind()
  {
    sc = (Scalars *)cache->scal.ptr;
    part_d = (double *)cache->part.ptr;
  }

  template <typename T, int MODE>
  int reduce(const T *a, const T *b)
  {
    reduce_kernel<T, MODE><<<kBlocks, kThreads, 0, st>>>(n, a, b, part_d, sc);
    SF_CUDA_TRY(cudaGetLastError());
    return SF_OK;
  }

  int begin(double tol2)
  {
    begin_solve_kernel<<<1, 1, 0, st>>>(sc, tol2);
    SF_CUDA_TRY(cudaGetLastError());
    return SF_OK;
  }

  template <typename T>
  int project(T *x)
  {
    int e = reduce<T, RED_SUM>(x, x);
    if (e) return e;
    subtract_mean<T><<<grid_for(n), kThreads, 0, st>>>(n, x, sc);
    SF_CUDA_TRY(cudaGetLastError());
    return SF_OK;
  }

  // queue a copy of the scalars into pinned slot `slot` and mark it
  int post(int slot)
  {
    SF_CUDA_TRY(cudaMemcpyAsync(cache->host + slot, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    SF_CUDA_TRY(cudaEventRecord(cache->ev[slot], st));
    return SF_OK;
  }

  // wait for slot `slot` and return its scalars
  int fetch(int slot, Scalars *out)
  {
    SF_CUDA_TRY(cudaEventSynchronize(cache->ev[slot]));
    *out = cache->host[slot];
    return SF_OK;
  }

  // synchronous read of the current scalars
  int read(Scalars *out)
  {
    int e = post(0);
    if (e) return e;
    return fetch(0, out);
  }

  int vmult(int prec, const void *x, void *y)
  {
    ++applies;
    return sf_vmult(op, prec, x, y, st);
  }
};

template <typename T>
int ensure_diag(Solver &S, PrecState &P)
{
  if (P.have_diag) return SF_OK;
  int r = P.dinv.alloc(sizeof(T) * S.n);
  if (r) return r;
  r = sf_diagonal(S.op, prec_of<T>(), P.dinv.ptr, S.st);
  if (r) return r;
  inverse_kernel<T><<<grid_for(S.n), kThreads, 0, S.st>>>(S.n, (T *)P.dinv.ptr);
  SF_CUDA_TRY(cudaGetLastError());
  P.have_diag = true;
  return SF_OK;
}

// lambda_max of D^-1 A from `steps` Jacobi-preconditioned CG iterations
// (setup only: one host read per step)
template <typename T>
int ensure_eig(Solver &S, PrecState &P, int steps, bool proj)
{
  if (P.have_eig) return SF_OK;
  const long long n = S.n;
  int e;
  if ((e = P.work.ensure<T>(n))) return e;
  DevBuf bx;
  if ((e = bx.alloc(sizeof(T) * n))) return e;
  T *r = (T *)P.work.r.ptr, *p = (T *)P.work.p.ptr, *ap = (T *)P.work.ap.ptr, *z = (T *)P.work.z.ptr,
    *x = (T *)bx.ptr;
  const T *dinv = (const T *)P.dinv.ptr;
  // deterministic pseudo-random start vector: fractional parts of i * golden ratio
  {
    std::vector<T> h((size_t)std::min<long long>(n, 1 << 20));
    for (size_t i = 0; i < h.size(); ++i) h[i] = T(std::fmod(0.6180339887498949 * (i + 1), 1.0) - 0.5);
    for (long long off = 0; off < n; off += (long long)h.size()) {
      const long long cnt = std::min<long long>((long long)h.size(), n - off);
      SF_CUDA_TRY(cudaMemcpyAsync(r + off, h.data(), sizeof(T) * cnt, cudaMemcpyHostToDevice, S.st));
    }
    SF_CUDA_TRY(cudaStreamSynchronize(S.st));
  }
  SF_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(T) * n, S.st));
  if ((e = S.begin(0.0))) return e;
  if (proj && (e = S.project(r))) return e;
  precond_first<T, PC_JACOBI><<<grid_for(n), kThreads, 0, S.st>>>(n, r, dinv, z, nullptr, T(1));
  if (proj && (e = S.project(z))) return e;
  copy_kernel<T><<<grid_for(n), kThreads, 0, S.st>>>(n, p, z);
  if ((e = S.reduce<T, RED_RZ>(r, z))) return e;
  std::vector<double> alpha, beta;
  Scalars h;
  for (int it = 0; it < steps; ++it) {
    if ((e = S.vmult(prec_of<T>(), p, ap))) return e;
    if ((e = S.reduce<T, RED_PAP>(p, ap))) return e;
    if ((e = S.read(&h))) return e;
    const double a = h.rz / h.pAp;
    if (h.done || !std::isfinite(a)) break;
    alpha.push_back(a);
    update_xr_precond<T, PC_JACOBI><<<grid_for(n), kThreads, 0, S.st>>>(n, x, r, p, ap, dinv, z, nullptr, T(1),
                                                                         S.sc);
    if (proj && (e = S.project(z))) return e;
    if ((e = S.reduce<T, RED_RZ>(r, z))) return e;
    if ((e = S.read(&h))) return e;
    const double b = h.rz / h.rz_old;
    if (h.done || !std::isfinite(b) || h.rz <= 0) break;
    beta.push_back(b);
    update_p<T><<<grid_for(n), kThreads, 0, S.st>>>(n, p, z, S.sc);
  }
  SF_CUDA_TRY(cudaGetLastError());
  if (alpha.empty()) {
    set_error("eigenvalue estimate failed (operator not positive)");
    return SF_ERR_BREAKDOWN;
  }
  // Lanczos tridiagonal from the CG coefficients
  const int m = (int)alpha.size();
  std::vector<double> d(m), off(m > 1 ? m - 1 : 0);
  for (int i = 0; i < m; ++i) {
    d[i] = 1.0 / alpha[i] + (i > 0 ? beta[i - 1] / alpha[i - 1] : 0.0);
    if (i + 1 < m) off[i] = std::sqrt(beta[i]) / alpha[i];
  }
  P.lambda_max = tridiag_max_eig(d, off);
  P.have_eig = true;
  return SF_OK;
}

struct ChebCoef {
  double theta, delta;
};

ChebCoef cheb_coef(const PrecState &P, const sf_solve_opts &o)
{
  const double lmax = 1.2 * P.lambda_max, lmin = lmax / o.cheb_range;
  return ChebCoef{0.5 * (lmax + lmin), 0.5 * (lmax - lmin)};
}

// the Chebyshev steps after the first (which the caller fused into its
// residual update): z = p_k(D^-1 A) D^-1 r
template <typename T>
int cheb_rest(Solver &S, PrecState &P, const sf_solve_opts &o, const T *r, T *z)
{
  const ChebCoef c = cheb_coef(P, o);
  T *t = (T *)P.t.ptr, *z2 = (T *)P.z2.ptr;
  double rho_old = c.delta / c.theta;
  T *cur = z, *nxt = z2;
  for (int k = 1; k < o.cheb_degree; ++k) {
    const double rho = 1.0 / (2.0 * c.theta / c.delta - rho_old);
    ++S.applies;
    const int e = sf_chebyshev_step(S.op, prec_of<T>(), r, P.dinv.ptr, cur, nxt, t, 2.0 * rho / c.delta,
                                    rho * rho_old, S.st);
    if (e) return e;
    rho_old = rho;
    T *tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  if (cur != z) {
    copy_kernel<T><<<grid_for(S.n), kThreads, 0, S.st>>>(S.n, z, cur);
    SF_CUDA_TRY(cudaGetLastError());
  }
  return SF_OK;
}

// reliable updates of an FP32 correction solve inside the FP64 refinement:
// the FP64 iterate, right-hand side and work vectors, and the scale of the
// FP32 system (|r| of the outer step: the FP32 right-hand side is r / rn)
struct Reliable {
  double *x64;
  const double *b64;
  double *r64, *ax64;
  double rn;
  int replacements = 0;
};

// preconditioned CG on A x = b (vectors of type T, x holds the start);
// stops when |r| <= tol_abs or after max_iter iterations.  In FP32 the
// recursively updated residual can stall above a tolerance close to the
// precision: the inner solves of the refinement also stop once |r| has not
// halved over kStall iterations (the outer step continues from there).
constexpr int kStall = 100;

template <typename T>
int pcg(Solver &S, PrecState &P, const sf_solve_opts &o, const T *b, T *x, double tol_abs, int max_iter,
        bool proj, int &iters, double &rr_final, Reliable *rel = nullptr)
{
  const long long n = S.n;
  const int g = grid_for(n);
  int e;
  Work &W = P.work;
  T *r = (T *)W.r.ptr, *p = (T *)W.p.ptr, *ap = (T *)W.ap.ptr;
  T *z = o.precond == SF_PRECOND_NONE ? r : (T *)W.z.ptr;
  T *t = (T *)P.t.ptr;
  const T *dinv = (const T *)P.dinv.ptr;
  const T s0 = o.precond == SF_PRECOND_CHEBYSHEV ? T(1.0 / cheb_coef(P, o).theta) : T(1);
  if ((e = S.begin(tol_abs * tol_abs))) return e;
  // r = b - A x, z = M r, p = z
  if ((e = S.vmult(prec_of<T>(), x, ap))) return e;
  sub_kernel<T><<<g, kThreads, 0, S.st>>>(n, r, b, ap);
  if (proj && (e = S.project(r))) return e;
  if (o.precond == SF_PRECOND_JACOBI)
    precond_first<T, PC_JACOBI><<<g, kThreads, 0, S.st>>>(n, r, dinv, z, t, s0);
  if (o.precond == SF_PRECOND_CHEBYSHEV) {
    precond_first<T, PC_CHEB><<<g, kThreads, 0, S.st>>>(n, r, dinv, z, t, s0);
    if ((e = cheb_rest<T>(S, P, o, r, z))) return e;
  }
  if (proj && z != r && (e = S.project(z))) return e;
  copy_kernel<T><<<g, kThreads, 0, S.st>>>(n, p, z);
  if ((e = S.reduce<T, RED_RZ>(r, z))) return e;
  Scalars h;
  if ((e = S.read(&h))) return e;
  iters = 0;
  rr_final = h.rr;
  if (h.breakdown) {
    set_error("CG breakdown (non-finite residual)");
    return SF_ERR_BREAKDOWN;
  }
  if (h.done) return SF_OK;
  double best = h.rr;
  int best_k = 0;
  double rr_ref = h.rr; // recursive residual at the start or the last replacement
  // iterations, queued one ahead of the host's convergence check
  for (int k = 0; k < max_iter; ++k) {
    if ((e = S.vmult(prec_of<T>(), p, ap))) return e;
    if ((e = S.reduce<T, RED_PAP>(p, ap))) return e;
    if (o.precond == SF_PRECOND_NONE)
      update_xr_precond<T, PC_NONE><<<g, kThreads, 0, S.st>>>(n, x, r, p, ap, dinv, z, t, s0, S.sc);
    else if (o.precond == SF_PRECOND_JACOBI)
      update_xr_precond<T, PC_JACOBI><<<g, kThreads, 0, S.st>>>(n, x, r, p, ap, dinv, z, t, s0, S.sc);
    else
      update_xr_precond<T, PC_CHEB><<<g, kThreads, 0, S.st>>>(n, x, r, p, ap, dinv, z, t, s0, S.sc);
    SF_CUDA_TRY(cudaGetLastError());
    if (o.precond == SF_PRECOND_CHEBYSHEV && (e = cheb_rest<T>(S, P, o, r, z))) return e;
    if (proj && z != r && (e = S.project(z))) return e;
    if ((e = S.reduce<T, RED_RZ>(r, z))) return e;
    update_p<T><<<g, kThreads, 0, S.st>>>(n, p, z, S.sc);
    SF_CUDA_TRY(cudaGetLastError());
    if ((e = S.post(k & 1))) return e;
    if (k > 0) {
      if ((e = S.fetch((k - 1) & 1, &h))) return e;
      if (h.done) {
        iters = k; // iteration k was queued after convergence and changed nothing
        break;
      }
      if constexpr (sizeof(T) == 4) if (rel && h.rr < o.inner_rtol * o.inner_rtol * rr_ref) {
        // residual replacement after the queued iteration k: fold the FP32
        // correction into the FP64 iterate, form the true residual in FP64,
        // take it (in the FP32 system's scale) as the residual, precondition
        // it and continue with the same search direction p
        add_f32_scaled<<<g, kThreads, 0, S.st>>>(n, rel->x64, x, rel->rn);
        SF_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(T) * n, S.st));
        if ((e = S.vmult(SF_FP64, rel->x64, rel->ax64))) return e;
        sub_kernel<double><<<g, kThreads, 0, S.st>>>(n, rel->r64, rel->b64, rel->ax64);
        if (proj && (e = S.project(rel->r64))) return e;
        to_f32_times<<<g, kThreads, 0, S.st>>>(n, r, rel->r64, 1.0 / rel->rn);
        if (o.precond == SF_PRECOND_JACOBI)
          precond_first<T, PC_JACOBI><<<g, kThreads, 0, S.st>>>(n, r, dinv, z, t, s0);
        if (o.precond == SF_PRECOND_CHEBYSHEV) {
          precond_first<T, PC_CHEB><<<g, kThreads, 0, S.st>>>(n, r, dinv, z, t, s0);
          if ((e = cheb_rest<T>(S, P, o, r, z))) return e;
        }
        if (proj && z != r && (e = S.project(z))) return e;
        if ((e = S.reduce<T, RED_RZ>(r, z))) return e;
        SF_CUDA_TRY(cudaGetLastError());
        ++rel->replacements;
        rr_ref = h.rr;
        best = h.rr;
        best_k = k;
      }
      if (h.rr < 0.25 * best) {
        best = h.rr;
        best_k = k;
      } else if (sizeof(T) == 4 && k - best_k > kStall) {
        iters = k + 1;
        break;
      }
    }
    iters = k + 1;
  }
  if ((e = S.read(&h))) return e;
  if (h.breakdown) {
    set_error("CG breakdown (non-positive curvature or non-finite residual)");
    return SF_ERR_BREAKDOWN;
  }
  rr_final = h.rr;
  return SF_OK;
}

// solver caches live beside the handle (keyed by handle address)
std::vector<SolverCache *> g_caches;
std::mutex g_cache_mutex;

SolverCache *solver_cache(sf_op *op)
{
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  for (auto *c : g_caches)
    if (c->op == op) return c;
  auto *c = new SolverCache();
  c->op = op;
  g_caches.push_back(c);
  return c;
}

template <typename T>
int prepare_precision(Solver &S, PrecState &P, const sf_solve_opts &o, bool proj)
{
  int e;
  if ((e = P.work.ensure<T>(S.n))) return e;
  if (o.precond != SF_PRECOND_NONE && (e = ensure_diag<T>(S, P))) return e;
  if (o.precond == SF_PRECOND_CHEBYSHEV) {
    if ((e = ensure_eig<T>(S, P, o.eig_iterations, proj))) return e;
    const size_t b = sizeof(T) * (size_t)S.n;
    if (P.t.bytes != b && ((e = P.t.alloc(b)) || (e = P.z2.alloc(b)))) return e;
  }
  return SF_OK;
}

int ensure_buf(DevBuf &d, size_t bytes) { return d.bytes == bytes ? SF_OK : d.alloc(bytes); }

} // namespace

void release_solver_cache(sf_op *op)
{
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  for (size_t i = 0; i < g_caches.size(); ++i)
    if (g_caches[i]->op == op) {
      delete g_caches[i];
      g_caches.erase(g_caches.begin() + i);
      return;
    }
}

} // namespace sf

using namespace sf;

extern "C" void sf_solve_opts_default(sf_solve_opts *o)
{
  if (!o) return;
  o->mode = SF_SOLVE_FP64;
  o->precond = SF_PRECOND_CHEBYSHEV;
  o->cheb_degree = 5;
  o->cheb_range = 15.0;
  o->eig_iterations = 12;
  o->rtol = 1e-10;
  o->max_iter = 2000;
  o->inner_rtol = 0.03;
  o->project_constant = 0;
}

extern "C" int sf_cg_solve(sf_op *op, const double *b, double *x, const sf_solve_opts *opts,
                           sf_solve_stats *stats, void *stream)
{
  if (!op || !b || !x || !opts) {
    set_error("op/b/x/opts is NULL");
    return SF_ERR_NULL;
  }
  if (reinterpret_cast<uintptr_t>(b) % sizeof(double) || reinterpret_cast<uintptr_t>(x) % sizeof(double)) {
    set_error("b/x not aligned to the element size");
    return SF_ERR_ALIGN;
  }
  const sf_solve_opts o = *opts;
  if (o.mode != SF_SOLVE_FP64 && o.mode != SF_SOLVE_MIXED) {
    set_error("unknown solve mode");
    return SF_ERR_INVALID;
  }
  if (o.precond < SF_PRECOND_NONE || o.precond > SF_PRECOND_CHEBYSHEV || o.cheb_degree < 1 ||
      o.cheb_degree > 64 || !(o.cheb_range > 1.0) || !(o.rtol > 0) || o.max_iter < 1 ||
      o.eig_iterations < 2 || o.eig_iterations > 200 || !(o.inner_rtol > 0 && o.inner_rtol < 1)) {
    set_error("invalid solver options");
    return SF_ERR_INVALID;
  }
  if (op->desc.kind == SF_OP_DG_ADVECT || op->desc.kind == SF_OP_CONVECTION ||
      op->desc.kind == SF_OP_LAPLACE_FACES || op->desc.kind == SF_OP_CONVECTION_FACES) {
    set_error("CG needs a symmetric operator; advection, convection and the face-term operators are not");
    return SF_ERR_STATE;
  }
  if (!(op->desc.precisions & 1) || (o.mode == SF_SOLVE_MIXED && !(op->desc.precisions & 2))) {
    set_error("solver needs FP64 (and for mixed mode FP32) prepared in desc.precisions");
    return SF_ERR_STATE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  Solver S;
  S.op = op;
  S.st = st;
  S.n = op->n_dofs;
  S.cache = solver_cache(op);
  int e = S.cache->init();
  if (e) return e;
  S.bind();
  const bool proj = o.project_constant != 0;
  const long long n = S.n;
  const int g = grid_for(n);
  const bool mixed = o.mode == SF_SOLVE_MIXED;
  PrecState &P = S.cache->st[mixed ? 1 : 0];
  // buffers and preconditioner setup (cached per handle) before the clock
  SolverCache &Cc = *S.cache;
  if ((e = ensure_buf(Cc.bcopy, sizeof(double) * n)) || (e = ensure_buf(Cc.r64, sizeof(double) * n)) ||
      (e = ensure_buf(Cc.ax64, sizeof(double) * n)))
    return e;
  if (mixed) {
    if ((e = ensure_buf(Cc.r32, sizeof(float) * n)) || (e = ensure_buf(Cc.d32, sizeof(float) * n))) return e;
    if ((e = prepare_precision<float>(S, P, o, proj))) return e;
  } else {
    if ((e = prepare_precision<double>(S, P, o, proj))) return e;
  }
  SF_CUDA_TRY(cudaStreamSynchronize(st));
  S.applies = 0;
  const auto t0 = std::chrono::steady_clock::now();

  // |b| (after projection of a copy when requested)
  double *bp = (double *)Cc.bcopy.ptr;
  SF_CUDA_TRY(cudaMemcpyAsync(bp, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  if ((e = S.begin(0.0))) return e;
  if (proj && (e = S.project(bp))) return e;
  if (proj && (e = S.project(x))) return e;
  if ((e = S.reduce<double, RED_RZ>(bp, bp))) return e;
  Scalars h;
  if ((e = S.read(&h))) return e;
  const double bnorm = std::sqrt(h.rr);
  int total_iters = 0, outer = 0, replacements = 0;
  double relres = 0.0;
  if (bnorm == 0.0) {
    SF_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
  } else if (!mixed) {
    double rr;
    if ((e = pcg<double>(S, P, o, bp, x, o.rtol * bnorm, o.max_iter, proj, total_iters, rr))) return e;
  } else {
    double *r = (double *)Cc.r64.ptr, *ax = (double *)Cc.ax64.ptr;
    float *r32 = (float *)Cc.r32.ptr, *d32 = (float *)Cc.d32.ptr;
    const int max_outer = 60;
    while (outer < max_outer) {
      if ((e = S.vmult(SF_FP64, x, ax))) return e;
      sub_kernel<double><<<g, kThreads, 0, st>>>(n, r, bp, ax);
      if (proj && (e = S.project(r))) return e;
      if ((e = S.begin(0.0))) return e;
      if ((e = S.reduce<double, RED_RZ>(r, r))) return e;
      if ((e = S.read(&h))) return e;
      const double rn = std::sqrt(h.rr);
      if (!std::isfinite(rn)) {
        set_error("non-finite residual");
        return SF_ERR_BREAKDOWN;
      }
      if (rn <= o.rtol * bnorm || total_iters >= o.max_iter) break;
      to_f32_scaled<<<g, kThreads, 0, st>>>(n, r32, r, S.sc);
      SF_CUDA_TRY(cudaMemsetAsync(d32, 0, sizeof(float) * n, st));
      // the FP32 solve, with reliable updates, reduces its unit residual as
      // far as the outer tolerance needs (with a factor 2 of margin)
      const double inner = std::fmin(0.5, 0.5 * o.rtol * bnorm / rn);
      int it = 0;
      double rr32;
      Reliable rel{x, bp, r, ax, rn};
      if ((e = pcg<float>(S, P, o, r32, d32, inner, o.max_iter - total_iters, proj, it, rr32, &rel))) return e;
      total_iters += it;
      replacements += rel.replacements;
      add_f32_scaled<<<g, kThreads, 0, st>>>(n, x, d32, rn);
      SF_CUDA_TRY(cudaGetLastError());
      ++outer;
      if (it == 0) break; // no progress possible
    }
  }
  // final true residual in FP64
  {
    double *r = (double *)Cc.r64.ptr, *ax = (double *)Cc.ax64.ptr;
    if ((e = S.vmult(SF_FP64, x, ax))) return e;
    sub_kernel<double><<<g, kThreads, 0, st>>>(n, r, bp, ax);
    if (proj && (e = S.project(r))) return e;
    if ((e = S.begin(0.0))) return e;
    if ((e = S.reduce<double, RED_RZ>(r, r))) return e;
    if ((e = S.read(&h))) return e;
    relres = bnorm > 0 ? std::sqrt(h.rr) / bnorm : 0.0;
  }
  SF_CUDA_TRY(cudaStreamSynchronize(st));
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) {
    stats->iterations = total_iters;
    stats->outer_iterations = outer + replacements;
    stats->rel_residual = relres;
    stats->lambda_max = P.lambda_max;
    stats->seconds = secs;
    stats->operator_applies = S.applies;
  }
  if (!(relres <= o.rtol * 1.0000001)) {
    set_error("not converged: relative residual " + std::to_string(relres));
    return SF_ERR_NOT_CONVERGED;
  }
  return SF_OK;
}
