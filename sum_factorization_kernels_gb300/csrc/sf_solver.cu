// sf_solver.cu -- conjugate gradients around the operators (no reference
// counterpart: the reference times operator applications only).
//
//  * SF_SOLVE_FP64: preconditioned CG with FP64 vectors and the FP64 operator.
//  * SF_SOLVE_MIXED: FP64 iterative refinement.  Each outer step forms the
//    true residual r = b - A x with the FP64 operator, solves A d = r / |r|
//    approximately with an FP32 preconditioned CG (FP32 operator, FP32
//    vectors, FP64 reductions) and updates x += |r| d in FP64.
//  * Preconditioners: none, Jacobi (inverse diagonal) or a Chebyshev
//    polynomial of D^-1 A (the smoother form of the reference's fused
//    Chebyshev step, evaluation_dg_laplacian.h:485-502) with lambda_max from
//    a Lanczos estimate built out of the CG coefficients of a few Jacobi-CG
//    steps, range [lambda_max / range, 1.2 lambda_max].
//  * Scalars (alpha, beta, dot products) stay on the device; the host reads
//    one residual norm per iteration to decide convergence.
//  * Periodic DG SIPG has the constants as null space: with
//    project_constant the right-hand side and every preconditioned residual
//    are projected to mean zero.
#include <chrono>
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
};

int grid_for(long long n)
{
  long long g = (n + kThreads - 1) / kThreads;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

template <typename T>
__global__ void dot2_partial(long long n, const T *__restrict__ r, const T *__restrict__ z,
                             double *__restrict__ part)
{
  __shared__ double s1[kThreads], s2[kThreads];
  double a = 0, b = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double ri = r[i];
    a = fma(ri, double(z[i]), a);
    b = fma(ri, ri, b);
  }
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
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = s2[0];
  }
}

// slot: 0 -> rz (and rr), 1 -> pAp, 2 -> sum
__global__ void dot2_final(const double *__restrict__ part, int nb, Scalars *sc, int slot)
{
  __shared__ double s1[kThreads], s2[kThreads];
  double a = 0, b = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    a += part[2 * i];
    b += part[2 * i + 1];
  }
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
  if (threadIdx.x == 0) {
    if (slot == 0) {
      sc->rz_old = sc->rz;
      sc->rz = s1[0];
      sc->rr = s2[0];
    } else if (slot == 1) {
      sc->pAp = s1[0];
    } else {
      sc->sum = s1[0];
    }
  }
}

template <typename T>
__global__ void sum_partial(long long n, const T *__restrict__ x, double *__restrict__ part)
{
  __shared__ double s1[kThreads];
  double a = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    a += double(x[i]);
  s1[threadIdx.x] = a;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s1[threadIdx.x] += s1[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = 0.0;
  }
}

template <typename T>
__global__ void subtract_mean(long long n, T *__restrict__ x, const Scalars *sc)
{
  const T m = T(sc->sum / double(n));
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] -= m;
}

// x += alpha p, r -= alpha Ap with alpha = rz / pAp
template <typename T>
__global__ void update_xr(long long n, T *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
                          const T *__restrict__ Ap, const Scalars *sc)
{
  const double al = sc->rz / sc->pAp;
  const T a = T(al);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    r[i] -= a * Ap[i];
  }
}

// p = z + beta p, beta = rz / rz_old
template <typename T>
__global__ void update_p(long long n, T *__restrict__ p, const T *__restrict__ z, const Scalars *sc)
{
  const T be = T(sc->rz / sc->rz_old);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = z[i] + be * p[i];
}

template <typename T>
__global__ void mul_kernel(long long n, T *__restrict__ z, const T *__restrict__ d, const T *__restrict__ r,
                           T s)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    z[i] = s * d[i] * r[i];
}

// z = s d r, t = -z (first Chebyshev step from a zero start)
template <typename T>
__global__ void cheb_first(long long n, T *__restrict__ z, T *__restrict__ t, const T *__restrict__ d,
                           const T *__restrict__ r, T s)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const T v = s * d[i] * r[i];
    z[i] = v;
    t[i] = -v;
  }
}

template <typename T>
__global__ void inverse_kernel(long long n, T *__restrict__ d)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    d[i] = d[i] != T(0) ? T(1) / d[i] : T(1);
}

// r = b - Ax  (FP64), also used to form scaled FP32 right-hand sides
__global__ void residual_kernel(long long n, double *__restrict__ r, const double *__restrict__ b,
                                const double *__restrict__ ax)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    r[i] = b[i] - ax[i];
}

__global__ void to_f32_scaled(long long n, float *__restrict__ y, const double *__restrict__ x,
                              const Scalars *sc)
{
  const double s = 1.0 / sqrt(sc->rr);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = float(x[i] * s);
}

__global__ void add_f32_scaled(long long n, double *__restrict__ x, const float *__restrict__ d,
                               const Scalars *sc)
{
  const double s = sqrt(sc->rr);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] += s * double(d[i]);
}

template <typename T>
__global__ void sub_kernel(long long n, T *__restrict__ r, const T *__restrict__ b, const T *__restrict__ ax)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    r[i] = b[i] - ax[i];
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

struct Solver {
  sf_op *op;
  cudaStream_t st;
  long long n;
  DevBuf part, scal;
  Scalars *sc = nullptr;
  double *part_d = nullptr;
  Scalars *host_sc = nullptr; // pinned
  int applies = 0;

  int init()
  {
    int r = part.alloc(sizeof(double) * 2 * kBlocks);
    if (r) return r;
    r = scal.alloc(sizeof(Scalars));
    if (r) return r;
    part_d = (double *)part.ptr;
    sc = (Scalars *)scal.ptr;
    SF_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(Scalars), st));
    SF_CUDA_TRY(cudaMallocHost(&host_sc, sizeof(Scalars)));
    return SF_OK;
  }
  ~Solver()
  {
    if (host_sc) cudaFreeHost(host_sc);
  }

  template <typename T>
  int dot2(const T *r, const T *z, int slot)
  {
    dot2_partial<T><<<kBlocks, kThreads, 0, st>>>(n, r, z, part_d);
    dot2_final<<<1, kThreads, 0, st>>>(part_d, kBlocks, sc, slot);
    SF_CUDA_TRY(cudaGetLastError());
    return SF_OK;
  }

  template <typename T>
  int project(T *x)
  {
    sum_partial<T><<<kBlocks, kThreads, 0, st>>>(n, x, part_d);
    dot2_final<<<1, kThreads, 0, st>>>(part_d, kBlocks, sc, 2);
    subtract_mean<T><<<grid_for(n), kThreads, 0, st>>>(n, x, sc);
    SF_CUDA_TRY(cudaGetLastError());
    return SF_OK;
  }

  int read_scalars()
  {
    SF_CUDA_TRY(cudaMemcpyAsync(host_sc, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    SF_CUDA_TRY(cudaStreamSynchronize(st));
    return SF_OK;
  }

  int vmult(int prec, const void *x, void *y)
  {
    ++applies;
    return sf_vmult(op, prec, x, y, st);
  }
};

// per-precision preconditioner state cached in the handle
struct PrecState {
  DevBuf dinv, z2, t;
  double lambda_max = 0.0;
  bool have_diag = false, have_eig = false;
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
template <typename T>
int ensure_eig(Solver &S, PrecState &P, int steps, bool proj)
{
  if (P.have_eig) return SF_OK;
  const long long n = S.n;
  DevBuf bx, rx, px, apx, zx;
  int e;
  if ((e = bx.alloc(sizeof(T) * n)) || (e = rx.alloc(sizeof(T) * n)) || (e = px.alloc(sizeof(T) * n)) ||
      (e = apx.alloc(sizeof(T) * n)) || (e = zx.alloc(sizeof(T) * n)))
    return e;
  T *r = (T *)rx.ptr, *p = (T *)px.ptr, *ap = (T *)apx.ptr, *z = (T *)zx.ptr, *x = (T *)bx.ptr;
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
  if (proj && (e = S.project(r))) return e;
  mul_kernel<T><<<grid_for(n), kThreads, 0, S.st>>>(n, z, (const T *)P.dinv.ptr, r, T(1));
  if (proj && (e = S.project(z))) return e;
  SF_CUDA_TRY(cudaMemcpyAsync(p, z, sizeof(T) * n, cudaMemcpyDeviceToDevice, S.st));
  if ((e = S.dot2(r, z, 0))) return e;
  std::vector<double> alpha, beta;
  for (int it = 0; it < steps; ++it) {
    if ((e = S.vmult(prec_of<T>(), p, ap))) return e;
    if ((e = S.dot2(p, ap, 1))) return e;
    if ((e = S.read_scalars())) return e;
    const double a = S.host_sc->rz / S.host_sc->pAp;
    if (!(S.host_sc->pAp > 0) || !std::isfinite(a)) break;
    alpha.push_back(a);
    update_xr<T><<<grid_for(n), kThreads, 0, S.st>>>(n, x, r, p, ap, S.sc);
    mul_kernel<T><<<grid_for(n), kThreads, 0, S.st>>>(n, z, (const T *)P.dinv.ptr, r, T(1));
    if (proj && (e = S.project(z))) return e;
    if ((e = S.dot2(r, z, 0))) return e;
    if ((e = S.read_scalars())) return e;
    const double b = S.host_sc->rz / S.host_sc->rz_old;
    if (!std::isfinite(b) || S.host_sc->rz <= 0) break;
    beta.push_back(b);
    update_p<T><<<grid_for(n), kThreads, 0, S.st>>>(n, p, z, S.sc);
  }
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

// z = M r
template <typename T>
int apply_precond(Solver &S, PrecState &P, const sf_solve_opts &o, const T *r, T *z, bool proj)
{
  const long long n = S.n;
  int e;
  if (o.precond == SF_PRECOND_NONE) {
    SF_CUDA_TRY(cudaMemcpyAsync(z, r, sizeof(T) * n, cudaMemcpyDeviceToDevice, S.st));
  } else if (o.precond == SF_PRECOND_JACOBI) {
    mul_kernel<T><<<grid_for(n), kThreads, 0, S.st>>>(n, z, (const T *)P.dinv.ptr, r, T(1));
  } else {
    const double lmax = 1.2 * P.lambda_max, lmin = lmax / o.cheb_range;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    T *t = (T *)P.t.ptr, *z2 = (T *)P.z2.ptr;
    cheb_first<T><<<grid_for(n), kThreads, 0, S.st>>>(n, z, t, (const T *)P.dinv.ptr, r, T(1.0 / theta));
    SF_CUDA_TRY(cudaGetLastError());
    double rho_old = delta / theta;
    T *cur = z, *nxt = z2;
    for (int k = 1; k < o.cheb_degree; ++k) {
      const double rho = 1.0 / (2.0 * theta / delta - rho_old);
      ++S.applies;
      e = sf_chebyshev_step(S.op, prec_of<T>(), r, P.dinv.ptr, cur, nxt, t, 2.0 * rho / delta,
                            rho * rho_old, S.st);
      if (e) return e;
      rho_old = rho;
      T *tmp = cur;
      cur = nxt;
      nxt = tmp;
    }
    if (cur != z) SF_CUDA_TRY(cudaMemcpyAsync(z, cur, sizeof(T) * n, cudaMemcpyDeviceToDevice, S.st));
  }
  SF_CUDA_TRY(cudaGetLastError());
  if (proj) return S.project(z);
  return SF_OK;
}

// CG work vectors of one precision
struct Work {
  DevBuf r, p, ap, z;
  template <typename T>
  int alloc(long long n)
  {
    int e;
    if ((e = r.alloc(sizeof(T) * n)) || (e = p.alloc(sizeof(T) * n)) || (e = ap.alloc(sizeof(T) * n)) ||
        (e = z.alloc(sizeof(T) * n)))
      return e;
    return SF_OK;
  }
};

// preconditioned CG on A x = b (vectors of type T, x holds the start);
// stops when |r| <= tol_abs or after max_iter iterations
template <typename T>
int pcg(Solver &S, PrecState &P, Work &W, const sf_solve_opts &o, const T *b, T *x, double tol_abs,
        int max_iter, bool proj, int &iters, double &rr_final)
{
  const long long n = S.n;
  int e;
  T *r = (T *)W.r.ptr, *p = (T *)W.p.ptr, *ap = (T *)W.ap.ptr, *z = (T *)W.z.ptr;
  if ((e = S.vmult(prec_of<T>(), x, ap))) return e;
  sub_kernel<T><<<grid_for(n), kThreads, 0, S.st>>>(n, r, b, ap);
  SF_CUDA_TRY(cudaGetLastError());
  if (proj && (e = S.project(r))) return e;
  if ((e = apply_precond<T>(S, P, o, r, z, proj))) return e;
  SF_CUDA_TRY(cudaMemcpyAsync(p, z, sizeof(T) * n, cudaMemcpyDeviceToDevice, S.st));
  if ((e = S.dot2(r, z, 0))) return e;
  if ((e = S.read_scalars())) return e;
  iters = 0;
  rr_final = S.host_sc->rr;
  while (iters < max_iter && std::sqrt(S.host_sc->rr) > tol_abs) {
    if ((e = S.vmult(prec_of<T>(), p, ap))) return e;
    if ((e = S.dot2(p, ap, 1))) return e;
    update_xr<T><<<grid_for(n), kThreads, 0, S.st>>>(n, x, r, p, ap, S.sc);
    if ((e = apply_precond<T>(S, P, o, r, z, proj))) return e;
    if ((e = S.dot2(r, z, 0))) return e;
    update_p<T><<<grid_for(n), kThreads, 0, S.st>>>(n, p, z, S.sc);
    SF_CUDA_TRY(cudaGetLastError());
    ++iters;
    if ((e = S.read_scalars())) return e;
    if (!(S.host_sc->pAp > 0) || !std::isfinite(S.host_sc->rr)) {
      set_error("CG breakdown (non-positive curvature or non-finite residual)");
      return SF_ERR_BREAKDOWN;
    }
    rr_final = S.host_sc->rr;
  }
  return SF_OK;
}

} // namespace

// preconditioner caches live beside the handle (keyed by handle address)
namespace {
struct PrecCache {
  sf_op *op;
  PrecState st[2];
};
std::vector<PrecCache *> g_caches;
std::mutex g_cache_mutex;

PrecState &prec_state(sf_op *op, int prec)
{
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  for (auto *c : g_caches)
    if (c->op == op) return c->st[prec];
  g_caches.push_back(new PrecCache{op, {}});
  return g_caches.back()->st[prec];
}
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
  o->inner_rtol = 1e-3;
  o->project_constant = 0;
}

extern "C" int sf_cg_solve(sf_op *op, const double *b, double *x, const sf_solve_opts *opts,
                           sf_solve_stats *stats, void *stream)
{
  if (!op || !b || !x || !opts) {
    set_error("op/b/x/opts is NULL");
    return SF_ERR_NULL;
  }
  const sf_solve_opts o = *opts;
  if (o.mode != SF_SOLVE_FP64 && o.mode != SF_SOLVE_MIXED) {
    set_error("unknown solve mode");
    return SF_ERR_INVALID;
  }
  if (o.precond < SF_PRECOND_NONE || o.precond > SF_PRECOND_CHEBYSHEV || o.cheb_degree < 1 ||
      o.cheb_degree > 64 || !(o.cheb_range > 1.0) || !(o.rtol > 0) || o.max_iter < 1 ||
      o.eig_iterations < 2 || o.eig_iterations > 200) {
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
  int e = S.init();
  if (e) return e;
  const bool proj = o.project_constant != 0;
  const long long n = S.n;
  SF_CUDA_TRY(cudaStreamSynchronize(st));
  const auto t0 = std::chrono::steady_clock::now();

  // |b| (after projection of a copy when requested)
  DevBuf bb;
  if ((e = bb.alloc(sizeof(double) * n))) return e;
  double *bp = (double *)bb.ptr;
  SF_CUDA_TRY(cudaMemcpyAsync(bp, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  if (proj && (e = S.project(bp))) return e;
  if (proj && (e = S.project(x))) return e;
  if ((e = S.dot2(bp, bp, 0))) return e;
  if ((e = S.read_scalars())) return e;
  const double bnorm = std::sqrt(S.host_sc->rr);
  int total_iters = 0, outer = 0;
  double relres = 0.0;
  if (bnorm == 0.0) {
    SF_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
  } else if (o.mode == SF_SOLVE_FP64) {
    PrecState &P = prec_state(op, 0);
    if (o.precond != SF_PRECOND_NONE && (e = ensure_diag<double>(S, P))) return e;
    if (o.precond == SF_PRECOND_CHEBYSHEV) {
      if ((e = ensure_eig<double>(S, P, o.eig_iterations, proj))) return e;
      if (P.t.bytes < sizeof(double) * n && ((e = P.t.alloc(sizeof(double) * n)) || (e = P.z2.alloc(sizeof(double) * n))))
        return e;
    }
    double rr;
    Work W;
    if ((e = W.alloc<double>(n))) return e;
    if ((e = pcg<double>(S, P, W, o, bp, x, o.rtol * bnorm, o.max_iter, proj, total_iters, rr))) return e;
  } else {
    PrecState &P = prec_state(op, 1);
    if (o.precond != SF_PRECOND_NONE && (e = ensure_diag<float>(S, P))) return e;
    if (o.precond == SF_PRECOND_CHEBYSHEV) {
      if ((e = ensure_eig<float>(S, P, o.eig_iterations, proj))) return e;
      if (P.t.bytes < sizeof(float) * n && ((e = P.t.alloc(sizeof(float) * n)) || (e = P.z2.alloc(sizeof(float) * n))))
        return e;
    }
    DevBuf rb, axb, r32b, d32b;
    if ((e = rb.alloc(sizeof(double) * n)) || (e = axb.alloc(sizeof(double) * n)) ||
        (e = r32b.alloc(sizeof(float) * n)) || (e = d32b.alloc(sizeof(float) * n)))
      return e;
    double *r = (double *)rb.ptr, *ax = (double *)axb.ptr;
    float *r32 = (float *)r32b.ptr, *d32 = (float *)d32b.ptr;
    Work W;
    if ((e = W.alloc<float>(n))) return e;
    const int max_outer = 60;
    while (outer < max_outer) {
      if ((e = S.vmult(SF_FP64, x, ax))) return e;
      residual_kernel<<<grid_for(n), kThreads, 0, st>>>(n, r, bp, ax);
      if (proj && (e = S.project(r))) return e;
      if ((e = S.dot2(r, r, 0))) return e;
      if ((e = S.read_scalars())) return e;
      const double rn = std::sqrt(S.host_sc->rr);
      if (!std::isfinite(rn)) {
        set_error("non-finite residual");
        return SF_ERR_BREAKDOWN;
      }
      if (rn <= o.rtol * bnorm || total_iters >= o.max_iter) break;
      to_f32_scaled<<<grid_for(n), kThreads, 0, st>>>(n, r32, r, S.sc);
      SF_CUDA_TRY(cudaMemsetAsync(d32, 0, sizeof(float) * n, st));
      // keep |r| for the back-scaling: stash it in sum slot via a tiny copy
      Scalars keep = *S.host_sc;
      int it = 0;
      double rr32;
      // inner tolerance relative to the unit right-hand side; never ask for
      // more than FP32 can deliver
      const double inner = std::fmax(o.inner_rtol, 1e-6);
      if ((e = pcg<float>(S, P, W, o, r32, d32, inner, o.max_iter - total_iters, proj, it, rr32))) return e;
      total_iters += it;
      // restore |r|^2 into the device scalars for the back-scaling
      SF_CUDA_TRY(cudaMemcpyAsync(&S.sc->rr, &keep.rr, sizeof(double), cudaMemcpyHostToDevice, st));
      add_f32_scaled<<<grid_for(n), kThreads, 0, st>>>(n, x, d32, S.sc);
      SF_CUDA_TRY(cudaGetLastError());
      SF_CUDA_TRY(cudaStreamSynchronize(st));
      ++outer;
      if (it == 0) break; // no progress possible
    }
  }
  // final true residual in FP64
  {
    DevBuf rb, axb;
    if ((e = rb.alloc(sizeof(double) * n)) || (e = axb.alloc(sizeof(double) * n))) return e;
    if ((e = S.vmult(SF_FP64, x, axb.ptr))) return e;
    residual_kernel<<<grid_for(n), kThreads, 0, st>>>(n, (double *)rb.ptr, bp, (const double *)axb.ptr);
    if (proj && (e = S.project((double *)rb.ptr))) return e;
    if ((e = S.dot2((double *)rb.ptr, (double *)rb.ptr, 0))) return e;
    if ((e = S.read_scalars())) return e;
    relres = bnorm > 0 ? std::sqrt(S.host_sc->rr) / bnorm : 0.0;
  }
  SF_CUDA_TRY(cudaStreamSynchronize(st));
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) {
    stats->iterations = total_iters;
    stats->outer_iterations = outer;
    stats->rel_residual = relres;
    stats->lambda_max = prec_state(op, o.mode == SF_SOLVE_MIXED ? 1 : 0).lambda_max;
    stats->seconds = secs;
    stats->operator_applies = S.applies;
  }
  if (!(relres <= o.rtol * 1.0000001)) {
    set_error("not converged: relative residual " + std::to_string(relres));
    return SF_ERR_NOT_CONVERGED;
  }
  return SF_OK;
}
