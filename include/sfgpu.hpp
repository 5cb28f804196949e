// sfgpu.hpp -- C++ host layer over the C ABI (sfgpu.h) that mirrors the
// reference's evaluator classes, so that code written against
//   EvaluationCellLaplacian   (legacy/include/evaluation_cell_laplacian.h:26)
//   EvaluationDGLaplacian     (legacy/include/evaluation_dg_laplacian.h:33)
//   EvaluationDGAdvection     (legacy/include/evaluation_dg_advect.h:96)
// keeps its member-function names and argument meaning.  Differences:
//   - the vectors the reference keeps as private AlignedVector members are
//     DeviceVector members here (device memory, owned by the evaluator);
//   - failures throw sfgpu::Error (the reference aborts or throws a bare
//     `throw;`), carrying the sf_status code and sf_last_error() text;
//   - dim is fixed to 3; the degree is a template parameter as in the
//     reference; Number is float or double.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "sfgpu.h"

namespace sfgpu {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m + " (sf_status " + std::to_string(c) + ")"), code(c) {}
};

inline void check(int code)
{
  if (code != SF_OK) throw Error(code, sf_last_error());
}

inline void check_cuda(cudaError_t e)
{
  if (e != cudaSuccess) throw Error(SF_ERR_CUDA, cudaGetErrorString(e));
}

template <typename Number>
constexpr int precision_of() { return sizeof(Number) == 8 ? SF_FP64 : SF_FP32; }

// device array with host transfer helpers (replaces AlignedVector)
template <typename Number>
class DeviceVector {
public:
  DeviceVector() = default;
  explicit DeviceVector(std::size_t n) { resize(n); }
  DeviceVector(const DeviceVector &) = delete;
  DeviceVector &operator=(const DeviceVector &) = delete;
  DeviceVector(DeviceVector &&o) noexcept : ptr_(o.ptr_), n_(o.n_) { o.ptr_ = nullptr; o.n_ = 0; }
  DeviceVector &operator=(DeviceVector &&o) noexcept
  {
    if (this != &o) {
      if (ptr_) cudaFree(ptr_);
      ptr_ = o.ptr_;
      n_ = o.n_;
      o.ptr_ = nullptr;
      o.n_ = 0;
    }
    return *this;
  }
  ~DeviceVector() { if (ptr_) cudaFree(ptr_); }
  void resize(std::size_t n)
  {
    if (ptr_) cudaFree(ptr_);
    ptr_ = nullptr;
    n_ = 0;
    if (n) check_cuda(cudaMalloc(&ptr_, n * sizeof(Number)));
    n_ = n;
  }
  void fill(Number v)
  {
    std::vector<Number> h(n_, v);
    upload(h);
  }
  void upload(const std::vector<Number> &h)
  {
    if (h.size() != n_) throw Error(SF_ERR_INVALID, "upload size mismatch");
    check_cuda(cudaMemcpy(ptr_, h.data(), n_ * sizeof(Number), cudaMemcpyHostToDevice));
  }
  std::vector<Number> download() const
  {
    std::vector<Number> h(n_);
    check_cuda(cudaMemcpy(h.data(), ptr_, n_ * sizeof(Number), cudaMemcpyDeviceToHost));
    return h;
  }
  Number *begin() { return ptr_; }
  const Number *begin() const { return ptr_; }
  std::size_t size() const { return n_; }

private:
  Number *ptr_ = nullptr;
  std::size_t n_ = 0;
};

// a vector handed in by the caller must hold at least n entries: the C ABI
// cannot see buffer sizes, and a short one would be written past its end
template <typename Number>
inline void check_size(const DeviceVector<Number> &v, long long n, const char *name)
{
  if ((long long)v.size() < n)
    throw Error(SF_ERR_INVALID, std::string(name) + " holds " + std::to_string(v.size()) +
                                    " entries, the operator needs " + std::to_string(n));
}

// owning handle of one operator
class Operator {
public:
  Operator() = default;
  explicit Operator(const sf_desc &d) { check(sf_create(&d, &op_)); }
  Operator(const Operator &) = delete;
  Operator &operator=(const Operator &) = delete;
  Operator(Operator &&o) noexcept : op_(o.op_) { o.op_ = nullptr; }
  Operator &operator=(Operator &&o) noexcept
  {
    if (op_) sf_destroy(op_);
    op_ = o.op_;
    o.op_ = nullptr;
    return *this;
  }
  ~Operator() { if (op_) sf_destroy(op_); }
  sf_op *get() const { return op_; }
  // SF_KERNEL_AUTO (default) or SF_KERNEL_GENERIC: see sf_set_kernel_variant
  void set_kernel_variant(int variant) { check(sf_set_kernel_variant(op_, variant)); }
  long long n_dofs() const
  {
    long long n = 0, c = 0;
    check(sf_sizes(op_, &n, &c));
    return n;
  }

private:
  sf_op *op_ = nullptr;
};

inline sf_desc make_desc(int kind, int degree, const unsigned *n_cells, const double *length)
{
  sf_desc d{};
  d.kind = kind;
  d.degree = degree;
  for (int k = 0; k < 3; ++k) {
    d.n_cells[k] = (int)n_cells[k];
    d.length[k] = length ? length[k] : 1.0;
  }
  d.basis = SF_BASIS_GLL;
  d.dirichlet = 1;
  d.penalty = 1.0;
  d.velocity[0] = 1.0;
  d.velocity[1] = 0.15;
  d.velocity[2] = -0.05;
  d.inverse_mass = 1;
  d.precisions = 3;
  return d;
}

// Continuous FE Laplacian with global numbering and homogeneous Dirichlet
// conditions (evaluation_cell_laplacian.h:26-908 operates on a cell-local
// E-vector; here the vectors are global).  matrix_vector_product():
// output_array = A input_array.
template <int degree, typename Number>
class EvaluationCellLaplacian {
public:
  static constexpr unsigned int dimension = 3;
  static constexpr unsigned int dofs_per_cell = (degree + 1) * (degree + 1) * (degree + 1);

  // the reference's compile-time variants of this class, DO_MASS_MATRIX and
  // DO_CONVECTION (evaluation_cell_laplacian.h:22-24, :299-354): set to
  // SF_OP_MASS or SF_OP_CONVECTION before initialize() (affine meshes);
  // the convection velocity defaults to the reference's b_d = d + 1.
  // DO_FACES (:505-797): SF_OP_LAPLACE_FACES or SF_OP_CONVECTION_FACES, which
  // act on a cell-major E-vector (n_cells (degree+1)^3 entries, Hermite-like
  // basis) as the reference's class does
  int cell_operator = SF_OP_LAPLACE;
  double convection[3] = {1.0, 2.0, 3.0};

  void initialize(const unsigned *n_cells, const double *length = nullptr, double deform = 0.0,
                  int basis = SF_BASIS_GLL, bool dirichlet = true)
  {
    sf_desc d = make_desc(cell_operator, degree, n_cells, length);
    for (int k = 0; k < 3; ++k) d.velocity[k] = convection[k];
    d.deform = deform;
    d.basis = basis;
    d.dirichlet = dirichlet ? 1 : 0;
    op_ = Operator(d);
    input_array.resize((std::size_t)op_.n_dofs());
    output_array.resize((std::size_t)op_.n_dofs());
  }
  std::size_t n_dofs() const { return input_array.size(); }
  void matrix_vector_product(cudaStream_t s = 0)
  {
    check(sf_vmult(op_.get(), precision_of<Number>(), input_array.begin(), output_array.begin(), s));
  }
  const Operator &op() const { return op_; }

  DeviceVector<Number> input_array, output_array;

private:
  Operator op_;
};

// DG SIPG Laplacian on a periodic box (evaluation_dg_laplacian.h:33-716).
template <int degree, typename Number>
class EvaluationDGLaplacian {
public:
  static constexpr unsigned int dimension = 3;
  static constexpr unsigned int dofs_per_cell = (degree + 1) * (degree + 1) * (degree + 1);
  // cache blocking of the reference's OpenMP loops; accepted and ignored
  unsigned int blx = 0, bly = 0, blz = 0;

  // evaluation_dg_laplacian.h:43-108: vectors initialised to
  // sol_old = 1, sol_new = 0, mat_diagonal = 1, sol_tmp = 0, sol_rhs = 1
  void initialize(const unsigned *n_cells, const double *length = nullptr, double penalty = 1.0)
  {
    sf_desc d = make_desc(SF_OP_DG_SIPG, degree, n_cells, length);
    d.penalty = penalty;
    op_ = Operator(d);
    const std::size_t n = (std::size_t)op_.n_dofs();
    for (auto *v : {&sol_old, &sol_new, &mat_diagonal, &sol_tmp, &sol_rhs}) v->resize(n);
    sol_old.fill(Number(1));
    sol_new.fill(Number(0));
    mat_diagonal.fill(Number(1));
    sol_tmp.fill(Number(0));
    sol_rhs.fill(Number(1));
  }
  std::size_t n_elements() const { return sol_old.size() / dofs_per_cell; }

  // evaluation_dg_laplacian.h:121-123: sol_tmp = A sol_new
  void do_matvec(cudaStream_t s = 0)
  {
    check(sf_vmult(op_.get(), precision_of<Number>(), sol_new.begin(), sol_tmp.begin(), s));
  }
  // evaluation_dg_laplacian.h:125-127 with the reference's coefficients
  void do_chebyshev(cudaStream_t s = 0)
  {
    do_cheby_iter<true>(sol_rhs, sol_old, mat_diagonal, sol_new, sol_tmp, Number(0.5), Number(0.5), s);
  }
  // evaluation_dg_laplacian.h:513-554.  With evaluate_chebyshev = false:
  // sol_new = A sol_old.  With true: vec_tm = c_tm vec_tm + c_np
  // mat_diagonal (A sol_old - src); sol_new = sol_old - vec_tm.
  template <bool evaluate_chebyshev = true>
  void do_cheby_iter(const DeviceVector<Number> &src, const DeviceVector<Number> &sol_old_,
                     const DeviceVector<Number> &mat_diagonal_, DeviceVector<Number> &sol_new_,
                     DeviceVector<Number> &vec_tm, Number coefficient_np, Number coefficient_tm,
                     cudaStream_t s = 0)
  {
    const long long n = op_.n_dofs();
    check_size(sol_old_, n, "sol_old");
    check_size(sol_new_, n, "sol_new");
    if (evaluate_chebyshev) {
      check_size(src, n, "src");
      check_size(mat_diagonal_, n, "mat_diagonal");
      check_size(vec_tm, n, "vec_tm");
    }
    if (!evaluate_chebyshev)
      check(sf_vmult(op_.get(), precision_of<Number>(), sol_old_.begin(), sol_new_.begin(), s));
    else
      check(sf_chebyshev_step(op_.get(), precision_of<Number>(), src.begin(), mat_diagonal_.begin(),
                              sol_old_.begin(), sol_new_.begin(), vec_tm.begin(), coefficient_np,
                              coefficient_tm, s));
  }
  // evaluation_dg_laplacian.h:556-601 (coefficients 0.6 and 0.45)
  void emulate_cheby_vector_updates(cudaStream_t s = 0)
  {
    check(sf_vector_update((long long)sol_new.size(), precision_of<Number>(), sol_new.begin(),
                           sol_rhs.begin(), mat_diagonal.begin(), sol_old.begin(), sol_new.begin(),
                           sol_tmp.begin(), 0.45, 0.6, s));
  }
  const Operator &op() const { return op_; }

  DeviceVector<Number> sol_old, sol_new, sol_rhs, sol_tmp, mat_diagonal;

private:
  Operator op_;
};

// DG SIPG Laplacian in tensor-product form with precomputed 1D matrices
// (precomputed_dg_laplacian.h:33-391): unit cells unless lengths are given.
template <int degree, typename Number>
class PrecomputedDGLaplacian {
public:
  static constexpr unsigned int dimension = 3;
  static constexpr unsigned int dofs_per_cell = (degree + 1) * (degree + 1) * (degree + 1);
  unsigned int blx = 0, bly = 0, blz = 0;

  // precomputed_dg_laplacian.h:44-82: input_array = 1, output_array = 0
  void initialize(const unsigned *n_cells, const double *length = nullptr)
  {
    double unit[3] = {double(n_cells[0]), double(n_cells[1]), double(n_cells[2])};
    sf_desc d = make_desc(SF_OP_DG_PRECOMPUTED, degree, n_cells, length ? length : unit);
    op_ = Operator(d);
    const std::size_t n = (std::size_t)op_.n_dofs();
    input_array.resize(n);
    output_array.resize(n);
    input_array.fill(Number(1));
    output_array.fill(Number(0));
  }
  std::size_t n_elements() const { return input_array.size() / dofs_per_cell; }
  // precomputed_dg_laplacian.h:279-305: output_array = A input_array
  void matrix_vector_product(cudaStream_t s = 0)
  {
    check(sf_vmult(op_.get(), precision_of<Number>(), input_array.begin(), output_array.begin(), s));
  }
  const Operator &op() const { return op_; }

  DeviceVector<Number> input_array, output_array;

private:
  Operator op_;
};

// DG upwind advection on the periodic box [0,2]^3 (evaluation_dg_advect.h:96-845).
template <int degree, typename Number>
class EvaluationDGAdvection {
public:
  static constexpr unsigned int dimension = 3;
  static constexpr unsigned int dofs_per_cell = (degree + 1) * (degree + 1) * (degree + 1);
  unsigned int blx = 0, bly = 0, blz = 0;

  // evaluation_dg_advect.h:107-180: sol_new = the analytic wave
  // sin(4 pi x) cos(4 pi y) cos(4 pi z) at the GLL nodes, domain [0,2]^3,
  // velocity (1, 0.15, -0.05); sol_old = sol_tmp = 0
  void initialize(const unsigned *n_cells, const double *velocity = nullptr)
  {
    const double L[3] = {2.0, 2.0, 2.0};
    sf_desc d = make_desc(SF_OP_DG_ADVECT, degree, n_cells, L);
    if (velocity)
      for (int k = 0; k < 3; ++k) d.velocity[k] = velocity[k];
    op_ = Operator(d);
    const std::size_t n = (std::size_t)op_.n_dofs();
    for (auto *v : {&sol_old, &sol_new, &sol_tmp}) v->resize(n);
    sol_old.fill(Number(0));
    sol_tmp.fill(Number(0));
    // GLL nodes on [0,1] from the Gauss-point table interface
    double S[81], D[81], xq[9], w[9];
    check(sf_shape_tables(degree, SF_BASIS_GLL, S, D, xq, w));
    std::vector<double> gll = gll_points();
    std::vector<Number> h(n);
    const double pi = 3.14159265358979323846, k = 4.0;
    std::size_t c = 0;
    for (unsigned iz = 0; iz < n_cells[2]; ++iz)
      for (unsigned iy = 0; iy < n_cells[1]; ++iy)
        for (unsigned ix = 0; ix < n_cells[0]; ++ix)
          for (int lz = 0; lz <= degree; ++lz)
            for (int ly = 0; ly <= degree; ++ly)
              for (int lx = 0; lx <= degree; ++lx, ++c) {
                const double x = (ix + gll[lx]) * 2.0 / n_cells[0];
                const double y = (iy + gll[ly]) * 2.0 / n_cells[1];
                const double z = (iz + gll[lz]) * 2.0 / n_cells[2];
                h[c] = Number(std::sin(k * x * pi) * std::cos(k * y * pi) * std::cos(k * z * pi));
              }
    sol_new.upload(h);
    for (int k2 = 0; k2 < 3; ++k2) {
      n_cells_[k2] = n_cells[k2];
      velocity_[k2] = d.velocity[k2];
    }
    // evaluation_dg_advect.h:160-165: 0.2 / (cells per unit length) / |a| / p
    const double an = std::sqrt(velocity_[0] * velocity_[0] + velocity_[1] * velocity_[1] +
                                velocity_[2] * velocity_[2]);
    time_step = 0.2 / (n_cells[0] / 2.0) / an / degree;
  }
  std::size_t n_elements() const { return sol_new.size() / dofs_per_cell; }
  // evaluation_dg_advect.h:216-219: sol_tmp = M^-1 A sol_new
  void do_matvec(cudaStream_t s = 0)
  {
    check(sf_vmult(op_.get(), precision_of<Number>(), sol_new.begin(), sol_tmp.begin(), s));
  }
  // evaluation_dg_advect.h:679-707: with evaluate_stage, vec_np = upd +
  // c_np M^-1 A src and vec_tm = vec_np + c_tm M^-1 A src (when c_tm != 0);
  // without, vec_np = M^-1 A src.  current_time only names the transport
  // direction in the reference; the handle's velocity is used here.
  template <bool evaluate_stage = true>
  void do_rk_stage(const DeviceVector<Number> &src, const DeviceVector<Number> &upd,
                   DeviceVector<Number> &vec_np, DeviceVector<Number> &vec_tm, double /*current_time*/,
                   Number c_np, Number c_tm, cudaStream_t s = 0)
  {
    const long long n = op_.n_dofs();
    check_size(src, n, "src");
    check_size(vec_np, n, "vec_np");
    if (evaluate_stage) {
      check_size(upd, n, "upd");
      if (c_tm != Number(0)) check_size(vec_tm, n, "vec_tm");
    }
    if (evaluate_stage)
      check(sf_rk_stage(op_.get(), precision_of<Number>(), 1, src.begin(), upd.begin(), vec_np.begin(),
                        vec_tm.begin(), double(c_np), double(c_tm), s));
    else
      check(sf_vmult(op_.get(), precision_of<Number>(), src.begin(), vec_np.begin(), s));
  }
  // evaluation_dg_advect.h:190-214: one LSRK(5,4) step of size time_step
  void do_time_step(double &current_time, cudaStream_t s = 0)
  {
    check(sf_lsrk_step(op_.get(), precision_of<Number>(), 1, sol_new.begin(), sol_old.begin(), sol_tmp.begin(),
                       time_step, s));
    current_time += time_step;
  }
  // evaluation_dg_advect.h:253-283: max |exact(time) - sol_new| over the nodes
  double compute_max_error(double time) const
  {
    const std::vector<Number> u = sol_new.download();
    const std::vector<double> gll = gll_points();
    const double pi = 3.14159265358979323846, k = 4.0;
    double err = 0.0;
    std::size_t c = 0;
    for (unsigned iz = 0; iz < n_cells_[2]; ++iz)
      for (unsigned iy = 0; iy < n_cells_[1]; ++iy)
        for (unsigned ix = 0; ix < n_cells_[0]; ++ix)
          for (int lz = 0; lz <= degree; ++lz)
            for (int ly = 0; ly <= degree; ++ly)
              for (int lx = 0; lx <= degree; ++lx, ++c) {
                const double x = (ix + gll[lx]) * 2.0 / n_cells_[0] - time * velocity_[0];
                const double y = (iy + gll[ly]) * 2.0 / n_cells_[1] - time * velocity_[1];
                const double z = (iz + gll[lz]) * 2.0 / n_cells_[2] - time * velocity_[2];
                const double e = std::sin(k * x * pi) * std::cos(k * y * pi) * std::cos(k * z * pi);
                err = std::fmax(err, std::fabs(e - double(u[c])));
              }
    return err;
  }
  const Operator &op() const { return op_; }

  DeviceVector<Number> sol_old, sol_new, sol_tmp;
  double time_step = 0.0;

private:
  static std::vector<double> gll_points()
  {
    // zeros of P'_{p}: Newton on the Legendre recurrence derivative
    std::vector<double> x(degree + 1);
    x[0] = 0.0;
    x[degree] = 1.0;
    for (int i = 1; i < degree; ++i) {
      double z = -std::cos(3.14159265358979323846 * i / degree);
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = z;
        for (int k2 = 2; k2 <= degree; ++k2) {
          const double p2 = ((2.0 * k2 - 1.0) * z * p1 - (k2 - 1.0) * p0) / k2;
          p0 = p1;
          p1 = p2;
        }
        const double dp = degree * (z * p1 - p0) / (z * z - 1.0);           // P'_p
        const double d2p = (2.0 * z * dp - degree * (degree + 1.0) * p1) / (1.0 - z * z); // P''_p
        const double dz = dp / d2p;
        z -= dz;
        if (std::fabs(dz) < 1e-15) break;
      }
      x[i] = 0.5 + 0.5 * z;
    }
    return x;
  }
  Operator op_;
  unsigned n_cells_[3] = {0, 0, 0};
  double velocity_[3] = {0.0, 0.0, 0.0};
};

} // namespace sfgpu
