// Drives the C++ evaluator classes of include/sfgpu.hpp the way the
// reference's drivers drive theirs (initialize, matrix_vector_product /
// do_matvec / do_chebyshev / emulate_cheby_vector_updates) and checks the
// results against the CPU oracle.  Built and run by tests/test_cpp_api_gpu.py.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "sf_oracle.h"
#include "sfgpu.hpp"

static double rel(const std::vector<double> &a, const std::vector<double> &b)
{
  double d = 0, n = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    d += (a[i] - b[i]) * (a[i] - b[i]);
    n += b[i] * b[i];
  }
  return std::sqrt(d / (n > 0 ? n : 1e-300));
}

int main()
{
  int fails = 0;
  std::mt19937_64 gen(20241203);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  // continuous Laplacian, deformed, p = 4
  {
    const unsigned nc[3] = {6, 5, 4};
    const double L[3] = {1.0, 0.9, 0.7};
    sfgpu::EvaluationCellLaplacian<4, double> ev;
    ev.initialize(nc, L, 0.05);
    std::vector<double> x(ev.n_dofs());
    for (auto &v : x) v = U(gen);
    ev.input_array.upload(x);
    ev.matrix_vector_product();
    cudaDeviceSynchronize();
    const std::vector<double> y = ev.output_array.download();
    sfo_mesh m{4, SFO_BASIS_GLL, {6, 5, 4}, {1.0, 0.9, 0.7}, 0.05, 1};
    std::vector<double> G((size_t)6 * 5 * 4 * 6 * 125), yr(y.size());
    sfo_cont_geometry(&m, G.data());
    sfo_cont_apply(&m, G.data(), nullptr, x.data(), yr.data(), 0);
    const double e = rel(y, yr);
    std::printf("EvaluationCellLaplacian<4,double>::matrix_vector_product rel err %.3e\n", e);
    fails += !(e < 1e-12);
  }
  // the DO_MASS_MATRIX / DO_CONVECTION variants of the cell evaluator, p = 3
  for (int kind : {SF_OP_MASS, SF_OP_CONVECTION}) {
    const unsigned nc[3] = {5, 4, 3};
    const double L[3] = {1.0, 0.8, 0.6};
    sfgpu::EvaluationCellLaplacian<3, double> ev;
    ev.cell_operator = kind;
    ev.initialize(nc, L);
    std::vector<double> x(ev.n_dofs());
    for (auto &v : x) v = U(gen);
    ev.input_array.upload(x);
    ev.matrix_vector_product();
    cudaDeviceSynchronize();
    const std::vector<double> y = ev.output_array.download();
    sfo_mesh m{3, SFO_BASIS_GLL, {5, 4, 3}, {1.0, 0.8, 0.6}, 0.0, 1};
    std::vector<double> yr(y.size());
    const double b[3] = {1.0, 2.0, 3.0};
    sfo_cont_apply_op(&m, kind == SF_OP_MASS ? 1 : 2, b, x.data(), yr.data());
    const double e = rel(y, yr);
    std::printf("EvaluationCellLaplacian<3,double> (%s) rel err %.3e\n",
                kind == SF_OP_MASS ? "DO_MASS_MATRIX" : "DO_CONVECTION", e);
    fails += !(e < 1e-12);
  }
  // the DO_FACES variants (cell-major E-vector), p = 4
  for (int kind : {SF_OP_LAPLACE_FACES, SF_OP_CONVECTION_FACES}) {
    const unsigned nc[3] = {3, 2, 2};
    const double L[3] = {0.75, 1.0, 1.5};
    sfgpu::EvaluationCellLaplacian<4, float> ev;
    ev.cell_operator = kind;
    ev.initialize(nc, L);
    std::vector<double> x(ev.n_dofs()), yr(ev.n_dofs());
    std::vector<float> xf(x.size());
    for (size_t i = 0; i < x.size(); ++i) xf[i] = (float)(x[i] = U(gen));
    ev.input_array.upload(xf);
    ev.matrix_vector_product();
    cudaDeviceSynchronize();
    const std::vector<float> yf = ev.output_array.download();
    const std::vector<double> y(yf.begin(), yf.end());
    const double h[3] = {0.25, 0.5, 0.75}, b[3] = {1.0, 2.0, 3.0};
    sfo_cell_faces_apply(4, kind == SF_OP_CONVECTION_FACES, 12, h, b, x.data(), yr.data());
    const double e = rel(y, yr);
    std::printf("EvaluationCellLaplacian<4,float> (%s) rel err %.3e\n",
                kind == SF_OP_LAPLACE_FACES ? "DO_FACES" : "DO_FACES + DO_CONVECTION", e);
    fails += !(e < 6e-6);
  }
  // DG SIPG, p = 5: do_matvec, do_chebyshev, emulate_cheby_vector_updates
  {
    const unsigned nc[3] = {4, 3, 3};
    const double L[3] = {1.0, 0.75, 0.75};
    sfgpu::EvaluationDGLaplacian<5, double> ev;
    ev.blx = ev.bly = ev.blz = 4;
    ev.initialize(nc, L);
    std::vector<double> x(ev.sol_new.size());
    for (auto &v : x) v = U(gen);
    ev.sol_new.upload(x);
    ev.do_matvec();
    cudaDeviceSynchronize();
    sfo_dg g{5, {4, 3, 3}, {0.25, 0.25, 0.25}, 1.0, {1, 0.5, 0.25}, 1};
    std::vector<double> yr(x.size());
    sfo_dg_sipg_apply(&g, x.data(), yr.data());
    const double e = rel(ev.sol_tmp.download(), yr);
    std::printf("EvaluationDGLaplacian<5,double>::do_matvec rel err %.3e\n", e);
    fails += !(e < 1e-12);
    // reference data: sol_old = 1 (A 1 = 0), rhs = 1, diag = 1, tmp = 0 ->
    // tmp = 0.5 * (0 - 1) = -0.5, sol_new = 1.5
    ev.sol_tmp.fill(0.0);
    ev.do_chebyshev();
    cudaDeviceSynchronize();
    double emax = 0;
    for (double v : ev.sol_new.download()) emax = std::fmax(emax, std::fabs(v - 1.5));
    std::printf("EvaluationDGLaplacian<5,double>::do_chebyshev max err %.3e\n", emax);
    fails += !(emax < 1e-12);
    // tmp = 0.6 tmp + 0.45 (new - rhs) = 0.6*(-0.5) + 0.45*0.5 = -0.075; new = 1 + 0.075
    ev.emulate_cheby_vector_updates();
    cudaDeviceSynchronize();
    emax = 0;
    for (double v : ev.sol_new.download()) emax = std::fmax(emax, std::fabs(v - 1.075));
    std::printf("EvaluationDGLaplacian<5,double>::emulate_cheby_vector_updates max err %.3e\n", emax);
    fails += !(emax < 1e-12);
  }
  // DG advection, p = 6, analytic initial field: M^-1 A u ~ du/dt
  {
    const unsigned nc[3] = {4, 4, 4};
    sfgpu::EvaluationDGAdvection<6, float> ev;
    ev.initialize(nc);
    ev.do_matvec();
    cudaDeviceSynchronize();
    const std::vector<float> y = ev.sol_tmp.download();
    const std::vector<float> u = ev.sol_new.download();
    sfo_dg g{6, {4, 4, 4}, {0.5, 0.5, 0.5}, 1.0, {1.0, 0.15, -0.05}, 1};
    std::vector<double> ud(u.begin(), u.end()), yr(u.size());
    sfo_dg_advect_apply(&g, ud.data(), yr.data());
    std::vector<double> yd(y.begin(), y.end());
    const double e = rel(yd, yr);
    std::printf("EvaluationDGAdvection<6,float>::do_matvec rel err %.3e\n", e);
    fails += !(e < 1e-5);
  }
  // DG advection time stepping, p = 4, FP64: LSRK(5,4) of the analytic wave
  // (the reference's do_time_step / compute_max_error driver)
  {
    const unsigned nc[3] = {16, 16, 16};
    sfgpu::EvaluationDGAdvection<4, double> ev;
    ev.initialize(nc);
    double t = 0.0;
    const double e0 = ev.compute_max_error(t);
    std::vector<double> xo = ev.sol_new.download(), oo(xo.size(), 0.0), to(xo.size(), 0.0);
    for (int s = 0; s < 20; ++s) ev.do_time_step(t);
    cudaDeviceSynchronize();
    const double e1 = ev.compute_max_error(t);
    sfo_dg g{4, {16, 16, 16}, {0.125, 0.125, 0.125}, 1.0, {1.0, 0.15, -0.05}, 1};
    for (int s = 0; s < 20; ++s) sfo_dg_lsrk_step(&g, ev.time_step, xo.data(), oo.data(), to.data());
    const double ep = rel(ev.sol_new.download(), xo);
    std::printf("EvaluationDGAdvection<4,double>::do_time_step x20 (t = %.4f): max error %.3e vs the exact "
                "wave (initial %.3e), rel. difference to the oracle %.3e\n", t, e1, e0, ep);
    fails += !(e1 < 2e-3 && e0 < 1e-14 && ep < 1e-12);
  }
  // precomputed tensor-product SIPG, p = 3, unit cells: the constant input of
  // initialize() is in the null space; a random field matches the oracle
  {
    const unsigned nc[3] = {4, 3, 2};
    sfgpu::PrecomputedDGLaplacian<3, double> ev;
    ev.initialize(nc);
    ev.matrix_vector_product();
    cudaDeviceSynchronize();
    double emax = 0;
    for (double v : ev.output_array.download()) emax = std::fmax(emax, std::fabs(v));
    std::vector<double> xr(ev.input_array.size()), yr(xr.size());
    for (std::size_t i = 0; i < xr.size(); ++i) xr[i] = std::sin(0.37 * double(i));
    ev.input_array.upload(xr);
    ev.matrix_vector_product();
    cudaDeviceSynchronize();
    sfo_dg g{3, {4, 3, 2}, {1.0, 1.0, 1.0}, 1.0, {0.0, 0.0, 0.0}, 0};
    sfo_dg_precomputed_apply(&g, xr.data(), yr.data());
    const double e = rel(ev.output_array.download(), yr);
    std::printf("PrecomputedDGLaplacian<3,double>::matrix_vector_product: constant -> %.3e, rel err %.3e\n", emax,
                e);
    fails += !(emax < 1e-12 && e < 1e-13);
  }
  std::printf(fails ? "FAILED\n" : "OK\n");
  return fails;
}
