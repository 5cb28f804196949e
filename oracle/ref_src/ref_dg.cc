/*
 * Golden-vector adapter for the reference's DG operators
 * (legacy/include/evaluation_dg_laplacian.h, evaluation_dg_advect.h),
 * compiled from copies that oracle/build.py patches at build time
 * (see oracle/build.py: PATCHES).  TEST INFRASTRUCTURE ONLY.
 */
#include "ref_shim.h"
#include "evaluation_dg_laplacian.h"
#include "evaluation_dg_advect.h"
#include "precomputed_dg_laplacian.h"

template <typename Ev>
static void set_geometry(Ev &ev, const double *h)
{
  for (int d = 0; d < 3; ++d) ev.jacobian_data[d] = 1. / h[d];
  ev.jxw_data[0] = h[0] * h[1] * h[2];
}

/* mode 0: y = A x;  mode 1: fused Chebyshev step with rhs b, inverse
 * diagonal dinv, coefficients c_np, c_tm; x_new -> y, t updated in place */
template <int p>
static void sipg(const int *nc, const double *h, int mode, const double *x,
                 const double *b, const double *dinv, double *t, double c_np,
                 double c_tm, double *y)
{
  EvaluationDGLaplacian<3, p, double> ev;
  ev.blx = 2; ev.bly = 2; ev.blz = 2;
  unsigned int n_cells[3] = {(unsigned)nc[0], (unsigned)nc[1], (unsigned)nc[2]};
  ev.initialize(n_cells);
  set_geometry(ev, h);
  const std::size_t N = ev.n_elements() * ev.dofs_per_cell;
  AlignedVector<double> src(N), xo(N), dg(N), yo(N), tmp(N);
  for (std::size_t i = 0; i < N; ++i) xo[i] = x[i];
  if (mode == 0) {
    ev.template do_cheby_iter<false>(src, xo, dg, yo, tmp, 0., 0.);
  } else {
    for (std::size_t i = 0; i < N; ++i) { ev.sol_rhs[i] = b[i]; src[i] = b[i]; dg[i] = dinv[i]; tmp[i] = t[i]; }
    ev.template do_cheby_iter<true>(src, xo, dg, yo, tmp, c_np, c_tm);
    for (std::size_t i = 0; i < N; ++i) t[i] = tmp[i];
  }
  for (std::size_t i = 0; i < N; ++i) y[i] = yo[i];
}

/* y = M^-1 K x with the reference's velocity (1, 0.15, -0.05) */
template <int p>
static void advect(const int *nc, const double *h, const double *x, double *y)
{
  EvaluationDGAdvection<3, p, double> ev;
  ev.blx = 2; ev.bly = 2; ev.blz = 2;
  unsigned int n_cells[3] = {(unsigned)nc[0], (unsigned)nc[1], (unsigned)nc[2]};
  ev.initialize(n_cells);
  set_geometry(ev, h);
  const std::size_t N = ev.n_elements() * ev.dofs_per_cell;
  AlignedVector<double> src(N), upd(N), np(N), tm(N);
  for (std::size_t i = 0; i < N; ++i) src[i] = x[i];
  ev.template do_rk_stage<false>(src, upd, np, tm, 0., 0., 0.);
  for (std::size_t i = 0; i < N; ++i) y[i] = np[i];
}

/* one fused Runge-Kutta stage of the reference: r = M^-1 K src,
 * vec_np = upd + c_np r, vec_tm = vec_np + c_tm r (when c_tm != 0) */
template <int p>
static void rk_stage(const int *nc, const double *h, const double *src, const double *upd,
                     double c_np, double c_tm, double *vnp, double *vtm)
{
  EvaluationDGAdvection<3, p, double> ev;
  ev.blx = 2; ev.bly = 2; ev.blz = 2;
  unsigned int n_cells[3] = {(unsigned)nc[0], (unsigned)nc[1], (unsigned)nc[2]};
  ev.initialize(n_cells);
  set_geometry(ev, h);
  const std::size_t N = ev.n_elements() * ev.dofs_per_cell;
  AlignedVector<double> s(N), u(N), np(N), tm(N);
  for (std::size_t i = 0; i < N; ++i) { s[i] = src[i]; u[i] = upd[i]; tm[i] = vtm[i]; }
  ev.template do_rk_stage<true>(s, u, np, tm, 0., c_np, c_tm);
  for (std::size_t i = 0; i < N; ++i) { vnp[i] = np[i]; vtm[i] = tm[i]; }
}

/* nsteps calls of the reference's do_time_step (LSRK(5,4)) from sol_new = x,
 * sol_old = sol_tmp = 0, with the given time step */
template <int p>
static void time_steps(const int *nc, const double *h, int nsteps, double dt, double *x)
{
  EvaluationDGAdvection<3, p, double> ev;
  ev.blx = 2; ev.bly = 2; ev.blz = 2;
  unsigned int n_cells[3] = {(unsigned)nc[0], (unsigned)nc[1], (unsigned)nc[2]};
  ev.initialize(n_cells);
  set_geometry(ev, h);
  const std::size_t N = ev.n_elements() * ev.dofs_per_cell;
  for (std::size_t i = 0; i < N; ++i) { ev.sol_new[i] = x[i]; ev.sol_old[i] = 0.; ev.sol_tmp[i] = 0.; }
  ev.time_step = dt;
  double t = 0.;
  for (int s = 0; s < nsteps; ++s) ev.do_time_step(t);
  for (std::size_t i = 0; i < N; ++i) x[i] = ev.sol_new[i];
}

/* y = A x of the tensor-product SIPG Laplacian with precomputed 1D matrices
 * (unit Cartesian cells, periodic) */
template <int p>
static void precomputed(const int *nc, const double *x, double *y)
{
  PrecomputedDGLaplacian<3, p, double> ev;
  ev.blx = 2; ev.bly = 2; ev.blz = 2;
  unsigned int n_cells[3] = {(unsigned)nc[0], (unsigned)nc[1], (unsigned)nc[2]};
  ev.initialize(n_cells);
  const std::size_t N = ev.n_elements() * ev.dofs_per_cell;
  for (std::size_t i = 0; i < N; ++i) ev.input_array[i] = x[i];
  ev.matrix_vector_product();
  for (std::size_t i = 0; i < N; ++i) y[i] = ev.output_array[i];
}

template <int p>
static void face_tables(double *face_eo, double *Sinv_eo)
{
  EvaluationDGAdvection<3, p, double> ev;
  ev.blx = 2; ev.bly = 2; ev.blz = 2;
  unsigned int n_cells[3] = {1, 1, 1};
  ev.initialize(n_cells);
  const int n = p + 1, st = (n + 1) / 2;
  for (int i = 0; i < 2 * n; ++i) face_eo[i] = ev.shape_values_on_face_eo[i][0];
  for (int i = 0; i < n * st; ++i) Sinv_eo[i] = ev.inv_shape_values_eo[i][0];
}

#define SF_DISPATCH(fn, ...)                                                   \
  switch (degree) {                                                            \
  case 1: fn<1>(__VA_ARGS__); return 0;                                        \
  case 2: fn<2>(__VA_ARGS__); return 0;                                        \
  case 3: fn<3>(__VA_ARGS__); return 0;                                        \
  case 4: fn<4>(__VA_ARGS__); return 0;                                        \
  case 5: fn<5>(__VA_ARGS__); return 0;                                        \
  case 6: fn<6>(__VA_ARGS__); return 0;                                        \
  case 7: fn<7>(__VA_ARGS__); return 0;                                        \
  case 8: fn<8>(__VA_ARGS__); return 0;                                        \
  default: return -1;                                                          \
  }

extern "C" int sfref_dg_sipg(int degree, const int *nc, const double *h, int mode,
                             const double *x, const double *b, const double *dinv,
                             double *t, double c_np, double c_tm, double *y)
{ SF_DISPATCH(sipg, nc, h, mode, x, b, dinv, t, c_np, c_tm, y) }

extern "C" int sfref_dg_advect(int degree, const int *nc, const double *h,
                               const double *x, double *y)
{ SF_DISPATCH(advect, nc, h, x, y) }

extern "C" int sfref_dg_tables(int degree, double *face_eo, double *Sinv_eo)
{ SF_DISPATCH(face_tables, face_eo, Sinv_eo) }

extern "C" int sfref_dg_rk_stage(int degree, const int *nc, const double *h, const double *src,
                                 const double *upd, double c_np, double c_tm, double *vnp,
                                 double *vtm)
{ SF_DISPATCH(rk_stage, nc, h, src, upd, c_np, c_tm, vnp, vtm) }

extern "C" int sfref_dg_time_steps(int degree, const int *nc, const double *h, int nsteps,
                                   double dt, double *x)
{ SF_DISPATCH(time_steps, nc, h, nsteps, dt, x) }

extern "C" int sfref_dg_precomputed(int degree, const int *nc, const double *x, double *y)
{ SF_DISPATCH(precomputed, nc, x, y) }
