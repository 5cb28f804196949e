/*
 * Golden-vector adapter for the reference's 1D even-odd kernel
 * (legacy/include/matrix_vector_kernel.h:30-185) and its quadrature and
 * basis code (gauss_formula.h, lagrange_polynomials.h).
 * TEST INFRASTRUCTURE ONLY: compiled by oracle/build.py into oracle/_ref/.
 */
#include "ref_shim.h"
#include "gauss_formula.h"
#include "lagrange_polynomials.h"
#include "vectorization.h"
#include "utilities.h"
#include "matrix_vector_kernel.h"

typedef VectorizedArray<double> VA;

template <int nn, int type, bool cor, bool add, int do_dg>
static void run1(const double *coef, const double *in, double *out,
                 const double *dg, double *face)
{
  VA c[nn * nn], x[nn], y[nn], a[nn], d[2 * nn], f[4];
  for (int i = 0; i < nn * nn; ++i) c[i] = coef[i];
  for (int i = 0; i < nn; ++i) { x[i] = in[i]; a[i] = out[i]; }
  if (do_dg) {
    for (int i = 0; i < 2 * nn; ++i) d[i] = dg[i];
    for (int i = 0; i < 4; ++i) f[i] = face[i];
  }
  apply_1d_matvec_kernel<nn, 1, type, cor, add, VA, VA, false, do_dg>(
      c, x, y, add ? a : nullptr, do_dg ? d : nullptr, do_dg ? f : nullptr);
  for (int i = 0; i < nn; ++i) out[i] = y[i][0];
  if (do_dg && cor)
    for (int i = 0; i < 2 * do_dg; ++i) face[i] = f[i][0];
}

template <int nn>
static int dispatch_nn(int type, int cor, int add, int do_dg, const double *coef,
                       const double *in, double *out, const double *dg, double *face)
{
#define R(T, C, A, G) if (type == T && cor == C && add == A && do_dg == G) { run1<nn, T, C, A, G>(coef, in, out, dg, face); return 0; }
  R(0, 1, 0, 0) R(0, 0, 0, 0) R(0, 1, 1, 0) R(0, 0, 1, 0)
  R(1, 1, 0, 0) R(1, 0, 0, 0) R(1, 1, 1, 0) R(1, 0, 1, 0)
  R(1, 1, 0, 1) R(1, 0, 0, 1) R(1, 1, 0, 2) R(1, 0, 0, 2) R(1, 0, 1, 2)
  R(2, 1, 0, 0) R(2, 1, 1, 0)
#undef R
  return -1;
}

extern "C" int sfref_apply_1d(int nn, int type, int cor, int add, int do_dg,
                              const double *coef, const double *in, double *out,
                              const double *dg, double *face)
{
  switch (nn) {
  case 2: return dispatch_nn<2>(type, cor, add, do_dg, coef, in, out, dg, face);
  case 3: return dispatch_nn<3>(type, cor, add, do_dg, coef, in, out, dg, face);
  case 4: return dispatch_nn<4>(type, cor, add, do_dg, coef, in, out, dg, face);
  case 5: return dispatch_nn<5>(type, cor, add, do_dg, coef, in, out, dg, face);
  case 6: return dispatch_nn<6>(type, cor, add, do_dg, coef, in, out, dg, face);
  case 7: return dispatch_nn<7>(type, cor, add, do_dg, coef, in, out, dg, face);
  case 8: return dispatch_nn<8>(type, cor, add, do_dg, coef, in, out, dg, face);
  case 9: return dispatch_nn<9>(type, cor, add, do_dg, coef, in, out, dg, face);
  default: return -1;
  }
}

extern "C" void sfref_gauss(int n, double *points, double *weights)
{
  std::vector<double> p = get_gauss_points(n), w = get_gauss_weights(n);
  for (int i = 0; i < n; ++i) { points[i] = p[i]; weights[i] = w[i]; }
}

extern "C" void sfref_gll(int n, double *points)
{
  std::vector<double> p = get_gauss_lobatto_points(n);
  for (int i = 0; i < n; ++i) points[i] = p[i];
}

/* Hermite-like basis values/derivatives at given points */
extern "C" void sfref_hermite(int degree, int n_x, const double *x, double *val, double *der)
{
  HermiteLikePolynomialBasis b(degree);
  for (int i = 0; i <= degree; ++i)
    for (int k = 0; k < n_x; ++k) {
      val[i * n_x + k] = b.value(i, x[k]);
      der[i * n_x + k] = b.derivative(i, x[k]);
    }
}
