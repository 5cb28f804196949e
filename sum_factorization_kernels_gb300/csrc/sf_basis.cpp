// sf_basis.cpp -- 1D quadrature, bases and shape tables (host, FP64).
//
// The kernels need, per polynomial degree p (n = p+1):
//   S[q][i]  basis function i at Gauss point q (GLL-Lagrange or Hermite-like)
//   D[q][j]  derivative of the Gauss-point Lagrange polynomial j at Gauss
//            point q (collocation derivative)
//   Sinv     Gauss-Lagrange polynomials at the GLL points (change of basis
//            from Gauss-point values to GLL nodal values)
//   face values and derivatives of the Gauss-Lagrange polynomials at 0 and 1
// These are the quantities of the reference's fill_shape_values()
// (evaluation_cell_laplacian.h:815-886, benchmark_loops.cc:1387-1470,
// evaluation_dg_laplacian.h:615-695, evaluation_dg_advect.h:729-825), built
// from the same published constructions: Gauss-Legendre points by Newton's
// method on the Legendre three-term recurrence, Gauss-Lobatto points as the
// zeros of the Jacobi polynomial P^(1,1)_{n-2}, and the Hermite-like basis of
// Kronbichler & Kormann (doubled nodes at 0 and 1, interior nodes at the
// zeros of P^(2,2)_{p-3}, first node shifted so that the two functions
// living at x=0 are orthogonal).
#include "sf_internal.h"

#include <cmath>
#include <cfloat>
#include <cstring>

namespace sf {

namespace {

const double kPi = 3.14159265358979323846;

// Legendre P_n(z) and P_{n-1}(z) by the three-term recurrence
void legendre(int n, double z, double &pn, double &pn1)
{
  double p0 = 1.0, p1 = z;
  if (n == 0) { pn = 1.0; pn1 = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  pn = p1;
  pn1 = p0;
}

// Jacobi polynomial P^(al,be)_m(x) by its recurrence
double jacobi(int m, int al, int be, double x)
{
  if (m == 0) return 1.0;
  double pm1 = 1.0;
  double p = 0.5 * ((al + be + 2) * x + (al - be));
  for (int k = 1; k < m; ++k) {
    const double v = 2.0 * k + al + be;
    const double a1 = 2.0 * (k + 1) * (k + al + be + 1) * v;
    const double a2 = (v + 1) * (double(al) * al - double(be) * be);
    const double a3 = v * (v + 1) * (v + 2);
    const double a4 = 2.0 * (k + al) * (k + be) * (v + 2);
    const double pn = ((a2 + a3 * x) * p - a4 * pm1) / a1;
    pm1 = p;
    p = pn;
  }
  return p;
}

// zeros of P^(al,be)_m on (-1,1), ascending; Newton with deflation of the
// zeros found so far, started between the previous zero and a Chebyshev guess
void jacobi_zeros(int m, int al, int be, double *z)
{
  for (int k = 0; k < m; ++k) {
    double r = -std::cos((2.0 * k + 1.0) / (2.0 * m) * kPi);
    if (k > 0) r = 0.5 * (r + z[k - 1]);
    for (int it = 0; it < 200; ++it) {
      double s = 0.0;
      for (int i = 0; i < k; ++i) s += 1.0 / (r - z[i]);
      const double f = jacobi(m, al, be, r);
      const double df = 0.5 * (al + be + m + 1) * jacobi(m - 1, al + 1, be + 1, r);
      const double delta = f / (df - f * s);
      r -= delta;
      if (std::fabs(delta) < 5.0 * DBL_EPSILON) break;
    }
    z[k] = r;
  }
}

struct Lagrange {
  int n;
  double x[kMaxN], den[kMaxN];
  Lagrange(int n_, const double *pts) : n(n_)
  {
    for (int i = 0; i < n; ++i) x[i] = pts[i];
    for (int i = 0; i < n; ++i) {
      double d = 1.0;
      for (int j = 0; j < n; ++j)
        if (j != i) d *= x[i] - x[j];
      den[i] = 1.0 / d;
    }
  }
  double value(int i, double t) const
  {
    double v = den[i];
    for (int j = 0; j < n; ++j)
      if (j != i) v *= t - x[j];
    return v;
  }
  double deriv(int i, double t) const
  {
    // product rule accumulated alongside the value
    double v = den[i], d = 0.0;
    for (int j = 0; j < n; ++j)
      if (j != i) {
        d = d * (t - x[j]) + v;
        v *= t - x[j];
      }
    return d;
  }
};

// Hermite-like basis of degree p >= 3: nodes {0,0,z_1..z_{p-3},1,1}; the
// function attached to the first 0 node is built from the shifted factor
// (x - x*) instead of (x - 0), symmetric at the right end.
struct HermiteLike {
  int p;
  double nodes[kMaxN], den[kMaxN], xs;
  double raw(int i, double t, double *dv) const
  {
    const int n = p + 1;
    double v = 1.0, d = 0.0;
    auto mul = [&](double f) { d = d * f + v; v *= f; };
    if (p == 1) { if (dv) *dv = i == 0 ? -1.0 : 1.0; return i == 0 ? 1.0 - t : t; }
    if (p == 2) {
      if (i == 0) { if (dv) *dv = -2.0 * (1.0 - t); return (1.0 - t) * (1.0 - t); }
      if (i == 1) { if (dv) *dv = 2.0 - 4.0 * t; return 2.0 * t * (1.0 - t); }
      if (dv) *dv = 2.0 * t;
      return t * t;
    }
    if (i == 0) {
      mul(t - xs);
      for (int j = 2; j < n; ++j) mul(t - nodes[j]);
    } else if (i == p) {
      mul(t - 1.0 + xs);
      for (int j = 0; j < n - 2; ++j) mul(t - nodes[j]);
    } else {
      for (int j = 0; j < n; ++j)
        if (j != i) mul(t - nodes[j]);
    }
    if (dv) *dv = d;
    return v;
  }
  double value(int i, double t) const { return p <= 2 ? raw(i, t, nullptr) : den[i] * raw(i, t, nullptr); }
  double deriv(int i, double t) const
  {
    double d;
    raw(i, t, &d);
    return p <= 2 ? d : den[i] * d;
  }
  explicit HermiteLike(int p_) : p(p_), xs(0.0)
  {
    for (int i = 0; i < kMaxN; ++i) den[i] = 1.0;
    if (p < 3) return;
    double z[kMaxN];
    jacobi_zeros(p - 3, 2, 2, z);
    nodes[0] = nodes[1] = 0.0;
    for (int m = 0; m < p - 3; ++m) nodes[m + 2] = 0.5 * z[m] + 0.5;
    nodes[p - 1] = nodes[p] = 1.0;
    // x* from  int_0^1 x prod(x-z_j)^2 (x-1)^4 (x - x*) dx = 0, evaluated
    // exactly with p+1 Gauss points (integrand degree 2p)
    double gx[kMaxN + 1], gw[kMaxN + 1];
    gauss_points(p + 1, gx, gw);
    double num = 0.0, dnm = 0.0;
    for (int q = 0; q <= p; ++q) {
      const double t = gx[q];
      double c = t;
      for (int j = 0; j < p - 3; ++j) c *= (t - nodes[j + 2]) * (t - nodes[j + 2]);
      c *= (t - 1.0) * (t - 1.0) * (t - 1.0) * (t - 1.0);
      num += gw[q] * c * t;
      dnm += gw[q] * c;
    }
    xs = num / dnm;
    // normalisation: unit value at the own node for the interior functions
    // and for the two end functions; the second function at each end is
    // scaled so that its derivative cancels that of the end function
    for (int m = 2; m < p - 1; ++m) den[m] = 1.0 / raw(m, nodes[m], nullptr);
    den[0] = 1.0 / raw(0, 0.0, nullptr);
    den[p] = 1.0 / raw(p, 1.0, nullptr);
    double d0, d1;
    raw(0, 0.0, &d0);
    raw(1, 0.0, &d1);
    den[1] = -(den[0] * d0) / d1;
    raw(p, 1.0, &d0);
    raw(p - 1, 1.0, &d1);
    den[p - 1] = -(den[p] * d0) / d1;
  }
};

} // namespace

void gauss_points(int n, double *x, double *w)
{
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
    double pn = 0, pn1 = 0, dp = 1;
    for (int it = 0; it < 100; ++it) {
      legendre(n, z, pn, pn1);
      dp = n * (z * pn - pn1) / (z * z - 1.0);
      const double dz = pn / dp;
      z -= dz;
      if (std::fabs(dz) < 5.0 * DBL_EPSILON) break;
    }
    legendre(n, z, pn, pn1);
    dp = n * (z * pn - pn1) / (z * z - 1.0);
    // map [-1,1] -> [0,1]
    x[i] = 0.5 - 0.5 * z;
    x[n - 1 - i] = 0.5 + 0.5 * z;
    const double wi = 1.0 / ((1.0 - z * z) * dp * dp);
    w[i] = w[n - 1 - i] = wi;
  }
  if (n % 2 == 1) x[n / 2] = 0.5;
}

void gll_points(int n, double *x)
{
  double z[kMaxN];
  jacobi_zeros(n - 2, 1, 1, z);
  x[0] = 0.0;
  for (int i = 0; i < n - 2; ++i) x[i + 1] = 0.5 + 0.5 * z[i];
  x[n - 1] = 1.0;
  // exact symmetry about 1/2
  for (int i = 0; i < n / 2; ++i) {
    const double s = 0.5 * ((1.0 - x[n - 1 - i]) + x[i]);
    x[i] = s;
    x[n - 1 - i] = 1.0 - s;
  }
  if (n % 2 == 1) x[n / 2] = 0.5;
}

int fill_shape(int degree, int basis, Shape1D &s)
{
  if (degree < 1 || degree > kMaxDegree) return -1;
  std::memset(&s, 0, sizeof(s));
  const int n = degree + 1;
  s.degree = degree;
  s.n = n;
  s.basis = basis;
  gauss_points(n, s.xq, s.wq);
  gll_points(n, s.xgll);
  Lagrange gll(n, s.xgll), gauss(n, s.xq);
  HermiteLike herm(degree);
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i) {
      s.S[q][i] = basis == 0 ? gll.value(i, s.xq[q]) : herm.value(i, s.xq[q]);
      s.D[q][i] = gauss.deriv(i, s.xq[q]);
      s.Sinv[q][i] = gauss.value(i, s.xgll[q]);
    }
  for (int j = 0; j < n; ++j) {
    s.fv[0][j] = gauss.value(j, 0.0);
    s.fv[1][j] = gauss.value(j, 1.0);
    s.fd[0][j] = gauss.deriv(j, 0.0);
    s.fd[1][j] = gauss.deriv(j, 1.0);
  }
  s.hermite_d0 = herm.deriv(0, 0.0);
  return 0;
}

} // namespace sf
