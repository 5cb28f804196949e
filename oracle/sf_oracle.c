/*
 * sf_oracle.c -- FP64 CPU oracle (TEST INFRASTRUCTURE ONLY; see sf_oracle.h).
 *
 * Every function names the reference file:line range it restates.  Paths
 * are relative to the reference's legacy/ directory.
 *
 * Deviations from the reference, all deliberate and listed here:
 *  (1) periodic x-wrap index: evaluation_dg_laplacian.h:270 and
 *      evaluation_dg_advect.h:435 add dofs_per_cell where they must multiply;
 *      the oracle uses the corrected neighbour index.
 *  (2) evaluation_dg_laplacian.h:482 integrates the final x sweep with the
 *      forward shape matrix (contract_over_rows=true) instead of its
 *      transpose, which makes the SIPG operator non-symmetric; the oracle
 *      uses the transpose.
 *  (3) the transposed values kernel (type 0, contract_over_rows=false) of
 *      matrix_vector_kernel.h:130-131 drops the middle quadrature point for
 *      odd n; that term vanishes for the GLL basis and the Hermite-like
 *      basis of degree >= 3, but not for the Hermite-like basis of degree 2.
 *      The oracle keeps the term.
 *  (4) the Chebyshev step uses its right-hand-side argument, not the class
 *      member (evaluation_dg_laplacian.h:490-491).
 */
#include "sf_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double SFO_PI = 3.14159265358979323846;

/* ------------------------------------------------------------------------ */
/* quadrature: gauss_formula.h:35-94                                          */
/* ------------------------------------------------------------------------ */
static void gauss_newton(unsigned n_points, unsigned i, double *x, double *w)
{
  const double tol = DBL_EPSILON * 5.;
  double z = cos(SFO_PI * (i - .25) / (n_points + .5));
  double pp, p1;
  do {
    p1 = 1.;
    double p2 = 0.;
    for (unsigned j = 0; j < n_points; ++j) {
      const double p3 = p2;
      p2 = p1;
      p1 = ((2. * j + 1.) * z * p2 - j * p3) / (j + 1);
    }
    pp = n_points * (z * p1 - p2) / (z * z - 1);
    z = z - p1 / pp;
  } while (fabs(p1 / pp) > tol);
  *x = 0.5 * z;
  *w = 1. / ((1. - z * z) * pp * pp);
}

void sfo_gauss(int n, double *points, double *weights)
{
  double x, w;
  if (points)
    for (int i = 1; i <= n; ++i) {
      gauss_newton((unsigned)n, (unsigned)i, &x, &w);
      points[i - 1] = .5 - x;
      points[n - i] = .5 + x;
    }
  if (weights)
    for (int i = 1; i <= (n + 1) / 2; ++i) {
      gauss_newton((unsigned)n, (unsigned)i, &x, &w);
      weights[i - 1] = w;
      weights[n - i] = w;
    }
}

/* gauss_formula.h:97-123 */
static double jacobi_poly(double x, int alpha, int beta, unsigned n)
{
  double p[SFO_MAX_N + 4];
  p[0] = 1.0;
  if (n == 0) return p[0];
  p[1] = ((alpha + beta + 2) * x + (alpha - beta)) / 2;
  if (n == 1) return p[1];
  for (unsigned i = 1; i <= n - 1; ++i) {
    const int v = 2 * (int)i + alpha + beta;
    const int a1 = 2 * ((int)i + 1) * ((int)i + alpha + beta + 1) * v;
    const int a2 = (v + 1) * (alpha * alpha - beta * beta);
    const int a3 = v * (v + 1) * (v + 2);
    const int a4 = 2 * ((int)i + alpha) * ((int)i + beta) * (v + 2);
    p[i + 1] = ((a2 + a3 * x) * p[i] - a4 * p[i - 1]) / a1;
  }
  return p[n];
}

/* gauss_formula.h:125-163; returns m = degree - alpha - beta zeros in x */
static int jacobi_zeros(unsigned degree, int alpha, int beta, double *x)
{
  const double tol = DBL_EPSILON * 5.;
  const int m = (int)degree - alpha - beta;
  if (m <= 0) return 0;
  for (int i = 0; i < m; ++i)
    x[i] = -cos((double)(2 * i + 1) / (2 * m) * SFO_PI);
  for (int k = 0; k < m; ++k) {
    long double r = x[k];
    if (k > 0) r = (r + x[k - 1]) / 2;
    double delta;
    do {
      double s = 0.;
      for (int i = 0; i < k; ++i) s += 1. / (r - x[i]);
      const double J_x = 0.5 * (alpha + beta + m + 1) *
                         jacobi_poly((double)r, alpha + 1, beta + 1, (unsigned)m - 1);
      const double f = jacobi_poly((double)r, alpha, beta, (unsigned)m);
      delta = f / (f * s - J_x);
      r += delta;
    } while (fabs(delta) >= tol);
    x[k] = (double)r;
  }
  return m;
}

/* gauss_formula.h:165-175 */
void sfo_gll_points(int n, double *points)
{
  double z[SFO_MAX_N];
  const int m = jacobi_zeros((unsigned)n, 1, 1, z);
  points[0] = -1.;
  for (int i = 0; i < m; ++i) points[i + 1] = z[i];
  points[m + 1] = 1.;
  for (int i = 0; i < m + 2; ++i) points[i] = 0.5 + 0.5 * points[i];
}

/* ------------------------------------------------------------------------ */
/* bases: lagrange_polynomials.h:31-274                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
  int n;
  double pts[SFO_MAX_N];
  double den[SFO_MAX_N];
} lagr_t;

static void lagr_init(lagr_t *b, int n, const double *pts)
{
  b->n = n;
  for (int i = 0; i < n; ++i) b->pts[i] = pts[i];
  for (int i = 0; i < n; ++i) {
    double d = 1.;
    for (int j = 0; j < n; ++j)
      if (j != i) d *= pts[i] - pts[j];
    b->den[i] = 1. / d;
  }
}

static double lagr_value(const lagr_t *b, int idx, double x)
{
  double v = b->den[idx];
  for (int i = 0; i < b->n; ++i)
    if (i != idx) v *= x - b->pts[i];
  return v;
}

static double lagr_deriv(const lagr_t *b, int idx, double x)
{
  double v = b->den[idx], d = 0;
  for (int i = 0; i < b->n; ++i)
    if (i != idx) {
      const double t = x - b->pts[i];
      d = d * t + v;
      v *= t;
    }
  return d;
}

typedef struct {
  int n; /* degree + 1 */
  double pts[SFO_MAX_N];
  double den[SFO_MAX_N];
  double zero_one;
} herm_t;

static double herm_value(const herm_t *b, int idx, double x)
{
  const int n = b->n;
  if (n == 1) return 1.;
  if (n == 2) return idx == 0 ? 1. - x : x;
  if (n == 3) {
    if (idx == 0) return (1. - x) * (1. - x);
    if (idx == 1) return 2. * x * (1. - x);
    return x * x;
  }
  double v = b->den[idx];
  if (idx == 0) {
    v *= (x - b->zero_one);
    for (int i = 2; i < n; ++i) v *= x - b->pts[i];
  } else if (idx == n - 1) {
    v *= (x - 1. + b->zero_one);
    for (int i = 0; i < n - 2; ++i) v *= x - b->pts[i];
  } else {
    for (int i = 0; i < n; ++i)
      if (i != idx) v *= x - b->pts[i];
  }
  return v;
}

static double herm_deriv(const herm_t *b, int idx, double x)
{
  const int n = b->n;
  if (n == 1) return 0;
  if (n == 2) return idx == 0 ? -1. : 1.;
  if (n == 3) {
    if (idx == 0) return -2. * (1. - x);
    if (idx == 1) return 2. - 4. * x;
    return 2. * x;
  }
  double v = b->den[idx], d = 0;
  if (idx == 0) {
    d = v;
    v *= (x - b->zero_one);
    for (int i = 2; i < n; ++i) {
      const double t = x - b->pts[i];
      d = d * t + v;
      v *= t;
    }
  } else if (idx == n - 1) {
    d = v;
    v *= (x - 1. + b->zero_one);
    for (int i = 0; i < n - 2; ++i) {
      const double t = x - b->pts[i];
      d = d * t + v;
      v *= t;
    }
  } else {
    for (int i = 0; i < n; ++i)
      if (i != idx) {
        const double t = x - b->pts[i];
        d = d * t + v;
        v *= t;
      }
  }
  return d;
}

/* lagrange_polynomials.h:89-123 */
static double herm_support_point(const double *roots, int n_roots)
{
  const double gl = 0, gr = 0.5;
  const int degree = n_roots + 3;
  double pts[SFO_MAX_N + 1], w[SFO_MAX_N + 1];
  sfo_gauss(degree + 1, pts, w);
  double il = 0, ir = 0;
  for (int q = 0; q < degree + 1; ++q) {
    const double x = pts[q];
    double c = x;
    for (int j = 0; j < degree - 3; ++j) c *= (x - roots[j]) * (x - roots[j]);
    c *= (x - 1.) * (x - 1.) * (x - 1.) * (x - 1.);
    il += w[q] * (c * (x - gl));
    ir += w[q] * (c * (x - gr));
  }
  return gr - (gr - gl) / (ir - il) * ir;
}

/* lagrange_polynomials.h:126-156 */
static void herm_init(herm_t *b, int degree)
{
  memset(b, 0, sizeof(*b));
  b->n = degree + 1;
  if (degree >= 3) {
    double roots[SFO_MAX_N + 1];
    jacobi_zeros((unsigned)degree + 1, 2, 2, roots);
    for (int i = 0; i < degree - 3; ++i) roots[i] = 0.5 * roots[i] + 0.5;
    b->pts[0] = 0.;
    b->pts[1] = 0.;
    for (int m = 0; m < degree - 3; ++m) b->pts[m + 2] = roots[m];
    b->pts[degree - 1] = 1.;
    b->pts[degree] = 1.;
    b->zero_one = herm_support_point(roots, degree - 3);
    for (int i = 0; i <= degree; ++i) b->den[i] = 1.;
    for (int m = 2; m < degree - 1; ++m) b->den[m] = 1. / herm_value(b, m, b->pts[m]);
    b->den[0] = 1. / herm_value(b, 0, 0.);
    b->den[degree] = 1. / herm_value(b, degree, 1.);
    b->den[1] = -herm_deriv(b, 0, 0.) / herm_deriv(b, 1, 0.);
    b->den[degree - 1] = -(herm_deriv(b, degree, 1.) / herm_deriv(b, degree - 1, 1.));
  }
}

/* ------------------------------------------------------------------------ */
/* shape tables                                                               */
/*   values/gradients eo: evaluation_cell_laplacian.h:815-853 (Hermite),     */
/*   benchmark_loops.cc:1387-1440 (GLL); face eo: evaluation_dg_laplacian.h: */
/*   659-670; inverse eo: evaluation_dg_advect.h:791-803                     */
/* ------------------------------------------------------------------------ */
typedef double (*basis_fn)(const void *, int, double);
static double gll_val(const void *b, int i, double x) { return lagr_value((const lagr_t *)b, i, x); }
static double herm_val(const void *b, int i, double x) { return herm_value((const herm_t *)b, i, x); }

static void fill_eo(int degree, const double *xq, const void *basis, basis_fn f,
                    double *eo)
{
  const int n = degree + 1, stride = (n + 1) / 2;
  for (int i = 0; i < (degree + 1) / 2; ++i)
    for (int q = 0; q < stride; ++q) {
      const double p1 = f(basis, i, xq[q]);
      const double p2 = f(basis, i, xq[n - 1 - q]);
      eo[i * stride + q] = 0.5 * (p1 + p2);
      eo[(degree - i) * stride + q] = 0.5 * (p1 - p2);
    }
  if (degree % 2 == 0)
    for (int q = 0; q < stride; ++q)
      eo[degree / 2 * stride + q] = f(basis, degree / 2, xq[q]);
}

static double lagr_der_fn(const void *b, int i, double x) { return lagr_deriv((const lagr_t *)b, i, x); }

int sfo_shape_init(int degree, int basis, sfo_shape *s)
{
  if (degree < 1 || degree + 1 > SFO_MAX_N) return -1;
  memset(s, 0, sizeof(*s));
  const int n = degree + 1;
  s->degree = degree;
  s->n = n;
  s->basis = basis;
  sfo_gauss(n, s->xq, s->wq);
  sfo_gll_points(n, s->xgll);

  lagr_t gll, gauss;
  lagr_init(&gll, n, s->xgll);
  lagr_init(&gauss, n, s->xq);
  herm_t herm;
  herm_init(&herm, degree);

  const void *b = basis == SFO_BASIS_GLL ? (const void *)&gll : (const void *)&herm;
  basis_fn f = basis == SFO_BASIS_GLL ? gll_val : herm_val;
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i) {
      s->S[q * n + i] = f(b, i, s->xq[q]);
      s->D[q * n + i] = lagr_deriv(&gauss, i, s->xq[q]);
      s->Sinv[q * n + i] = lagr_value(&gauss, i, s->xgll[q]);
    }
  for (int j = 0; j < n; ++j) {
    s->face_v[0][j] = lagr_value(&gauss, j, 0.);
    s->face_v[1][j] = lagr_value(&gauss, j, 1.);
    s->face_d[0][j] = lagr_deriv(&gauss, j, 0.);
    s->face_d[1][j] = lagr_deriv(&gauss, j, 1.);
  }
  s->hermite_d0 = herm_deriv(&herm, 0, 0.);

  fill_eo(degree, s->xq, b, f, s->S_eo);
  fill_eo(degree, s->xq, &gauss, lagr_der_fn, s->D_eo);
  /* inverse: rows are Gauss-Lagrange functions evaluated at GLL points */
  {
    const int stride = (n + 1) / 2;
    for (int i = 0; i < (degree + 1) / 2; ++i)
      for (int q = 0; q < stride; ++q) {
        s->Sinv_eo[i * stride + q] = 0.5 * (lagr_value(&gauss, i, s->xgll[q]) +
                                            lagr_value(&gauss, i, s->xgll[degree - q]));
        s->Sinv_eo[(degree - i) * stride + q] =
            0.5 * (lagr_value(&gauss, i, s->xgll[q]) - lagr_value(&gauss, i, s->xgll[degree - q]));
      }
    if (degree % 2 == 0)
      for (int q = 0; q < stride; ++q)
        s->Sinv_eo[degree / 2 * stride + q] = lagr_value(&gauss, degree / 2, s->xgll[q]);
  }
  for (int i = 0; i < degree / 2 + 1; ++i) {
    const double v0 = lagr_value(&gauss, i, 0), v1 = lagr_value(&gauss, i, 1);
    s->face_eo[degree - i] = 0.5 * (v0 - v1);
    s->face_eo[i] = 0.5 * (v0 + v1);
    const double d0 = lagr_deriv(&gauss, i, 0), d1 = lagr_deriv(&gauss, i, 1);
    s->face_eo[n + i] = 0.5 * (d0 + d1);
    s->face_eo[n + degree - i] = 0.5 * (d0 - d1);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* 1D even-odd contraction: matrix_vector_kernel.h:30-185                    */
/* ------------------------------------------------------------------------ */
#define SFO_INLINE static inline __attribute__((always_inline))

SFO_INLINE void apply_1d_impl(int nn, int stride, int type, int cor, int add_into,
                              const double *c, const double *in, double *out,
                              const double *add, int do_dg, const double *dg, double *face)
{
  const int mid = nn / 2, offset = (nn + 1) / 2;
  double xp[SFO_MAX_N], xm[SFO_MAX_N];
  for (int i = 0; i < mid; ++i) {
    if (cor && type == 1) {
      xp[i] = in[stride * i] - in[stride * (nn - 1 - i)];
      xm[i] = in[stride * i] + in[stride * (nn - 1 - i)];
    } else {
      xp[i] = in[i * stride] + in[(nn - 1 - i) * stride];
      xm[i] = in[i * stride] - in[(nn - 1 - i) * stride];
    }
  }
  const double xmid = in[stride * mid];
  if (cor) {
    for (int col = 0; col < mid; ++col) {
      double r0 = c[col] * xp[0];
      double r1 = c[(nn - 1) * offset + col] * xm[0];
      for (int ind = 1; ind < mid; ++ind) {
        r0 += c[ind * offset + col] * xp[ind];
        r1 += c[(nn - 1 - ind) * offset + col] * xm[ind];
      }
      if (nn % 2 == 1) {
        if (type == 1) r1 += c[mid * offset + col] * xmid;
        else r0 += c[mid * offset + col] * xmid;
      }
      const double t = r0;
      const double o0 = (add_into ? add[col * stride] + t : t) + r1;
      const double o1 = (add_into ? add[(nn - 1 - col) * stride] + t : t) - r1;
      out[col * stride] = o0;
      out[(nn - 1 - col) * stride] = o1;
    }
    if (nn % 2 == 1) {
      double r0 = add_into ? add[mid] + c[mid * offset + mid] * xmid
                           : c[mid * offset + mid] * xmid;
      for (int ind = 0; ind < mid; ++ind) r0 += c[ind * offset + mid] * xp[ind];
      out[mid * stride] = r0;
    }
    if (do_dg > 0) {
      double r0 = dg[0] * xm[0], r1 = dg[nn - 1] * xp[0];
      for (int ind = 1; ind < mid; ++ind) {
        r0 += dg[ind] * xm[ind];
        r1 += dg[nn - 1 - ind] * xp[ind];
      }
      if (nn % 2 == 1) r0 += dg[mid] * xmid;
      face[0] = r0 + r1;
      face[1] = r0 - r1;
    }
    if (do_dg > 1) {
      double r0 = dg[nn] * xp[0], r1 = dg[nn + nn - 1] * xm[0];
      for (int ind = 1; ind < mid; ++ind) {
        r0 += dg[nn + ind] * xp[ind];
        r1 += dg[nn + nn - 1 - ind] * xm[ind];
      }
      if (nn % 2 == 1) r1 += dg[nn + mid] * xmid;
      face[2] = r0 + r1;
      face[3] = r0 - r1;
    }
  } else {
    for (int col = 0; col < mid; ++col) {
      double r0 = c[col * offset] * xp[0];
      double r1 = c[(nn - 1 - col) * offset] * xm[0];
      for (int ind = 1; ind < mid; ++ind) {
        r0 += c[col * offset + ind] * xp[ind];
        r1 += c[(nn - 1 - col) * offset + ind] * xm[ind];
      }
      /* deviation (3): the middle point is kept for type 0 as well */
      if (nn % 2 == 1) r0 += c[col * offset + mid] * xmid;
      if (do_dg > 0) {
        r1 += dg[col] * face[0];
        r0 += dg[nn - 1 - col] * face[1];
      }
      if (do_dg > 1) {
        r0 += dg[nn + col] * face[2];
        r1 += dg[nn + nn - 1 - col] * face[3];
      }
      const double t = r0;
      const double o0 = (add_into ? add[col * stride] + t : t) + r1;
      double o1;
      if (type != 1) o1 = (add_into ? add[(nn - 1 - col) * stride] + t : t) - r1;
      else o1 = (add_into ? add[(nn - 1 - col) * stride] + r1 : r1) - t;
      out[col * stride] = o0;
      out[(nn - 1 - col) * stride] = o1;
    }
    if (nn % 2 == 1) {
      double r0 = add_into ? add[mid * stride] + c[mid * offset + mid] * xmid
                           : c[mid * offset + mid] * xmid;
      if (type == 1 && add_into) r0 = add[mid * stride];
      else if (type == 1) r0 = 0.;
      if (type == 1)
        for (int ind = 0; ind < mid; ++ind) r0 += c[mid * offset + ind] * xm[ind];
      else
        for (int ind = 0; ind < mid; ++ind) r0 += c[mid * offset + ind] * xp[ind];
      if (do_dg > 0) r0 += dg[mid] * face[0];
      if (do_dg > 1) r0 += dg[nn + mid] * face[3];
      out[mid * stride] = r0;
    }
  }
}

void sfo_apply_1d(int nn, int stride, int type, int cor, int add_into,
                  const double *c, const double *in, double *out,
                  const double *add, int do_dg, const double *dg, double *face)
{
  apply_1d_impl(nn, stride, type, cor, add_into, c, in, out, add, do_dg, dg, face);
}

/* test_multiplication.cc:18-60 style plain contraction (no even-odd) */
void sfo_apply_1d_plain(int n, int stride, const double *M, int transpose,
                        const double *in, double *out)
{
  double tmp[SFO_MAX_N];
  for (int i = 0; i < n; ++i) {
    double s = 0;
    for (int j = 0; j < n; ++j)
      s += (transpose ? M[j * n + i] : M[i * n + j]) * in[j * stride];
    tmp[i] = s;
  }
  for (int i = 0; i < n; ++i) out[i * stride] = tmp[i];
}

/* one tensor direction over all n^2 lines of a cell-local array */
SFO_INLINE void sweep(int n, int dir, int type, int cor, int add, const double *eo,
                      const double *in, double *out)
{
  const int stride = dir == 0 ? 1 : (dir == 1 ? n : n * n);
  for (int i2 = 0; i2 < n; ++i2)
    for (int i1 = 0; i1 < n; ++i1) {
      const int base = dir == 0 ? (i1 * n + i2 * n * n)
                                : (dir == 1 ? (i1 + i2 * n * n) : (i1 + i2 * n));
      apply_1d_impl(n, stride, type, cor, add, eo, in + base, out + base,
                    add ? out + base : NULL, 0, NULL, NULL);
    }
}

/* ------------------------------------------------------------------------ */
/* cell Laplacian: sweep order of benchmark_loops.cc:1316-1384, merged      */
/* quadrature-point tensor of evaluation_cell_laplacian.h:392-415 generalised */
/* to one 6-entry tensor per quadrature point (including JxW and kappa)      */
/* ------------------------------------------------------------------------ */
#define SFO_MAX_NQ (SFO_MAX_N * SFO_MAX_N * SFO_MAX_N)

SFO_INLINE void cell_grad_n(int n, const sfo_shape *s, const double *in, double *uq,
                            double *gx, double *gy, double *gz)
{
  const int nq = n * n * n;
  double t[SFO_MAX_NQ];
  sweep(n, 0, 0, 1, 0, s->S_eo, in, t);
  sweep(n, 1, 0, 1, 0, s->S_eo, t, uq);
  sweep(n, 2, 0, 1, 0, s->S_eo, uq, t);
  memcpy(uq, t, sizeof(double) * nq);
  sweep(n, 2, 1, 1, 0, s->D_eo, uq, gz);
  sweep(n, 1, 1, 1, 0, s->D_eo, uq, gy);
  sweep(n, 0, 1, 1, 0, s->D_eo, uq, gx);
}

static void cell_grad(const sfo_shape *s, const double *in, double *uq,
                      double *gx, double *gy, double *gz)
{
  cell_grad_n(s->n, s, in, uq, gx, gy, gz);
}

SFO_INLINE void cell_integrate_n(int n, const sfo_shape *s, const double *tx, const double *ty,
                                 const double *tz, double *out)
{
  double a[SFO_MAX_NQ], b[SFO_MAX_NQ];
  sweep(n, 0, 1, 0, 0, s->D_eo, tx, a);
  sweep(n, 1, 1, 0, 1, s->D_eo, ty, a);
  sweep(n, 2, 1, 0, 1, s->D_eo, tz, a);
  sweep(n, 2, 0, 0, 0, s->S_eo, a, b);
  sweep(n, 1, 0, 0, 0, s->S_eo, b, a);
  sweep(n, 0, 0, 0, 0, s->S_eo, a, out);
}

/* geometry pointer Gcell has 6 blocks of geo_stride entries, quadrature
 * weight included; geo_stride 0: G holds the 6 entries of one constant
 * tensor for the whole cell and the weight w_q is applied here, the
 * reference's Cartesian form (evaluation_cell_laplacian.h:368-371,:395-411) */
SFO_INLINE void cell_apply_n(int n, const sfo_shape *s, const double *G, int gs,
                             const double *kappa, const double *in, double *out)
{
  const int nq = n * n * n;
  double buf[4 * SFO_MAX_NQ];
  double *uq = buf, *gx = buf + nq, *gy = buf + 2 * nq, *gz = buf + 3 * nq;
  cell_grad_n(n, s, in, uq, gx, gy, gz);
  for (int q = 0; q < nq; ++q) {
    const int o = gs ? q : 0;
    const double *g = G + o;
    const int S6 = gs ? gs : 1;
    const double wq = gs ? 1. : s->wq[q / (n * n)] * s->wq[(q / n) % n] * s->wq[q % n];
    const double k = kappa ? kappa[q] : 1.;
    const double t0 = gx[q] * g[0] + gy[q] * g[3 * S6] + gz[q] * g[4 * S6];
    const double t1 = gx[q] * g[3 * S6] + gy[q] * g[1 * S6] + gz[q] * g[5 * S6];
    const double t2 = gx[q] * g[4 * S6] + gy[q] * g[5 * S6] + gz[q] * g[2 * S6];
    gx[q] = t0 * wq * k;
    gy[q] = t1 * wq * k;
    gz[q] = t2 * wq * k;
  }
  cell_integrate_n(n, s, gx, gy, gz, out);
}

/* one specialised copy of the cell operator per degree */
static void cell_apply_k(const sfo_shape *s, const double *G, int gs,
                         const double *kappa, const double *in, double *out)
{
  switch (s->n) {
  case 2: cell_apply_n(2, s, G, gs, kappa, in, out); break;
  case 3: cell_apply_n(3, s, G, gs, kappa, in, out); break;
  case 4: cell_apply_n(4, s, G, gs, kappa, in, out); break;
  case 5: cell_apply_n(5, s, G, gs, kappa, in, out); break;
  case 6: cell_apply_n(6, s, G, gs, kappa, in, out); break;
  case 7: cell_apply_n(7, s, G, gs, kappa, in, out); break;
  case 8: cell_apply_n(8, s, G, gs, kappa, in, out); break;
  case 9: cell_apply_n(9, s, G, gs, kappa, in, out); break;
  default: cell_apply_n(s->n, s, G, gs, kappa, in, out); break;
  }
}

void sfo_cell_apply(const sfo_shape *s, const double *Gcell, int geo_stride,
                    const double *in, double *out)
{
  cell_apply_k(s, Gcell, geo_stride, NULL, in, out);
}

/* mass matrix and convection form of one Cartesian cell
 * (evaluation_cell_laplacian.h:299-326 and :328-354): u_q = S x at the Gauss
 * points, r_q = u_q JxW w_q; mass: S^T r; convection: t_d = ij_d b_d r,
 * integrated with D^T and S^T as the Laplacian's second half */
SFO_INLINE void cell_op_n(int n, const sfo_shape *s, int kind, const double *ij, double jxw,
                          const double *b, const double *in, double *out)
{
  double t[SFO_MAX_NQ], uq[SFO_MAX_NQ];
  sweep(n, 0, 0, 1, 0, s->S_eo, in, t);
  sweep(n, 1, 0, 1, 0, s->S_eo, t, uq);
  sweep(n, 2, 0, 1, 0, s->S_eo, uq, t);
  for (int qz = 0; qz < n; ++qz)
    for (int qy = 0; qy < n; ++qy)
      for (int qx = 0; qx < n; ++qx) {
        const int q = (qz * n + qy) * n + qx;
        t[q] *= jxw * ((s->wq[qz] * s->wq[qy]) * s->wq[qx]);
      }
  if (kind == 1) {
    sweep(n, 2, 0, 0, 0, s->S_eo, t, uq);
    sweep(n, 1, 0, 0, 0, s->S_eo, uq, t);
    sweep(n, 0, 0, 0, 0, s->S_eo, t, out);
    return;
  }
  double tx[SFO_MAX_NQ], ty[SFO_MAX_NQ], tz[SFO_MAX_NQ];
  for (int q = 0; q < n * n * n; ++q) {
    tx[q] = t[q] * (ij[0] * b[0]);
    ty[q] = t[q] * (ij[1] * b[1]);
    tz[q] = t[q] * (ij[2] * b[2]);
  }
  cell_integrate_n(n, s, tx, ty, tz, out);
}

void sfo_cell_op(const sfo_shape *s, int kind, const double *ij, double jxw,
                 const double *b, const double *in, double *out)
{
  cell_op_n(s->n, s, kind, ij, jxw, b, in, out);
}

/* face values of one cell layer: F[i2 n + i1] <- S (along i1) then S (along
 * i2) of the node layer, or the transposes (back to the nodes) */
static void face_interp2(int n, const double *S, int transpose, const double *in, double *out)
{
  double t[SFO_MAX_N * SFO_MAX_N];
  for (int i2 = 0; i2 < n; ++i2)
    for (int a = 0; a < n; ++a) {
      double v = 0.;
      for (int i1 = 0; i1 < n; ++i1) v += (transpose ? S[i1 * n + a] : S[a * n + i1]) * in[i2 * n + i1];
      t[i2 * n + a] = v;
    }
  for (int bq = 0; bq < n; ++bq)
    for (int a = 0; a < n; ++a) {
      double v = 0.;
      for (int i2 = 0; i2 < n; ++i2) v += (transpose ? S[i2 * n + bq] : S[bq * n + i2]) * t[i2 * n + a];
      out[bq * n + a] = v;
    }
}

/* The face terms of the DO_FACES build of the cell Laplacian
 * (evaluation_cell_laplacian.h:505-797, set-up :84-100): per direction f the
 * cell's own faces at 1 ("right", node layer p) and at 0 ("left", layer 0)
 * act as the two sides of one face, with no neighbour.  Face-local
 * coordinates (i1, i2) run along directions f+1 and f+2 (mod 3).  The values
 * and the Hermite-like normal derivatives hd (u_{p-1} - u_p), hd (u_1 - u_0)
 * (hd = phi_0'(0)) are interpolated to the face Gauss points; with
 * W = -w_q1 w_q2 / prod_{e != f} ij_e:
 *  Laplacian (:688-708): a = (uR + uL) / 2, g = ij_f (nR + nL),
 *    v = W (2 sigma a - g / 2), sigma = (p+1)^2 ij_f; the right face tests
 *    with -v, the left with +v, and both normal-derivative slots with
 *    d = W ij_f a, mapped back with the forward S (:756-759, as the
 *    reference) and injected through the two end layers (:760-766);
 *  convection (:558-567): flux = ((uR + uL) b_f + |b_f| (uR - uL)) / 2, the
 *    right face tests with W flux, the left with -W flux.
 * The reference also adds tangential-gradient terms with a zero normal
 * Jacobian (normal_jac[f][0..1] = 0, :88-93): they are zero and left out. */
static void cell_faces_term(const sfo_shape *s, int conv, const double *ij, const double *b,
                            const double *in, double *out)
{
  const int n = s->n, p = n - 1;
  const int str[3] = {1, n, n * n};
  const double hd = s->hermite_d0;
  for (int f = 0; f < 3; ++f) {
    const int o1 = str[f], s1 = str[(f + 1) % 3], s2 = str[(f + 2) % 3];
    double fjxw = 1.;
    for (int e = 0; e < 3; ++e)
      if (e != f) fjxw /= ij[e];
    double uR[SFO_MAX_N * SFO_MAX_N], uL[SFO_MAX_N * SFO_MAX_N], dR[SFO_MAX_N * SFO_MAX_N],
        dL[SFO_MAX_N * SFO_MAX_N];
    for (int i2 = 0; i2 < n; ++i2)
      for (int i1 = 0; i1 < n; ++i1) {
        const int k = i2 * n + i1, base = i2 * s2 + i1 * s1;
        uR[k] = in[p * o1 + base];
        uL[k] = in[base];
        dR[k] = hd * (in[(p - 1) * o1 + base] - uR[k]);
        dL[k] = hd * (in[o1 + base] - uL[k]);
      }
    face_interp2(n, s->S, 0, uR, uR);
    face_interp2(n, s->S, 0, uL, uL);
    face_interp2(n, s->S, 0, dR, dR);
    face_interp2(n, s->S, 0, dL, dL);
    double cR[SFO_MAX_N * SFO_MAX_N], cL[SFO_MAX_N * SFO_MAX_N], dv[SFO_MAX_N * SFO_MAX_N];
    for (int q2 = 0; q2 < n; ++q2)
      for (int q1 = 0; q1 < n; ++q1) {
        const int q = q2 * n + q1;
        const double W = -(s->wq[q2] * s->wq[q1]) * fjxw;
        if (conv) {
          const double flux = 0.5 * (b[f] * (uR[q] + uL[q]) + fabs(b[f]) * (uR[q] - uL[q]));
          cR[q] = flux * W;
          cL[q] = -(flux * W);
          dv[q] = 0.;
        } else {
          const double sigma = (double)(n * n) * ij[f];
          const double a = 0.5 * (uR[q] + uL[q]);
          const double g = ij[f] * dR[q] + ij[f] * dL[q];
          const double v = W * (a * 2. * sigma - g * 0.5);
          cR[q] = -v;
          cL[q] = v;
          dv[q] = W * ij[f] * a;
        }
      }
    face_interp2(n, s->S, 1, cR, cR);
    face_interp2(n, s->S, 1, cL, cL);
    if (!conv) face_interp2(n, s->S, 0, dv, dv);
    for (int i2 = 0; i2 < n; ++i2)
      for (int i1 = 0; i1 < n; ++i1) {
        const int k = i2 * n + i1, base = i2 * s2 + i1 * s1;
        if (conv) {
          out[p * o1 + base] += cR[k];
        } else {
          out[p * o1 + base] += cR[k] - dv[k] * hd;
          out[(p - 1) * o1 + base] += hd * dv[k];
        }
      }
    for (int i2 = 0; i2 < n; ++i2)
      for (int i1 = 0; i1 < n; ++i1) {
        const int k = i2 * n + i1, base = i2 * s2 + i1 * s1;
        if (conv) {
          out[base] += cL[k];
        } else {
          out[base] += cL[k] - dv[k] * hd;
          out[o1 + base] += hd * dv[k];
        }
      }
  }
}

void sfo_cell_faces(const sfo_shape *s, int conv, const double *ij, double jxw, const double *b,
                    const double *in, double *out)
{
  if (conv) {
    cell_op_n(s->n, s, 2, ij, jxw, b, in, out);
  } else {
    const double G[6] = {jxw * ij[0] * ij[0], jxw * ij[1] * ij[1], jxw * ij[2] * ij[2], 0., 0., 0.};
    cell_apply_k(s, G, 0, NULL, in, out);
  }
  cell_faces_term(s, conv, ij, b, in, out);
}

void sfo_cell_faces_apply(int degree, int conv, long long n_cells, const double *h, const double *b,
                          const double *x, double *y)
{
  sfo_shape s;
  sfo_shape_init(degree, SFO_BASIS_HERMITE, &s);
  const long long nq = (long long)s.n * s.n * s.n;
  const double ij[3] = {1. / h[0], 1. / h[1], 1. / h[2]};
  const double jxw = h[0] * h[1] * h[2];
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < n_cells; ++e) sfo_cell_faces(&s, conv, ij, jxw, b, x + e * nq, y + e * nq);
}

/* ------------------------------------------------------------------------ */
/* continuous numbering (no counterpart in the reference; the cell-local     */
/* order restricts to the reference's lexicographic cell order,              */
/* evaluation_cell_laplacian.h:157-160)                                      */
/* ------------------------------------------------------------------------ */
long long sfo_cont_n_dofs(const sfo_mesh *m)
{
  const long long p = m->degree;
  return (p * m->n_cells[0] + 1) * (p * m->n_cells[1] + 1) * (p * m->n_cells[2] + 1);
}

static inline long long cont_index(const sfo_mesh *m, int i, int j, int k, int a,
                                   int b, int c, int *on_boundary)
{
  const int p = m->degree;
  const long long Nx = (long long)p * m->n_cells[0] + 1;
  const long long Ny = (long long)p * m->n_cells[1] + 1;
  const long long Nz = (long long)p * m->n_cells[2] + 1;
  const long long X = (long long)i * p + a, Y = (long long)j * p + b,
                  Z = (long long)k * p + c;
  *on_boundary = m->dirichlet && (X == 0 || Y == 0 || Z == 0 || X == Nx - 1 ||
                                  Y == Ny - 1 || Z == Nz - 1);
  return (Z * Ny + Y) * Nx + X;
}

/* analytic deformed mapping x_i <- x_i + a sin(2 pi x_j) sin(2 pi x_k),
 * (i,j,k) cyclic; J = d x / d xi (xi the unit-cell coordinate) */
static void mapping_jacobian(const sfo_mesh *m, const double X[3], const double h[3],
                             double J[3][3])
{
  const double a = m->deform, tp = 2. * SFO_PI;
  const double s0 = sin(tp * X[0]), s1 = sin(tp * X[1]), s2 = sin(tp * X[2]);
  const double c0 = cos(tp * X[0]), c1 = cos(tp * X[1]), c2 = cos(tp * X[2]);
  J[0][0] = h[0];
  J[0][1] = h[1] * a * tp * c1 * s2;
  J[0][2] = h[2] * a * tp * s1 * c2;
  J[1][0] = h[0] * a * tp * s2 * c0;
  J[1][1] = h[1];
  J[1][2] = h[2] * a * tp * c2 * s0;
  J[2][0] = h[0] * a * tp * c0 * s1;
  J[2][1] = h[1] * a * tp * s0 * c1;
  J[2][2] = h[2];
}

/* merged tensor JxW J^-1 J^-T (times the Gauss weights) of cell (i, j, k) at
 * its n^3 Gauss points: g[e n^3 + q], e = xx, yy, zz, xy, xz, yz */
static void cont_cell_geometry(const sfo_mesh *m, const sfo_shape *s, int i, int j, int k,
                               const double h[3], double *g)
{
  const int n = s->n, nq = n * n * n;
  for (int qz = 0; qz < n; ++qz)
    for (int qy = 0; qy < n; ++qy)
      for (int qx = 0; qx < n; ++qx) {
        const int q = (qz * n + qy) * n + qx;
        const double X[3] = {(i + s->xq[qx]) * h[0], (j + s->xq[qy]) * h[1],
                             (k + s->xq[qz]) * h[2]};
        double J[3][3];
        mapping_jacobian(m, X, h, J);
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        double Ji[3][3];
        Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        const double jxw = det * ((s->wq[qz] * s->wq[qy]) * s->wq[qx]);
        static const int pr[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
        for (int e = 0; e < 6; ++e) {
          const int d0 = pr[e][0], d1 = pr[e][1];
          const double v = Ji[d0][0] * Ji[d1][0] + Ji[d0][1] * Ji[d1][1] +
                           Ji[d0][2] * Ji[d1][2];
          g[e * nq + q] = jxw * v;
        }
      }
}

void sfo_cont_geometry(const sfo_mesh *m, double *G)
{
  sfo_shape s;
  sfo_shape_init(m->degree, m->basis, &s);
  const int nq = s.n * s.n * s.n;
  const long long C = (long long)m->n_cells[0] * m->n_cells[1] * m->n_cells[2];
  double h[3];
  for (int d = 0; d < 3; ++d) h[d] = m->length[d] / m->n_cells[d];
#pragma omp parallel for schedule(static)
  for (long long cell = 0; cell < C; ++cell) {
    const int i = (int)(cell % m->n_cells[0]);
    const int j = (int)((cell / m->n_cells[0]) % m->n_cells[1]);
    const int k = (int)(cell / ((long long)m->n_cells[0] * m->n_cells[1]));
    cont_cell_geometry(m, &s, i, j, k, h, G + cell * 6 * nq);
  }
}

static void cont_gather(const sfo_mesh *m, int i, int j, int k, const double *x,
                        double *u)
{
  const int n = m->degree + 1;
  for (int c = 0; c < n; ++c)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        int bd;
        const long long g = cont_index(m, i, j, k, a, b, c, &bd);
        u[(c * n + b) * n + a] = bd ? 0. : x[g];
      }
}

void sfo_cont_apply(const sfo_mesh *m, const double *G, const double *kappa,
                    const double *x, double *y, int n_threads)
{
  sfo_shape s;
  sfo_shape_init(m->degree, m->basis, &s);
  const int n = s.n, nq = n * n * n;
  const long long N = sfo_cont_n_dofs(m);
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < N; ++i) y[i] = 0.;
  const int nx = m->n_cells[0], ny = m->n_cells[1], nz = m->n_cells[2];
  double h[3];
  for (int d = 0; d < 3; ++d) h[d] = m->length[d] / m->n_cells[d];
  /* 8-colour cell order: cells of one colour share no node */
  for (int color = 0; color < 8; ++color) {
    const int cx = color & 1, cy = (color >> 1) & 1, cz = (color >> 2) & 1;
    const int mx = (nx - cx + 1) / 2, my = (ny - cy + 1) / 2, mz = (nz - cz + 1) / 2;
    const long long count = (long long)mx * my * mz;
#pragma omp parallel
    {
      /* G == NULL: each cell's geometry is computed where it is used */
      double *u = (double *)malloc(sizeof(double) * nq * (G ? 2 : 8));
      double *v = u + nq, *gc = u + 2 * nq;
#pragma omp for schedule(static)
      for (long long t = 0; t < count; ++t) {
        const int i = 2 * (int)(t % mx) + cx;
        const int j = 2 * (int)((t / mx) % my) + cy;
        const int k = 2 * (int)(t / ((long long)mx * my)) + cz;
        const long long cell = ((long long)k * ny + j) * nx + i;
        const double *Gc = G ? G + cell * 6 * nq : gc;
        if (!G) cont_cell_geometry(m, &s, i, j, k, h, gc);
        cont_gather(m, i, j, k, x, u);
        cell_apply_k(&s, Gc, nq, kappa ? kappa + cell * nq : NULL, u, v);
        for (int c = 0; c < n; ++c)
          for (int b = 0; b < n; ++b)
            for (int a = 0; a < n; ++a) {
              int bd;
              const long long g = cont_index(m, i, j, k, a, b, c, &bd);
              if (!bd) y[g] += v[(c * n + b) * n + a];
            }
      }
      free(u);
    }
  }
  if (m->dirichlet) {
    const int p = m->degree;
    const long long Nx = (long long)p * nx + 1, Ny = (long long)p * ny + 1,
                    Nz = (long long)p * nz + 1;
#pragma omp parallel for schedule(static)
    for (long long Z = 0; Z < Nz; ++Z)
      for (long long Y = 0; Y < Ny; ++Y)
        for (long long X = 0; X < Nx; ++X)
          if (X == 0 || Y == 0 || Z == 0 || X == Nx - 1 || Y == Ny - 1 || Z == Nz - 1) {
            const long long g = (Z * Ny + Y) * Nx + X;
            y[g] = x[g];
          }
  }
}

void sfo_cont_apply_op(const sfo_mesh *m, int kind, const double *b,
                       const double *x, double *y)
{
  sfo_shape s;
  sfo_shape_init(m->degree, m->basis, &s);
  const int n = s.n, nq = n * n * n;
  const long long N = sfo_cont_n_dofs(m);
  memset(y, 0, sizeof(double) * N);
  const int nx = m->n_cells[0], ny = m->n_cells[1], nz = m->n_cells[2];
  double ij[3], jxw = 1.;
  for (int d = 0; d < 3; ++d) {
    const double h = m->length[d] / m->n_cells[d];
    ij[d] = 1. / h;
    jxw *= h;
  }
  double *u = (double *)malloc(sizeof(double) * nq * 2);
  double *v = u + nq;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        cont_gather(m, i, j, k, x, u);
        cell_op_n(n, &s, kind, ij, jxw, b, u, v);
        for (int c = 0; c < n; ++c)
          for (int bb = 0; bb < n; ++bb)
            for (int a = 0; a < n; ++a) {
              int bd;
              const long long g = cont_index(m, i, j, k, a, bb, c, &bd);
              if (!bd) y[g] += v[(c * n + bb) * n + a];
            }
      }
  free(u);
  if (m->dirichlet) {
    const int p = m->degree;
    const long long Nx = (long long)p * nx + 1, Ny = (long long)p * ny + 1,
                    Nz = (long long)p * nz + 1;
    for (long long Z = 0; Z < Nz; ++Z)
      for (long long Y = 0; Y < Ny; ++Y)
        for (long long X = 0; X < Nx; ++X)
          if (X == 0 || Y == 0 || Z == 0 || X == Nx - 1 || Y == Ny - 1 || Z == Nz - 1) {
            const long long g = (Z * Ny + Y) * Nx + X;
            y[g] = x[g];
          }
  }
}

/* unstructured meshes: no counterpart in the reference (its evaluators take
 * structured meshes); the cell operator is cell_apply_k */
void sfo_unstructured_apply(int degree, int basis, long long n_cells, long long n_nodes,
                            const int *idx, const double *G, const unsigned char *dirichlet,
                            const double *x, double *y)
{
  sfo_shape s;
  sfo_shape_init(degree, basis, &s);
  const int nq = s.n * s.n * s.n;
  memset(y, 0, sizeof(double) * n_nodes);
  double *u = (double *)malloc(sizeof(double) * nq * 2);
  double *v = u + nq;
  for (long long e = 0; e < n_cells; ++e) {
    const int *id = idx + e * nq;
    for (int q = 0; q < nq; ++q) u[q] = (dirichlet && dirichlet[id[q]]) ? 0. : x[id[q]];
    cell_apply_k(&s, G + e * 6 * nq, nq, NULL, u, v);
    for (int q = 0; q < nq; ++q)
      if (!(dirichlet && dirichlet[id[q]])) y[id[q]] += v[q];
  }
  free(u);
  if (dirichlet)
    for (long long i = 0; i < n_nodes; ++i)
      if (dirichlet[i]) y[i] = x[i];
}

void sfo_cont_kappa_grad(const sfo_mesh *m, const double *G, const double *u,
                         const double *lam, double *dk)
{
  sfo_shape s;
  sfo_shape_init(m->degree, m->basis, &s);
  const int n = s.n, nq = n * n * n;
  const int nx = m->n_cells[0], ny = m->n_cells[1], nz = m->n_cells[2];
  const long long C = (long long)nx * ny * nz;
#pragma omp parallel
  {
    double *buf = (double *)malloc(sizeof(double) * nq * 10);
    double *cu = buf, *cl = buf + nq, *g1 = buf + 2 * nq, *g2 = buf + 6 * nq;
#pragma omp for schedule(static)
    for (long long cell = 0; cell < C; ++cell) {
      const int i = (int)(cell % nx), j = (int)((cell / nx) % ny),
                k = (int)(cell / ((long long)nx * ny));
      cont_gather(m, i, j, k, u, cu);
      cont_gather(m, i, j, k, lam, cl);
      cell_grad(&s, cu, g1, g1 + nq, g1 + 2 * nq, g1 + 3 * nq);
      cell_grad(&s, cl, g2, g2 + nq, g2 + 2 * nq, g2 + 3 * nq);
      const double *g = G + cell * 6 * nq;
      for (int q = 0; q < nq; ++q) {
        const double ax = g1[nq + q], ay = g1[2 * nq + q], az = g1[3 * nq + q];
        const double bx = g2[nq + q], by = g2[2 * nq + q], bz = g2[3 * nq + q];
        const double t0 = bx * g[q] + by * g[3 * nq + q] + bz * g[4 * nq + q];
        const double t1 = bx * g[3 * nq + q] + by * g[nq + q] + bz * g[5 * nq + q];
        const double t2 = bx * g[4 * nq + q] + by * g[5 * nq + q] + bz * g[2 * nq + q];
        dk[cell * nq + q] = ax * t0 + ay * t1 + az * t2;
      }
    }
    free(buf);
  }
}

void sfo_cont_diagonal(const sfo_mesh *m, const double *G, const double *kappa,
                       double *diag)
{
  sfo_shape s;
  sfo_shape_init(m->degree, m->basis, &s);
  const int n = s.n, nq = n * n * n;
  const long long N = sfo_cont_n_dofs(m);
  memset(diag, 0, sizeof(double) * N);
  const int nx = m->n_cells[0], ny = m->n_cells[1], nz = m->n_cells[2];
  double *e = (double *)calloc(nq, sizeof(double));
  double *v = (double *)malloc(sizeof(double) * nq);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long long cell = ((long long)k * ny + j) * nx + i;
        for (int l = 0; l < nq; ++l) {
          e[l] = 1.;
          cell_apply_k(&s, G + cell * 6 * nq, nq, kappa ? kappa + cell * nq : NULL, e, v);
          e[l] = 0.;
          const int a = l % n, b = (l / n) % n, c = l / (n * n);
          int bd;
          const long long g = cont_index(m, i, j, k, a, b, c, &bd);
          if (!bd) diag[g] += v[l];
        }
      }
  if (m->dirichlet) {
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
          for (int l = 0; l < nq; ++l) {
            int bd;
            const long long g = cont_index(m, i, j, k, l % n, (l / n) % n, l / (n * n), &bd);
            if (bd) diag[g] = 1.;
          }
  }
  free(e);
  free(v);
}

/* ------------------------------------------------------------------------ */
/* DG operators, cell-major layout (the reference's layout with one lane)    */
/* ------------------------------------------------------------------------ */
long long sfo_dg_n_dofs(const sfo_dg *g)
{
  const long long n = g->degree + 1;
  return (long long)g->n_cells[0] * g->n_cells[1] * g->n_cells[2] * n * n * n;
}

static inline long long dg_cell(const sfo_dg *g, int ix, int iy, int iz)
{
  const int nx = g->n_cells[0], ny = g->n_cells[1], nz = g->n_cells[2];
  ix = (ix + nx) % nx;
  iy = (iy + ny) % ny;
  iz = (iz + nz) % nz;
  return ((long long)iz * ny + iy) * nx + ix;
}

/* interpolate a face array (n x n, x fastest) to Gauss points in both
 * tangential directions (evaluation_dg_laplacian.h:205-219) */
static void face_interp(const sfo_shape *s, double *a)
{
  const int n = s->n;
  for (int i1 = 0; i1 < n; ++i1) sfo_apply_1d(n, 1, 0, 1, 0, s->S_eo, a + i1 * n, a + i1 * n, NULL, 0, NULL, NULL);
  for (int i1 = 0; i1 < n; ++i1) sfo_apply_1d(n, n, 0, 1, 0, s->S_eo, a + i1, a + i1, NULL, 0, NULL, NULL);
}

/* evaluation_dg_laplacian.h:130-510 with one lane (deviations (1), (2)) */
static void sipg_cell(const sfo_dg *g, const sfo_shape *s, int ix, int iy, int iz,
                      const double *x, double *out)
{
  const int deg = g->degree, n = deg + 1, dpf = n * n, dpc = n * n * n;
  double fw[SFO_MAX_N * SFO_MAX_N], qw[SFO_MAX_N * SFO_MAX_N * SFO_MAX_N];
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < n; ++a) fw[b * n + a] = s->wq[b] * s->wq[a];
  for (int c = 0; c < n; ++c)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) qw[(c * n + b) * n + a] = (s->wq[c] * s->wq[b]) * s->wq[a];
  const double ij[3] = {1. / g->h[0], 1. / g->h[1], 1. / g->h[2]};
  const double jxw = 1. / (ij[0] * ij[1] * ij[2]);
  const double h0 = s->hermite_d0;
  const double pf = g->penalty;
  double *data = (double *)malloc(sizeof(double) * 2 * dpc);
  double *af[6], *afd[6];
  double *fbuf = (double *)malloc(sizeof(double) * 12 * dpf);
  for (int f = 0; f < 6; ++f) {
    af[f] = fbuf + 2 * f * dpf;
    afd[f] = fbuf + (2 * f + 1) * dpf;
  }
  const double *src = x + dg_cell(g, ix, iy, iz) * dpc;

  for (int i2 = 0; i2 < n; ++i2) {
    double *in = data + i2 * n * n;
    for (int i1 = 0; i1 < n; ++i1)
      sfo_apply_1d(n, 1, 0, 1, 0, s->S_eo, src + i2 * n * n + i1 * n, in + i1 * n, NULL, 0, NULL, NULL);
    for (int i1 = 0; i1 < n; ++i1)
      sfo_apply_1d(n, n, 0, 1, 0, s->S_eo, in + i1, in + i1, NULL, 0, NULL, NULL);
  }
  /* z neighbours */
  {
    const long long idx[2] = {dg_cell(g, ix, iy, iz - 1) * dpc, dg_cell(g, ix, iy, iz + 1) * dpc};
    for (int f = 4; f < 6; ++f) {
      const double w0 = (f == 4 ? 1. : -1.) * h0;
      const int o1 = f == 4 ? dpf * deg : 0;
      const int o2 = dpf * (f == 4 ? deg - 1 : 1);
      for (int i = 0; i < dpf; ++i) {
        af[f][i] = x[idx[f % 2] + o1 + i];
        afd[f][i] = x[idx[f % 2] + o2 + i];
        afd[f][i] = w0 * (afd[f][i] - af[f][i]);
      }
      face_interp(s, af[f]);
      face_interp(s, afd[f]);
    }
    const double tau = (deg + 1) * (deg + 1) * pf * ij[2];
    const double jf = jxw * ij[2];
    for (int i2 = 0; i2 < dpf; ++i2) {
      sfo_apply_1d(n, dpf, 0, 1, 0, s->S_eo, data + i2, data + i2, NULL, 0, NULL, NULL);
      double fa[4];
      sfo_apply_1d(n, dpf, 1, 1, 0, s->D_eo, data + i2, data + dpc + i2, NULL, 2, s->face_eo, fa);
      {
        const double avg = 0.5 * ij[2] * (fa[2] + afd[4][i2]);
        const double jump = fa[0] - af[4][i2];
        af[4][i2] = (avg + jump * tau) * jf * fw[i2];
        afd[4][i2] = (0.5 * ij[2] * jf) * jump * fw[i2];
      }
      {
        const double avg = -0.5 * ij[2] * (fa[3] + afd[5][i2]);
        const double jump = fa[1] - af[5][i2];
        af[5][i2] = (avg + jump * tau) * jf * fw[i2];
        afd[5][i2] = (-0.5 * ij[2] * jf) * jump * fw[i2];
      }
    }
  }
  /* x neighbours (deviation (1): periodic right neighbour index) */
  {
    const long long idx[2] = {dg_cell(g, ix - 1, iy, iz) * dpc, dg_cell(g, ix + 1, iy, iz) * dpc};
    for (int f = 0; f < 2; ++f) {
      const double w0 = (f == 0 ? 1. : -1.) * h0;
      const int o1 = f == 0 ? deg : 0, o2 = f == 0 ? deg - 1 : 1;
      for (int i = 0; i < dpf; ++i) {
        af[f][i] = x[idx[f] + o1 + i * n];
        afd[f][i] = x[idx[f] + o2 + i * n];
        afd[f][i] = w0 * (afd[f][i] - af[f][i]);
      }
      face_interp(s, af[f]);
      face_interp(s, afd[f]);
    }
  }
  /* y neighbours */
  {
    const long long idx[2] = {dg_cell(g, ix, iy - 1, iz) * dpc, dg_cell(g, ix, iy + 1, iz) * dpc};
    for (int f = 2; f < 4; ++f) {
      const double w0 = (f == 2 ? 1. : -1.) * h0;
      for (int i1 = 0; i1 < n; ++i1) {
        const int b1 = i1 * n * n + (f == 2 ? deg : 0) * n;
        const int b2 = i1 * n * n + (f == 2 ? deg - 1 : 1) * n;
        for (int i2 = 0; i2 < n; ++i2) {
          const int i = i1 * n + i2;
          af[f][i] = x[idx[f % 2] + b1 + i2];
          afd[f][i] = x[idx[f % 2] + b2 + i2];
          afd[f][i] = w0 * (afd[f][i] - af[f][i]);
        }
      }
      face_interp(s, af[f]);
      face_interp(s, afd[f]);
    }
  }
  const double tauy = (deg + 1) * (deg + 1) * pf * ij[1], jfy = jxw * ij[1];
  const double taux = (deg + 1) * (deg + 1) * pf * ij[0], jfx = jxw * ij[0];
  double *a0 = (double *)malloc(sizeof(double) * dpf);
  double *a1 = (double *)malloc(sizeof(double) * dpf);
  for (int i2 = 0; i2 < n; ++i2) {
    const int off = i2 * dpf;
    double *ap = data + off, *a2p = data + dpc + off;
    const double *qp = qw + off;
    for (int i = 0; i < n; ++i) {
      const int i1 = i2 * n + i;
      double fa[4];
      sfo_apply_1d(n, n, 1, 1, 0, s->D_eo, ap + i, a1 + i, NULL, 2, s->face_eo, fa);
      const double w = fw[i1];
      {
        const double avg = 0.5 * ij[1] * (fa[2] + afd[2][i1]);
        const double jump = fa[0] - af[2][i1];
        af[2][i1] = (avg + jump * tauy) * jfy * w;
        afd[2][i1] = (0.5 * ij[1] * jfy) * jump * w;
      }
      {
        const double avg = -0.5 * ij[1] * (fa[3] + afd[3][i1]);
        const double jump = fa[1] - af[3][i1];
        af[3][i1] = (avg + jump * tauy) * jfy * w;
        afd[3][i1] = (-0.5 * ij[1] * jfy) * jump * w;
      }
      sfo_apply_1d(n, 1, 1, 1, 0, s->D_eo, ap + i * n, a0 + i * n, NULL, 2, s->face_eo, fa);
      {
        const double avg = 0.5 * ij[0] * (fa[2] + afd[0][i1]);
        const double jump = fa[0] - af[0][i1];
        af[0][i1] = (avg + jump * taux) * jfx * w;
        afd[0][i1] = (0.5 * ij[0] * jfx) * jump * w;
      }
      {
        const double avg = -0.5 * ij[0] * (fa[3] + afd[1][i1]);
        const double jump = fa[1] - af[1][i1];
        af[1][i1] = (avg + jump * taux) * jfx * w;
        afd[1][i1] = (-0.5 * ij[0] * jfx) * jump * w;
      }
    }
    for (int q = 0; q < dpf; ++q) {
      a0[q] *= (ij[0] * ij[0] * jxw) * qp[q];
      a1[q] *= (ij[1] * ij[1] * jxw) * qp[q];
      a2p[q] *= (ij[2] * ij[2] * jxw) * qp[q];
    }
    for (int i = 0; i < n; ++i) {
      const int i1 = i2 * n + i;
      double fa[4] = {af[0][i1] + af[1][i1], af[0][i1] - af[1][i1],
                      afd[0][i1] + afd[1][i1], afd[0][i1] - afd[1][i1]};
      sfo_apply_1d(n, 1, 1, 0, 0, s->D_eo, a0 + i * n, ap + i * n, NULL, 2, s->face_eo, fa);
    }
    for (int i = 0; i < n; ++i) {
      const int i1 = i2 * n + i;
      double fa[4] = {af[2][i1] + af[3][i1], af[2][i1] - af[3][i1],
                      afd[2][i1] + afd[3][i1], afd[2][i1] - afd[3][i1]};
      sfo_apply_1d(n, n, 1, 0, 1, s->D_eo, a1 + i, ap + i, ap + i, 2, s->face_eo, fa);
    }
  }
  for (int i2 = 0; i2 < dpf; ++i2) {
    double fa[4] = {af[4][i2] + af[5][i2], af[4][i2] - af[5][i2],
                    afd[4][i2] + afd[5][i2], afd[4][i2] - afd[5][i2]};
    sfo_apply_1d(n, dpf, 1, 0, 1, s->D_eo, data + dpc + i2, data + i2, data + i2, 2, s->face_eo, fa);
    sfo_apply_1d(n, dpf, 0, 0, 0, s->S_eo, data + i2, data + i2, NULL, 0, NULL, NULL);
  }
  for (int i2 = 0; i2 < n; ++i2) {
    const int off = i2 * dpf;
    for (int i1 = 0; i1 < n; ++i1)
      sfo_apply_1d(n, n, 0, 0, 0, s->S_eo, data + off + i1, data + off + i1, NULL, 0, NULL, NULL);
    /* deviation (2): transposed values in x */
    for (int i1 = 0; i1 < n; ++i1)
      sfo_apply_1d(n, 1, 0, 0, 0, s->S_eo, data + off + i1 * n, data + off + i1 * n, NULL, 0, NULL, NULL);
  }
  memcpy(out, data, sizeof(double) * dpc);
  free(a0);
  free(a1);
  free(fbuf);
  free(data);
}

void sfo_dg_sipg_apply(const sfo_dg *g, const double *x, double *y)
{
  sfo_shape s;
  sfo_shape_init(g->degree, SFO_BASIS_HERMITE, &s);
  const int dpc = s.n * s.n * s.n;
  const int nx = g->n_cells[0], ny = g->n_cells[1], nz = g->n_cells[2];
  const long long C = (long long)nx * ny * nz;
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < C; ++c) {
    const int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((long long)nx * ny));
    sipg_cell(g, &s, ix, iy, iz, x, y + c * dpc);
  }
}

/* diagonal by unit vectors on a cell-local basis: A_ii only involves the
 * cell itself, so apply the operator to e_i and read entry i (neighbour
 * contributions of e_i land in other cells' rows) */
void sfo_dg_sipg_diagonal(const sfo_dg *g, double *diag)
{
  sfo_shape s;
  sfo_shape_init(g->degree, SFO_BASIS_HERMITE, &s);
  const int dpc = s.n * s.n * s.n;
  const long long N = sfo_dg_n_dofs(g);
  const int nx = g->n_cells[0], ny = g->n_cells[1], nz = g->n_cells[2];
  const long long C = (long long)nx * ny * nz;
  double *e = (double *)calloc(N, sizeof(double));
  double *v = (double *)malloc(sizeof(double) * dpc);
  for (long long c = 0; c < C; ++c) {
    const int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((long long)nx * ny));
    for (int l = 0; l < dpc; ++l) {
      e[c * dpc + l] = 1.;
      sipg_cell(g, &s, ix, iy, iz, e, v);
      e[c * dpc + l] = 0.;
      diag[c * dpc + l] = v[l];
    }
  }
  free(e);
  free(v);
}

/* evaluation_dg_advect.h:286-676 with one lane (deviation (1)).
 * transpose == 0: y = [M^-1] K x; transpose == 1: y = K^T z with z = x
 * (the caller applies M^-1 first for the transposed inverse-mass form). */
static void advect_cell(const sfo_dg *g, const sfo_shape *s, int ix, int iy, int iz,
                        const double *x, int transpose, double *out)
{
  const int deg = g->degree, n = deg + 1, dpf = n * n, dpc = n * n * n, mid = n / 2;
  double fw[SFO_MAX_N * SFO_MAX_N], qw[SFO_MAX_N * SFO_MAX_N * SFO_MAX_N];
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < n; ++a) fw[b * n + a] = s->wq[b] * s->wq[a];
  for (int c = 0; c < n; ++c)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) qw[(c * n + b) * n + a] = (s->wq[c] * s->wq[b]) * s->wq[a];
  const double ij[3] = {1. / g->h[0], 1. / g->h[1], 1. / g->h[2]};
  const double jxw = 1. / (ij[0] * ij[1] * ij[2]);
  const double *adv = g->velocity;
  const double *fe = s->face_eo;
  double *data = (double *)malloc(sizeof(double) * 2 * dpc);
  double *fbuf = (double *)malloc(sizeof(double) * 6 * dpf);
  double *af[6];
  for (int f = 0; f < 6; ++f) af[f] = fbuf + f * dpf;
  const double *src = x + dg_cell(g, ix, iy, iz) * dpc;

  for (int i2 = 0; i2 < n; ++i2) {
    double *in = data + i2 * n * n;
    for (int i1 = 0; i1 < n; ++i1)
      sfo_apply_1d(n, 1, 0, 1, 0, s->S_eo, src + i2 * n * n + i1 * n, in + i1 * n, NULL, 0, NULL, NULL);
    for (int i1 = 0; i1 < n; ++i1)
      sfo_apply_1d(n, n, 0, 1, 0, s->S_eo, in + i1, in + i1, NULL, 0, NULL, NULL);
  }
  /* flux: forward -1/2((u-+u+) an + |an| (u- - u+)); transpose
   * -1/2 (an + |an|)(u- - u+) (the adjoint of the upwind flux) */
#define FLUX(um, up, an, J, w)                                                   \
  (transpose ? (-0.5 * ((an) + fabs(an)) * ((um) - (up)) * (J) * (w))            \
             : (-0.5 * (((um) + (up)) * (an) + fabs(an) * ((um) - (up))) * (J) * (w)))
  {
    const long long idx[2] = {dg_cell(g, ix, iy, iz - 1) * dpc, dg_cell(g, ix, iy, iz + 1) * dpc};
    for (int f = 4; f < 6; ++f) {
      const int o1 = f == 4 ? dpf * deg : 0;
      for (int i = 0; i < dpf; ++i) af[f][i] = x[idx[f % 2] + o1 + i];
      face_interp(s, af[f]);
    }
    const double jf = jxw * ij[2];
    for (int i2 = 0; i2 < dpf; ++i2) {
      sfo_apply_1d(n, dpf, 0, 1, 0, s->S_eo, data + i2, data + i2, NULL, 0, NULL, NULL);
      double r0 = fe[0] * (data[i2] + data[i2 + dpf * (n - 1)]);
      double r1 = fe[n - 1] * (data[i2] - data[i2 + dpf * (n - 1)]);
      for (int ind = 1; ind < mid; ++ind) {
        r0 += fe[ind] * (data[i2 + dpf * ind] + data[i2 + dpf * (n - 1 - ind)]);
        r1 += fe[n - 1 - ind] * (data[i2 + dpf * ind] - data[i2 + dpf * (n - 1 - ind)]);
      }
      if (n % 2 == 1) r0 += fe[mid] * data[i2 + dpf * mid];
      af[4][i2] = FLUX(r0 + r1, af[4][i2], -adv[2], jf, fw[i2]);
      af[5][i2] = FLUX(r0 - r1, af[5][i2], adv[2], jf, fw[i2]);
    }
  }
  {
    const long long idx[2] = {dg_cell(g, ix - 1, iy, iz) * dpc, dg_cell(g, ix + 1, iy, iz) * dpc};
    for (int f = 0; f < 2; ++f) {
      const int o1 = f == 0 ? deg : 0;
      for (int i = 0; i < dpf; ++i) af[f][i] = x[idx[f] + o1 + i * n];
      face_interp(s, af[f]);
    }
  }
  {
    const long long idx[2] = {dg_cell(g, ix, iy - 1, iz) * dpc, dg_cell(g, ix, iy + 1, iz) * dpc};
    for (int f = 2; f < 4; ++f) {
      for (int i1 = 0; i1 < n; ++i1) {
        const int b1 = i1 * n * n + (f == 2 ? deg : 0) * n;
        for (int i2 = 0; i2 < n; ++i2) af[f][i1 * n + i2] = x[idx[f % 2] + b1 + i2];
      }
      face_interp(s, af[f]);
    }
  }
  const double jfy = jxw * ij[1], jfx = jxw * ij[0];
  double *a0 = (double *)malloc(sizeof(double) * dpf);
  double *a1 = (double *)malloc(sizeof(double) * dpf);
  for (int i2 = 0; i2 < n; ++i2) {
    const int off = i2 * dpf;
    double *ap = data + off, *a2p = data + dpc + off;
    const double *qp = qw + off;
    for (int i = 0; i < n; ++i) {
      const int i1 = i2 * n + i;
      const double w = fw[i1];
      double r0 = fe[0] * (ap[i] + ap[i + n * (n - 1)]);
      double r1 = fe[n - 1] * (ap[i] - ap[i + n * (n - 1)]);
      for (int ind = 1; ind < mid; ++ind) {
        r0 += fe[ind] * (ap[i + n * ind] + ap[i + n * (n - 1 - ind)]);
        r1 += fe[n - 1 - ind] * (ap[i + n * ind] - ap[i + n * (n - 1 - ind)]);
      }
      if (n % 2 == 1) r0 += fe[mid] * ap[i + n * mid];
      af[2][i1] = FLUX(r0 + r1, af[2][i1], -adv[1], jfy, w);
      af[3][i1] = FLUX(r0 - r1, af[3][i1], adv[1], jfy, w);
      r0 = fe[0] * (ap[i * n] + ap[i * n + (n - 1)]);
      r1 = fe[n - 1] * (ap[i * n] - ap[i * n + (n - 1)]);
      for (int ind = 1; ind < mid; ++ind) {
        r0 += fe[ind] * (ap[i * n + ind] + ap[i * n + (n - 1 - ind)]);
        r1 += fe[n - 1 - ind] * (ap[i * n + ind] - ap[i * n + (n - 1 - ind)]);
      }
      if (n % 2 == 1) r0 += fe[mid] * ap[i * n + mid];
      af[0][i1] = FLUX(r0 + r1, af[0][i1], -adv[0], jfx, w);
      af[1][i1] = FLUX(r0 - r1, af[1][i1], adv[0], jfx, w);
    }
    if (!transpose) {
      /* cell term a_d J^-1_d JxW w u, integrated with D^T */
      for (int q = 0; q < dpf; ++q) {
        a0[q] = adv[0] * ij[0] * (jxw * qp[q] * ap[q]);
        a1[q] = adv[1] * ij[1] * (jxw * qp[q] * ap[q]);
        a2p[q] = adv[2] * ij[2] * (jxw * qp[q] * ap[q]);
      }
      for (int i = 0; i < n; ++i) {
        const int i1 = i2 * n + i;
        double fa[2] = {af[0][i1] + af[1][i1], af[0][i1] - af[1][i1]};
        sfo_apply_1d(n, 1, 1, 0, 0, s->D_eo, a0 + i * n, ap + i * n, NULL, 1, fe, fa);
      }
      for (int i = 0; i < n; ++i) {
        const int i1 = i2 * n + i;
        double fa[2] = {af[2][i1] + af[3][i1], af[2][i1] - af[3][i1]};
        sfo_apply_1d(n, n, 1, 0, 1, s->D_eo, a1 + i, ap + i, ap + i, 1, fe, fa);
      }
    }
  }
  if (transpose) {
    /* adjoint cell term: JxW w sum_d a_d J^-1_d (D_d u)_q, then the face
     * terms injected with the transposed face evaluation */
    double *gq = (double *)malloc(sizeof(double) * dpc);
    double *tq = (double *)malloc(sizeof(double) * dpc);
    memcpy(gq, data, sizeof(double) * dpc);
    sweep(n, 0, 1, 1, 0, s->D_eo, gq, tq);
    for (int q = 0; q < dpc; ++q) data[dpc + q] = adv[0] * ij[0] * (jxw * qw[q] * tq[q]);
    sweep(n, 1, 1, 1, 0, s->D_eo, gq, tq);
    for (int q = 0; q < dpc; ++q) data[dpc + q] += adv[1] * ij[1] * (jxw * qw[q] * tq[q]);
    sweep(n, 2, 1, 1, 0, s->D_eo, gq, tq);
    for (int q = 0; q < dpc; ++q) data[dpc + q] += adv[2] * ij[2] * (jxw * qw[q] * tq[q]);
    /* face injections: value at 0 / 1 along each direction */
    for (int c = 0; c < n; ++c)
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const int q = (c * n + b) * n + a;
          double v = data[dpc + q];
          v += s->face_v[0][a] * af[0][c * n + b] + s->face_v[1][a] * af[1][c * n + b];
          v += s->face_v[0][b] * af[2][c * n + a] + s->face_v[1][b] * af[3][c * n + a];
          v += s->face_v[0][c] * af[4][b * n + a] + s->face_v[1][c] * af[5][b * n + a];
          tq[q] = v;
        }
    /* integrate with the transposed values */
    sweep(n, 2, 0, 0, 0, s->S_eo, tq, gq);
    sweep(n, 1, 0, 0, 0, s->S_eo, gq, tq);
    sweep(n, 0, 0, 0, 0, s->S_eo, tq, out);
    free(gq);
    free(tq);
  } else {
    for (int i2 = 0; i2 < dpf; ++i2) {
      double fa[2] = {af[4][i2] + af[5][i2], af[4][i2] - af[5][i2]};
      sfo_apply_1d(n, dpf, 1, 0, 1, s->D_eo, data + dpc + i2, data + i2, data + i2, 1, fe, fa);
      if (g->inverse_mass) {
        for (int i = 0; i < n; ++i) data[i2 + i * dpf] /= jxw * qw[i2 + i * dpf];
        sfo_apply_1d(n, dpf, 0, 1, 0, s->Sinv_eo, data + i2, data + i2, NULL, 0, NULL, NULL);
      } else {
        sfo_apply_1d(n, dpf, 0, 0, 0, s->S_eo, data + i2, data + i2, NULL, 0, NULL, NULL);
      }
    }
    for (int i2 = 0; i2 < n; ++i2) {
      const int off = i2 * dpf;
      for (int i1 = 0; i1 < n; ++i1) {
        if (g->inverse_mass)
          sfo_apply_1d(n, n, 0, 1, 0, s->Sinv_eo, data + off + i1, data + off + i1, NULL, 0, NULL, NULL);
        else
          sfo_apply_1d(n, n, 0, 0, 0, s->S_eo, data + off + i1, data + off + i1, NULL, 0, NULL, NULL);
      }
      for (int i1 = 0; i1 < n; ++i1) {
        if (g->inverse_mass)
          sfo_apply_1d(n, 1, 0, 1, 0, s->Sinv_eo, data + off + i1 * n, data + off + i1 * n, NULL, 0, NULL, NULL);
        else
          sfo_apply_1d(n, 1, 0, 0, 0, s->S_eo, data + off + i1 * n, data + off + i1 * n, NULL, 0, NULL, NULL);
      }
    }
    memcpy(out, data, sizeof(double) * dpc);
  }
#undef FLUX
  free(a0);
  free(a1);
  free(fbuf);
  free(data);
}

void sfo_dg_advect_apply(const sfo_dg *g, const double *x, double *y)
{
  sfo_shape s;
  sfo_shape_init(g->degree, SFO_BASIS_GLL, &s);
  const int dpc = s.n * s.n * s.n;
  const int nx = g->n_cells[0], ny = g->n_cells[1], nz = g->n_cells[2];
  const long long C = (long long)nx * ny * nz;
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < C; ++c) {
    const int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((long long)nx * ny));
    advect_cell(g, &s, ix, iy, iz, x, 0, y + c * dpc);
  }
}

/* 1D matrices of precomputed_dg_laplacian.h:307-377 (fill_shape_values),
 * formed from the Hermite-like values S and collocation derivatives D at the
 * Gauss points (exact for the degree-p basis), with the corrected
 * neighbour couplings */
void sfo_dg_precomputed_matrices(int degree, double *M, double *L, double *iv)
{
  sfo_shape s;
  sfo_shape_init(degree, SFO_BASIS_HERMITE, &s);
  const int n = s.n;
  double v0[SFO_MAX_N], v1[SFO_MAX_N], d0[SFO_MAX_N], d1[SFO_MAX_N], dq[SFO_MAX_N * SFO_MAX_N];
  for (int i = 0; i < n; ++i) {
    v0[i] = v1[i] = d0[i] = d1[i] = 0.0;
    for (int q = 0; q < n; ++q) {
      v0[i] += s.face_v[0][q] * s.S[q * n + i];
      v1[i] += s.face_v[1][q] * s.S[q * n + i];
      d0[i] += s.face_d[0][q] * s.S[q * n + i];
      d1[i] += s.face_d[1][q] * s.S[q * n + i];
      double t = 0.0;
      for (int j = 0; j < n; ++j) t += s.D[q * n + j] * s.S[j * n + i];
      dq[q * n + i] = t;
    }
  }
  const double pen = (double)degree * (degree + 1);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double m = 0.0, l = 0.0;
      for (int q = 0; q < n; ++q) {
        m += s.wq[q] * s.S[q * n + i] * s.S[q * n + j];
        l += s.wq[q] * dq[q * n + i] * dq[q * n + j];
      }
      l += pen * v0[i] * v0[j] + 0.5 * d0[i] * v0[j] + 0.5 * d0[j] * v0[i];
      l += pen * v1[i] * v1[j] - 0.5 * d1[i] * v1[j] - 0.5 * d1[j] * v1[i];
      M[i * n + j] = m;
      L[i * n + j] = l;
    }
  iv[0] = -pen * v0[0] * v1[n - 1] - 0.5 * d0[0] * v1[n - 1] + 0.5 * d1[n - 1] * v0[0];
  iv[1] = -pen * v0[0] * v1[n - 2] - 0.5 * d0[0] * v1[n - 2] + 0.5 * d1[n - 2] * v0[0];
}

/* out += c * A along direction dir of an n^3 cell block (x fastest) */
static void block_matvec(int n, const double *A, int dir, double c, const double *in, double *out)
{
  const int st = dir == 0 ? 1 : (dir == 1 ? n : n * n);
  for (int k = 0; k < n * n; ++k) {
    const int base = dir == 0 ? k * n : (dir == 1 ? (k % n) + (k / n) * n * n : k);
    for (int i = 0; i < n; ++i) {
      double t = 0.0;
      for (int j = 0; j < n; ++j) t += A[i * n + j] * in[base + j * st];
      out[base + i * st] += c * t;
    }
  }
}

void sfo_dg_precomputed_apply(const sfo_dg *g, const double *x, double *y)
{
  const int n = g->degree + 1, dpc = n * n * n;
  double M[SFO_MAX_N * SFO_MAX_N], L[SFO_MAX_N * SFO_MAX_N], iv[2];
  sfo_dg_precomputed_matrices(g->degree, M, L, iv);
  const int nx = g->n_cells[0], ny = g->n_cells[1], nz = g->n_cells[2];
  const long long C = (long long)nx * ny * nz;
  const double vol = g->h[0] * g->h[1] * g->h[2];
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < C; ++c) {
    const int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((long long)nx * ny));
    const int ic[3] = {ix, iy, iz}, ncs[3] = {nx, ny, nz};
    const double *u = x + c * dpc;
    double t[1000], t2[1000], t3[1000];
    double *out = y + c * dpc;
    for (int q = 0; q < dpc; ++q) out[q] = 0.0;
    for (int d = 0; d < 3; ++d) {
      const int st = d == 0 ? 1 : (d == 1 ? n : n * n);
      int jl[3] = {ix, iy, iz}, jr[3] = {ix, iy, iz};
      jl[d] = ic[d] == 0 ? ncs[d] - 1 : ic[d] - 1;
      jr[d] = ic[d] == ncs[d] - 1 ? 0 : ic[d] + 1;
      const double *ul = x + (((long long)jl[2] * ny + jl[1]) * nx + jl[0]) * dpc;
      const double *ur = x + (((long long)jr[2] * ny + jr[1]) * nx + jr[0]) * dpc;
      for (int q = 0; q < dpc; ++q) t[q] = 0.0;
      block_matvec(n, L, d, 1.0, u, t);
      /* neighbour layers: lines along d, base index without the d coordinate */
      for (int k = 0; k < n * n; ++k) {
        const int base = d == 0 ? k * n : (d == 1 ? (k % n) + (k / n) * n * n : k);
        t[base] += iv[0] * ul[base + (n - 1) * st] + iv[1] * ul[base + (n - 2) * st];
        t[base + st] += iv[1] * ul[base + (n - 1) * st];
        t[base + (n - 1) * st] += iv[0] * ur[base] + iv[1] * ur[base + st];
        t[base + (n - 2) * st] += iv[1] * ur[base];
      }
      /* mass matrices in the two other directions */
      const int e = (d + 1) % 3, f = (d + 2) % 3;
      for (int q = 0; q < dpc; ++q) t2[q] = 0.0;
      block_matvec(n, M, e, 1.0, t, t2);
      for (int q = 0; q < dpc; ++q) t3[q] = 0.0;
      block_matvec(n, M, f, 1.0, t2, t3);
      const double cd = vol / (g->h[d] * g->h[d]);
      for (int q = 0; q < dpc; ++q) out[q] += cd * t3[q];
    }
  }
}

void sfo_dg_precomputed_diagonal(const sfo_dg *g, double *diag)
{
  const int n = g->degree + 1, dpc = n * n * n;
  double M[SFO_MAX_N * SFO_MAX_N], L[SFO_MAX_N * SFO_MAX_N], iv[2];
  sfo_dg_precomputed_matrices(g->degree, M, L, iv);
  const double vol = g->h[0] * g->h[1] * g->h[2];
  const double c[3] = {vol / (g->h[0] * g->h[0]), vol / (g->h[1] * g->h[1]), vol / (g->h[2] * g->h[2])};
  const long long C = (long long)g->n_cells[0] * g->n_cells[1] * g->n_cells[2];
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double v = c[0] * L[i * n + i] * M[j * n + j] * M[k * n + k] +
                         c[1] * M[i * n + i] * L[j * n + j] * M[k * n + k] +
                         c[2] * M[i * n + i] * M[j * n + j] * L[k * n + k];
        for (long long cc = 0; cc < C; ++cc) diag[cc * dpc + (k * n + j) * n + i] = v;
      }
}

void sfo_dg_rk_stage(const sfo_dg *g, const double *src, const double *upd,
                     double *vec_np, double *vec_tm, double c_np, double c_tm)
{
  const long long N = sfo_dg_n_dofs(g);
  double *r = (double *)malloc(sizeof(double) * N);
  sfo_dg_advect_apply(g, src, r);
  for (long long i = 0; i < N; ++i) {
    const double np = upd[i] + c_np * r[i];
    vec_np[i] = np;
    if (c_tm != 0.) vec_tm[i] = np + c_tm * r[i];
  }
  free(r);
}

/* LSRK(5,4) coefficients and the register rotation of do_time_step
 * (evaluation_dg_advect.h:192-212) */
void sfo_dg_lsrk_step(const sfo_dg *g, double dt, double *sol_new, double *sol_old,
                      double *sol_tmp)
{
  const double a21 = 970286171893. / 4311952581923.;
  const double a32 = 6584761158862. / 12103376702013.;
  const double a43 = 2251764453980. / 15575788980749.;
  const double a54 = 26877169314380. / 34165994151039.;
  const double b1 = 1153189308089. / 22510343858157.;
  const double b2 = 1772645290293. / 4653164025191.;
  const double b3 = -1672844663538. / 4480602732383.;
  const double b4 = 2114624349019. / 3568978502595.;
  const double b5 = 5198255086312. / 14908931495163.;
  sfo_dg_rk_stage(g, sol_new, sol_new, sol_old, sol_tmp, a21 * dt, (b1 - a21) * dt);
  sfo_dg_rk_stage(g, sol_old, sol_tmp, sol_new, sol_tmp, a32 * dt, (b2 - a32) * dt);
  sfo_dg_rk_stage(g, sol_new, sol_tmp, sol_old, sol_tmp, a43 * dt, (b3 - a43) * dt);
  sfo_dg_rk_stage(g, sol_old, sol_tmp, sol_tmp, sol_new, a54 * dt, (b4 - a54) * dt);
  sfo_dg_rk_stage(g, sol_tmp, sol_new, sol_new, sol_tmp, b5 * dt, 0.0);
}

/* inverse mass matrix of the GLL basis with Gauss quadrature,
 * M^-1 = P W^-1 P^T per cell, P = Sinv (Gauss values -> GLL nodal values);
 * the reference applies P W^-1 on collocation residuals
 * (evaluation_dg_advect.h:619-648); M^-1 is symmetric */
static void dg_inverse_mass(const sfo_dg *g, const sfo_shape *s,
                            const double *x, double *y)
{
  const int n = s->n, dpc = n * n * n;
  const long long C = (long long)g->n_cells[0] * g->n_cells[1] * g->n_cells[2];
  const double jxw = g->h[0] * g->h[1] * g->h[2];
  double *t = (double *)malloc(sizeof(double) * dpc);
  double *u = (double *)malloc(sizeof(double) * dpc);
  for (long long c = 0; c < C; ++c) {
    sweep(n, 0, 0, 0, 0, s->Sinv_eo, x + c * dpc, t);
    sweep(n, 1, 0, 0, 0, s->Sinv_eo, t, u);
    sweep(n, 2, 0, 0, 0, s->Sinv_eo, u, t);
    for (int cz = 0; cz < n; ++cz)
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const int q = (cz * n + b) * n + a;
          t[q] /= jxw * ((s->wq[cz] * s->wq[b]) * s->wq[a]);
        }
    sweep(n, 2, 0, 1, 0, s->Sinv_eo, t, u);
    sweep(n, 1, 0, 1, 0, s->Sinv_eo, u, t);
    sweep(n, 0, 0, 1, 0, s->Sinv_eo, t, y + c * dpc);
  }
  free(t);
  free(u);
}

void sfo_dg_advect_apply_transpose(const sfo_dg *g, const double *x, double *y)
{
  sfo_shape s;
  sfo_shape_init(g->degree, SFO_BASIS_GLL, &s);
  const int dpc = s.n * s.n * s.n;
  const int nx = g->n_cells[0], ny = g->n_cells[1], nz = g->n_cells[2];
  const long long C = (long long)nx * ny * nz;
  const double *z = x;
  double *tmp = NULL;
  if (g->inverse_mass) {
    tmp = (double *)malloc(sizeof(double) * C * dpc);
    dg_inverse_mass(g, &s, x, tmp);
    z = tmp;
  }
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < C; ++c) {
    const int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((long long)nx * ny));
    advect_cell(g, &s, ix, iy, iz, z, 1, y + c * dpc);
  }
  free(tmp);
}

/* evaluation_dg_laplacian.h:485-502 (deviation (4)) */
void sfo_chebyshev_update(long long n, const double *ax, const double *b,
                          const double *diag_inv, const double *x_old,
                          double *x_new, double *t, double c_np, double c_tm)
{
  for (long long i = 0; i < n; ++i) {
    const double res = ax[i] - b[i];
    const double tmp = c_tm * t[i] + c_np * diag_inv[i] * res;
    t[i] = tmp;
    x_new[i] = x_old[i] - tmp;
  }
}
