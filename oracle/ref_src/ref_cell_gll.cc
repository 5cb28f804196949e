/*
 * Golden-vector adapter for the GLL-basis cell Laplacian of
 * legacy/src/benchmark_loops.cc:1154-1488 (class EvaluationCellLaplacian,
 * even-odd kernel 4).  The translation unit includes that source file with
 * its main() renamed.  TEST INFRASTRUCTURE ONLY (oracle/build.py).
 */
#include "ref_shim.h"
#define main sfref_benchmark_loops_main
#include "benchmark_loops.cc"
#undef main

template <int p>
static void gll_tables(double *S_eo, double *D_eo, double *w)
{
  EvaluationCellLaplacian<3, p, double> ev;
  ev.initialize(1, true);
  const int n = p + 1, st = (n + 1) / 2;
  for (int i = 0; i < n * st; ++i) { S_eo[i] = ev.shape_values_eo[i][0]; D_eo[i] = ev.shape_gradients_eo[i][0]; }
  for (int i = 0; i < n * n * n; ++i) w[i] = ev.quadrature_weights[i];
}

/* one cell: out = S^T D^T (w_q G6 D S in) with a constant merged tensor G6
 * (order xx,yy,zz,xy,xz,yz, no quadrature weight) */
template <int p>
static void gll_cell(const double *G6, const double *in, double *out)
{
  EvaluationCellLaplacian<3, p, double> ev;
  ev.initialize(1, true);
  for (int e = 0; e < 6; ++e) ev.jacobian_data[e] = G6[e];
  const int nq = (p + 1) * (p + 1) * (p + 1);
  for (int i = 0; i < nq; ++i) ev.input_array[i] = in[i];
  ev.template matrix_vector_product<4>();
  for (int i = 0; i < nq; ++i) out[i] = ev.output_array[i][0];
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

extern "C" int sfref_gll_tables(int degree, double *S_eo, double *D_eo, double *w)
{ SF_DISPATCH(gll_tables, S_eo, D_eo, w) }

extern "C" int sfref_gll_cell(int degree, const double *G6, const double *in, double *out)
{ SF_DISPATCH(gll_cell, G6, in, out) }
