/*
 * Golden-vector adapter for the Hermite-like-basis cell Laplacian of
 * legacy/include/evaluation_cell_laplacian.h:26-908 (Cartesian branch).
 * TEST INFRASTRUCTURE ONLY (oracle/build.py).
 */
#include "ref_shim.h"
#include "evaluation_cell_laplacian.h"

template <int p>
static void herm_tables(double *S_eo, double *D_eo, double *w, double *hd0)
{
  EvaluationCellLaplacian<3, p, double> ev;
  ev.initialize(1, true);
  const int n = p + 1, st = (n + 1) / 2;
  for (int i = 0; i < n * st; ++i) { S_eo[i] = ev.shape_values[i][0]; D_eo[i] = ev.shape_gradients[i][0]; }
  for (int i = 0; i < n * n * n; ++i) w[i] = ev.quadrature_weights[i];
  *hd0 = ev.hermite_derivative_on_face[0];
}

/* one cell with inverse Jacobian diag(ij) and JxW factor jxw */
template <int p>
static void herm_cell(const double *ij, double jxw, const double *in, double *out)
{
  EvaluationCellLaplacian<3, p, double> ev;
  ev.initialize(1, true);
  for (int d = 0; d < 3; ++d) ev.jacobian_data[d] = ij[d];
  ev.jxw_data[0] = jxw;
  const int nq = (p + 1) * (p + 1) * (p + 1);
  for (int i = 0; i < nq; ++i) ev.input_array[i] = in[i];
  ev.matrix_vector_product();
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

extern "C" int sfref_herm_tables(int degree, double *S_eo, double *D_eo, double *w, double *hd0)
{ SF_DISPATCH(herm_tables, S_eo, D_eo, w, hd0) }

extern "C" int sfref_herm_cell(int degree, const double *ij, double jxw, const double *in, double *out)
{ SF_DISPATCH(herm_cell, ij, jxw, in, out) }
