// sf_cell_faces.cu -- the DO_FACES build of the reference's cell operator
// (evaluation_cell_laplacian.h:505-797, set-up :84-100): per cell of a
// cell-major vector (n^3 entries per cell, Hermite-like basis, Cartesian
// cells of size h), the cell Laplacian (SF_OP_LAPLACE_FACES) or the cell
// convection form (SF_OP_CONVECTION_FACES) plus face terms in which the
// cell's own faces at 1 ("right", node layer p) and at 0 ("left", layer 0)
// of each direction f act as the two sides of one face.  No neighbour is
// read: the operator is block diagonal.
//
// Face terms, face coordinates (i1, i2) along directions f+1, f+2 (mod 3),
// face Gauss weights W = -w_q1 w_q2 prod_{e != f} h_e, hd = phi_0'(0):
//   values uR, uL and normal derivatives nR = hd (u_{p-1} - u_p),
//   nL = hd (u_1 - u_0) interpolated by S x S;
//   Laplacian:  a = (uR + uL) / 2, v = W (2 sigma_f a - ij_f (nR + nL) / 2),
//               sigma_f = (p+1)^2 ij_f, d = W ij_f a;
//               layer p   += (S x S)^T (-v) - hd (S x S) d,  layer p-1 += hd (S x S) d,
//               layer 0   += (S x S)^T v    - hd (S x S) d,  layer 1   += hd (S x S) d
//               (the forward S on d is the reference's, :756-759);
//   convection: flux = ((uR + uL) b_f + |b_f| (uR - uL)) / 2,
//               layer p += (S x S)^T (W flux), layer 0 -= (S x S)^T (W flux).
// The reference also forms tangential-gradient terms weighted by zero
// entries of its normal Jacobian (:88-93); they vanish and are not computed.
//
// GPU mapping as the DG kernels: CPB consecutive cells per block, n^2
// threads per cell, z columns read and written straight from the vector.
// Per cell: the input slab X (kept for the face terms), three work slabs
// and four face arrays in shared memory, laid out per degree and precision
// by faces_layout.  Thread (a, b) owns the z column
// (x, y) = (a, b), the x line (y, z) = (a, b) and the y line (x, z) = (a, b)
// in the cell term, and face point (q1, q2) = (a, b) in the face terms.
#include "sf_launch.h"
#include "sf_tables.h"

namespace sf {
namespace {

// Shared-memory layout per cell: four slabs (X, Sa, Sb, Sc) RS words apart
// with entry (x, y, z) at SX x + SY y + SZ z, four face arrays FA words apart
// with entry (i2, i1) at FN i2 + i1, and a cell stride of CW words.
struct FacesLayout {
  int SX, SY, SZ, RS, FN, FA, CW;
};

// Layouts from a shared-memory bank model of every access of the kernel
// (faces_cost in sum_factorization_kernels_gb300/bank_model.py: the cell
// term's z, x and y line patterns on the four slabs, the face phases' layer
// reads, row and column passes and injections): stride
// permutations of (1, P1, P2), slab size, face-array strides and the cell
// stride searched with the per-cell words held at most 8 above those of the
// padded layout (strides (1, n + 1, n (n + 1) + 1), dense face arrays), so
// that residency does not drop.  Modelled wavefronts per cell
// (Laplacian, FP32) against the padded layout: n=2 31/56, 3 125/268,
// 4 198/348, 5 382/513, 6 619/805, 7 832/1045, 8 1008/2208, 9 1478/1919;
// ncu counts 532 per cell for the padded layout at n=5 (model 513).
constexpr FacesLayout faces_layout(int n, int elem)
{
  return elem == 4 ? (n == 2   ? FacesLayout{5, 2, 1, 9, 3, 6, 60}
                      : n == 3 ? FacesLayout{3, 1, 10, 29, 6, 21, 200}
                      : n == 4 ? FacesLayout{19, 4, 1, 76, 5, 24, 400}
                      : n == 5 ? FacesLayout{5, 25, 1, 130, 5, 25, 637}
                      : n == 6 ? FacesLayout{1, 6, 39, 237, 7, 44, 1124}
                      : n == 7 ? FacesLayout{1, 7, 52, 361, 7, 56, 1681}
                      : n == 8 ? FacesLayout{67, 1, 8, 533, 9, 72, 2420}
                               : FacesLayout{1, 9, 81, 731, 9, 81, 3249})
                   : (n == 2   ? FacesLayout{5, 2, 1, 9, 3, 6, 60}
                      : n == 3 ? FacesLayout{5, 1, 13, 40, 3, 9, 196}
                      : n == 4 ? FacesLayout{19, 4, 1, 73, 5, 20, 372}
                      : n == 5 ? FacesLayout{1, 5, 25, 126, 5, 25, 617}
                      : n == 6 ? FacesLayout{41, 1, 6, 241, 6, 40, 1124}
                      : n == 7 ? FacesLayout{1, 7, 49, 343, 7, 56, 1601}
                      : n == 8 ? FacesLayout{66, 1, 8, 526, 9, 72, 2392}
                               : FacesLayout{1, 9, 81, 729, 9, 89, 3281});
}

// every slab entry on its own word inside RS, everything inside CW
constexpr bool faces_layout_fits(int n, FacesLayout L)
{
  bool seen[4096] = {};
  if (L.RS > 4096 || L.FN < n || L.FA < n * L.FN || L.CW < 4 * L.RS + 4 * L.FA) return false;
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        const int i = L.SX * x + L.SY * y + L.SZ * z;
        if (i < 0 || i >= L.RS || seen[i]) return false;
        seen[i] = true;
      }
  return true;
}

template <int N, typename T>
struct FacesCfg {
  static constexpr int CPB = CellsPerBlock<N>::value;
  static constexpr FacesLayout L = faces_layout(N, (int)sizeof(T));
  static constexpr size_t SMEM = (size_t)CPB * L.CW * sizeof(T);
  static_assert(faces_layout_fits(N, L), "face-operator layout overlaps");
};

template <int N, typename T>
struct FacesArgs {
  EOMat<N, T> S, ST, D, DT;
  T w[N];       // 1D Gauss weights
  T c[3];       // cell term: Laplacian JxW ij_d^2, convection b_d ij_d
  T jxw;        // hx hy hz
  T fw[3];      // -prod_{e != f} h_e
  T ij[3];      // 1 / h_f
  T sigma[3];   // (p+1)^2 / h_f
  T bn[3];      // b_f
  T hd;         // phi_0'(0)
  long long n_cells;
  const T *x;
  T *y;
};

template <int N, typename T, bool CONV>
__global__ void __launch_bounds__(FacesCfg<N, T>::CPB * N * N)
    cell_faces_kernel(const __grid_constant__ FacesArgs<N, T> A)
{
  using Cfg = FacesCfg<N, T>;
  constexpr int N2 = N * N, N3 = N2 * N, P = N - 1;
  constexpr int SX = Cfg::L.SX, SY = Cfg::L.SY, SZ = Cfg::L.SZ, FN = Cfg::L.FN, FA = Cfg::L.FA;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k = threadIdx.x / N2, l = threadIdx.x % N2;
  const int a = l % N, b = l / N;
  T *X = reinterpret_cast<T *>(smem_raw) + k * Cfg::L.CW;
  T *Sa = X + Cfg::L.RS, *Sb = Sa + Cfg::L.RS, *Sc = Sb + Cfg::L.RS;
  T *F = Sc + Cfg::L.RS;
  const long long cell = (long long)blockIdx.x * Cfg::CPB + k;
  const bool valid = cell < A.n_cells;
  const long long base = ((long long)blockIdx.y * A.n_cells + (valid ? cell : 0)) * N3;
  // line bases: z column (x, y) = (a, b), x line (y, z) = (a, b), y line (x, z) = (a, b)
  const int zc = SX * a + SY * b, xl = SY * a + SZ * b, yl = SX * a + SZ * b;
  const int fq = FN * b + a; // face point (q1, q2) = (a, b)
  T v[N], g[N];

  // ---- input z column; S_z ----
#pragma unroll
  for (int c = 0; c < N; ++c) v[c] = valid ? __ldg(A.x + base + c * N2 + l) : T(0);
#pragma unroll
  for (int c = 0; c < N; ++c) X[zc + SZ * c] = v[c];
  eo_apply<N, 1>(A.S, v, v);
#pragma unroll
  for (int c = 0; c < N; ++c) Sa[zc + SZ * c] = v[c];
  __syncthreads();
  // ---- S_x ----
#pragma unroll
  for (int m = 0; m < N; ++m) v[m] = Sa[xl + SX * m];
  eo_apply<N, 1>(A.S, v, v);
#pragma unroll
  for (int m = 0; m < N; ++m) Sa[xl + SX * m] = v[m];
  __syncthreads();
  T *Y;
  if constexpr (!CONV) {
    // ---- S_y, D_y ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sa[yl + SY * m];
    eo_apply<N, 1>(A.S, v, v);
    eo_apply<N, -1>(A.D, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      Sa[yl + SY * m] = v[m];
      Sc[yl + SY * m] = g[m];
    }
    __syncthreads();
    // ---- D_x into Sb; D_z in registers ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sa[xl + SX * m];
    eo_apply<N, -1>(A.D, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) Sb[xl + SX * m] = g[m];
    T gz[N];
#pragma unroll
    for (int c = 0; c < N; ++c) v[c] = Sa[zc + SZ * c];
    eo_apply<N, -1>(A.D, v, gz);
    __syncthreads();
    // ---- quadrature points of the z column; D_z^T ----
    const T wab = A.w[a] * A.w[b];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const T wq = wab * A.w[c];
      const int s = zc + SZ * c;
      Sb[s] = A.c[0] * wq * Sb[s];
      Sc[s] = A.c[1] * wq * Sc[s];
      gz[c] = A.c[2] * wq * gz[c];
    }
    eo_apply<N, -1>(A.DT, gz, g);
#pragma unroll
    for (int c = 0; c < N; ++c) Sa[zc + SZ * c] = g[c];
    __syncthreads();
    // ---- + D_x^T ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sb[xl + SX * m];
    eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) Sa[xl + SX * m] += g[m];
    __syncthreads();
    // ---- + D_y^T, S_y^T ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sc[yl + SY * m];
    eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) g[m] += Sa[yl + SY * m];
    eo_apply<N, 1>(A.ST, g, v);
#pragma unroll
    for (int m = 0; m < N; ++m) Sa[yl + SY * m] = v[m];
    __syncthreads();
    // ---- S_x^T ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sa[xl + SX * m];
    eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m) Sa[xl + SX * m] = v[m];
    __syncthreads();
    // ---- S_z^T ----
#pragma unroll
    for (int c = 0; c < N; ++c) v[c] = Sa[zc + SZ * c];
    eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
    for (int c = 0; c < N; ++c) Sa[zc + SZ * c] = v[c];
    Y = Sa;
  } else {
    // ---- S_y; r = u JxW w; b_y / h_y D_y^T r into Sc ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sa[yl + SY * m];
    eo_apply<N, 1>(A.S, v, v);
    const T wxz = A.jxw * A.w[a] * A.w[b];
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] *= wxz * A.w[m];
    eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      Sa[yl + SY * m] = v[m];
      Sc[yl + SY * m] = A.c[1] * g[m];
    }
    __syncthreads();
    // ---- + b_x / h_x D_x^T r ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sa[xl + SX * m];
    eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
    for (int m = 0; m < N; ++m) Sc[xl + SX * m] = fma(A.c[0], g[m], Sc[xl + SX * m]);
    __syncthreads();
    // ---- + b_z / h_z D_z^T r, S_z^T ----
#pragma unroll
    for (int c = 0; c < N; ++c) v[c] = Sa[zc + SZ * c];
    eo_apply<N, -1>(A.DT, v, g);
#pragma unroll
    for (int c = 0; c < N; ++c) v[c] = fma(A.c[2], g[c], Sc[zc + SZ * c]);
    eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
    for (int c = 0; c < N; ++c) Sc[zc + SZ * c] = v[c];
    __syncthreads();
    // ---- S_y^T ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sc[yl + SY * m];
    eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m) Sc[yl + SY * m] = v[m];
    __syncthreads();
    // ---- S_x^T ----
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = Sc[xl + SX * m];
    eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
    for (int m = 0; m < N; ++m) Sc[xl + SX * m] = v[m];
    Y = Sc;
  }
  __syncthreads();

  // ---- face terms, direction by direction ----
  // face arrays: 0 right (layer p), 1 left (layer 0), 2 layer p-1 / the
  // derivative test, 3 layer 1
  constexpr int NL = CONV ? 2 : 4; // node layers read
  constexpr int NB = CONV ? 2 : 3; // face arrays mapped back
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const int so = f == 0 ? SX : f == 1 ? SY : SZ; // stride along f
    const int s1 = f == 0 ? SY : f == 1 ? SZ : SX; // along f+1 (i1)
    const int s2 = f == 0 ? SZ : f == 1 ? SX : SY; // along f+2 (i2)
    // interpolate the node layers: along i1, then along i2
    for (int t = l; t < NL * N; t += N2) {
      const int kk = t / N, i2 = t % N;
      const int layer = kk == 0 ? P : kk == 1 ? 0 : kk == 2 ? P - 1 : 1;
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = X[layer * so + i2 * s2 + j * s1];
      eo_apply<N, 1>(A.S, v, v);
#pragma unroll
      for (int j = 0; j < N; ++j) F[kk * FA + i2 * FN + j] = v[j];
    }
    __syncthreads();
    for (int t = l; t < NL * N; t += N2) {
      const int kk = t / N, q1 = t % N;
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = F[kk * FA + j * FN + q1];
      eo_apply<N, 1>(A.S, v, v);
#pragma unroll
      for (int j = 0; j < N; ++j) F[kk * FA + j * FN + q1] = v[j];
    }
    __syncthreads();
    // face quadrature point (q1, q2) = (a, b)
    {
      const T W = A.fw[f] * (A.w[b] * A.w[a]);
      const T uR = F[fq], uL = F[FA + fq];
      if constexpr (CONV) {
        const T bn = A.bn[f];
        const T flux = T(0.5) * (bn * (uR + uL) + fabs(bn) * (uR - uL));
        F[fq] = flux * W;
        F[FA + fq] = -(flux * W);
      } else {
        const T nR = A.hd * (F[2 * FA + fq] - uR), nL = A.hd * (F[3 * FA + fq] - uL);
        const T avg = T(0.5) * (uR + uL);
        const T gs = A.ij[f] * nR + A.ij[f] * nL;
        const T vv = W * (avg * T(2) * A.sigma[f] - gs * T(0.5));
        F[fq] = -vv;
        F[FA + fq] = vv;
        F[2 * FA + fq] = W * A.ij[f] * avg;
      }
    }
    __syncthreads();
    // back to the face nodes: S^T for the value tests, S for the derivative test
    for (int t = l; t < NB * N; t += N2) {
      const int kk = t / N, r = t % N;
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = F[kk * FA + r * FN + j];
      if (kk == 2) eo_apply<N, 1>(A.S, v, v);
      else eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
      for (int j = 0; j < N; ++j) F[kk * FA + r * FN + j] = v[j];
    }
    __syncthreads();
    for (int t = l; t < NB * N; t += N2) {
      const int kk = t / N, q1 = t % N;
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = F[kk * FA + j * FN + q1];
      if (kk == 2) eo_apply<N, 1>(A.S, v, v);
      else eo_apply<N, 1>(A.ST, v, v);
#pragma unroll
      for (int j = 0; j < N; ++j) F[kk * FA + j * FN + q1] = v[j];
    }
    __syncthreads();
    // inject: one thread per face node, right face first, then left
    {
      const int off = b * s2 + a * s1;
      if constexpr (CONV) {
        Y[P * so + off] += F[fq];
        Y[off] += F[FA + fq];
      } else {
        const T td = F[2 * FA + fq];
        Y[P * so + off] += F[fq] - td * A.hd;
        Y[(P - 1) * so + off] += A.hd * td;
        Y[off] += F[FA + fq] - td * A.hd;
        Y[so + off] += A.hd * td;
      }
    }
    __syncthreads();
  }

  if (valid) {
#pragma unroll
    for (int c = 0; c < N; ++c) A.y[base + c * N2 + l] = Y[zc + SZ * c];
  }
}

template <int N, typename T>
int faces_impl(const sf_op *op, int nrhs, const T *x, T *y, cudaStream_t st)
{
  using Cfg = FacesCfg<N, T>;
  const bool conv = op->desc.kind == SF_OP_CONVECTION_FACES;
  FacesArgs<N, T> A{};
  A.S = eo_of<N, T>(op->shape.S, false);
  A.ST = eo_of<N, T>(op->shape.S, true);
  A.D = eo_of<N, T>(op->shape.D, false);
  A.DT = eo_of<N, T>(op->shape.D, true);
  for (int q = 0; q < N; ++q) A.w[q] = T(op->shape.wq[q]);
  const double jxw = op->h[0] * op->h[1] * op->h[2];
  for (int d = 0; d < 3; ++d) {
    const double ij = 1.0 / op->h[d];
    A.c[d] = conv ? T(op->desc.velocity[d] * ij) : T(jxw * ij * ij);
    A.fw[d] = T(-(jxw / op->h[d]));
    A.ij[d] = T(ij);
    A.sigma[d] = T(double(N * N) * ij);
    A.bn[d] = T(op->desc.velocity[d]);
  }
  A.jxw = T(jxw);
  A.hd = T(op->shape.hermite_d0);
  A.n_cells = op->n_cells;
  A.x = x;
  A.y = y;
  void (*kern)(const FacesArgs<N, T>) = conv ? cell_faces_kernel<N, T, true> : cell_faces_kernel<N, T, false>;
  SF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM));
  const long long blocks = (op->n_cells + Cfg::CPB - 1) / Cfg::CPB;
  kern<<<dim3((unsigned)blocks, (unsigned)nrhs), dim3(Cfg::CPB * N * N), Cfg::SMEM, st>>>(A);
  SF_CUDA_TRY(cudaGetLastError());
  return SF_OK;
}

template <int N>
int faces_n(const sf_op *op, int prec, int nrhs, const void *x, void *y, cudaStream_t st)
{
  if (prec == SF_FP64) return faces_impl<N, double>(op, nrhs, (const double *)x, (double *)y, st);
  return faces_impl<N, float>(op, nrhs, (const float *)x, (float *)y, st);
}

} // namespace

int launch_cell_faces(const sf_op *op, int prec, int nrhs, const void *x, void *y, cudaStream_t st)
{
  switch (op->n) {
  case 2: return faces_n<2>(op, prec, nrhs, x, y, st);
  case 3: return faces_n<3>(op, prec, nrhs, x, y, st);
  case 4: return faces_n<4>(op, prec, nrhs, x, y, st);
  case 5: return faces_n<5>(op, prec, nrhs, x, y, st);
  case 6: return faces_n<6>(op, prec, nrhs, x, y, st);
  case 7: return faces_n<7>(op, prec, nrhs, x, y, st);
  case 8: return faces_n<8>(op, prec, nrhs, x, y, st);
  case 9: return faces_n<9>(op, prec, nrhs, x, y, st);
  default: set_error("unsupported degree"); return SF_ERR_UNSUPPORTED;
  }
}

} // namespace sf
