// sf_tables.h -- host construction of the even-odd device tables.
#pragma once

#include "sf_device.cuh"
#include "sf_internal.h"

namespace sf {

// even-odd split of an n x n matrix given by m(i, j) (see sf_device.cuh)
template <int N, typename T, typename F>
EOMat<N, T> make_eo(F m)
{
  EOMat<N, T> r{};
  constexpr int H = N / 2;
  for (int i = 0; i < H; ++i)
    for (int j = 0; j < H; ++j) {
      r.e[i][j] = T(0.5 * (m(i, j) + m(i, N - 1 - j)));
      r.o[i][j] = T(0.5 * (m(i, j) - m(i, N - 1 - j)));
    }
  if (N % 2 == 1) {
    for (int i = 0; i < H; ++i) {
      r.mc[i] = T(m(i, H));
      r.mr[i] = T(m(H, i));
    }
    r.mm = T(m(H, H));
  }
  return r;
}

template <int N, typename T>
EOMat<N, T> eo_of(const double (&M)[kMaxN][kMaxN], bool transpose)
{
  if (transpose) return make_eo<N, T>([&](int i, int j) { return M[j][i]; });
  return make_eo<N, T>([&](int i, int j) { return M[i][j]; });
}

} // namespace sf
