// 1D tables of the Q2-Q1 tensor-product basis at the 3-point Gauss rule on [0,1].
//
// Velocity: FE_Q(2), nodes {0, 1/2, 1}; pressure: FE_Q(1), nodes {0, 1};
// quadrature: QGauss(3) (QGauss<1>(degree_v+1) of
// source/simulator/solver/stokes_matrix_free_local_smoothing.cc:1657).
//
// The cell kernels work in collocation form: nodal values are first
// interpolated to the Gauss points with S (values of the Q2 basis at the
// points), and derivatives are then taken with the collocation matrix D of the
// Lagrange basis on the Gauss points themselves (exact, since a quadratic is
// determined by its values at three points).
#pragma once
#include <type_traits>
#include <utility>

namespace gb {
namespace fe {

constexpr double SQ15 = 3.8729833462074168851792653997824;  // sqrt(15)

// S(q, n) = phi_n(g_q), g = 1/2 + {-1, 0, 1} sqrt(15)/10
__host__ __device__ constexpr double Sv(int q, int n) {
  return q == 1 ? (n == 1 ? 1.0 : 0.0)
                : (n == 1 ? 0.4 : (((q == 0) == (n == 0)) ? 0.3 + SQ15 / 10 : 0.3 - SQ15 / 10));
}

// D(q, a) = l_a'(g_q), l_a the Lagrange polynomials on the Gauss points
__host__ __device__ constexpr double Dv(int q, int a) {
  return q == 0 ? (a == 0 ? -SQ15 : a == 1 ? 4.0 * SQ15 / 3.0 : -SQ15 / 3.0)
       : q == 1 ? (a == 0 ? -SQ15 / 3.0 : a == 1 ? 0.0 : SQ15 / 3.0)
                : (a == 0 ? SQ15 / 3.0 : a == 1 ? -4.0 * SQ15 / 3.0 : SQ15);
}

// Gauss weights on [0,1]
__host__ __device__ constexpr double Wv(int q) { return q == 1 ? 8.0 / 18.0 : 5.0 / 18.0; }

// P1(q, n) = psi_n(g_q) for the Q1 basis {1-x, x}
__host__ __device__ constexpr double P1v(int q, int n) {
  return q == 1 ? 0.5 : (((q == 0) == (n == 0)) ? 0.5 + SQ15 / 10 : 0.5 - SQ15 / 10);
}

__host__ __device__ constexpr int pow3(int d) { return d == 0 ? 1 : 3 * pow3(d - 1); }
__host__ __device__ constexpr int pow2(int d) { return d == 0 ? 1 : 2 * pow2(d - 1); }

}  // namespace fe

// Compile-time loop: f(std::integral_constant<int, i>) for i = 0 .. N-1.
template <int I, int N, class F>
__host__ __device__ __forceinline__ void static_for_impl(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for_impl<I + 1, N>(f);
  }
}
template <int N, class F>
__host__ __device__ __forceinline__ void static_for(F&& f) {
  static_for_impl<0, N>(f);
}

}  // namespace gb
