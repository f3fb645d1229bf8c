// The outer Stokes operator with Newton-derivative and prescribed-dilation
// terms (StokesOperator::local_apply, source/simulator/solver/
// matrix_free_operators.cc:400-538), for the FGMRES product of a Newton solve.
//
// Per quadrature point, with eps = sym grad u, div = tr eps, p the (scaled)
// pressure, E the linearisation point's strain rate, D = deta/deps and
// dp = deta/dp (both already multiplied by the derivative scaling factor), the
// velocity test function sees
//   2 eta eps - s p I                     (- 2 eta / 3 div I if deviatoric)
//   + 2 E (D : eps) + 2 E dp p            (Newton, plain)
//   + E (D : eps) + D (E : eps) + 2 E dp p   (Newton, symmetrised)
//   deviatoric: - 2/3 tr(E) (D : eps) I (plain), or
//               - 1/3 D tr(E) div - 1/3 tr(E) (D : eps) I (symmetrised)
// and the pressure test function
//   - s div  - s^2 L p  + s (DD : eps + dpd s p)   (dilation; the last term with Newton)
// where L, DD, dpd are the dilation tables. "Averaged" Newton factors replace
// D : eps and dp p by their sums over the cell's points, and (symmetrised)
// E : eps and tr(E) div by JxW-weighted sums divided by the point's JxW.
// "Deviatoric" = compressible or prescribed dilation.
//
// Layout as velocity_cell_kernel: one velocity component per thread, dim threads
// per cell; the symmetric gradient's off-diagonal entries and every full
// contraction (D : eps, E : eps, div) are completed across the cell's threads by
// warp shuffles. Output: the per-cell contributions of the two-pass operator, in
// the layout the level's gather reads.
#include "ops.cuh"

namespace gb {
namespace {

template <int dim>
__device__ __forceinline__ int sym_slot(int a, int b) {
  if (a == b) return a;
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return dim == 2 ? 2 : (lo == 0 ? (hi == 1 ? 3 : 4) : 5);
}

template <typename T, int dim>
__device__ __forceinline__ T cell_sum(T v, int comp, int lb) {
  const unsigned full = 0xffffffffu;
  T t = v;
#pragma unroll
  for (int o = 1; o < dim; ++o) t += __shfl_sync(full, v, lb + (comp + o) % dim);
  return t;
}

template <typename T, int dim>
__global__ void __launch_bounds__(128) newton_stokes_cell_kernel(LevelView<T> L, NewtonView<T> N,
                                                                  const T* __restrict__ src_u,
                                                                  const T* __restrict__ src_p, T* __restrict__ Eu,
                                                                  T* __restrict__ Ep, int slot_major) {
  pdl_wait();
  constexpr int nv = Shape<dim>::nv, np = Shape<dim>::np, nq = Shape<dim>::nq, cpw = Shape<dim>::cpw;
  constexpr int ns = dim == 3 ? 6 : 3;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int grp = lane / dim;
  int comp = lane - grp * dim;
  bool active = grp < cpw;
  if (!active) { grp = cpw - 1; comp = 0; }
  const int lb = grp * dim;
  const int idx = warp * cpw + grp;
  active = active && idx < L.n_cells;
  const int cell = active ? idx : 0;
  StructuredCell<T, dim> sc{};
  if (L.structured) structured_cell_lex<T, dim>(L, cell, sc);
  T box[4] = {T(0), T(0), T(0), T(0)};
  if (L.geom == GEOM_BOX && active)
#pragma unroll
    for (int d = 0; d <= dim; ++d) box[d] = L.gbox[(size_t)cell * (dim + 1) + d];
  T U[nv], V[nv], P[np], YP[np];
#pragma unroll
  for (int n = 0; n < nv; ++n) {
    T v = T(0);
    if (active) {
      if (L.structured) {
        if (!structured_zero<T, dim>(L, sc, comp, n))
          v = src_u[comp * L.n_nodes + sc.node0 + structured_node_offset<dim>(L.Nn, n)];
      } else {
        v = gather_general(src_u, L.cdu[(size_t)cell * dim * nv + comp * nv + n], L.lptr, L.lcol, L.lw);
      }
    }
    U[n] = v;
    V[n] = T(0);
  }
#pragma unroll
  for (int n = 0; n < np; ++n) {
    T v = T(0);
    if (active) {
      if (L.structured) v = src_p[sc.pnode0 + structured_pnode_offset<dim>(L.Np, n)];
      else v = gather_general(src_p, L.cdp[(size_t)cell * np + n], L.plptr, L.plcol, L.plw);
    }
    P[n] = v;
    YP[n] = T(0);
  }
  interpolate<T, dim, false>(U);
  const T eta_cell = L.eta_n == 1 ? L.eta[cell] : T(0);
  const T* __restrict__ eta_q = L.eta_n == 1 ? nullptr : L.eta + (size_t)cell * L.eta_n;
  const T s = L.s;
  const bool deviatoric = L.compressible || N.dilation;
  const size_t cq0 = (size_t)cell * nq;

  // real-space gradient row g[e] = d u_comp / d x_e, the row eps[comp][e], div and p at point q
  auto point = [&](auto qc, QGeom<T, dim>& G, T (&eps)[3], T& div, T& pq) {
    constexpr int q = decltype(qc)::value;
    if (L.geom == GEOM_CART) {
#pragma unroll
      for (int d = 0; d < dim; ++d)
#pragma unroll
        for (int e = 0; e < dim; ++e) G.iJ[d][e] = d == e ? L.inv_h[d] : T(0);
      G.jxw = L.det * T(qweight<dim, q>());
    } else {
      qgeom<T, dim, q>(L, cell, box, G);
    }
    T gr[3] = {T(0), T(0), T(0)}, g[3] = {T(0), T(0), T(0)};
    gr[0] = colloc_d<T, dim, q, 0>(U);
    gr[1] = colloc_d<T, dim, q, 1>(U);
    if constexpr (dim == 3) gr[2] = colloc_d<T, dim, q, 2>(U);
#pragma unroll
    for (int e = 0; e < dim; ++e) {
      T t = T(0);
#pragma unroll
      for (int d = 0; d < dim; ++d) t += gr[d] * G.iJ[d][e];
      g[e] = t;
    }
    // eps[comp][e] = (d_e u_comp + d_comp u_e) / 2: thread e sends d_comp u_e
#pragma unroll
    for (int o = 1; o < dim; ++o) {
      const int e = (comp + o) % dim;         // the sibling this thread receives from
      const int ask = (comp + dim - o) % dim;  // the direction the thread comp - o asks this thread for
      const T send = dim == 3 ? sel3(g[0], g[1], g[2], ask) : (ask == 0 ? g[0] : g[1]);
      const T r = __shfl_sync(full, send, lb + e);
      const T ge = dim == 3 ? sel3(g[0], g[1], g[2], e) : (e == 0 ? g[0] : g[1]);
      eps[e] = T(0.5) * (ge + r);
    }
    const T gcc = dim == 3 ? sel3(g[0], g[1], g[2], comp) : (comp == 0 ? g[0] : g[1]);
    eps[comp] = gcc;
    div = cell_sum<T, dim>(gcc, comp, lb);
    pq = T(0);
    static_for<np>([&](auto nc) {
      constexpr int n = decltype(nc)::value;
      pq += T(psi_at<dim, q, n>()) * P[n];
    });
  };
  auto row_dot = [&](const T* t, const T (&eps)[3]) {
    T v = T(0);
#pragma unroll
    for (int e = 0; e < dim; ++e) v += t[sym_slot<dim>(comp, e)] * eps[e];
    return v;
  };
  auto trace = [&](const T* t) {
    T v = T(0);
#pragma unroll
    for (int e = 0; e < dim; ++e) v += t[e];
    return v;
  };

  // averaged Newton factors: sums over the cell's points (matrix_free_operators.cc:411-445)
  T avg_a = T(0), avg_bp = T(0), avg_eu = T(0), avg_th = T(0);
  if (N.newton && N.average) {
    T pa = T(0), pe = T(0);
    static_for<nq>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      QGeom<T, dim> G;
      T eps[3], div, pq;
      point(qc, G, eps, div, pq);
      const T* Eq = N.E + (cq0 + q) * ns;
      const T* Dq = N.D + (cq0 + q) * ns;
      pa += row_dot(Dq, eps);
      if (N.symmetrize) pe += G.jxw * row_dot(Eq, eps);
      avg_bp += N.dp[cq0 + q] * pq;
      if (N.symmetrize && deviatoric) avg_th += G.jxw * trace(Eq) * div;
    });
    avg_a = cell_sum<T, dim>(pa, comp, lb);
    avg_eu = cell_sum<T, dim>(pe, comp, lb);
  }

  static_for<nq>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    QGeom<T, dim> G;
    T eps[3], div, pq;
    point(qc, G, eps, div, pq);
    const T eta = eta_q ? eta_q[q] : eta_cell;
    T F[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int e = 0; e < dim; ++e) F[e] = T(2) * eta * eps[e];
    F[comp] -= s * pq;
    if (deviatoric) F[comp] -= T(2) * eta / T(3) * div;
    T ptest = -s * div;
    if (N.dilation) ptest -= s * s * N.lhs[cq0 + q] * pq;
    if (N.newton) {
      const T* Eq = N.E + (cq0 + q) * ns;
      const T* Dq = N.D + (cq0 + q) * ns;
      const T a = N.average ? avg_a : cell_sum<T, dim>(row_dot(Dq, eps), comp, lb);
      const T bp = N.average ? avg_bp : N.dp[cq0 + q] * pq;
      T ee = T(0);
      if (N.symmetrize) ee = N.average ? avg_eu / G.jxw : cell_sum<T, dim>(row_dot(Eq, eps), comp, lb);
      const T trE = trace(Eq);
#pragma unroll
      for (int e = 0; e < dim; ++e) {
        const T Ece = Eq[sym_slot<dim>(comp, e)], Dce = Dq[sym_slot<dim>(comp, e)];
        F[e] += N.symmetrize ? Ece * a + Dce * ee : T(2) * Ece * a;
        F[e] += T(2) * Ece * bp;
      }
      if (deviatoric) {
        if (N.symmetrize) {
          const T th = N.average ? avg_th / G.jxw : trE * div;
#pragma unroll
          for (int e = 0; e < dim; ++e) F[e] -= T(1.0 / 3.0) * Dq[sym_slot<dim>(comp, e)] * th;
          F[comp] -= T(1.0 / 3.0) * trE * a;
        } else {
          F[comp] -= T(2.0 / 3.0) * trE * a;
        }
        if (N.dilation) {
          const T* DDq = N.DD + (cq0 + q) * ns;
          const T dde = cell_sum<T, dim>(row_dot(DDq, eps), comp, lb);
          ptest += (dde + N.dpd[cq0 + q] * s * pq) * s;
        }
      }
    }
    // reference-direction flux R[d] = JxW sum_e F[e] invJ[d][e]
    T R[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int d = 0; d < dim; ++d) {
      T t = T(0);
#pragma unroll
      for (int e = 0; e < dim; ++e) t += F[e] * G.iJ[d][e];
      R[d] = t * G.jxw;
    }
    colloc_dT<T, dim, q, 0>(V, R[0]);
    colloc_dT<T, dim, q, 1>(V, R[1]);
    if constexpr (dim == 3) colloc_dT<T, dim, q, 2>(V, R[2]);
    // the pressure test is the same in all threads of the cell: thread 0 adds it
    const T f = comp == 0 ? ptest * G.jxw : T(0);
    static_for<np>([&](auto nc) {
      constexpr int n = decltype(nc)::value;
      YP[n] += T(psi_at<dim, q, n>()) * f;
    });
  });
  interpolate<T, dim, true>(V);
  if (active) {
#pragma unroll
    for (int n = 0; n < nv; ++n) {
      const int slot = comp * nv + n;
      Eu[slot_major ? (size_t)slot * L.n_cells + cell : (size_t)cell * dim * nv + slot] = V[n];
    }
  }
#pragma unroll
  for (int n = 0; n < np; ++n) YP[n] = cell_sum<T, dim>(YP[n], comp, lb);
  if (active) {
#pragma unroll
    for (int n = 0; n < np; ++n)
      if (n % dim == comp) Ep[slot_major ? (size_t)n * L.n_cells + cell : (size_t)cell * np + n] = YP[n];
  }
}

template <typename T>
void launch(const LevelView<T>& L, const NewtonView<T>& N, const T* su, const T* sp, T* Eu, T* Ep, bool slot_major,
            cudaStream_t s) {
  if (L.n_cells <= 0) return;
  if (L.dim == 3)
    newton_stokes_cell_kernel<T, 3><<<ceil_div(L.n_cells, 4 * Shape<3>::cpw), 128, 0, s>>>(L, N, su, sp, Eu, Ep,
                                                                                          slot_major);
  else
    newton_stokes_cell_kernel<T, 2><<<ceil_div(L.n_cells, 4 * Shape<2>::cpw), 128, 0, s>>>(L, N, su, sp, Eu, Ep,
                                                                                          slot_major);
}

}  // namespace

template <>
void launch_newton_stokes<double>(const LevelView<double>& L, const NewtonView<double>& N, const double* su,
                                  const double* sp, double* Eu, double* Ep, bool slot_major, cudaStream_t s) {
  launch<double>(L, N, su, sp, Eu, Ep, slot_major, s);
}
template <>
void launch_newton_stokes<float>(const LevelView<float>& L, const NewtonView<float>& N, const float* su,
                                 const float* sp, float* Eu, float* Ep, bool slot_major, cudaStream_t s) {
  launch<float>(L, N, su, sp, Eu, Ep, slot_major, s);
}

}  // namespace gb
