// Adjoint viscosity gradient (no counterpart in the reference):
//   g_c = -int_c 2 eta eps(u) : eps(lambda) dx      (deviatoric eps if compressible)
// = d/d ln(eta_c) of lambda . (F - K(eta) u) for a cellwise viscosity. With u the
// forward solution and lambda the adjoint solution (K lambda = dJ/du; K is
// symmetric) this is dJ/d ln(eta_c). One velocity component per thread, `dim`
// threads per cell, as in the forward cell kernels; each cell writes only its
// own entry.
#include "ops.cuh"

namespace gb {

template <int dim>
__global__ void __launch_bounds__(128) adjoint_gradient_kernel(LevelView<double> L, int colour, int colour_begin,
                                                                int colour_count, const double* __restrict__ u,
                                                                const double* __restrict__ lam,
                                                                double* __restrict__ grad) {
  pdl_wait();
  using T = double;
  constexpr int nv = Shape<dim>::nv, cpw = Shape<dim>::cpw;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int grp = lane / dim;
  int comp = lane - grp * dim;
  bool active = grp < cpw;
  if (!active) { grp = cpw - 1; comp = 0; }
  const unsigned lane_base = grp * dim;
  const int idx = warp * cpw + grp;
  active = active && idx < colour_count;
  int cell = 0;
  StructuredCell<T, dim> sc{};
  if (L.structured) {
    bool v;
    structured_cell<T, dim>(L, colour, active ? idx : 0, cell, sc, v);
    active = active && v;
  } else {
    cell = colour_begin + (active ? idx : 0);
  }
  T U[nv], W[nv];
#pragma unroll
  for (int n = 0; n < nv; ++n) {
    T a = T(0), b = T(0);
    if (active) {
      if (L.structured) {
        if (!structured_zero<T, dim>(L, sc, comp, n)) {
          const int g = comp * L.n_nodes + sc.node0 + structured_node_offset<dim>(L.Nn, n);
          a = u[g];
          b = lam[g];
        }
      } else {
        const int e = L.cdu[(size_t)cell * dim * nv + comp * nv + n];
        a = gather_general(u, e, L.lptr, L.lcol, L.lw);
        b = gather_general(lam, e, L.lptr, L.lcol, L.lw);
      }
    }
    U[n] = a;
    W[n] = b;
  }
  T box[4] = {T(0), T(0), T(0), T(0)};
  if (L.geom == GEOM_BOX && active)
#pragma unroll
    for (int d = 0; d <= dim; ++d) box[d] = L.gbox[(size_t)cell * (dim + 1) + d];
  T eta_cell = T(1);
  const T* eta_q = nullptr;
  if (active) {
    if (L.eta_n == 1) eta_cell = L.eta[cell];
    else eta_q = L.eta + (size_t)cell * L.eta_n;
  }
  interpolate<T, dim, false>(U);
  interpolate<T, dim, false>(W);
  T acc = T(0);
  static_for<nv>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    QGeom<T, dim> G;
    if (L.geom == GEOM_CART) {
#pragma unroll
      for (int d = 0; d < dim; ++d)
#pragma unroll
        for (int e = 0; e < dim; ++e) G.iJ[d][e] = d == e ? L.inv_h[d] : T(0);
      G.jxw = L.det * T(qweight<dim, q>());
    } else {
      qgeom<T, dim, q>(L, cell, box, G);
    }
    const T eta = eta_q ? eta_q[q] : eta_cell;
    T gu[3] = {0, 0, 0}, gl[3] = {0, 0, 0}, ru[3], rl[3];
    ru[0] = colloc_d<T, dim, q, 0>(U);
    ru[1] = colloc_d<T, dim, q, 1>(U);
    rl[0] = colloc_d<T, dim, q, 0>(W);
    rl[1] = colloc_d<T, dim, q, 1>(W);
    if constexpr (dim == 3) {
      ru[2] = colloc_d<T, dim, q, 2>(U);
      rl[2] = colloc_d<T, dim, q, 2>(W);
    }
#pragma unroll
    for (int e = 0; e < dim; ++e) {
      T a = 0, b = 0;
#pragma unroll
      for (int d = 0; d < dim; ++d) {
        a += ru[d] * G.iJ[d][e];
        b += rl[d] * G.iJ[d][e];
      }
      gu[e] = a;
      gl[e] = b;
    }
    // eps rows of this component; off-diagonal partners from the sibling threads
    T eu[3], el[3];
    T divu = 0, divl = 0;
    if constexpr (dim == 3) {
      const int k1 = (comp + 1) % 3, k2 = (comp + 2) % 3;
      const int l1 = lane_base + k1, l2 = lane_base + k2;
      const T ru1 = __shfl_sync(full, sel3(gu[0], gu[1], gu[2], k2), l1);
      const T ru2 = __shfl_sync(full, sel3(gu[0], gu[1], gu[2], k1), l2);
      const T rl1 = __shfl_sync(full, sel3(gl[0], gl[1], gl[2], k2), l1);
      const T rl2 = __shfl_sync(full, sel3(gl[0], gl[1], gl[2], k1), l2);
      const T uc = sel3(gu[0], gu[1], gu[2], comp), lc = sel3(gl[0], gl[1], gl[2], comp);
      eu[0] = uc;
      eu[1] = 0.5 * (sel3(gu[0], gu[1], gu[2], k1) + ru1);
      eu[2] = 0.5 * (sel3(gu[0], gu[1], gu[2], k2) + ru2);
      el[0] = lc;
      el[1] = 0.5 * (sel3(gl[0], gl[1], gl[2], k1) + rl1);
      el[2] = 0.5 * (sel3(gl[0], gl[1], gl[2], k2) + rl2);
      if (L.compressible) {
        divu = uc + __shfl_sync(full, uc, l1) + __shfl_sync(full, uc, l2);
        divl = lc + __shfl_sync(full, lc, l1) + __shfl_sync(full, lc, l2);
      }
    } else {
      const int o = lane_base + (1 - comp);
      const T ru1 = __shfl_sync(full, comp == 0 ? gu[1] : gu[0], o);
      const T rl1 = __shfl_sync(full, comp == 0 ? gl[1] : gl[0], o);
      const T uc = comp == 0 ? gu[0] : gu[1], lc = comp == 0 ? gl[0] : gl[1];
      eu[0] = uc;
      eu[1] = 0.5 * ((comp == 0 ? gu[1] : gu[0]) + ru1);
      el[0] = lc;
      el[1] = 0.5 * ((comp == 0 ? gl[1] : gl[0]) + rl1);
      eu[2] = el[2] = 0;
      if (L.compressible) {
        divu = uc + __shfl_sync(full, uc, o);
        divl = lc + __shfl_sync(full, lc, o);
      }
    }
    T contr = 0;
#pragma unroll
    for (int e = 0; e < dim; ++e) contr += eu[e] * el[e];
    if (L.compressible) contr -= divu * el[0] / T(3);  // (eps(u) - div u I/3) : eps(l), row part
    acc += T(2) * eta * G.jxw * contr;
  });
  T tot = acc;
#pragma unroll
  for (int o = 1; o < dim; ++o) tot += __shfl_sync(full, acc, lane_base + (comp + o) % dim);
  if (active && comp == 0) grad[cell] = -tot;
}

void launch_adjoint_gradient_impl(const LevelView<double>& L, int colour, int begin, int count, const double* u,
                                  const double* lam, double* grad, cudaStream_t s) {
  if (count <= 0) return;
  const int threads = 128;
  if (L.dim == 3) {
    const int g = ceil_div(count, (threads / 32) * Shape<3>::cpw);
    adjoint_gradient_kernel<3><<<g, threads, 0, s>>>(L, colour, begin, count, u, lam, grad);
  } else {
    const int g = ceil_div(count, (threads / 32) * Shape<2>::cpw);
    adjoint_gradient_kernel<2><<<g, threads, 0, s>>>(L, colour, begin, count, u, lam, grad);
  }
}

}  // namespace gb
