// Matrix-free cell kernels of the Q2-Q1 Stokes operators (sm_103a).
//
// Physics per quadrature point follows
// source/simulator/solver/matrix_free_operators.cc:
//   StokesOperator::local_apply   :376-547  (velocity test 2 eta eps(u) - s p I,
//                                            pressure test -s div u)
//   BTBlockOperator::local_apply  :668-701  (-s p I : eps(v))
//   MassMatrixOperator            :787-845  (s^2 / eta p q)
//   ABlockOperator                :974-1009 (2 eta eps(u), deviatoric if compressible)
// Constrained rows are the identity and constrained columns are resolved
// through the constraint lines, as MatrixFreeOperators::Base::vmult does.
//
// GB300 mapping (not the reference's SIMD-over-cells layout): one velocity
// component per thread, `dim` threads per cell (10 cells per warp in 3D, 16 in
// 2D). Each thread keeps the 3^dim nodal values of its component in registers,
// interpolates them to the Gauss points (collocation), forms its row of the
// velocity gradient, and exchanges the off-diagonal entries it needs for the
// symmetric gradient with its sibling threads through warp shuffles. The cells
// of one launch form one colour of a conflict-free colouring, so the scatter
// is a plain read-modify-write and every result is bit-reproducible.
#pragma once
#include "common.cuh"
#include "fe_tables.cuh"

namespace gb {

enum OpKind { OPK_STOKES = 0, OPK_A = 1, OPK_BT = 2, OPK_MASS = 3 };
enum GeomKind { GEOM_CART = 0, GEOM_BOX = 1, GEOM_TABLE = 2 };

// Device view of one level, passed by value to every kernel.
template <typename T>
struct LevelView {
  int dim;
  int deg;        // velocity degree: 2 (Q2-Q1) or 3 (Q3-Q2, general levels only)
  int n_cells, n_u, n_p;
  int structured;
  // structured box levels (internal lexicographic numbering, components blocked)
  int nc[3];      // cells per direction
  int Nn[3];      // Q2 nodes per direction
  int Np[3];      // Q1 nodes per direction
  int n_nodes;    // Q2 nodes
  uint32_t zero_faces;  // bit (2*d+side)*3+comp: component comp is zero on that face
  T inv_h[3];     // 1/h per direction
  T det;          // cell volume
  // general levels (cells sorted by colour)
  const int* cdu;       // [n_cells][dim*3^dim]  >=0 dof, -1 zero, <=-2 line -(v+2)
  const int* cdp;       // [n_cells][2^dim]
  const int* lptr;      // velocity lines
  const int* lcol;
  const T* lw;
  const int* plptr;     // pressure lines
  const int* plcol;
  const T* plw;
  int geom;             // GeomKind
  const T* gbox;        // [n_cells][dim+1]: 1/h_d, det
  const T* gtab;        // [n_cells][nq][dim*dim+1]: invJ (dxi_d/dx_e at [d*dim+e]), JxW/w_q
  const T* eta;         // [n_cells][eta_n]
  int eta_n;
  const T* Mp;          // per-cell pressure mass matrices of the level table ([cell][np][np], internal
                        // order), or null: the mass cell pass integrates at the quadrature points
  T s;                  // pressure scaling
  int compressible;
};

template <int dim>
struct Shape {
  static constexpr int nv = fe::pow3(dim);
  static constexpr int np = fe::pow2(dim);
  static constexpr int nq = nv;
  static constexpr int tpc = dim;                 // threads per cell
  static constexpr int cpw = 32 / dim;            // cells per warp
};

// ---------------------------------------------------------------------------
// 1D sweeps over registers (fully unrolled; matrices are compile-time).
template <typename T, int dim, int dir, bool transpose>
__device__ __forceinline__ void sweep_S(T* x) {
  constexpr int st = fe::pow3(dir);
#pragma unroll
  for (int b = 0; b < fe::pow3(dim); ++b) {
    if ((b / st) % 3 != 0) continue;
    const T a0 = x[b], a1 = x[b + st], a2 = x[b + 2 * st];
    if (!transpose) {
      x[b] = T(fe::Sv(0, 0)) * a0 + T(fe::Sv(0, 1)) * a1 + T(fe::Sv(0, 2)) * a2;
      x[b + st] = a1;
      x[b + 2 * st] = T(fe::Sv(2, 0)) * a0 + T(fe::Sv(2, 1)) * a1 + T(fe::Sv(2, 2)) * a2;
    } else {
      x[b] = T(fe::Sv(0, 0)) * a0 + T(fe::Sv(2, 0)) * a2;
      x[b + st] = T(fe::Sv(0, 1)) * a0 + a1 + T(fe::Sv(2, 1)) * a2;
      x[b + 2 * st] = T(fe::Sv(0, 2)) * a0 + T(fe::Sv(2, 2)) * a2;
    }
  }
}

template <typename T, int dim, bool transpose>
__device__ __forceinline__ void interpolate(T* x) {
  sweep_S<T, dim, 0, transpose>(x);
  sweep_S<T, dim, 1, transpose>(x);
  if constexpr (dim == 3) sweep_S<T, dim, 2, transpose>(x);
}

// derivative along `dir` at Gauss point q of a collocated field. The middle
// point's middle coefficient is zero; its term is left out at compile time (the
// compiler may not drop a multiplication by 0.0 itself), which changes no
// result for finite inputs.
template <typename T, int dim, int q, int dir>
__device__ __forceinline__ T colloc_d(const T* x) {
  constexpr int st = fe::pow3(dir);
  constexpr int qd = (q / st) % 3;
  constexpr int b = q - qd * st;
  if constexpr (qd == 1) return T(fe::Dv(1, 0)) * x[b] + T(fe::Dv(1, 2)) * x[b + 2 * st];
  else return T(fe::Dv(qd, 0)) * x[b] + T(fe::Dv(qd, 1)) * x[b + st] + T(fe::Dv(qd, 2)) * x[b + 2 * st];
}
template <typename T, int dim, int q, int dir>
__device__ __forceinline__ void colloc_dT(T* x, T r) {
  constexpr int st = fe::pow3(dir);
  constexpr int qd = (q / st) % 3;
  constexpr int b = q - qd * st;
  x[b] += T(fe::Dv(qd, 0)) * r;
  if constexpr (qd != 1) x[b + st] += T(fe::Dv(qd, 1)) * r;
  x[b + 2 * st] += T(fe::Dv(qd, 2)) * r;
}

template <int dim, int q>
__host__ __device__ constexpr double qweight() {
  return dim == 2 ? fe::Wv(q % 3) * fe::Wv(q / 3) : fe::Wv(q % 3) * fe::Wv((q / 3) % 3) * fe::Wv(q / 9);
}
template <int dim, int q, int n>
__host__ __device__ constexpr double psi_at() {
  double v = fe::P1v(q % 3, n & 1) * fe::P1v((q / 3) % 3, (n >> 1) & 1);
  if (dim == 3) v *= fe::P1v(q / 9, (n >> 2) & 1);
  return v;
}

// select among values indexed relative to the thread's component
template <typename T>
__device__ __forceinline__ T sel3(T r0, T r1, T r2, int k) { return k == 0 ? r0 : (k == 1 ? r1 : r2); }

// ---------------------------------------------------------------------------
// DoF access
template <typename T, int dim>
struct StructuredCell {
  int i, j, k;
  int node0;  // Q2 node index of the cell's first node
  int pnode0;
};

template <typename T, int dim>
__device__ __forceinline__ void structured_cell(const LevelView<T>& L, int colour, int idx, int& cell,
                                                StructuredCell<T, dim>& sc, bool& valid) {
  const int ci = colour & 1, cj = (colour >> 1) & 1, ck = (colour >> 2) & 1;
  const int mx = (L.nc[0] - ci + 1) >> 1, my = (L.nc[1] - cj + 1) >> 1;
  const int mz = dim == 3 ? (L.nc[2] - ck + 1) >> 1 : 1;
  valid = idx < mx * my * mz;
  const int a = idx % mx, b = (idx / mx) % my, c = idx / (mx * my);
  sc.i = 2 * a + ci;
  sc.j = 2 * b + cj;
  sc.k = dim == 3 ? 2 * c + ck : 0;
  cell = (sc.k * L.nc[1] + sc.j) * L.nc[0] + sc.i;
  sc.node0 = (2 * sc.k * L.Nn[1] + 2 * sc.j) * L.Nn[0] + 2 * sc.i;
  sc.pnode0 = (sc.k * L.Np[1] + sc.j) * L.Np[0] + sc.i;
}

// Is velocity component `comp` of local node n of a structured cell constrained?
template <typename T, int dim>
__device__ __forceinline__ bool structured_zero(const LevelView<T>& L, const StructuredCell<T, dim>& sc,
                                                int comp, int n) {
  if (!L.zero_faces) return false;
  const int gi[3] = {2 * sc.i + n % 3, 2 * sc.j + (n / 3) % 3, dim == 3 ? 2 * sc.k + n / 9 : 0};
  bool z = false;
#pragma unroll
  for (int d = 0; d < dim; ++d) {
    if (gi[d] == 0 && ((L.zero_faces >> ((2 * d) * 3 + comp)) & 1u)) z = true;
    if (gi[d] == L.Nn[d] - 1 && ((L.zero_faces >> ((2 * d + 1) * 3 + comp)) & 1u)) z = true;
  }
  return z;
}

template <int dim>
__device__ __forceinline__ int structured_node_offset(const int* Nn, int n) {
  const int a = n % 3, b = (n / 3) % 3, c = dim == 3 ? n / 9 : 0;
  return (c * Nn[1] + b) * Nn[0] + a;
}
template <int dim>
__device__ __forceinline__ int structured_pnode_offset(const int* Np, int n) {
  const int a = n & 1, b = (n >> 1) & 1, c = dim == 3 ? (n >> 2) & 1 : 0;
  return (c * Np[1] + b) * Np[0] + a;
}

template <typename T>
__device__ __forceinline__ T gather_general(const T* __restrict__ src, int e, const int* lptr, const int* lcol,
                                            const T* lw) {
  if (e >= 0) return src[e];
  if (e == -1) return T(0);
  const int l = -(e + 2);
  T v = T(0);
  for (int k = lptr[l]; k < lptr[l + 1]; ++k) v += lw[k] * src[lcol[k]];
  return v;
}
template <typename T>
__device__ __forceinline__ void scatter_general(T* __restrict__ dst, int e, T v, const int* lptr, const int* lcol,
                                                const T* lw) {
  if (e >= 0) { dst[e] += v; return; }
  if (e == -1) return;
  const int l = -(e + 2);
  for (int k = lptr[l]; k < lptr[l + 1]; ++k) dst[lcol[k]] += lw[k] * v;
}

// ---------------------------------------------------------------------------
// Geometry at one quadrature point: invJ[d][e] = dxi_d/dx_e and JxW.
template <typename T, int dim>
struct QGeom {
  T iJ[dim][dim];
  T jxw;
};

// GK >= 0: the level's geometry kind known at compile time (GeomKind)
template <typename T, int dim, int q, int GK = -1>
__device__ __forceinline__ void qgeom(const LevelView<T>& L, int cell, const T* box, QGeom<T, dim>& g) {
  const int geom = GK >= 0 ? GK : L.geom;
  if (geom == GEOM_TABLE) {
    const T* t = L.gtab + ((size_t)cell * Shape<dim>::nq + q) * (dim * dim + 1);
#pragma unroll
    for (int d = 0; d < dim; ++d)
#pragma unroll
      for (int e = 0; e < dim; ++e) g.iJ[d][e] = t[d * dim + e];
    g.jxw = t[dim * dim] * T(qweight<dim, q>());
  } else {
#pragma unroll
    for (int d = 0; d < dim; ++d)
#pragma unroll
      for (int e = 0; e < dim; ++e) g.iJ[d][e] = d == e ? box[d] : T(0);
    g.jxw = box[dim] * T(qweight<dim, q>());
  }
}

// ---------------------------------------------------------------------------
// The velocity-test cell operator on registers.
//   U: nodal values of this thread's velocity component (OPK_STOKES / OPK_A)
//   P: nodal pressure values (OPK_STOKES / OPK_BT)
// Output: V (nodal velocity-test contributions, this component),
//         YP (partial pressure-test contributions of this component; STOKES)
template <typename T, int dim, int op, int GK = -1>
__device__ __forceinline__ void velocity_cell_op(const LevelView<T>& L, int cell, int comp, unsigned lane_base,
                                                 T* U, const T* P, T* V, T* YP, const T* box, T eta_cell,
                                                 const T* __restrict__ eta_q) {
  const int geom = GK >= 0 ? GK : L.geom;
  constexpr int nv = Shape<dim>::nv, np = Shape<dim>::np;
  constexpr bool need_u = (op == OPK_STOKES || op == OPK_A);
  constexpr bool need_p = (op == OPK_STOKES || op == OPK_BT);
  const unsigned full = 0xffffffffu;
  const int l1 = lane_base + (comp + 1) % dim;
  const int l2 = lane_base + (comp + 2) % dim;
  if (need_u) interpolate<T, dim, false>(U);
#pragma unroll
  for (int n = 0; n < nv; ++n) V[n] = T(0);
  if (op == OPK_STOKES)
#pragma unroll
    for (int n = 0; n < np; ++n) YP[n] = T(0);
  const T s = L.s;

  static_for<nv>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    QGeom<T, dim> G;
    if (geom == GEOM_CART) {
#pragma unroll
      for (int d = 0; d < dim; ++d)
#pragma unroll
        for (int e = 0; e < dim; ++e) G.iJ[d][e] = d == e ? L.inv_h[d] : T(0);
      G.jxw = L.det * T(qweight<dim, q>());
    } else {
      qgeom<T, dim, q, GK>(L, cell, box, G);
    }
    const T eta = eta_q ? eta_q[q] : eta_cell;
    // real-space gradient row of this component: g[e] = d u_comp / d x_e
    T g[3] = {T(0), T(0), T(0)};
    if (need_u) {
      T gr[3];
      gr[0] = colloc_d<T, dim, q, 0>(U);
      gr[1] = colloc_d<T, dim, q, 1>(U);
      if constexpr (dim == 3) gr[2] = colloc_d<T, dim, q, 2>(U);
      if (geom == GEOM_TABLE) {
#pragma unroll
        for (int e = 0; e < dim; ++e) {
          T t = T(0);
#pragma unroll
          for (int d = 0; d < dim; ++d) t += gr[d] * G.iJ[d][e];
          g[e] = t;
        }
      } else {
#pragma unroll
        for (int e = 0; e < dim; ++e) g[e] = gr[e] * G.iJ[e][e];
      }
    }
    T pq = T(0);
    if constexpr (need_p) {
      static_for<np>([&](auto nc) {
        constexpr int n = decltype(nc)::value;
        pq += T(psi_at<dim, q, n>()) * P[n];
      });
    }
    // flux row F[comp][e] (absolute e)
    T F[3] = {T(0), T(0), T(0)};
    if (need_u) {
      if constexpr (dim == 3) {
        const int k1 = (comp + 1) % 3, k2 = (comp + 2) % 3;
        // first exchange: receive d_comp u_{comp+1}; second: receive d_comp u_{comp+2}
        const T send1 = sel3(g[0], g[1], g[2], k2);
        const T send2 = sel3(g[0], g[1], g[2], k1);
        const T r1 = __shfl_sync(full, send1, l1);
        const T r2 = __shfl_sync(full, send2, l2);
        const T gcc = sel3(g[0], g[1], g[2], comp);
        const T f0 = T(2) * eta * gcc;
        const T f1 = eta * (sel3(g[0], g[1], g[2], k1) + r1);
        const T f2 = eta * (sel3(g[0], g[1], g[2], k2) + r2);
        T fdiag = f0;
        if (L.compressible) {
          // d_{c+1} u_{c+1} and d_{c+2} u_{c+2}
          const T d1 = __shfl_sync(full, gcc, l1);
          const T d2 = __shfl_sync(full, gcc, l2);
          fdiag -= T(2) * eta / T(3) * (gcc + d1 + d2);
        }
        // absolute e: relative index (e - comp) mod 3
        F[0] = sel3(fdiag, f1, f2, (3 - comp) % 3);
        F[1] = sel3(fdiag, f1, f2, (4 - comp) % 3);
        F[2] = sel3(fdiag, f1, f2, (5 - comp) % 3);
      } else {
        const int o = 1 - comp;
        const T send = comp == 0 ? g[1] : g[0];
        const T r = __shfl_sync(full, send, lane_base + o);
        const T gcc = comp == 0 ? g[0] : g[1];
        T fdiag = T(2) * eta * gcc;
        if (L.compressible) {
          const T d1 = __shfl_sync(full, gcc, lane_base + o);
          fdiag -= T(2) * eta / T(3) * (gcc + d1);
        }
        const T foff = eta * ((comp == 0 ? g[1] : g[0]) + r);
        F[0] = comp == 0 ? fdiag : foff;
        F[1] = comp == 0 ? foff : fdiag;
      }
    }
    if (need_p) {
      // -s p on the diagonal entry of this row
#pragma unroll
      for (int e = 0; e < dim; ++e)
        if (e == comp) F[e] -= s * pq;
    }
    // reference-direction flux R[d] = JxW sum_e F[e] invJ[d][e]
    T R[3];
    if (geom == GEOM_TABLE) {
#pragma unroll
      for (int d = 0; d < dim; ++d) {
        T t = T(0);
#pragma unroll
        for (int e = 0; e < dim; ++e) t += F[e] * G.iJ[d][e];
        R[d] = t * G.jxw;
      }
    } else {
#pragma unroll
      for (int d = 0; d < dim; ++d) R[d] = F[d] * G.iJ[d][d] * G.jxw;
    }
    colloc_dT<T, dim, q, 0>(V, R[0]);
    colloc_dT<T, dim, q, 1>(V, R[1]);
    if constexpr (dim == 3) colloc_dT<T, dim, q, 2>(V, R[2]);
    if (op == OPK_STOKES) {
      // partial divergence of this component: -s JxW d_comp u_comp
      const T gcc = dim == 3 ? sel3(g[0], g[1], g[2], comp) : (comp == 0 ? g[0] : g[1]);
      const T f = -s * G.jxw * gcc;
#pragma unroll
      static_for<np>([&](auto nc) {
        constexpr int n = decltype(nc)::value;
        YP[n] += T(psi_at<dim, q, n>()) * f;
      });
    }
  });
  interpolate<T, dim, true>(V);
  (void)lane_base;
}

// ---------------------------------------------------------------------------
// Operator application in two passes, both over the whole level:
//   pass 1 (one thread group per cell, all cells in one launch): the cell's
//          contributions to its own local DoFs, stored per cell (Eu, Ep);
//   pass 2 (one thread per DoF): each DoF sums the contributions of its cells in a
//          fixed order (lattice arithmetic, or a CSR list that also folds in the
//          constraint lines) and applies a fused epilogue (plain store,
//          Chebyshev update or residual).
// No colouring, no atomics: one launch per pass keeps every SM busy and the sum
// order is fixed, so results are bit-reproducible.

template <typename T, int dim>
__device__ __forceinline__ void structured_cell_lex(const LevelView<T>& L, int cell, StructuredCell<T, dim>& sc) {
  sc.i = cell % L.nc[0];
  sc.j = (cell / L.nc[0]) % L.nc[1];
  sc.k = dim == 3 ? cell / (L.nc[0] * L.nc[1]) : 0;
  sc.node0 = (2 * sc.k * L.Nn[1] + 2 * sc.j) * L.Nn[0] + 2 * sc.i;
  sc.pnode0 = (sc.k * L.Np[1] + sc.j) * L.Np[0] + sc.i;
}

// Per-point geometry tables (GK = GEOM_TABLE): at most 96 registers, five
// blocks per SM. The kernel waits on global loads (cell DoF codes, values,
// geometry), so the extra resident warps pay for the few spilled registers
// (measured on the shell: FP32 A cell pass 95 -> 91 us, FP32 Stokes 194 -> 170 us;
// on box-geometry levels the same cap measured slower, so they keep the default).
template <typename T, int dim, int op, int GK = -1>
__global__ void __launch_bounds__(128, (GK == GEOM_TABLE ? 5 : 1)) velocity_cell_kernel(LevelView<T> L, const T* __restrict__ src_u,
                                                             const T* __restrict__ src_p, T* __restrict__ Eu,
                                                             T* __restrict__ Ep) {
  pdl_wait();
  constexpr int nv = Shape<dim>::nv, np = Shape<dim>::np, cpw = Shape<dim>::cpw;
  constexpr bool need_u = (op == OPK_STOKES || op == OPK_A);
  constexpr bool need_p = (op == OPK_STOKES || op == OPK_BT);
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int grp = lane / dim;
  int comp = lane - grp * dim;
  bool active = grp < cpw;
  if (!active) { grp = cpw - 1; comp = 0; }
  const unsigned lane_base = grp * dim;
  const int idx = warp * cpw + grp;
  active = active && idx < L.n_cells;
  const int cell = active ? idx : 0;
  StructuredCell<T, dim> sc{};
  if (L.structured) structured_cell_lex<T, dim>(L, cell, sc);

  T U[nv], V[nv], P[np], YP[np];
  T box[4] = {T(0), T(0), T(0), T(0)};
  if ((GK >= 0 ? GK : L.geom) == GEOM_BOX && active)
#pragma unroll
    for (int d = 0; d <= dim; ++d) box[d] = L.gbox[(size_t)cell * (dim + 1) + d];
  if (need_u) {
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
    }
  }
  if (need_p) {
#pragma unroll
    for (int n = 0; n < np; ++n) {
      T v = T(0);
      if (active) {
        if (L.structured) v = src_p[sc.pnode0 + structured_pnode_offset<dim>(L.Np, n)];
        else v = gather_general(src_p, L.cdp[(size_t)cell * np + n], L.plptr, L.plcol, L.plw);
      }
      P[n] = v;
    }
  }
  T eta_cell = T(1);
  const T* eta_q = nullptr;
  if (op != OPK_BT && active) {
    if (L.eta_n == 1) eta_cell = L.eta[cell];
    else eta_q = L.eta + (size_t)cell * L.eta_n;
  }
  velocity_cell_op<T, dim, op, GK>(L, cell, comp, lane_base, U, P, V, YP, box, eta_cell, eta_q);
  if (active) {
    T* e = Eu + ((size_t)cell * dim + comp) * nv;
#pragma unroll
    for (int n = 0; n < nv; ++n) e[n] = V[n];
  }
  if (op == OPK_STOKES) {
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int n = 0; n < np; ++n) {
      const T v = YP[n];
      T t = v;
#pragma unroll
      for (int o = 1; o < dim; ++o) t += __shfl_sync(full, v, lane_base + (comp + o) % dim);
      YP[n] = t;
    }
    if (active) {
#pragma unroll
      for (int n = 0; n < np; ++n)
        if (n % dim == comp) Ep[(size_t)cell * np + n] = YP[n];
    }
  }
}

// ---------------------------------------------------------------------------
// Pressure mass operator: one thread per cell.
template <typename T, int dim>
__device__ __forceinline__ void mass_cell_op(const LevelView<T>& L, int cell, const T* P, T* YP, const T* box,
                                             T eta_cell, const T* __restrict__ eta_q) {
  constexpr int np = Shape<dim>::np, nq = Shape<dim>::nq;
  const T s2 = L.s * L.s;
#pragma unroll
  for (int n = 0; n < np; ++n) YP[n] = T(0);
  static_for<nq>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    T jxw;
    if (L.geom == GEOM_CART) jxw = L.det * T(qweight<dim, q>());
    else if (L.geom == GEOM_BOX) jxw = box[dim] * T(qweight<dim, q>());
    else jxw = L.gtab[((size_t)cell * nq + q) * (dim * dim + 1) + dim * dim] * T(qweight<dim, q>());
    const T eta = eta_q ? eta_q[q] : eta_cell;
    T pq = T(0);
    static_for<np>([&](auto nc) {
      constexpr int n = decltype(nc)::value;
      pq += T(psi_at<dim, q, n>()) * P[n];
    });
    const T f = s2 / eta * pq * jxw;
    static_for<np>([&](auto nc) {
      constexpr int n = decltype(nc)::value;
      YP[n] += T(psi_at<dim, q, n>()) * f;
    });
  });
}

// FP32, 3D lattice levels: one thread per cell. All 81 nodal values stay in
// registers with compile-time component indices, so no shuffles, selects or
// runtime geometry branches are needed, and the viscosity is read once per
// point. The per-cell contributions are written slot-major (E[slot][cell]), so
// the stores of a warp are coalesced.
template <int op, bool eta_per_q>
__device__ __forceinline__ void lattice_cell_f32(const LevelView<float>& L, const float* __restrict__ src_u,
                                                 const float* __restrict__ src_p, int cell, float (&V)[3][27],
                                                 float (&YP)[8], const float* eta_q = nullptr, int eta_stride = 1) {
  constexpr bool need_u = (op == OPK_STOKES || op == OPK_A);
  constexpr bool need_p = (op == OPK_STOKES || op == OPK_BT);
  using T = float;
  StructuredCell<T, 3> sc;
  structured_cell_lex<T, 3>(L, cell, sc);
  T U[3][27], P[8];
  if constexpr (need_u) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int n = 0; n < 27; ++n)
        U[c][n] = structured_zero<T, 3>(L, sc, c, n)
                      ? T(0)
                      : src_u[c * L.n_nodes + sc.node0 + structured_node_offset<3>(L.Nn, n)];
#pragma unroll
    for (int c = 0; c < 3; ++c) interpolate<T, 3, false>(U[c]);
  }
  if constexpr (need_p) {
#pragma unroll
    for (int n = 0; n < 8; ++n) P[n] = src_p[sc.pnode0 + structured_pnode_offset<3>(L.Np, n)];
  }
#pragma unroll
  for (int n = 0; n < 8; ++n) YP[n] = T(0);
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int n = 0; n < 27; ++n) V[c][n] = T(0);
  const T ih0 = L.inv_h[0], ih1 = L.inv_h[1], ih2 = L.inv_h[2];
  const T s = L.s;
  const T eta_cell = eta_per_q ? T(0) : L.eta[cell];
  // per-point viscosity: the level table, or the caller's copy (eta_q[q * eta_stride])
  const T* eq = eta_q ? eta_q : L.eta + (size_t)cell * 27;
  const int es = eta_q ? eta_stride : 1;
  static_for<27>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const T jxw = L.det * T(qweight<3, q>());
    const T eta = eta_per_q ? eq[q * es] : eta_cell;
    T G[3][3] = {{T(0)}};
    if constexpr (need_u) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        G[c][0] = colloc_d<T, 3, q, 0>(U[c]) * ih0;
        G[c][1] = colloc_d<T, 3, q, 1>(U[c]) * ih1;
        G[c][2] = colloc_d<T, 3, q, 2>(U[c]) * ih2;
      }
    }
    T pq = T(0);
    if constexpr (need_p) {
      static_for<8>([&](auto nc) {
        constexpr int n = decltype(nc)::value;
        pq += T(psi_at<3, q, n>()) * P[n];
      });
    }
    T F[3][3];
    const T div = G[0][0] + G[1][1] + G[2][2];
    if constexpr (need_u) {
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) F[a][b] = eta * (G[a][b] + G[b][a]);
      if (L.compressible) {
        const T t = T(2) * eta / T(3) * div;
        F[0][0] -= t; F[1][1] -= t; F[2][2] -= t;
      }
    } else {
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) F[a][b] = T(0);
    }
    if constexpr (need_p) {
      F[0][0] -= s * pq; F[1][1] -= s * pq; F[2][2] -= s * pq;
    }
    const T w0 = ih0 * jxw, w1 = ih1 * jxw, w2 = ih2 * jxw;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      colloc_dT<T, 3, q, 0>(V[c], F[c][0] * w0);
      colloc_dT<T, 3, q, 1>(V[c], F[c][1] * w1);
      colloc_dT<T, 3, q, 2>(V[c], F[c][2] * w2);
    }
    if constexpr (op == OPK_STOKES) {
      const T f = -s * jxw * div;
      static_for<8>([&](auto nc) {
        constexpr int n = decltype(nc)::value;
        YP[n] += T(psi_at<3, q, n>()) * f;
      });
    }
  });
#pragma unroll
  for (int c = 0; c < 3; ++c) interpolate<T, 3, true>(V[c]);
}

template <int op, bool eta_per_q>
__global__ void __launch_bounds__(128) lattice_cell_kernel_f32(LevelView<float> L, const float* __restrict__ src_u,
                                                                const float* __restrict__ src_p,
                                                                float* __restrict__ Eu, float* __restrict__ Ep) {
  // per-point viscosity (fixed over a V-cycle) copied to shared memory before
  // pdl_wait, so that under the V-cycle graphs' programmatic edges its latency
  // overlaps the preceding kernel; each thread reads back only its own column
  // after waiting for its own copies
  __shared__ float eta_s[eta_per_q ? 27 : 1][128];
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = cell < L.n_cells;
  if (eta_per_q && live) {
    const float* src = L.eta + (size_t)cell * 27;
#pragma unroll
    for (int q = 0; q < 27; ++q) {
      const unsigned sa = (unsigned)__cvta_generic_to_shared(&eta_s[q][threadIdx.x]);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(src + q) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  pdl_wait();
  if (!live) return;
  if (eta_per_q) asm volatile("cp.async.wait_all;\n" ::: "memory");
  float V[3][27], YP[8];
  lattice_cell_f32<op, eta_per_q>(L, src_u, src_p, cell, V, YP, eta_per_q ? &eta_s[0][threadIdx.x] : nullptr, 128);
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int n = 0; n < 27; ++n) Eu[(size_t)(c * 27 + n) * L.n_cells + cell] = V[c][n];
  if constexpr (op == OPK_STOKES) {
#pragma unroll
    for (int n = 0; n < 8; ++n) Ep[(size_t)n * L.n_cells + cell] = YP[n];
  }
}

// ---------------------------------------------------------------------------
// FP64 cell pass of isotropic 3D lattice levels (cubic cells, h the same in
// every direction: the box workloads). GB300 issues about two FP64 FMAs per SM
// and clock, 1/64 of its FP32 rate, so this kernel is written to spend as few
// FP64 instructions as possible; shuffles, selects and integer work are almost
// free next to them.
//  * One velocity component per thread, three threads per cell, as in
//    velocity_cell_kernel; the symmetric gradient's off-diagonal entries come
//    from the sibling threads by warp shuffles.
//  * The geometry is folded into two per-point constants (IsoCoef): with
//    g = ih gr (gr the reference gradient), the reference-direction fluxes are
//      R_cc = 2 K_q eta gr_cc - M_q p,  R_ce = K_q eta (gr_ce + gr_ec),
//    K_q = ih^2 |det J| w_q, M_q = s ih |det J| w_q.
//  * The Q1 pressure work is done once per cell, not once per component: thread
//    c interpolates the pressure to the nine Gauss points of plane z = c (sum
//    factorisation, 38 operations) and the other threads read them by shuffle;
//    the divergence at each point is summed by shuffles, kept by the thread of
//    that point's plane, and integrated back plane by plane (transposed sum
//    factorisation), the three partial results then summed by shuffles.
// Output layout and summation into nodes are those of velocity_cell_kernel
// (cell-major contributions), so the gathers are shared.
template <typename T>
struct IsoCoef {
  T K[27];  // ih^2 |det J| w_q
  T M[27];  // s ih |det J| w_q
};

template <int op, bool eta_per_q>
__global__ void __launch_bounds__(128) lattice_iso_kernel_f64(LevelView<double> L, IsoCoef<double> C,
                                                               const double* __restrict__ src_u,
                                                               const double* __restrict__ src_p,
                                                               double* __restrict__ Eu, double* __restrict__ Ep) {
  pdl_wait();
  using T = double;
  constexpr bool need_u = (op == OPK_STOKES || op == OPK_A);
  constexpr bool need_p = (op == OPK_STOKES || op == OPK_BT);
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int grp = lane / 3;
  int comp = lane - 3 * grp;
  bool active = grp < 10;
  if (!active) { grp = 9; comp = 0; }  // lanes 30, 31 shadow lane 27 and write nothing
  const int lb = 3 * grp;
  const int l1 = lb + (comp + 1) % 3, l2 = lb + (comp + 2) % 3;
  const int k1 = (comp + 1) % 3, k2 = (comp + 2) % 3;
  const int idx = warp * 10 + grp;
  active = active && idx < L.n_cells;
  const int cell = active ? idx : 0;
  StructuredCell<T, 3> sc;
  structured_cell_lex<T, 3>(L, cell, sc);

  T U[27], V[27];
  if constexpr (need_u) {
#pragma unroll
    for (int n = 0; n < 27; ++n) {
      T v = T(0);
      if (active && !structured_zero<T, 3>(L, sc, comp, n))
        v = src_u[comp * L.n_nodes + sc.node0 + structured_node_offset<3>(L.Nn, n)];
      U[n] = v;
    }
    interpolate<T, 3, false>(U);
  }
#pragma unroll
  for (int n = 0; n < 27; ++n) V[n] = T(0);

  // scaled pressure at the nine points of plane z = comp: spl[qy*3+qx] = M_q p(q)
  T spl[9];
  if constexpr (need_p) {
    T P[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) P[n] = active ? src_p[sc.pnode0 + structured_pnode_offset<3>(L.Np, n)] : T(0);
    const T z0 = sel3(T(fe::P1v(0, 0)), T(fe::P1v(1, 0)), T(fe::P1v(2, 0)), comp);
    const T z1 = sel3(T(fe::P1v(0, 1)), T(fe::P1v(1, 1)), T(fe::P1v(2, 1)), comp);
    T a[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = z0 * P[i] + z1 * P[i + 4];
    T b[6];
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int qx = 0; qx < 3; ++qx) b[y * 3 + qx] = T(fe::P1v(qx, 0)) * a[2 * y] + T(fe::P1v(qx, 1)) * a[2 * y + 1];
#pragma unroll
    for (int qy = 0; qy < 3; ++qy)
#pragma unroll
      for (int qx = 0; qx < 3; ++qx) {
        const int j = qy * 3 + qx;
        const T m = sel3(C.M[j], C.M[9 + j], C.M[18 + j], comp);
        spl[j] = m * (T(fe::P1v(qy, 0)) * b[qx] + T(fe::P1v(qy, 1)) * b[3 + qx]);
      }
  } else {
#pragma unroll
    for (int j = 0; j < 9; ++j) spl[j] = T(0);
  }

  const T* __restrict__ eq = eta_per_q ? L.eta + (size_t)cell * 27 : L.eta;
  const T eta_cell = eta_per_q ? T(1) : L.eta[cell];
  T dq[9];  // reference divergence at the points of plane z = comp
#pragma unroll
  for (int j = 0; j < 9; ++j) dq[j] = T(0);
  const bool compressible = L.compressible != 0;

  static_for<27>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    constexpr int qz = q / 9, j = q % 9;
    T pq = T(0);
    if constexpr (need_p) pq = __shfl_sync(full, spl[j], lb + qz);
    T R0, R1, R2;
    if constexpr (need_u) {
      const T g0 = colloc_d<T, 3, q, 0>(U);
      const T g1 = colloc_d<T, 3, q, 1>(U);
      const T g2 = colloc_d<T, 3, q, 2>(U);
      const T gcc = sel3(g0, g1, g2, comp);
      const T gk1 = sel3(g0, g1, g2, k1);
      const T gk2 = sel3(g0, g1, g2, k2);
      const T r1 = __shfl_sync(full, gk2, l1);  // d_comp u_k1
      const T r2 = __shfl_sync(full, gk1, l2);  // d_comp u_k2
      const T eta = eta_per_q ? eq[q] : eta_cell;
      const T a = eta * C.K[q];
      T Rc;
      if constexpr (op == OPK_STOKES) Rc = T(2) * (a * gcc) - pq;
      else Rc = T(2) * (a * gcc);
      if (op == OPK_STOKES || compressible) {
        const T tot = gcc + __shfl_sync(full, gcc, l1) + __shfl_sync(full, gcc, l2);
        if (compressible) Rc -= T(2.0 / 3.0) * (a * tot);
        if (op == OPK_STOKES) dq[j] = comp == qz ? tot : dq[j];
      }
      const T Rk1 = a * (gk1 + r1);
      const T Rk2 = a * (gk2 + r2);
      R0 = sel3(Rc, Rk2, Rk1, comp);
      R1 = sel3(Rk1, Rc, Rk2, comp);
      R2 = sel3(Rk2, Rk1, Rc, comp);
    } else {
      R0 = comp == 0 ? -pq : T(0);
      R1 = comp == 1 ? -pq : T(0);
      R2 = comp == 2 ? -pq : T(0);
    }
    colloc_dT<T, 3, q, 0>(V, R0);
    colloc_dT<T, 3, q, 1>(V, R1);
    colloc_dT<T, 3, q, 2>(V, R2);
  });
  interpolate<T, 3, true>(V);
  if (active) {
    T* e = Eu + ((size_t)cell * 3 + comp) * 27;
#pragma unroll
    for (int n = 0; n < 27; ++n) e[n] = V[n];
  }
  if constexpr (op == OPK_STOKES) {
    // pressure test -s JxW div, plane z = comp: f = -M_q dq, then back to the 8 nodes
    T f[9];
#pragma unroll
    for (int jj = 0; jj < 9; ++jj) f[jj] = -sel3(C.M[jj], C.M[9 + jj], C.M[18 + jj], comp) * dq[jj];
    T b[6];  // [ny][qx]
#pragma unroll
    for (int ny = 0; ny < 2; ++ny)
#pragma unroll
      for (int qx = 0; qx < 3; ++qx)
        b[ny * 3 + qx] = T(fe::P1v(0, ny)) * f[qx] + T(fe::P1v(1, ny)) * f[3 + qx] + T(fe::P1v(2, ny)) * f[6 + qx];
    T a[4];  // [ny][nx]
#pragma unroll
    for (int ny = 0; ny < 2; ++ny)
#pragma unroll
      for (int nx = 0; nx < 2; ++nx)
        a[ny * 2 + nx] = T(fe::P1v(0, nx)) * b[ny * 3] + T(fe::P1v(1, nx)) * b[ny * 3 + 1] +
                         T(fe::P1v(2, nx)) * b[ny * 3 + 2];
    const T z0 = sel3(T(fe::P1v(0, 0)), T(fe::P1v(1, 0)), T(fe::P1v(2, 0)), comp);
    const T z1 = sel3(T(fe::P1v(0, 1)), T(fe::P1v(1, 1)), T(fe::P1v(2, 1)), comp);
    T YP[8];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      YP[i] = z0 * a[i];
      YP[i + 4] = z1 * a[i];
    }
#pragma unroll
    for (int n = 0; n < 8; ++n) YP[n] += __shfl_sync(full, YP[n], l1) + __shfl_sync(full, YP[n], l2);
    if (active) {
#pragma unroll
      for (int n = 0; n < 8; ++n)
        if (n % 3 == comp) Ep[(size_t)cell * 8 + n] = YP[n];
    }
  }
}

// FP32 A-block cell pass for small 3D lattice levels (the coarse levels of the
// V-cycle): one cell per block, one thread per (component, node). The
// register-resident kernel above runs each cell's ~5k straight-line
// instructions on one thread, and with only a few hundred cells nothing hides
// that chain (about 8-14 us per launch whatever the level's size). Here every
// sum-factorisation sweep is a 3-term dot per thread followed by a barrier, so
// the chain is a few dozen operations. Same arithmetic as the lattice kernel up
// to the order of the sums; slot-major output, so the gather pass is shared.
struct SmallLatticeTables {
  float S[3][3];   // S[q][n]: node n -> Gauss point q (1D)
  float D[3][3];   // D[q][a]: collocation derivative at Gauss point q
  float W[27];     // 3D Gauss weights
};
__constant__ SmallLatticeTables c_small_tables = {
    {{(float)fe::Sv(0, 0), (float)fe::Sv(0, 1), (float)fe::Sv(0, 2)},
     {(float)fe::Sv(1, 0), (float)fe::Sv(1, 1), (float)fe::Sv(1, 2)},
     {(float)fe::Sv(2, 0), (float)fe::Sv(2, 1), (float)fe::Sv(2, 2)}},
    {{(float)fe::Dv(0, 0), (float)fe::Dv(0, 1), (float)fe::Dv(0, 2)},
     {(float)fe::Dv(1, 0), (float)fe::Dv(1, 1), (float)fe::Dv(1, 2)},
     {(float)fe::Dv(2, 0), (float)fe::Dv(2, 1), (float)fe::Dv(2, 2)}},
    {(float)qweight<3, 0>(),  (float)qweight<3, 1>(),  (float)qweight<3, 2>(),  (float)qweight<3, 3>(),
     (float)qweight<3, 4>(),  (float)qweight<3, 5>(),  (float)qweight<3, 6>(),  (float)qweight<3, 7>(),
     (float)qweight<3, 8>(),  (float)qweight<3, 9>(),  (float)qweight<3, 10>(), (float)qweight<3, 11>(),
     (float)qweight<3, 12>(), (float)qweight<3, 13>(), (float)qweight<3, 14>(), (float)qweight<3, 15>(),
     (float)qweight<3, 16>(), (float)qweight<3, 17>(), (float)qweight<3, 18>(), (float)qweight<3, 19>(),
     (float)qweight<3, 20>(), (float)qweight<3, 21>(), (float)qweight<3, 22>(), (float)qweight<3, 23>(),
     (float)qweight<3, 24>(), (float)qweight<3, 25>(), (float)qweight<3, 26>()}};

constexpr int kSmallCellThreads = 96;  // 81 active: (component, node)

// The cell pass of the small-level kernel once A[0] holds the cell's 81 nodal
// values (zero at constrained DoFs) and all threads have passed a barrier.
template <bool eta_per_q>
__device__ __forceinline__ void small_cell_pass(const LevelView<float>& L, int cell, float eta_pre,
                                                float (&A)[2][81], float (&G)[9][27], float* __restrict__ Eu) {
  const SmallLatticeTables& K = c_small_tables;
  const int t = threadIdx.x;
  const bool act = t < 81;
  const int c = act ? t / 27 : 0;
  const int n = act ? t - 27 * c : 0;
  const int dig[3] = {n % 3, (n / 3) % 3, n / 9};
  const int st[3] = {1, 3, 9};
  // nodes -> Gauss points, directions 0, 1, 2
  int cur = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (act) {
      const int k = dig[d];
      const float* a = &A[cur][c * 27 + n - k * st[d]];
      A[cur ^ 1][t] = K.S[k][0] * a[0] + K.S[k][1] * a[st[d]] + K.S[k][2] * a[2 * st[d]];
    }
    cur ^= 1;
    __syncthreads();
  }
  // gradient of component c at point q = n
  if (act) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int k = dig[d];
      const float* a = &A[cur][c * 27 + n - k * st[d]];
      G[c * 3 + d][n] = (K.D[k][0] * a[0] + K.D[k][1] * a[st[d]] + K.D[k][2] * a[2 * st[d]]) * L.inv_h[d];
    }
  }
  __syncthreads();
  // fluxes at point q (27 threads): R[a][b] = eta (G[a][b] + G[b][a]) (deviatoric if compressible) * JxW / h_b
  if (t < 27) {
    const int q = t;
    const float jxw = L.det * K.W[q];
    const float eta = eta_pre;
    float g[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) g[a][b] = G[a * 3 + b][q];
    const float div = g[0][0] + g[1][1] + g[2][2];
    float F[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) F[a][b] = eta * (g[a][b] + g[b][a]);
    if (L.compressible) {
      const float tr = 2.0f * eta / 3.0f * div;
      F[0][0] -= tr; F[1][1] -= tr; F[2][2] -= tr;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) G[a * 3 + b][q] = F[a][b] * (L.inv_h[b] * jxw);
  }
  __syncthreads();
  // transposed derivative: value at node-position n of component c
  if (act) {
    float v = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int k = dig[d];
      const int base = n - k * st[d];
      const float* r = &G[c * 3 + d][base];
      v += K.D[0][k] * r[0] + K.D[1][k] * r[st[d]] + K.D[2][k] * r[2 * st[d]];
    }
    A[cur][t] = v;
  }
  __syncthreads();
  // Gauss points -> nodes (transposed interpolation), directions 0, 1, 2
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (act) {
      const int k = dig[d];
      const float* a = &A[cur][c * 27 + n - k * st[d]];
      A[cur ^ 1][t] = K.S[0][k] * a[0] + K.S[1][k] * a[st[d]] + K.S[2][k] * a[2 * st[d]];
    }
    cur ^= 1;
    __syncthreads();
  }
  if (act) Eu[(size_t)(c * 27 + n) * L.n_cells + cell] = A[cur][t];
}


template <bool eta_per_q>
__global__ void __launch_bounds__(kSmallCellThreads) lattice_cell_kernel_small(LevelView<float> L,
                                                                               const float* __restrict__ src_u,
                                                                               float* __restrict__ Eu) {
  // the cell's viscosity (fixed over a V-cycle) before pdl_wait, overlapping the
  // preceding kernel in the V-cycle graphs' programmatic edges
  const float eta_pre = threadIdx.x < 27 ? (eta_per_q ? L.eta[(size_t)blockIdx.x * 27 + threadIdx.x] : L.eta[blockIdx.x])
                                         : 0.0f;
  pdl_wait();
  __shared__ float A[2][81];   // nodal / Gauss-point values, ping-pong between sweeps
  __shared__ float G[9][27];   // G[c*3+d][q] = d u_c / d x_d, then the fluxes R in place
  const int cell = blockIdx.x;
  const int t = threadIdx.x;
  const bool act = t < 81;
  const int c = act ? t / 27 : 0;
  const int n = act ? t - 27 * c : 0;
  StructuredCell<float, 3> sc;
  structured_cell_lex<float, 3>(L, cell, sc);
  if (act)
    A[0][t] = structured_zero<float, 3>(L, sc, c, n) ? 0.0f
                                                     : src_u[c * L.n_nodes + sc.node0 + structured_node_offset<3>(L.Nn, n)];
  __syncthreads();
  small_cell_pass<eta_per_q>(L, cell, eta_pre, A, G, Eu);
}

// One Chebyshev step of the FP32 A-block smoother of a small lattice level with
// the next step's cell pass fused in (one launch instead of a gather and a cell
// pass): each block gathers its cell's 81 DoFs from the previous cell pass's
// contributions E (the sum of structured_dof_sum, as the gathers form it), runs
// the Chebyshev update of the gathers' epilogue (first: the zero-start step
// d = f2 dinv b, x = d), writes the DoFs whose owner it is (a node belongs to
// the cell holding it at local coordinate 0 or 1 along every direction, or 2
// on the level's upper faces) to the other buffers of a ping-pong pair, and
// runs the cell pass on the new values into E_out. Shared nodes are updated by
// up to eight blocks with the same arithmetic; only the owner stores.
template <typename T, int dim>
__device__ __forceinline__ T structured_dof_sum(const LevelView<T>& L, const T* __restrict__ E, int cs, int ss,
                                                int comp, int node, bool& constrained);
struct ChebSmallArgs {
  const float* E;      // slot-major contributions of the previous cell pass (not read when first)
  float* E_out;        // slot-major contributions of this step's cell pass
  const float* x_in;
  const float* d_in;
  float* x_out;
  float* d_out;
  const float* b;
  const float* dinv;
  float f1, f2;
};
template <bool first, bool eta_per_q>
__global__ void __launch_bounds__(kSmallCellThreads) lattice_cheb_small(LevelView<float> L, ChebSmallArgs a) {
  const int cell = blockIdx.x;
  const int t = threadIdx.x;
  const bool act = t < 81;
  const int c = act ? t / 27 : 0;
  const int n = act ? t - 27 * c : 0;
  StructuredCell<float, 3> sc;
  structured_cell_lex<float, 3>(L, cell, sc);
  const int node = sc.node0 + structured_node_offset<3>(L.Nn, n);
  const long g = (long)c * L.n_nodes + node;
  // fixed over a V-cycle: viscosity and diagonal before pdl_wait
  const float eta_pre = t < 27 ? (eta_per_q ? L.eta[(size_t)cell * 27 + t] : L.eta[cell]) : 0.0f;
  const float dg = act ? a.dinv[g] : 0.0f;
  pdl_wait();
  __shared__ float A[2][81];
  __shared__ float G[9][27];
  if (act) {
    float xn, dn;
    if (first) {
      dn = a.f2 * dg * a.b[g];
      xn = dn;
    } else {
      bool cons = false;
      const float sum = structured_dof_sum<float, 3>(L, a.E, 1, L.n_cells, c, node, cons);
      const float xg = a.x_in[g];
      const float tt = cons ? xg : sum;
      dn = a.f1 * a.d_in[g] + a.f2 * dg * (a.b[g] - tt);
      xn = xg + dn;
    }
    const int gi[3] = {2 * sc.i + n % 3, 2 * sc.j + (n / 3) % 3, 2 * sc.k + n / 9};
    const int ci[3] = {sc.i, sc.j, sc.k};
    bool owner = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) owner = owner && ci[d] == min(gi[d] >> 1, L.nc[d] - 1);
    if (owner) {
      a.x_out[g] = xn;
      a.d_out[g] = dn;
    }
    A[0][t] = structured_zero<float, 3>(L, sc, c, n) ? 0.0f : xn;
  }
  __syncthreads();
  small_cell_pass<eta_per_q>(L, cell, eta_pre, A, G, a.E_out);
}

// (generic loads: the rows may live in global or in shared memory)
template <typename T, int np>
__device__ __forceinline__ void load_row(const T* __restrict__ row, T (&r)[np]) {
  if constexpr (sizeof(T) == 4 && np % 4 == 0) {
#pragma unroll
    for (int j = 0; j < np; j += 4) {
      const float4 v = *reinterpret_cast<const float4*>(row + j);
      r[j] = v.x; r[j + 1] = v.y; r[j + 2] = v.z; r[j + 3] = v.w;
    }
  } else if constexpr (sizeof(T) == 8 && np % 2 == 0) {
#pragma unroll
    for (int j = 0; j < np; j += 2) {
      const double2 v = *reinterpret_cast<const double2*>(row + j);
      r[j] = v.x; r[j + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < np; ++j) r[j] = row[j];
  }
}

template <typename T, int dim>
__global__ void __launch_bounds__(128) mass_cell_kernel(LevelView<T> L, const T* __restrict__ src_p,
                                                         T* __restrict__ Ep) {
  pdl_wait();
  constexpr int np = Shape<dim>::np;
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= L.n_cells) return;
  StructuredCell<T, dim> sc{};
  if (L.structured) structured_cell_lex<T, dim>(L, cell, sc);
  T P[np], YP[np];
#pragma unroll
  for (int n = 0; n < np; ++n)
    P[n] = L.structured ? src_p[sc.pnode0 + structured_pnode_offset<dim>(L.Np, n)]
                        : gather_general(src_p, L.cdp[(size_t)cell * np + n], L.plptr, L.plcol, L.plw);
  if (L.Mp) {  // the cell's matrix of the level table: np x np multiply-adds, no geometry reads
    const T* __restrict__ M = L.Mp + (size_t)cell * np * np;
#pragma unroll
    for (int i = 0; i < np; ++i) {
      T r[np];
      load_row<T, np>(M + i * np, r);
      T t = T(0);
#pragma unroll
      for (int j = 0; j < np; ++j) t += r[j] * P[j];
      YP[i] = t;
    }
  } else {
    T box[4] = {T(0), T(0), T(0), T(0)};
    if (L.geom == GEOM_BOX)
#pragma unroll
      for (int d = 0; d <= dim; ++d) box[d] = L.gbox[(size_t)cell * (dim + 1) + d];
    const T eta_cell = L.eta_n == 1 ? L.eta[cell] : T(1);
    const T* eta_q = L.eta_n == 1 ? nullptr : L.eta + (size_t)cell * L.eta_n;
    mass_cell_op<T, dim>(L, cell, P, YP, box, eta_cell, eta_q);
  }
#pragma unroll
  for (int n = 0; n < np; ++n) Ep[(size_t)cell * np + n] = YP[n];
}

// ---------------------------------------------------------------------------
// Pass 2: per-DoF gather with a fused epilogue.
enum Epilogue {
  EPI_STORE = 0,    // y = K x; constrained rows y = x
  EPI_BT = 1,       // y = B^T p; constrained velocity rows y = 0
  EPI_RESID = 2,    // y = b - K x; constrained rows y = b - x
  EPI_CHEB = 3,     // t = K x; d = f1 d + f2 dinv (b - t); x += d (x updated in place)
  EPI_CHEB_OUT = 4  // as EPI_CHEB, but the new iterate goes to y (x is only read)
};

template <typename T>
struct GatherArgs {
  const T* E;      // per-cell contributions
  T* x;            // operator input (identity rows; updated by EPI_CHEB)
  T* y;            // output (EPI_STORE / EPI_BT / EPI_RESID)
  const T* b;      // right-hand side (EPI_RESID / EPI_CHEB)
  const T* dinv;   // inverse diagonal (EPI_CHEB)
  T* d;            // Chebyshev update vector (EPI_CHEB)
  T f1, f2;
  // layout of E on lattice levels: entry (cell, slot) at cell * cs + slot * ss;
  // cell-major (cs = slots per cell, ss = 1) or slot-major (cs = 1, ss = n_cells)
  long cs, ss;
};

// General levels: CSR of (cell-local slot, weight) per DoF, built at set-up
// with the constraint lines folded in; cmask marks constrained DoFs.
template <typename T>
struct GatherCsr {
  const int* ptr;
  const int* slot;
  const T* w;
  const unsigned char* cmask;
};

template <typename T, int epi>
__device__ __forceinline__ void gather_epilogue_dinv(const GatherArgs<T>& a, long g, T sum, bool constrained,
                                                    T dinv_g) {
  if (epi == EPI_STORE) {
    a.y[g] = constrained ? a.x[g] : sum;
  } else if (epi == EPI_BT) {
    a.y[g] = constrained ? T(0) : sum;
  } else if (epi == EPI_RESID) {
    a.y[g] = a.b[g] - (constrained ? a.x[g] : sum);
  } else {
    const T xg = a.x[g];
    const T t = constrained ? xg : sum;
    const T dn = a.f1 * a.d[g] + a.f2 * dinv_g * (a.b[g] - t);
    a.d[g] = dn;
    if (epi == EPI_CHEB) a.x[g] = xg + dn;
    else a.y[g] = xg + dn;
  }
}
template <typename T, int epi>
__device__ __forceinline__ void gather_epilogue(const GatherArgs<T>& a, long g, T sum, bool constrained) {
  gather_epilogue_dinv<T, epi>(a, g, sum, constrained,
                               (epi == EPI_CHEB || epi == EPI_CHEB_OUT) ? a.dinv[g] : T(0));
}

// Velocity DoFs of a lattice level: a node's cells follow from its coordinates.
// Sum of the per-cell contributions E (cell stride cs, slot stride ss) of
// velocity DoF (comp, node) of a lattice level, lower cell first along z, y, x;
// constrained: the DoF is on a zero face (the sum is then 0).
template <typename T, int dim>
__device__ __forceinline__ T structured_dof_sum(const LevelView<T>& L, const T* __restrict__ E, int cs, int ss,
                                                int comp, int node, bool& constrained) {
  constexpr int nv = Shape<dim>::nv;
  const int gc[3] = {node % L.Nn[0], (node / L.Nn[0]) % L.Nn[1], dim == 3 ? node / (L.Nn[0] * L.Nn[1]) : 0};
  int cidx[3][2], loc[3][2], cnt[3];
  constrained = false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    cnt[d] = 0;
    if (d >= dim) { cnt[d] = 1; cidx[d][0] = 0; loc[d][0] = 0; continue; }
    const int x = gc[d];
    if (x & 1) {
      cidx[d][0] = (x - 1) >> 1; loc[d][0] = 1; cnt[d] = 1;
    } else {
      if (x > 0) { cidx[d][cnt[d]] = (x >> 1) - 1; loc[d][cnt[d]] = 2; ++cnt[d]; }
      if (x < L.Nn[d] - 1) { cidx[d][cnt[d]] = x >> 1; loc[d][cnt[d]] = 0; ++cnt[d]; }
    }
    if (x == 0 && ((L.zero_faces >> ((2 * d) * 3 + comp)) & 1u)) constrained = true;
    if (x == L.Nn[d] - 1 && ((L.zero_faces >> ((2 * d + 1) * 3 + comp)) & 1u)) constrained = true;
  }
  T sum = T(0);
  if (!constrained) {
    for (int kz = 0; kz < cnt[2]; ++kz)
      for (int ky = 0; ky < cnt[1]; ++ky)
        for (int kx = 0; kx < cnt[0]; ++kx) {
          const int cell = (cidx[2][kz] * L.nc[1] + cidx[1][ky]) * L.nc[0] + cidx[0][kx];
          const int l = loc[0][kx] + 3 * loc[1][ky] + 9 * loc[2][kz];
          sum += E[(size_t)cell * cs + (size_t)(comp * nv + l) * ss];
        }
  }
  return sum;
}

template <typename T, int dim, int epi>
__global__ void __launch_bounds__(256) velocity_gather_structured(LevelView<T> L, GatherArgs<T> a) {
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  // the diagonal inverse (fixed over a V-cycle) before pdl_wait
  const T dg = ((epi == EPI_CHEB || epi == EPI_CHEB_OUT) && g < L.n_u) ? a.dinv[g] : T(0);
  pdl_wait();
  if (g >= L.n_u) return;
  const int comp = (int)(g / L.n_nodes);
  const int node = (int)(g - (long)comp * L.n_nodes);
  bool constrained = false;
  const T sum = structured_dof_sum<T, dim>(L, a.E, a.cs, a.ss, comp, node, constrained);
  gather_epilogue_dinv<T, epi>(a, g, sum, constrained, dg);
}

// Velocity DoFs of a 3D lattice level, one thread per Q2 node for all three
// components: the node's (at most 2 per direction) cells and local positions
// are found once and the 3 x 8 candidate contributions are predicated loads in
// registers (no run-time indexed arrays, so no local memory). Candidates are
// summed in the same order as velocity_gather_structured (z, y, x; the lower
// cell along a direction first), so the two give bit-identical sums.
template <typename T, int epi>
__device__ __forceinline__ void velocity_lattice_node_d(const LevelView<T>& L, const GatherArgs<T>& a, int node,
                                                        const T (&dv)[3]) {
  const int nxy = L.Nn[0] * L.Nn[1];
  const int gz = node / nxy;
  const int rem = node - gz * nxy;
  const int gy = rem / L.Nn[0];
  const int gx = rem - gy * L.Nn[0];
  const int g3[3] = {gx, gy, gz};
  // per direction: candidate 0 (lower cell / the cell of an odd node) and 1 (upper cell)
  int c0[3], l0[3], c1[3], l1[3];
  bool v0[3], v1[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int x = g3[d];
    if (x & 1) {
      c0[d] = (x - 1) >> 1; l0[d] = 1; v0[d] = true;
      c1[d] = 0; l1[d] = 0; v1[d] = false;
    } else {
      c0[d] = (x >> 1) - 1; l0[d] = 2; v0[d] = x > 0;
      c1[d] = x >> 1; l1[d] = 0; v1[d] = x < L.Nn[d] - 1;
    }
  }
  bool cons[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    bool z = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (g3[d] == 0 && ((L.zero_faces >> ((2 * d) * 3 + c)) & 1u)) z = true;
      if (g3[d] == L.Nn[d] - 1 && ((L.zero_faces >> ((2 * d + 1) * 3 + c)) & 1u)) z = true;
    }
    cons[c] = z;
  }
  T sum[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int kz = 0; kz < 2; ++kz)
#pragma unroll
    for (int ky = 0; ky < 2; ++ky)
#pragma unroll
      for (int kx = 0; kx < 2; ++kx) {
        const bool ok = (kz ? v1[2] : v0[2]) && (ky ? v1[1] : v0[1]) && (kx ? v1[0] : v0[0]);
        if (!ok) continue;
        const int cell = ((kz ? c1[2] : c0[2]) * L.nc[1] + (ky ? c1[1] : c0[1])) * L.nc[0] + (kx ? c1[0] : c0[0]);
        const int l = (kx ? l1[0] : l0[0]) + 3 * (ky ? l1[1] : l0[1]) + 9 * (kz ? l1[2] : l0[2]);
#pragma unroll
        for (int c = 0; c < 3; ++c)
          if (!cons[c]) sum[c] += a.E[(size_t)cell * a.cs + (size_t)(c * 27 + l) * a.ss];
      }
#pragma unroll
  for (int c = 0; c < 3; ++c) gather_epilogue_dinv<T, epi>(a, (long)c * L.n_nodes + node, sum[c], cons[c], dv[c]);
}
// the diagonal inverse of the node's three DoFs (Chebyshev epilogues only)
template <typename T, int epi>
__device__ __forceinline__ void velocity_lattice_dinv(const LevelView<T>& L, const GatherArgs<T>& a, int node,
                                                      T (&dv)[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
    dv[c] = (epi == EPI_CHEB || epi == EPI_CHEB_OUT) ? a.dinv[(long)c * L.n_nodes + node] : T(0);
}
template <typename T, int epi>
__device__ __forceinline__ void velocity_lattice_node(const LevelView<T>& L, const GatherArgs<T>& a, int node) {
  T dv[3];
  velocity_lattice_dinv<T, epi>(L, a, node, dv);
  velocity_lattice_node_d<T, epi>(L, a, node, dv);
}
// The diagonal inverse (fixed over a V-cycle, written only by the preconditioner
// set-up) is loaded before pdl_wait, overlapping the preceding kernel in the
// V-cycle graphs' programmatic edges.
template <typename T, int epi>
__global__ void __launch_bounds__(256) velocity_gather_lattice3(LevelView<T> L, GatherArgs<T> a) {
  const int node = blockIdx.x * blockDim.x + threadIdx.x;
  T dv[3] = {T(0), T(0), T(0)};
  if (node < L.n_nodes) velocity_lattice_dinv<T, epi>(L, a, node, dv);
  pdl_wait();
  if (node >= L.n_nodes) return;
  velocity_lattice_node_d<T, epi>(L, a, node, dv);
}

// Pressure DoFs of a lattice level (never constrained there).
template <typename T, int dim, int epi>
__global__ void __launch_bounds__(256) pressure_gather_structured(LevelView<T> L, GatherArgs<T> a) {
  pdl_wait();
  constexpr int np = Shape<dim>::np;
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (g >= L.n_p) return;
  const int node = (int)g;
  const int gc[3] = {node % L.Np[0], (node / L.Np[0]) % L.Np[1], dim == 3 ? node / (L.Np[0] * L.Np[1]) : 0};
  int cidx[3][2], loc[3][2], cnt[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    cnt[d] = 0;
    if (d >= dim) { cnt[d] = 1; cidx[d][0] = 0; loc[d][0] = 0; continue; }
    const int x = gc[d];
    if (x > 0) { cidx[d][cnt[d]] = x - 1; loc[d][cnt[d]] = 1; ++cnt[d]; }
    if (x < L.Np[d] - 1) { cidx[d][cnt[d]] = x; loc[d][cnt[d]] = 0; ++cnt[d]; }
  }
  T sum = T(0);
  for (int kz = 0; kz < cnt[2]; ++kz)
    for (int ky = 0; ky < cnt[1]; ++ky)
      for (int kx = 0; kx < cnt[0]; ++kx) {
        const int cell = (cidx[2][kz] * L.nc[1] + cidx[1][ky]) * L.nc[0] + cidx[0][kx];
        const int l = loc[0][kx] + 2 * loc[1][ky] + 4 * loc[2][kz];
        sum += a.E[(size_t)cell * a.cs + (size_t)l * a.ss];
      }
  gather_epilogue<T, epi>(a, g, sum, false);
}

// Pressure mass operator of a lattice level in one pass, from the cells'
// precomputed local mass matrices (Mc[cell][i][j] = sum_q s^2/eta_q JxW_q
// psi_i psi_j). A pressure node touches at most 2^dim cells; each (node, cell)
// pair gets its own thread (2^dim consecutive lanes per node), which reads the
// node's row of that cell's matrix with vector loads and dots it with the
// cell's pressure values; the lanes of a node are summed with xor shuffles and
// the first lane runs the epilogue. (One thread per node left too few warps to
// hide the L2 latency of the 2^dim rows.) The operator reads x at neighbouring
// nodes, so a Chebyshev step writes its new iterate to a separate vector
// (EPI_CHEB_OUT).
constexpr int kMassLatticeThreads = 256;

// Task t = (node t / 2^dim, cell slot t % 2^dim). All 32 lanes of a warp must
// call it together (the lanes of a node are summed with shuffles); tasks past
// the last node only take part in the shuffles. In two parts: the operands that
// stay fixed over a whole V-cycle (the cell's mass-matrix row, the node's
// diagonal inverse) and then the dot with the iterate and the epilogue.
template <typename T, int dim>
struct MassLatticeRow {
  T r[Shape<dim>::np];
  T dinv;
  long g;
  int s, p0;
  bool ok, node_ok;
};
template <typename T, int dim, int epi>
__device__ __forceinline__ void mass_lattice_row(const LevelView<T>& L, const T* __restrict__ Mc,
                                                 const GatherArgs<T>& a, long t, MassLatticeRow<T, dim>& m) {
  constexpr int np = Shape<dim>::np;  // = lanes per node
  m.g = t / np;
  m.s = (int)(t % np);
  m.node_ok = m.g < L.n_p;
  const int node = m.node_ok ? (int)m.g : 0;
  const int gc[3] = {node % L.Np[0], (node / L.Np[0]) % L.Np[1], dim == 3 ? node / (L.Np[0] * L.Np[1]) : 0};
  // slot bit d = 0: the cell below the node along d (node at its local 1), 1: above (local 0)
  int c[3] = {0, 0, 0}, l = 0;
  bool ok = m.node_ok;
#pragma unroll
  for (int d = 0; d < dim; ++d) {
    const int bit = (m.s >> d) & 1;
    c[d] = gc[d] - 1 + bit;
    ok = ok && c[d] >= 0 && c[d] < L.nc[d];
    l += (bit ? 0 : 1) << d;
  }
  m.ok = ok;
  m.p0 = (c[2] * L.Np[1] + c[1]) * L.Np[0] + c[0];
  if (ok) {
    const int cell = (c[2] * L.nc[1] + c[1]) * L.nc[0] + c[0];
    load_row<T, np>(Mc + ((size_t)cell * np + l) * np, m.r);
  }
  m.dinv = T(0);
  if ((epi == EPI_CHEB || epi == EPI_CHEB_OUT) && m.node_ok && m.s == 0) m.dinv = a.dinv[m.g];
}
template <typename T, int dim, int epi>
__device__ __forceinline__ void mass_lattice_dot(const LevelView<T>& L, const GatherArgs<T>& a,
                                                 const MassLatticeRow<T, dim>& m) {
  constexpr int np = Shape<dim>::np;
  T sum = T(0);
  if (m.ok) {
    const T* __restrict__ xin = a.x;
#pragma unroll
    for (int j = 0; j < np; ++j) sum += m.r[j] * xin[m.p0 + structured_pnode_offset<dim>(L.Np, j)];
  }
#pragma unroll
  for (int o = 1; o < np; o <<= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (m.node_ok && m.s == 0) gather_epilogue_dinv<T, epi>(a, m.g, sum, false, m.dinv);
}
template <typename T, int dim, int epi>
__device__ __forceinline__ void mass_lattice_task(const LevelView<T>& L, const T* __restrict__ Mc,
                                                  const GatherArgs<T>& a, long t) {
  MassLatticeRow<T, dim> m;
  mass_lattice_row<T, dim, epi>(L, Mc, a, t, m);
  mass_lattice_dot<T, dim, epi>(L, a, m);
}

// The fixed operands are loaded before pdl_wait: in the V-cycle graphs, whose
// kernel edges are programmatic, that load overlaps the preceding kernel (the
// mass matrices and diagonals are written only by the preconditioner set-up,
// before any V-cycle runs).
template <typename T, int dim, int epi>
__global__ void __launch_bounds__(kMassLatticeThreads) mass_apply_lattice(LevelView<T> L, const T* __restrict__ Mc,
                                                                          GatherArgs<T> a) {
  MassLatticeRow<T, dim> m;
  mass_lattice_row<T, dim, epi>(L, Mc, a, blockIdx.x * (long)blockDim.x + threadIdx.x, m);
  pdl_wait();
  mass_lattice_dot<T, dim, epi>(L, a, m);
}

template <typename T, int epi>
__global__ void __launch_bounds__(256) gather_csr(long n, GatherCsr<T> G, GatherArgs<T> a) {
  pdl_wait();
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (g >= n) return;
  const bool constrained = G.cmask[g] != 0;
  T sum = T(0);
  if (!constrained)
    for (int k = G.ptr[g]; k < G.ptr[g + 1]; ++k) sum += G.w[k] * a.E[G.slot[k]];
  gather_epilogue<T, epi>(a, g, sum, constrained);
}

// ---------------------------------------------------------------------------
// Diagonals (MatrixFreeTools::compute_diagonal semantics): for every global DoF
// g touched by a cell, v = local expansion of e_g, diag[g] += v . (K_cell v).
// General levels use per-cell probe lists: probe k = (global dof, entries
// (local index, weight)). Structured levels probe each unconstrained local DoF.
template <typename T, int dim>
__global__ void __launch_bounds__(128) velocity_diag_kernel(LevelView<T> L, int colour, int colour_begin,
                                                             int colour_count, const int* __restrict__ probe_ptr,
                                                             const int* __restrict__ probe_g,
                                                             const int* __restrict__ probe_eptr,
                                                             const int* __restrict__ probe_li,
                                                             const T* __restrict__ probe_w, T* __restrict__ diag) {
  pdl_wait();
  constexpr int nv = Shape<dim>::nv, cpw = Shape<dim>::cpw;
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
  // number of probes is uniform within a warp only for structured levels; loop to
  // the maximum over the warp so that every lane takes part in the shuffles
  int my_probes = 0, p0 = 0;
  if (L.structured) my_probes = dim * nv;
  else if (active) { p0 = probe_ptr[cell]; my_probes = probe_ptr[cell + 1] - p0; }
  int max_probes = my_probes;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) max_probes = max(max_probes, __shfl_xor_sync(0xffffffffu, max_probes, o));
  for (int k = 0; k < max_probes; ++k) {
    T U[nv], V[nv];
    bool probe_ok = active && k < my_probes;
    int target = -1;
#pragma unroll
    for (int n = 0; n < nv; ++n) U[n] = T(0);
    if (probe_ok) {
      if (L.structured) {
        const int pc = k / nv, pn = k % nv;
        if (structured_zero<T, dim>(L, sc, pc, pn)) probe_ok = false;
        else {
#pragma unroll
          for (int n = 0; n < nv; ++n) U[n] = (pc == comp && pn == n) ? T(1) : T(0);
          target = pc * L.n_nodes + sc.node0 + structured_node_offset<dim>(L.Nn, pn);
        }
      } else {
        target = probe_g[p0 + k];
        for (int e = probe_eptr[p0 + k]; e < probe_eptr[p0 + k + 1]; ++e) {
          const int li = probe_li[e];
          const T w = probe_w[e];
#pragma unroll
          for (int n = 0; n < nv; ++n)
            if (li == comp * nv + n) U[n] += w;
        }
      }
    }
    T Uc[nv];
#pragma unroll
    for (int n = 0; n < nv; ++n) Uc[n] = U[n];
    velocity_cell_op<T, dim, OPK_A>(L, cell, comp, lane_base, U, nullptr, V, nullptr, box, eta_cell, eta_q);
    T part = T(0);
#pragma unroll
    for (int n = 0; n < nv; ++n) part += Uc[n] * V[n];
    T tot = part;
#pragma unroll
    for (int o = 1; o < dim; ++o) tot += __shfl_sync(0xffffffffu, part, lane_base + (comp + o) % dim);
    // all probes of structured levels have one owner thread (component pc)
    const bool owner = L.structured ? (k / nv == comp) : (comp == 0);
    if (probe_ok && owner && target >= 0) diag[target] += tot;
  }
}

// A-block diagonal of lattice levels, directly: for the local DoF (component c,
// node n), 2 eta eps(phi):eps(phi) = eta (|grad phi_n|^2 + kappa (d_c phi_n)^2)
// with kappa = 1 (kappa = 1/3 with the compressible term), so
//   K_cell[(c,n),(c,n)] = |det J| sum_e ih_e^2 A_e(n) + kappa |det J| ih_c^2 A_c(n),
//   A_e(n) = sum_q w_q eta_q (d phi_n / d xi_e (q))^2,
// 27 x 27 FMAs per direction with compile-time coefficients instead of 81
// applications of the cell operator. Thread `comp` of a cell accumulates
// A_comp(n) for all n; the three threads exchange them by shuffles and thread
// comp writes the diagonal of its component. Constrained local DoFs get 0 (the
// caller sets constrained rows). Output layout as the operator's cell pass
// (slot-major E[slot][cell] or cell-major E[cell][slot]), so the level's gather
// sums it into nodes.
__host__ __device__ constexpr double q2_deriv_at_gauss(int q, int n) {
  // phi_0' = 4x - 3, phi_1' = 4 - 8x, phi_2' = 4x - 1 at x = 1/2 + (q - 1) sqrt(15)/10
  return n == 0 ? 4.0 * (0.5 + (q - 1) * fe::SQ15 / 10) - 3.0
       : n == 1 ? 4.0 - 8.0 * (0.5 + (q - 1) * fe::SQ15 / 10)
                : 4.0 * (0.5 + (q - 1) * fe::SQ15 / 10) - 1.0;
}
template <int dim, int e, int n, int q>
__host__ __device__ constexpr double diag_weight() {
  double g = 1.0;
  for (int d = 0; d < dim; ++d) {
    const int qd = (q / fe::pow3(d)) % 3, nd = (n / fe::pow3(d)) % 3;
    g *= d == e ? q2_deriv_at_gauss(qd, nd) : fe::Sv(qd, nd);
  }
  return g * g * qweight<dim, q>();
}

template <typename T, int dim>
__global__ void __launch_bounds__(128) lattice_diag_kernel(LevelView<T> L, T* __restrict__ Eu, int slot_major) {
  pdl_wait();
  constexpr int nv = Shape<dim>::nv, cpw = Shape<dim>::cpw;
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
  StructuredCell<T, dim> sc;
  structured_cell_lex<T, dim>(L, cell, sc);
  const bool per_q = L.eta_n != 1;
  const T eta_cell = per_q ? T(0) : L.eta[cell];
  const T* __restrict__ eq = per_q ? L.eta + (size_t)cell * nv : L.eta;
  T acc[nv];
#pragma unroll
  for (int n = 0; n < nv; ++n) acc[n] = T(0);
  static_for<nv>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const T eta = per_q ? eq[q] : eta_cell;
    static_for<nv>([&](auto nc) {
      constexpr int n = decltype(nc)::value;
      T w;
      if constexpr (dim == 3)
        w = sel3(T(diag_weight<3, 0, n, q>()), T(diag_weight<3, 1, n, q>()), T(diag_weight<3, 2, n, q>()), comp);
      else
        w = comp == 0 ? T(diag_weight<2, 0, n, q>()) : T(diag_weight<2, 1, n, q>());
      acc[n] += eta * w;
    });
  });
  const T kappa = L.compressible ? T(1.0 / 3.0) : T(1);
  T ih2[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) ih2[d] = d < dim ? L.inv_h[d] * L.inv_h[d] : T(0);
  const T own = (T(1) + kappa) * (dim == 3 ? sel3(ih2[0], ih2[1], ih2[2], comp) : (comp == 0 ? ih2[0] : ih2[1]));
  const T w1 = dim == 3 ? sel3(ih2[1], ih2[2], ih2[0], comp) : (comp == 0 ? ih2[1] : ih2[0]);
  const T w2 = dim == 3 ? sel3(ih2[2], ih2[0], ih2[1], comp) : T(0);
#pragma unroll
  for (int n = 0; n < nv; ++n) {
    const T a1 = __shfl_sync(full, acc[n], lb + (comp + 1) % dim);
    T v = own * acc[n] + w1 * a1;
    if constexpr (dim == 3) v += w2 * __shfl_sync(full, acc[n], lb + (comp + 2) % dim);
    v *= L.det;
    if (active) {
      const int slot = comp * nv + n;
      Eu[slot_major ? (size_t)slot * L.n_cells + cell : (size_t)cell * dim * nv + slot] =
          structured_zero<T, dim>(L, sc, comp, n) ? T(0) : v;
    }
  }
}

template <typename T, int dim>
__global__ void __launch_bounds__(128) mass_diag_kernel(LevelView<T> L, int colour, int colour_begin,
                                                         int colour_count, const int* __restrict__ probe_ptr,
                                                         const int* __restrict__ probe_g,
                                                         const int* __restrict__ probe_eptr,
                                                         const int* __restrict__ probe_li,
                                                         const T* __restrict__ probe_w, T* __restrict__ diag) {
  pdl_wait();
  constexpr int np = Shape<dim>::np;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= colour_count) return;
  int cell;
  StructuredCell<T, dim> sc{};
  if (L.structured) {
    bool v;
    structured_cell<T, dim>(L, colour, idx, cell, sc, v);
    if (!v) return;
  } else {
    cell = colour_begin + idx;
  }
  T box[4] = {T(0), T(0), T(0), T(0)};
  if (L.geom == GEOM_BOX)
#pragma unroll
    for (int d = 0; d <= dim; ++d) box[d] = L.gbox[(size_t)cell * (dim + 1) + d];
  const T eta_cell = L.eta_n == 1 ? L.eta[cell] : T(1);
  const T* eta_q = L.eta_n == 1 ? nullptr : L.eta + (size_t)cell * L.eta_n;
  int n_probes = L.structured ? np : probe_ptr[cell + 1] - probe_ptr[cell];
  const int p0 = L.structured ? 0 : probe_ptr[cell];
  for (int k = 0; k < n_probes; ++k) {
    T P[np], YP[np];
    int target;
#pragma unroll
    for (int n = 0; n < np; ++n) P[n] = T(0);
    if (L.structured) {
#pragma unroll
      for (int n = 0; n < np; ++n) P[n] = n == k ? T(1) : T(0);
      target = sc.pnode0 + structured_pnode_offset<dim>(L.Np, k);
    } else {
      target = probe_g[p0 + k];
      for (int e = probe_eptr[p0 + k]; e < probe_eptr[p0 + k + 1]; ++e) {
        const int li = probe_li[e];
#pragma unroll
        for (int n = 0; n < np; ++n)
          if (li == n) P[n] += probe_w[e];
      }
    }
    mass_cell_op<T, dim>(L, cell, P, YP, box, eta_cell, eta_q);
    T tot = T(0);
#pragma unroll
    for (int n = 0; n < np; ++n) tot += P[n] * YP[n];
    diag[target] += tot;
  }
}

}  // namespace gb
