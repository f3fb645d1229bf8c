// Cell operators of higher velocity degree (Q3 velocity, Q2 pressure, QGauss(4);
// the reference's degree-3 instantiation, source/simulator/solver/
// stokes_matrix_free.cc:39-40,53-54), on general (indexed) levels.
//
// Same physics per quadrature point as the Q2 kernels
// (matrix_free_operators.cc:376-547 Stokes, :668-701 B^T, :787-845 mass,
// :974-1009 A block), laid out for 64 (27 in 2D: 16) nodes per component:
// one thread group of (degree+1)^dim threads per cell, the tensor-product sum
// factorisation done through shared memory. Per component the nodal values are
// taken to the Gauss points (one sweep per direction with S(q, n) = phi_n(x_q)),
// the reference gradient is the collocation derivative there (D(q, m) =
// l_m'(x_q), l the Lagrange polynomials on the Gauss points), each thread forms
// the flux of its point, and the transposed sweeps integrate back to the nodes.
// The Q2 pressure goes to the points and back through Sp(q, n) = psi_n(x_q).
// Output: the per-cell contributions of the two-pass operator (cell-major), so
// the level's CSR gather distributes them through the constraints.
//
// Diagonals (MatrixFreeTools::compute_diagonal semantics) use the same cell
// operator on probe vectors: per cell and unconstrained DoF it touches, the
// constraint expansion of that DoF restricted to the cell, K_cell applied, and
// the probe-weighted sum added to the DoF's diagonal. One launch per cell
// colour; within a colour every (cell, probe) pair writes its own DoF.
#include "level.cuh"

namespace gb {
namespace {

constexpr int kHoThreads = 128;
constexpr int kMaxN1 = 4;  // points / velocity nodes per direction

template <typename T>
struct HOBasis {
  T S[kMaxN1][kMaxN1];   // velocity basis at the Gauss points [q][n]
  T D[kMaxN1][kMaxN1];   // collocation derivative on the Gauss points [q][m]
  T Sp[kMaxN1][kMaxN1];  // pressure basis at the Gauss points [q][n] (n < N1 - 1)
  T w[kMaxN1];           // Gauss weights on [0, 1]
};

// One tensor-product sweep along axis `ax` over an item's array: extents
// (e0, e1, e2) in, the axis' extent becomes `eo` out. Forward (TR = false):
// out(.., r, ..) = sum_k M[r][k] in(.., k, ..); transposed: sum_k M[k][r].
// The item's nt threads split the outputs.
template <typename T, int K, bool TR, bool ADD>
__device__ __forceinline__ void sweep(const T (*M)[kMaxN1], const T* __restrict__ in, T* __restrict__ out, int ax,
                                      int e0, int e1, int e2, int eo, int tid, int nt) {
  const int o0 = ax == 0 ? eo : e0, o1 = ax == 1 ? eo : e1, o2 = ax == 2 ? eo : e2;
  const int osize = o0 * o1 * o2;
  const int s_ax = ax == 0 ? 1 : ax == 1 ? e0 : e0 * e1;
  for (int o = tid; o < osize; o += nt) {
    const int i0 = o % o0, i1 = (o / o0) % o1, i2 = o / (o0 * o1);
    const int r = ax == 0 ? i0 : ax == 1 ? i1 : i2;
    const int base = (ax == 0 ? 0 : i0) + (ax == 1 ? 0 : i1 * e0) + (ax == 2 ? 0 : i2 * e0 * e1);
    T acc = ADD ? out[o] : T(0);
#pragma unroll
    for (int k = 0; k < K; ++k) acc += (TR ? M[k][r] : M[r][k]) * in[base + k * s_ax];
    out[o] = acc;
  }
}

template <typename T, int dim, int N1>
struct HoShape {
  static constexpr int nq = N1 * N1 * (dim == 3 ? N1 : 1);   // points = velocity nodes per component
  static constexpr int npn = N1 - 1;                          // pressure nodes per direction
  static constexpr int np = npn * npn * (dim == 3 ? npn : 1);
  static constexpr int items = kHoThreads / nq;               // cells per block
  // per item: U, W (dim x nq each), G (dim x dim x nq), P, Q (nq each)
  static constexpr int smem = (2 * dim + dim * dim + 2) * nq;
};

// the item's cell operator: inputs in U (velocity, dim x nq nodal) and P
// (pressure, np nodal); outputs in W (velocity, dim x nq nodal) and Q (pressure,
// np nodal). Every thread of the block calls it (barriers inside).
template <typename T, int dim, int N1, int op>
__device__ void ho_cell_op(const LevelView<T>& L, const HOBasis<T>& B, int cell, bool active, T* U, T* W, T* G,
                           T* P, T* Q, int tid) {
  using S = HoShape<T, dim, N1>;
  constexpr int nq = S::nq, npn = S::npn;
  constexpr bool need_u = op == OPK_STOKES || op == OPK_A;
  constexpr bool need_p = op != OPK_A;
  constexpr bool out_u = op != OPK_MASS;
  constexpr bool out_p = op == OPK_STOKES || op == OPK_MASS;
  const int e2 = dim == 3 ? N1 : 1;
  // --- velocity to the points: U -> (W, U alternating), then gradients into G
  if (need_u) {
    T* a = U;
    T* b = W;
#pragma unroll
    for (int ax = 0; ax < dim; ++ax) {
#pragma unroll
      for (int c = 0; c < dim; ++c) sweep<T, N1, false, false>(B.S, a + c * nq, b + c * nq, ax, N1, N1, e2, N1, tid, nq);
      __syncthreads();
      T* t = a; a = b; b = t;
    }
    // point values now in `a`; G[c][e] = D along e
#pragma unroll
    for (int c = 0; c < dim; ++c)
#pragma unroll
      for (int e = 0; e < dim; ++e)
        sweep<T, N1, false, false>(B.D, a + c * nq, G + (c * dim + e) * nq, e, N1, N1, e2, N1, tid, nq);
  }
  // --- pressure to the points: P (np) -> Q -> P -> (Q): extents grow axis by axis
  T* pq_arr = P;
  if (need_p) {
    T* a = P;
    T* b = Q;
    int x0 = npn, x1 = npn, x2 = dim == 3 ? npn : 1;
#pragma unroll
    for (int ax = 0; ax < dim; ++ax) {
      sweep<T, N1 - 1, false, false>(B.Sp, a, b, ax, x0, x1, x2, N1, tid, nq);
      __syncthreads();
      if (ax == 0) x0 = N1; else if (ax == 1) x1 = N1; else x2 = N1;
      T* t = a; a = b; b = t;
    }
    pq_arr = a;
  }
  __syncthreads();
  // --- point operation: thread tid owns point q = tid
  T pres = T(0);
  {
    const int q = tid;
    const int q0 = q % N1, q1 = (q / N1) % N1, q2 = dim == 3 ? q / (N1 * N1) : 0;
    T wq = B.w[q0] * B.w[q1];
    if (dim == 3) wq *= B.w[q2];
    T iJ[dim][dim];
    T jxw;
    if (!active) {
#pragma unroll
      for (int d = 0; d < dim; ++d)
#pragma unroll
        for (int e = 0; e < dim; ++e) iJ[d][e] = T(0);
      jxw = T(0);
    } else if (L.geom == GEOM_TABLE) {
      const T* t = L.gtab + ((size_t)cell * nq + q) * (dim * dim + 1);
#pragma unroll
      for (int d = 0; d < dim; ++d)
#pragma unroll
        for (int e = 0; e < dim; ++e) iJ[d][e] = t[d * dim + e];
      jxw = t[dim * dim] * wq;
    } else {
      const T* bx = L.gbox + (size_t)cell * (dim + 1);
#pragma unroll
      for (int d = 0; d < dim; ++d)
#pragma unroll
        for (int e = 0; e < dim; ++e) iJ[d][e] = d == e ? bx[d] : T(0);
      jxw = bx[dim] * wq;
    }
    const T eta = active ? (L.eta_n == 1 ? L.eta[cell] : L.eta[(size_t)cell * L.eta_n + q]) : T(1);
    const T s = L.s;
    const T p = need_p ? pq_arr[q] : T(0);
    if (op == OPK_MASS) {
      pres = s * s / eta * p * jxw;
    } else {
      // physical gradient g[c][e] = sum_d Gref[c][d] iJ[d][e]
      T g[dim][dim];
      T div = T(0);
#pragma unroll
      for (int c = 0; c < dim; ++c)
#pragma unroll
        for (int e = 0; e < dim; ++e) {
          T t = T(0);
          if (need_u)
#pragma unroll
            for (int d = 0; d < dim; ++d) t += G[(c * dim + d) * nq + q] * iJ[d][e];
          g[c][e] = t;
        }
#pragma unroll
      for (int c = 0; c < dim; ++c) div += g[c][c];
      T F[dim][dim];
#pragma unroll
      for (int c = 0; c < dim; ++c)
#pragma unroll
        for (int e = 0; e < dim; ++e) {
          T f = need_u ? (c == e ? T(2) * eta * g[c][c] : eta * (g[c][e] + g[e][c])) : T(0);
          if (c == e) {
            if (need_u && L.compressible) f -= T(2) * eta / T(3) * div;
            if (need_p) f -= s * p;
          }
          F[c][e] = f;
        }
      __syncthreads();  // every thread has read G before it is overwritten
#pragma unroll
      for (int c = 0; c < dim; ++c)
#pragma unroll
        for (int d = 0; d < dim; ++d) {
          T t = T(0);
#pragma unroll
          for (int e = 0; e < dim; ++e) t += F[c][e] * iJ[d][e];
          G[(c * dim + d) * nq + q] = t * jxw;
        }
      if (op == OPK_STOKES) pres = -s * jxw * div;
    }
  }
  if (op == OPK_MASS || op == OPK_BT) __syncthreads();  // pq_arr read by all before reuse
  if (out_p) pq_arr[tid] = pres;
  __syncthreads();
  // --- velocity back to the nodes: W[c] = sum_e D_e^T G[c][e], then S^T sweeps
  if (out_u) {
#pragma unroll
    for (int e = 0; e < dim; ++e) {
#pragma unroll
      for (int c = 0; c < dim; ++c) {
        if (e == 0) sweep<T, N1, true, false>(B.D, G + (c * dim + e) * nq, W + c * nq, e, N1, N1, e2, N1, tid, nq);
        else sweep<T, N1, true, true>(B.D, G + (c * dim + e) * nq, W + c * nq, e, N1, N1, e2, N1, tid, nq);
      }
      __syncthreads();
    }
    T* a = W;
    T* b = U;
#pragma unroll
    for (int ax = 0; ax < dim; ++ax) {
#pragma unroll
      for (int c = 0; c < dim; ++c) sweep<T, N1, true, false>(B.S, a + c * nq, b + c * nq, ax, N1, N1, e2, N1, tid, nq);
      __syncthreads();
      T* t = a; a = b; b = t;
    }
    // result in `a`: W after an even number of sweeps, U after an odd one
    if (a != W) {
#pragma unroll
      for (int c = 0; c < dim; ++c) W[c * nq + tid] = a[c * nq + tid];
      __syncthreads();
    }
  }
  // --- pressure back to the nodes: extents shrink axis by axis, result in Q
  if (out_p) {
    T* a = pq_arr;
    T* b = pq_arr == P ? Q : P;
    int x0 = N1, x1 = N1, x2 = dim == 3 ? N1 : 1;
#pragma unroll
    for (int ax = 0; ax < dim; ++ax) {
      sweep<T, N1, true, false>(B.Sp, a, b, ax, x0, x1, x2, npn, tid, nq);
      __syncthreads();
      if (ax == 0) x0 = npn; else if (ax == 1) x1 = npn; else x2 = npn;
      T* t = a; a = b; b = t;
    }
    if (a != Q) {
      if (tid < S::np) Q[tid] = a[tid];
      __syncthreads();
    }
  }
}

template <typename T, int dim, int N1>
__device__ __forceinline__ void load_basis(const HOBasis<T>& src, HOBasis<T>& dst) {
  const T* s = reinterpret_cast<const T*>(&src);
  T* d = reinterpret_cast<T*>(&dst);
  for (int i = threadIdx.x; i < (int)(sizeof(HOBasis<T>) / sizeof(T)); i += blockDim.x) d[i] = s[i];
}

template <typename T, int dim, int N1, int op>
__global__ void __launch_bounds__(kHoThreads) ho_cell_kernel(LevelView<T> L, HOBasis<T> Bp,
                                                             const T* __restrict__ src_u, const T* __restrict__ src_p,
                                                             T* __restrict__ Eu, T* __restrict__ Ep) {
  pdl_wait();
  using S = HoShape<T, dim, N1>;
  constexpr int nq = S::nq, np = S::np;
  __shared__ HOBasis<T> B;
  __shared__ T sm[S::items * S::smem];
  load_basis<T, dim, N1>(Bp, B);
  const int item = threadIdx.x / nq, tid = threadIdx.x - item * nq;
  const int cell = blockIdx.x * S::items + item;
  const bool active = cell < L.n_cells;
  T* U = sm + item * S::smem;
  T* W = U + dim * nq;
  T* G = W + dim * nq;
  T* P = G + dim * dim * nq;
  T* Q = P + nq;
  constexpr bool need_u = op == OPK_STOKES || op == OPK_A;
  constexpr bool need_p = op != OPK_A;
  if (need_u)
#pragma unroll
    for (int c = 0; c < dim; ++c)
      U[c * nq + tid] = active ? gather_general(src_u, L.cdu[(size_t)cell * dim * nq + c * nq + tid], L.lptr, L.lcol, L.lw)
                               : T(0);
  if (need_p && tid < np)
    P[tid] = active ? gather_general(src_p, L.cdp[(size_t)cell * np + tid], L.plptr, L.plcol, L.plw) : T(0);
  __syncthreads();
  ho_cell_op<T, dim, N1, op>(L, B, cell, active, U, W, G, P, Q, tid);
  if (!active) return;
  if (op != OPK_MASS)
#pragma unroll
    for (int c = 0; c < dim; ++c) Eu[(size_t)cell * dim * nq + c * nq + tid] = W[c * nq + tid];
  if ((op == OPK_STOKES || op == OPK_MASS) && tid < np) Ep[(size_t)cell * np + tid] = Q[tid];
}

// block 0: A-block diagonal, block 1: mass diagonal. Items = the probes of the
// colour's cells [probe_ptr[begin], probe_ptr[begin + count]).
template <typename T, int dim, int N1, int block>
__global__ void __launch_bounds__(kHoThreads) ho_diag_kernel(LevelView<T> L, HOBasis<T> Bp, int begin, int count,
                                                             ProbesView<T> pr, T* __restrict__ diag) {
  pdl_wait();
  using S = HoShape<T, dim, N1>;
  constexpr int nq = S::nq, np = S::np;
  constexpr int op = block == 0 ? OPK_A : OPK_MASS;
  __shared__ HOBasis<T> B;
  __shared__ T sm[S::items * S::smem];
  __shared__ T part[kHoThreads];
  load_basis<T, dim, N1>(Bp, B);
  const int item = threadIdx.x / nq, tid = threadIdx.x - item * nq;
  const int p_lo = pr.ptr[begin], p_hi = pr.ptr[begin + count];
  const int probe = p_lo + blockIdx.x * S::items + item;
  const bool active = probe < p_hi;
  // the probe's cell: last c in [begin, begin + count) with ptr[c] <= probe
  int cell = begin;
  if (active) {
    int lo = begin, hi = begin + count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (pr.ptr[mid] <= probe) lo = mid; else hi = mid - 1;
    }
    cell = lo;
  }
  T* U = sm + item * S::smem;
  T* W = U + dim * nq;
  T* G = W + dim * nq;
  T* P = G + dim * dim * nq;
  T* Q = P + nq;
  const int nin = block == 0 ? dim * nq : np;
  T* in = block == 0 ? U : P;
  for (int i = tid; i < nin; i += nq) in[i] = T(0);
  __syncthreads();
  const int e_lo = active ? pr.eptr[probe] : 0, e_hi = active ? pr.eptr[probe + 1] : 0;
  for (int e = e_lo + tid; e < e_hi; e += nq) in[pr.li[e]] = pr.w[e];
  __syncthreads();
  ho_cell_op<T, dim, N1, op>(L, B, cell, active, U, W, G, P, Q, tid);
  const T* out = block == 0 ? W : Q;
  T acc = T(0);
  for (int e = e_lo + tid; e < e_hi; e += nq) acc += pr.w[e] * out[pr.li[e]];
  part[threadIdx.x] = acc;
  __syncthreads();
  if (active && tid == 0) {
    T sum = T(0);
    for (int k = 0; k < nq; ++k) sum += part[item * nq + k];
    diag[pr.g[probe]] += sum;
  }
}

// 1D matrices of a velocity degree in precision T
template <typename T>
HOBasis<T> make_basis(int degree) {
  const Basis1D b = basis1d(degree);
  HOBasis<T> B{};
  for (int q = 0; q < b.nq1; ++q) {
    double v[4], d[4];
    lagrange_basis(b.vn, b.nvn, b.gq[q], v, d);
    for (int n = 0; n < b.nvn; ++n) B.S[q][n] = (T)v[n];
    lagrange_basis(b.gq, b.nq1, b.gq[q], v, d);
    for (int m = 0; m < b.nq1; ++m) B.D[q][m] = (T)d[m];
    lagrange_basis(b.pn, b.npn, b.gq[q], v, d);
    for (int n = 0; n < b.npn; ++n) B.Sp[q][n] = (T)v[n];
    B.w[q] = (T)b.gw[q];
  }
  return B;
}

template <typename T, int dim, int N1>
void cell_pass(const LevelView<T>& L, int op, const T* su, const T* sp, T* Eu, T* Ep, cudaStream_t s) {
  using S = HoShape<T, dim, N1>;
  const HOBasis<T> B = make_basis<T>(N1 - 1);
  const int g = ceil_div(L.n_cells, S::items);
  if (op == OPK_STOKES) ho_cell_kernel<T, dim, N1, OPK_STOKES><<<g, kHoThreads, 0, s>>>(L, B, su, sp, Eu, Ep);
  else if (op == OPK_A) ho_cell_kernel<T, dim, N1, OPK_A><<<g, kHoThreads, 0, s>>>(L, B, su, sp, Eu, Ep);
  else if (op == OPK_BT) ho_cell_kernel<T, dim, N1, OPK_BT><<<g, kHoThreads, 0, s>>>(L, B, su, sp, Eu, Ep);
  else ho_cell_kernel<T, dim, N1, OPK_MASS><<<g, kHoThreads, 0, s>>>(L, B, su, sp, Eu, Ep);
}

template <typename T, int dim, int N1>
void diag_pass(const LevelView<T>& L, int block, int begin, int count, const ProbesView<T>& pr, int n_probes, T* diag,
               cudaStream_t s) {
  using S = HoShape<T, dim, N1>;
  const HOBasis<T> B = make_basis<T>(N1 - 1);
  const int g = ceil_div(n_probes, S::items);
  if (block == 0) ho_diag_kernel<T, dim, N1, 0><<<g, kHoThreads, 0, s>>>(L, B, begin, count, pr, diag);
  else ho_diag_kernel<T, dim, N1, 1><<<g, kHoThreads, 0, s>>>(L, B, begin, count, pr, diag);
}

}  // namespace

template <typename T>
void launch_ho_cell_pass(const LevelView<T>& L, int op, const T* su, const T* sp, T* Eu, T* Ep, cudaStream_t s) {
  if (L.n_cells <= 0) return;
  GB_CHECK(L.deg == 3 && !L.structured, 1, "higher-degree cell pass: degree 3 on an indexed level");
  if (L.dim == 3) cell_pass<T, 3, 4>(L, op, su, sp, Eu, Ep, s);
  else cell_pass<T, 2, 4>(L, op, su, sp, Eu, Ep, s);
  GB_CUDA(cudaGetLastError());
}

template <typename T>
void launch_ho_diag(const LevelView<T>& L, int block, int begin, int count, const ProbesView<T>& pr, int n_probes,
                    T* diag, cudaStream_t s) {
  if (n_probes <= 0) return;
  if (L.dim == 3) diag_pass<T, 3, 4>(L, block, begin, count, pr, n_probes, diag, s);
  else diag_pass<T, 2, 4>(L, block, begin, count, pr, n_probes, diag, s);
  GB_CUDA(cudaGetLastError());
}

template void launch_ho_cell_pass<double>(const LevelView<double>&, int, const double*, const double*, double*,
                                          double*, cudaStream_t);
template void launch_ho_cell_pass<float>(const LevelView<float>&, int, const float*, const float*, float*, float*,
                                         cudaStream_t);
template void launch_ho_diag<double>(const LevelView<double>&, int, int, int, const ProbesView<double>&, int, double*,
                                     cudaStream_t);
template void launch_ho_diag<float>(const LevelView<float>&, int, int, int, const ProbesView<float>&, int, float*,
                                    cudaStream_t);

}  // namespace gb
