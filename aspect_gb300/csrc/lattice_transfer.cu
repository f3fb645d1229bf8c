// Matrix-free level transfers of structured levels (see lattice_transfer.cuh).
#include "lattice_transfer.cuh"
#include "vec.cuh"

namespace gb {
namespace {

constexpr int kXferThreads = 256;

__device__ __forceinline__ void node_xyz(long node, const int* N, int& x, int& y, int& z) {
  x = (int)(node % N[0]);
  y = (int)((node / N[0]) % N[1]);
  z = (int)(node / ((long)N[0] * N[1]));
}

// 1D stencil of one direction as M fixed candidate slots (weights in the
// vector's type: they are dyadic, so their products are exact in FP32 as in
// FP64, the values of the CSR entries), a slot used when its node exists and is
// not on a zero face of component comp; fully unrolled loops keep it in
// registers. The used slots are in increasing node order, as the lattice_r1d /
// lattice_p1d lists are.
template <typename T, int M>
struct Stencil1D {
  int idx[M];
  T w[M];
  bool ok[M];
};
template <typename T, int M>
__device__ __forceinline__ void stencil_dir(bool restrict_, int q2, int i, int N, uint32_t zf, int d, int comp,
                                            Stencil1D<T, M>& s) {
  int c[5] = {0, 0, 0, 0, 0};
  double w[5] = {0, 0, 0, 0, 0};
  bool v[5] = {false, false, false, false, false};
  if (N == 1) {
    v[0] = true;
    w[0] = 1.0;
  } else if (restrict_) {  // fine nodes of coarse node i
    if (!q2) {
      c[0] = 2 * i - 1; c[1] = 2 * i; c[2] = 2 * i + 1;
      w[0] = 0.5; w[1] = 1.0; w[2] = 0.5;
      v[0] = v[1] = v[2] = true;
    } else if (!(i & 1)) {
      const int q = i >> 1;
      c[0] = 4 * q - 3; c[1] = 4 * q - 1; c[2] = 4 * q; c[3] = 4 * q + 1; c[4] = 4 * q + 3;
      w[0] = -0.125; w[1] = 0.375; w[2] = 1.0; w[3] = 0.375; w[4] = -0.125;
      v[0] = v[1] = v[2] = v[3] = v[4] = true;
    } else {
      const int q = i >> 1;
      c[0] = 4 * q + 1; c[1] = 4 * q + 2; c[2] = 4 * q + 3;
      w[0] = 0.75; w[1] = 1.0; w[2] = 0.75;
      v[0] = v[1] = v[2] = true;
    }
  } else {  // coarse nodes of fine node i
    if (!q2) {
      c[0] = i >> 1; c[1] = (i >> 1) + 1;
      if (i & 1) { w[0] = 0.5; w[1] = 0.5; v[0] = v[1] = true; }
      else { w[0] = 1.0; v[0] = true; }
    } else {
      const int q = i >> 2, r = i & 3;
      if (r == 0 || r == 2) {
        c[0] = 2 * q + (r >> 1); w[0] = 1.0; v[0] = true;
      } else {
        c[0] = 2 * q; c[1] = 2 * q + 1; c[2] = 2 * q + 2;
        w[0] = r == 1 ? 0.375 : -0.125; w[1] = 0.75; w[2] = r == 1 ? -0.125 : 0.375;
        v[0] = v[1] = v[2] = true;
      }
    }
  }
  const bool lo = (zf >> ((2 * d) * 3 + comp)) & 1u, hi = (zf >> ((2 * d + 1) * 3 + comp)) & 1u;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    s.idx[k] = c[k];
    s.w[k] = (T)w[k];
    s.ok[k] = v[k] && c[k] >= 0 && c[k] < N && !(q2 && N > 1 && ((lo && c[k] == 0) || (hi && c[k] == N - 1)));
  }
}

// the stencil sum in z, y, x order (the CSR row order)
template <typename T, int M>
__device__ __forceinline__ T stencil_sum(const Stencil1D<T, M>& sx, const Stencil1D<T, M>& sy,
                                         const Stencil1D<T, M>& sz, const T* __restrict__ src, int Nx, int Ny) {
  T t = T(0);
#pragma unroll
  for (int c = 0; c < M; ++c) {
    if (!sz.ok[c]) continue;
#pragma unroll
    for (int b = 0; b < M; ++b) {
      if (!sy.ok[b]) continue;
      const T wyz = sy.w[b] * sz.w[c];
      const T* __restrict__ row = src + ((long)sz.idx[c] * Ny + sy.idx[b]) * Nx;
#pragma unroll
      for (int a = 0; a < M; ++a)
        if (sx.ok[a]) t += (sx.w[a] * wyz) * row[sx.idx[a]];
    }
  }
  return t;
}

// one thread per coarse DoF
template <typename T>
__global__ void __launch_bounds__(kXferThreads) k_lattice_restrict(const LatticeTransfer X,
                                                                   const T* __restrict__ fine,
                                                                   T* __restrict__ coarse) {
  pdl_wait();
  const long n = X.ncomp * X.nc_nodes;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    const int comp = (int)(r / X.nc_nodes);
    const long node = r - (long)comp * X.nc_nodes;
    int cx, cy, cz;
    node_xyz(node, X.Nc, cx, cy, cz);
    T t = T(0);
    if (!(X.q2 && lattice_zero(X.zf_c, X.Nc, comp, cx, cy, cz))) {
      Stencil1D<T, 5> sx, sy, sz;
      stencil_dir<T, 5>(true, X.q2, cx, X.Nf[0], X.zf_f, 0, comp, sx);
      stencil_dir<T, 5>(true, X.q2, cy, X.Nf[1], X.zf_f, 1, comp, sy);
      stencil_dir<T, 5>(true, X.q2, cz, X.Nf[2], X.zf_f, 2, comp, sz);
      t = stencil_sum<T, 5>(sx, sy, sz, fine + (long)comp * X.nf_nodes, X.Nf[0], X.Nf[1]);
    }
    coarse[r] = T(0) + t;
  }
}

// one thread per fine DoF
template <typename T>
__global__ void __launch_bounds__(kXferThreads) k_lattice_prolong_add(const LatticeTransfer X,
                                                                      const T* __restrict__ coarse,
                                                                      T* __restrict__ fine) {
  pdl_wait();
  const long n = X.ncomp * X.nf_nodes;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    const int comp = (int)(r / X.nf_nodes);
    const long node = r - (long)comp * X.nf_nodes;
    int fx, fy, fz;
    node_xyz(node, X.Nf, fx, fy, fz);
    T t = T(0);
    if (!(X.q2 && lattice_zero(X.zf_f, X.Nf, comp, fx, fy, fz))) {  // a constrained DoF has no row
      Stencil1D<T, 3> sx, sy, sz;
      stencil_dir<T, 3>(false, X.q2, fx, X.Nc[0], X.zf_c, 0, comp, sx);
      stencil_dir<T, 3>(false, X.q2, fy, X.Nc[1], X.zf_c, 1, comp, sy);
      stencil_dir<T, 3>(false, X.q2, fz, X.Nc[2], X.zf_c, 2, comp, sz);
      t = stencil_sum<T, 3>(sx, sy, sz, coarse + (long)comp * X.nc_nodes, X.Nc[0], X.Nc[1]);
    }
    fine[r] += t;
  }
}

inline int xfer_grid(long n) {
  long b = (n + kXferThreads - 1) / kXferThreads;
  if (b > 152L * 16) b = 152L * 16;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

template <typename T>
void lattice_restrict(const LatticeTransfer& X, const T* fine, T* coarse, cudaStream_t s) {
  const long n = X.ncomp * X.nc_nodes;
  if (n <= 0) return;
  k_lattice_restrict<T><<<xfer_grid(n), kXferThreads, 0, s>>>(X, fine, coarse);
  GB_CUDA(cudaGetLastError());
  ++VecCounter::launches();
}
template <typename T>
void lattice_prolong_add(const LatticeTransfer& X, const T* coarse, T* fine, cudaStream_t s) {
  const long n = X.ncomp * X.nf_nodes;
  if (n <= 0) return;
  k_lattice_prolong_add<T><<<xfer_grid(n), kXferThreads, 0, s>>>(X, coarse, fine);
  GB_CUDA(cudaGetLastError());
  ++VecCounter::launches();
}

template void lattice_restrict<float>(const LatticeTransfer&, const float*, float*, cudaStream_t);
template void lattice_restrict<double>(const LatticeTransfer&, const double*, double*, cudaStream_t);
template void lattice_prolong_add<float>(const LatticeTransfer&, const float*, float*, cudaStream_t);
template void lattice_prolong_add<double>(const LatticeTransfer&, const double*, double*, cudaStream_t);

}  // namespace gb
