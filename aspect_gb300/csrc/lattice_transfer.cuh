// Level transfers between two structured (lattice) levels as tensor products of
// 1D stencils: the same operator as the CSR transfer matrices those levels also
// carry, with the sums in the same order (increasing internal index), so the
// results are identical to the CSR products; only the vectors are read.
//
// Q2 velocity (nodes 2 nc + 1 per direction), one coarse cell = two fine cells
// per direction, fine node f = 4 q + r inside coarse cell q (coarse nodes 2q,
// 2q+1, 2q+2 at 0, 1/2, 1): quadratic interpolation at 0, 1/4, 1/2, 3/4 gives
//   r = 0: (1) at 2q;  r = 1: (3/8, 3/4, -1/8);  r = 2: (1) at 2q+1;
//   r = 3: (-1/8, 3/4, 3/8).
// Q1 pressure (nodes nc + 1): fine 2q -> (1) at q, fine 2q+1 -> (1/2, 1/2).
// Constrained velocity DoFs (Dirichlet faces of either level, per component)
// drop out: no prolongation row, no restriction column.
#pragma once
#include "common.cuh"

namespace gb {

struct LatticeTransfer {
  int q2;              // 1: Q2 velocity (ncomp components, zero faces); 0: Q1 pressure
  int ncomp;
  int Nf[3], Nc[3];    // nodes per direction, fine and coarse (1 beyond dim)
  long nf_nodes, nc_nodes;
  uint32_t zf_f, zf_c; // zero-face masks, bit (2*d+side)*3+comp
};

// coarse nodes and weights of fine node f (1D, increasing); returns the count
__host__ __device__ inline int lattice_p1d(int q2, int f, int* c, double* w) {
  if (!q2) {
    if (!(f & 1)) { c[0] = f >> 1; w[0] = 1.0; return 1; }
    c[0] = f >> 1; c[1] = (f >> 1) + 1; w[0] = 0.5; w[1] = 0.5;
    return 2;
  }
  const int q = f >> 2, r = f & 3;
  if (r == 0 || r == 2) { c[0] = 2 * q + (r >> 1); w[0] = 1.0; return 1; }
  c[0] = 2 * q; c[1] = 2 * q + 1; c[2] = 2 * q + 2;
  w[0] = r == 1 ? 0.375 : -0.125;
  w[1] = 0.75;
  w[2] = r == 1 ? -0.125 : 0.375;
  return 3;
}
// fine nodes and weights of coarse node c within [0, Nf) (1D, increasing)
__host__ __device__ inline int lattice_r1d(int q2, int c, int Nf, int* f, double* w) {
  int cand[5];
  double cw[5];
  int m = 0;
  if (!q2) {
    cand[0] = 2 * c - 1; cand[1] = 2 * c; cand[2] = 2 * c + 1;
    cw[0] = 0.5; cw[1] = 1.0; cw[2] = 0.5;
    m = 3;
  } else if (!(c & 1)) {
    const int q = c >> 1;
    cand[0] = 4 * q - 3; cand[1] = 4 * q - 1; cand[2] = 4 * q; cand[3] = 4 * q + 1; cand[4] = 4 * q + 3;
    cw[0] = -0.125; cw[1] = 0.375; cw[2] = 1.0; cw[3] = 0.375; cw[4] = -0.125;
    m = 5;
  } else {
    const int q = c >> 1;
    cand[0] = 4 * q + 1; cand[1] = 4 * q + 2; cand[2] = 4 * q + 3;
    cw[0] = 0.75; cw[1] = 1.0; cw[2] = 0.75;
    m = 3;
  }
  int k = 0;
  for (int i = 0; i < m; ++i)
    if (cand[i] >= 0 && cand[i] < Nf) { f[k] = cand[i]; w[k] = cw[i]; ++k; }
  return k;
}
// is component comp of node (x, y, z) on a zero face of a level with N nodes per direction?
__host__ __device__ inline bool lattice_zero(uint32_t zf, const int* N, int comp, int x, int y, int z) {
  if (!zf) return false;
  const int g[3] = {x, y, z};
  for (int d = 0; d < 3; ++d) {
    if (N[d] == 1) continue;
    if (g[d] == 0 && ((zf >> ((2 * d) * 3 + comp)) & 1u)) return true;
    if (g[d] == N[d] - 1 && ((zf >> ((2 * d + 1) * 3 + comp)) & 1u)) return true;
  }
  return false;
}

// coarse = P^T fine (every coarse entry written)
template <typename T>
void lattice_restrict(const LatticeTransfer& X, const T* fine, T* coarse, cudaStream_t s);
// fine += P coarse (unconstrained fine entries)
template <typename T>
void lattice_prolong_add(const LatticeTransfer& X, const T* coarse, T* fine, cudaStream_t s);

}  // namespace gb
