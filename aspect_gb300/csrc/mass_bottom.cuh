// Arguments of the single-block kernel that runs the lower levels of the FP32
// pressure-mass V-cycle (mass_bottom.cu).
#pragma once
#include "cell_kernels.cuh"

namespace gb {

constexpr int kMaxBottomLevels = 4;
constexpr int kMaxBottomDegree = 16;
// Levels above this many pressure nodes keep the per-step launches. Measured on
// the 32^3 lattice hierarchy (Schur V-cycle, FP32, one GB300): nothing fused
// 0.474 ms, levels of <= 27 nodes 0.470 ms, <= 125 nodes 0.445 ms, <= 729 nodes
// 0.555 ms -- one block is slower than the whole GPU on the 729-node level.
constexpr int kMaxBottomNodes = 200;

struct MassBottomLevel {
  LevelView<float> L;  // lattice geometry (n_p, Np, nc)
  // device vectors of the level; the kernel replaces them by shared-memory
  // copies (the defect of the top level is its input, the solution its output)
  const float* Mc;     // per-cell 8x8 mass matrices
  const float* dinv;
  float* sol;
  float* def;
  float* d;
  float* t;
  // transfers to the next coarser level (levels >= 1): restriction P^T, prolongation P
  int pt_rows, p_rows;
  const int* pt_ptr;
  const int* pt_col;
  const float* pt_val;
  const int* p_ptr;
  const int* p_col;
  const float* p_val;
  // Chebyshev: degree, sweeps per smoothing call, f2 of the first step (1/theta),
  // and (f1, f2) of steps 1 .. degree-1
  int degree, steps;
  float inv_theta;
  float f1[kMaxBottomDegree], f2[kMaxBottomDegree];
  // offsets (in floats, multiples of 4) of this level's shared-memory copies:
  // Mc, dinv, sol, def, d, t
  int off[6];
};

struct MassBottomArgs {
  int n_levels;  // levels 0 .. n_levels-1 of the hierarchy
  MassBottomLevel lev[kMaxBottomLevels];
  // batch mode (non-null): block b runs the cycle on the unit vector e_b as the
  // top level's defect and writes the result to column b (column-major, n x n,
  // n = pressure nodes of the top level) instead of the top level's solution
  float* batch_out;
};

// The cycle of levels 0..K as an explicit matrix: its columns (batch mode) are
// computed once per preconditioner build, after which one dense product
// replaces every launch of those levels. Levels of at most this many pressure
// nodes qualify (the matrix is n x n floats).
constexpr int kMaxDenseBottomNodes = 1000;
// The lattice level above those (at most this many pressure nodes, the matrix
// n x n floats) is built from theirs by the batched steps below.
constexpr int kMaxDenseNextNodes = 6000;

// Fills lev[l].off for levels 0..n_levels-1 and returns the dynamic shared
// memory the launch needs, in bytes.
int mass_bottom_layout(MassBottomArgs& A);
// Largest dynamic shared memory a launch may use, in bytes (sets the kernel
// attribute the first time; call outside stream capture).
int mass_bottom_reserve();
void launch_mass_vcycle_bottom(const MassBottomArgs& A, int smem_bytes, cudaStream_t s);
// batch mode: n_cols blocks, A.batch_out set
void launch_mass_vcycle_bottom_batch(const MassBottomArgs& A, int smem_bytes, int n_cols, cudaStream_t s);
// y = B x for a column-major n x n matrix B (fixed summation order)
void launch_dense_gemv_colmajor(int n, const float* B, const float* x, float* y, cudaStream_t s);

// Batched forms of one lattice level's FP32 mass-cycle steps, over m column
// vectors of length n stored one after another (column c at c * n): used to
// apply the cycle of levels 0..K+1 to all unit vectors of level K+1 at once.
// mass operator with epilogue EPI_CHEB_OUT or EPI_RESID; a's vectors (x, y, b,
// d) are the first columns, dinv is shared
void launch_mass_lattice_batched(const LevelView<float>& L, const float* Mc, int epi, const GatherArgs<float>& a,
                                 int m, cudaStream_t s);
// d = f2 dinv b; x = d (the first Chebyshev step from a zero start)
void launch_cheb_first_batched(long n, int m, const float* b, const float* dinv, float f2, float* d, float* x,
                               cudaStream_t s);
// y[:, c] = x[:, c]
void launch_copy_batched(long n, int m, const float* x, float* y, cudaStream_t s);
// columns of the identity: x[i + c n] = (i == c)
void launch_unit_columns(long n, int m, float* x, cudaStream_t s);
// CSR product per column: y[:, c] = A x[:, c] (add = 0) or y[:, c] += A x[:, c];
// x columns of length nx, y columns of length ny (rows of A <= ny; rows past it untouched)
void launch_spmv_batched(int rows, const int* ptr, const int* col, const float* val, const float* x, long nx,
                         float* y, long ny, int m, bool add, cudaStream_t s);

}  // namespace gb
