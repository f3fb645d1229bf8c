// Arguments of the single-block kernel that runs the lower lattice levels of the
// FP32 A-block (velocity) V-cycle (a_bottom.cu); used in batch mode to build
// that sub-cycle's explicit matrix.
#pragma once
#include "mass_bottom.cuh"

namespace gb {

constexpr int kMaxABottomLevels = 3;
// levels of at most this many velocity DoFs qualify (the matrix is n x n floats)
constexpr int kMaxDenseANodes = 2200;

struct ABottomLevel {
  LevelView<float> L;  // 3D lattice level (geometry, viscosity, zero faces)
  // device vectors of the level; the kernel replaces them by shared-memory copies
  const float* dinv;
  float* sol;
  float* def;
  float* d;
  float* t;
  float* E;  // per-cell contributions (shared memory only)
  // transfers to the next coarser level (levels >= 1): restriction P^T, prolongation P
  int pt_rows, p_rows;
  const int* pt_ptr;
  const int* pt_col;
  const float* pt_val;
  const int* p_ptr;
  const int* p_col;
  const float* p_val;
  // Chebyshev: degree, f2 of the first step (1/theta), (f1, f2) of steps 1 .. degree-1
  int degree;
  float inv_theta;
  float f1[kMaxBottomDegree], f2[kMaxBottomDegree];
  // offsets (in floats, multiples of 4) of dinv, sol, def, d, t, E in shared memory
  int off[6];
};

struct ABottomArgs {
  int n_levels;  // levels 0 .. n_levels-1
  int eta_per_q; // 1: per-point viscosity tables on these levels
  ABottomLevel lev[kMaxABottomLevels];
  // block b runs the cycle on the unit vector e_b as the top level's defect and
  // writes column b (column-major, n x n, n = velocity DoFs of the top level)
  float* batch_out;
};

int a_bottom_layout(ABottomArgs& A);
int a_bottom_reserve();
void launch_a_vcycle_bottom_batch(const ABottomArgs& A, int smem_bytes, int n_cols, cudaStream_t s);

}  // namespace gb
