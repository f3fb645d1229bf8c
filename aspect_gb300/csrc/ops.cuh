// Host-side launchers of the cell kernels.
#pragma once
#include "cell_kernels.cuh"

namespace gb {

// Per-cell diagonal probes of a general level (device pointers).
template <typename T>
struct ProbesView {
  const int* ptr = nullptr;   // [n_cells+1]
  const int* g = nullptr;     // [n_probes] target DoF
  const int* eptr = nullptr;  // [n_probes+1]
  const int* li = nullptr;    // [n_entries] cell-local index
  const T* w = nullptr;       // [n_entries]
};

// true when pass 1 of `op` writes its per-cell contributions slot-major
// (E[slot][cell]) instead of cell-major (E[cell][slot])
template <typename T>
bool cell_pass_slot_major(const LevelView<T>& L, int op);
// pass 1 of an operator (op: OPK_*), all cells of the level
template <typename T>
void launch_cell_pass(const LevelView<T>& L, int op, const T* src_u, const T* src_p, T* Eu, T* Ep, cudaStream_t s);
// pass 2 for block 0 (velocity DoFs) or 1 (pressure DoFs); csr == nullptr on lattice levels
template <typename T>
void launch_gather(const LevelView<T>& L, int block, int epi, const GatherCsr<T>* csr, const GatherArgs<T>& a,
                   cudaStream_t s);
// FP32 A-block levels whose cell pass is the one-cell-per-block small-level
// kernel (the levels lattice_cheb_small serves)
bool small_lattice_a_level(const LevelView<float>& L);
// one fused Chebyshev step (gather, update, next cell pass) of such a level
void launch_cheb_small(const LevelView<float>& L, bool first, const ChebSmallArgs& a, cudaStream_t s);
// one-pass pressure mass operator of a lattice level (Mc: per-cell local matrices)
template <typename T>
void launch_mass_lattice(const LevelView<T>& L, const T* Mc, int epi, const GatherArgs<T>& a, cudaStream_t s);
// Newton-derivative and prescribed-dilation tables of the outer Stokes operator
// (newton.cu): per internal cell and quadrature point, symmetric tensors in
// deal.II's unrolled component order.
template <typename T>
struct NewtonView {
  int newton, symmetrize, average, dilation;
  const T* E;    // strain_rate_table
  const T* D;    // newton_factor_wrt_strain_rate_table
  const T* dp;   // newton_factor_wrt_pressure_table
  const T* lhs;  // dilation_lhs_term_table
  const T* DD;   // dilation_derivative_wrt_strain_rate_table
  const T* dpd;  // dilation_derivative_wrt_pressure_table
};
// cell pass of the outer Stokes operator with those terms (the level's gathers follow)
template <typename T>
void launch_newton_stokes(const LevelView<T>& L, const NewtonView<T>& N, const T* su, const T* sp, T* Eu, T* Ep,
                          bool slot_major, cudaStream_t s);

// Degree-3 velocity (Q3-Q2) cell operators of indexed levels (ho_kernels.cu):
// the cell pass of any operator, and the A-block (block 0) / mass (block 1)
// diagonal of one cell colour from its probes (n_probes of the colour's cells)
template <typename T>
void launch_ho_cell_pass(const LevelView<T>& L, int op, const T* su, const T* sp, T* Eu, T* Ep, cudaStream_t s);
template <typename T>
void launch_ho_diag(const LevelView<T>& L, int block, int begin, int count, const ProbesView<T>& pr, int n_probes,
                    T* diag, cudaStream_t s);

// Free-surface faces of the finest level (free_surface.cu), grouped by internal
// cell: the faces of cell gcell[g] are gptr[g] .. gptr[g+1]-1; per face its
// number 2*d + side, the constraint codes of its 3^(dim-1) nodes per component
// ([face][comp][node], first tangential axis fastest) and per point the
// stabilisation vector T and the outward normal times JxW ([face][point][2*dim]).
template <typename T>
struct FreeSurfaceView {
  int n_groups;
  const int* gptr;
  const int* gcell;
  const int* fno;
  const int* codes;
  const T* tab;
};
// adds the face terms of src to the per-cell velocity contributions E (before the gather)
template <typename T>
void launch_free_surface(const LevelView<T>& L, const FreeSurfaceView<T>& F, const T* src, T* E, bool slot_major,
                         cudaStream_t s);
// host: outward normal x surface JxW at the face's QGauss(3) points ([point][dim]);
// geom_kind 0: cell_geom = (x0[dim], h[dim]), 1: the 3^dim Q2 support points
void face_normal_jxw(int dim, int geom_kind, const double* cell_geom, int fno, double* out);

// Fused FP32 A-block operator of large 3D lattice levels (ablock_fused.cu):
// cell layers per tile for a level (0: the level does not qualify), the face
// buffer it needs (floats), the one-time kernel attribute set-up (call outside
// stream capture), and the two launches of one application with epilogue
// EPI_STORE, EPI_RESID or EPI_CHEB.
int fused_a_tile_layers(const LevelView<float>& L, int n_sm, long min_cells);
size_t fused_a_face_floats(const LevelView<float>& L, int tz);
bool fused_a_prepare();
void launch_fused_a(const LevelView<float>& L, int epi, const GatherArgs<float>& a, float* F, int tz,
                    cudaStream_t s);
// A-block diagonal contributions of a lattice level, one pass over all cells
// (set-up only; the level's gather sums them)
template <typename T>
void launch_lattice_diag(const LevelView<T>& L, T* Eu, bool slot_major, cudaStream_t s);
// diagonals, colour by colour (set-up only)
template <typename T>
void launch_velocity_diag(const LevelView<T>& L, int colour, int begin, int count, const ProbesView<T>& pr,
                          T* diag, cudaStream_t s);
template <typename T>
void launch_mass_diag(const LevelView<T>& L, int colour, int begin, int count, const ProbesView<T>& pr, T* diag,
                      cudaStream_t s);

}  // namespace gb
