// Host-side level data of the GB300 GMG Stokes library.
#pragma once
#include <array>
#include <map>
#include <set>
#include <vector>

#include "lattice_transfer.cuh"
#include "ops.cuh"
#include "vec.cuh"

namespace gb {

// child index of a cell that is the same cell on the next coarser level
constexpr int kSameCell = 255;

// Closed constraints of one block, caller numbering.
struct HostCons {
  std::vector<int> line_of;  // per DoF: -1 or line index
  std::vector<int> ptr{0}, cols;
  std::vector<double> w, inhom;
  void init(long n) {
    line_of.assign(n, -1);
    ptr.assign(1, 0);
    cols.clear();
    w.clear();
    inhom.clear();
  }
  bool constrained(int g) const { return line_of[g] >= 0; }
  int n_entries(int g) const {
    const int l = line_of[g];
    return l < 0 ? -1 : ptr[l + 1] - ptr[l];
  }
};

// A (DoF, weight) expansion of a cell-local DoF in unconstrained DoFs.
struct Expansion {
  int n = 0;
  int g[16];
  double w[16];
};
Expansion expand(const HostCons& c, int g);

struct Csr {
  std::vector<int> ptr{0}, col;
  std::vector<double> val;
  long rows() const { return (long)ptr.size() - 1; }
  Csr transpose(long n_cols) const;
};

template <typename T>
struct LevelDev {
  DevBuf<T> lw, plw, gbox, gtab, eta;
  DevBuf<T> probe_w, pprobe_w;
  DevBuf<T> Pu_val, PuT_val, Pp_val, PpT_val;  // transfer from the next coarser level
  DevBuf<T> dinvA, dinvM;
  DevBuf<T> gu_w, gp_w;  // gather weights (general levels)
  DevBuf<T> Eu, Ep;      // per-cell contributions of pass 1
  DevBuf<T> Mp;          // per-cell pressure mass matrices of the level table [cell][np][np] (velocity degree 2)
  DevBuf<T> Fa;          // fused A-block operator (FP32): per-tile partial sums of face nodes
  DevBuf<T> eta_active;  // finest level without averaging: per-point table of the outer operators
  // V-cycle work vectors (A block: n_u, Schur block: n_p)
  DevBuf<T> solA, defA, tA, dA, solM, defM, tM, dM;
  // the other halves of the iterate, direction and contribution ping-pong pairs
  // of the fused small-level A-block smoother (FP32 small lattice levels only)
  DevBuf<T> xalt, dalt, Ealt;
  double eigA[2] = {0, 0}, eigM[2] = {0, 0};
  bool eig_given[2] = {false, false};
};

// 1D data of a velocity degree (2 or 3): velocity nodes (deal.II's FE_Q(p):
// Gauss-Lobatto points), pressure nodes (FE_Q(p-1)), and QGauss(p+1) on [0, 1]
struct Basis1D {
  int deg = 2, nvn = 3, npn = 2, nq1 = 3;  // per direction: velocity nodes, pressure nodes, points
  double vn[4], pn[3], gq[4], gw[4];
};
Basis1D basis1d(int degree);
// Lagrange basis on `nodes` at x: values and first derivatives
void lagrange_basis(const double* nodes, int n, double x, double* val, double* der);
inline int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

struct Level {
  int dim = 3;
  int degree = 2;  // velocity degree
  int nv() const { return ipow(degree + 1, dim); }  // velocity nodes per cell (one component)
  int np() const { return ipow(degree, dim); }      // pressure nodes per cell
  int nq() const { return ipow(degree + 1, dim); }  // quadrature points per cell
  long n_cells = 0, n_u = 0, n_p = 0;
  // caller data
  std::vector<int> cdu, cdp;
  int geom_kind = 0;
  std::vector<double> geom;
  HostCons cu, cp;
  std::vector<int> parent;
  std::vector<unsigned char> child;
  bool has_transfer = false;
  // internal layout
  bool structured = false;
  int nc[3] = {1, 1, 1};
  double h[3] = {1, 1, 1};
  uint32_t zero_faces = 0;
  std::vector<int> perm_u, perm_p;        // caller DoF -> internal DoF
  std::vector<int> internal_of_cell;      // caller cell -> internal cell
  std::vector<int> cell_of_internal;      // internal cell -> caller cell
  int fused_tz = 0;  // > 0: FP32 A-block applications use the fused kernel, tiles of this many layers
  int n_colours = 0;
  std::vector<int> colour_begin, colour_count;
  std::vector<int> cons_u, cons_p;        // internal constrained DoFs
  // device data
  DevBuf<int> cdu_d, cdp_d, lptr_d, lcol_d, plptr_d, plcol_d;
  DevBuf<int> perm_u_d, perm_p_d, cons_u_d, cons_p_d;
  DevBuf<int> cdu_raw_d, cdp_raw_d;  // internal cells x internal DoFs, no constraint codes (plain reads)
  DevBuf<int> probe_ptr, probe_g, probe_eptr, probe_li;
  std::vector<int> probe_ptr_h, pprobe_ptr_h;  // host copies of the per-cell probe offsets
  DevBuf<int> pprobe_ptr, pprobe_g, pprobe_eptr, pprobe_li;
  DevBuf<int> Pu_ptr, Pu_col, PuT_ptr, PuT_col, Pp_ptr, Pp_col, PpT_ptr, PpT_col;
  long Pu_rows = 0, PuT_rows = 0, Pp_rows = 0, PpT_rows = 0;
  // both this level and the next coarser one structured, and the transfer
  // matrices equal to the lattice stencils (checked entry by entry at set-up):
  // the V-cycle applies them matrix-free ([0] velocity, [1] pressure)
  bool xfer_lattice[2] = {false, false};
  LatticeTransfer xfer[2] = {};
  // pass-2 gather lists of general levels (caller numbering = internal numbering)
  DevBuf<int> gu_ptr, gu_slot, gp_ptr, gp_slot;
  DevBuf<unsigned char> cmask_u, cmask_p;
  LevelDev<float> f32;
  LevelDev<double> f64;
  // viscosity table, internal cell order
  std::vector<double> eta;
  int eta_n = 1;
  // without averaging (GB_GMG_VISC_NONE), finest level only: the outer operators
  // also have a per-point table (eta_active_n = 0: none)
  int eta_active_n = 0;
  // device coefficient pipeline (coefficients.cu): caller -> internal cells, the
  // children of every cell of the next coarser level (CSR by fine-cell index),
  // child indices, the finest level's JxW per point and input values, DG fields
  DevBuf<int> ioc_d, kid_ptr_d, kid_d;
  DevBuf<unsigned char> child_d;
  DevBuf<double> jxw_d, eta_in_d, dg_d;

  template <typename T>
  LevelDev<T>& dev();
  template <typename T>
  LevelView<T> view(double s, int compressible);
  // the view of the outer operators: the per-point table where the level keeps one
  template <typename T>
  LevelView<T> view_outer(double s, int compressible) {
    LevelView<T> v = view<T>(s, compressible);
    if (eta_active_n > 0) {
      v.eta = dev<T>().eta_active.p;
      v.eta_n = eta_active_n;
      v.Mp = nullptr;  // the per-cell mass matrices belong to the level table
    }
    return v;
  }
  template <typename T>
  GatherCsr<T> csr(int block) {
    LevelDev<T>& D = dev<T>();
    if (block == 0) return GatherCsr<T>{gu_ptr.p, gu_slot.p, D.gu_w.p, cmask_u.p};
    return GatherCsr<T>{gp_ptr.p, gp_slot.p, D.gp_w.p, cmask_p.p};
  }
  size_t device_bytes() const;
};

template <>
inline LevelDev<float>& Level::dev<float>() { return f32; }
template <>
inline LevelDev<double>& Level::dev<double>() { return f64; }

// set-up steps (level_setup.cu)
void setup_level(Level& L, bool force_indexed);
void setup_transfer(Level& fine, const Level& coarse);
// device coefficient pipeline (coefficients.cu): the static maps once per mesh,
// then every level's viscosity table (both precisions, internal cell order) and
// the lattice levels' pressure mass matrices from the finest level's values
void setup_coefficient_maps(std::vector<Level>& levels);
void device_level_viscosity(std::vector<Level>& levels, const double* eta_in, int n_per_cell, int projection,
                            double pressure_scaling, double& eta_min, double& eta_max, cudaStream_t st);
// per-cell body-force contributions sum_q JxW f . phi (internal cells, cell-major)
void launch_body_force(const LevelView<double>& L, const double* force, double* Eu, cudaStream_t st);

}  // namespace gb
