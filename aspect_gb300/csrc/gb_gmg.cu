// GB300 matrix-free GMG Stokes solver: operators, V-cycle, block
// preconditioner, Krylov solvers and the C ABI of include/gb_gmg.h.
//
// Solver composition follows source/simulator/solver/stokes_matrix_free_local_smoothing.cc:
//   smoothers / coarse solve     :774-861 (Chebyshev degree 4, range 15, 10
//                                  eigenvalue-CG steps on levels > 0; degree 8,
//                                  range 1e-3, 100 steps on level 0; 4 Schur
//                                  smoothing steps; coarse = one smoother apply)
//   V-cycle / PreconditionMG     :896-916 (deal.II Multigrid: pre-smoothing from
//                                  zero, residual, restrict, recurse,
//                                  prolongate, post-smoothing)
//   initial residual, tolerance  :977-1041
//   cheap GMRES, FGMRES fallback :1262-1397
// and include/aspect/simulator/solver/block_stokes_preconditioner.h:101-352.
// Everything runs on one GPU; the V-cycle runs in FP32 or FP64, the Krylov
// solver, the Stokes residual and the Schur update in FP64.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cublas_v2.h>
#include <cusolverDn.h>

#include "../../include/gb_gmg.h"
#include "level.cuh"
#include "mass_bottom.cuh"
#include "a_bottom.cuh"

namespace gb {

void launch_adjoint_gradient_impl(const LevelView<double>& L, int colour, int begin, int count, const double* u,
                                  const double* lam, double* grad, cudaStream_t s);

struct Handle {
  gb_gmg_options opt{};
  int dim = 3, n_levels = 0;
  int degree = 2;  // velocity degree (2: Q2-Q1, 3: Q3-Q2)
  std::vector<Level> levels;
  cudaStream_t st = nullptr;
  std::string err;
  double s = 1.0;
  int compressible = 0, projection = 0;
  int visc_n_per_cell = 0;  // n_per_cell of the last successful set_viscosity
  // Newton / prescribed-dilation terms of the outer Stokes operator (finest level,
  // internal cell order): flags and tables in both precisions
  struct Newton {
    int newton = 0, symmetrize = 0, average = 0, dilation = 0;
    DevBuf<double> t64[6];
    DevBuf<float> t32[6];
    bool on() const { return newton || dilation; }
    template <typename T>
    NewtonView<T> view() const {
      const auto& t = pick(t64, t32, T());
      return NewtonView<T>{newton, symmetrize, average, dilation, t[0].p, t[1].p, t[2].p, t[3].p, t[4].p, t[5].p};
    }
    static const DevBuf<double> (&pick(const DevBuf<double> (&a)[6], const DevBuf<float> (&)[6], double))[6] {
      return a;
    }
    static const DevBuf<float> (&pick(const DevBuf<double> (&)[6], const DevBuf<float> (&b)[6], float))[6] {
      return b;
    }
    void clear() {
      newton = symmetrize = average = dilation = 0;
      for (auto& b : t64) b.release();
      for (auto& b : t32) b.release();
    }
  } newton_terms;
  // free-surface faces of the outer Stokes operator (finest level; see FreeSurfaceView):
  // codes read through the constraints (operator) or plain (rhs correction)
  struct FreeSurface {
    int n_groups = 0;
    long n_faces = 0;
    DevBuf<int> gptr, gcell, fno, codes, raw;
    DevBuf<double> t64;
    DevBuf<float> t32;
    bool on() const { return n_faces > 0; }
    template <typename T>
    FreeSurfaceView<T> view(bool plain = false) const {
      const T* tab;
      if constexpr (std::is_same<T, double>::value) tab = t64.p;
      else tab = t32.p;
      return FreeSurfaceView<T>{n_groups, gptr.p, gcell.p, fno.p, plain ? raw.p : codes.p, tab};
    }
    void clear() {
      n_groups = 0;
      n_faces = 0;
      for (auto* b : {&gptr, &gcell, &fno, &codes, &raw}) b->release();
      t64.release();
      t32.release();
    }
  } free_surface;
  int n_sm = 1;             // streaming multiprocessors of the handle's GPU
  double eta_min = 0, eta_max = 0;
  bool setup_done = false, visc_done = false;
  bool prec_done[2] = {false, false};  // per precision (0 fp64, 1 fp32)
  // build_preconditioner ran but left the FP64 levels (diagonals, eigenvalue
  // estimates) to their first use: a solve with FP32 V-cycles never needs them
  bool fp64_pending = false;
  long long cell_launches = 0;
  // staging and FP64 active-level workspace
  DevBuf<double> stage_a, stage_b, partial, dots_d;
  double* dots_h = nullptr;
  DevBuf<double> V, Z, wv, xv, rv, bv, tv, t2v, coef_d;
  DevBuf<double> idrP, idrG, idrU;  // IDR(s): shadow space, G and U blocks (s vectors each)
  int idr_s_alloc = 0;
  DevBuf<double> hcol_d, arn_d;  // Arnoldi column and scalars (|w|^2, |w| before, 1/|w|) on the device
  DevBuf<int> arn_flag;          // 1: the step needs its second Gram-Schmidt pass
  // float-pair copy of the Krylov basis V (column stride lds) and the scale
  // exponents of the Arnoldi steps (double-buffered: step j reads [j & 1])
  DevBuf<float2> Vs;
  long lds = 0;
  DevBuf<int> gs_shift;
  // eigenvalue-estimate CG: device scalars and alpha/beta history, flags
  DevBuf<double> eig_s;
  DevBuf<int> eig_f;
  DevBuf<double> cg_r, cg_z, cg_p, cg_q, cg_x;
  DevBuf<float> f32_a, f32_b;
  int restart_alloc = -1;
  int nA = 0, nS = 0, n_stokes64 = 0;
  int* flag_d = nullptr;
  // captured V-cycles [block][precision 0 fp64 / 1 fp32] and their staging vectors
  cudaGraphExec_t vgraph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  long long vgraph_kernels[2][2] = {{0, 0}, {0, 0}};
  DevBuf<double> vin, vout;
  // FP64 dense coarse solve: pseudo-inverses of the level-0 A and mass matrices
  DevBuf<double> coarse_pinv[2], coarse_x, coarse_y;
  bool coarse_ready = false;
  // levels 0..mass_bottom_top of the FP32 mass V-cycle run in one single-block launch (-1: none)
  int mass_bottom_top = -1;
  // levels 0..mass_dense_top of the FP32 mass V-cycle as one column-major matrix (-1: none):
  // mass_dense for the levels the single-block cycle covers (top mass_dense_base),
  // mass_dense2 when the lattice level above them is included (built from mass_dense)
  int mass_dense_top = -1, mass_dense_base = -1;
  DevBuf<float> mass_dense, mass_dense2;
  // the same for the FP32 A-block V-cycle
  int a_dense_top = -1;
  DevBuf<float> a_dense;

  Level& top() { return levels.back(); }
  void reset_graphs() {
    for (auto& r : vgraph)
      for (auto& g : r)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
  }
  long n_top() { return top().n_u + top().n_p; }
};

namespace {

// ---------------------------------------------------------------- tridiagonal eigenvalues
void tridiag_eigs(std::vector<double> d, std::vector<double> e, double& lmin, double& lmax) {
  const int n = (int)d.size();
  if (n == 0) { lmin = lmax = 0; return; }
  e.resize(n, 0.0);
  for (int l = 0; l < n; ++l) {
    int iter = 0, m;
    do {
      for (m = l; m < n - 1; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-15 * dd) break;
      }
      if (m != l) {
        if (iter++ == 200) break;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = std::hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
        double s_ = 1, c = 1, p = 0;
        int i;
        for (i = m - 1; i >= l; --i) {
          const double f = s_ * e[i], b = c * e[i];
          r = std::hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0) { d[i + 1] -= p; e[m] = 0.0; break; }
          s_ = f / r; c = g / r; g = d[i + 1] - p; r = (d[i] - g) * s_ + 2.0 * c * b;
          p = s_ * r; d[i + 1] = g + p; g = c * r - b;
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p; e[l] = g; e[m] = 0.0;
      }
    } while (m != l);
  }
  lmin = *std::min_element(d.begin(), d.end());
  lmax = *std::max_element(d.begin(), d.end());
}

double dot_host(Handle& H, long n, const double* a, const double* b) {
  v_dot<double>(n, a, b, H.dots_d.p, H.partial.p, H.st);
  GB_CUDA(cudaMemcpyAsync(H.dots_h, H.dots_d.p, sizeof(double), cudaMemcpyDeviceToHost, H.st));
  GB_CUDA(cudaStreamSynchronize(H.st));
  return H.dots_h[0];
}
template <typename T>
double dot_host_T(Handle& H, long n, const T* a, const T* b) {
  v_dot<T>(n, a, b, H.dots_d.p, H.partial.p, H.st);
  GB_CUDA(cudaMemcpyAsync(H.dots_h, H.dots_d.p, sizeof(double), cudaMemcpyDeviceToHost, H.st));
  GB_CUDA(cudaStreamSynchronize(H.st));
  return H.dots_h[0];
}

// ---------------------------------------------------------------- operators
template <typename T>
void gather(Handle& H, Level& L, const LevelView<T>& v, int block, int epi, GatherArgs<T> a, int op) {
  const int nl = block == 0 ? L.dim * L.nv() : L.np();
  if (cell_pass_slot_major<T>(v, op)) {
    a.cs = 1;
    a.ss = L.n_cells;
  } else {
    a.cs = nl;
    a.ss = 1;
  }
  GatherCsr<T> csr;
  const GatherCsr<T>* pc = nullptr;
  if (!L.structured) {
    csr = L.csr<T>(block);
    pc = &csr;
  }
  launch_gather<T>(v, block, epi, pc, a, H.st);
  ++H.cell_launches;
}

// y = op(x) on a level; constrained rows act as the identity (zero for B^T)
template <typename T>
void mass_lattice(Handle& H, Level& L, const LevelView<T>& v, int epi, GatherArgs<T> a) {
  launch_mass_lattice<T>(v, L.dev<T>().Mp.p, epi, a, H.st);
  ++H.cell_launches;
}

// FP32 A-block application of a large lattice level through the fused kernel
// (one cell-and-gather pass plus the face pass); false when the level does not use it
template <typename T>
bool fused_a(Handle& H, Level& L, int epi, const GatherArgs<T>& a) {
  if constexpr (std::is_same<T, float>::value) {
    if (L.fused_tz > 0) {
      launch_fused_a(L.view<float>(H.s, H.compressible), epi, a, L.f32.Fa.p, L.fused_tz, H.st);
      H.cell_launches += 2;
      return true;
    }
  }
  return false;
}

// outer = true: an operator of the outer solver (FGMRES product, expensive inner
// solves, rhs correction); it takes the level's per-point table where the level
// keeps one for them (no averaging), the multigrid operators the level table.
template <typename T>
void apply_op(Handle& H, int lev, int op, const T* su, const T* sp, T* du, T* dp, bool outer = false) {
  Level& L = H.levels[lev];
  LevelDev<T>& D = L.dev<T>();
  const bool own_table = outer && L.eta_active_n > 0;
  LevelView<T> v = own_table ? L.view_outer<T>(H.s, H.compressible) : L.view<T>(H.s, H.compressible);
  const bool newton = outer && lev == H.n_levels - 1 && H.newton_terms.on();
  // free-surface faces: the outer Stokes operator of the finest level only
  const bool free_surface = outer && lev == H.n_levels - 1 && op == OPK_STOKES && H.free_surface.on();
  // a prescribed dilation makes the outer viscous terms deviatoric (not the levels')
  if (newton && H.newton_terms.dilation) v.compressible = 1;
  if (newton && op == OPK_STOKES) {
    launch_newton_stokes<T>(v, H.newton_terms.view<T>(), su, sp, D.Eu.p, D.Ep.p, cell_pass_slot_major<T>(v, op),
                            H.st);
    ++H.cell_launches;
    if (free_surface) {
      launch_free_surface<T>(v, H.free_surface.view<T>(), su, D.Eu.p, cell_pass_slot_major<T>(v, op), H.st);
      ++H.cell_launches;
    }
    for (int block = 0; block < 2; ++block) {
      GatherArgs<T> a{};
      a.E = block == 0 ? D.Eu.p : D.Ep.p;
      a.x = const_cast<T*>(block == 0 ? su : sp);
      a.y = block == 0 ? du : dp;
      gather<T>(H, L, v, block, EPI_STORE, a, op);
    }
    return;
  }
  if (op == OPK_A && !own_table && !newton) {
    GatherArgs<T> a{};
    a.x = const_cast<T*>(su);
    a.y = du;
    if (fused_a<T>(H, L, EPI_STORE, a)) return;
  }
  if (op == OPK_MASS && L.structured && !own_table) {  // per-cell matrices of the level table
    GatherArgs<T> a{};
    a.x = const_cast<T*>(sp);
    a.y = dp;
    mass_lattice<T>(H, L, v, EPI_STORE, a);
    return;
  }
  launch_cell_pass<T>(v, op, su, sp, D.Eu.p, D.Ep.p, H.st);
  ++H.cell_launches;
  if (free_surface) {
    launch_free_surface<T>(v, H.free_surface.view<T>(), su, D.Eu.p, cell_pass_slot_major<T>(v, op), H.st);
    ++H.cell_launches;
  }
  if (op == OPK_STOKES || op == OPK_A || op == OPK_BT) {
    GatherArgs<T> a{};
    a.E = D.Eu.p;
    a.x = const_cast<T*>(su);
    a.y = du;
    gather<T>(H, L, v, 0, op == OPK_BT ? EPI_BT : EPI_STORE, a, op);
  }
  if (op == OPK_STOKES || op == OPK_MASS) {
    GatherArgs<T> a{};
    a.E = D.Ep.p;
    a.x = const_cast<T*>(sp);
    a.y = dp;
    gather<T>(H, L, v, 1, EPI_STORE, a, op);
  }
}

template <typename T>
void level_op(Handle& H, int lev, int block, const T* x, T* y) {
  if (block == 0) apply_op<T>(H, lev, OPK_A, x, nullptr, y, nullptr);
  else apply_op<T>(H, lev, OPK_MASS, nullptr, x, nullptr, y);
}

// Chebyshev step fused into the gather: t = K x; d = f1 d + f2 D^-1 (b - t); x += d
template <typename T>
void level_op_cheb(Handle& H, int lev, int block, T* x, const T* b, const T* dinv, T* d, double f1, double f2) {
  Level& L = H.levels[lev];
  LevelDev<T>& D = L.dev<T>();
  if (block == 0) {
    GatherArgs<T> a{};
    a.x = x;
    a.b = b;
    a.dinv = dinv;
    a.d = d;
    a.f1 = (T)f1;
    a.f2 = (T)f2;
    if (fused_a<T>(H, L, EPI_CHEB, a)) return;
  }
  const LevelView<T> v = L.view<T>(H.s, H.compressible);
  launch_cell_pass<T>(v, block == 0 ? OPK_A : OPK_MASS, x, x, D.Eu.p, D.Ep.p, H.st);
  ++H.cell_launches;
  GatherArgs<T> a{};
  a.E = block == 0 ? D.Eu.p : D.Ep.p;
  a.x = x;
  a.b = b;
  a.dinv = dinv;
  a.d = d;
  a.f1 = (T)f1;
  a.f2 = (T)f2;
  gather<T>(H, L, v, block, EPI_CHEB, a, block == 0 ? OPK_A : OPK_MASS);
}

// residual fused into the gather: y = b - K x
template <typename T>
void level_op_resid(Handle& H, int lev, int block, const T* x, const T* b, T* y) {
  Level& L = H.levels[lev];
  LevelDev<T>& D = L.dev<T>();
  if (block == 0) {
    GatherArgs<T> a{};
    a.x = const_cast<T*>(x);
    a.b = b;
    a.y = y;
    if (fused_a<T>(H, L, EPI_RESID, a)) return;
  }
  const LevelView<T> v = L.view<T>(H.s, H.compressible);
  if (block == 1 && L.structured) {
    GatherArgs<T> a{};
    a.x = const_cast<T*>(x);
    a.y = y;
    a.b = b;
    mass_lattice<T>(H, L, v, EPI_RESID, a);
    return;
  }
  launch_cell_pass<T>(v, block == 0 ? OPK_A : OPK_MASS, x, x, D.Eu.p, D.Ep.p, H.st);
  ++H.cell_launches;
  GatherArgs<T> a{};
  a.E = block == 0 ? D.Eu.p : D.Ep.p;
  a.x = const_cast<T*>(x);
  a.y = y;
  a.b = b;
  gather<T>(H, L, v, block, EPI_RESID, a, block == 0 ? OPK_A : OPK_MASS);
}

// ---------------------------------------------------------------- diagonals
template <typename T>
void compute_diagonals(Handle& H, int lev) {
  Level& L = H.levels[lev];
  LevelDev<T>& D = L.dev<T>();
  const LevelView<T> v = L.view<T>(H.s, H.compressible);
  D.dinvA.alloc(L.n_u);
  D.dinvM.alloc(L.n_p);
  D.dinvA.zero(H.st);
  D.dinvM.zero(H.st);
  ProbesView<T> pu{L.probe_ptr.p, L.probe_g.p, L.probe_eptr.p, L.probe_li.p, D.probe_w.p};
  ProbesView<T> pp{L.pprobe_ptr.p, L.pprobe_g.p, L.pprobe_eptr.p, L.pprobe_li.p, D.pprobe_w.p};
  // lattice levels: the velocity diagonal directly per cell (lattice_diag_kernel),
  // summed into nodes by the level's own gather (constrained rows are set below)
  const bool direct = L.structured && v.geom == GEOM_CART;
  if (direct) {
    launch_lattice_diag<T>(v, D.Eu.p, cell_pass_slot_major<T>(v, OPK_A), H.st);
    ++H.cell_launches;
    GatherArgs<T> a{};
    a.E = D.Eu.p;
    a.x = D.dinvA.p;
    a.y = D.dinvA.p;
    gather<T>(H, L, v, 0, EPI_STORE, a, OPK_A);
  }
  for (int k = 0; k < L.n_colours; ++k) {
    const int cnt = L.colour_count[k];
    if (!cnt) continue;
    const int begin = L.structured ? 0 : L.colour_begin[k];
    if (L.degree == 3) {  // Q3-Q2: the cell operators on the colour's probes
      launch_ho_diag<T>(v, 0, begin, cnt, pu, L.probe_ptr_h[begin + cnt] - L.probe_ptr_h[begin], D.dinvA.p, H.st);
      launch_ho_diag<T>(v, 1, begin, cnt, pp, L.pprobe_ptr_h[begin + cnt] - L.pprobe_ptr_h[begin], D.dinvM.p, H.st);
      H.cell_launches += 2;
      continue;
    }
    if (!direct) {
      launch_velocity_diag<T>(v, k, begin, cnt, pu, D.dinvA.p, H.st);
      ++H.cell_launches;
    }
    launch_mass_diag<T>(v, k, begin, cnt, pp, D.dinvM.p, H.st);
    ++H.cell_launches;
  }
  GB_CUDA(cudaStreamSynchronize(H.st));
  for (int block = 0; block < 2; ++block) {
    DevBuf<T>& buf = block == 0 ? D.dinvA : D.dinvM;
    std::vector<T> d = buf.download();
    const std::vector<int>& cons = block == 0 ? L.cons_u : L.cons_p;
    for (int c : cons) d[c] = T(1);
    for (size_t i = 0; i < d.size(); ++i) {
      GB_CHECK(d[i] > T(0) && std::isfinite((double)d[i]), 6,
               "No diagonal entry in a positive definite operator should be zero or negative.");
      d[i] = T(1) / d[i];
    }
    buf.upload(d);
  }
}

// ---------------------------------------------------------------- Chebyshev smoother
struct ChebParams {
  int degree, eig_its;
  double range;
};
ChebParams cheb_params(const Handle& H, int lev) {
  if (lev > 0) return {H.opt.smoother_degree, H.opt.eig_cg_iterations, H.opt.smoothing_range};
  return {H.opt.coarse_degree, H.opt.coarse_eig_cg_iterations, H.opt.coarse_range};
}

template <typename T>
void estimate_eigenvalues(Handle& H, int lev, int block) {
  Level& L = H.levels[lev];
  LevelDev<T>& D = L.dev<T>();
  if (D.eig_given[block]) return;
  const long n = block == 0 ? L.n_u : L.n_p;
  const HostCons& C = block == 0 ? L.cu : L.cp;
  const std::vector<int>& perm = block == 0 ? L.perm_u : L.perm_p;
  const ChebParams cp = cheb_params(H, lev);
  // PreconditionChebyshev's start vector: a period-11 mode (i mod 11, caller
  // numbering) with its mean removed, over all entries. The pressure mass
  // matrix has no null space and its largest eigenvector on small coarse levels
  // is the constant mode, so for block 1 the mean is kept (else the Lanczos
  // estimate misses that eigenvalue and the Chebyshev polynomial amplifies it).
  std::vector<T> b(n, T(0));
  double mean = 0;
  if (block == 0) {
    for (long i = 0; i < n; ++i) mean += (double)(i % 11);
    mean /= std::max(n, 1L);
  }
  for (long i = 0; i < n; ++i) b[perm[i]] = (T)((double)(i % 11) - mean);
  (void)C;
  // use the level's work vectors: r = def, z = sol, p = d, Ap = t
  T* r = block == 0 ? D.defA.p : D.defM.p;
  T* z = block == 0 ? D.solA.p : D.solM.p;
  T* p = block == 0 ? D.dA.p : D.dM.p;
  T* Ap = block == 0 ? D.tA.p : D.tM.p;
  const T* dinv = block == 0 ? D.dinvA.p : D.dinvM.p;
  GB_CUDA(cudaMemcpyAsync(r, b.data(), n * sizeof(T), cudaMemcpyHostToDevice, H.st));
  // CG with the scalars on the device (v_eig_step): alpha = r.z / p.Ap, r -= alpha Ap,
  // stop when |r| < 1e-2 (SolverControl(eig_cg_n_iterations, 1e-2), absolute),
  // z = D^-1 r, beta = r.z new / r.z, p = z + beta p; the host looks at the
  // running flag every kEigCheck steps and reads the alpha/beta history once
  const int its = cp.eig_its;
  if (H.eig_s.n < (size_t)(kEigHist + 2 * its)) H.eig_s.alloc(kEigHist + 2 * its);
  if (H.eig_f.n < 3) H.eig_f.alloc(3);
  double* sd = H.eig_s.p;
  int* fd = H.eig_f.p;
  v_eig_start(fd, H.st);
  v_cheb_first<T>(n, r, dinv, T(1), p, z, H.st);  // z = D^-1 r ; p = z
  v_dot<T>(n, r, z, sd, H.partial.p, H.st);       // s[0] = r.z
  constexpr int kEigCheck = 8;
  int flags[3] = {1, 0, 0};
  for (int it = 0; it < its; ++it) {
    level_op<T>(H, lev, block, p, Ap);
    v_eig_step<T>(n, p, Ap, r, z, dinv, sd, fd, its, H.partial.p, H.st);
    if ((it + 1) % kEigCheck == 0 && it + 1 < its) {
      GB_CUDA(cudaMemcpyAsync(flags, fd, sizeof(int), cudaMemcpyDeviceToHost, H.st));
      GB_CUDA(cudaStreamSynchronize(H.st));
      if (flags[0] == 0) break;
    }
  }
  std::vector<double> hist(kEigHist + 2 * its);
  GB_CUDA(cudaMemcpyAsync(flags, fd, 3 * sizeof(int), cudaMemcpyDeviceToHost, H.st));
  GB_CUDA(cudaMemcpyAsync(hist.data(), sd, hist.size() * sizeof(double), cudaMemcpyDeviceToHost, H.st));
  GB_CUDA(cudaStreamSynchronize(H.st));
  const std::vector<double> alphas(hist.begin() + kEigHist, hist.begin() + kEigHist + flags[1]);
  const std::vector<double> betas(hist.begin() + kEigHist + its, hist.begin() + kEigHist + its + flags[2]);
  const int k = (int)alphas.size();
  std::vector<double> dd(k), ee(k, 0.0);
  for (int i = 0; i < k; ++i) {
    dd[i] = 1.0 / alphas[i] + (i > 0 ? betas[i - 1] / alphas[i - 1] : 0.0);
    if (i + 1 < k) ee[i] = std::sqrt(betas[i]) / alphas[i];
  }
  double* eig = block == 0 ? D.eigA : D.eigM;
  tridiag_eigs(dd, ee, eig[0], eig[1]);
  // leave the work vectors clean (the smoother relies on finite values)
  GB_CUDA(cudaMemsetAsync(z, 0, n * sizeof(T), H.st));
  GB_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), H.st));
}

template <typename T>
void chebyshev_bounds(Handle& H, int lev, int block, double& theta, double& delta) {
  LevelDev<T>& D = H.levels[lev].dev<T>();
  const double* eig = block == 0 ? D.eigA : D.eigM;
  const ChebParams cp = cheb_params(H, lev);
  // a level without unconstrained DoFs has no spectrum; any positive bound is inert there
  const double emax = eig[1] > 0 ? eig[1] : 1.0;
  const double emin = eig[1] > 0 ? eig[0] : 1.0;
  const double lmax = 1.2 * emax;
  const double alpha = cp.range > 1.0 ? lmax / cp.range : std::min(0.9 * lmax, emin);
  theta = 0.5 * (lmax + alpha);
  delta = 0.5 * (lmax - alpha);
}

// x = Cheb(b) from zero (zero_start) or one step from x (PreconditionChebyshev vmult / step)
template <typename T>
void chebyshev(Handle& H, int lev, int block, T* x, const T* b, bool zero_start) {
  Level& L = H.levels[lev];
  LevelDev<T>& D = L.dev<T>();
  const long n = block == 0 ? L.n_u : L.n_p;
  const ChebParams cp = cheb_params(H, lev);
  double theta, delta;
  chebyshev_bounds<T>(H, lev, block, theta, delta);
  const T* dinv = block == 0 ? D.dinvA.p : D.dinvM.p;
  T* d = block == 0 ? D.dA.p : D.dM.p;
  T* t = block == 0 ? D.tA.p : D.tM.p;
  // the one-pass mass operator of lattice levels reads neighbouring entries of
  // the iterate, so its Chebyshev steps alternate between x and t
  const bool ping_pong = block == 1 && L.structured;
  T* cur = x;
  auto step = [&](double f1, double f2) {
    if (!ping_pong) {
      level_op_cheb<T>(H, lev, block, x, b, dinv, d, f1, f2);
      return;
    }
    T* nxt = cur == x ? t : x;
    GatherArgs<T> a{};
    a.x = cur;
    a.y = nxt;
    a.b = b;
    a.dinv = dinv;
    a.d = d;
    a.f1 = (T)f1;
    a.f2 = (T)f2;
    mass_lattice<T>(H, L, L.view<T>(H.s, H.compressible), EPI_CHEB_OUT, a);
    cur = nxt;
  };
  if (zero_start) v_cheb_first<T>(n, b, dinv, (T)(1.0 / theta), d, x, H.st);
  else step(0.0, 1.0 / theta);
  double rhok = delta / theta;
  const double sigma = theta / delta;
  for (int k = 1; k < cp.degree; ++k) {
    const double rhokp = 1.0 / (2.0 * sigma - rhok);
    const double f1 = rhokp * rhok, f2 = 2.0 * rhokp / delta;
    rhok = rhokp;
    step(f1, f2);
  }
  if (cur != x) v_copy<T>(n, cur, x, H.st);
}

int smoothing_steps(const Handle& H, int block) { return block == 0 ? 1 : H.opt.schur_smoothing_steps; }

template <typename T>
void smoother_apply(Handle& H, int lev, int block, T* x, const T* b) {
  chebyshev<T>(H, lev, block, x, b, true);
  for (int k = 1; k < smoothing_steps(H, block); ++k) chebyshev<T>(H, lev, block, x, b, false);
}
template <typename T>
void smoother_smooth(Handle& H, int lev, int block, T* x, const T* b) {
  for (int k = 0; k < smoothing_steps(H, block); ++k) chebyshev<T>(H, lev, block, x, b, false);
}

// FP64 coarse-grid solve: sol = pinv(A_0) def, with the V-cycle's own precision at
// the boundary (the coarse vectors are cast to FP64 and back)
template <typename T>
void coarse_dense(Handle& H, int block, T* sol, const T* def) {
  Level& L = H.levels[0];
  const long n = block == 0 ? L.n_u : L.n_p;
  if constexpr (std::is_same<T, double>::value) {
    v_symv_dense(n, H.coarse_pinv[block].p, def, sol, H.st);
  } else {
    v_cast<float, double>(n, def, H.coarse_x.p, H.st);
    v_symv_dense(n, H.coarse_pinv[block].p, H.coarse_x.p, H.coarse_y.p, H.st);
    v_cast<double, float>(n, H.coarse_y.p, sol, H.st);
  }
}

// Levels 0..K of the FP32 mass V-cycle as one launch (see mass_bottom.cu): the
// same steps, coefficients and vectors as the multi-launch recursion below.
void fill_mass_bottom(Handle& H, int K, MassBottomArgs& A) {
  A = MassBottomArgs{};
  A.n_levels = K + 1;
  for (int l = 0; l <= K; ++l) {
    Level& L = H.levels[l];
    LevelDev<float>& D = L.f32;
    MassBottomLevel& V = A.lev[l];
    V.L = L.view<float>(H.s, H.compressible);
    V.Mc = D.Mp.p;
    V.dinv = D.dinvM.p;
    V.sol = D.solM.p;
    V.def = D.defM.p;
    V.d = D.dM.p;
    V.t = D.tM.p;
    if (l >= 1) {
      V.pt_rows = (int)L.PpT_rows;
      V.pt_ptr = L.PpT_ptr.p;
      V.pt_col = L.PpT_col.p;
      V.pt_val = D.PpT_val.p;
      V.p_rows = (int)L.Pp_rows;
      V.p_ptr = L.Pp_ptr.p;
      V.p_col = L.Pp_col.p;
      V.p_val = D.Pp_val.p;
    }
    const ChebParams cp = cheb_params(H, l);
    double theta, delta;
    chebyshev_bounds<float>(H, l, 1, theta, delta);
    V.degree = cp.degree;
    V.steps = smoothing_steps(H, 1);
    V.inv_theta = (float)(1.0 / theta);
    double rhok = delta / theta;
    const double sigma = theta / delta;
    for (int k = 1; k < cp.degree; ++k) {
      const double rhokp = 1.0 / (2.0 * sigma - rhok);
      V.f1[k] = (float)(rhokp * rhok);
      V.f2[k] = (float)(2.0 * rhokp / delta);
      rhok = rhokp;
    }
  }
}
void mass_bottom(Handle& H, int K) {
  MassBottomArgs A;
  fill_mass_bottom(H, K, A);
  launch_mass_vcycle_bottom(A, mass_bottom_layout(A), H.st);
  ++H.cell_launches;
}

// the highest level K such that levels 0..K qualify for mass_bottom: 3D lattice
// levels of at most kMaxBottomNodes pressure nodes whose shared-memory copies
// fit one block, the Chebyshev coarse solver, degrees that fit the argument
// block
int plan_mass_bottom(const Handle& H) {
  if (H.opt.coarse_solver != GB_GMG_COARSE_CHEBYSHEV) return -1;
  const int smem_limit = mass_bottom_reserve();
  MassBottomArgs A{};
  int K = -1;
  for (int l = 0; l < H.n_levels && l < kMaxBottomLevels; ++l) {
    const Level& L = H.levels[l];
    const int degree = cheb_params(H, l).degree;
    if (!L.structured || L.dim != 3 || L.n_p > kMaxBottomNodes || degree < 1 || degree > kMaxBottomDegree) break;
    A.n_levels = l + 1;
    A.lev[l].L.n_cells = (int)L.n_cells;
    A.lev[l].L.n_p = (int)L.n_p;
    if (mass_bottom_layout(A) > smem_limit) break;
    K = l;
  }
  return K;
}

// the highest level K whose cycle of levels 0..K becomes an explicit matrix
// (options.dense_mass_cycle_nodes; same qualification as plan_mass_bottom)
int plan_mass_dense(const Handle& H) {
  const int max_nodes = std::min(H.opt.dense_mass_cycle_nodes, kMaxDenseBottomNodes);
  if (H.opt.coarse_solver != GB_GMG_COARSE_CHEBYSHEV || max_nodes <= 0) return -1;
  const int smem_limit = mass_bottom_reserve();
  MassBottomArgs A{};
  int K = -1;
  for (int l = 0; l < H.n_levels && l < kMaxBottomLevels; ++l) {
    const Level& L = H.levels[l];
    const int degree = cheb_params(H, l).degree;
    if (!L.structured || L.dim != 3 || L.n_p > max_nodes || degree < 1 || degree > kMaxBottomDegree) break;
    A.n_levels = l + 1;
    A.lev[l].L.n_cells = (int)L.n_cells;
    A.lev[l].L.n_p = (int)L.n_p;
    if (mass_bottom_layout(A) > smem_limit) break;
    K = l;
  }
  return K;
}

// The FP32 mass cycle of levels 0..K is linear in its defect (Chebyshev steps
// with fixed coefficients from a zero start, the smoother as the coarse solver),
// so its matrix is the cycle applied to the unit vectors: one block per column,
// each running the single-block cycle (batch mode of mass_vcycle_bottom). Built
// after the eigenvalue estimates and again whenever they or the level tables change.
void build_mass_dense_next(Handle& H);
void build_mass_dense(Handle& H) {
  H.mass_dense_top = H.mass_dense_base = -1;
  if (!H.prec_done[1]) return;
  const int K = plan_mass_dense(H);
  if (K < 0) {
    H.mass_dense.release();
    H.mass_dense2.release();
    return;
  }
  const int n = (int)H.levels[K].n_p;
  MassBottomArgs A;
  fill_mass_bottom(H, K, A);
  H.mass_dense.alloc((size_t)n * n);
  A.batch_out = H.mass_dense.p;
  launch_mass_vcycle_bottom_batch(A, mass_bottom_layout(A), n, H.st);
  ++H.cell_launches;
  GB_CUDA(cudaStreamSynchronize(H.st));
  H.mass_dense_top = H.mass_dense_base = K;
  build_mass_dense_next(H);
}
const float* mass_dense_matrix(const Handle& H) {
  return H.mass_dense_top > H.mass_dense_base ? H.mass_dense2.p : H.mass_dense.p;
}

// The A-block counterpart: levels 0..K of 3D lattices with at most
// options.dense_a_cycle_dofs velocity DoFs on level K and one viscosity layout
void fill_a_bottom(Handle& H, int K, ABottomArgs& A) {
  A = ABottomArgs{};
  A.n_levels = K + 1;
  A.eta_per_q = H.levels[0].eta_n > 1;
  for (int l = 0; l <= K; ++l) {
    Level& L = H.levels[l];
    LevelDev<float>& D = L.f32;
    ABottomLevel& V = A.lev[l];
    V.L = L.view<float>(H.s, H.compressible);
    V.dinv = D.dinvA.p;
    if (l >= 1) {
      V.pt_rows = (int)L.PuT_rows;
      V.pt_ptr = L.PuT_ptr.p;
      V.pt_col = L.PuT_col.p;
      V.pt_val = D.PuT_val.p;
      V.p_rows = (int)L.Pu_rows;
      V.p_ptr = L.Pu_ptr.p;
      V.p_col = L.Pu_col.p;
      V.p_val = D.Pu_val.p;
    }
    const ChebParams cp = cheb_params(H, l);
    double theta, delta;
    chebyshev_bounds<float>(H, l, 0, theta, delta);
    V.degree = cp.degree;
    V.inv_theta = (float)(1.0 / theta);
    double rhok = delta / theta;
    const double sigma = theta / delta;
    for (int k = 1; k < cp.degree; ++k) {
      const double rhokp = 1.0 / (2.0 * sigma - rhok);
      V.f1[k] = (float)(rhokp * rhok);
      V.f2[k] = (float)(2.0 * rhokp / delta);
      rhok = rhokp;
    }
  }
}
int plan_a_dense(const Handle& H) {
  const int max_dofs = std::min(H.opt.dense_a_cycle_dofs, kMaxDenseANodes);
  if (H.opt.coarse_solver != GB_GMG_COARSE_CHEBYSHEV || max_dofs <= 0) return -1;
  const int smem_limit = a_bottom_reserve();
  ABottomArgs A{};
  int K = -1;
  for (int l = 0; l < H.n_levels && l < kMaxABottomLevels; ++l) {
    const Level& L = H.levels[l];
    const int degree = cheb_params(H, l).degree;
    if (!L.structured || L.dim != 3 || L.n_u > max_dofs || degree < 1 || degree > kMaxBottomDegree ||
        (L.eta_n > 1) != (H.levels[0].eta_n > 1))
      break;
    A.n_levels = l + 1;
    A.lev[l].L.n_cells = (int)L.n_cells;
    A.lev[l].L.n_u = (int)L.n_u;
    if (a_bottom_layout(A) > smem_limit) break;
    K = l;
  }
  return K;
}
void build_a_dense(Handle& H) {
  H.a_dense_top = -1;
  if (!H.prec_done[1]) return;
  const int K = plan_a_dense(H);
  if (K < 0) {
    H.a_dense.release();
    return;
  }
  const int n = (int)H.levels[K].n_u;
  ABottomArgs A;
  fill_a_bottom(H, K, A);
  H.a_dense.alloc((size_t)n * n);
  A.batch_out = H.a_dense.p;
  launch_a_vcycle_bottom_batch(A, a_bottom_layout(A), n, H.st);
  ++H.cell_launches;
  GB_CUDA(cudaStreamSynchronize(H.st));
  H.a_dense_top = K;
}

// FP32 A-block smoothing of small lattice levels with fused steps
// (lattice_cheb_small): each Chebyshev step's gather and the next step's cell
// pass in one launch, the iterate, direction and contributions in ping-pong
// pairs (sol/xalt, dA/dalt, Eu/Ealt). The same steps, coefficients, sums and
// residual as chebyshev() + level_op_resid(); pre-smoothing and residual in
// degree + 1 launches instead of 2 degree + 1, post-smoothing in degree + 1
// instead of 2 degree.
bool small_fused_level(Handle& H, int lev, int block) {
  Level& L = H.levels[lev];
  return block == 0 && H.opt.fused_small_smoother && L.f32.xalt.p && L.fused_tz == 0 &&
         small_lattice_a_level(L.view<float>(H.s, H.compressible));
}
// Chebyshev step coefficients (f1, f2) of a level, step 0 first (chebyshev())
std::vector<std::pair<float, float>> cheb_steps(Handle& H, int lev, int block) {
  const ChebParams cp = cheb_params(H, lev);
  double theta, delta;
  chebyshev_bounds<float>(H, lev, block, theta, delta);
  std::vector<std::pair<float, float>> c;
  c.push_back({0.0f, (float)(1.0 / theta)});
  double rhok = delta / theta;
  const double sigma = theta / delta;
  for (int k = 1; k < cp.degree; ++k) {
    const double rhokp = 1.0 / (2.0 * sigma - rhok);
    c.push_back({(float)(rhokp * rhok), (float)(2.0 * rhokp / delta)});
    rhok = rhokp;
  }
  return c;
}
// pre-smoothing from a zero start, then t = b - A sol
void small_presmooth_resid(Handle& H, int lev, float* sol, const float* b, float* t) {
  Level& L = H.levels[lev];
  LevelDev<float>& D = L.f32;
  const LevelView<float> v = L.view<float>(H.s, H.compressible);
  const std::vector<std::pair<float, float>> c = cheb_steps(H, lev, 0);
  float* X[2] = {sol, D.xalt.p};
  float* Dv[2] = {D.dA.p, D.dalt.p};
  float* E[2] = {D.Eu.p, D.Ealt.p};
  ChebSmallArgs a{};
  a.b = b;
  a.dinv = D.dinvA.p;
  a.x_out = X[1];
  a.d_out = Dv[1];
  a.E_out = E[0];
  a.f1 = 0.0f;
  a.f2 = c[0].second;
  launch_cheb_small(v, true, a, H.st);
  ++H.cell_launches;
  int cx = 1, ce = 0;
  for (size_t k = 1; k < c.size(); ++k) {
    a.E = E[ce];
    a.x_in = X[cx];
    a.d_in = Dv[cx];
    a.x_out = X[cx ^ 1];
    a.d_out = Dv[cx ^ 1];
    a.E_out = E[ce ^ 1];
    a.f1 = c[k].first;
    a.f2 = c[k].second;
    launch_cheb_small(v, false, a, H.st);
    ++H.cell_launches;
    cx ^= 1;
    ce ^= 1;
  }
  GatherArgs<float> g{};
  g.E = E[ce];
  g.x = X[cx];
  g.b = b;
  g.y = t;
  gather<float>(H, L, v, 0, EPI_RESID, g, OPK_A);
  if (X[cx] != sol) v_copy<float>(L.n_u, X[cx], sol, H.st);
}
// post-smoothing from sol
void small_postsmooth(Handle& H, int lev, float* sol, const float* b) {
  Level& L = H.levels[lev];
  LevelDev<float>& D = L.f32;
  const LevelView<float> v = L.view<float>(H.s, H.compressible);
  const std::vector<std::pair<float, float>> c = cheb_steps(H, lev, 0);
  float* X[2] = {sol, D.xalt.p};
  float* Dv[2] = {D.dA.p, D.dalt.p};
  float* E[2] = {D.Eu.p, D.Ealt.p};
  launch_cell_pass<float>(v, OPK_A, sol, sol, E[0], D.Ep.p, H.st);
  ++H.cell_launches;
  int cx = 0, ce = 0;
  ChebSmallArgs a{};
  a.b = b;
  a.dinv = D.dinvA.p;
  for (size_t k = 0; k + 1 < c.size(); ++k) {
    a.E = E[ce];
    a.x_in = X[cx];
    a.d_in = Dv[cx];
    a.x_out = X[cx ^ 1];
    a.d_out = Dv[cx ^ 1];
    a.E_out = E[ce ^ 1];
    a.f1 = c[k].first;
    a.f2 = c[k].second;
    launch_cheb_small(v, false, a, H.st);
    ++H.cell_launches;
    cx ^= 1;
    ce ^= 1;
  }
  GatherArgs<float> g{};
  g.E = E[ce];
  g.x = X[cx];
  g.y = X[cx ^ 1];
  g.b = b;
  g.dinv = D.dinvA.p;
  g.d = Dv[cx];
  g.f1 = c.back().first;
  g.f2 = c.back().second;
  gather<float>(H, L, v, 0, EPI_CHEB_OUT, g, OPK_A);
  cx ^= 1;
  if (X[cx] != sol) v_copy<float>(L.n_u, X[cx], sol, H.st);
}

template <typename T>
void vcycle_level(Handle& H, int lev, int block) {
  if constexpr (std::is_same<T, float>::value) {
    if (block == 0 && lev == H.a_dense_top) {
      const Level& L = H.levels[lev];
      launch_dense_gemv_colmajor((int)L.n_u, H.a_dense.p, L.f32.defA.p, H.levels[lev].f32.solA.p, H.st);
      ++H.cell_launches;
      return;
    }
    if (block == 1 && lev == H.mass_dense_top) {
      const Level& L = H.levels[lev];
      launch_dense_gemv_colmajor((int)L.n_p, mass_dense_matrix(H), L.f32.defM.p, H.levels[lev].f32.solM.p, H.st);
      ++H.cell_launches;
      return;
    }
    if (block == 1 && lev <= H.mass_bottom_top) {
      mass_bottom(H, lev);
      return;
    }
  }
  Level& L = H.levels[lev];
  LevelDev<T>& D = L.dev<T>();
  T* sol = block == 0 ? D.solA.p : D.solM.p;
  T* def = block == 0 ? D.defA.p : D.defM.p;
  T* t = block == 0 ? D.tA.p : D.tM.p;
  const long n = block == 0 ? L.n_u : L.n_p;
  if (lev == 0) {
    if (H.opt.coarse_solver == GB_GMG_COARSE_DENSE_FP64) coarse_dense<T>(H, block, sol, def);
    else smoother_apply<T>(H, 0, block, sol, def);
    return;
  }
  Level& C = H.levels[lev - 1];
  LevelDev<T>& DC = C.dev<T>();
  T* csol = block == 0 ? DC.solA.p : DC.solM.p;
  T* cdef = block == 0 ? DC.defA.p : DC.defM.p;
  const long nc = block == 0 ? C.n_u : C.n_p;
  bool fused = false;
  if constexpr (std::is_same<T, float>::value) fused = small_fused_level(H, lev, block);
  if constexpr (std::is_same<T, float>::value) {
    if (fused) small_presmooth_resid(H, lev, sol, def, t);
  }
  if (!fused) {
    smoother_apply<T>(H, lev, block, sol, def);
    level_op_resid<T>(H, lev, block, sol, def, t);
  }
  // restriction (zero fill and product in one launch)
  if (L.xfer_lattice[block]) lattice_restrict<T>(L.xfer[block], t, cdef, H.st);
  else if (block == 0) v_spmv_set<T>(L.PuT_rows, nc, L.PuT_ptr.p, L.PuT_col.p, D.PuT_val.p, t, cdef, H.st);
  else v_spmv_set<T>(L.PpT_rows, nc, L.PpT_ptr.p, L.PpT_col.p, D.PpT_val.p, t, cdef, H.st);
  // the coarse solution needs no zero fill: every coarse solve (the smoother from
  // a zero start, the single-block bottom, the dense coarse solve) writes all of it
  vcycle_level<T>(H, lev - 1, block);
  if (L.xfer_lattice[block]) lattice_prolong_add<T>(L.xfer[block], csol, sol, H.st);
  else if (block == 0) v_spmv_add<T>(L.Pu_rows, L.Pu_ptr.p, L.Pu_col.p, D.Pu_val.p, csol, sol, H.st);
  else v_spmv_add<T>(L.Pp_rows, L.Pp_ptr.p, L.Pp_col.p, D.Pp_val.p, csol, sol, H.st);
  if constexpr (std::is_same<T, float>::value) {
    if (fused) {
      small_postsmooth(H, lev, sol, def);
      return;
    }
  }
  smoother_smooth<T>(H, lev, block, sol, def);
}

// PreconditionMG::vmult: dst = V(src), FP64 internal vectors of the finest level
template <typename T>
void vcycle_T(Handle& H, int block, const double* src, double* dst) {
  const int top = H.n_levels - 1;
  Level& F = H.levels[top];
  LevelDev<T>& D = F.dev<T>();
  const long n = block == 0 ? F.n_u : F.n_p;
  T* def = block == 0 ? D.defA.p : D.defM.p;
  T* sol = block == 0 ? D.solA.p : D.solM.p;
  if constexpr (std::is_same<T, double>::value) v_copy<double>(n, src, def, H.st);
  else v_cast<double, float>(n, src, def, H.st);
  vcycle_level<T>(H, top, block);
  if constexpr (std::is_same<T, double>::value) v_copy<double>(n, sol, dst, H.st);
  else v_cast<float, double>(n, sol, dst, H.st);
}
// The V-cycle of one block and precision is a fixed launch sequence (all
// Chebyshev coefficients are known once the eigenvalues are), so it is captured
// once into a CUDA graph and replayed; the FP64 input and output go through
// staging vectors whose addresses are baked into the graph.
//
// GB_GMG_VCYCLE_GRAPHS=0 in the environment (read once per process) issues the
// same launch sequence directly on the stream instead, so that profilers that
// replay kernels one at a time see ordinary launches.
bool vcycle_graphs_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GB_GMG_VCYCLE_GRAPHS");
    return !(e && std::strcmp(e, "0") == 0);
  }();
  return on;
}

// Turns every kernel -> kernel edge of a captured graph into a programmatic
// dependency on the launch completion of the upstream kernel: the downstream
// kernel may be scheduled once all blocks of its predecessor have started, and
// its blocks wait in pdl_wait() until the predecessor has finished. This hides
// the launch latency between the ~100 short kernels of a V-cycle; the order and
// the arithmetic are unchanged.
void programmatic_kernel_edges(cudaGraph_t g) {
  size_t ne = 0;
  GB_CUDA(cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &ne));
  if (!ne) return;
  std::vector<cudaGraphNode_t> from(ne), to(ne);
  std::vector<cudaGraphEdgeData> data(ne);
  GB_CUDA(cudaGraphGetEdges(g, from.data(), to.data(), data.data(), &ne));
  for (size_t i = 0; i < ne; ++i) {
    cudaGraphNodeType tf, tt;
    GB_CUDA(cudaGraphNodeGetType(from[i], &tf));
    GB_CUDA(cudaGraphNodeGetType(to[i], &tt));
    if (tf != cudaGraphNodeTypeKernel || tt != cudaGraphNodeTypeKernel) continue;
    if (data[i].type != cudaGraphDependencyTypeDefault || data[i].from_port != cudaGraphKernelNodePortDefault) continue;
    GB_CUDA(cudaGraphRemoveDependencies(g, &from[i], &to[i], &data[i], 1));
    cudaGraphEdgeData e{};
    e.from_port = cudaGraphKernelNodePortLaunchCompletion;
    e.type = cudaGraphDependencyTypeProgrammatic;
    GB_CUDA(cudaGraphAddDependencies(g, &from[i], &to[i], &e, 1));
  }
}

void vcycle_exec(Handle& H, int block, int prec, const double* src, double* dst) {
  const int pi = prec == GB_GMG_FP32 ? 1 : 0;
  Level& F = H.top();
  const long n = block == 0 ? F.n_u : F.n_p;
  if (!vcycle_graphs_enabled()) {
    if (pi) vcycle_T<float>(H, block, src, dst);
    else vcycle_T<double>(H, block, src, dst);
    return;
  }
  if (!H.vgraph[block][pi]) {
    const long long c0 = H.cell_launches, v0 = VecCounter::launches();
    cudaGraph_t graph = nullptr;
    GB_CUDA(cudaStreamBeginCapture(H.st, cudaStreamCaptureModeThreadLocal));
    try {
      if (pi) vcycle_T<float>(H, block, H.vin.p, H.vout.p);
      else vcycle_T<double>(H, block, H.vin.p, H.vout.p);
    } catch (...) {
      cudaStreamEndCapture(H.st, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    GB_CUDA(cudaStreamEndCapture(H.st, &graph));
    programmatic_kernel_edges(graph);
    GB_CUDA(cudaGraphInstantiate(&H.vgraph[block][pi], graph, 0));
    size_t nn = 0;
    GB_CUDA(cudaGraphGetNodes(graph, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    GB_CUDA(cudaGraphGetNodes(graph, nodes.data(), &nn));
    long long nk = 0;
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      GB_CUDA(cudaGraphNodeGetType(nd, &t));
      if (t == cudaGraphNodeTypeKernel) ++nk;
    }
    H.vgraph_kernels[block][pi] = nk;
    cudaGraphDestroy(graph);
    H.cell_launches = c0;  // capture issued nothing; replays are counted below
    VecCounter::launches() = v0;
  }
  v_copy<double>(n, src, H.vin.p, H.st);
  GB_CUDA(cudaGraphLaunch(H.vgraph[block][pi], H.st));
  H.cell_launches += H.vgraph_kernels[block][pi];
  v_copy<double>(n, H.vout.p, dst, H.st);
}

void vcycle(Handle& H, int block, int prec, const double* src, double* dst) {
  if (block == 0) ++H.nA; else ++H.nS;
  vcycle_exec(H, block, prec, src, dst);
}

// ---------------------------------------------------------------- FP64 active-level operators
void stokes64(Handle& H, const double* x, double* y) {
  Level& F = H.top();
  apply_op<double>(H, H.n_levels - 1, OPK_STOKES, x, x + F.n_u, y, y + F.n_u, true);
  ++H.n_stokes64;
}
// Stokes operator with FP32 arithmetic on FP64 vectors (inner solves of GMRES_IR)
void stokes32(Handle& H, const double* x, double* y) {
  Level& F = H.top();
  const long n = F.n_u + F.n_p;
  v_cast<double, float>(n, x, H.f32_a.p, H.st);
  apply_op<float>(H, H.n_levels - 1, OPK_STOKES, H.f32_a.p, H.f32_a.p + F.n_u, H.f32_b.p, H.f32_b.p + F.n_u, true);
  v_cast<float, double>(n, H.f32_b.p, y, H.st);
}

// ---------------------------------------------------------------- block preconditioner
int cg_solve(Handle& H, int block, int prec, long n, double* x, const double* b, double tol, int maxit);

void block_preconditioner(Handle& H, int prec, bool expensive, const gb_gmg_solve_params* P, const double* src,
                          double* dst) {
  Level& F = H.top();
  const long nu = F.n_u, np = F.n_p;
  if (!expensive) {
    vcycle(H, 1, prec, src + nu, dst + nu);
  } else {
    const double sn = std::sqrt(dot_host(H, np, src + nu, src + nu));
    GB_CUDA(cudaMemsetAsync(dst + nu, 0, np * sizeof(double), H.st));
    if (sn > 1e-50) H.nS += cg_solve(H, 1, prec, np, dst + nu, src + nu, sn * P->tol_S, 100) - 0;
  }
  v_scale<double>(np, -1.0, dst + nu, H.st);
  if (prec == GB_GMG_FP32) {
    // with FP32 V-cycles the B^T product of the preconditioner is FP32 as well:
    // its result only feeds the FP32 velocity V-cycle
    float* p32 = H.f32_a.p + nu;
    float* bt32 = H.f32_b.p;
    v_cast<double, float>(np, dst + nu, p32, H.st);
    apply_op<float>(H, H.n_levels - 1, OPK_BT, nullptr, p32, bt32, nullptr);
    v_cast<float, double>(nu, bt32, H.t2v.p, H.st);
  } else {
    apply_op<double>(H, H.n_levels - 1, OPK_BT, nullptr, dst + nu, H.t2v.p, nullptr);
  }
  v_axpby<double>(nu, 1.0, src, -1.0, H.t2v.p, H.st);  // t = src_u - B^T p
  if (!expensive) {
    vcycle(H, 0, prec, H.t2v.p, dst);
  } else {
    const double tn = std::sqrt(dot_host(H, nu, H.t2v.p, H.t2v.p));
    H.nA += cg_solve(H, 0, prec, nu, dst, H.t2v.p, tn * P->tol_A, 10000);
  }
}

// preconditioned CG of the expensive inner solves (FP64 operator, V-cycle preconditioner)
int cg_solve(Handle& H, int block, int prec, long n, double* x, const double* b, double tol, int maxit) {
  const int top = H.n_levels - 1;
  double* r = H.cg_r.p;
  double* z = H.cg_z.p;
  double* p = H.cg_p.p;
  double* q = H.cg_q.p;
  auto op = [&](const double* a, double* y) {
    if (block == 0) apply_op<double>(H, top, OPK_A, a, nullptr, y, nullptr, true);
    else apply_op<double>(H, top, OPK_MASS, nullptr, a, nullptr, y, true);
  };
  auto pre = [&](const double* a, double* y) { vcycle_exec(H, block, prec, a, y); };
  GB_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), H.st));
  v_copy<double>(n, b, r, H.st);
  double rn = std::sqrt(dot_host(H, n, r, r));
  if (rn <= tol) return 0;
  pre(r, z);
  v_copy<double>(n, z, p, H.st);
  double rz = dot_host(H, n, r, z);
  for (int it = 1; it <= maxit; ++it) {
    op(p, q);
    const double alpha = rz / dot_host(H, n, p, q);
    v_axpby<double>(n, alpha, p, 1.0, x, H.st);
    v_axpby<double>(n, -alpha, q, 1.0, r, H.st);
    rn = std::sqrt(dot_host(H, n, r, r));
    if (rn <= tol) return it;
    pre(r, z);
    const double rz2 = dot_host(H, n, r, z);
    const double beta = rz2 / rz;
    rz = rz2;
    v_axpby<double>(n, 1.0, z, beta, p, H.st);
  }
  throw Error(GB_GMG_NO_CONVERGENCE, "iterative inner CG solver did not converge");
}

// ---------------------------------------------------------------- GMRES / FGMRES
void ensure_krylov(Handle& H, int restart) {
  const long n = H.n_top();
  if (H.restart_alloc >= restart) return;
  H.V.alloc((size_t)(restart + 1) * n);
  H.Z.alloc((size_t)restart * n);
  H.lds = (n + 1) / 2 * 2;  // even: 16-byte aligned columns of float pairs
  H.Vs.alloc((size_t)(restart + 1) * H.lds);
  H.gs_shift.alloc(2);
  GB_CUDA(cudaMemsetAsync(H.gs_shift.p, 0, 2 * sizeof(int), H.st));
  H.coef_d.alloc(restart + 2);
  H.hcol_d.alloc(restart + 2);
  H.arn_d.alloc(3);
  H.arn_flag.alloc(1);
  if (H.dots_d.n < (size_t)restart + 2) {
    H.dots_d.alloc(restart + 2);
    if (H.dots_h) cudaFreeHost(H.dots_h);
    H.dots_h = nullptr;
    GB_CUDA(cudaMallocHost(&H.dots_h, (restart + 2) * sizeof(double)));
  }
  H.restart_alloc = restart;
}

// next basis vector v = w / h[j+1] (the reciprocal is formed once, in k_cgs_update)
__global__ void k_next_basis(long n, const double* __restrict__ arn, const double* __restrict__ w,
                             double* __restrict__ v) {
  pdl_wait();
  const double sc = arn[2];
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    v[i] = sc * w[i];
}

// Solves K x = b (right preconditioning). Returns iterations.
int gmres(Handle& H, double* x, const double* b, double tol, int maxit, int restart, bool flexible,
          bool expensive, int prec, bool fp32_operator, const gb_gmg_solve_params* P, bool& converged,
          double& final_res) {
  const long n = H.n_top();
  ensure_krylov(H, restart);
  const bool float_pair = !P || P->orthogonalization == GB_GMG_GS_FLOAT_PAIR;
  double* V = H.V.p;
  double* Z = H.Z.p;
  double* w = H.wv.p;
  double* r = H.rv.p;
  double* tmp = H.tv.p;
  auto K = [&](const double* a, double* y) {
    if (fp32_operator) stokes32(H, a, y);
    else stokes64(H, a, y);
  };
  int it = 0;
  converged = false;
  while (true) {
    K(x, tmp);
    v_copy<double>(n, b, r, H.st);
    v_axpby<double>(n, -1.0, tmp, 1.0, r, H.st);
    const double beta = std::sqrt(dot_host(H, n, r, r));
    final_res = beta;
    GB_CHECK(std::isfinite(beta), GB_GMG_NAN_DETECTED, "NaN or Inf in the Stokes residual");
    if (beta <= tol) { converged = true; return it; }
    if (it >= maxit) return it;
    if (float_pair) {
      v_basis_df(n, nullptr, 1.0 / beta, r, V, H.Vs.p, H.st);
    } else {
      v_copy<double>(n, r, V, H.st);
      v_scale<double>(n, 1.0 / beta, V, H.st);
    }
    std::vector<std::vector<double>> Hc;
    std::vector<double> cs, sn, g(1, beta);
    int j = 0;
    for (; j < restart && it < maxit; ++j) {
      double* vj = V + (size_t)j * n;
      double* zj = flexible ? Z + (size_t)j * n : H.xv.p;
      block_preconditioner(H, prec, expensive, P, vj, zj);
      K(zj, w);
      ++it;
      // classical Gram-Schmidt with one conditional re-orthogonalisation, all
      // scalars on the device: the second pass runs only if the device finds
      // |w| <= 0.7 |w before|, and the one round trip per step is the copy of
      // the finished Hessenberg column for the Givens update below
      double* hcol = H.hcol_d.p;
      double* arn = H.arn_d.p;
      int* need2 = H.arn_flag.p;
      double* vnext = V + (size_t)(j + 1) * n;
      int* shift = H.gs_shift.p;
      if (float_pair && j >= 1 && j + 1 <= kGsMaxK) {
        v_arnoldi_step_df(n, j, H.Vs.p, H.lds, w, vnext, H.Vs.p + (size_t)(j + 1) * H.lds, hcol, arn, need2,
                          shift + (j & 1), shift + ((j + 1) & 1), H.partial.p, H.st);
      } else {
        // FP64 passes (also the first step of a float-pair solve: it sets the
        // scale exponent of the next step)
        v_multidot(n, w, V, n, j + 1, true, H.dots_d.p, H.partial.p, H.st);
        v_cgs_update(n, j, 0, H.dots_d.p, V, n, w, hcol, arn, need2, H.partial.p, H.st,
                     float_pair ? shift + ((j + 1) & 1) : nullptr);
        v_multidot(n, w, V, n, j + 1, false, H.dots_d.p, H.partial.p, H.st, need2);
        v_cgs_update(n, j, 1, H.dots_d.p, V, n, w, hcol, arn, need2, H.partial.p, H.st);
        if (float_pair) {
          v_basis_df(n, arn + 2, 0.0, w, vnext, H.Vs.p + (size_t)(j + 1) * H.lds, H.st);
        } else {
          k_next_basis<<<ceil_div(n, 256), 256, 0, H.st>>>(n, arn, w, vnext);
          VecCounter::launches() += 1;
        }
      }
      GB_CUDA(cudaMemcpyAsync(H.dots_h, hcol, (j + 2) * sizeof(double), cudaMemcpyDeviceToHost, H.st));
      GB_CUDA(cudaStreamSynchronize(H.st));
      std::vector<double> h(H.dots_h, H.dots_h + j + 2);
      const double hn = h[j + 1];
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * h[i] + sn[i] * h[i + 1];
        h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
        h[i] = t;
      }
      const double den = std::hypot(h[j], h[j + 1]);
      GB_CHECK(den > 0 && std::isfinite(den), GB_GMG_BREAKDOWN, "GMRES breakdown");
      const double c_ = h[j] / den, s_ = h[j + 1] / den;
      cs.push_back(c_);
      sn.push_back(s_);
      h[j] = den;
      h[j + 1] = 0;
      g.push_back(-s_ * g[j]);
      g[j] = c_ * g[j];
      Hc.push_back(h);
      (void)hn;
      final_res = std::fabs(g[j + 1]);
      if (final_res <= tol) { ++j; break; }
    }
    const int m = j;
    std::vector<double> y(m);
    for (int i = m - 1; i >= 0; --i) {
      double t = g[i];
      for (int k = i + 1; k < m; ++k) t -= Hc[k][i] * y[k];
      y[i] = t / Hc[i][i];
    }
    GB_CUDA(cudaMemcpyAsync(H.coef_d.p, y.data(), m * sizeof(double), cudaMemcpyHostToDevice, H.st));
    if (flexible) {
      v_multiaxpy(n, m, H.coef_d.p, Z, n, x, H.st);
    } else {
      GB_CUDA(cudaMemsetAsync(tmp, 0, n * sizeof(double), H.st));
      v_multiaxpy(n, m, H.coef_d.p, V, n, tmp, H.st);
      block_preconditioner(H, prec, expensive, P, tmp, H.xv.p);
      v_axpby<double>(n, 1.0, H.xv.p, 1.0, x, H.st);
    }
    // the next pass starts from the true FP64 residual of the updated iterate:
    // convergence is only reported on that residual
  }
}

// ---------------------------------------------------------------- IDR(s)
void to_internal(Handle& H, int lev, const double* d_caller, double* d_internal, bool with_u, bool with_p);

// Shadow space of IDR(s): s vectors in the caller's numbering, entries uniform
// in [-1, 1) from a SplitMix64 stream per vector (seed + i), orthonormalised by
// modified Gram-Schmidt in FP64. The oracle builds the same vectors, so both
// run IDR(s) with the same space.
uint64_t splitmix64_next(uint64_t& state) {
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
std::vector<double> idr_shadow_space(long n, int s, uint64_t seed) {
  std::vector<double> P((size_t)s * n);
  for (int i = 0; i < s; ++i) {
    uint64_t st = seed + (uint64_t)i;
    double* p = P.data() + (size_t)i * n;
    for (long k = 0; k < n; ++k) p[k] = 2.0 * ((double)(splitmix64_next(st) >> 11) * 0x1.0p-53) - 1.0;
    for (int j = 0; j < i; ++j) {
      const double* q = P.data() + (size_t)j * n;
      double d = 0;
      for (long k = 0; k < n; ++k) d += p[k] * q[k];
      for (long k = 0; k < n; ++k) p[k] -= d * q[k];
    }
    double nn = 0;
    for (long k = 0; k < n; ++k) nn += p[k] * p[k];
    nn = std::sqrt(nn);
    for (long k = 0; k < n; ++k) p[k] /= nn;
  }
  return P;
}
constexpr uint64_t kIdrSeed = 20261204ull;

// IDR(s) with bi-orthogonalisation and right preconditioning: the published
// algorithm of van Gijzen and Sonneveld ("Algorithm 913", ACM TOMS 38, 2011),
// the method behind the reference's "Krylov method for cheap solver steps =
// IDR(s)" (source/simulator/solver/stokes_matrix_free_local_smoothing.cc:1290-1299,
// deal.II SolverIDR). One iteration = s inner steps plus one dimension-reduction
// step, s + 1 preconditioner and operator applications; convergence is checked
// after every residual update and counted in iterations, as the reference
// prints them. omega = (t, r) / (t, t). The recursively updated residual is
// confirmed against the true FP64 residual at the end; if they disagree (FP32
// V-cycles are not exactly linear) IDR(s) restarts from the true residual.
int idr(Handle& H, double* x, const double* b, double tol, int maxit, int s, int prec,
        const gb_gmg_solve_params* P, bool& converged, double& final_res) {
  const long n = H.n_top();
  GB_CHECK(s >= 1 && s <= 8, GB_GMG_INVALID_ARGUMENT, "IDR(s) parameter must be in 1..8");
  if (H.coef_d.n < (size_t)s) H.coef_d.alloc(s);  // (GMRES sizes it restart + 2 when it runs first)
  if (H.idr_s_alloc != s) {
    H.idrP.alloc((size_t)s * n);
    H.idrG.alloc((size_t)s * n);
    H.idrU.alloc((size_t)s * n);
    // built in the caller's numbering, staged in the G block, mapped to the internal one
    const std::vector<double> Ph = idr_shadow_space(n, s, kIdrSeed);
    GB_CUDA(cudaMemcpyAsync(H.idrG.p, Ph.data(), Ph.size() * sizeof(double), cudaMemcpyHostToDevice, H.st));
    for (int i = 0; i < s; ++i)
      to_internal(H, H.n_levels - 1, H.idrG.p + (size_t)i * n, H.idrP.p + (size_t)i * n, true, true);
    GB_CUDA(cudaStreamSynchronize(H.st));
    H.idr_s_alloc = s;
  }
  const double* Pm = H.idrP.p;
  double* G = H.idrG.p;
  double* U = H.idrU.p;
  double* r = H.rv.p;
  double* v = H.wv.p;
  double* t = H.tv.p;
  double* tmp = H.xv.p;  // not t2v: block_preconditioner uses t2v as scratch
  double* dd = H.dots_d.p;
  auto fetch = [&](int k) {  // k doubles of dots_d -> host
    GB_CUDA(cudaMemcpyAsync(H.dots_h, dd, k * sizeof(double), cudaMemcpyDeviceToHost, H.st));
    GB_CUDA(cudaStreamSynchronize(H.st));
    return std::vector<double>(H.dots_h, H.dots_h + k);
  };
  auto upload_coef = [&](const std::vector<double>& c) {
    GB_CUDA(cudaMemcpyAsync(H.coef_d.p, c.data(), c.size() * sizeof(double), cudaMemcpyHostToDevice, H.st));
  };
  int it = 0;
  converged = false;
  while (true) {
    stokes64(H, x, t);
    v_copy<double>(n, b, r, H.st);
    v_axpby<double>(n, -1.0, t, 1.0, r, H.st);
    double normr = std::sqrt(dot_host(H, n, r, r));
    final_res = normr;
    GB_CHECK(std::isfinite(normr), GB_GMG_NAN_DETECTED, "NaN or Inf in the Stokes residual");
    if (normr <= tol) { converged = true; return it; }
    if (it >= maxit) return it;
    v_zero<double>((size_t)s * n, G, H.st);
    v_zero<double>((size_t)s * n, U, H.st);
    std::vector<double> M((size_t)s * s, 0.0);  // M[i*s + k] = (P_i, G_k)
    for (int i = 0; i < s; ++i) M[(size_t)i * s + i] = 1.0;
    double om = 1.0;
    bool inner_conv = false;
    while (it < maxit && !inner_conv) {
      ++it;
      v_multidot(n, r, Pm, n, s, false, dd, H.partial.p, H.st);
      std::vector<double> f = fetch(s);
      for (int k = 0; k < s && !inner_conv; ++k) {
        // c from the lower-triangular system M(k:s, k:s) c = f(k:s)
        std::vector<double> c(s - k);
        for (int i = k; i < s; ++i) {
          double acc = f[i];
          for (int l = k; l < i; ++l) acc -= M[(size_t)i * s + l] * c[l - k];
          c[i - k] = acc / M[(size_t)i * s + i];
        }
        // v = r - sum c_i G_i, preconditioned; U_k = om v + sum c_i U_i; G_k = K U_k
        v_copy<double>(n, r, tmp, H.st);
        std::vector<double> mc(s - k);
        for (int i = 0; i < s - k; ++i) mc[i] = -c[i];
        upload_coef(mc);
        v_multiaxpy(n, s - k, H.coef_d.p, G + (size_t)k * n, n, tmp, H.st);
        block_preconditioner(H, prec, false, P, tmp, v);
        v_copy<double>(n, v, tmp, H.st);
        v_scale<double>(n, om, tmp, H.st);
        upload_coef(c);
        v_multiaxpy(n, s - k, H.coef_d.p, U + (size_t)k * n, n, tmp, H.st);
        double* Uk = U + (size_t)k * n;
        double* Gk = G + (size_t)k * n;
        v_copy<double>(n, tmp, Uk, H.st);
        stokes64(H, Uk, Gk);
        // bi-orthogonalise G_k against P_0 .. P_{k-1}
        for (int i = 0; i < k; ++i) {
          const double alpha = dot_host(H, n, Pm + (size_t)i * n, Gk) / M[(size_t)i * s + i];
          v_axpby<double>(n, -alpha, G + (size_t)i * n, 1.0, Gk, H.st);
          v_axpby<double>(n, -alpha, U + (size_t)i * n, 1.0, Uk, H.st);
        }
        v_multidot(n, Gk, Pm + (size_t)k * n, n, s - k, false, dd, H.partial.p, H.st);
        const std::vector<double> mk = fetch(s - k);
        for (int i = k; i < s; ++i) M[(size_t)i * s + k] = mk[i - k];
        const double mkk = M[(size_t)k * s + k];
        GB_CHECK(mkk != 0.0 && std::isfinite(mkk), GB_GMG_BREAKDOWN, "IDR(s) breakdown");
        const double beta = f[k] / mkk;
        v_axpby<double>(n, -beta, Gk, 1.0, r, H.st);
        v_axpby<double>(n, beta, Uk, 1.0, x, H.st);
        normr = std::sqrt(dot_host(H, n, r, r));
        final_res = normr;
        GB_CHECK(std::isfinite(normr), GB_GMG_NAN_DETECTED, "NaN or Inf in the IDR(s) residual");
        if (normr <= tol) { inner_conv = true; break; }
        for (int i = k + 1; i < s; ++i) f[i] -= beta * M[(size_t)i * s + k];
      }
      if (inner_conv) break;
      // dimension reduction: v = B r, t = K v, om = (t, r) / (t, t)
      block_preconditioner(H, prec, false, P, r, v);
      stokes64(H, v, t);
      v_multidot(n, t, r, n, 1, true, dd, H.partial.p, H.st);
      const std::vector<double> tr = fetch(2);
      GB_CHECK(tr[1] > 0 && std::isfinite(tr[1]), GB_GMG_BREAKDOWN, "IDR(s) breakdown");
      om = tr[0] / tr[1];
      v_axpby<double>(n, om, v, 1.0, x, H.st);
      v_axpby<double>(n, -om, t, 1.0, r, H.st);
      normr = std::sqrt(dot_host(H, n, r, r));
      final_res = normr;
      GB_CHECK(std::isfinite(normr), GB_GMG_NAN_DETECTED, "NaN or Inf in the IDR(s) residual");
      if (normr <= tol) inner_conv = true;
    }
    // loop back: the true residual of the iterate decides
  }
}

// ---------------------------------------------------------------- the solve
void ensure_workspace(Handle& H) {
  const long n = H.n_top();
  long nmax = 0;
  for (auto& L : H.levels) nmax = std::max(nmax, L.n_u + L.n_p);
  H.stage_a.alloc(nmax);
  H.stage_b.alloc(nmax);
  for (DevBuf<double>* b : {&H.wv, &H.xv, &H.rv, &H.bv, &H.tv, &H.t2v, &H.cg_r, &H.cg_z, &H.cg_p, &H.cg_q, &H.cg_x})
    if (b->n != (size_t)n) { b->alloc(n); b->zero(H.st); }
  H.f32_a.alloc(n);
  H.f32_b.alloc(n);
  H.vin.alloc(n);
  H.vout.alloc(n);
  if (H.partial.n != (size_t)kDotWorkspaceDoubles) {
    H.partial.alloc(kDotWorkspaceDoubles);
    H.partial.zero(H.st);  // the arrival counters start at zero
  }
  H.dots_d.alloc(256);
  if (!H.dots_h) GB_CUDA(cudaMallocHost(&H.dots_h, 256 * sizeof(double)));
  if (!H.flag_d) GB_CUDA(cudaMalloc(&H.flag_d, sizeof(int)));
}

template <typename T>
void alloc_level_work(Level& L, cudaStream_t st) {
  LevelDev<T>& D = L.dev<T>();
  for (DevBuf<T>* b : {&D.solA, &D.defA, &D.tA, &D.dA}) { b->alloc(L.n_u); b->zero(st); }
  for (DevBuf<T>* b : {&D.solM, &D.defM, &D.tM, &D.dM}) { b->alloc(L.n_p); b->zero(st); }
}

__global__ void k_symmetrize(long n, double* M) {
  pdl_wait();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n * n) return;
  const long r = i % n, c = i / n;
  if (r < c) {
    const double v = 0.5 * (M[r + c * n] + M[c + r * n]);
    M[r + c * n] = v;
    M[c + r * n] = v;
  }
}
__global__ void k_scale_columns(long n, const double* V, const double* sc, double* U) {
  pdl_wait();
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n * n) return;
  U[i] = V[i] * sc[i / n];
}

#define GB_CUSOLVER(x)                                                                     \
  do {                                                                                     \
    if ((x) != CUSOLVER_STATUS_SUCCESS) throw ::gb::Error(3, "cuSOLVER error in " #x);     \
  } while (0)
#define GB_CUBLAS(x)                                                                       \
  do {                                                                                     \
    if ((x) != CUBLAS_STATUS_SUCCESS) throw ::gb::Error(3, "cuBLAS error in " #x);         \
  } while (0)

// The FP32 mass cycle of levels 0..K+1 as a matrix, from that of levels 0..K
// (mass_dense): the multi-launch steps of level K+1 -- Chebyshev pre-smoothing
// from a zero start, the residual, the restriction, the coarse product, the
// prolongation, the post-smoothing -- each run once over all n unit vectors of
// level K+1 as n columns (batched kernels, the coarse product one SGEMM),
// with the coefficients and vectors of the multi-launch cycle.
void build_mass_dense_next(Handle& H) {
  const int K = H.mass_dense_base;
  const int max_nodes = std::min(H.opt.dense_mass_cycle_nodes, kMaxDenseNextNodes);
  if (K < 0 || K + 1 >= H.n_levels) {
    H.mass_dense2.release();
    return;
  }
  Level& L = H.levels[K + 1];
  if (!L.structured || L.dim != 3 || L.n_p > max_nodes) {
    H.mass_dense2.release();
    return;
  }
  const int n = (int)L.n_p, m = n, nc = (int)H.levels[K].n_p;
  LevelDev<float>& D = L.f32;
  const LevelView<float> v = L.view<float>(H.s, H.compressible);
  const size_t nm = (size_t)n * m;
  DevBuf<float> X, T, Dd, B, CD, CS;
  X.alloc(nm);
  T.alloc(nm);
  Dd.alloc(nm);
  B.alloc(nm);
  CD.alloc((size_t)nc * m);
  CS.alloc((size_t)nc * m);
  launch_unit_columns(n, m, B.p, H.st);
  const ChebParams cp = cheb_params(H, K + 1);
  double theta, delta;
  chebyshev_bounds<float>(H, K + 1, 1, theta, delta);
  auto cheb = [&](bool zero_start) {
    float* cur = X.p;
    auto step = [&](double f1, double f2) {
      float* nxt = cur == X.p ? T.p : X.p;
      GatherArgs<float> a{};
      a.x = cur;
      a.y = nxt;
      a.b = B.p;
      a.dinv = D.dinvM.p;
      a.d = Dd.p;
      a.f1 = (float)f1;
      a.f2 = (float)f2;
      launch_mass_lattice_batched(v, D.Mp.p, EPI_CHEB_OUT, a, m, H.st);
      cur = nxt;
    };
    if (zero_start) launch_cheb_first_batched(n, m, B.p, D.dinvM.p, (float)(1.0 / theta), Dd.p, X.p, H.st);
    else step(0.0, 1.0 / theta);
    double rhok = delta / theta;
    const double sigma = theta / delta;
    for (int k = 1; k < cp.degree; ++k) {
      const double rhokp = 1.0 / (2.0 * sigma - rhok);
      const double f1 = rhokp * rhok, f2 = 2.0 * rhokp / delta;
      rhok = rhokp;
      step(f1, f2);
    }
    if (cur != X.p) launch_copy_batched(n, m, cur, X.p, H.st);
  };
  const int steps = smoothing_steps(H, 1);
  cheb(true);
  for (int k = 1; k < steps; ++k) cheb(false);
  {
    GatherArgs<float> a{};
    a.x = X.p;
    a.b = B.p;
    a.y = T.p;
    launch_mass_lattice_batched(v, D.Mp.p, EPI_RESID, a, m, H.st);
  }
  launch_spmv_batched((int)L.PpT_rows, L.PpT_ptr.p, L.PpT_col.p, D.PpT_val.p, T.p, n, CD.p, nc, m, false, H.st);
  {
    cublasHandle_t blas = nullptr;
    GB_CUBLAS(cublasCreate(&blas));
    const float one = 1.0f, zero = 0.0f;
    const cublasStatus_t st1 = cublasSetStream(blas, H.st);
    const cublasStatus_t st2 = st1 != CUBLAS_STATUS_SUCCESS
                                   ? st1
                                   : cublasSgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, nc, m, nc, &one, H.mass_dense.p, nc,
                                                 CD.p, nc, &zero, CS.p, nc);
    GB_CUDA(cudaStreamSynchronize(H.st));
    cublasDestroy(blas);
    GB_CUBLAS(st2);
  }
  launch_spmv_batched((int)L.Pp_rows, L.Pp_ptr.p, L.Pp_col.p, D.Pp_val.p, CS.p, nc, X.p, n, m, true, H.st);
  for (int k = 0; k < steps; ++k) cheb(false);
  H.mass_dense2.alloc(nm);  // same size on a rebuild: same address for captured V-cycles
  GB_CUDA(cudaMemcpyAsync(H.mass_dense2.p, X.p, nm * sizeof(float), cudaMemcpyDeviceToDevice, H.st));
  GB_CUDA(cudaStreamSynchronize(H.st));
  H.cell_launches += 8 * (long long)cp.degree + 8;
  H.mass_dense_top = K + 1;
}

// Dense FP64 pseudo-inverses of the level-0 A and mass matrices: the matrices are
// assembled column by column from the FP64 level operator, eigendecomposed once
// (cuSOLVER syevd), and eigenvalues below 1e-10 lambda_max (null spaces) dropped.
void build_dense_coarse(Handle& H) {
  Level& L = H.levels[0];
  cusolverDnHandle_t sol = nullptr;
  cublasHandle_t blas = nullptr;
  GB_CUSOLVER(cusolverDnCreate(&sol));
  GB_CUBLAS(cublasCreate(&blas));
  try {
    GB_CUSOLVER(cusolverDnSetStream(sol, H.st));
    GB_CUBLAS(cublasSetStream(blas, H.st));
    const long nmax = std::max(L.n_u, L.n_p);
    H.coarse_x.alloc(nmax);
    H.coarse_y.alloc(nmax);
    for (int block = 0; block < 2; ++block) {
      const long n = block == 0 ? L.n_u : L.n_p;
      DevBuf<double> M, U, W, work;
      M.alloc((size_t)n * n);
      U.alloc((size_t)n * n);
      W.alloc(n);
      double* e = H.coarse_x.p;
      GB_CUDA(cudaMemsetAsync(e, 0, n * sizeof(double), H.st));
      const double one = 1.0, zero = 0.0;
      for (long j = 0; j < n; ++j) {
        GB_CUDA(cudaMemcpyAsync(e + j, &one, sizeof(double), cudaMemcpyHostToDevice, H.st));
        level_op<double>(H, 0, block, e, M.p + (size_t)j * n);
        GB_CUDA(cudaMemcpyAsync(e + j, &zero, sizeof(double), cudaMemcpyHostToDevice, H.st));
        GB_CUDA(cudaStreamSynchronize(H.st));  // the host scalars above must outlive the copies
      }
      k_symmetrize<<<ceil_div(n * n, 256), 256, 0, H.st>>>(n, M.p);
      int lwork = 0;
      GB_CUSOLVER(cusolverDnDsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, (int)n, M.p,
                                             (int)n, W.p, &lwork));
      work.alloc(lwork);
      DevBuf<int> info;
      info.alloc(1);
      GB_CUSOLVER(cusolverDnDsyevd(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, (int)n, M.p, (int)n, W.p,
                                  work.p, lwork, info.p));
      std::vector<double> w = W.download();
      const int inf = info.download()[0];
      GB_CHECK(inf == 0, GB_GMG_CUDA_ERROR, "coarse eigendecomposition failed");
      const double wmax = w.back();
      for (double& v : w) v = v > 1e-10 * wmax ? 1.0 / v : 0.0;
      W.upload(w);
      k_scale_columns<<<ceil_div(n * n, 256), 256, 0, H.st>>>(n, M.p, W.p, U.p);
      H.coarse_pinv[block].alloc((size_t)n * n);
      // pinv = (V diag(s)) V^T
      GB_CUBLAS(cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_T, (int)n, (int)n, (int)n, &one, U.p, (int)n, M.p, (int)n,
                            &zero, H.coarse_pinv[block].p, (int)n));
      GB_CUDA(cudaStreamSynchronize(H.st));
    }
  } catch (...) {
    cusolverDnDestroy(sol);
    cublasDestroy(blas);
    throw;
  }
  cusolverDnDestroy(sol);
  cublasDestroy(blas);
  H.coarse_ready = true;
}

template <typename T>
void build_preconditioner_T(Handle& H) {
  for (int l = 0; l < H.n_levels; ++l) {
    alloc_level_work<T>(H.levels[l], H.st);
    compute_diagonals<T>(H, l);
  }
  for (int l = 0; l < H.n_levels; ++l) {
    estimate_eigenvalues<T>(H, l, 0);
    estimate_eigenvalues<T>(H, l, 1);
  }
  GB_CUDA(cudaStreamSynchronize(H.st));
}

// The FP64 levels of the last build_preconditioner, built on their first use.
void ensure_fp64(Handle& H) {
  if (H.prec_done[0] || !H.fp64_pending) return;
  build_preconditioner_T<double>(H);
  H.prec_done[0] = true;
  H.fp64_pending = false;
}
// ensure_fp64 when `precision` is FP64
void ensure_precision(Handle& H, int precision) {
  if (precision != GB_GMG_FP32) ensure_fp64(H);
}

void to_internal(Handle& H, int lev, const double* d_caller, double* d_internal, bool with_u, bool with_p) {
  Level& L = H.levels[lev];
  if (with_u) v_permute_scatter<double, double>(L.n_u, L.perm_u_d.p, d_caller, d_internal, H.st);
  if (with_p)
    v_permute_scatter<double, double>(L.n_p, L.perm_p_d.p, d_caller + (with_u ? L.n_u : 0),
                                      d_internal + (with_u ? L.n_u : 0), H.st);
}
void to_caller(Handle& H, int lev, const double* d_internal, double* d_caller, bool with_u, bool with_p) {
  Level& L = H.levels[lev];
  if (with_u) v_permute_gather<double, double>(L.n_u, L.perm_u_d.p, d_internal, d_caller, H.st);
  if (with_p)
    v_permute_gather<double, double>(L.n_p, L.perm_p_d.p, d_internal + (with_u ? L.n_u : 0),
                                     d_caller + (with_u ? L.n_u : 0), H.st);
}

void solve_internal(Handle& H, const gb_gmg_solve_params* P, gb_gmg_outputs* out) {
  Level& F = H.top();
  const long nu = F.n_u, n = H.n_top();
  double* x = H.cg_x.p;   // solution (internal)
  double* b = H.bv.p;     // rhs (internal)
  const int prec = P->mg_precision;
  ensure_precision(H, prec);
  GB_CHECK(H.prec_done[prec == GB_GMG_FP32 ? 1 : 0], GB_GMG_NOT_READY, "build_preconditioner has not been called");
  // constrained entries of the initial guess are zero during the solve
  v_zero_indexed<double>((long)F.cons_u.size(), F.cons_u_d.p, x, H.st);
  v_zero_indexed<double>((long)F.cons_p.size(), F.cons_p_d.p, x + nu, H.st);
  H.nA = H.nS = H.n_stokes64 = 0;
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  GB_CUDA(cudaEventRecord(e0, H.st));
  // initial residual and tolerance (:977-1041)
  double* t = H.tv.p;
  double ru, rp;
  if (P->solve_newton_system) {
    // a Newton update: zero initial guess, residual and tolerance from |rhs| (:959-970, :1026-1040)
    GB_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), H.st));
    ru = std::sqrt(dot_host(H, nu, b, b));
    rp = std::sqrt(dot_host(H, n - nu, b + nu, b + nu));
    out->initial_nonlinear_residual = std::sqrt(ru * ru + rp * rp);
  } else {
    stokes64(H, x, t);
    v_copy<double>(n, b, H.rv.p, H.st);
    v_axpby<double>(n, -1.0, t, 1.0, H.rv.p, H.st);
    out->initial_nonlinear_residual = std::sqrt(dot_host(H, n, H.rv.p, H.rv.p));
    v_copy<double>(n, x, H.wv.p, H.st);
    GB_CUDA(cudaMemsetAsync(H.wv.p, 0, nu * sizeof(double), H.st));
    stokes64(H, H.wv.p, t);
    v_copy<double>(nu, b, H.rv.p, H.st);
    v_axpby<double>(nu, -1.0, t, 1.0, H.rv.p, H.st);
    ru = std::sqrt(dot_host(H, nu, H.rv.p, H.rv.p));
    rp = std::sqrt(dot_host(H, n - nu, b + nu, b + nu));
  }
  const double tol = P->absolute_tolerance > 0 ? P->absolute_tolerance
                                               : P->linear_solver_tolerance * std::sqrt(ru * ru + rp * rp);
  out->solver_tolerance = tol;
  bool conv = false;
  double fr = 0;
  out->cheap_iterations = out->expensive_iterations = 0;
  if (P->krylov == GB_GMG_GMRES_IR) {
    // FP64 iterative refinement: r = b - K x in FP64, inner FGMRES with the FP32
    // operator and FP32 V-cycles on K d = r, x += d.
    double* d = H.xv.p;
    double* rr = H.rv.p;
    int outer = 0;
    while (true) {
      stokes64(H, x, t);
      v_copy<double>(n, b, rr, H.st);
      v_axpby<double>(n, -1.0, t, 1.0, rr, H.st);
      fr = std::sqrt(dot_host(H, n, rr, rr));
      GB_CHECK(std::isfinite(fr), GB_GMG_NAN_DETECTED, "NaN or Inf in the Stokes residual");
      if (fr <= tol) { conv = true; break; }
      if (outer >= 50 || out->cheap_iterations >= P->n_cheap_steps) break;
      ++outer;
      GB_CUDA(cudaMemsetAsync(d, 0, n * sizeof(double), H.st));
      bool c2;
      double f2;
      const double inner_tol = std::max(tol, P->ir_inner_tolerance * fr) * 0.5;
      // the inner solve keeps its own copies of b (rr) in bv-sized storage
      v_copy<double>(n, rr, H.cg_r.p, H.st);
      out->cheap_iterations += gmres(H, d, H.cg_r.p, inner_tol, P->n_cheap_steps, P->restart, true, false, prec,
                                     true, P, c2, f2);
      v_axpby<double>(n, 1.0, d, 1.0, x, H.st);
    }
  } else {
    // The cheap phase of the reference is plain GMRES because its preconditioner
    // is a fixed linear operator. A V-cycle in FP32 is not exactly linear any
    // more, so with FP32 levels the cheap phase is flexible GMRES (FGMRES).
    const bool flexible_cheap = prec == GB_GMG_FP32;
    if (P->n_cheap_steps > 0 && P->krylov == GB_GMG_IDR)
      out->cheap_iterations = idr(H, x, b, tol, P->n_cheap_steps, P->idr_s, prec, P, conv, fr);
    else if (P->n_cheap_steps > 0)
      out->cheap_iterations =
          gmres(H, x, b, tol, P->n_cheap_steps, P->restart, flexible_cheap, false, prec, false, P, conv, fr);
    if (!conv && P->n_expensive_steps > 0)
      out->expensive_iterations =
          gmres(H, x, b, tol, P->n_expensive_steps, P->restart, true, true, prec, false, P, conv, fr);
  }
  GB_CUDA(cudaEventRecord(e1, H.st));
  GB_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  out->solve_seconds = ms * 1e-3;
  out->final_linear_residual = fr;
  out->A_preconditioner_applications = H.nA;
  out->S_preconditioner_applications = H.nS;
  out->fp64_stokes_applications = H.n_stokes64;
  out->status = conv ? GB_GMG_OK : GB_GMG_NO_CONVERGENCE;
}

}  // namespace
}  // namespace gb

// =====================================================================================
// C ABI
// =====================================================================================
using gb::Handle;

struct gb_gmg {
  Handle h;
};

#define ABI_TRY(H, ...)                                        \
  try {                                                        \
    __VA_ARGS__;                                               \
    return GB_GMG_OK;                                          \
  } catch (const gb::Error& e) {                               \
    (H)->h.err = e.what();                                     \
    return e.code;                                             \
  } catch (const std::bad_alloc& e) {                          \
    (H)->h.err = "out of host memory";                         \
    return GB_GMG_OUT_OF_MEMORY;                               \
  } catch (const std::exception& e) {                          \
    (H)->h.err = e.what();                                     \
    return GB_GMG_INVALID_ARGUMENT;                            \
  }

extern "C" {

void gb_gmg_default_options(gb_gmg_options* o) {
  o->verbose = 0;
  o->smoother_degree = 4;
  o->smoothing_range = 15.0;
  o->eig_cg_iterations = 10;
  o->coarse_degree = 8;
  o->coarse_range = 1e-3;
  o->coarse_eig_cg_iterations = 100;
  o->schur_smoothing_steps = 4;
  o->force_indexed_layout = 0;
  o->coarse_solver = GB_GMG_COARSE_CHEBYSHEV;
  o->fused_a_min_cells = 0;  // measured slower than the two-pass form (see ablock_fused.cu)
  // 1000: the single-block levels only. Up to kMaxDenseNextNodes adds the lattice
  // level above them (32^3 workload: Schur V-cycle 0.243 -> 0.207 ms, solve
  // 81.7 -> 79.2 ms) at 160 ms more per preconditioner build (batched build) --
  // worth it only when several solves share one build.
  o->dense_mass_cycle_nodes = gb::kMaxDenseBottomNodes;
  o->dense_a_cycle_dofs = gb::kMaxDenseANodes;
  o->fused_small_smoother = 1;
}

void gb_gmg_default_solve_params(gb_gmg_solve_params* p) {
  p->linear_solver_tolerance = 1e-7;
  p->absolute_tolerance = 0.0;
  p->n_cheap_steps = 1000;
  p->n_expensive_steps = 1000;
  p->restart = 100;
  p->tol_A = 1e-2;
  p->tol_S = 1e-6;
  p->mg_precision = GB_GMG_FP64;
  p->krylov = GB_GMG_GMRES;
  p->idr_s = 2;
  p->solve_newton_system = 0;
  p->ir_inner_tolerance = 1e-3;
  p->orthogonalization = GB_GMG_GS_FLOAT_PAIR;
}

int gb_gmg_create(const gb_gmg_options* opt, int dim, int degree_v, int n_levels, gb_gmg** out) {
  if (!out) return GB_GMG_INVALID_ARGUMENT;
  *out = nullptr;
  if ((dim != 2 && dim != 3) || (degree_v != 2 && degree_v != 3) || n_levels < 1) return GB_GMG_INVALID_ARGUMENT;
  gb_gmg* g = new gb_gmg();
  if (opt) g->h.opt = *opt;
  else gb_gmg_default_options(&g->h.opt);
  g->h.dim = dim;
  g->h.degree = degree_v;
  g->h.n_levels = n_levels;
  g->h.levels.resize(n_levels);
  for (auto& L : g->h.levels) {
    L.dim = dim;
    L.degree = degree_v;
  }
  int dev = 0;
  if (cudaStreamCreateWithFlags(&g->h.st, cudaStreamNonBlocking) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&g->h.n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    if (g->h.st) cudaStreamDestroy(g->h.st);
    delete g;
    return GB_GMG_CUDA_ERROR;
  }
  *out = g;
  return GB_GMG_OK;
}

void gb_gmg_destroy(gb_gmg* g) {
  if (!g) return;
  cudaStreamSynchronize(g->h.st);
  g->h.reset_graphs();
  if (g->h.dots_h) cudaFreeHost(g->h.dots_h);
  if (g->h.flag_d) cudaFree(g->h.flag_d);
  cudaStreamDestroy(g->h.st);
  delete g;
}

const char* gb_gmg_last_error(const gb_gmg* g) { return g ? g->h.err.c_str() : "null handle"; }

int gb_gmg_set_level_mesh(gb_gmg* g, int level, int64_t n_cells, const int32_t* cdu, const int32_t* cdp,
                          int geometry_kind, const double* geom, int64_t n_u, int64_t n_p) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(level >= 0 && level < H.n_levels, 1, "level out of range");
    GB_CHECK(n_cells > 0 && n_u > 0 && n_p > 0 && cdu && cdp && geom, 1, "empty mesh or null array");
    GB_CHECK(n_u < (1LL << 31) && n_p < (1LL << 31), 1, "more than 2^31 DoFs per block");
    GB_CHECK(geometry_kind >= 0 && geometry_kind <= 2, 1, "unknown geometry kind");
    gb::Level& L = H.levels[level];
    L.dim = H.dim;
    L.degree = H.degree;
    const int nv = L.nv(), np = L.np(), nq = L.nq(), nm = H.dim == 3 ? 27 : 9;  // nm: Q2 mapping points
    L.n_cells = n_cells;
    L.n_u = n_u;
    L.n_p = n_p;
    L.cdu.assign(cdu, cdu + n_cells * H.dim * nv);
    L.cdp.assign(cdp, cdp + n_cells * np);
    for (int v : L.cdu) GB_CHECK(v >= 0 && v < n_u, 1, "velocity DoF index out of range");
    for (int v : L.cdp) GB_CHECK(v >= 0 && v < n_p, 1, "pressure DoF index out of range");
    L.geom_kind = geometry_kind;
    const size_t ng = geometry_kind == 0   ? (size_t)n_cells * 2 * H.dim
                      : geometry_kind == 1 ? (size_t)n_cells * nm * H.dim
                                           : (size_t)n_cells * nq * (H.dim * H.dim + 1);
    L.geom.assign(geom, geom + ng);
    L.cu.init(n_u);
    L.cp.init(n_p);
    H.setup_done = false;
  })
}

int gb_gmg_set_level_constraints(gb_gmg* g, int level, int block, int64_t n_lines, const int32_t* rows,
                                 const int32_t* ptr, const int32_t* cols, const double* w, const double* inhom) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(level >= 0 && level < H.n_levels && (block == 0 || block == 1), 1, "level/block out of range");
    gb::Level& L = H.levels[level];
    GB_CHECK(L.n_cells > 0, 2, "set the level mesh before its constraints");
    gb::HostCons& C = block == 0 ? L.cu : L.cp;
    const long n = block == 0 ? L.n_u : L.n_p;
    C.init(n);
    for (int64_t i = 0; i < n_lines; ++i) {
      GB_CHECK(rows[i] >= 0 && rows[i] < n, 1, "constraint row out of range");
      GB_CHECK(C.line_of[rows[i]] < 0, 1, "duplicate constraint line");
      C.line_of[rows[i]] = (int)i;
      for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        GB_CHECK(cols[k] >= 0 && cols[k] < n, 1, "constraint entry out of range");
        C.cols.push_back(cols[k]);
        C.w.push_back(w[k]);
      }
      C.ptr.push_back((int)C.cols.size());
      C.inhom.push_back(inhom ? inhom[i] : 0.0);
    }
    H.setup_done = false;
  })
}

int gb_gmg_set_transfer(gb_gmg* g, int level, const int32_t* parent, const uint8_t* child) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(level >= 1 && level < H.n_levels, 1, "transfer level out of range");
    gb::Level& L = H.levels[level];
    GB_CHECK(L.n_cells > 0, 2, "set the level mesh before its transfer");
    L.parent.assign(parent, parent + L.n_cells);
    L.child.assign(child, child + L.n_cells);
    for (unsigned char c : L.child) GB_CHECK(c < (1u << H.dim) || c == gb::kSameCell, 1, "child index out of range");
    L.has_transfer = true;
    H.setup_done = false;
  })
}

int gb_gmg_finalize_setup(gb_gmg* g) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    for (auto& L : H.levels) GB_CHECK(L.n_cells > 0, 2, "a level has no mesh");
    for (auto& L : H.levels) gb::setup_level(L, H.opt.force_indexed_layout != 0);
    for (int l = 1; l < H.n_levels; ++l) {
      gb::setup_transfer(H.levels[l], H.levels[l - 1]);
      if (H.opt.verbose)
        std::fprintf(stderr, "gb_gmg: transfer %d -> %d: velocity %s, pressure %s\n", l - 1, l,
                     H.levels[l].xfer_lattice[0] ? "lattice" : "csr", H.levels[l].xfer_lattice[1] ? "lattice" : "csr");
    }
    gb::setup_coefficient_maps(H.levels);
    for (auto& L : H.levels) {  // ping-pong halves of the fused small-level smoother
      L.f32.xalt.release();
      L.f32.dalt.release();
      L.f32.Ealt.release();
      if (!gb::small_lattice_a_level(L.view<float>(1.0, 0))) continue;
      L.f32.xalt.alloc(L.n_u);
      L.f32.dalt.alloc(L.n_u);
      L.f32.Ealt.alloc((size_t)L.n_cells * 81);
      GB_CUDA(cudaMemsetAsync(L.f32.xalt.p, 0, L.n_u * sizeof(float), H.st));
      GB_CUDA(cudaMemsetAsync(L.f32.dalt.p, 0, L.n_u * sizeof(float), H.st));
      GB_CUDA(cudaMemsetAsync(L.f32.Ealt.p, 0, (size_t)L.n_cells * 81 * sizeof(float), H.st));
    }
    for (auto& L : H.levels) {  // FP32 A-block applications of large lattice levels: fused kernel
      L.fused_tz = 0;
      L.f32.Fa.release();
      const long min_cells = H.opt.fused_a_min_cells > 0 ? H.opt.fused_a_min_cells : -1;
      if (min_cells < 0) continue;
      const gb::LevelView<float> v = L.view<float>(H.s, 0);
      const int tz = gb::fused_a_tile_layers(v, H.n_sm, min_cells);
      if (tz > 0 && gb::fused_a_prepare()) {
        L.f32.Fa.alloc(gb::fused_a_face_floats(v, tz));
        L.fused_tz = tz;
      }
    }
    gb::ensure_workspace(H);
    GB_CUDA(cudaStreamSynchronize(H.st));
    H.reset_graphs();
    H.restart_alloc = -1;  // Krylov and IDR(s) blocks are sized by the finest level: rebuilt on next use
    H.idr_s_alloc = 0;
    for (auto& L : H.levels) {  // raw cell-DoF tables of correct_stokes_rhs follow the new numbering
      L.cdu_raw_d.release();
      L.cdp_raw_d.release();
    }
    H.newton_terms.clear();
    H.free_surface.clear();
    H.setup_done = true;
    H.visc_done = false;
    H.prec_done[0] = H.prec_done[1] = false;
    H.fp64_pending = false;
  })
}

int gb_gmg_set_viscosity(gb_gmg* g, const double* eta, int n_per_cell, int projection, double s, int compressible) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.setup_done, GB_GMG_NOT_READY, "finalize_setup has not been called");
    const int nq = H.top().nq();
    GB_CHECK(n_per_cell == 1 || n_per_cell == nq, 1, "n_per_cell must be 1 or (degree+1)^dim");
    GB_CHECK(s > 0 && std::isfinite(s), 1, "pressure scaling must be positive");
    H.s = s;
    H.compressible = compressible;
    H.projection = projection;
    H.visc_done = false;
    H.mass_dense_top = -1;  // rebuilt by build_preconditioner
    H.a_dense_top = -1;
    GB_CHECK(eta, 1, "null viscosity");
    gb::device_level_viscosity(H.levels, eta, n_per_cell, projection, s, H.eta_min, H.eta_max, H.st);
    H.visc_n_per_cell = n_per_cell;
    H.reset_graphs();
    H.visc_done = true;
    H.prec_done[0] = H.prec_done[1] = false;
    H.fp64_pending = false;
  })
}

int gb_gmg_update_viscosity(gb_gmg* g, const double* eta, int n_per_cell) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.visc_done, GB_GMG_NOT_READY, "set_viscosity has not been called");
    GB_CHECK(eta, 1, "null viscosity");
    // The device tables, the level views built from Level::eta_n and the captured
    // V-cycles all assume the layout of the last set_viscosity: a different one
    // is rejected before anything changes.
    GB_CHECK(n_per_cell == H.visc_n_per_cell, 1, "viscosity layout differs from the last set_viscosity");
    // the kept preconditioner is the one of the old tables in both precisions:
    // FP64 levels left to their first use are built now
    gb::ensure_fp64(H);
    // the values are checked before any table changes; the tables keep their
    // sizes, so device addresses (and captured graphs) stay valid
    double mn, mx;
    gb::device_level_viscosity(H.levels, eta, n_per_cell, H.projection, H.s, mn, mx, H.st);
    H.eta_min = mn;
    H.eta_max = mx;
    // the explicit coarse mass cycle holds the levels' mass matrices (same size:
    // same buffer, so captured V-cycles stay valid)
    if (H.mass_dense_top >= 0) gb::build_mass_dense(H);
    if (H.a_dense_top >= 0) gb::build_a_dense(H);
  })
}

int gb_gmg_set_newton_terms(gb_gmg* g, const gb_gmg_newton_terms* t) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.setup_done, GB_GMG_NOT_READY, "finalize_setup has not been called");
    auto& N = H.newton_terms;
    if (!t || !(t->enable_newton_derivatives || t->enable_prescribed_dilation)) {
      N.clear();
      return GB_GMG_OK;
    }
    GB_CHECK(H.degree == 2, 1, "Newton / dilation terms are built for velocity degree 2");
    const bool newton = t->enable_newton_derivatives != 0, dil = t->enable_prescribed_dilation != 0;
    GB_CHECK(!newton || (t->strain_rate && t->newton_factor_wrt_strain_rate && t->newton_factor_wrt_pressure), 1,
             "Newton derivatives need the strain-rate and both Newton-factor tables");
    GB_CHECK(!dil || t->dilation_lhs, 1, "a prescribed dilation needs its lhs table");
    GB_CHECK(!(newton && dil) || (t->dilation_derivative_wrt_strain_rate && t->dilation_derivative_wrt_pressure), 1,
             "Newton derivatives with a prescribed dilation need both dilation-derivative tables");
    gb::Level& F = H.top();
    const int nq = H.dim == 3 ? 27 : 9, ns = H.dim == 3 ? 6 : 3;
    const double* src[6] = {t->strain_rate, t->newton_factor_wrt_strain_rate, t->newton_factor_wrt_pressure,
                            t->dilation_lhs, t->dilation_derivative_wrt_strain_rate,
                            t->dilation_derivative_wrt_pressure};
    const int width[6] = {ns, ns, 1, 1, ns, 1};
    const bool used[6] = {newton, newton, newton, dil, newton && dil, newton && dil};
    N.clear();
    for (int k = 0; k < 6; ++k) {
      if (!used[k]) continue;
      const size_t per_cell = (size_t)nq * width[k];
      std::vector<double> h((size_t)F.n_cells * per_cell);
      for (long c = 0; c < F.n_cells; ++c) {
        const long ic = F.internal_of_cell[c];
        for (size_t i = 0; i < per_cell; ++i) {
          const double v = src[k][(size_t)c * per_cell + i];
          GB_CHECK(std::isfinite(v), GB_GMG_NAN_DETECTED, "non-finite value in a Newton / dilation table");
          h[(size_t)ic * per_cell + i] = v;
        }
      }
      N.t64[k].upload(h);
      N.t32[k].upload(std::vector<float>(h.begin(), h.end()));
    }
    N.newton = newton;
    N.symmetrize = t->symmetrize_newton_system != 0;
    N.average = t->average_newton_factors != 0;
    N.dilation = dil;
  })
}

int gb_gmg_set_free_surface(gb_gmg* g, int64_t n_faces, const int32_t* face_cell, const int32_t* face_no,
                            const double* stabilization, const double* normal_jxw) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.setup_done, GB_GMG_NOT_READY, "finalize_setup has not been called");
    auto& FS = H.free_surface;
    if (n_faces <= 0 || !face_cell || !face_no || !stabilization) {
      GB_CHECK(n_faces <= 0, 1, "free-surface faces need face_cell, face_no and stabilization");
      FS.clear();
      return GB_GMG_OK;
    }
    GB_CHECK(H.degree == 2, 1, "free-surface faces are built for velocity degree 2");
    gb::Level& F = H.top();
    const int d = F.dim, nv = d == 3 ? 27 : 9, nf = d == 3 ? 9 : 3, ncu = d * nv;
    GB_CHECK(normal_jxw || F.geom_kind != GB_GMG_GEOM_TABLE, 1,
             "a geometry table level needs the caller's normal_jxw for free-surface faces");
    std::vector<long> order(n_faces);
    std::set<long> seen;
    for (long i = 0; i < n_faces; ++i) {
      GB_CHECK(face_cell[i] >= 0 && face_cell[i] < F.n_cells, 1, "free-surface face_cell out of range");
      GB_CHECK(face_no[i] >= 0 && face_no[i] < 2 * d, 1, "free-surface face_no out of range");
      GB_CHECK(seen.insert((long)face_cell[i] * 6 + face_no[i]).second, 1, "free-surface face listed twice");
      order[i] = i;
    }
    std::stable_sort(order.begin(), order.end(), [&](long a, long b) {
      return F.internal_of_cell[face_cell[a]] < F.internal_of_cell[face_cell[b]];
    });
    // constraint-line ids as the level's device tables number them (lines with
    // entries); indexed levels keep the caller's numbering (perm_u is the identity)
    std::vector<int> lid;
    if (!F.structured) {
      lid.assign(F.n_u, -1);
      int next = 0;
      for (long gd = 0; gd < F.n_u; ++gd)
        if (F.cu.constrained((int)gd) && F.cu.n_entries((int)gd) > 0) lid[gd] = next++;
    }
    std::vector<int> gptr{0}, gcell, fno(n_faces), codes((size_t)n_faces * d * nf), raw(codes.size());
    std::vector<double> tab((size_t)n_faces * nf * 2 * d);
    std::vector<double> nj(nf * d);
    for (long j = 0; j < n_faces; ++j) {
      const long i = order[j];
      const long cc = face_cell[i], ic = F.internal_of_cell[cc];
      if (gcell.empty() || gcell.back() != ic) {
        if (!gcell.empty()) gptr.push_back((int)j);
        gcell.push_back((int)ic);
      }
      const int fn = face_no[i], dn = fn >> 1, side = fn & 1;
      const int ta = dn == 0 ? 1 : 0, tb = d == 3 ? (dn == 2 ? 1 : 2) : 0;
      const int st[3] = {1, 3, 9};
      fno[j] = fn;
      for (int c = 0; c < d; ++c)
        for (int k = 0; k < nf; ++k) {
          const int l = 2 * side * st[dn] + (k % 3) * st[ta] + (d == 3 ? (k / 3) * st[tb] : 0);
          const int gd = F.cdu[(size_t)cc * ncu + c * nv + l];
          const int in = F.perm_u.empty() ? gd : F.perm_u[gd];
          int code = in;
          if (F.cu.constrained(gd)) code = F.structured || lid[gd] < 0 ? -1 : -(lid[gd] + 2);
          codes[((size_t)j * d + c) * nf + k] = code;
          raw[((size_t)j * d + c) * nf + k] = in;
        }
      if (normal_jxw) {
        for (int q = 0; q < nf * d; ++q) nj[q] = normal_jxw[(size_t)i * nf * d + q];
      } else {
        const size_t per = F.geom_kind == GB_GMG_GEOM_BOX ? 2 * d : (size_t)nv * d;
        gb::face_normal_jxw(d, F.geom_kind, &F.geom[(size_t)cc * per], fn, nj.data());
      }
      for (int q = 0; q < nf; ++q)
        for (int e = 0; e < d; ++e) {
          const double t = stabilization[((size_t)i * nf + q) * d + e], n = nj[q * d + e];
          GB_CHECK(std::isfinite(t) && std::isfinite(n), GB_GMG_NAN_DETECTED, "non-finite free-surface table entry");
          tab[((size_t)j * nf + q) * 2 * d + e] = t;
          tab[((size_t)j * nf + q) * 2 * d + d + e] = n;
        }
    }
    gptr.push_back((int)n_faces);
    FS.clear();
    FS.gptr.upload(gptr);
    FS.gcell.upload(gcell);
    FS.fno.upload(fno);
    FS.codes.upload(codes);
    FS.raw.upload(raw);
    FS.t64.upload(tab);
    FS.t32.upload(std::vector<float>(tab.begin(), tab.end()));
    FS.n_groups = (int)gcell.size();
    FS.n_faces = n_faces;
  })
}

int gb_gmg_build_preconditioner(gb_gmg* g) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.visc_done, GB_GMG_NOT_READY, "set_viscosity has not been called");
    H.reset_graphs();
    H.prec_done[0] = H.prec_done[1] = false;
    H.fp64_pending = false;
    if (H.opt.coarse_solver == GB_GMG_COARSE_DENSE_FP64) {
      gb::build_preconditioner_T<double>(H);
      gb::build_dense_coarse(H);
      H.prec_done[0] = true;
    } else {
      H.fp64_pending = true;  // gb::ensure_fp64 builds them on first use
    }
    gb::build_preconditioner_T<float>(H);
    H.mass_bottom_top = gb::plan_mass_bottom(H);
    H.prec_done[1] = true;
    gb::build_mass_dense(H);
    gb::build_a_dense(H);
  })
}

// correct_stokes_rhs (stokes_matrix_free_local_smoothing.cc:618-754): rhs -= K u0 with
// plain reads of u0 (read_dof_values_plain: the constrained entries carry the
// inhomogeneities), contributions distributed through the constraints and
// nothing added to constrained rows. The cell pass is the FP64 Stokes cell pass
// over a table of raw internal DoF indices (no constraint codes); the gather is
// the level's own with the "constrained rows are zero" epilogue.
int gb_gmg_correct_stokes_rhs(gb_gmg* g, const double* u0, double* rhs) {
  if (!g || !u0 || !rhs) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.visc_done, GB_GMG_NOT_READY, "set_viscosity has not been called");
    const int top = H.n_levels - 1;
    gb::Level& F = H.levels[top];
    const long nu = F.n_u, n = F.n_u + F.n_p;
    const int nv = F.nv(), npc = F.np(), ncu = F.dim * nv;
    if (!F.cdu_raw_d.p) {
      std::vector<int> ru((size_t)F.n_cells * ncu), rp((size_t)F.n_cells * npc);
      for (long ic = 0; ic < F.n_cells; ++ic) {
        const long cc = F.cell_of_internal.empty() ? ic : F.cell_of_internal[ic];
        for (int k = 0; k < ncu; ++k) {
          const int gdof = F.cdu[(size_t)cc * ncu + k];
          ru[(size_t)ic * ncu + k] = F.perm_u.empty() ? gdof : F.perm_u[gdof];
        }
        for (int k = 0; k < npc; ++k) {
          const int gdof = F.cdp[(size_t)cc * npc + k];
          rp[(size_t)ic * npc + k] = F.perm_p.empty() ? gdof : F.perm_p[gdof];
        }
      }
      F.cdu_raw_d.upload(ru);
      F.cdp_raw_d.upload(rp);
    }
    double* a = H.stage_a.p;
    double* b = H.stage_b.p;
    double* y = H.tv.p;
    GB_CUDA(cudaMemcpyAsync(a, u0, n * sizeof(double), cudaMemcpyHostToDevice, H.st));
    gb::to_internal(H, top, a, b, true, true);
    gb::LevelDev<double>& D = F.f64;
    const gb::LevelView<double> v = F.view_outer<double>(H.s, H.compressible);
    gb::LevelView<double> plain = v;
    plain.structured = 0;
    plain.cdu = F.cdu_raw_d.p;
    plain.cdp = F.cdp_raw_d.p;
    gb::launch_cell_pass<double>(plain, gb::OPK_STOKES, b, b + nu, D.Eu.p, D.Ep.p, H.st);
    ++H.cell_launches;
    if (H.free_surface.on()) {  // the face term of K u0, plain reads (the reference's :709-746)
      gb::launch_free_surface<double>(plain, H.free_surface.view<double>(true), b, D.Eu.p, false, H.st);
      ++H.cell_launches;
    }
    for (int block = 0; block < 2; ++block) {
      gb::GatherArgs<double> ga{};
      ga.E = block == 0 ? D.Eu.p : D.Ep.p;
      ga.x = block == 0 ? b : b + nu;
      ga.y = block == 0 ? y : y + nu;
      gb::gather<double>(H, F, v, block, gb::EPI_BT, ga, gb::OPK_STOKES);
    }
    gb::to_caller(H, top, y, a, true, true);
    std::vector<double> corr(n);
    GB_CUDA(cudaMemcpyAsync(corr.data(), a, n * sizeof(double), cudaMemcpyDeviceToHost, H.st));
    GB_CUDA(cudaStreamSynchronize(H.st));
    for (long i = 0; i < n; ++i) rhs[i] -= corr[i];
  })
}

int gb_gmg_assemble_rhs(gb_gmg* g, const double* force, double* rhs) {
  if (!g || !force || !rhs) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.setup_done, GB_GMG_NOT_READY, "finalize_setup has not been called");
    const int top = H.n_levels - 1;
    gb::Level& F = H.levels[top];
    GB_CHECK(H.degree == 2, 1, "the device body force is built for velocity degree 2");
    const int d = F.dim, nq = d == 3 ? 27 : 9;
    const size_t per_cell = (size_t)nq * d;
    std::vector<double> f((size_t)F.n_cells * per_cell);  // internal cell order
    for (long c = 0; c < F.n_cells; ++c) {
      const long ic = F.internal_of_cell[c];
      for (size_t k = 0; k < per_cell; ++k) {
        GB_CHECK(std::isfinite(force[c * per_cell + k]), GB_GMG_NAN_DETECTED, "non-finite body force");
        f[ic * per_cell + k] = force[c * per_cell + k];
      }
    }
    F.eta_in_d.release();  // the upload buffer of the viscosity pipeline is free between calls
    gb::DevBuf<double> fd;
    fd.upload(f);
    gb::LevelDev<double>& D = F.f64;
    const gb::LevelView<double> v = F.view<double>(H.s, H.compressible);
    gb::launch_body_force(v, fd.p, D.Eu.p, H.st);
    ++H.cell_launches;
    gb::GatherArgs<double> a{};
    a.E = D.Eu.p;
    a.y = H.tv.p;
    gb::gather<double>(H, F, v, 0, gb::EPI_BT, a, gb::OPK_STOKES);  // constrained rows zero
    gb::to_caller(H, top, H.tv.p, H.stage_a.p, true, false);
    GB_CUDA(cudaMemcpyAsync(rhs, H.stage_a.p, F.n_u * sizeof(double), cudaMemcpyDeviceToHost, H.st));
    GB_CUDA(cudaStreamSynchronize(H.st));
    std::fill(rhs + F.n_u, rhs + F.n_u + F.n_p, 0.0);
  })
}

int gb_gmg_vmult(gb_gmg* g, int op, int level, int precision, const double* src, double* dst) {
  if (!g || !src || !dst) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.visc_done, GB_GMG_NOT_READY, "set_viscosity has not been called");
    GB_CHECK(level >= 0 && level < H.n_levels && op >= 0 && op <= 3, 1, "level/op out of range");
    gb::Level& L = H.levels[level];
    const long nin = op == 0 ? L.n_u + L.n_p : (op == 1 ? L.n_u : L.n_p);
    const long nout = op == 0 ? L.n_u + L.n_p : (op == 3 ? L.n_p : L.n_u);
    GB_CUDA(cudaMemcpyAsync(H.stage_a.p, src, nin * sizeof(double), cudaMemcpyHostToDevice, H.st));
    double* a = H.stage_a.p;
    double* b = H.stage_b.p;
    // caller -> internal into b, apply into a, internal -> caller into b
    const bool in_u = op <= 1, in_p = op == 0 || op >= 2;
    const bool out_u = op <= 2, out_p = op == 0 || op == 3;
    if (in_u && in_p) gb::to_internal(H, level, a, b, true, true);
    else if (in_u) gb::to_internal(H, level, a, b, true, false);
    else gb::v_permute_scatter<double, double>(L.n_p, L.perm_p_d.p, a, b, H.st);
    const double* su = in_u ? b : nullptr;
    const double* sp = in_p ? (in_u ? b + L.n_u : b) : nullptr;
    // the Stokes operator of the finest level is the outer one (per-point table
    // without averaging, Newton / dilation terms); all others the multigrid's
    const bool outer = op == gb::OPK_STOKES && level == H.n_levels - 1;
    if (precision == GB_GMG_FP64) {
      double* du = out_u ? a : nullptr;
      double* dp = out_p ? (out_u ? a + L.n_u : a) : nullptr;
      gb::apply_op<double>(H, level, op, su, sp, du, dp, outer);
    } else {
      gb::v_cast<double, float>(nin, b, H.f32_a.p, H.st);
      const float* fu = in_u ? H.f32_a.p : nullptr;
      const float* fp = in_p ? (in_u ? H.f32_a.p + L.n_u : H.f32_a.p) : nullptr;
      float* du = out_u ? H.f32_b.p : nullptr;
      float* dp = out_p ? (out_u ? H.f32_b.p + L.n_u : H.f32_b.p) : nullptr;
      gb::apply_op<float>(H, level, op, fu, fp, du, dp, outer);
      gb::v_cast<float, double>(nout, H.f32_b.p, a, H.st);
    }
    if (out_u && out_p) gb::to_caller(H, level, a, b, true, true);
    else if (out_u) gb::to_caller(H, level, a, b, true, false);
    else gb::v_permute_gather<double, double>(L.n_p, L.perm_p_d.p, a, b, H.st);
    GB_CUDA(cudaMemcpyAsync(dst, b, nout * sizeof(double), cudaMemcpyDeviceToHost, H.st));
    GB_CUDA(cudaStreamSynchronize(H.st));
  })
}

int gb_gmg_vmult_device(gb_gmg* g, int op, int precision, const double* d_src, double* d_dst) {
  if (!g || !d_src || !d_dst) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.visc_done, GB_GMG_NOT_READY, "set_viscosity has not been called");
    GB_CHECK(op == 0, 1, "vmult_device supports the Stokes operator");
    const int top = H.n_levels - 1;
    gb::Level& L = H.levels[top];
    gb::to_internal(H, top, d_src, H.stage_a.p, true, true);
    if (precision == GB_GMG_FP64) {
      gb::apply_op<double>(H, top, 0, H.stage_a.p, H.stage_a.p + L.n_u, H.stage_b.p, H.stage_b.p + L.n_u, true);
    } else {
      gb::stokes32(H, H.stage_a.p, H.stage_b.p);
    }
    gb::to_caller(H, top, H.stage_b.p, d_dst, true, true);
    GB_CUDA(cudaStreamSynchronize(H.st));
  })
}

int gb_gmg_get_diagonal_inverse(gb_gmg* g, int level, int block, int precision, double* out) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(block == 0 || block == 1, 1, "block must be 0 (velocity) or 1 (pressure)");
    GB_CHECK(out, 1, "null output");
    const int pi = precision == GB_GMG_FP32 ? 1 : 0;
    gb::ensure_precision(H, precision);
    GB_CHECK(H.prec_done[pi], GB_GMG_NOT_READY, "build_preconditioner has not been called");
    gb::Level& L = H.levels.at(level);
    const std::vector<int>& perm = block == 0 ? L.perm_u : L.perm_p;
    std::vector<double> v;
    if (pi) {
      auto d = (block == 0 ? L.f32.dinvA : L.f32.dinvM).download();
      v.assign(d.begin(), d.end());
    } else {
      v = (block == 0 ? L.f64.dinvA : L.f64.dinvM).download();
    }
    for (size_t i = 0; i < perm.size(); ++i) out[i] = v[perm[i]];
  })
}

int gb_gmg_get_eigenvalues(gb_gmg* g, int level, int block, int precision, double* mm) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    GB_CHECK(block == 0 || block == 1, 1, "block must be 0 (velocity) or 1 (pressure)");
    GB_CHECK(mm, 1, "null output");
    gb::ensure_precision(g->h, precision);
    gb::Level& L = g->h.levels.at(level);
    const double* e = precision == GB_GMG_FP32 ? (block == 0 ? L.f32.eigA : L.f32.eigM)
                                               : (block == 0 ? L.f64.eigA : L.f64.eigM);
    mm[0] = e[0];
    mm[1] = e[1];
  })
}

int gb_gmg_set_eigenvalues(gb_gmg* g, int level, int block, int precision, const double* mm) {
  if (!g) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    GB_CHECK(block == 0 || block == 1, 1, "block must be 0 (velocity) or 1 (pressure)");
    GB_CHECK(mm, 1, "null interval");
    gb::Level& L = g->h.levels.at(level);
    double* e;
    bool* given;
    if (precision == GB_GMG_FP32) {
      e = block == 0 ? L.f32.eigA : L.f32.eigM;
      given = &L.f32.eig_given[block];
    } else {
      e = block == 0 ? L.f64.eigA : L.f64.eigM;
      given = &L.f64.eig_given[block];
    }
    e[0] = mm[0];
    e[1] = mm[1];
    *given = true;
    g->h.reset_graphs();
    // the explicit coarse mass cycle holds these coefficients
    if (precision == GB_GMG_FP32 && block == 1 && level <= g->h.mass_dense_top) gb::build_mass_dense(g->h);
    if (precision == GB_GMG_FP32 && block == 0 && level <= g->h.a_dense_top) gb::build_a_dense(g->h);
  })
}

int gb_gmg_transfer(gb_gmg* g, int fine_level, int block, int precision, int restrict_, const double* src,
                    double* dst) {
  if (!g || !src || !dst) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.setup_done && fine_level >= 1 && fine_level < H.n_levels, 1, "bad transfer level");
    GB_CHECK(block == 0 || block == 1, 1, "block must be 0 (velocity) or 1 (pressure)");
    gb::Level& F = H.levels[fine_level];
    gb::Level& C = H.levels[fine_level - 1];
    const long nf = block == 0 ? F.n_u : F.n_p, nc = block == 0 ? C.n_u : C.n_p;
    const long nin = restrict_ ? nf : nc, nout = restrict_ ? nc : nf;
    const gb::Level& Lin = restrict_ ? F : C;
    const gb::Level& Lout = restrict_ ? C : F;
    const int* pin = block == 0 ? Lin.perm_u_d.p : Lin.perm_p_d.p;
    const int* pout = block == 0 ? Lout.perm_u_d.p : Lout.perm_p_d.p;
    GB_CUDA(cudaMemcpyAsync(H.stage_a.p, src, nin * sizeof(double), cudaMemcpyHostToDevice, H.st));
    gb::v_permute_scatter<double, double>(nin, pin, H.stage_a.p, H.stage_b.p, H.st);
    GB_CUDA(cudaMemsetAsync(H.stage_a.p, 0, nout * sizeof(double), H.st));
    auto run = [&](auto tag) {
      using T = decltype(tag);
      gb::LevelDev<T>& D = F.dev<T>();
      const T* x;
      T* y;
      if constexpr (std::is_same<T, double>::value) {
        x = H.stage_b.p;
        y = H.stage_a.p;
      } else {
        gb::v_cast<double, float>(nin, H.stage_b.p, H.f32_a.p, H.st);
        GB_CUDA(cudaMemsetAsync(H.f32_b.p, 0, nout * sizeof(float), H.st));
        x = H.f32_a.p;
        y = H.f32_b.p;
      }
      if (restrict_) {
        if (F.xfer_lattice[block]) gb::lattice_restrict<T>(F.xfer[block], x, y, H.st);
        else if (block == 0) gb::v_spmv_add<T>(F.PuT_rows, F.PuT_ptr.p, F.PuT_col.p, D.PuT_val.p, x, y, H.st);
        else gb::v_spmv_add<T>(F.PpT_rows, F.PpT_ptr.p, F.PpT_col.p, D.PpT_val.p, x, y, H.st);
      } else {
        if (F.xfer_lattice[block]) gb::lattice_prolong_add<T>(F.xfer[block], x, y, H.st);
        else if (block == 0) gb::v_spmv_add<T>(F.Pu_rows, F.Pu_ptr.p, F.Pu_col.p, D.Pu_val.p, x, y, H.st);
        else gb::v_spmv_add<T>(F.Pp_rows, F.Pp_ptr.p, F.Pp_col.p, D.Pp_val.p, x, y, H.st);
      }
      if constexpr (!std::is_same<T, double>::value) gb::v_cast<float, double>(nout, H.f32_b.p, H.stage_a.p, H.st);
    };
    if (precision == GB_GMG_FP32) run(float()); else run(double());
    gb::v_permute_gather<double, double>(nout, pout, H.stage_a.p, H.stage_b.p, H.st);
    GB_CUDA(cudaMemcpyAsync(dst, H.stage_b.p, nout * sizeof(double), cudaMemcpyDeviceToHost, H.st));
    GB_CUDA(cudaStreamSynchronize(H.st));
  })
}

int gb_gmg_vcycle(gb_gmg* g, int block, int precision, const double* src, double* dst) {
  if (!g || !src || !dst) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(block == 0 || block == 1, 1, "block must be 0 (velocity) or 1 (pressure)");
    gb::ensure_precision(H, precision);
    GB_CHECK(H.prec_done[precision == GB_GMG_FP32 ? 1 : 0], GB_GMG_NOT_READY, "build_preconditioner missing");
    const int top = H.n_levels - 1;
    gb::Level& F = H.levels[top];
    const long n = block == 0 ? F.n_u : F.n_p;
    const int* perm = block == 0 ? F.perm_u_d.p : F.perm_p_d.p;
    GB_CUDA(cudaMemcpyAsync(H.stage_a.p, src, n * sizeof(double), cudaMemcpyHostToDevice, H.st));
    gb::v_permute_scatter<double, double>(n, perm, H.stage_a.p, H.stage_b.p, H.st);
    gb::vcycle(H, block, precision, H.stage_b.p, H.stage_a.p);
    gb::v_permute_gather<double, double>(n, perm, H.stage_a.p, H.stage_b.p, H.st);
    GB_CUDA(cudaMemcpyAsync(dst, H.stage_b.p, n * sizeof(double), cudaMemcpyDeviceToHost, H.st));
    GB_CUDA(cudaStreamSynchronize(H.st));
  })
}

int gb_gmg_block_preconditioner(gb_gmg* g, int precision, const double* src, double* dst) {
  if (!g || !src || !dst) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    gb::ensure_precision(H, precision);
    GB_CHECK(H.prec_done[precision == GB_GMG_FP32 ? 1 : 0], GB_GMG_NOT_READY, "build_preconditioner missing");
    const int top = H.n_levels - 1;
    const long n = H.n_top();
    GB_CUDA(cudaMemcpyAsync(H.stage_a.p, src, n * sizeof(double), cudaMemcpyHostToDevice, H.st));
    gb::to_internal(H, top, H.stage_a.p, H.stage_b.p, true, true);
    gb_gmg_solve_params P;
    gb_gmg_default_solve_params(&P);
    gb::block_preconditioner(H, precision, false, &P, H.stage_b.p, H.stage_a.p);
    gb::to_caller(H, top, H.stage_a.p, H.stage_b.p, true, true);
    GB_CUDA(cudaMemcpyAsync(dst, H.stage_b.p, n * sizeof(double), cudaMemcpyDeviceToHost, H.st));
    GB_CUDA(cudaStreamSynchronize(H.st));
  })
}

int gb_gmg_solve_device(gb_gmg* g, const double* d_rhs, double* d_sol, const gb_gmg_solve_params* prm,
                        gb_gmg_outputs* out) {
  if (!g || !d_rhs || !d_sol || !out) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    // before the permutation kernels below read the level tables
    GB_CHECK(H.prec_done[0] || H.prec_done[1], GB_GMG_NOT_READY, "build_preconditioner has not been called");
    gb_gmg_solve_params P;
    if (prm) P = *prm; else gb_gmg_default_solve_params(&P);
    GB_CHECK(P.restart >= 1, 1, "restart must be >= 1");
    GB_CHECK(P.orthogonalization == GB_GMG_GS_FLOAT_PAIR || P.orthogonalization == GB_GMG_GS_FP64, 1,
             "orthogonalization must be GB_GMG_GS_FLOAT_PAIR or GB_GMG_GS_FP64");
    const int top = H.n_levels - 1;
    gb::to_internal(H, top, d_rhs, H.bv.p, true, true);
    gb::to_internal(H, top, d_sol, H.cg_x.p, true, true);
    *out = gb_gmg_outputs{};
    gb::solve_internal(H, &P, out);
    gb::to_caller(H, top, H.cg_x.p, d_sol, true, true);
    GB_CUDA(cudaStreamSynchronize(H.st));
    if (out->status != GB_GMG_OK) {
      H.err = "the iterative Stokes solver did not converge";
      return out->status;
    }
  })
}

int gb_gmg_solve(gb_gmg* g, const double* rhs, double* sol, const gb_gmg_solve_params* prm, gb_gmg_outputs* out) {
  if (!g || !rhs || !sol || !out) return GB_GMG_INVALID_ARGUMENT;
  Handle& H = g->h;
  const long n = H.setup_done ? H.n_top() : 0;
  if (!n) { H.err = "finalize_setup has not been called"; return GB_GMG_NOT_READY; }
  int rc;
  try {
    GB_CUDA(cudaMemcpyAsync(H.stage_a.p, rhs, n * sizeof(double), cudaMemcpyHostToDevice, H.st));
    GB_CUDA(cudaMemcpyAsync(H.stage_b.p, sol, n * sizeof(double), cudaMemcpyHostToDevice, H.st));
  } catch (const gb::Error& e) { H.err = e.what(); return e.code; }
  rc = gb_gmg_solve_device(g, H.stage_a.p, H.stage_b.p, prm, out);
  if (rc == GB_GMG_OK || rc == GB_GMG_NO_CONVERGENCE) {
    if (cudaMemcpyAsync(sol, H.stage_b.p, n * sizeof(double), cudaMemcpyDeviceToHost, H.st) != cudaSuccess ||
        cudaStreamSynchronize(H.st) != cudaSuccess) {
      H.err = "CUDA error copying the solution";
      return GB_GMG_CUDA_ERROR;
    }
  }
  return rc;
}

int gb_gmg_adjoint_gradient(gb_gmg* g, const double* u, const double* lambda, double* grad) {
  if (!g || !u || !lambda || !grad) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    GB_CHECK(H.visc_done, GB_GMG_NOT_READY, "set_viscosity has not been called");
    GB_CHECK(H.degree == 2, 1, "the adjoint gradient is built for velocity degree 2");
    const int top = H.n_levels - 1;
    gb::Level& F = H.levels[top];
    GB_CUDA(cudaMemcpyAsync(H.stage_a.p, u, F.n_u * sizeof(double), cudaMemcpyHostToDevice, H.st));
    gb::to_internal(H, top, H.stage_a.p, H.stage_b.p, true, false);
    GB_CUDA(cudaMemcpyAsync(H.stage_a.p, lambda, F.n_u * sizeof(double), cudaMemcpyHostToDevice, H.st));
    gb::to_internal(H, top, H.stage_a.p, H.wv.p, true, false);
    double* gcell = H.tv.p;  // n_cells <= n_u
    GB_CUDA(cudaMemsetAsync(gcell, 0, F.n_cells * sizeof(double), H.st));
    const gb::LevelView<double> v = F.view_outer<double>(H.s, H.compressible);
    for (int k = 0; k < F.n_colours; ++k) {
      const int cnt = F.colour_count[k];
      if (!cnt) continue;
      gb::launch_adjoint_gradient_impl(v, k, F.structured ? 0 : F.colour_begin[k], cnt, H.stage_b.p, H.wv.p, gcell,
                                       H.st);
      ++H.cell_launches;
    }
    std::vector<double> gi(F.n_cells);
    GB_CUDA(cudaMemcpyAsync(gi.data(), gcell, F.n_cells * sizeof(double), cudaMemcpyDeviceToHost, H.st));
    GB_CUDA(cudaStreamSynchronize(H.st));
    for (long c = 0; c < F.n_cells; ++c) grad[c] = gi[F.internal_of_cell[c]];
  })
}

int gb_gmg_time_operation(gb_gmg* g, int what, int precision, int repeats, double* seconds) {
  if (!g || !seconds || repeats < 1) return GB_GMG_INVALID_ARGUMENT;
  ABI_TRY(g, {
    Handle& H = g->h;
    const int pi = precision == GB_GMG_FP32 ? 1 : 0;
    GB_CHECK(what >= 0 && what <= 7, 1, "unknown operation");
    if (what >= 3 && what <= 5) {
      gb::ensure_precision(H, precision);
      GB_CHECK(H.prec_done[pi], GB_GMG_NOT_READY, "build_preconditioner has not been called");
    }
    else GB_CHECK(H.visc_done, GB_GMG_NOT_READY, "set_viscosity has not been called");
    const int top = H.n_levels - 1;
    gb::Level& F = H.levels[top];
    const long n = H.n_top(), nu = F.n_u;
    // deterministic source data
    std::vector<double> src(n);
    for (long i = 0; i < n; ++i) src[i] = (double)(i % 11) - 5.0;
    GB_CUDA(cudaMemcpyAsync(H.stage_a.p, src.data(), n * sizeof(double), cudaMemcpyHostToDevice, H.st));
    gb::v_cast<double, float>(n, H.stage_a.p, H.f32_a.p, H.st);
    auto call = [&]() {
      double* a = H.stage_a.p;
      double* b = H.stage_b.p;
      switch (what) {
        case 0:
          if (pi) gb::apply_op<float>(H, top, 0, H.f32_a.p, H.f32_a.p + nu, H.f32_b.p, H.f32_b.p + nu);
          else gb::apply_op<double>(H, top, 0, a, a + nu, b, b + nu);
          break;
        case 1:
          if (pi) gb::apply_op<float>(H, top, 1, H.f32_a.p, nullptr, H.f32_b.p, nullptr);
          else gb::apply_op<double>(H, top, 1, a, nullptr, b, nullptr);
          break;
        case 2:
          if (pi) gb::apply_op<float>(H, top, 3, nullptr, H.f32_a.p, nullptr, H.f32_b.p);
          else gb::apply_op<double>(H, top, 3, nullptr, a, nullptr, b);
          break;
        case 3: {
          gb_gmg_solve_params P;
          gb_gmg_default_solve_params(&P);
          gb::block_preconditioner(H, precision, false, &P, a, b);
          break;
        }
        case 4: gb::vcycle(H, 0, precision, a, b); break;
        case 5: gb::vcycle(H, 1, precision, a + nu, b + nu); break;
        case 6: {
          if (pi) {
            gb::LevelDev<float>& D = F.f32;
            gb::launch_cell_pass<float>(F.view<float>(H.s, H.compressible), gb::OPK_A, H.f32_a.p, nullptr, D.Eu.p,
                                        D.Ep.p, H.st);
          } else {
            gb::LevelDev<double>& D = F.f64;
            gb::launch_cell_pass<double>(F.view<double>(H.s, H.compressible), gb::OPK_A, a, nullptr, D.Eu.p, D.Ep.p,
                                         H.st);
          }
          break;
        }
        case 7: {
          if (pi) {
            gb::LevelDev<float>& D = F.f32;
            gb::launch_cell_pass<float>(F.view<float>(H.s, H.compressible), gb::OPK_STOKES, H.f32_a.p,
                                        H.f32_a.p + nu, D.Eu.p, D.Ep.p, H.st);
          } else {
            gb::LevelDev<double>& D = F.f64;
            gb::launch_cell_pass<double>(F.view<double>(H.s, H.compressible), gb::OPK_STOKES, a, a + nu, D.Eu.p,
                                         D.Ep.p, H.st);
          }
          break;
        }
      }
    };
    call();
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    GB_CUDA(cudaEventRecord(e0, H.st));
    for (int r = 0; r < repeats; ++r) call();
    GB_CUDA(cudaEventRecord(e1, H.st));
    GB_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *seconds = ms * 1e-3 / repeats;
  })
}

int gb_gmg_memory_consumption(const gb_gmg* g, size_t* bytes) {
  if (!g || !bytes) return GB_GMG_INVALID_ARGUMENT;
  const Handle& H = g->h;
  size_t b = 0;
  for (const auto& L : H.levels) b += L.device_bytes();
  for (const gb::DevBuf<double>* x : {&H.stage_a, &H.stage_b, &H.partial, &H.dots_d, &H.V, &H.Z, &H.wv, &H.xv,
                                      &H.rv, &H.bv, &H.tv, &H.t2v, &H.coef_d, &H.cg_r, &H.cg_z, &H.cg_p, &H.cg_q,
                                      &H.cg_x})
    b += x->bytes();
  b += H.f32_a.bytes() + H.f32_b.bytes() + H.Vs.bytes();
  *bytes = b;
  return GB_GMG_OK;
}

int64_t gb_gmg_kernel_launches(const gb_gmg* g) {
  if (!g) return 0;
  return g->h.cell_launches + gb::VecCounter::launches();
}

}  // extern "C"
