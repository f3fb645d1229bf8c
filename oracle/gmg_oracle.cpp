// CPU oracle for the matrix-free GMG Stokes path (Q2-Q1 Taylor-Hood).
//
// TEST INFRASTRUCTURE ONLY. This file is a plain CPU restatement of the
// reference algorithm; the product (the CUDA library) never links, loads or
// calls it. Only the tests, the smoke check and the CPU-baseline leg of the
// benchmark use it, as the checker.
//
// Parity pins: the end-to-end solve is pinned against the reference's SolCx
// regression outputs (tests/sol_cx_2_gmg/screen-output,
// tests/sol_cx_4_gmg/screen-output: iteration counts and analytic error
// norms). Operator-level results have no reference fixture (the reference
// tests no single vmult); there the oracle is checked against brute-force
// element matrices assembled in numpy.
//
// The arithmetic is written from the mathematics with plain quadrature loops
// (no sum factorisation), so it is independent of the GPU kernels:
//   * cell physics follows source/simulator/solver/matrix_free_operators.cc
//     (Stokes :448-542, B^T :668-701, pressure mass :787-845, A block
//     :974-1009, diagonals :861-908 and :1068-1098);
//   * constrained rows act as the identity, constrained columns are resolved
//     through the constraint lines, as deal.II's MatrixFreeOperators::Base
//     vmult does (zero constrained src entries, apply, dst = src there);
//   * level viscosity follows stokes_matrix_free_local_smoothing.cc:174-294;
//   * smoother / V-cycle / coarse solve follow
//     stokes_matrix_free_local_smoothing.cc:774-916 (Chebyshev degree 4 and
//     range 15 on levels > 0, degree 8 and range 1e-3 on level 0, 4 Schur
//     smoothing steps, coarse = one smoother application);
//   * block preconditioner follows
//     include/aspect/simulator/solver/block_stokes_preconditioner.h:101-352;
//   * the solve (tolerance rule, cheap GMRES with restart+2 vectors, FGMRES
//     fallback) follows stokes_matrix_free_local_smoothing.cc:952-1397.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

enum Op { OP_STOKES = 0, OP_A = 1, OP_BT = 2, OP_MASS = 3 };

// ---------------------------------------------------------------- FE tables
static void lagrange1d(const double* nodes, int n, double x, double* val, double* der) {
  for (int i = 0; i < n; ++i) {
    double v = 1.0, d = 0.0, den = 1.0;
    for (int m = 0; m < n; ++m) {
      if (m == i) continue;
      den *= nodes[i] - nodes[m];
    }
    for (int m = 0; m < n; ++m) {
      if (m == i) continue;
      double t = 1.0;
      for (int k = 0; k < n; ++k)
        if (k != i && k != m) t *= x - nodes[k];
      d += t;
      v *= x - nodes[m];
    }
    val[i] = v / den;
    der[i] = d / den;
  }
}

struct FE {
  int dim = 3, degree = 2, n1 = 3, nv = 27, np = 8, nq = 27, nu = 81, nm = 27;
  double vnodes[4], pnodes[3];           // 1D velocity (FE_Q(degree), Gauss-Lobatto) / pressure nodes
  std::vector<double> qpts, qw;          // QGauss(degree+1): [nq][dim], [nq]
  std::vector<double> vval, vgrad;       // velocity basis: [nq][nv], [nq][nv][dim]
  std::vector<double> pval;              // pressure basis (FE_Q(degree-1)): [nq][np]
  std::vector<double> q1val;             // Q1 basis (viscosity projection): [nq][2^dim]
  std::vector<double> mgrad;             // Q2 mapping basis gradients: [nq][nm][dim]
  void init(int d, int deg = 2) {
    dim = d;
    degree = deg;
    n1 = deg + 1;
    const int pn = deg;  // pressure nodes per direction
    nv = d == 3 ? n1 * n1 * n1 : n1 * n1;
    np = d == 3 ? pn * pn * pn : pn * pn;
    nq = nv;
    nu = d * nv;
    nm = d == 3 ? 27 : 9;
    double g[4], gw[4];
    if (deg == 2) {
      const double g3[3] = {0.5 - 0.5 * std::sqrt(0.6), 0.5, 0.5 + 0.5 * std::sqrt(0.6)};
      const double w3[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};
      for (int i = 0; i < 3; ++i) { g[i] = g3[i]; gw[i] = w3[i]; }
      vnodes[0] = 0.0; vnodes[1] = 0.5; vnodes[2] = 1.0;
      pnodes[0] = 0.0; pnodes[1] = 1.0;
    } else {
      // QGauss(4): (1 -+ sqrt(3/7 +- 2/7 sqrt(6/5))) / 2, weights (18 -+ sqrt 30) / 72;
      // FE_Q(3) nodes: Gauss-Lobatto 0, (1 -+ 1/sqrt 5) / 2, 1
      const double t1 = std::sqrt(3.0 / 7 - 2.0 / 7 * std::sqrt(1.2)), t2 = std::sqrt(3.0 / 7 + 2.0 / 7 * std::sqrt(1.2));
      g[0] = 0.5 - 0.5 * t2; g[1] = 0.5 - 0.5 * t1; g[2] = 0.5 + 0.5 * t1; g[3] = 0.5 + 0.5 * t2;
      gw[0] = gw[3] = (18.0 - std::sqrt(30.0)) / 72;
      gw[1] = gw[2] = (18.0 + std::sqrt(30.0)) / 72;
      vnodes[0] = 0.0; vnodes[1] = 0.5 - 0.5 / std::sqrt(5.0); vnodes[2] = 0.5 + 0.5 / std::sqrt(5.0); vnodes[3] = 1.0;
      pnodes[0] = 0.0; pnodes[1] = 0.5; pnodes[2] = 1.0;
    }
    const double q2n[3] = {0.0, 0.5, 1.0}, q1n[2] = {0.0, 1.0};
    const int nc1 = d == 3 ? 8 : 4;
    qpts.assign(nq * dim, 0.0);
    qw.assign(nq, 1.0);
    vval.assign(nq * nv, 1.0);
    vgrad.assign(nq * nv * dim, 1.0);
    pval.assign(nq * np, 1.0);
    q1val.assign(nq * nc1, 1.0);
    mgrad.assign(nq * nm * dim, 1.0);
    for (int q = 0; q < nq; ++q) {
      int qi[3] = {q % n1, (q / n1) % n1, q / (n1 * n1)};
      double vv[3][4], dv[3][4], vp[3][3], dp_[3][3], v1[3][2], d1[3][2], vm[3][3], dm[3][3];
      for (int e = 0; e < dim; ++e) {
        qpts[q * dim + e] = g[qi[e]];
        qw[q] *= gw[qi[e]];
        lagrange1d(vnodes, n1, g[qi[e]], vv[e], dv[e]);
        lagrange1d(pnodes, pn, g[qi[e]], vp[e], dp_[e]);
        lagrange1d(q1n, 2, g[qi[e]], v1[e], d1[e]);
        lagrange1d(q2n, 3, g[qi[e]], vm[e], dm[e]);
      }
      for (int n = 0; n < nv; ++n) {
        int ni[3] = {n % n1, (n / n1) % n1, n / (n1 * n1)};
        double v = 1.0;
        for (int e = 0; e < dim; ++e) v *= vv[e][ni[e]];
        vval[q * nv + n] = v;
        for (int gdir = 0; gdir < dim; ++gdir) {
          double t = 1.0;
          for (int e = 0; e < dim; ++e) t *= (e == gdir ? dv[e][ni[e]] : vv[e][ni[e]]);
          vgrad[(q * nv + n) * dim + gdir] = t;
        }
      }
      for (int n = 0; n < nm; ++n) {
        int ni[3] = {n % 3, (n / 3) % 3, n / 9};
        for (int gdir = 0; gdir < dim; ++gdir) {
          double t = 1.0;
          for (int e = 0; e < dim; ++e) t *= (e == gdir ? dm[e][ni[e]] : vm[e][ni[e]]);
          mgrad[(q * nm + n) * dim + gdir] = t;
        }
      }
      for (int n = 0; n < np; ++n) {
        int ni[3] = {n % pn, (n / pn) % pn, n / (pn * pn)};
        double v = 1.0;
        for (int e = 0; e < dim; ++e) v *= vp[e][ni[e]];
        pval[q * np + n] = v;
      }
      for (int n = 0; n < nc1; ++n) {
        int ni[3] = {n % 2, (n / 2) % 2, n / 4};
        double v = 1.0;
        for (int e = 0; e < dim; ++e) v *= v1[e][ni[e]];
        q1val[q * nc1 + n] = v;
      }
    }
  }
  // basis values of the velocity (block 0) or pressure (block 1) element at a
  // reference point
  void basis_at(int block, const double* xi, double* out) const {
    const int n = block == 0 ? n1 : degree;
    const double* nodes = block == 0 ? vnodes : pnodes;
    double v[3][4], dd[3][4];
    for (int e = 0; e < dim; ++e) lagrange1d(nodes, n, xi[e], v[e], dd[e]);
    const int cnt = dim == 3 ? n * n * n : n * n;
    for (int m = 0; m < cnt; ++m) {
      const int mi[3] = {m % n, (m / n) % n, m / (n * n)};
      double t = 1.0;
      for (int e = 0; e < dim; ++e) t *= v[e][mi[e]];
      out[m] = t;
    }
  }
};
// Value of the Q2 / Q1 basis at a reference point (for transfer matrices).
static void q2_basis_at(int dim, const double* xi, double* out) {
  const double nodes[3] = {0.0, 0.5, 1.0};
  double v[3][3], d[3][3];
  for (int e = 0; e < dim; ++e) lagrange1d(nodes, 3, xi[e], v[e], d[e]);
  int nv = dim == 3 ? 27 : 9;
  for (int n = 0; n < nv; ++n) {
    int ni[3] = {n % 3, (n / 3) % 3, n / 9};
    double t = 1.0;
    for (int e = 0; e < dim; ++e) t *= v[e][ni[e]];
    out[n] = t;
  }
}
static void q1_basis_at(int dim, const double* xi, double* out) {
  int np = dim == 3 ? 8 : 4;
  for (int n = 0; n < np; ++n) {
    int ni[3] = {n % 2, (n / 2) % 2, n / 4};
    double t = 1.0;
    for (int e = 0; e < dim; ++e) t *= ni[e] ? xi[e] : 1.0 - xi[e];
    out[n] = t;
  }
}

// ---------------------------------------------------------------- constraints
struct Constraints {
  std::vector<int> line_of;  // per dof: -1 unconstrained, else line index
  std::vector<int> ptr, cols;
  std::vector<double> w, inhom;
  void init(int n) { line_of.assign(n, -1); ptr.assign(1, 0); cols.clear(); w.clear(); inhom.clear(); }
  void set(int n, int n_lines, const int* rows, const int* p, const int* c, const double* ww, const double* b) {
    init(n);
    for (int i = 0; i < n_lines; ++i) {
      line_of[rows[i]] = i;
      for (int k = p[i]; k < p[i + 1]; ++k) { cols.push_back(c[k]); w.push_back(ww[k]); }
      ptr.push_back((int)cols.size());
      inhom.push_back(b ? b[i] : 0.0);
    }
  }
  bool constrained(int g) const { return line_of[g] >= 0; }
};

// Local-to-global expansion of one cell-local DoF.
struct Expansion { int n; int g[16]; double w[16]; };

static inline Expansion expand(const Constraints& c, int g) {
  Expansion e;
  int l = c.line_of[g];
  if (l < 0) { e.n = 1; e.g[0] = g; e.w[0] = 1.0; return e; }
  e.n = c.ptr[l + 1] - c.ptr[l];
  if (e.n > 16) throw std::runtime_error("constraint line with more than 16 entries");
  for (int k = 0; k < e.n; ++k) { e.g[k] = c.cols[c.ptr[l] + k]; e.w[k] = c.w[c.ptr[l] + k]; }
  return e;
}

// ---------------------------------------------------------------- level
struct Level {
  int dim = 3, n_cells = 0, n_u = 0, n_p = 0;
  std::vector<int> cdu, cdp;             // [n_cells][nu], [n_cells][np]
  int geom_kind = 0;
  std::vector<double> geom;
  Constraints cu, cp;
  std::vector<double> invJ, JxW;         // [n_cells][nq][dim][dim] (dxi/dx), [n_cells][nq]
  std::vector<int> parent;               // into level-1
  std::vector<unsigned char> child;
  std::vector<double> eta;               // [n_cells][eta_n]
  int eta_n = 1;
  std::vector<int> colour_ptr, colour_cells;  // cells grouped by colour
  // transfers from the coarser level (CSR rows = this level's dofs)
  std::vector<int> Pu_ptr, Pu_col, Pp_ptr, Pp_col;
  std::vector<double> Pu_val, Pp_val;
  // their transposes, built on first use in fast mode
  std::vector<int> PuT_ptr, PuT_col, PpT_ptr, PpT_col;
  std::vector<double> PuT_val, PpT_val;
  bool PT_built = false;
  // smoother data
  std::vector<double> diagA_inv, diagM_inv;
  double eigA[2] = {0, 0}, eigM[2] = {0, 0};  // (min, max) estimates
  bool eig_set = false;
};

static void compute_geometry(Level& L, const FE& fe) {
  const int d = L.dim, nq = fe.nq;
  L.invJ.assign((size_t)L.n_cells * nq * d * d, 0.0);
  L.JxW.assign((size_t)L.n_cells * nq, 0.0);
  for (int c = 0; c < L.n_cells; ++c) {
    for (int q = 0; q < nq; ++q) {
      if (L.geom_kind == 2) {  // caller's table: inverse Jacobian, then |det J|
        const double* t = &L.geom[((size_t)c * nq + q) * (d * d + 1)];
        for (int a = 0; a < d * d; ++a) L.invJ[((size_t)c * nq + q) * d * d + a] = t[a];
        L.JxW[(size_t)c * nq + q] = t[d * d] * fe.qw[q];
        continue;
      }
      double J[3][3] = {{0}};
      if (L.geom_kind == 0) {
        for (int e = 0; e < d; ++e) J[e][e] = L.geom[(size_t)c * 2 * d + d + e];
      } else {
        const double* X = &L.geom[(size_t)c * fe.nm * d];  // Q2 mapping support points
        for (int n = 0; n < fe.nm; ++n)
          for (int a = 0; a < d; ++a)
            for (int b = 0; b < d; ++b) J[a][b] += X[n * d + a] * fe.mgrad[(q * fe.nm + n) * d + b];
      }
      double det, inv[3][3];
      if (d == 2) {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        inv[0][0] = J[1][1] / det; inv[0][1] = -J[0][1] / det;
        inv[1][0] = -J[1][0] / det; inv[1][1] = J[0][0] / det;
      } else {
        det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
              J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
              J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
      }
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) L.invJ[(((size_t)c * nq + q) * d + a) * d + b] = inv[a][b];
      L.JxW[(size_t)c * nq + q] = std::fabs(det) * fe.qw[q];
    }
  }
}

// Greedy colouring: cells of one colour write disjoint global DoFs.
static void colour_cells(Level& L, const FE& fe) {
  std::vector<std::vector<int>> writes(L.n_cells);
  for (int c = 0; c < L.n_cells; ++c) {
    std::set<int> s;
    for (int i = 0; i < fe.nu; ++i) {
      Expansion e = expand(L.cu, L.cdu[(size_t)c * fe.nu + i]);
      for (int k = 0; k < e.n; ++k) s.insert(e.g[k]);
    }
    for (int i = 0; i < fe.np; ++i) {
      Expansion e = expand(L.cp, L.cdp[(size_t)c * fe.np + i]);
      for (int k = 0; k < e.n; ++k) s.insert(L.n_u + e.g[k]);
    }
    writes[c].assign(s.begin(), s.end());
  }
  std::vector<std::vector<int>> cells_of(L.n_u + L.n_p);
  for (int c = 0; c < L.n_cells; ++c)
    for (int g : writes[c]) cells_of[g].push_back(c);
  std::vector<int> col(L.n_cells, -1);
  int n_col = 0;
  for (int c = 0; c < L.n_cells; ++c) {
    std::vector<char> used(n_col + 1, 0);
    for (int g : writes[c])
      for (int o : cells_of[g])
        if (col[o] >= 0) used[col[o]] = 1;
    int k = 0;
    while (used[k]) ++k;
    col[c] = k;
    n_col = std::max(n_col, k + 1);
  }
  L.colour_ptr.assign(n_col + 1, 0);
  for (int c = 0; c < L.n_cells; ++c) L.colour_ptr[col[c] + 1]++;
  for (int k = 0; k < n_col; ++k) L.colour_ptr[k + 1] += L.colour_ptr[k];
  L.colour_cells.assign(L.n_cells, 0);
  std::vector<int> fill(L.colour_ptr.begin(), L.colour_ptr.end() - 1);
  for (int c = 0; c < L.n_cells; ++c) L.colour_cells[fill[col[c]]++] = c;
}

// ---------------------------------------------------------------- Newton / dilation terms
// Per finest cell and quadrature point, the tables of OperatorCellData
// (include/aspect/simulator/solver/matrix_free_operators.h:92-208) that the outer
// Stokes operator reads when Newton derivatives or a prescribed dilation are
// enabled (matrix_free_operators.cc:400-538). Symmetric tensors are stored as
// deal.II unrolls them: (00, 11, 22, 01, 02, 12) in 3D, (00, 11, 01) in 2D.
struct NewtonTerms {
  bool newton = false, symmetrize = false, average = false, dilation = false;
  std::vector<double> E;    // strain_rate_table (the linearisation point's strain rate)
  std::vector<double> D;    // newton_factor_wrt_strain_rate_table
  std::vector<double> dp;   // newton_factor_wrt_pressure_table
  std::vector<double> lhs;  // dilation_lhs_term_table
  std::vector<double> DD;   // dilation_derivative_wrt_strain_rate_table
  std::vector<double> dpd;  // dilation_derivative_wrt_pressure_table
};
static inline int sym_index(int dim, int a, int b) {
  if (a == b) return a;
  if (a > b) std::swap(a, b);
  return dim == 2 ? 2 : (a == 0 ? (b == 1 ? 3 : 4) : 5);
}
template <class T>
static inline void sym_full(const double* t, int dim, T (&M)[3][3]) {
  for (int a = 0; a < dim; ++a)
    for (int b = 0; b < dim; ++b) M[a][b] = (T)t[sym_index(dim, a, b)];
}

// ---------------------------------------------------------------- cell kernel
// Applies one operator to the cell-local vectors; results are added to yu/yp.
// nt (outer Stokes operator of the finest level only): Newton / dilation terms.
template <class T>
static void cell_apply(const Level& L, const FE& fe, int c, int op, double s, int compressible,
                       const T* eta_tab, const T* xu, const T* xp, T* yu, T* yp, const NewtonTerms* nt = nullptr) {
  const int d = L.dim, nq = fe.nq, nv = fe.nv, np = fe.np;
  const int ns = d == 3 ? 6 : 3;
  // a prescribed dilation makes the outer viscous term deviatoric, as compressibility does
  const bool deviatoric = compressible || (nt && nt->dilation);
  if (op != OP_STOKES && op != OP_A) nt = nullptr;
  const NewtonTerms* ntS = op == OP_STOKES ? nt : nullptr;  // Newton / dilation terms: Stokes only
  // real-space velocity gradient and pressure at a point
  auto grad_at = [&](int q, T (&G)[3][3], T& pq) {
    const double* iJ = &L.invJ[((size_t)c * nq + q) * d * d];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) G[a][b] = 0;
    for (int n = 0; n < nv; ++n)
      for (int e = 0; e < d; ++e) {
        double t = 0;
        for (int a = 0; a < d; ++a) t += fe.vgrad[(q * nv + n) * d + a] * iJ[a * d + e];
        for (int cc = 0; cc < d; ++cc) G[cc][e] += xu[cc * nv + n] * (T)t;
      }
    pq = 0;
    for (int n = 0; n < np; ++n) pq += xp[n] * (T)fe.pval[q * np + n];
  };
  // averaged Newton factors: cell sums over the points (matrix_free_operators.cc:411-445)
  T avg_a = 0, avg_bp = 0, avg_eu = 0, avg_th = 0;
  if (ntS && ntS->newton && ntS->average) {
    const NewtonTerms* nt = ntS;
    for (int q = 0; q < nq; ++q) {
      T G[3][3], pq;
      grad_at(q, G, pq);
      T Dm[3][3], Em[3][3];
      sym_full(&nt->D[((size_t)c * nq + q) * ns], d, Dm);
      sym_full(&nt->E[((size_t)c * nq + q) * ns], d, Em);
      const T jxw = (T)L.JxW[(size_t)c * nq + q];
      T div = 0, trE = 0;
      for (int a = 0; a < d; ++a) { div += G[a][a]; trE += Em[a][a]; }
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) {
          const T eps = (T)0.5 * (G[a][b] + G[b][a]);
          avg_a += Dm[a][b] * eps;
          if (nt->symmetrize) avg_eu += Em[a][b] * eps * jxw;
        }
      avg_bp += (T)nt->dp[(size_t)c * nq + q] * pq;
      if (nt->symmetrize && (compressible || nt->dilation)) avg_th += trE * div * jxw;
    }
  }
  for (int q = 0; q < nq; ++q) {
    const double* iJ = &L.invJ[((size_t)c * nq + q) * d * d];
    const T jxw = (T)L.JxW[(size_t)c * nq + q];
    const T eta = eta_tab[(size_t)c * L.eta_n + (L.eta_n == 1 ? 0 : q)];
    // real-space gradients of the velocity basis at q
    T G[3][3] = {{0}};
    T pq = 0;
    T grad_phi[64][3];
    if (op != OP_MASS) {
      for (int n = 0; n < nv; ++n)
        for (int e = 0; e < d; ++e) {
          double t = 0;
          for (int a = 0; a < d; ++a) t += fe.vgrad[(q * nv + n) * d + a] * iJ[a * d + e];
          grad_phi[n][e] = (T)t;
        }
    }
    if (op == OP_STOKES || op == OP_A)
      for (int cc = 0; cc < d; ++cc)
        for (int n = 0; n < nv; ++n) {
          T u = xu[cc * nv + n];
          for (int e = 0; e < d; ++e) G[cc][e] += u * grad_phi[n][e];
        }
    if (op == OP_STOKES || op == OP_BT || op == OP_MASS)
      for (int n = 0; n < np; ++n) pq += xp[n] * (T)fe.pval[q * np + n];
    if (op == OP_MASS) {
      T f = (T)(s * s) / eta * pq * jxw;
      for (int n = 0; n < np; ++n) yp[n] += f * (T)fe.pval[q * np + n];
      continue;
    }
    T F[3][3] = {{0}};
    T div = 0;
    for (int e = 0; e < d; ++e) div += G[e][e];
    if (op == OP_STOKES || op == OP_A) {
      const T eta2 = (T)2 * eta;
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) F[a][b] = eta2 * (T)0.5 * (G[a][b] + G[b][a]);
      if (deviatoric)
        for (int a = 0; a < d; ++a) F[a][a] -= eta2 / (T)3 * div;
    }
    if (op == OP_STOKES || op == OP_BT)
      for (int a = 0; a < d; ++a) F[a][a] -= (T)s * pq;
    T ptest = -(T)s * div;  // terms tested by the pressure basis
    if (ntS) {
      const NewtonTerms* nt = ntS;
      const size_t cq = (size_t)c * nq + q;
      if (nt->dilation) ptest -= (T)(s * s) * (T)nt->lhs[cq] * pq;
      if (nt->newton) {
        T Dm[3][3], Em[3][3];
        sym_full(&nt->D[cq * ns], d, Dm);
        sym_full(&nt->E[cq * ns], d, Em);
        T de = 0, ee = 0, trE = 0;
        for (int a = 0; a < d; ++a) {
          trE += Em[a][a];
          for (int b = 0; b < d; ++b) {
            const T eps = (T)0.5 * (G[a][b] + G[b][a]);
            de += Dm[a][b] * eps;
            ee += Em[a][b] * eps;
          }
        }
        T a_ = nt->average ? avg_a : de;                          // deta_deps : sym_grad_u
        const T bp = nt->average ? avg_bp : (T)nt->dp[cq] * pq;   // deta_dp p
        if (nt->symmetrize && nt->average) ee = avg_eu / jxw;    // eps : sym_grad_u
        for (int x = 0; x < d; ++x)
          for (int y = 0; y < d; ++y) {
            if (nt->symmetrize) F[x][y] += Em[x][y] * a_ + Dm[x][y] * ee;
            else F[x][y] += (T)2 * Em[x][y] * a_;
            F[x][y] += (T)2 * Em[x][y] * bp;
          }
        if (deviatoric) {
          if (nt->symmetrize) {
            const T th = nt->average ? avg_th / jxw : trE * div;
            for (int x = 0; x < d; ++x)
              for (int y = 0; y < d; ++y) F[x][y] -= (T)(1.0 / 3.0) * Dm[x][y] * th;
            for (int x = 0; x < d; ++x) F[x][x] -= (T)(1.0 / 3.0) * trE * a_;
          } else {
            for (int x = 0; x < d; ++x) F[x][x] -= (T)(2.0 / 3.0) * trE * a_;
          }
          if (nt->dilation) {
            T DDm[3][3];
            sym_full(&nt->DD[cq * ns], d, DDm);
            T dde = 0;
            for (int x = 0; x < d; ++x)
              for (int y = 0; y < d; ++y) dde += DDm[x][y] * (T)0.5 * (G[x][y] + G[y][x]);
            ptest += (dde + (T)nt->dpd[cq] * (T)s * pq) * (T)s;
          }
        }
      }
    }
    for (int cc = 0; cc < d; ++cc)
      for (int n = 0; n < nv; ++n) {
        T t = 0;
        for (int e = 0; e < d; ++e) t += F[cc][e] * grad_phi[n][e];
        yu[cc * nv + n] += t * jxw;
      }
    if (op == OP_STOKES) {
      T f = ptest * jxw;
      for (int n = 0; n < np; ++n) yp[n] += f * (T)fe.pval[q * np + n];
    }
  }
}

// ---------------------------------------------------------------- sum-factorised cell kernel
// The same cell operator as cell_apply, evaluated by sum factorisation the way
// the reference's CPU code does (deal.II FEEvaluation: tensor-product sweeps
// of the 1D basis values and derivatives at the Gauss points, then the
// quadrature-point physics, then the transposed sweeps). It serves the CPU
// baseline timing ("fast" mode); the checker keeps the plain quadrature loops
// above, and tests compare the two.
struct Basis1D {
  double S[3][3], D[3][3];  // phi_n(g_q), phi_n'(g_q) of the Q2 basis at the 3 Gauss points
};
static Basis1D make_basis1d() {
  Basis1D b;
  const double g[3] = {0.5 - 0.5 * std::sqrt(0.6), 0.5, 0.5 + 0.5 * std::sqrt(0.6)};
  const double q2n[3] = {0.0, 0.5, 1.0};
  for (int q = 0; q < 3; ++q) lagrange1d(q2n, 3, g[q], b.S[q], b.D[q]);
  return b;
}
static const Basis1D& basis1d() {
  static const Basis1D b = make_basis1d();
  return b;
}

// out[.. q_dir ..] = sum_n M[q][n] in[.. n_dir ..] (or M^T), 3 points per direction
template <class T, int dim, int dir, bool transpose>
static inline void sf_sweep(const double (&M)[3][3], const T* in, T* out) {
  constexpr int st = dir == 0 ? 1 : dir == 1 ? 3 : 9;
  constexpr int N = dim == 3 ? 27 : 9;
  for (int b = 0; b < N; ++b) {
    if ((b / st) % 3 != 0) continue;
    const T a0 = in[b], a1 = in[b + st], a2 = in[b + 2 * st];
    for (int q = 0; q < 3; ++q) {
      const T m0 = (T)(transpose ? M[0][q] : M[q][0]);
      const T m1 = (T)(transpose ? M[1][q] : M[q][1]);
      const T m2 = (T)(transpose ? M[2][q] : M[q][2]);
      out[b + q * st] = m0 * a0 + m1 * a1 + m2 * a2;
    }
  }
}

// reference gradient g[dir][q] of one nodal field u
template <class T, int dim>
static inline void sf_grad(const Basis1D& B, const T* u, T (*g)[27]) {
  if (dim == 2) {
    T t[9];
    sf_sweep<T, 2, 1, false>(B.S, u, t);
    sf_sweep<T, 2, 0, false>(B.D, t, g[0]);
    sf_sweep<T, 2, 1, false>(B.D, u, t);
    sf_sweep<T, 2, 0, false>(B.S, t, g[1]);
  } else {
    T t1[27], t2[27];
    sf_sweep<T, 3, 2, false>(B.S, u, t1);
    sf_sweep<T, 3, 1, false>(B.S, t1, t2);
    sf_sweep<T, 3, 0, false>(B.D, t2, g[0]);
    sf_sweep<T, 3, 1, false>(B.D, t1, t2);
    sf_sweep<T, 3, 0, false>(B.S, t2, g[1]);
    sf_sweep<T, 3, 2, false>(B.D, u, t1);
    sf_sweep<T, 3, 1, false>(B.S, t1, t2);
    sf_sweep<T, 3, 0, false>(B.S, t2, g[2]);
  }
}

// y += sum_dir (gradient in direction dir)^T r[dir]
template <class T, int dim>
static inline void sf_grad_t(const Basis1D& B, T (*r)[27], T* y) {
  if (dim == 2) {
    T a[9], b[9];
    sf_sweep<T, 2, 0, true>(B.D, r[0], a);
    sf_sweep<T, 2, 1, true>(B.S, a, b);
    for (int n = 0; n < 9; ++n) y[n] += b[n];
    sf_sweep<T, 2, 0, true>(B.S, r[1], a);
    sf_sweep<T, 2, 1, true>(B.D, a, b);
    for (int n = 0; n < 9; ++n) y[n] += b[n];
  } else {
    T a[27], b[27], s1[27];
    sf_sweep<T, 3, 0, true>(B.D, r[0], a);
    sf_sweep<T, 3, 1, true>(B.S, a, s1);
    sf_sweep<T, 3, 0, true>(B.S, r[1], a);
    sf_sweep<T, 3, 1, true>(B.D, a, b);
    for (int n = 0; n < 27; ++n) s1[n] += b[n];
    sf_sweep<T, 3, 2, true>(B.S, s1, a);
    for (int n = 0; n < 27; ++n) y[n] += a[n];
    sf_sweep<T, 3, 0, true>(B.S, r[2], a);
    sf_sweep<T, 3, 1, true>(B.S, a, b);
    sf_sweep<T, 3, 2, true>(B.D, b, a);
    for (int n = 0; n < 27; ++n) y[n] += a[n];
  }
}

template <class T, int dim>
static void cell_apply_sf(const Level& L, const FE& fe, int c, int op, double s, int compressible,
                          const T* eta_tab, const T* xu, const T* xp, T* yu, T* yp) {
  constexpr int d = dim, nq = dim == 3 ? 27 : 9, nv = nq, np = dim == 3 ? 8 : 4;
  const Basis1D& B = basis1d();
  const bool use_u = (op == OP_STOKES || op == OP_A), use_p = (op == OP_STOKES || op == OP_BT);
  const bool cart = L.geom_kind == 0;
  T gref[3][3][27];  // [component][reference direction][q]
  if (use_u)
    for (int cc = 0; cc < d; ++cc) sf_grad<T, dim>(B, xu + cc * nv, gref[cc]);
  T rref[3][3][27];
  T fp[27];
  for (int q = 0; q < nq; ++q) {
    const double* iJ = &L.invJ[((size_t)c * nq + q) * d * d];
    const T jxw = (T)L.JxW[(size_t)c * nq + q];
    const T eta = eta_tab[(size_t)c * L.eta_n + (L.eta_n == 1 ? 0 : q)];
    T G[3][3] = {{0}};
    if (use_u && cart) {  // box cells: diagonal inverse Jacobian
      for (int cc = 0; cc < d; ++cc)
        for (int e = 0; e < d; ++e) G[cc][e] = gref[cc][e][q] * (T)iJ[e * d + e];
    } else if (use_u) {
      for (int cc = 0; cc < d; ++cc)
        for (int e = 0; e < d; ++e) {
          T t = 0;
          for (int a = 0; a < d; ++a) t += gref[cc][a][q] * (T)iJ[a * d + e];
          G[cc][e] = t;
        }
    }
    T pq = 0;
    if (use_p)
      for (int n = 0; n < np; ++n) pq += xp[n] * (T)fe.pval[q * np + n];
    T F[3][3] = {{0}};
    T div = 0;
    for (int e = 0; e < d; ++e) div += G[e][e];
    if (use_u) {
      const T eta2 = (T)2 * eta;
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) F[a][b] = eta2 * (T)0.5 * (G[a][b] + G[b][a]);
      if (compressible)
        for (int a = 0; a < d; ++a) F[a][a] -= eta2 / (T)3 * div;
    }
    if (use_p)
      for (int a = 0; a < d; ++a) F[a][a] -= (T)s * pq;
    for (int cc = 0; cc < d; ++cc)
      for (int a = 0; a < d; ++a) {
        if (cart) {
          rref[cc][a][q] = F[cc][a] * (T)iJ[a * d + a] * jxw;
          continue;
        }
        T t = 0;
        for (int e = 0; e < d; ++e) t += F[cc][e] * (T)iJ[a * d + e];
        rref[cc][a][q] = t * jxw;
      }
    if (op == OP_STOKES) fp[q] = -(T)s * div * jxw;
  }
  for (int cc = 0; cc < d; ++cc) sf_grad_t<T, dim>(B, rref[cc], yu + cc * nv);
  if (op == OP_STOKES)
    for (int n = 0; n < np; ++n) {
      T t = 0;
      for (int q = 0; q < nq; ++q) t += (T)fe.pval[q * np + n] * fp[q];
      yp[n] += t;
    }
}

// "fast" mode (CPU baseline timing only): sum-factorised cell operators and
// deterministic parallel reductions (fixed chunks summed in order).
static bool g_fast = false;

template <class T>
static void cell_apply_any(const Level& L, const FE& fe, int c, int op, double s, int compressible,
                           const T* eta_tab, const T* xu, const T* xp, T* yu, T* yp,
                           const NewtonTerms* nt = nullptr) {
  if (g_fast && op != OP_MASS && !nt && fe.degree == 2) {
    if (L.dim == 3) cell_apply_sf<T, 3>(L, fe, c, op, s, compressible, eta_tab, xu, xp, yu, yp);
    else cell_apply_sf<T, 2>(L, fe, c, op, s, compressible, eta_tab, xu, xp, yu, yp);
    return;
  }
  cell_apply<T>(L, fe, c, op, s, compressible, eta_tab, xu, xp, yu, yp, nt);
}

// sum a[i] b[i]: serial in the checker; in fast mode 256 fixed chunks summed
// in parallel and then in chunk order, so the result does not depend on the
// number of threads
static double dot_n(const double* a, const double* b, long n) {
  if (!g_fast || n < 65536) {
    double s_ = 0;
    for (long i = 0; i < n; ++i) s_ += a[i] * b[i];
    return s_;
  }
  constexpr int K = 256;
  double part[K];
  const long chunk = (n + K - 1) / K;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < K; ++k) {
    double s_ = 0;
    const long e = std::min(n, (k + 1) * chunk);
    for (long i = k * chunk; i < e; ++i) s_ += a[i] * b[i];
    part[k] = s_;
  }
  double s_ = 0;
  for (int k = 0; k < K; ++k) s_ += part[k];
  return s_;
}

// ---------------------------------------------------------------- solver state
struct Params {
  double tol_rel = 1e-7;        // Linear solver tolerance
  double abs_tol = 0.0;         // >0: use as absolute tolerance directly
  int n_cheap = 1000, n_expensive = 1000, restart = 100;
  double tol_A = 1e-2, tol_S = 1e-6;
  int mg_float = 0;             // level operators in float
  int A_symmetric = 1;
  int krylov = 0;               // cheap phase: 0 GMRES, 2 IDR(s)
  int idr_s = 2;                // IDR(s) parameter
};

struct Outputs {
  double initial_nonlinear_residual, final_linear_residual, solver_tolerance;
  int cheap_iterations, expensive_iterations, A_prec_applications, S_prec_applications;
  int status;  // 0 ok, 1 no convergence
};

struct Oracle {
  int dim = 3;
  FE fe;
  std::vector<Level> levels;
  double s = 1.0;
  int compressible = 0;
  int projection = 0;  // 0: DGQ0, 1: DGQ1 (project to Q1)
  double eta_min = 0, eta_max = 0;
  std::string err;
  // float copies of level data
  std::vector<std::vector<float>> eta_f, dA_f, dM_f;
  int a_cg_iterations = 0;
  // Newton / prescribed-dilation tables of the outer operators (finest level)
  NewtonTerms newton;
  const NewtonTerms* apply_nt = nullptr;  // set while an outer operator is applied
  // free-surface stabilisation faces of the outer Stokes operator (finest level):
  // caller cell, face number 2*d + side, per face point T then n JxW (2*dim values)
  struct FreeSurface {
    std::vector<int> cell, fno;
    std::vector<double> tab;
  } fs;
  bool apply_fs = false;
  struct OuterTerms {  // makes apply() add the Newton / dilation / face terms for one call
    Oracle& o;
    explicit OuterTerms(Oracle& o_) : o(o_) {
      if (o.newton.newton || o.newton.dilation) o.apply_nt = &o.newton;
      o.apply_fs = !o.fs.cell.empty();
    }
    ~OuterTerms() {
      o.apply_nt = nullptr;
      o.apply_fs = false;
    }
  };

  // Free-surface face term (StokesOperator::local_apply_boundary_face,
  // matrix_free_operators.cc:563-602): dst_u(phi) += sum_q -(T_q . u(x_q)) (n JxW)_q . phi(x_q)
  // over each face's QGauss(3) points, u read and the result distributed through
  // the constraints; plain basis evaluation at the face points.
  template <class T>
  void face_terms(const Level& L, const T* src_u, T* dst_u, bool plain = false) {
    const int d = dim, nv = fe.nv, nf = d == 3 ? 9 : 3;
    const double gp[3] = {0.5 - std::sqrt(15.0) / 10, 0.5, 0.5 + std::sqrt(15.0) / 10};
    for (size_t f = 0; f < fs.cell.size(); ++f) {
      const int c = fs.cell[f], dn = fs.fno[f] >> 1, side = fs.fno[f] & 1;
      int tang[2], m = 0;
      for (int a = 0; a < d; ++a)
        if (a != dn) tang[m++] = a;
      T xu[81] = {0}, yu[81] = {0};
      for (int i = 0; i < d * nv; ++i) {
        const int gd = L.cdu[(size_t)c * d * nv + i];
        if (plain) { xu[i] = src_u[gd]; continue; }
        Expansion e = expand(L.cu, gd);
        for (int k = 0; k < e.n; ++k) xu[i] += (T)e.w[k] * src_u[e.g[k]];
      }
      for (int q = 0; q < nf; ++q) {
        double xi[3] = {0, 0, 0};
        xi[dn] = side;
        xi[tang[0]] = gp[q % 3];
        if (d == 3) xi[tang[1]] = gp[q / 3];
        double phi[27];
        q2_basis_at(d, xi, phi);
        const double* t = &fs.tab[(f * nf + q) * 2 * d];
        T uq[3] = {0, 0, 0};
        for (int a = 0; a < d; ++a)
          for (int n = 0; n < nv; ++n) uq[a] += (T)phi[n] * xu[a * nv + n];
        T tu = 0;
        for (int a = 0; a < d; ++a) tu += (T)t[a] * uq[a];
        for (int a = 0; a < d; ++a)
          for (int n = 0; n < nv; ++n) yu[a * nv + n] += (T)phi[n] * (-tu * (T)t[d + a]);
      }
      for (int i = 0; i < d * nv; ++i) {
        Expansion e = expand(L.cu, L.cdu[(size_t)c * d * nv + i]);
        for (int k = 0; k < e.n; ++k) dst_u[e.g[k]] += (T)e.w[k] * yu[i];
      }
    }
  }

  Level& fine() { return levels.back(); }

  // -------- operator application on a level (constrained rows = identity)
  template <class T>
  void apply(int lev, int op, const T* src_u, const T* src_p, T* dst_u, T* dst_p, const T* eta_tab) {
    Level& L = levels[lev];
    const int nu = fe.nu, np = fe.np;
    bool wu = (op == OP_STOKES || op == OP_A || op == OP_BT);
    bool wp = (op == OP_STOKES || op == OP_MASS);
    bool ru = (op == OP_STOKES || op == OP_A);
    bool rp = (op != OP_A);
    if (wu) std::fill(dst_u, dst_u + L.n_u, (T)0);
    if (wp) std::fill(dst_p, dst_p + L.n_p, (T)0);
    for (size_t k = 0; k + 1 < L.colour_ptr.size(); ++k) {
#pragma omp parallel for schedule(static)
      for (int ci = L.colour_ptr[k]; ci < L.colour_ptr[k + 1]; ++ci) {
        int c = L.colour_cells[ci];
        T xu[192] = {0}, xp[27] = {0}, yu[192] = {0}, yp[27] = {0};
        if (ru)
          for (int i = 0; i < nu; ++i) {
            Expansion e = expand(L.cu, L.cdu[(size_t)c * nu + i]);
            T v = 0;
            for (int m = 0; m < e.n; ++m) v += (T)e.w[m] * src_u[e.g[m]];
            xu[i] = v;
          }
        if (rp)
          for (int i = 0; i < np; ++i) {
            Expansion e = expand(L.cp, L.cdp[(size_t)c * np + i]);
            T v = 0;
            for (int m = 0; m < e.n; ++m) v += (T)e.w[m] * src_p[e.g[m]];
            xp[i] = v;
          }
        cell_apply_any<T>(L, fe, c, op, s, compressible, eta_tab, xu, xp, yu, yp, apply_nt);
        if (wu)
          for (int i = 0; i < nu; ++i) {
            Expansion e = expand(L.cu, L.cdu[(size_t)c * nu + i]);
            for (int m = 0; m < e.n; ++m) dst_u[e.g[m]] += (T)e.w[m] * yu[i];
          }
        if (wp)
          for (int i = 0; i < np; ++i) {
            Expansion e = expand(L.cp, L.cdp[(size_t)c * np + i]);
            for (int m = 0; m < e.n; ++m) dst_p[e.g[m]] += (T)e.w[m] * yp[i];
          }
      }
    }
    if (apply_fs && op == OP_STOKES && lev == (int)levels.size() - 1) face_terms<T>(L, src_u, dst_u);
    // identity on constrained rows (Base::vmult: dst = src there)
    if (op == OP_BT) {
      for (int g = 0; g < L.n_u; ++g)
        if (L.cu.constrained(g)) dst_u[g] = 0;  // BT maps p -> u; no u input
    } else {
      if (wu)
        for (int g = 0; g < L.n_u; ++g)
          if (L.cu.constrained(g)) dst_u[g] = src_u[g];
      if (wp)
        for (int g = 0; g < L.n_p; ++g)
          if (L.cp.constrained(g)) dst_p[g] = src_p[g];
    }
  }

  template <class T>
  const T* eta_table(int lev);

  // -------- diagonal of A (block 0) or the mass matrix (block 1), inverted
  void compute_diagonal(int lev, int block, std::vector<double>& dinv) {
    Level& L = levels[lev];
    const int nl = block == 0 ? fe.nu : fe.np;
    const int n = block == 0 ? L.n_u : L.n_p;
    const Constraints& C = block == 0 ? L.cu : L.cp;
    const std::vector<int>& cd = block == 0 ? L.cdu : L.cdp;
    std::vector<double> diag(n, 0.0);
    for (size_t k = 0; k + 1 < L.colour_ptr.size(); ++k) {
#pragma omp parallel for schedule(dynamic, 16)
      for (int ci = L.colour_ptr[k]; ci < L.colour_ptr[k + 1]; ++ci) {
        int c = L.colour_cells[ci];
        std::vector<Expansion> ex(nl);
        std::set<int> gs;
        for (int i = 0; i < nl; ++i) {
          ex[i] = expand(C, cd[(size_t)c * nl + i]);
          for (int m = 0; m < ex[i].n; ++m) gs.insert(ex[i].g[m]);
        }
        // element matrix by unit vectors
        std::vector<double> K((size_t)nl * nl, 0.0);
        for (int j = 0; j < nl; ++j) {
          double xu[192] = {0}, xp[27] = {0}, yu[192] = {0}, yp[27] = {0};
          if (block == 0) xu[j] = 1.0; else xp[j] = 1.0;
          cell_apply_any<double>(L, fe, c, block == 0 ? OP_A : OP_MASS, s, compressible, L.eta.data(), xu, xp, yu, yp);
          for (int i = 0; i < nl; ++i) K[(size_t)i * nl + j] = block == 0 ? yu[i] : yp[i];
        }
        for (int g : gs) {
          double v[192];
          for (int i = 0; i < nl; ++i) {
            v[i] = 0;
            for (int m = 0; m < ex[i].n; ++m)
              if (ex[i].g[m] == g) v[i] += ex[i].w[m];
          }
          double acc = 0;
          for (int i = 0; i < nl; ++i) {
            if (v[i] == 0) continue;
            double t = 0;
            for (int j = 0; j < nl; ++j) t += K[(size_t)i * nl + j] * v[j];
            acc += v[i] * t;
          }
          diag[g] += acc;
        }
      }
    }
    dinv.assign(n, 1.0);
    for (int g = 0; g < n; ++g) {
      if (C.constrained(g)) { dinv[g] = 1.0; continue; }
      if (!(diag[g] > 0)) throw std::runtime_error("non-positive diagonal entry");
      dinv[g] = 1.0 / diag[g];
    }
  }

  // -------- transfer matrices: rows = fine level unconstrained dofs
  void build_transfer(int lev) {
    Level& F = levels[lev];
    Level& C = levels[lev - 1];
    const int d = dim;
    for (int block = 0; block < 2; ++block) {
      const int nl = block == 0 ? fe.nv : fe.np;
      const int ncomp = block == 0 ? d : 1;
      const int nf = block == 0 ? F.n_u : F.n_p;
      std::vector<std::map<int, double>> rows(nf);
      std::vector<char> done(nf, 0);
      for (int fc = 0; fc < F.n_cells; ++fc) {
        int pc = F.parent[fc], ch = F.child[fc];
        for (int n = 0; n < nl; ++n) {
          double xi[3];
          const int n1 = block == 0 ? fe.n1 : fe.degree;  // nodes per direction
          const double* nodes = block == 0 ? fe.vnodes : fe.pnodes;
          for (int e = 0; e < d; ++e) {
            int idx = (e == 0 ? n : e == 1 ? n / n1 : n / (n1 * n1)) % n1;
            double loc = nodes[idx];
            xi[e] = ch == 255 ? loc : 0.5 * (((ch >> e) & 1) + loc);  // 255: the same cell
          }
          double phi[64];
          fe.basis_at(block, xi, phi);
          for (int comp = 0; comp < ncomp; ++comp) {
            int gf = block == 0 ? F.cdu[(size_t)fc * fe.nu + comp * nl + n] : F.cdp[(size_t)fc * fe.np + n];
            const Constraints& FC = block == 0 ? F.cu : F.cp;
            if (FC.constrained(gf) || done[gf]) continue;
            done[gf] = 1;
            for (int m = 0; m < nl; ++m) {
              if (std::fabs(phi[m]) < 1e-14) continue;
              int gc = block == 0 ? C.cdu[(size_t)pc * fe.nu + comp * nl + m] : C.cdp[(size_t)pc * fe.np + m];
              Expansion e = expand(block == 0 ? C.cu : C.cp, gc);
              for (int k = 0; k < e.n; ++k) rows[gf][e.g[k]] += phi[m] * e.w[k];
            }
          }
        }
      }
      std::vector<int>& ptr = block == 0 ? F.Pu_ptr : F.Pp_ptr;
      std::vector<int>& col = block == 0 ? F.Pu_col : F.Pp_col;
      std::vector<double>& val = block == 0 ? F.Pu_val : F.Pp_val;
      ptr.assign(1, 0); col.clear(); val.clear();
      for (int r = 0; r < nf; ++r) {
        for (auto& kv : rows[r])
          if (std::fabs(kv.second) > 1e-14) { col.push_back(kv.first); val.push_back(kv.second); }
        ptr.push_back((int)col.size());
      }
    }
  }

  template <class T>
  void prolongate_add(int lev, int block, const T* coarse, T* fine_v) {
    Level& F = levels[lev];
    const auto& ptr = block == 0 ? F.Pu_ptr : F.Pp_ptr;
    const auto& col = block == 0 ? F.Pu_col : F.Pp_col;
    const auto& val = block == 0 ? F.Pu_val : F.Pp_val;
    int n = (int)ptr.size() - 1;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n; ++r) {
      T t = 0;
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) t += (T)val[k] * coarse[col[k]];
      fine_v[r] += t;
    }
  }
  template <class T>
  void restrict_add(int lev, int block, const T* fine_v, T* coarse) {
    Level& F = levels[lev];
    if (g_fast) {  // rows of P^T in parallel (fast mode builds the transpose once)
      build_transfer_transpose(lev);
      const auto& ptr = block == 0 ? F.PuT_ptr : F.PpT_ptr;
      const auto& col = block == 0 ? F.PuT_col : F.PpT_col;
      const auto& val = block == 0 ? F.PuT_val : F.PpT_val;
      const int n = (int)ptr.size() - 1;
#pragma omp parallel for schedule(static)
      for (int r = 0; r < n; ++r) {
        T t = 0;
        for (int k = ptr[r]; k < ptr[r + 1]; ++k) t += (T)val[k] * fine_v[col[k]];
        coarse[r] += t;
      }
      return;
    }
    const auto& ptr = block == 0 ? F.Pu_ptr : F.Pp_ptr;
    const auto& col = block == 0 ? F.Pu_col : F.Pp_col;
    const auto& val = block == 0 ? F.Pu_val : F.Pp_val;
    int n = (int)ptr.size() - 1;
    for (int r = 0; r < n; ++r)
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) coarse[col[k]] += (T)val[k] * fine_v[r];
  }
  void build_transfer_transpose(int lev) {
    Level& F = levels[lev];
    if (F.PT_built) return;
    for (int block = 0; block < 2; ++block) {
      const auto& ptr = block == 0 ? F.Pu_ptr : F.Pp_ptr;
      const auto& col = block == 0 ? F.Pu_col : F.Pp_col;
      const auto& val = block == 0 ? F.Pu_val : F.Pp_val;
      const int nc = block == 0 ? levels[lev - 1].n_u : levels[lev - 1].n_p;
      auto& tp = block == 0 ? F.PuT_ptr : F.PpT_ptr;
      auto& tc = block == 0 ? F.PuT_col : F.PpT_col;
      auto& tv = block == 0 ? F.PuT_val : F.PpT_val;
      tp.assign(nc + 1, 0);
      for (int c : col) tp[c + 1]++;
      for (int r = 0; r < nc; ++r) tp[r + 1] += tp[r];
      tc.assign(col.size(), 0);
      tv.assign(col.size(), 0.0);
      std::vector<int> fill(tp.begin(), tp.end() - 1);
      const int nf = (int)ptr.size() - 1;
      for (int r = 0; r < nf; ++r)
        for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
          tc[fill[col[k]]] = r;
          tv[fill[col[k]]++] = val[k];
        }
    }
    F.PT_built = true;
  }

  // -------- viscosity on levels (stokes_matrix_free_local_smoothing.cc:174-294)
  // Input: raw material-model values on the finest level, per cell (1 value,
  // already averaged: DGQ0) or per quadrature point (projection = 1: DGQ1).
  // mg_finest_projected (per-point input with DGQ0 only): the multigrid levels,
  // the finest included, take the DGQ0 projection while the outer operators keep
  // the per-point values -- what the reference does without averaging
  // (stokes_matrix_free_local_smoothing.cc:211-294 fills level_cell_data for every
  // level from the projected vector; matrix_free_operators.cc:137-330 keeps the raw
  // values in active_cell_data for the outer operators).
  std::vector<double> active_eta;
  int active_eta_n = 0;
  struct ActiveTable {  // swaps the outer-operator table into the finest level for one call
    Oracle& o;
    bool on;
    explicit ActiveTable(Oracle& o_) : o(o_), on(!o_.active_eta.empty()) { swap(); }
    ~ActiveTable() { swap(); }
    void swap() {
      if (!on) return;
      Level& F = o.levels.back();
      std::swap(F.eta, o.active_eta);
      std::swap(F.eta_n, o.active_eta_n);
    }
  };

  void set_viscosity(const double* eta_in, int n_per_cell, int proj, double s_in, int comp,
                     bool mg_finest_projected = false) {
    s = s_in; compressible = comp; projection = proj;
    active_eta.clear();
    active_eta_n = 0;
    const int nq = fe.nq, nc_v = dim == 3 ? 8 : 4;
    const int nlev = (int)levels.size();
    // DG coefficient fields per level: DGQ0 -> 1 value, DGQ1 -> vertex values
    std::vector<std::vector<double>> dg(nlev);
    Level& Fl = fine();
    eta_min = 1e300; eta_max = -1e300;
    for (int i = 0; i < Fl.n_cells * n_per_cell; ++i) {
      eta_min = std::min(eta_min, eta_in[i]);
      eta_max = std::max(eta_max, eta_in[i]);
    }
    if (proj == 0) {
      dg[nlev - 1].assign(Fl.n_cells, 0.0);
      for (int c = 0; c < Fl.n_cells; ++c) {
        if (n_per_cell == 1) dg[nlev - 1][c] = eta_in[c];
        else {  // L2 projection onto constants: JxW-weighted mean
          double a = 0, v = 0;
          for (int q = 0; q < nq; ++q) { a += Fl.JxW[(size_t)c * nq + q] * eta_in[(size_t)c * nq + q]; v += Fl.JxW[(size_t)c * nq + q]; }
          dg[nlev - 1][c] = a / v;
        }
      }
      for (int l = nlev - 1; l > 0; --l) {
        Level& F = levels[l];
        std::vector<double> sum(levels[l - 1].n_cells, 0.0), cnt(levels[l - 1].n_cells, 0.0);
        for (int c = 0; c < F.n_cells; ++c) { sum[F.parent[c]] += dg[l][c]; cnt[F.parent[c]] += 1; }
        dg[l - 1].resize(levels[l - 1].n_cells);
        for (size_t c = 0; c < sum.size(); ++c) dg[l - 1][c] = sum[c] / cnt[c];
      }
      if (mg_finest_projected && n_per_cell == nq) {
        active_eta.assign(eta_in, eta_in + (size_t)Fl.n_cells * nq);
        active_eta_n = nq;
      }
      for (int l = 0; l < nlev; ++l) {
        Level& L = levels[l];
        bool active_per_q = (l == nlev - 1 && n_per_cell == nq && !mg_finest_projected);
        L.eta_n = active_per_q ? nq : 1;
        L.eta.assign((size_t)L.n_cells * L.eta_n, 0);
        for (int c = 0; c < L.n_cells; ++c) {
          if (active_per_q)
            for (int q = 0; q < nq; ++q) L.eta[(size_t)c * nq + q] = eta_in[(size_t)c * nq + q];
          else
            L.eta[c] = dg[l][c];
        }
      }
    } else {
      if (n_per_cell != nq) throw std::runtime_error("project to Q1 needs per-quadrature-point values");
      // per-cell L2 projection onto Q1 (Utilities::project_cellwise)
      dg[nlev - 1].assign((size_t)Fl.n_cells * nc_v, 0.0);
      for (int c = 0; c < Fl.n_cells; ++c) {
        double M[8][8] = {{0}}, b[8] = {0};
        for (int q = 0; q < nq; ++q) {
          double jw = Fl.JxW[(size_t)c * nq + q];
          for (int i = 0; i < nc_v; ++i) {
            b[i] += jw * fe.q1val[q * nc_v + i] * eta_in[(size_t)c * nq + q];
            for (int j = 0; j < nc_v; ++j) M[i][j] += jw * fe.q1val[q * nc_v + i] * fe.q1val[q * nc_v + j];
          }
        }
        // Gaussian elimination (SPD, small)
        for (int i = 0; i < nc_v; ++i) {
          for (int r = i + 1; r < nc_v; ++r) {
            double f = M[r][i] / M[i][i];
            for (int k = i; k < nc_v; ++k) M[r][k] -= f * M[i][k];
            b[r] -= f * b[i];
          }
        }
        for (int i = nc_v - 1; i >= 0; --i) {
          double t = b[i];
          for (int k = i + 1; k < nc_v; ++k) t -= M[i][k] * dg[nlev - 1][(size_t)c * nc_v + k];
          dg[nlev - 1][(size_t)c * nc_v + i] = t / M[i][i];
        }
      }
      // interpolate to coarser levels: a parent vertex is a vertex of exactly one child
      for (int l = nlev - 1; l > 0; --l) {
        Level& F = levels[l];
        dg[l - 1].assign((size_t)levels[l - 1].n_cells * nc_v, 0.0);
        for (int c = 0; c < F.n_cells; ++c) {
          int ch = F.child[c], p = F.parent[c];
          // the parent vertex lying at this child's corner "ch" is parent vertex ch,
          // and it is the child's own vertex ch; an unchanged cell keeps all four/eight
          if (ch == 255)
            for (int i = 0; i < nc_v; ++i) dg[l - 1][(size_t)p * nc_v + i] = dg[l][(size_t)c * nc_v + i];
          else
            dg[l - 1][(size_t)p * nc_v + ch] = dg[l][(size_t)c * nc_v + ch];
        }
      }
      for (int l = 0; l < nlev; ++l) {
        Level& L = levels[l];
        L.eta_n = nq;
        L.eta.assign((size_t)L.n_cells * nq, 0);
        for (int c = 0; c < L.n_cells; ++c)
          for (int q = 0; q < nq; ++q) {
            double v = 0;
            for (int i = 0; i < nc_v; ++i) v += fe.q1val[q * nc_v + i] * dg[l][(size_t)c * nc_v + i];
            L.eta[(size_t)c * nq + q] = std::clamp(v, eta_min, eta_max);
          }
      }
    }
    eta_f.assign(nlev, {});
    for (int l = 0; l < nlev; ++l) eta_f[l].assign(levels[l].eta.begin(), levels[l].eta.end());
  }

  // -------- Chebyshev smoother (deal.II PreconditionChebyshev semantics)
  struct Cheb { int degree; double range; int eig_its; };
  Cheb cheb_params(int lev) const { return lev > 0 ? Cheb{4, 15.0, 10} : Cheb{8, 1e-3, 100}; }

  template <class T>
  void level_op(int lev, int block, const T* x, T* y) {
    if (block == 0) apply<T>(lev, OP_A, x, nullptr, y, nullptr, eta_table<T>(lev));
    else apply<T>(lev, OP_MASS, nullptr, x, nullptr, y, eta_table<T>(lev));
  }
  template <class T>
  const T* dinv_table(int lev, int block);

  // tridiagonal eigenvalues (symmetric, via bisection-free QL): use Jacobi-like simple QR
  static void tridiag_eigs(std::vector<double> d, std::vector<double> e, double& lmin, double& lmax) {
    int n = (int)d.size();
    if (n == 0) { lmin = lmax = 0; return; }
    e.resize(n, 0.0);
    // implicit QL (tql1)
    for (int l = 0; l < n; ++l) {
      int iter = 0, m;
      do {
        for (m = l; m < n - 1; ++m) {
          double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
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
            double f = s_ * e[i], b = c * e[i];
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

  template <class T>
  void estimate_eigenvalues(int lev, int block) {
    Level& L = levels[lev];
    const int n = block == 0 ? L.n_u : L.n_p;
    const Constraints& C = block == 0 ? L.cu : L.cp;
    Cheb cp = cheb_params(lev);
    std::vector<T> b(n), x(n, 0), r(n), z(n), p(n), Ap(n);
    // PreconditionChebyshev's start vector: a period-11 mode (i mod 11) with its
    // mean removed, over all entries (the smoother data carries no constraints).
    // The pressure mass matrix has no null space and its largest eigenvector on
    // small coarse levels is the constant mode, so there the mean is kept.
    double mean = 0;
    if (block == 0) {
      for (int i = 0; i < n; ++i) mean += (double)(i % 11);
      mean /= std::max(n, 1);
    }
    for (int i = 0; i < n; ++i) b[i] = (T)((double)(i % 11) - mean);
    (void)C;
    const T* dinv = dinv_table<T>(lev, block);
    r = b;
    for (int i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
    p = z;
    double rz = 0;
    for (int i = 0; i < n; ++i) rz += (double)r[i] * z[i];
    std::vector<double> alphas, betas;
    for (int it = 0; it < cp.eig_its; ++it) {
      level_op<T>(lev, block, p.data(), Ap.data());
      double pAp = 0;
      for (int i = 0; i < n; ++i) pAp += (double)p[i] * Ap[i];
      if (!(pAp > 0)) break;
      double alpha = rz / pAp;
      alphas.push_back(alpha);
      for (int i = 0; i < n; ++i) { x[i] += (T)alpha * p[i]; r[i] -= (T)alpha * Ap[i]; }
      // SolverControl(eig_cg_n_iterations, eig_cg_residual = 1e-2), absolute
      double res = 0;
      for (int i = 0; i < n; ++i) res += (double)r[i] * r[i];
      if (std::sqrt(res) < 1e-2) break;
      for (int i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
      double rz_new = 0;
      for (int i = 0; i < n; ++i) rz_new += (double)r[i] * z[i];
      double beta = rz_new / rz;
      betas.push_back(beta);
      rz = rz_new;
      for (int i = 0; i < n; ++i) p[i] = z[i] + (T)beta * p[i];
    }
    // Lanczos tridiagonal from CG coefficients
    int k = (int)alphas.size();
    std::vector<double> dd(k), ee(k, 0.0);
    for (int i = 0; i < k; ++i) {
      dd[i] = 1.0 / alphas[i] + (i > 0 ? betas[i - 1] / alphas[i - 1] : 0.0);
      if (i + 1 < k) ee[i] = std::sqrt(betas[i]) / alphas[i];
    }
    double lmin, lmax;
    tridiag_eigs(dd, ee, lmin, lmax);
    double* eig = block == 0 ? L.eigA : L.eigM;
    eig[0] = lmin; eig[1] = lmax;
  }

  void chebyshev_bounds(int lev, int block, double& theta, double& delta) {
    Level& L = levels[lev];
    double* eig = block == 0 ? L.eigA : L.eigM;
    Cheb cp = cheb_params(lev);
    const double emax = eig[1] > 0 ? eig[1] : 1.0, emin = eig[1] > 0 ? eig[0] : 1.0;
    double lmax = 1.2 * emax;
    double alpha = cp.range > 1.0 ? lmax / cp.range : std::min(0.9 * lmax, emin);
    theta = 0.5 * (lmax + alpha);
    delta = 0.5 * (lmax - alpha);
  }

  // x = Cheb(b) from x = 0 (zero_start) or one step from the given x
  template <class T>
  void chebyshev(int lev, int block, T* x, const T* b, bool zero_start) {
    Level& L = levels[lev];
    const int n = block == 0 ? L.n_u : L.n_p;
    Cheb cp = cheb_params(lev);
    double theta, delta;
    chebyshev_bounds(lev, block, theta, delta);
    const T* dinv = dinv_table<T>(lev, block);
    std::vector<T> d(n), t(n);
    int k0;
    if (zero_start) {
#pragma omp parallel for schedule(static) if (g_fast && n > 16384)
      for (int i = 0; i < n; ++i) { d[i] = (T)(1.0 / theta) * dinv[i] * b[i]; x[i] = d[i]; }
      k0 = 1;
    } else {
      level_op<T>(lev, block, x, t.data());
#pragma omp parallel for schedule(static) if (g_fast && n > 16384)
      for (int i = 0; i < n; ++i) { d[i] = (T)(1.0 / theta) * dinv[i] * (b[i] - t[i]); x[i] += d[i]; }
      k0 = 1;
    }
    double rhok = delta / theta, sigma = theta / delta;
    for (int k = k0; k < cp.degree; ++k) {
      level_op<T>(lev, block, x, t.data());
      double rhokp = 1.0 / (2.0 * sigma - rhok);
      double f1 = rhokp * rhok, f2 = 2.0 * rhokp / delta;
      rhok = rhokp;
#pragma omp parallel for schedule(static) if (g_fast && n > 16384)
      for (int i = 0; i < n; ++i) {
        d[i] = (T)f1 * d[i] + (T)f2 * dinv[i] * (b[i] - t[i]);
        x[i] += d[i];
      }
    }
  }

  int smoothing_steps(int block) const { return block == 0 ? 1 : 4; }

  // mg::SmootherRelaxation::apply (from zero) and ::smooth (from x)
  template <class T>
  void smoother_apply(int lev, int block, T* x, const T* b) {
    chebyshev<T>(lev, block, x, b, true);
    for (int s_ = 1; s_ < smoothing_steps(block); ++s_) chebyshev<T>(lev, block, x, b, false);
  }
  template <class T>
  void smoother_smooth(int lev, int block, T* x, const T* b) {
    for (int s_ = 0; s_ < smoothing_steps(block); ++s_) chebyshev<T>(lev, block, x, b, false);
  }

  template <class T>
  void vcycle_level(int lev, int block, std::vector<std::vector<T>>& sol, std::vector<std::vector<T>>& def) {
    if (lev == 0) { smoother_apply<T>(0, block, sol[0].data(), def[0].data()); return; }
    Level& L = levels[lev];
    const int n = block == 0 ? L.n_u : L.n_p;
    smoother_apply<T>(lev, block, sol[lev].data(), def[lev].data());
    std::vector<T> t(n);
    level_op<T>(lev, block, sol[lev].data(), t.data());
    for (int i = 0; i < n; ++i) t[i] = def[lev][i] - t[i];
    std::fill(def[lev - 1].begin(), def[lev - 1].end(), (T)0);
    restrict_add<T>(lev, block, t.data(), def[lev - 1].data());
    std::fill(sol[lev - 1].begin(), sol[lev - 1].end(), (T)0);
    vcycle_level<T>(lev - 1, block, sol, def);
    prolongate_add<T>(lev, block, sol[lev - 1].data(), sol[lev].data());
    smoother_smooth<T>(lev, block, sol[lev].data(), def[lev].data());
  }

  // PreconditionMG::vmult on the finest level: dst = V(src)
  template <class T>
  void vcycle_T(int block, const double* src, double* dst) {
    int nlev = (int)levels.size();
    std::vector<std::vector<T>> sol(nlev), def(nlev);
    for (int l = 0; l < nlev; ++l) {
      int n = block == 0 ? levels[l].n_u : levels[l].n_p;
      sol[l].assign(n, 0); def[l].assign(n, 0);
    }
    int n = block == 0 ? fine().n_u : fine().n_p;
    for (int i = 0; i < n; ++i) def[nlev - 1][i] = (T)src[i];
    vcycle_level<T>(nlev - 1, block, sol, def);
    for (int i = 0; i < n; ++i) dst[i] = (double)sol[nlev - 1][i];
  }
  bool mg_float = false;
  void vcycle(int block, const double* src, double* dst) {
    if (mg_float) vcycle_T<float>(block, src, dst); else vcycle_T<double>(block, src, dst);
  }

  void build_preconditioner(bool use_float) {
    mg_float = use_float;
    int nlev = (int)levels.size();
    dA_f.assign(nlev, {}); dM_f.assign(nlev, {});
    for (int l = 0; l < nlev; ++l) {
      compute_diagonal(l, 0, levels[l].diagA_inv);
      compute_diagonal(l, 1, levels[l].diagM_inv);
      dA_f[l].assign(levels[l].diagA_inv.begin(), levels[l].diagA_inv.end());
      dM_f[l].assign(levels[l].diagM_inv.begin(), levels[l].diagM_inv.end());
    }
  }
  void estimate_all() {
    for (int l = 0; l < (int)levels.size(); ++l) {
      if (levels[l].eig_set) continue;
      if (mg_float) { estimate_eigenvalues<float>(l, 0); estimate_eigenvalues<float>(l, 1); }
      else { estimate_eigenvalues<double>(l, 0); estimate_eigenvalues<double>(l, 1); }
    }
  }

  // -------- outer (FP64) operators on the finest level
  void stokes_vmult(const double* x, double* y) {
    ActiveTable at(*this);
    OuterTerms ot(*this);
    Level& F = fine();
    apply<double>((int)levels.size() - 1, OP_STOKES, x, x + F.n_u, y, y + F.n_u, F.eta.data());
  }
  void a_vmult(const double* x, double* y) {
    ActiveTable at(*this);
    OuterTerms ot(*this);
    apply<double>((int)levels.size() - 1, OP_A, x, nullptr, y, nullptr, fine().eta.data());
  }
  void mass_vmult(const double* x, double* y) {
    ActiveTable at(*this);
    apply<double>((int)levels.size() - 1, OP_MASS, nullptr, x, nullptr, y, fine().eta.data());
  }
  void bt_vmult(const double* xp, double* yu) {
    ActiveTable at(*this);
    apply<double>((int)levels.size() - 1, OP_BT, nullptr, xp, yu, nullptr, fine().eta.data());
  }

  static double dot(const std::vector<double>& a, const std::vector<double>& b) {
    return dot_n(a.data(), b.data(), (long)a.size());
  }
  static double dotp(const double* a, const double* b, int n) { return dot_n(a, b, n); }

  // preconditioned CG (expensive inner solves), returns iterations
  template <class Mat, class Prec>
  int cg(Mat mat, Prec prec, int n, double* x, const double* b, double tol, int maxit) {
    std::vector<double> r(n), z(n), p(n), Ap(n);
    std::fill(x, x + n, 0.0);
    std::copy(b, b + n, r.begin());
    double rn = std::sqrt(dotp(r.data(), r.data(), n));
    if (rn <= tol) return 0;
    prec(r.data(), z.data());
    p = z;
    double rz = dotp(r.data(), z.data(), n);
    for (int it = 1; it <= maxit; ++it) {
      mat(p.data(), Ap.data());
      double alpha = rz / dotp(p.data(), Ap.data(), n);
      for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
      rn = std::sqrt(dotp(r.data(), r.data(), n));
      if (rn <= tol) return it;
      prec(r.data(), z.data());
      double rz2 = dotp(r.data(), z.data(), n);
      double beta = rz2 / rz;
      rz = rz2;
      for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    throw std::runtime_error("inner CG did not converge");
  }

  int nA = 0, nS = 0;
  // BlockSchurPreconditioner::vmult (block_stokes_preconditioner.h:220-255)
  void block_prec(const double* src, double* dst, bool expensive, const Params& P) {
    Level& F = fine();
    const int nu = F.n_u, np = F.n_p;
    // dst_p = -S^-1 src_p
    if (!expensive) {
      vcycle(1, src + nu, dst + nu);
      nS += 1;
    } else {
      double sn = std::sqrt(dotp(src + nu, src + nu, np));
      std::fill(dst + nu, dst + nu + np, 0.0);
      if (sn > 1e-50)
        nS += cg([&](const double* a, double* b) { mass_vmult(a, b); },
                 [&](const double* a, double* b) { vcycle(1, a, b); }, np, dst + nu, src + nu,
                 sn * P.tol_S, 100);
    }
    for (int i = 0; i < np; ++i) dst[nu + i] = -dst[nu + i];
    std::vector<double> t(nu);
    bt_vmult(dst + nu, t.data());
    for (int i = 0; i < nu; ++i) t[i] = src[i] - t[i];
    if (!expensive) {
      vcycle(0, t.data(), dst);
      nA += 1;
    } else {
      double tn = std::sqrt(dotp(t.data(), t.data(), nu));
      nA += cg([&](const double* a, double* b) { a_vmult(a, b); },
               [&](const double* a, double* b) { vcycle(0, a, b); }, nu, dst, t.data(),
               tn * P.tol_A, 10000);
    }
  }

  // GMRES (right preconditioning) and FGMRES; returns iterations, sets converged
  int gmres(double* x, const double* b, double tol, int maxit, int restart, bool flexible,
            bool expensive, const Params& P, bool& converged, double& final_res) {
    Level& F = fine();
    const int n = F.n_u + F.n_p;
    std::vector<std::vector<double>> V, Z;
    std::vector<double> r(n), w(n), tmp(n);
    int it = 0;
    converged = false;
    while (true) {
      stokes_vmult(x, tmp.data());
      for (int i = 0; i < n; ++i) r[i] = b[i] - tmp[i];
      double beta = std::sqrt(dot(r, r));
      final_res = beta;
      if (beta <= tol) { converged = true; return it; }
      if (it >= maxit) return it;
      V.assign(1, r);
      for (double& v : V[0]) v /= beta;
      Z.clear();
      std::vector<std::vector<double>> H;
      std::vector<double> cs, sn, g(1, beta);
      int j = 0;
      for (; j < restart && it < maxit; ++j) {
        std::vector<double> z(n);
        block_prec(V[j].data(), z.data(), expensive, P);
        stokes_vmult(z.data(), w.data());
        if (flexible) Z.push_back(z);
        ++it;
        std::vector<double> h(j + 2, 0.0);
        // classical Gram-Schmidt with one conditional re-orthogonalisation
        double norm_before = std::sqrt(dot(w, w));
        for (int pass = 0; pass < 2; ++pass) {
          std::vector<double> hh(j + 1);
          for (int i = 0; i <= j; ++i) hh[i] = dot(w, V[i]);
#pragma omp parallel for schedule(static) if (g_fast)
          for (int k = 0; k < n; ++k) {
            double t = w[k];
            for (int i = 0; i <= j; ++i) t -= hh[i] * V[i][k];
            w[k] = t;
          }
          for (int i = 0; i <= j; ++i) h[i] += hh[i];
          double nw = std::sqrt(dot(w, w));
          if (pass == 0 && nw > 0.7 * norm_before) break;
        }
        h[j + 1] = std::sqrt(dot(w, w));
        for (int i = 0; i < j; ++i) {
          double t = cs[i] * h[i] + sn[i] * h[i + 1];
          h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
          h[i] = t;
        }
        double den = std::hypot(h[j], h[j + 1]);
        double c_ = h[j] / den, s_ = h[j + 1] / den;
        cs.push_back(c_); sn.push_back(s_);
        h[j] = den; h[j + 1] = 0;
        g.push_back(-s_ * g[j]);
        g[j] = c_ * g[j];
        H.push_back(h);
        std::vector<double> vn(w);
        double hn = std::sqrt(dot(w, w));
        for (double& v : vn) v /= (hn > 0 ? hn : 1.0);
        V.push_back(vn);
        final_res = std::fabs(g[j + 1]);
        if (final_res <= tol) { ++j; break; }
      }
      // solve H y = g
      int m = j;
      std::vector<double> y(m);
      for (int i = m - 1; i >= 0; --i) {
        double t = g[i];
        for (int k = i + 1; k < m; ++k) t -= H[k][i] * y[k];
        y[i] = t / H[i][i];
      }
      if (flexible) {
#pragma omp parallel for schedule(static) if (g_fast)
        for (int k = 0; k < n; ++k) {
          double t = x[k];
          for (int i = 0; i < m; ++i) t += y[i] * Z[i][k];
          x[k] = t;
        }
      } else {
#pragma omp parallel for schedule(static) if (g_fast)
        for (int k = 0; k < n; ++k) {
          double t = 0.0;
          for (int i = 0; i < m; ++i) t += y[i] * V[i][k];
          tmp[k] = t;
        }
        std::vector<double> z(n);
        block_prec(tmp.data(), z.data(), expensive, P);
        for (int k = 0; k < n; ++k) x[k] += z[k];
      }
      if (final_res <= tol) {
        // report the true residual of the final iterate
        stokes_vmult(x, tmp.data());
        for (int i = 0; i < n; ++i) r[i] = b[i] - tmp[i];
        final_res = std::sqrt(dot(r, r));
        converged = true;
        return it;
      }
    }
  }

  // IDR(s) shadow space: s vectors, entries uniform in [-1, 1) from a SplitMix64
  // stream per vector (seed + i), orthonormalised by modified Gram-Schmidt.
  static uint64_t splitmix64_next(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  static std::vector<std::vector<double>> idr_shadow_space(int n, int s, uint64_t seed) {
    std::vector<std::vector<double>> P(s, std::vector<double>(n));
    for (int i = 0; i < s; ++i) {
      uint64_t st = seed + (uint64_t)i;
      std::vector<double>& p = P[i];
      for (int k = 0; k < n; ++k) p[k] = 2.0 * ((double)(splitmix64_next(st) >> 11) * 0x1.0p-53) - 1.0;
      for (int j = 0; j < i; ++j) {
        double d = 0;
        for (int k = 0; k < n; ++k) d += p[k] * P[j][k];
        for (int k = 0; k < n; ++k) p[k] -= d * P[j][k];
      }
      double nn = 0;
      for (int k = 0; k < n; ++k) nn += p[k] * p[k];
      nn = std::sqrt(nn);
      for (int k = 0; k < n; ++k) p[k] /= nn;
    }
    return P;
  }

  // IDR(s) with bi-orthogonalisation and right preconditioning, restated from
  // van Gijzen and Sonneveld, "Algorithm 913: An elegant IDR(s) variant that
  // efficiently exploits biorthogonality properties", ACM TOMS 38 (2011): the
  // method the reference selects with "Krylov method for cheap solver steps =
  // IDR(s)" (stokes_matrix_free_local_smoothing.cc:1290-1299; deal.II SolverIDR,
  // not vendored). Iterations count outer steps (s + 1 preconditioner
  // applications each); convergence is checked after every residual update;
  // omega = (t, r) / (t, t). Ends on the true residual, restarting if needed.
  int idr(double* x, const double* b, double tol, int maxit, const Params& P, bool& converged, double& final_res) {
    Level& F = fine();
    const int n = F.n_u + F.n_p, s = P.idr_s;
    if (s < 1) throw std::runtime_error("IDR(s) parameter must be >= 1");
    const std::vector<std::vector<double>> Pm = idr_shadow_space(n, s, 20261204ull);
    std::vector<double> r(n), v(n), t(n), tmp(n);
    int it = 0;
    converged = false;
    while (true) {
      stokes_vmult(x, t.data());
      for (int i = 0; i < n; ++i) r[i] = b[i] - t[i];
      double normr = std::sqrt(dot(r, r));
      final_res = normr;
      if (normr <= tol) { converged = true; return it; }
      if (it >= maxit) return it;
      std::vector<std::vector<double>> G(s, std::vector<double>(n, 0.0)), U(s, std::vector<double>(n, 0.0));
      std::vector<double> M((size_t)s * s, 0.0);
      for (int i = 0; i < s; ++i) M[(size_t)i * s + i] = 1.0;
      double om = 1.0;
      bool inner_conv = false;
      while (it < maxit && !inner_conv) {
        ++it;
        std::vector<double> f(s);
        for (int i = 0; i < s; ++i) f[i] = dot(r, Pm[i]);
        for (int k = 0; k < s && !inner_conv; ++k) {
          std::vector<double> c(s - k);
          for (int i = k; i < s; ++i) {
            double acc = f[i];
            for (int l = k; l < i; ++l) acc -= M[(size_t)i * s + l] * c[l - k];
            c[i - k] = acc / M[(size_t)i * s + i];
          }
          for (int q = 0; q < n; ++q) {
            double a = r[q];
            for (int i = k; i < s; ++i) a -= c[i - k] * G[i][q];
            tmp[q] = a;
          }
          block_prec(tmp.data(), v.data(), false, P);
          for (int q = 0; q < n; ++q) {
            double a = om * v[q];
            for (int i = k; i < s; ++i) a += c[i - k] * U[i][q];
            tmp[q] = a;
          }
          U[k] = tmp;
          stokes_vmult(U[k].data(), G[k].data());
          for (int i = 0; i < k; ++i) {
            const double alpha = dot(Pm[i], G[k]) / M[(size_t)i * s + i];
            for (int q = 0; q < n; ++q) {
              G[k][q] -= alpha * G[i][q];
              U[k][q] -= alpha * U[i][q];
            }
          }
          for (int i = k; i < s; ++i) M[(size_t)i * s + k] = dot(G[k], Pm[i]);
          const double mkk = M[(size_t)k * s + k];
          if (mkk == 0.0 || !std::isfinite(mkk)) throw std::runtime_error("IDR(s) breakdown");
          const double beta = f[k] / mkk;
          for (int q = 0; q < n; ++q) {
            r[q] -= beta * G[k][q];
            x[q] += beta * U[k][q];
          }
          normr = std::sqrt(dot(r, r));
          final_res = normr;
          if (normr <= tol) { inner_conv = true; break; }
          for (int i = k + 1; i < s; ++i) f[i] -= beta * M[(size_t)i * s + k];
        }
        if (inner_conv) break;
        block_prec(r.data(), v.data(), false, P);
        stokes_vmult(v.data(), t.data());
        const double tt = dot(t, t);
        if (!(tt > 0) || !std::isfinite(tt)) throw std::runtime_error("IDR(s) breakdown");
        om = dot(t, r) / tt;
        for (int q = 0; q < n; ++q) {
          x[q] += om * v[q];
          r[q] -= om * t[q];
        }
        normr = std::sqrt(dot(r, r));
        final_res = normr;
        if (normr <= tol) inner_conv = true;
      }
    }
  }

  // StokesMatrixFreeHandler::solve (scaled pressure unknown p/s in and out)
  void solve(const double* rhs, double* sol, const Params& P, Outputs& out) {
    Level& F = fine();
    const int nu = F.n_u, np = F.n_p, n = nu + np;
    std::vector<double> x(sol, sol + n), t(n), z(n);
    for (int g = 0; g < nu; ++g) if (F.cu.constrained(g)) x[g] = 0;
    for (int g = 0; g < np; ++g) if (F.cp.constrained(g)) x[nu + g] = 0;
    estimate_all();
    stokes_vmult(x.data(), t.data());
    double r2 = 0;
    for (int i = 0; i < n; ++i) r2 += (rhs[i] - t[i]) * (rhs[i] - t[i]);
    out.initial_nonlinear_residual = std::sqrt(r2);
    std::copy(x.begin(), x.end(), z.begin());
    std::fill(z.begin(), z.begin() + nu, 0.0);
    stokes_vmult(z.data(), t.data());
    double ru = 0, rp = 0;
    for (int i = 0; i < nu; ++i) ru += (rhs[i] - t[i]) * (rhs[i] - t[i]);
    for (int i = 0; i < np; ++i) rp += rhs[nu + i] * rhs[nu + i];
    double tol = P.abs_tol > 0 ? P.abs_tol : P.tol_rel * std::sqrt(ru + rp);
    out.solver_tolerance = tol;
    nA = nS = 0;
    bool conv = false;
    double fr = 0;
    out.cheap_iterations = out.expensive_iterations = 0;
    if (P.n_cheap > 0 && P.krylov == 2)
      out.cheap_iterations = idr(x.data(), rhs, tol, P.n_cheap, P, conv, fr);
    else if (P.n_cheap > 0)
      out.cheap_iterations = gmres(x.data(), rhs, tol, P.n_cheap, P.restart, false, false, P, conv, fr);
    if (!conv && P.n_expensive > 0) {
      out.expensive_iterations = gmres(x.data(), rhs, tol, P.n_expensive, P.restart, true, true, P, conv, fr);
    }
    out.final_linear_residual = fr;
    out.A_prec_applications = nA;
    out.S_prec_applications = nS;
    out.status = conv ? 0 : 1;
    std::copy(x.begin(), x.end(), sol);
  }
};

template <> const double* Oracle::eta_table<double>(int lev) { return levels[lev].eta.data(); }
template <> const float* Oracle::eta_table<float>(int lev) { return eta_f[lev].data(); }
template <> const double* Oracle::dinv_table<double>(int lev, int block) {
  return block == 0 ? levels[lev].diagA_inv.data() : levels[lev].diagM_inv.data();
}
template <> const float* Oracle::dinv_table<float>(int lev, int block) {
  return block == 0 ? dA_f[lev].data() : dM_f[lev].data();
}

}  // namespace orc

// ---------------------------------------------------------------- C API
using orc::Oracle;
#define GUARD(...)                          \
  try { __VA_ARGS__; return 0; }            \
  catch (const std::exception& e) { h->err = e.what(); return 1; }

extern "C" {

void* orc_create(int dim, int n_levels) {
  Oracle* h = new Oracle();
  h->dim = dim;
  h->fe.init(dim);
  h->levels.resize(n_levels);
  for (auto& L : h->levels) L.dim = dim;
  return h;
}
// velocity degree 2 (Q2-Q1) or 3 (Q3-Q2)
void* orc_create_degree(int dim, int degree, int n_levels) {
  if (degree != 2 && degree != 3) return nullptr;
  Oracle* h = new Oracle();
  h->dim = dim;
  h->fe.init(dim, degree);
  h->levels.resize(n_levels);
  for (auto& L : h->levels) L.dim = dim;
  return h;
}
void orc_destroy(void* p) { delete (Oracle*)p; }
const char* orc_last_error(void* p) { return ((Oracle*)p)->err.c_str(); }
// Newton / prescribed-dilation tables of the finest level (caller cell order, per
// QGauss(3) point; symmetric tensors as deal.II unrolls them). flags: bit 0 Newton
// derivatives, bit 1 symmetrize, bit 2 average Newton factors, bit 3 prescribed
// dilation. Null arrays: not used by the flags set.
int orc_set_newton(void* p, int flags, const double* E, const double* D, const double* dp, const double* lhs,
                   const double* DD, const double* dpd) {
  Oracle* h = (Oracle*)p;
  GUARD({
    orc::NewtonTerms& t = h->newton;
    const auto& F = h->levels.back();
    const size_t nq = (size_t)F.n_cells * h->fe.nq, ns = h->dim == 3 ? 6 : 3;
    t = orc::NewtonTerms{};
    t.newton = flags & 1;
    t.symmetrize = flags & 2;
    t.average = flags & 4;
    t.dilation = flags & 8;
    if (t.newton) {
      if (!E || !D || !dp) throw std::runtime_error("Newton terms need E, D and dp");
      t.E.assign(E, E + nq * ns);
      t.D.assign(D, D + nq * ns);
      t.dp.assign(dp, dp + nq);
    }
    if (t.dilation) {
      if (!lhs) throw std::runtime_error("a prescribed dilation needs its lhs table");
      t.lhs.assign(lhs, lhs + nq);
      if (t.newton) {
        if (!DD || !dpd) throw std::runtime_error("Newton terms with a dilation need DD and dpd");
        t.DD.assign(DD, DD + nq * ns);
        t.dpd.assign(dpd, dpd + nq);
      }
    }
  })
}

// Free-surface faces of the finest level's outer Stokes operator: caller cell,
// face number 2*d + side, per face point T[dim] then n JxW[dim]. n = 0 removes them.
int orc_set_free_surface(void* p, int n, const int* cell, const int* fno, const double* tab) {
  Oracle* h = (Oracle*)p;
  GUARD({
    const int nf = h->dim == 3 ? 9 : 3;
    h->fs = orc::Oracle::FreeSurface{};
    if (n > 0 && h->fe.degree != 2) throw std::runtime_error("free-surface faces are built for velocity degree 2");
    if (n > 0) {
      h->fs.cell.assign(cell, cell + n);
      h->fs.fno.assign(fno, fno + n);
      h->fs.tab.assign(tab, tab + (size_t)n * nf * 2 * h->dim);
    }
  })
}

// 1: sum-factorised cell operators and parallel reductions (CPU baseline timing);
// 0 (default): the checker's plain quadrature loops and serial reductions
int orc_set_fast(int on) {
  orc::g_fast = on != 0;
  return 0;
}
int orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int orc_set_level_mesh(void* p, int lev, int n_cells, const int* cdu, const int* cdp, int geom_kind,
                       const double* geom, int n_u, int n_p) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& L = h->levels.at(lev);
    L.n_cells = n_cells; L.n_u = n_u; L.n_p = n_p;
    L.cdu.assign(cdu, cdu + (size_t)n_cells * h->fe.nu);
    L.cdp.assign(cdp, cdp + (size_t)n_cells * h->fe.np);
    L.geom_kind = geom_kind;
    size_t ng = geom_kind == 0   ? (size_t)n_cells * 2 * h->dim
                : geom_kind == 1 ? (size_t)n_cells * h->fe.nm * h->dim
                                 : (size_t)n_cells * h->fe.nq * (h->dim * h->dim + 1);
    L.geom.assign(geom, geom + ng);
    L.cu.init(n_u); L.cp.init(n_p);
    orc::compute_geometry(L, h->fe);
  })
}
int orc_set_level_constraints(void* p, int lev, int block, int n_lines, const int* rows, const int* ptr,
                              const int* cols, const double* w, const double* inhom) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& L = h->levels.at(lev);
    if (block == 0) L.cu.set(L.n_u, n_lines, rows, ptr, cols, w, inhom);
    else L.cp.set(L.n_p, n_lines, rows, ptr, cols, w, inhom);
  })
}
int orc_set_transfer(void* p, int lev, const int* parent, const unsigned char* child) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& L = h->levels.at(lev);
    L.parent.assign(parent, parent + L.n_cells);
    L.child.assign(child, child + L.n_cells);
  })
}
// Call after all meshes/constraints/transfers are set.
int orc_finalize(void* p) {
  Oracle* h = (Oracle*)p;
  GUARD({
    for (auto& L : h->levels) orc::colour_cells(L, h->fe);
    for (int l = 1; l < (int)h->levels.size(); ++l) h->build_transfer(l);
  })
}
int orc_set_viscosity(void* p, const double* eta, int n_per_cell, int projection, double s, int compressible,
                      int mg_finest_projected) {
  Oracle* h = (Oracle*)p;
  GUARD(h->set_viscosity(eta, n_per_cell, projection, s, compressible, mg_finest_projected != 0))
}
int orc_get_level_viscosity(void* p, int lev, double* out, int* n_per_cell) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& L = h->levels.at(lev);
    std::copy(L.eta.begin(), L.eta.end(), out);
    *n_per_cell = L.eta_n;
  })
}
int orc_build_preconditioner(void* p, int mg_float) {
  Oracle* h = (Oracle*)p;
  GUARD(h->build_preconditioner(mg_float != 0))
}
// op: 0 Stokes (src/dst = [u;p]), 1 A (u), 2 BT (p -> u), 3 mass (p)
int orc_vmult(void* p, int op, int lev, int use_float, const double* src, double* dst) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& L = h->levels.at(lev);
    int nin = op == 0 ? L.n_u + L.n_p : (op == 1 ? L.n_u : L.n_p);
    int nout = op == 0 ? L.n_u + L.n_p : (op == 3 ? L.n_p : L.n_u);
    const double* su = op == 0 || op == 1 ? src : nullptr;
    const double* sp = op == 0 ? src + L.n_u : (op >= 2 ? src : nullptr);
    // the Stokes operator of the finest level is the outer one (per-point table
    // without averaging, Newton / dilation terms); everything else the multigrid's
    const bool outer = op == 0 && lev == (int)h->levels.size() - 1;
    std::unique_ptr<orc::Oracle::ActiveTable> at(outer ? new orc::Oracle::ActiveTable(*h) : nullptr);
    std::unique_ptr<orc::Oracle::OuterTerms> ot(outer ? new orc::Oracle::OuterTerms(*h) : nullptr);
    if (!use_float) {
      double* du = op == 3 ? nullptr : dst;
      double* dp = op == 0 ? dst + L.n_u : (op == 3 ? dst : nullptr);
      h->apply<double>(lev, op, su, sp, du, dp, L.eta.data());
    } else {
      std::vector<float> s32(src, src + nin), d32(nout);
      const float* fu = su ? s32.data() : nullptr;
      const float* fp = op == 0 ? s32.data() + L.n_u : (op >= 2 ? s32.data() : nullptr);
      float* du = op == 3 ? nullptr : d32.data();
      float* dp = op == 0 ? d32.data() + L.n_u : (op == 3 ? d32.data() : nullptr);
      h->apply<float>(lev, op, fu, fp, du, dp, h->eta_f[lev].data());
      for (int i = 0; i < nout; ++i) dst[i] = d32[i];
    }
  })
}
int orc_get_diagonal(void* p, int lev, int block, double* out) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& v = block == 0 ? h->levels.at(lev).diagA_inv : h->levels.at(lev).diagM_inv;
    std::copy(v.begin(), v.end(), out);
  })
}
int orc_transfer(void* p, int lev, int block, int restrict_, const double* src, double* dst) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& F = h->levels.at(lev);
    auto& C = h->levels.at(lev - 1);
    int nf = block == 0 ? F.n_u : F.n_p, nc = block == 0 ? C.n_u : C.n_p;
    if (restrict_) { std::fill(dst, dst + nc, 0.0); h->restrict_add<double>(lev, block, src, dst); }
    else { std::fill(dst, dst + nf, 0.0); h->prolongate_add<double>(lev, block, src, dst); }
  })
}
int orc_estimate_eigenvalues(void* p) {
  Oracle* h = (Oracle*)p;
  GUARD(h->estimate_all())
}
int orc_get_eigenvalues(void* p, int lev, int block, double* minmax) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& L = h->levels.at(lev);
    double* e = block == 0 ? L.eigA : L.eigM;
    minmax[0] = e[0]; minmax[1] = e[1];
  })
}
int orc_set_eigenvalues(void* p, int lev, int block, const double* minmax) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& L = h->levels.at(lev);
    double* e = block == 0 ? L.eigA : L.eigM;
    e[0] = minmax[0]; e[1] = minmax[1];
    L.eig_set = true;
  })
}
int orc_vcycle(void* p, int block, const double* src, double* dst) {
  Oracle* h = (Oracle*)p;
  GUARD({ h->estimate_all(); h->vcycle(block, src, dst); })
}
int orc_block_preconditioner(void* p, int expensive, const double* src, double* dst) {
  Oracle* h = (Oracle*)p;
  GUARD({ h->estimate_all(); orc::Params P; h->block_prec(src, dst, expensive != 0, P); })
}
// FP64 CPU adjoint gradient: g_c = -int_c 2 eta eps(u) : eps(lambda) (deviatoric
// strain if compressible), the derivative of lambda . (F - K u) w.r.t. ln(eta_c).
int orc_adjoint_gradient(void* p, const double* u, const double* lam, double* grad) {
  Oracle* h = (Oracle*)p;
  GUARD({
    auto& L = h->fine();
    const auto& fe = h->fe;
    const int d = L.dim, nq = fe.nq, nv = fe.nv, nu = fe.nu;
    if (fe.degree != 2) throw std::runtime_error("the adjoint gradient is built for velocity degree 2");
    for (int c = 0; c < L.n_cells; ++c) {
      double xu[81], xl[81];
      for (int i = 0; i < nu; ++i) {
        orc::Expansion e = orc::expand(L.cu, L.cdu[(size_t)c * nu + i]);
        double a = 0, b = 0;
        for (int m = 0; m < e.n; ++m) { a += e.w[m] * u[e.g[m]]; b += e.w[m] * lam[e.g[m]]; }
        xu[i] = a; xl[i] = b;
      }
      double acc = 0;
      for (int q = 0; q < nq; ++q) {
        const double* iJ = &L.invJ[((size_t)c * nq + q) * d * d];
        double Gu[3][3] = {{0}}, Gl[3][3] = {{0}};
        for (int n = 0; n < nv; ++n)
          for (int e = 0; e < d; ++e) {
            double gp = 0;
            for (int a = 0; a < d; ++a) gp += fe.vgrad[(q * nv + n) * d + a] * iJ[a * d + e];
            for (int cc = 0; cc < d; ++cc) { Gu[cc][e] += xu[cc * nv + n] * gp; Gl[cc][e] += xl[cc * nv + n] * gp; }
          }
        double eta = L.eta[(size_t)c * L.eta_n + (L.eta_n == 1 ? 0 : q)];
        double t = 0, du = 0, dl = 0;
        for (int a = 0; a < d; ++a) {
          du += Gu[a][a]; dl += Gl[a][a];
          for (int b = 0; b < d; ++b) t += 0.25 * (Gu[a][b] + Gu[b][a]) * (Gl[a][b] + Gl[b][a]);
        }
        if (h->compressible) t -= du * dl / 3.0;
        acc += 2.0 * eta * L.JxW[(size_t)c * nq + q] * t;
      }
      grad[c] = -acc;
    }
  })
}

// params: [tol_rel, abs_tol, n_cheap, n_expensive, restart, tol_A, tol_S, krylov, idr_s]
// outputs: [initial_res, final_res, tolerance, cheap_its, expensive_its, nA, nS, status]
int orc_solve(void* p, const double* params, const double* rhs, double* sol, double* outputs) {
  Oracle* h = (Oracle*)p;
  GUARD({
    orc::Params P;
    P.tol_rel = params[0]; P.abs_tol = params[1]; P.n_cheap = (int)params[2];
    P.n_expensive = (int)params[3]; P.restart = (int)params[4]; P.tol_A = params[5]; P.tol_S = params[6];
    P.krylov = (int)params[7]; P.idr_s = (int)params[8];
    orc::Outputs o;
    h->solve(rhs, sol, P, o);
    outputs[0] = o.initial_nonlinear_residual; outputs[1] = o.final_linear_residual;
    outputs[2] = o.solver_tolerance; outputs[3] = o.cheap_iterations; outputs[4] = o.expensive_iterations;
    outputs[5] = o.A_prec_applications; outputs[6] = o.S_prec_applications; outputs[7] = o.status;
  })
}

}  // extern "C"
