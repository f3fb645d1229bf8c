// Level set-up on the host: internal layout, colouring, constraint encoding,
// geometry tables, diagonal probes, transfer operators and viscosity tables.
//
// A level whose cells are equal axis-aligned boxes filling a lattice, with
// velocity constraints that are whole (face, component) Dirichlet sets, is
// renumbered lexicographically with the velocity components blocked; its cell
// kernels then compute every index and constraint from the cell's lattice
// position and read no index arrays at all. Every other level keeps the
// caller's numbering and uses index arrays with encoded constraint lines.
#include <algorithm>
#include <cmath>
#include <map>
#include <set>

#include "level.cuh"

namespace gb {

Expansion expand(const HostCons& c, int g) {
  Expansion e;
  const int l = c.line_of[g];
  if (l < 0) {
    e.n = 1;
    e.g[0] = g;
    e.w[0] = 1.0;
    return e;
  }
  e.n = c.ptr[l + 1] - c.ptr[l];
  GB_CHECK(e.n <= 16, 1, "constraint line with more than 16 entries");
  for (int k = 0; k < e.n; ++k) {
    e.g[k] = c.cols[c.ptr[l] + k];
    e.w[k] = c.w[c.ptr[l] + k];
  }
  return e;
}

Csr Csr::transpose(long n_cols) const {
  Csr t;
  t.ptr.assign(n_cols + 1, 0);
  for (int c : col) t.ptr[c + 1]++;
  for (long i = 0; i < n_cols; ++i) t.ptr[i + 1] += t.ptr[i];
  t.col.resize(col.size());
  t.val.resize(val.size());
  std::vector<int> fill(t.ptr.begin(), t.ptr.end() - 1);
  for (long r = 0; r < rows(); ++r)
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
      const int c = col[k];
      t.col[fill[c]] = (int)r;
      t.val[fill[c]] = val[k];
      ++fill[c];
    }
  return t;
}

Basis1D basis1d(int degree) {
  Basis1D b;
  b.deg = degree;
  b.nvn = degree + 1;
  b.npn = degree;
  b.nq1 = degree + 1;
  if (degree == 2) {
    const double vn[3] = {0.0, 0.5, 1.0}, g[3] = {0.5 - std::sqrt(15.0) / 10, 0.5, 0.5 + std::sqrt(15.0) / 10};
    const double w[3] = {5.0 / 18, 8.0 / 18, 5.0 / 18};
    for (int i = 0; i < 3; ++i) { b.vn[i] = vn[i]; b.gq[i] = g[i]; b.gw[i] = w[i]; }
    b.pn[0] = 0.0;
    b.pn[1] = 1.0;
  } else {
    // Gauss-Lobatto nodes of 4 points: 0, (1 -+ 1/sqrt 5) / 2, 1; Gauss-Legendre
    // of 4 points: (1 -+ sqrt(3/7 +- 2/7 sqrt(6/5))) / 2, weights (18 -+ sqrt 30) / 72
    const double a = 0.5 / std::sqrt(5.0);
    const double vn[4] = {0.0, 0.5 - a, 0.5 + a, 1.0};
    const double t1 = std::sqrt(3.0 / 7 - 2.0 / 7 * std::sqrt(6.0 / 5)), t2 = std::sqrt(3.0 / 7 + 2.0 / 7 * std::sqrt(6.0 / 5));
    const double g[4] = {0.5 - 0.5 * t2, 0.5 - 0.5 * t1, 0.5 + 0.5 * t1, 0.5 + 0.5 * t2};
    const double wi = (18.0 + std::sqrt(30.0)) / 72, wo = (18.0 - std::sqrt(30.0)) / 72;
    const double w[4] = {wo, wi, wi, wo};
    for (int i = 0; i < 4; ++i) { b.vn[i] = vn[i]; b.gq[i] = g[i]; b.gw[i] = w[i]; }
    b.pn[0] = 0.0;
    b.pn[1] = 0.5;
    b.pn[2] = 1.0;
  }
  return b;
}

void lagrange_basis(const double* nodes, int n, double x, double* val, double* der) {
  for (int i = 0; i < n; ++i) {
    double v = 1, d = 0, den = 1;
    for (int m = 0; m < n; ++m)
      if (m != i) den *= nodes[i] - nodes[m];
    for (int m = 0; m < n; ++m) {
      if (m == i) continue;
      double t = 1;
      for (int k = 0; k < n; ++k)
        if (k != i && k != m) t *= x - nodes[k];
      d += t;
      v *= x - nodes[m];
    }
    val[i] = v / den;
    der[i] = d / den;
  }
}

namespace {

int nv_of(const Level& L) { return L.nv(); }
int np_of(const Level& L) { return L.np(); }

// ---------------------------------------------------------------- 1D basis (host)
void lagrange(const double* nodes, int n, double x, double* val, double* der) {
  for (int i = 0; i < n; ++i) {
    double v = 1, d = 0, den = 1;
    for (int m = 0; m < n; ++m)
      if (m != i) den *= nodes[i] - nodes[m];
    for (int m = 0; m < n; ++m) {
      if (m == i) continue;
      double t = 1;
      for (int k = 0; k < n; ++k)
        if (k != i && k != m) t *= x - nodes[k];
      d += t;
      v *= x - nodes[m];
    }
    val[i] = v / den;
    der[i] = d / den;
  }
}

// ---------------------------------------------------------------- structure detection
bool detect_structured(Level& L) {
  const int d = L.dim, nv = nv_of(L), np = np_of(L), nu = d * nv;
  // the lattice kernels are Q2-Q1 kernels
  if (L.degree != 2 || L.geom_kind != 0 || L.n_cells == 0) return false;
  // pressure constraints are not part of the lattice fast path
  for (long g = 0; g < L.n_p; ++g)
    if (L.cp.constrained((int)g)) return false;
  double h[3], lo[3], hi[3];
  for (int e = 0; e < d; ++e) {
    h[e] = L.geom[d + e];
    lo[e] = 1e300;
    hi[e] = -1e300;
  }
  for (long c = 0; c < L.n_cells; ++c)
    for (int e = 0; e < d; ++e) {
      const double he = L.geom[c * 2 * d + d + e];
      if (std::fabs(he - h[e]) > 1e-12 * std::fabs(h[e])) return false;
      lo[e] = std::min(lo[e], L.geom[c * 2 * d + e]);
      hi[e] = std::max(hi[e], L.geom[c * 2 * d + e]);
    }
  long total = 1;
  int nc[3] = {1, 1, 1};
  for (int e = 0; e < d; ++e) {
    const double r = (hi[e] - lo[e]) / h[e];
    nc[e] = (int)std::lround(r) + 1;
    if (std::fabs(r - (nc[e] - 1)) > 1e-6) return false;
    total *= nc[e];
  }
  if (total != L.n_cells) return false;
  const int Nn[3] = {2 * nc[0] + 1, 2 * nc[1] + 1, d == 3 ? 2 * nc[2] + 1 : 1};
  const int Np[3] = {nc[0] + 1, nc[1] + 1, d == 3 ? nc[2] + 1 : 1};
  const long n_nodes = (long)Nn[0] * Nn[1] * Nn[2];
  const long n_pnodes = (long)Np[0] * Np[1] * Np[2];
  if (d * n_nodes != L.n_u || n_pnodes != L.n_p) return false;
  std::vector<int> perm_u(L.n_u, -1), perm_p(L.n_p, -1), used_u(L.n_u, 0), used_p(L.n_p, 0);
  std::vector<int> ioc(L.n_cells, -1);
  std::vector<char> cell_seen(L.n_cells, 0);
  for (long c = 0; c < L.n_cells; ++c) {
    int ijk[3] = {0, 0, 0};
    for (int e = 0; e < d; ++e) {
      const double r = (L.geom[c * 2 * d + e] - lo[e]) / h[e];
      ijk[e] = (int)std::lround(r);
      if (std::fabs(r - ijk[e]) > 1e-6) return false;
    }
    const long ic = ((long)ijk[2] * nc[1] + ijk[1]) * nc[0] + ijk[0];
    if (cell_seen[ic]) return false;
    cell_seen[ic] = 1;
    ioc[c] = (int)ic;
    for (int comp = 0; comp < d; ++comp)
      for (int n = 0; n < nv; ++n) {
        const int a = n % 3, b = (n / 3) % 3, cc = n / 9;
        const long node = ((long)(2 * ijk[2] + cc) * Nn[1] + (2 * ijk[1] + b)) * Nn[0] + 2 * ijk[0] + a;
        const long internal = comp * n_nodes + node;
        const int g = L.cdu[c * nu + comp * nv + n];
        if (g < 0 || g >= L.n_u) return false;
        if (perm_u[g] == -1) {
          if (used_u[internal]) return false;
          perm_u[g] = (int)internal;
          used_u[internal] = 1;
        } else if (perm_u[g] != internal) {
          return false;
        }
      }
    for (int n = 0; n < np; ++n) {
      const int a = n & 1, b = (n >> 1) & 1, cc = (n >> 2) & 1;
      const long node = ((long)(ijk[2] + cc) * Np[1] + (ijk[1] + b)) * Np[0] + ijk[0] + a;
      const int g = L.cdp[c * np + n];
      if (g < 0 || g >= L.n_p) return false;
      if (perm_p[g] == -1) {
        if (used_p[node]) return false;
        perm_p[g] = (int)node;
        used_p[node] = 1;
      } else if (perm_p[g] != node) {
        return false;
      }
    }
  }
  // velocity constraints: Dirichlet lines forming whole (face, component) sets
  std::vector<char> cons_internal(L.n_u, 0);
  for (long g = 0; g < L.n_u; ++g) {
    if (!L.cu.constrained((int)g)) continue;
    if (L.cu.n_entries((int)g) != 0) return false;
    cons_internal[perm_u[g]] = 1;
  }
  uint32_t zf = 0;
  for (int e = 0; e < d; ++e)
    for (int side = 0; side < 2; ++side)
      for (int comp = 0; comp < d; ++comp) {
        bool all = true;
        const int fixed = side ? Nn[e] - 1 : 0;
        for (long node = 0; node < n_nodes && all; ++node) {
          const int gi[3] = {(int)(node % Nn[0]), (int)((node / Nn[0]) % Nn[1]), (int)(node / ((long)Nn[0] * Nn[1]))};
          if (gi[e] != fixed) continue;
          if (!cons_internal[comp * n_nodes + node]) all = false;
        }
        if (all) zf |= 1u << ((2 * e + side) * 3 + comp);
      }
  // every constrained DoF must be covered by the face sets and vice versa
  std::vector<int> cons_list;
  for (long node = 0; node < n_nodes; ++node) {
    const int gi[3] = {(int)(node % Nn[0]), (int)((node / Nn[0]) % Nn[1]), (int)(node / ((long)Nn[0] * Nn[1]))};
    for (int comp = 0; comp < d; ++comp) {
      bool z = false;
      for (int e = 0; e < d; ++e) {
        if (gi[e] == 0 && ((zf >> ((2 * e) * 3 + comp)) & 1u)) z = true;
        if (gi[e] == Nn[e] - 1 && ((zf >> ((2 * e + 1) * 3 + comp)) & 1u)) z = true;
      }
      if (z != (bool)cons_internal[comp * n_nodes + node]) return false;
      if (z) cons_list.push_back((int)(comp * n_nodes + node));
    }
  }
  std::sort(cons_list.begin(), cons_list.end());
  // accepted
  L.structured = true;
  for (int e = 0; e < 3; ++e) {
    L.nc[e] = e < d ? nc[e] : 1;
    L.h[e] = e < d ? h[e] : 1.0;
  }
  L.zero_faces = zf;
  L.perm_u = std::move(perm_u);
  L.perm_p = std::move(perm_p);
  L.internal_of_cell = ioc;
  L.cell_of_internal.assign(L.n_cells, 0);
  for (long c = 0; c < L.n_cells; ++c) L.cell_of_internal[ioc[c]] = (int)c;
  L.cons_u = cons_list;
  L.cons_p.clear();
  const int ncol = d == 3 ? 8 : 4;
  L.n_colours = ncol;
  L.colour_begin.assign(ncol, 0);
  L.colour_count.assign(ncol, 0);
  for (int k = 0; k < ncol; ++k) {
    long cnt = 1;
    for (int e = 0; e < d; ++e) cnt *= (nc[e] - ((k >> e) & 1) + 1) / 2;
    L.colour_count[k] = (int)cnt;
  }
  return true;
}

// ---------------------------------------------------------------- general levels
void setup_general(Level& L) {
  const int d = L.dim, nv = nv_of(L), np = np_of(L), nu = d * nv, nq = L.nq();
  L.structured = false;
  L.perm_u.resize(L.n_u);
  L.perm_p.resize(L.n_p);
  for (long i = 0; i < L.n_u; ++i) L.perm_u[i] = (int)i;
  for (long i = 0; i < L.n_p; ++i) L.perm_p[i] = (int)i;
  // greedy colouring on the DoFs each cell writes (after constraint expansion)
  std::vector<std::vector<int>> writes(L.n_cells);
  for (long c = 0; c < L.n_cells; ++c) {
    std::set<int> s;
    for (int i = 0; i < nu; ++i) {
      Expansion e = expand(L.cu, L.cdu[c * nu + i]);
      for (int k = 0; k < e.n; ++k) s.insert(e.g[k]);
    }
    for (int i = 0; i < np; ++i) {
      Expansion e = expand(L.cp, L.cdp[c * np + i]);
      for (int k = 0; k < e.n; ++k) s.insert((int)(L.n_u + e.g[k]));
    }
    writes[c].assign(s.begin(), s.end());
  }
  std::vector<std::vector<int>> cells_of(L.n_u + L.n_p);
  for (long c = 0; c < L.n_cells; ++c)
    for (int g : writes[c]) cells_of[g].push_back((int)c);
  std::vector<int> col(L.n_cells, -1);
  int ncol = 0;
  for (long c = 0; c < L.n_cells; ++c) {
    std::vector<char> used(ncol + 1, 0);
    for (int g : writes[c])
      for (int o : cells_of[g])
        if (col[o] >= 0) used[col[o]] = 1;
    int k = 0;
    while (used[k]) ++k;
    col[c] = k;
    ncol = std::max(ncol, k + 1);
  }
  L.n_colours = ncol;
  L.colour_count.assign(ncol, 0);
  for (long c = 0; c < L.n_cells; ++c) L.colour_count[col[c]]++;
  L.colour_begin.assign(ncol, 0);
  for (int k = 1; k < ncol; ++k) L.colour_begin[k] = L.colour_begin[k - 1] + L.colour_count[k - 1];
  std::vector<int> fill(L.colour_begin);
  L.internal_of_cell.assign(L.n_cells, 0);
  L.cell_of_internal.assign(L.n_cells, 0);
  for (long c = 0; c < L.n_cells; ++c) {
    const int ic = fill[col[c]]++;
    L.internal_of_cell[c] = ic;
    L.cell_of_internal[ic] = (int)c;
  }
  // constraint lines with entries get compact ids; Dirichlet lines become -1
  auto encode_lines = [&](const HostCons& C, long n, std::vector<int>& line_id, std::vector<int>& lptr,
                          std::vector<int>& lcol, std::vector<double>& lw, std::vector<int>& cons) {
    line_id.assign(n, -1);
    lptr.assign(1, 0);
    lcol.clear();
    lw.clear();
    cons.clear();
    for (long g = 0; g < n; ++g) {
      if (!C.constrained((int)g)) continue;
      cons.push_back((int)g);
      const int ne = C.n_entries((int)g);
      if (ne == 0) continue;
      line_id[g] = (int)lptr.size() - 1;
      const int l = C.line_of[g];
      for (int k = C.ptr[l]; k < C.ptr[l + 1]; ++k) {
        GB_CHECK(!C.constrained(C.cols[k]), 1, "constraints are not closed (a master is constrained)");
        lcol.push_back(C.cols[k]);
        lw.push_back(C.w[k]);
      }
      lptr.push_back((int)lcol.size());
    }
  };
  std::vector<int> lid_u, lptr_u, lcol_u, lid_p, lptr_p, lcol_p;
  std::vector<double> lw_u, lw_p;
  encode_lines(L.cu, L.n_u, lid_u, lptr_u, lcol_u, lw_u, L.cons_u);
  encode_lines(L.cp, L.n_p, lid_p, lptr_p, lcol_p, lw_p, L.cons_p);
  auto code = [](const HostCons& C, const std::vector<int>& lid, int g) -> int {
    if (!C.constrained(g)) return g;
    return lid[g] < 0 ? -1 : -(lid[g] + 2);
  };
  std::vector<int> cdu(L.n_cells * nu), cdp(L.n_cells * np);
  for (long c = 0; c < L.n_cells; ++c) {
    const long ic = L.internal_of_cell[c];
    for (int i = 0; i < nu; ++i) cdu[ic * nu + i] = code(L.cu, lid_u, L.cdu[c * nu + i]);
    for (int i = 0; i < np; ++i) cdp[ic * np + i] = code(L.cp, lid_p, L.cdp[c * np + i]);
  }
  L.cdu_d.upload(cdu);
  L.cdp_d.upload(cdp);
  L.lptr_d.upload(lptr_u);
  L.lcol_d.upload(lcol_u);
  L.plptr_d.upload(lptr_p);
  L.plcol_d.upload(lcol_p);
  L.f64.lw.upload(lw_u);
  L.f64.plw.upload(lw_p);
  L.f32.lw.upload(std::vector<float>(lw_u.begin(), lw_u.end()));
  L.f32.plw.upload(std::vector<float>(lw_p.begin(), lw_p.end()));
  // geometry
  if (L.geom_kind == 0) {
    std::vector<double> gb((size_t)L.n_cells * (d + 1));
    for (long c = 0; c < L.n_cells; ++c) {
      const long ic = L.internal_of_cell[c];
      double det = 1;
      for (int e = 0; e < d; ++e) {
        const double he = L.geom[c * 2 * d + d + e];
        gb[ic * (d + 1) + e] = 1.0 / he;
        det *= he;
      }
      gb[ic * (d + 1) + d] = det;
    }
    L.f64.gbox.upload(gb);
    L.f32.gbox.upload(std::vector<float>(gb.begin(), gb.end()));
  } else if (L.geom_kind == 2) {
    // the caller's per-point inverse Jacobians and |det J|, in internal cell order
    const int stride = d * d + 1;
    std::vector<double> gt((size_t)L.n_cells * nq * stride);
    for (long c = 0; c < L.n_cells; ++c) {
      const long ic = L.internal_of_cell[c];
      for (int q = 0; q < nq; ++q) {
        const double* src = &L.geom[((size_t)c * nq + q) * stride];
        GB_CHECK(src[d * d] > 0 && std::isfinite(src[d * d]), 1, "|det J| of a geometry table entry must be positive");
        std::copy(src, src + stride, &gt[((size_t)ic * nq + q) * stride]);
      }
    }
    L.f64.gtab.upload(gt);
    L.f32.gtab.upload(std::vector<float>(gt.begin(), gt.end()));
  } else {
    // Q2 mapping (3^dim support points per cell) at the QGauss(degree+1) points
    const Basis1D B = basis1d(L.degree);
    const double q2n[3] = {0.0, 0.5, 1.0};
    const int nm = ipow(3, d), n1 = B.nq1;
    double v1[4][3], d1[4][3];
    for (int q = 0; q < n1; ++q) lagrange(q2n, 3, B.gq[q], v1[q], d1[q]);
    const int stride = d * d + 1;
    std::vector<double> gt((size_t)L.n_cells * nq * stride);
    for (long c = 0; c < L.n_cells; ++c) {
      const long ic = L.internal_of_cell[c];
      const double* X = &L.geom[(size_t)c * nm * d];
      for (int q = 0; q < nq; ++q) {
        const int qi[3] = {q % n1, (q / n1) % n1, q / (n1 * n1)};
        double J[3][3] = {{0}};
        for (int n = 0; n < nm; ++n) {
          const int ni[3] = {n % 3, (n / 3) % 3, n / 9};
          for (int b = 0; b < d; ++b) {
            double t = 1;
            for (int e = 0; e < d; ++e) t *= (e == b ? d1[qi[e]][ni[e]] : v1[qi[e]][ni[e]]);
            for (int a = 0; a < d; ++a) J[a][b] += X[n * d + a] * t;
          }
        }
        double det, inv[3][3];
        if (d == 2) {
          det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
          inv[0][0] = J[1][1] / det;
          inv[0][1] = -J[0][1] / det;
          inv[1][0] = -J[1][0] / det;
          inv[1][1] = J[0][0] / det;
        } else {
          det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
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
        GB_CHECK(det != 0, 1, "degenerate cell geometry");
        double* o = &gt[((size_t)ic * nq + q) * stride];
        for (int a = 0; a < d; ++a)
          for (int b = 0; b < d; ++b) o[a * d + b] = inv[a][b];
        o[d * d] = std::fabs(det);
      }
    }
    L.f64.gtab.upload(gt);
    L.f32.gtab.upload(std::vector<float>(gt.begin(), gt.end()));
  }
  // pass-2 gather lists: for every DoF, the (cell, local slot, weight) entries
  // that contribute to it, constraint lines folded in; sorted by slot
  auto build_gather = [&](const std::vector<int>& cd, const HostCons& C, int nl, long n, DevBuf<int>& gptr,
                          DevBuf<int>& gslot, DevBuf<double>& gw64, DevBuf<float>& gw32, DevBuf<unsigned char>& cm) {
    std::vector<std::vector<std::pair<long, double>>> ent(n);
    for (long ic = 0; ic < L.n_cells; ++ic) {
      const long c = L.cell_of_internal[ic];
      for (int i = 0; i < nl; ++i) {
        Expansion e = expand(C, cd[c * nl + i]);
        for (int k = 0; k < e.n; ++k) ent[e.g[k]].push_back({ic * nl + i, e.w[k]});
      }
    }
    std::vector<int> ptr(1, 0), slot;
    std::vector<double> w;
    std::vector<unsigned char> mask(n, 0);
    for (long g = 0; g < n; ++g) {
      mask[g] = C.constrained((int)g) ? 1 : 0;
      for (auto& pr : ent[g]) {
        GB_CHECK(pr.first < (1L << 31), 1, "level too large for 32-bit gather slots");
        slot.push_back((int)pr.first);
        w.push_back(pr.second);
      }
      ptr.push_back((int)slot.size());
    }
    gptr.upload(ptr);
    gslot.upload(slot);
    gw64.upload(w);
    gw32.upload(std::vector<float>(w.begin(), w.end()));
    cm.upload(mask);
  };
  build_gather(L.cdu, L.cu, nu, L.n_u, L.gu_ptr, L.gu_slot, L.f64.gu_w, L.f32.gu_w, L.cmask_u);
  build_gather(L.cdp, L.cp, np, L.n_p, L.gp_ptr, L.gp_slot, L.f64.gp_w, L.f32.gp_w, L.cmask_p);
  // diagonal probes: per internal cell, the unconstrained DoFs it touches
  auto build_probes = [&](const std::vector<int>& cd, const HostCons& C, int nl, DevBuf<int>& pptr, DevBuf<int>& pg,
                          DevBuf<int>& peptr, DevBuf<int>& pli, DevBuf<double>& pw64, DevBuf<float>& pw32,
                          std::vector<int>& ptr_h) {
    std::vector<int> ptr(1, 0), g, eptr(1, 0), li;
    std::vector<double> w;
    for (long ic = 0; ic < L.n_cells; ++ic) {
      const long c = L.cell_of_internal[ic];
      std::map<int, std::vector<std::pair<int, double>>> m;
      for (int i = 0; i < nl; ++i) {
        Expansion e = expand(C, cd[c * nl + i]);
        for (int k = 0; k < e.n; ++k) m[e.g[k]].push_back({i, e.w[k]});
      }
      for (auto& kv : m) {
        g.push_back(kv.first);
        for (auto& p : kv.second) {
          li.push_back(p.first);
          w.push_back(p.second);
        }
        eptr.push_back((int)li.size());
      }
      ptr.push_back((int)g.size());
    }
    pptr.upload(ptr);
    ptr_h = ptr;
    pg.upload(g);
    peptr.upload(eptr);
    pli.upload(li);
    pw64.upload(w);
    pw32.upload(std::vector<float>(w.begin(), w.end()));
  };
  build_probes(L.cdu, L.cu, nu, L.probe_ptr, L.probe_g, L.probe_eptr, L.probe_li, L.f64.probe_w, L.f32.probe_w,
               L.probe_ptr_h);
  build_probes(L.cdp, L.cp, np, L.pprobe_ptr, L.pprobe_g, L.pprobe_eptr, L.pprobe_li, L.f64.pprobe_w,
               L.f32.pprobe_w, L.pprobe_ptr_h);
}

}  // namespace

void setup_level(Level& L, bool force_indexed) {
  if (force_indexed || !detect_structured(L)) setup_general(L);
  const int nu = L.dim * nv_of(L), np = np_of(L);
  L.f64.Eu.alloc((size_t)L.n_cells * nu);
  L.f64.Ep.alloc((size_t)L.n_cells * np);
  L.f32.Eu.alloc((size_t)L.n_cells * nu);
  L.f32.Ep.alloc((size_t)L.n_cells * np);
  L.perm_u_d.upload(L.perm_u);
  L.perm_p_d.upload(L.perm_p);
  L.cons_u_d.upload(L.cons_u);
  L.cons_p_d.upload(L.cons_p);
}

// Prolongation from `coarse` to `fine` (rows: fine internal unconstrained DoFs,
// columns: coarse internal DoFs): the coarse FE function, with its constraints
// resolved, evaluated at the fine support points (reference coordinates of the
// child inside its parent). Restriction is the transpose.
// The lattice description of the transfer between two structured levels, if
// the CSR matrix P (rows: fine internal DoFs, columns sorted by coarse internal
// DoF) holds exactly the lattice stencils' entries: the same columns in the
// same order and the same values. Then the matrix-free kernels form the same
// sums as the CSR products.
static bool lattice_transfer_of(const Level& F, const Level& C, int block, const Csr& P, LatticeTransfer& X) {
  if (!F.structured || !C.structured || F.degree != 2 || C.degree != 2 || F.dim != C.dim) return false;
  const int d = F.dim;
  X = LatticeTransfer{};
  X.q2 = block == 0 ? 1 : 0;
  X.ncomp = block == 0 ? d : 1;
  for (int e = 0; e < 3; ++e) {
    if (e < d && F.nc[e] != 2 * C.nc[e]) return false;
    X.Nf[e] = e < d ? (block == 0 ? 2 * F.nc[e] + 1 : F.nc[e] + 1) : 1;
    X.Nc[e] = e < d ? (block == 0 ? 2 * C.nc[e] + 1 : C.nc[e] + 1) : 1;
  }
  X.nf_nodes = (long)X.Nf[0] * X.Nf[1] * X.Nf[2];
  X.nc_nodes = (long)X.Nc[0] * X.Nc[1] * X.Nc[2];
  X.zf_f = block == 0 ? F.zero_faces : 0u;
  X.zf_c = block == 0 ? C.zero_faces : 0u;
  const long nf = X.ncomp * X.nf_nodes;
  if (P.rows() != nf || nf != (block == 0 ? F.n_u : F.n_p) || X.ncomp * X.nc_nodes != (block == 0 ? C.n_u : C.n_p))
    return false;
  for (long r = 0; r < nf; ++r) {
    const int comp = (int)(r / X.nf_nodes);
    const long node = r - (long)comp * X.nf_nodes;
    const int f[3] = {(int)(node % X.Nf[0]), (int)((node / X.Nf[0]) % X.Nf[1]), (int)(node / ((long)X.Nf[0] * X.Nf[1]))};
    int k = P.ptr[r];
    const int e = P.ptr[r + 1];
    if (!(X.q2 && lattice_zero(X.zf_f, X.Nf, comp, f[0], f[1], f[2]))) {
      int c[3][3];
      double w[3][3];
      int m[3];
      for (int a = 0; a < 3; ++a) {
        if (X.Nf[a] > 1) m[a] = lattice_p1d(X.q2, f[a], c[a], w[a]);
        else { m[a] = 1; c[a][0] = 0; w[a][0] = 1.0; }
      }
      for (int z = 0; z < m[2]; ++z)
        for (int y = 0; y < m[1]; ++y)
          for (int x = 0; x < m[0]; ++x) {
            if (X.q2 && lattice_zero(X.zf_c, X.Nc, comp, c[0][x], c[1][y], c[2][z])) continue;
            const long col = (long)comp * X.nc_nodes + ((long)c[2][z] * X.Nc[1] + c[1][y]) * X.Nc[0] + c[0][x];
            const double val = w[0][x] * w[1][y] * w[2][z];
            if (k >= e || P.col[k] != col || P.val[k] != val) return false;
            ++k;
          }
    }
    if (k != e) return false;
  }
  return true;
}

void setup_transfer(Level& F, const Level& C) {
  const int d = F.dim, nv = nv_of(F), np = np_of(F), nu = d * nv;
  GB_CHECK(F.has_transfer, 2, "missing child/parent data for a level");
  const Basis1D B = basis1d(F.degree);
  for (int block = 0; block < 2; ++block) {
    const int n1 = block == 0 ? B.nvn : B.npn;  // nodes per direction
    const double* nodes = block == 0 ? B.vn : B.pn;
    const int nl = block == 0 ? nv : np;
    const int ncomp = block == 0 ? d : 1;
    const long nf = block == 0 ? F.n_u : F.n_p;
    const HostCons& FC = block == 0 ? F.cu : F.cp;
    const HostCons& CC = block == 0 ? C.cu : C.cp;
    const std::vector<int>& fperm = block == 0 ? F.perm_u : F.perm_p;
    const std::vector<int>& cperm = block == 0 ? C.perm_u : C.perm_p;
    // each fine DoF's entries are appended once, contiguously (the DoF is
    // handled when first met), then sorted by internal column and merged below
    std::vector<long> seg_begin(nf, -1);
    std::vector<int> seg_len(nf, 0);
    std::vector<int> ecol;
    std::vector<double> eval;
    ecol.reserve((size_t)nf * 8);
    eval.reserve((size_t)nf * 8);
    std::vector<char> done(nf, 0);
    for (long fc = 0; fc < F.n_cells; ++fc) {
      const int pc = F.parent[fc], ch = F.child[fc];
      GB_CHECK(pc >= 0 && pc < C.n_cells, 1, "parent index out of range");
      for (int n = 0; n < nl; ++n) {
        // a node shared with an earlier cell is done for every component
        bool any = false;
        for (int comp = 0; comp < ncomp && !any; ++comp) {
          const int gf = block == 0 ? F.cdu[fc * nu + comp * nl + n] : F.cdp[fc * np + n];
          any = !FC.constrained(gf) && !done[gf];
        }
        if (!any) continue;
        double xi[3];
        for (int e = 0; e < d; ++e) {
          const int idx = (e == 0 ? n : e == 1 ? n / n1 : n / (n1 * n1)) % n1;
          const double loc = nodes[idx];
          xi[e] = ch == kSameCell ? loc : 0.5 * (((ch >> e) & 1) + loc);
        }
        double phi[64];
        double vv[3][4], dd[3][4];
        for (int e = 0; e < d; ++e) lagrange(nodes, n1, xi[e], vv[e], dd[e]);
        for (int m = 0; m < nl; ++m) {
          double t = 1;
          for (int e = 0; e < d; ++e) t *= vv[e][(e == 0 ? m : e == 1 ? m / n1 : m / (n1 * n1)) % n1];
          phi[m] = t;
        }
        for (int comp = 0; comp < ncomp; ++comp) {
          const int gf = block == 0 ? F.cdu[fc * nu + comp * nl + n] : F.cdp[fc * np + n];
          if (FC.constrained(gf) || done[gf]) continue;
          done[gf] = 1;
          seg_begin[gf] = (long)ecol.size();
          for (int m = 0; m < nl; ++m) {
            if (std::fabs(phi[m]) < 1e-14) continue;
            const int gc = block == 0 ? C.cdu[(long)pc * nu + comp * nl + m] : C.cdp[(long)pc * np + m];
            if (!CC.constrained(gc)) {  // the common case: the DoF itself, weight 1
              ecol.push_back(gc);
              eval.push_back(phi[m] * 1.0);
              continue;
            }
            Expansion e = expand(CC, gc);
            for (int k = 0; k < e.n; ++k) {
              ecol.push_back(e.g[k]);
              eval.push_back(phi[m] * e.w[k]);
            }
          }
          seg_len[gf] = (int)((long)ecol.size() - seg_begin[gf]);
        }
      }
    }
    // internal numbering: rows in internal order, each row's entries sorted by
    // internal column (a stable sort, so repeated columns are summed in the
    // order they were generated), entries of magnitude <= 1e-14 dropped
    std::vector<long> caller_of(nf);
    for (long g = 0; g < nf; ++g) caller_of[fperm[g]] = g;
    Csr P;
    P.col.reserve(ecol.size());
    P.val.reserve(ecol.size());
    std::vector<std::pair<int, double>> row;
    for (long r = 0; r < nf; ++r) {
      const long g = caller_of[r];
      if (seg_begin[g] >= 0) {
        row.clear();
        for (long q = seg_begin[g]; q < seg_begin[g] + seg_len[g]; ++q) row.push_back({cperm[ecol[q]], eval[q]});
        // stable insertion sort (rows hold a few dozen entries)
        for (size_t q = 1; q < row.size(); ++q) {
          const std::pair<int, double> x = row[q];
          size_t z = q;
          for (; z > 0 && row[z - 1].first > x.first; --z) row[z] = row[z - 1];
          row[z] = x;
        }
        for (size_t q = 0; q < row.size();) {
          double v = 0;
          size_t q2 = q;
          for (; q2 < row.size() && row[q2].first == row[q].first; ++q2) v += row[q2].second;
          if (std::fabs(v) > 1e-14) {
            P.col.push_back(row[q].first);
            P.val.push_back(v);
          }
          q = q2;
        }
      }
      P.ptr.push_back((int)P.col.size());
    }
    F.xfer_lattice[block] = lattice_transfer_of(F, C, block, P, F.xfer[block]);
    Csr PT = P.transpose(block == 0 ? C.n_u : C.n_p);
    if (block == 0) {
      F.Pu_ptr.upload(P.ptr); F.Pu_col.upload(P.col); F.Pu_rows = P.rows();
      F.PuT_ptr.upload(PT.ptr); F.PuT_col.upload(PT.col); F.PuT_rows = PT.rows();
      F.f64.Pu_val.upload(P.val); F.f64.PuT_val.upload(PT.val);
      F.f32.Pu_val.upload(std::vector<float>(P.val.begin(), P.val.end()));
      F.f32.PuT_val.upload(std::vector<float>(PT.val.begin(), PT.val.end()));
    } else {
      F.Pp_ptr.upload(P.ptr); F.Pp_col.upload(P.col); F.Pp_rows = P.rows();
      F.PpT_ptr.upload(PT.ptr); F.PpT_col.upload(PT.col); F.PpT_rows = PT.rows();
      F.f64.Pp_val.upload(P.val); F.f64.PpT_val.upload(PT.val);
      F.f32.Pp_val.upload(std::vector<float>(P.val.begin(), P.val.end()));
      F.f32.PpT_val.upload(std::vector<float>(PT.val.begin(), PT.val.end()));
    }
  }
}

template <typename T>
LevelView<T> Level::view(double s, int compressible) {
  LevelView<T> v{};
  LevelDev<T>& D = dev<T>();
  v.dim = dim;
  v.deg = degree;
  v.n_cells = (int)n_cells;
  v.n_u = (int)n_u;
  v.n_p = (int)n_p;
  v.structured = structured ? 1 : 0;
  for (int e = 0; e < 3; ++e) {
    v.nc[e] = nc[e];
    v.Nn[e] = e < dim ? 2 * nc[e] + 1 : 1;
    v.Np[e] = e < dim ? nc[e] + 1 : 1;
    v.inv_h[e] = (T)(1.0 / h[e]);
  }
  double det = 1;
  for (int e = 0; e < dim; ++e) det *= h[e];
  v.det = (T)det;
  v.n_nodes = v.Nn[0] * v.Nn[1] * v.Nn[2];
  v.zero_faces = zero_faces;
  v.cdu = cdu_d.p;
  v.cdp = cdp_d.p;
  v.lptr = lptr_d.p;
  v.lcol = lcol_d.p;
  v.lw = D.lw.p;
  v.plptr = plptr_d.p;
  v.plcol = plcol_d.p;
  v.plw = D.plw.p;
  v.geom = structured ? GEOM_CART : (geom_kind == 0 ? GEOM_BOX : GEOM_TABLE);
  v.gbox = D.gbox.p;
  v.gtab = D.gtab.p;
  v.eta = D.eta.p;
  v.eta_n = eta_n;
  v.Mp = D.Mp.p;
  v.s = (T)s;
  v.compressible = compressible;
  return v;
}
template LevelView<float> Level::view<float>(double, int);
template LevelView<double> Level::view<double>(double, int);

size_t Level::device_bytes() const {
  size_t b = cdu_d.bytes() + cdp_d.bytes() + lptr_d.bytes() + lcol_d.bytes() + plptr_d.bytes() + plcol_d.bytes() +
             perm_u_d.bytes() + perm_p_d.bytes() + cons_u_d.bytes() + cons_p_d.bytes() + probe_ptr.bytes() +
             probe_g.bytes() + probe_eptr.bytes() + probe_li.bytes() + pprobe_ptr.bytes() + pprobe_g.bytes() +
             pprobe_eptr.bytes() + pprobe_li.bytes() + Pu_ptr.bytes() + Pu_col.bytes() + PuT_ptr.bytes() +
             PuT_col.bytes() + Pp_ptr.bytes() + Pp_col.bytes() + PpT_ptr.bytes() + PpT_col.bytes() + gu_ptr.bytes() +
             gu_slot.bytes() + gp_ptr.bytes() + gp_slot.bytes() + cmask_u.bytes() + cmask_p.bytes();
  auto add = [&](const auto& D) {
    b += D.lw.bytes() + D.plw.bytes() + D.gbox.bytes() + D.gtab.bytes() + D.eta.bytes() + D.probe_w.bytes() +
         D.pprobe_w.bytes() + D.Pu_val.bytes() + D.PuT_val.bytes() + D.Pp_val.bytes() + D.PpT_val.bytes() +
         D.dinvA.bytes() + D.dinvM.bytes() + D.solA.bytes() + D.defA.bytes() + D.tA.bytes() + D.dA.bytes() +
         D.solM.bytes() + D.defM.bytes() + D.tM.bytes() + D.dM.bytes() + D.gu_w.bytes() + D.gp_w.bytes() +
         D.Eu.bytes() + D.Ep.bytes() + D.Mp.bytes() + D.Fa.bytes() + D.eta_active.bytes() + D.xalt.bytes() +
         D.dalt.bytes() + D.Ealt.bytes();
  };
  b += ioc_d.bytes() + kid_ptr_d.bytes() + kid_d.bytes() + child_d.bytes() + jxw_d.bytes() + eta_in_d.bytes() +
       dg_d.bytes();
  add(f32);
  add(f64);
  return b;
}

}  // namespace gb
