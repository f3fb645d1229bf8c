// Level viscosity tables on the device (what ASPECT's assemble() rebuilds on
// every nonlinear iteration: source/simulator/solver/
// stokes_matrix_free_local_smoothing.cc:174-294, matrix_free_operators.cc:137-330).
//
// From the finest level's material values (one per cell, or one per QGauss(3)
// point) the kernels build, level by level:
//   DGQ0 (projection 0, and 2 = no averaging): the JxW-weighted cell mean on the
//        finest level, then each coarser cell the plain mean of its children;
//   DGQ1 (projection 1): the cellwise L2 projection onto Q1 on the finest level
//        (an 8 x 8 (4 x 4) mass system per cell, Gaussian elimination), then a
//        coarser cell's vertex value is the value of the child at that vertex,
//        and every level's per-point table is the Q1 interpolation clamped to
//        the finest level's range;
//   no averaging (2): the finest level also keeps the per-point values for the
//        outer operators;
// then writes each level's table in its internal cell order, in FP64 and FP32,
// and on lattice levels the per-cell pressure mass matrices
// M[i][j] = sum_q s^2 / eta_q |det J| w_q psi_i psi_j. Every sum runs in the
// order of the former host code (points ascending, children by fine-cell
// index), so the tables are the ones the oracle builds from the same rule.
// The caller's values are checked (positive, finite) and their range taken on
// the host before any table changes.
#include <algorithm>
#include <cmath>

#include "level.cuh"

namespace gb {
namespace {

constexpr int kCoefThreads = 128;

// Gauss points of QGauss(4) on [0, 1]: (1 -+ sqrt(3/7 +- 2/7 sqrt(6/5))) / 2
__device__ __forceinline__ double gauss4(int i) {
  return i == 0 ? 0.069431844202973712388 : i == 1 ? 0.33000947820757186760
       : i == 2 ? 0.66999052179242813240 : 0.93056815579702628761;
}
// Q1 basis {1 - x, x} at 1D Gauss point i of NQ1 points
template <int NQ1>
__device__ __forceinline__ double p1(int i, int n) {
  if constexpr (NQ1 == 3) return fe::P1v(i, n);
  else return n ? gauss4(i) : 1.0 - gauss4(i);
}
template <int dim, int NQ1 = 3>
__device__ __forceinline__ double psi1(int q, int n) {
  // Q1 basis n at Gauss point q (lexicographic digits)
  double v = p1<NQ1>(q % NQ1, n & 1) * p1<NQ1>((q / NQ1) % NQ1, (n >> 1) & 1);
  if (dim == 3) v *= p1<NQ1>(q / (NQ1 * NQ1), (n >> 2) & 1);
  return v;
}

template <int dim, int NQ1>
__global__ void k_dgq0_finest(long n_cells, int n_per_cell, const double* __restrict__ eta_in,
                              const double* __restrict__ jxw, double* __restrict__ dg) {
  constexpr int nq = NQ1 * NQ1 * (dim == 3 ? NQ1 : 1);
  const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  if (n_per_cell == 1) {
    dg[c] = eta_in[c];
    return;
  }
  double a = 0, v = 0;
  for (int q = 0; q < nq; ++q) {
    const double jw = jxw[c * nq + q];
    a += jw * eta_in[c * nq + q];
    v += jw;
  }
  dg[c] = a / v;
}

__global__ void k_dgq0_restrict(long n_coarse, const int* __restrict__ ptr, const int* __restrict__ kids,
                                const double* __restrict__ fine, double* __restrict__ coarse) {
  const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (p >= n_coarse) return;
  double sum = 0, cnt = 0;
  for (int k = ptr[p]; k < ptr[p + 1]; ++k) {
    sum += fine[kids[k]];
    cnt += 1;
  }
  coarse[p] = sum / cnt;
}

template <int dim, int NQ1>
__global__ void k_dgq1_finest(long n_cells, const double* __restrict__ eta_in, const double* __restrict__ jxw,
                              double* __restrict__ dg) {
  constexpr int nq = NQ1 * NQ1 * (dim == 3 ? NQ1 : 1), ncv = fe::pow2(dim);
  const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  double M[ncv][ncv], b[ncv], x[ncv];
  for (int i = 0; i < ncv; ++i) {
    b[i] = 0;
    for (int j = 0; j < ncv; ++j) M[i][j] = 0;
  }
  for (int q = 0; q < nq; ++q) {
    const double jw = jxw[c * nq + q];
    for (int i = 0; i < ncv; ++i) {
      b[i] += jw * psi1<dim, NQ1>(q, i) * eta_in[c * nq + q];
      for (int j = 0; j < ncv; ++j) M[i][j] += jw * psi1<dim, NQ1>(q, i) * psi1<dim, NQ1>(q, j);
    }
  }
  for (int i = 0; i < ncv; ++i)
    for (int r = i + 1; r < ncv; ++r) {
      const double f = M[r][i] / M[i][i];
      for (int k = i; k < ncv; ++k) M[r][k] -= f * M[i][k];
      b[r] -= f * b[i];
    }
  for (int i = ncv - 1; i >= 0; --i) {
    double t = b[i];
    for (int k = i + 1; k < ncv; ++k) t -= M[i][k] * x[k];
    x[i] = t / M[i][i];
  }
  for (int i = 0; i < ncv; ++i) dg[c * ncv + i] = x[i];
}

__global__ void k_dgq1_restrict(long n_coarse, int ncv, const int* __restrict__ ptr, const int* __restrict__ kids,
                                const unsigned char* __restrict__ child, const double* __restrict__ fine,
                                double* __restrict__ coarse) {
  const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (p >= n_coarse) return;
  for (int i = 0; i < ncv; ++i) coarse[p * ncv + i] = 0;
  for (int k = ptr[p]; k < ptr[p + 1]; ++k) {
    const int f = kids[k];
    const int ch = child[f];
    if (ch == kSameCell) {
      for (int i = 0; i < ncv; ++i) coarse[p * ncv + i] = fine[(long)f * ncv + i];
    } else {
      coarse[p * ncv + ch] = fine[(long)f * ncv + ch];
    }
  }
}

// a level's table in internal cell order, FP64 and FP32: mode 0 = one value per
// cell (dg), 1 = the caller's per-point values, 2 = the Q1 interpolation of dg
// clamped to [lo, hi]
template <int dim, int NQ1>
__global__ void k_level_table(long n_cells, int mode, const int* __restrict__ ioc, const double* __restrict__ dg,
                              const double* __restrict__ eta_in, double lo, double hi, double* __restrict__ t64,
                              float* __restrict__ t32) {
  constexpr int nq = NQ1 * NQ1 * (dim == 3 ? NQ1 : 1), ncv = fe::pow2(dim);
  const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  const long ic = ioc[c];
  if (mode == 0) {
    t64[ic] = dg[c];
    t32[ic] = (float)dg[c];
    return;
  }
  for (int q = 0; q < nq; ++q) {
    double v;
    if (mode == 1) {
      v = eta_in[c * nq + q];
    } else {
      v = 0;
      for (int i = 0; i < ncv; ++i) v += psi1<dim, NQ1>(q, i) * dg[c * ncv + i];
      v = fmin(fmax(v, lo), hi);
    }
    t64[ic * nq + q] = v;
    t32[ic * nq + q] = (float)v;
  }
}

// per-cell pressure mass matrices of a lattice level (internal cell order)
template <int dim>
__global__ void k_mass_matrices(long n_cells, int eta_n, const double* __restrict__ eta, double s2det,
                                double* __restrict__ m64, float* __restrict__ m32) {
  constexpr int nq = fe::pow3(dim), np = fe::pow2(dim);
  const long ic = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (ic >= n_cells) return;
  double m[np * np];
  for (int k = 0; k < np * np; ++k) m[k] = 0;
  for (int q = 0; q < nq; ++q) {
    double wq = fe::Wv(q % 3) * fe::Wv((q / 3) % 3);
    if (dim == 3) wq *= fe::Wv(q / 9);
    const double f = s2det / eta[ic * eta_n + (eta_n == 1 ? 0 : q)] * wq;
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j) m[i * np + j] += f * psi1<dim>(q, i) * psi1<dim>(q, j);
  }
  for (int k = 0; k < np * np; ++k) {
    m64[ic * np * np + k] = m[k];
    m32[ic * np * np + k] = (float)m[k];
  }
}

// per-cell pressure mass matrices of an indexed level (internal cell order):
// JxW from the level's box table (|det J|) or per-point geometry table
template <int dim>
__global__ void k_mass_matrices_general(long n_cells, int eta_n, const double* __restrict__ eta, double s2,
                                        int geom, const double* __restrict__ gbox, const double* __restrict__ gtab,
                                        double* __restrict__ m64, float* __restrict__ m32) {
  constexpr int nq = fe::pow3(dim), np = fe::pow2(dim);
  const long ic = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (ic >= n_cells) return;
  double m[np * np];
  for (int k = 0; k < np * np; ++k) m[k] = 0;
  for (int q = 0; q < nq; ++q) {
    double wq = fe::Wv(q % 3) * fe::Wv((q / 3) % 3);
    if (dim == 3) wq *= fe::Wv(q / 9);
    const double det = geom == GEOM_TABLE ? gtab[(ic * nq + q) * (dim * dim + 1) + dim * dim]
                                          : gbox[ic * (dim + 1) + dim];
    const double f = s2 / eta[ic * eta_n + (eta_n == 1 ? 0 : q)] * det * wq;
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j) m[i * np + j] += f * psi1<dim>(q, i) * psi1<dim>(q, j);
  }
  for (int k = 0; k < np * np; ++k) {
    m64[ic * np * np + k] = m[k];
    m32[ic * np * np + k] = (float)m[k];
  }
}

// Body-force right-hand side of one finest cell and velocity component:
// V[n] = sum_q JxW_q f_comp(q) phi_n(q) (source/simulator/assemblers/stokes.cc:
// 285-400, the rho g . phi_u term), by the transposed interpolation of the
// point values; one thread per (cell, component), output cell-major
// [cell][comp][node] as the velocity cell pass writes it.
template <int dim>
__global__ void __launch_bounds__(128) k_body_force(LevelView<double> L, const double* __restrict__ force,
                                                   double* __restrict__ Eu) {
  pdl_wait();
  constexpr int nv = fe::pow3(dim), nq = nv;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)L.n_cells * dim) return;
  const long cell = t / dim;
  const int comp = (int)(t - cell * dim);
  double V[nv];
  static_for<nq>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    double jxw;
    if (L.geom == GEOM_CART) jxw = L.det * qweight<dim, q>();
    else if (L.geom == GEOM_BOX) jxw = L.gbox[cell * (dim + 1) + dim] * qweight<dim, q>();
    else jxw = L.gtab[(cell * nq + q) * (dim * dim + 1) + dim * dim] * qweight<dim, q>();
    V[q] = jxw * force[(cell * nq + q) * dim + comp];
  });
  interpolate<double, dim, true>(V);
  double* e = Eu + (cell * dim + comp) * nv;
#pragma unroll
  for (int n = 0; n < nv; ++n) e[n] = V[n];
}

int grid(long n) { return (int)((n + kCoefThreads - 1) / kCoefThreads); }

// calls f(dim, points per direction) with both as compile-time constants
template <class F>
void dispatch_dq(int dim, int n1, F&& f) {
  if (dim == 3 && n1 == 3) f(std::integral_constant<int, 3>{}, std::integral_constant<int, 3>{});
  else if (dim == 3) f(std::integral_constant<int, 3>{}, std::integral_constant<int, 4>{});
  else if (n1 == 3) f(std::integral_constant<int, 2>{}, std::integral_constant<int, 3>{});
  else f(std::integral_constant<int, 2>{}, std::integral_constant<int, 4>{});
}

// Q2 basis on nodes {0, 1/2, 1}: values and derivatives at x
void q2_basis(double x, double* v, double* dv) {
  v[0] = 2.0 * (x - 0.5) * (x - 1.0);
  v[1] = 4.0 * x * (1.0 - x);
  v[2] = 2.0 * x * (x - 0.5);
  dv[0] = 4.0 * x - 3.0;
  dv[1] = 4.0 - 8.0 * x;
  dv[2] = 4.0 * x - 1.0;
}

}  // namespace

// Static per-mesh data of the device pipeline (once per gb_gmg_finalize_setup):
// caller -> internal cell maps, the children of every coarse cell (by fine-cell
// index), and the finest level's JxW per point.
void setup_coefficient_maps(std::vector<Level>& levels) {
  const int nlev = (int)levels.size();
  Level& Fl = levels.back();
  const int d = Fl.dim, nq = Fl.nq();
  for (int l = 0; l < nlev; ++l) {
    Level& L = levels[l];
    L.ioc_d.upload(L.internal_of_cell);
    if (l == 0) continue;
    const Level& C = levels[l - 1];
    std::vector<int> ptr(C.n_cells + 1, 0), kids(L.n_cells);
    for (long c = 0; c < L.n_cells; ++c) ptr[L.parent[c] + 1]++;
    for (long p = 0; p < C.n_cells; ++p) ptr[p + 1] += ptr[p];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (long c = 0; c < L.n_cells; ++c) kids[fill[L.parent[c]]++] = (int)c;  // ascending fine index
    L.kid_ptr_d.upload(ptr);
    L.kid_d.upload(kids);
    L.child_d.upload(L.child);
  }
  // finest JxW per point (QGauss(degree+1)), from the caller's geometry
  const Basis1D B = basis1d(Fl.degree);
  const int n1 = B.nq1, nm = ipow(3, d);  // points per direction, Q2 mapping support points
  double v1[4][3], d1[4][3];
  for (int q = 0; q < n1; ++q) q2_basis(B.gq[q], v1[q], d1[q]);
  std::vector<double> jxw((size_t)Fl.n_cells * nq);
  for (long c = 0; c < Fl.n_cells; ++c)
    for (int q = 0; q < nq; ++q) {
      const int qi[3] = {q % n1, (q / n1) % n1, q / (n1 * n1)};
      double w = 1;
      for (int e = 0; e < d; ++e) w *= B.gw[qi[e]];
      double det;
      if (Fl.geom_kind == 0) {
        det = 1;
        for (int e = 0; e < d; ++e) det *= Fl.geom[c * 2 * d + d + e];
      } else if (Fl.geom_kind == 2) {
        det = Fl.geom[((size_t)c * nq + q) * (d * d + 1) + d * d];
      } else {
        double J[3][3] = {{0}};
        const double* X = &Fl.geom[(size_t)c * nm * d];
        for (int n = 0; n < nm; ++n) {
          const int ni[3] = {n % 3, (n / 3) % 3, n / 9};
          for (int b = 0; b < d; ++b) {
            double t = 1;
            for (int e = 0; e < d; ++e) t *= (e == b ? d1[qi[e]][ni[e]] : v1[qi[e]][ni[e]]);
            for (int a = 0; a < d; ++a) J[a][b] += X[n * d + a] * t;
          }
        }
        det = std::fabs(d == 2 ? J[0][0] * J[1][1] - J[0][1] * J[1][0]
                               : J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]));
      }
      jxw[(size_t)c * nq + q] = w * det;
    }
  Fl.jxw_d.upload(jxw);
}

void device_level_viscosity(std::vector<Level>& levels, const double* eta_in, int n_per_cell, int projection,
                            double s, double& eta_min, double& eta_max, cudaStream_t st) {
  const int nlev = (int)levels.size();
  Level& Fl = levels.back();
  const int d = Fl.dim, nq = Fl.nq(), ncv = d == 3 ? 8 : 4, n1 = Fl.degree + 1;
  GB_CHECK(projection >= 0 && projection <= 2, 1, "unknown viscosity projection");
  GB_CHECK(projection == 0 || n_per_cell == nq, 1,
           "projection to Q1 and no averaging need one value per quadrature point");
  // the caller's values: checked and their range taken before any table changes
  eta_min = 1e300;
  eta_max = -1e300;
  for (long i = 0; i < Fl.n_cells * n_per_cell; ++i) {
    GB_CHECK(eta_in[i] > 0 && std::isfinite(eta_in[i]), 6, "viscosity must be positive and finite");
    eta_min = std::min(eta_min, eta_in[i]);
    eta_max = std::max(eta_max, eta_in[i]);
  }
  Fl.eta_in_d.upload(eta_in, (size_t)Fl.n_cells * n_per_cell);
  const double* ein = Fl.eta_in_d.p;
  // DG fields, finest to coarsest
  const int per = projection == 1 ? ncv : 1;
  for (auto& L : levels) L.dg_d.alloc((size_t)L.n_cells * per);
  if (projection == 1) {
    dispatch_dq(d, n1, [&](auto dc, auto nc) {
      k_dgq1_finest<decltype(dc)::value, decltype(nc)::value>
          <<<grid(Fl.n_cells), kCoefThreads, 0, st>>>(Fl.n_cells, ein, Fl.jxw_d.p, Fl.dg_d.p);
    });
    for (int l = nlev - 1; l > 0; --l) {
      Level& C = levels[l - 1];
      k_dgq1_restrict<<<grid(C.n_cells), kCoefThreads, 0, st>>>(C.n_cells, ncv, levels[l].kid_ptr_d.p,
                                                                 levels[l].kid_d.p, levels[l].child_d.p,
                                                                 levels[l].dg_d.p, C.dg_d.p);
    }
  } else {
    dispatch_dq(d, n1, [&](auto dc, auto nc) {
      k_dgq0_finest<decltype(dc)::value, decltype(nc)::value>
          <<<grid(Fl.n_cells), kCoefThreads, 0, st>>>(Fl.n_cells, n_per_cell, ein, Fl.jxw_d.p, Fl.dg_d.p);
    });
    for (int l = nlev - 1; l > 0; --l) {
      Level& C = levels[l - 1];
      k_dgq0_restrict<<<grid(C.n_cells), kCoefThreads, 0, st>>>(C.n_cells, levels[l].kid_ptr_d.p, levels[l].kid_d.p,
                                                                 levels[l].dg_d.p, C.dg_d.p);
    }
  }
  GB_CUDA(cudaGetLastError());
  // the tables, internal cell order
  for (int l = 0; l < nlev; ++l) {
    Level& L = levels[l];
    const bool top = l == nlev - 1;
    int mode;
    if (projection == 1) {
      mode = 2;
      L.eta_n = nq;
    } else if (top && projection == 0 && n_per_cell == nq) {
      mode = 1;
      L.eta_n = nq;
    } else {
      mode = 0;
      L.eta_n = 1;
    }
    const size_t n = (size_t)L.n_cells * L.eta_n;
    L.f64.eta.alloc(n);  // same size: same address, so captured V-cycles stay valid
    L.f32.eta.alloc(n);
    dispatch_dq(d, n1, [&](auto dc, auto nc) {
      k_level_table<decltype(dc)::value, decltype(nc)::value><<<grid(L.n_cells), kCoefThreads, 0, st>>>(
          L.n_cells, mode, L.ioc_d.p, L.dg_d.p, ein, eta_min, eta_max, L.f64.eta.p, L.f32.eta.p);
    });
    // no averaging: the outer operators' per-point table of the finest level
    L.eta_active_n = top && projection == 2 ? nq : 0;
    if (L.eta_active_n) {
      L.f64.eta_active.alloc((size_t)L.n_cells * nq);
      L.f32.eta_active.alloc((size_t)L.n_cells * nq);
      dispatch_dq(d, n1, [&](auto dc, auto nc) {
        k_level_table<decltype(dc)::value, decltype(nc)::value><<<grid(L.n_cells), kCoefThreads, 0, st>>>(
            L.n_cells, 1, L.ioc_d.p, nullptr, ein, 0, 0, L.f64.eta_active.p, L.f32.eta_active.p);
      });
    } else {
      L.f64.eta_active.release();
      L.f32.eta_active.release();
    }
    if (!L.structured && L.degree == 2) {
      // indexed levels: the same matrices from the level's JxW (the mass cell
      // pass then reads them instead of the per-point geometry)
      const int np = d == 3 ? 8 : 4;
      const LevelView<double> v = L.view<double>(s, 0);
      L.f64.Mp.alloc((size_t)L.n_cells * np * np);
      L.f32.Mp.alloc((size_t)L.n_cells * np * np);
      if (d == 3)
        k_mass_matrices_general<3><<<grid(L.n_cells), kCoefThreads, 0, st>>>(
            L.n_cells, L.eta_n, L.f64.eta.p, s * s, v.geom, v.gbox, v.gtab, L.f64.Mp.p, L.f32.Mp.p);
      else
        k_mass_matrices_general<2><<<grid(L.n_cells), kCoefThreads, 0, st>>>(
            L.n_cells, L.eta_n, L.f64.eta.p, s * s, v.geom, v.gbox, v.gtab, L.f64.Mp.p, L.f32.Mp.p);
    }
    if (L.structured) {
      const int np = d == 3 ? 8 : 4;
      double det = 1;
      for (int k = 0; k < d; ++k) det *= L.h[k];
      L.f64.Mp.alloc((size_t)L.n_cells * np * np);
      L.f32.Mp.alloc((size_t)L.n_cells * np * np);
      if (d == 3)
        k_mass_matrices<3><<<grid(L.n_cells), kCoefThreads, 0, st>>>(L.n_cells, L.eta_n, L.f64.eta.p, s * s * det,
                                                                     L.f64.Mp.p, L.f32.Mp.p);
      else
        k_mass_matrices<2><<<grid(L.n_cells), kCoefThreads, 0, st>>>(L.n_cells, L.eta_n, L.f64.eta.p, s * s * det,
                                                                     L.f64.Mp.p, L.f32.Mp.p);
    }
    GB_CUDA(cudaGetLastError());
  }
  GB_CUDA(cudaStreamSynchronize(st));
}

void launch_body_force(const LevelView<double>& L, const double* force, double* Eu, cudaStream_t st) {
  const long n = (long)L.n_cells * L.dim;
  if (L.dim == 3) k_body_force<3><<<grid(n), kCoefThreads, 0, st>>>(L, force, Eu);
  else k_body_force<2><<<grid(n), kCoefThreads, 0, st>>>(L, force, Eu);
  GB_CUDA(cudaGetLastError());
}

}  // namespace gb
