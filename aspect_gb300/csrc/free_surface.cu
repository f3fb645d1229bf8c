// Free-surface stabilisation of the outer Stokes operator
// (StokesOperator::local_apply_boundary_face, source/simulator/solver/
// matrix_free_operators.cc:563-602; table filled at
// stokes_matrix_free_local_smoothing.cc:520-612): on every free-surface face F
// of the finest level
//     dst_u(phi) += int_F -(T . u) (n . phi) dS,    T = rho dt theta |g| g_hat,
// at the face's QGauss(3) points. The reference applies it in the outer Stokes
// operator and in correct_stokes_rhs only (no multigrid level carries it).
//
// Here the face integrals are added into the cell pass's per-cell contributions
// before the level's gather distributes them, so the sum stays deterministic and
// the constraints are handled by the gather exactly as for the cell terms. One
// thread per cell that owns free-surface faces; its faces in order. The face's
// Q2 velocity depends only on the 3^(dim-1) nodes of that face, read through
// constraint codes prepared at set-up (internal DoF, -1 zero, <= -2 a line of
// the level's constraint tables). Per face and component: a 3 x 3 (x 3) tensor
// evaluation to the points, the point term, and the transposed evaluation.
#include <cmath>

#include "ops.cuh"

namespace gb {
namespace {

template <typename T, int dim>
__global__ void __launch_bounds__(128) free_surface_kernel(FreeSurfaceView<T> F, const T* __restrict__ src,
                                                            T* __restrict__ E, long cs, long ss, const int* lptr,
                                                            const int* lcol, const T* lw) {
  constexpr int nf = fe::pow3(dim - 1);  // face nodes = face points
  constexpr int nv = fe::pow3(dim);
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= F.n_groups) return;
  const long cell = F.gcell[g];
  for (int f = F.gptr[g]; f < F.gptr[g + 1]; ++f) {
    const int fno = F.fno[f];
    const int d = fno >> 1, side = fno & 1;
    // tangential axes in increasing order: a (fastest), b
    const int ta = d == 0 ? 1 : 0;
    const int tb = dim == 3 ? (d == 2 ? 1 : 2) : 0;
    T u[dim][nf];
#pragma unroll
    for (int c = 0; c < dim; ++c)
#pragma unroll
      for (int k = 0; k < nf; ++k) u[c][k] = gather_general(src, F.codes[((size_t)f * dim + c) * nf + k], lptr, lcol, lw);
    // values at the points: v[c][q] = sum_k S(qa, ka) S(qb, kb) u[c][k]
    T v[dim][nf];
#pragma unroll
    for (int c = 0; c < dim; ++c) {
      if (dim == 2) {
#pragma unroll
        for (int q = 0; q < 3; ++q)
          v[c][q] = T(fe::Sv(q, 0)) * u[c][0] + T(fe::Sv(q, 1)) * u[c][1] + T(fe::Sv(q, 2)) * u[c][2];
      } else {
        T w[9];
#pragma unroll
        for (int kb = 0; kb < 3; ++kb)
#pragma unroll
          for (int qa = 0; qa < 3; ++qa)
            w[kb * 3 + qa] = T(fe::Sv(qa, 0)) * u[c][kb * 3] + T(fe::Sv(qa, 1)) * u[c][kb * 3 + 1] +
                             T(fe::Sv(qa, 2)) * u[c][kb * 3 + 2];
#pragma unroll
        for (int qb = 0; qb < 3; ++qb)
#pragma unroll
          for (int qa = 0; qa < 3; ++qa)
            v[c][(qb * 3 + qa) % nf] = T(fe::Sv(qb, 0)) * w[qa] + T(fe::Sv(qb, 1)) * w[3 + qa] +
                                       T(fe::Sv(qb, 2)) * w[6 + qa];
      }
    }
    // point term: -(T . u) (n JxW), overwriting v
    const T* tab = F.tab + (size_t)f * nf * 2 * dim;
#pragma unroll
    for (int q = 0; q < nf; ++q) {
      T tu = T(0);
#pragma unroll
      for (int e = 0; e < dim; ++e) tu += tab[q * 2 * dim + e] * v[e][q];
#pragma unroll
      for (int e = 0; e < dim; ++e) v[e][q] = -tu * tab[q * 2 * dim + dim + e];
    }
    // transposed evaluation into the face nodes, added to the cell's slots
#pragma unroll
    for (int c = 0; c < dim; ++c) {
      T r[nf];
      if (dim == 2) {
#pragma unroll
        for (int k = 0; k < 3; ++k)
          r[k] = T(fe::Sv(0, k)) * v[c][0] + T(fe::Sv(1, k)) * v[c][1] + T(fe::Sv(2, k)) * v[c][2];
      } else {
        T w[9];
#pragma unroll
        for (int qb = 0; qb < 3; ++qb)
#pragma unroll
          for (int ka = 0; ka < 3; ++ka)
            w[qb * 3 + ka] = T(fe::Sv(0, ka)) * v[c][(qb * 3) % nf] + T(fe::Sv(1, ka)) * v[c][(qb * 3 + 1) % nf] +
                             T(fe::Sv(2, ka)) * v[c][(qb * 3 + 2) % nf];
#pragma unroll
        for (int kb = 0; kb < 3; ++kb)
#pragma unroll
          for (int ka = 0; ka < 3; ++ka)
            r[(kb * 3 + ka) % nf] = T(fe::Sv(0, kb)) * w[ka] + T(fe::Sv(1, kb)) * w[3 + ka] + T(fe::Sv(2, kb)) * w[6 + ka];
      }
#pragma unroll
      for (int k = 0; k < nf; ++k) {
        const int ka = k % 3, kb = k / 3;
        int l = 2 * side * (d == 0 ? 1 : d == 1 ? 3 : 9);
        l += ka * (ta == 0 ? 1 : ta == 1 ? 3 : 9);
        if (dim == 3) l += kb * (tb == 0 ? 1 : tb == 1 ? 3 : 9);
        E[cell * cs + (long)(c * nv + l) * ss] += r[k];
      }
    }
  }
}

}  // namespace

template <typename T>
void launch_free_surface(const LevelView<T>& L, const FreeSurfaceView<T>& F, const T* src, T* E, bool slot_major,
                         cudaStream_t s) {
  if (F.n_groups <= 0) return;
  const int nl = L.dim * (L.dim == 3 ? 27 : 9);
  const long cs = slot_major ? 1 : nl, ss = slot_major ? L.n_cells : 1;
  const int threads = 128, blocks = ceil_div(F.n_groups, threads);
  if (L.dim == 3)
    free_surface_kernel<T, 3><<<blocks, threads, 0, s>>>(F, src, E, cs, ss, L.lptr, L.lcol, L.lw);
  else
    free_surface_kernel<T, 2><<<blocks, threads, 0, s>>>(F, src, E, cs, ss, L.lptr, L.lcol, L.lw);
  GB_CUDA(cudaGetLastError());
}

template void launch_free_surface<double>(const LevelView<double>&, const FreeSurfaceView<double>&, const double*,
                                          double*, bool, cudaStream_t);
template void launch_free_surface<float>(const LevelView<float>&, const FreeSurfaceView<float>&, const float*,
                                         float*, bool, cudaStream_t);

// Outward normal times surface JxW at the QGauss(3) points of a face, from a
// box cell (x0, h) or the cell's Q2 support points, points as the kernel reads
// them (first tangential axis fastest).
void face_normal_jxw(int dim, int geom_kind, const double* cell_geom, int fno, double* out) {
  const int d = fno >> 1, side = fno & 1;
  const int ta = d == 0 ? 1 : 0, tb = dim == 3 ? (d == 2 ? 1 : 2) : -1;
  const double gp[3] = {0.5 - std::sqrt(15.0) / 10, 0.5, 0.5 + std::sqrt(15.0) / 10};
  const int nf = dim == 3 ? 9 : 3;
  for (int q = 0; q < nf; ++q) {
    const int qa = q % 3, qb = q / 3;
    double wq = fe::Wv(qa) * (dim == 3 ? fe::Wv(qb) : 1.0);
    double J[3][3] = {};  // J[i][k] = d x_i / d xi_k
    if (geom_kind == 0) {
      for (int i = 0; i < dim; ++i) J[i][i] = cell_geom[dim + i];
    } else {
      double xi[3] = {0, 0, 0};
      xi[d] = side;
      xi[ta] = gp[qa];
      if (dim == 3) xi[tb] = gp[qb];
      double val[3][3], der[3][3];  // per axis: Q2 basis values / derivatives at xi
      for (int k = 0; k < dim; ++k) {
        const double x = xi[k];
        val[k][0] = 2 * (x - 0.5) * (x - 1);
        val[k][1] = -4 * x * (x - 1);
        val[k][2] = 2 * x * (x - 0.5);
        der[k][0] = 4 * x - 3;
        der[k][1] = -8 * x + 4;
        der[k][2] = 4 * x - 1;
      }
      const int nv = dim == 3 ? 27 : 9;
      for (int n = 0; n < nv; ++n) {
        const int a[3] = {n % 3, (n / 3) % 3, n / 9};
        for (int k = 0; k < dim; ++k) {
          double g = 1.0;
          for (int m = 0; m < dim; ++m) g *= m == k ? der[m][a[m]] : val[m][a[m]];
          for (int i = 0; i < dim; ++i) J[i][k] += cell_geom[n * dim + i] * g;
        }
      }
    }
    double N[3] = {0, 0, 0};
    if (dim == 3) {
      N[0] = J[1][ta] * J[2][tb] - J[2][ta] * J[1][tb];
      N[1] = J[2][ta] * J[0][tb] - J[0][ta] * J[2][tb];
      N[2] = J[0][ta] * J[1][tb] - J[1][ta] * J[0][tb];
    } else {
      N[0] = J[1][ta];
      N[1] = -J[0][ta];
    }
    // outward: along +J[:, d] on side 1, against it on side 0
    double dn = 0;
    for (int i = 0; i < dim; ++i) dn += N[i] * J[i][d];
    const double sgn = ((dn >= 0) == (side == 1)) ? 1.0 : -1.0;
    for (int i = 0; i < dim; ++i) out[q * dim + i] = sgn * N[i] * wq;
  }
}

}  // namespace gb
