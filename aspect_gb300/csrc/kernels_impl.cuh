// Instantiates the launchers for one scalar type GB_T (included by
// kernels_f32.cu / kernels_f64.cu so that the two precisions compile in parallel).
#include "ops.cuh"

namespace gb {

namespace {
constexpr int kCellThreads = 128;
// FP32 A-block cell pass per launch on one GB300 (CUDA events), register
// lattice kernel vs lattice_cell_kernel_small: 8 cells 10.3 vs 4.1 us, 64 cells
// 10.3 vs 5.1, 512 cells 10.3 vs 6.2, 4096 cells 10.3 vs 14.4, 32768 cells 12.3 vs 86.
constexpr int kSmallLatticeMaxCells = 512;
// 3D lattice velocity gathers: one thread per node (three components) above
// this many nodes, one thread per DoF at or below it (the two form the same
// sums). Measured A-block V-cycle levels: per DoF 8 us faster at 16^3 (33^3
// nodes) and 3 us at 8^3, per node 65 us faster at 32^3.
constexpr int kGatherPerNodeMinNodes = 33 * 33 * 33;
constexpr int kGatherThreads = 256;
template <int dim>
int cell_grid(int count) {
  const int cells_per_block = (kCellThreads / 32) * Shape<dim>::cpw;
  return ceil_div(count, cells_per_block);
}

template <int dim>
void cell_pass_dim(const LevelView<GB_T>& L, int op, const GB_T* su, const GB_T* sp, GB_T* Eu, GB_T* Ep,
                   cudaStream_t s) {
  if (op == OPK_MASS) {
    mass_cell_kernel<GB_T, dim><<<ceil_div(L.n_cells, kCellThreads), kCellThreads, 0, s>>>(L, sp, Ep);
    return;
  }
  const int g = cell_grid<dim>(L.n_cells);
  // indexed levels: the geometry kind as a template argument (one code path per
  // point instead of three, a smaller kernel for the instruction cache)
  if (L.geom == GEOM_TABLE) {
    if (op == OPK_STOKES) velocity_cell_kernel<GB_T, dim, OPK_STOKES, GEOM_TABLE><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
    else if (op == OPK_A) velocity_cell_kernel<GB_T, dim, OPK_A, GEOM_TABLE><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
    else velocity_cell_kernel<GB_T, dim, OPK_BT, GEOM_TABLE><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
    return;
  }
  if (L.geom == GEOM_BOX) {
    if (op == OPK_STOKES) velocity_cell_kernel<GB_T, dim, OPK_STOKES, GEOM_BOX><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
    else if (op == OPK_A) velocity_cell_kernel<GB_T, dim, OPK_A, GEOM_BOX><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
    else velocity_cell_kernel<GB_T, dim, OPK_BT, GEOM_BOX><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
    return;
  }
  if (op == OPK_STOKES) velocity_cell_kernel<GB_T, dim, OPK_STOKES><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
  else if (op == OPK_A) velocity_cell_kernel<GB_T, dim, OPK_A><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
  else velocity_cell_kernel<GB_T, dim, OPK_BT><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
}

template <int dim, int epi>
void gather_dim_epi(const LevelView<GB_T>& L, int block, const GatherCsr<GB_T>* csr, const GatherArgs<GB_T>& a,
                    cudaStream_t s) {
  const long n = block == 0 ? L.n_u : L.n_p;
  const int g = ceil_div(n, kGatherThreads);
  if (csr) gather_csr<GB_T, epi><<<g, kGatherThreads, 0, s>>>(n, *csr, a);
  else if (block == 0 && dim == 3 && L.n_nodes > kGatherPerNodeMinNodes)
    velocity_gather_lattice3<GB_T, epi><<<ceil_div(L.n_nodes, kGatherThreads), kGatherThreads, 0, s>>>(L, a);
  else if (block == 0) velocity_gather_structured<GB_T, dim, epi><<<g, kGatherThreads, 0, s>>>(L, a);
  else pressure_gather_structured<GB_T, dim, epi><<<g, kGatherThreads, 0, s>>>(L, a);
}

template <int dim>
void gather_dim(const LevelView<GB_T>& L, int block, int epi, const GatherCsr<GB_T>* csr,
                const GatherArgs<GB_T>& a, cudaStream_t s) {
  switch (epi) {
    case EPI_STORE: gather_dim_epi<dim, EPI_STORE>(L, block, csr, a, s); break;
    case EPI_BT: gather_dim_epi<dim, EPI_BT>(L, block, csr, a, s); break;
    case EPI_RESID: gather_dim_epi<dim, EPI_RESID>(L, block, csr, a, s); break;
    case EPI_CHEB_OUT: gather_dim_epi<dim, EPI_CHEB_OUT>(L, block, csr, a, s); break;
    default: gather_dim_epi<dim, EPI_CHEB>(L, block, csr, a, s); break;
  }
}
}  // namespace

template <>
bool cell_pass_slot_major<GB_T>(const LevelView<GB_T>& L, int op) {
  return std::is_same<GB_T, float>::value && L.dim == 3 && L.structured &&
         (op == OPK_A || op == OPK_STOKES || op == OPK_BT);
}

template <>
void launch_cell_pass<GB_T>(const LevelView<GB_T>& L, int op, const GB_T* su, const GB_T* sp, GB_T* Eu, GB_T* Ep,
                            cudaStream_t s) {
  if (L.n_cells <= 0) return;
  if (L.deg == 3) {  // Q3-Q2 (indexed levels only)
    launch_ho_cell_pass<GB_T>(L, op, su, sp, Eu, Ep, s);
    return;
  }
#if defined(GB_T_IS_FLOAT)
  {
    if (cell_pass_slot_major<GB_T>(L, op) && op == OPK_A && L.n_cells <= kSmallLatticeMaxCells) {
      if (L.eta_n != 1) lattice_cell_kernel_small<true><<<L.n_cells, kSmallCellThreads, 0, s>>>(L, su, Eu);
      else lattice_cell_kernel_small<false><<<L.n_cells, kSmallCellThreads, 0, s>>>(L, su, Eu);
      return;
    }
    if (cell_pass_slot_major<GB_T>(L, op)) {
      const int g = ceil_div(L.n_cells, kCellThreads);
      const bool pq = L.eta_n != 1;
      if (op == OPK_A) {
        if (pq) lattice_cell_kernel_f32<OPK_A, true><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
        else lattice_cell_kernel_f32<OPK_A, false><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
      } else if (op == OPK_BT) {
        lattice_cell_kernel_f32<OPK_BT, false><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
      } else {
        if (pq) lattice_cell_kernel_f32<OPK_STOKES, true><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
        else lattice_cell_kernel_f32<OPK_STOKES, false><<<g, kCellThreads, 0, s>>>(L, su, sp, Eu, Ep);
      }
      return;
    }
  }
#else
  // FP64 velocity-test operators of isotropic 3D lattice levels (cubic cells)
  if (op != OPK_MASS && L.dim == 3 && L.structured && L.geom == GEOM_CART && L.inv_h[0] == L.inv_h[1] &&
      L.inv_h[1] == L.inv_h[2]) {
    IsoCoef<double> C;
    const double ih = L.inv_h[0];
    for (int q = 0; q < 27; ++q) {
      const double w = fe::Wv(q % 3) * fe::Wv((q / 3) % 3) * fe::Wv(q / 9);
      C.K[q] = ih * ih * L.det * w;
      C.M[q] = L.s * ih * L.det * w;
    }
    const int g = cell_grid<3>(L.n_cells);
    const bool pq = L.eta_n != 1;
#define GB_ISO(OP)                                                                                   \
  {                                                                                                  \
    if (pq) lattice_iso_kernel_f64<OP, true><<<g, kCellThreads, 0, s>>>(L, C, su, sp, Eu, Ep);       \
    else lattice_iso_kernel_f64<OP, false><<<g, kCellThreads, 0, s>>>(L, C, su, sp, Eu, Ep);         \
  }
    if (op == OPK_STOKES) GB_ISO(OPK_STOKES)
    else if (op == OPK_A) GB_ISO(OPK_A)
    else GB_ISO(OPK_BT)
#undef GB_ISO
    return;
  }
#endif
  if (L.dim == 3) cell_pass_dim<3>(L, op, su, sp, Eu, Ep, s);
  else cell_pass_dim<2>(L, op, su, sp, Eu, Ep, s);
}

template <>
void launch_gather<GB_T>(const LevelView<GB_T>& L, int block, int epi, const GatherCsr<GB_T>* csr,
                         const GatherArgs<GB_T>& a, cudaStream_t s) {
  if (L.dim == 3) gather_dim<3>(L, block, epi, csr, a, s);
  else gather_dim<2>(L, block, epi, csr, a, s);
}

template <>
void launch_mass_lattice<GB_T>(const LevelView<GB_T>& L, const GB_T* Mc, int epi, const GatherArgs<GB_T>& a,
                               cudaStream_t s) {
  constexpr int B = kMassLatticeThreads;
#define GB_MASS_LATTICE(DIM)                                                                      \
  {                                                                                               \
    const int g = ceil_div((long)L.n_p * Shape<DIM>::np, B);                                      \
    switch (epi) {                                                                                \
      case EPI_STORE: mass_apply_lattice<GB_T, DIM, EPI_STORE><<<g, B, 0, s>>>(L, Mc, a); break;  \
      case EPI_RESID: mass_apply_lattice<GB_T, DIM, EPI_RESID><<<g, B, 0, s>>>(L, Mc, a); break;  \
      default: mass_apply_lattice<GB_T, DIM, EPI_CHEB_OUT><<<g, B, 0, s>>>(L, Mc, a); break;      \
    }                                                                                             \
  }
  if (L.dim == 3) GB_MASS_LATTICE(3) else GB_MASS_LATTICE(2)
#undef GB_MASS_LATTICE
}

template <>
void launch_velocity_diag<GB_T>(const LevelView<GB_T>& L, int colour, int begin, int count,
                                const ProbesView<GB_T>& pr, GB_T* diag, cudaStream_t s) {
  if (count <= 0) return;
  if (L.dim == 3)
    velocity_diag_kernel<GB_T, 3><<<cell_grid<3>(count), kCellThreads, 0, s>>>(L, colour, begin, count, pr.ptr, pr.g, pr.eptr, pr.li, pr.w, diag);
  else
    velocity_diag_kernel<GB_T, 2><<<cell_grid<2>(count), kCellThreads, 0, s>>>(L, colour, begin, count, pr.ptr, pr.g, pr.eptr, pr.li, pr.w, diag);
}

template <>
void launch_lattice_diag<GB_T>(const LevelView<GB_T>& L, GB_T* Eu, bool slot_major, cudaStream_t s) {
  if (L.n_cells <= 0) return;
  if (L.dim == 3) lattice_diag_kernel<GB_T, 3><<<cell_grid<3>(L.n_cells), kCellThreads, 0, s>>>(L, Eu, slot_major);
  else lattice_diag_kernel<GB_T, 2><<<cell_grid<2>(L.n_cells), kCellThreads, 0, s>>>(L, Eu, slot_major);
}

template <>
void launch_mass_diag<GB_T>(const LevelView<GB_T>& L, int colour, int begin, int count, const ProbesView<GB_T>& pr,
                            GB_T* diag, cudaStream_t s) {
  if (count <= 0) return;
  const int g = ceil_div(count, kCellThreads);
  if (L.dim == 3) mass_diag_kernel<GB_T, 3><<<g, kCellThreads, 0, s>>>(L, colour, begin, count, pr.ptr, pr.g, pr.eptr, pr.li, pr.w, diag);
  else mass_diag_kernel<GB_T, 2><<<g, kCellThreads, 0, s>>>(L, colour, begin, count, pr.ptr, pr.g, pr.eptr, pr.li, pr.w, diag);
}

#if defined(GB_T_IS_FLOAT)
bool small_lattice_a_level(const LevelView<float>& L) {
  return cell_pass_slot_major<float>(L, OPK_A) && L.n_cells <= kSmallLatticeMaxCells && L.deg == 2;
}
void launch_cheb_small(const LevelView<float>& L, bool first, const ChebSmallArgs& a, cudaStream_t s) {
  if (L.n_cells <= 0) return;
  const bool pq = L.eta_n != 1;
  if (first) {
    if (pq) lattice_cheb_small<true, true><<<L.n_cells, kSmallCellThreads, 0, s>>>(L, a);
    else lattice_cheb_small<true, false><<<L.n_cells, kSmallCellThreads, 0, s>>>(L, a);
  } else {
    if (pq) lattice_cheb_small<false, true><<<L.n_cells, kSmallCellThreads, 0, s>>>(L, a);
    else lattice_cheb_small<false, false><<<L.n_cells, kSmallCellThreads, 0, s>>>(L, a);
  }
  GB_CUDA(cudaGetLastError());
}
#endif

}  // namespace gb
