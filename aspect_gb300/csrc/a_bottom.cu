// The lower lattice levels of the FP32 A-block (velocity) V-cycle in one thread
// block, run in batch mode: block b applies the sub-cycle of levels 0..K to the
// unit vector e_b, so one launch yields the sub-cycle's explicit matrix, which
// the V-cycle then applies as one dense product instead of the ~60 short
// launches of those levels.
//
// The steps are the multi-launch ones in the same order and with the same
// coefficients: Chebyshev pre-smoothing from a zero start, the residual, the
// restriction, the coarse level's degree-8 Chebyshev solve, the prolongation
// and the post-smoothing. The A operator of a lattice level is the register
// kernel's cell function (lattice_cell_f32, one thread per cell) into per-cell
// contributions in shared memory, then the lattice gather of each node
// (velocity_lattice_node) with its epilogue (Chebyshev update in place, or the
// residual), __syncthreads() between the two and between steps. Vectors,
// diagonals and contributions of all levels (about 77 KB for the 1, 8, 64-cell
// levels) live in shared memory; viscosity, geometry and transfers are read
// from global memory.
#include "a_bottom.cuh"
#include "ops.cuh"

namespace gb {
namespace {

constexpr int kABottomThreads = 256;

template <bool per_q>
__device__ void bottom_a_apply(const ABottomLevel& V, int epi, GatherArgs<float> a) {
  for (int c = threadIdx.x; c < V.L.n_cells; c += kABottomThreads) {
    float Vv[3][27], YP[8];
    lattice_cell_f32<OPK_A, per_q>(V.L, a.x, nullptr, c, Vv, YP);
    float* e = V.E + (size_t)c * 81;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int n = 0; n < 27; ++n) e[k * 27 + n] = Vv[k][n];
  }
  __syncthreads();
  a.E = V.E;
  a.cs = 81;
  a.ss = 1;
  for (int node = threadIdx.x; node < V.L.n_nodes; node += kABottomThreads) {
    if (epi == EPI_RESID) velocity_lattice_node<float, EPI_RESID>(V.L, a, node);
    else velocity_lattice_node<float, EPI_CHEB>(V.L, a, node);
  }
  __syncthreads();
}

// PreconditionChebyshev from a zero start or one more sweep from sol (the
// multi-launch chebyshev(): EPI_CHEB updates the iterate in place)
template <bool per_q>
__device__ void bottom_a_chebyshev(const ABottomLevel& V, bool zero_start) {
  const int n = V.L.n_u;
  auto step = [&](float f1, float f2) {
    GatherArgs<float> a{};
    a.x = V.sol;
    a.b = V.def;
    a.dinv = V.dinv;
    a.d = V.d;
    a.f1 = f1;
    a.f2 = f2;
    bottom_a_apply<per_q>(V, EPI_CHEB, a);
  };
  if (zero_start) {
    for (int i = threadIdx.x; i < n; i += kABottomThreads) {
      const float v = V.inv_theta * V.dinv[i] * V.def[i];
      V.d[i] = v;
      V.sol[i] = v;
    }
    __syncthreads();
  } else {
    step(0.0f, V.inv_theta);
  }
  for (int k = 1; k < V.degree; ++k) step(V.f1[k], V.f2[k]);
}

__device__ void bottom_a_spmv(int rows, const int* __restrict__ ptr, const int* __restrict__ col,
                              const float* __restrict__ val, const float* x, float* y, bool add) {
  for (int r = threadIdx.x; r < rows; r += kABottomThreads) {
    float t = 0.0f;
    const int e = ptr[r + 1];
    for (int k = ptr[r]; k < e; ++k) t += val[k] * x[col[k]];
    y[r] = add ? y[r] + t : t;
  }
  __syncthreads();
}

template <bool per_q>
__global__ void __launch_bounds__(kABottomThreads, 1) a_vcycle_bottom(const ABottomArgs args) {
  __shared__ ABottomArgs A;
  extern __shared__ float4 dyn4[];
  float* sm = reinterpret_cast<float*>(dyn4);
  if (threadIdx.x == 0) A = args;
  __syncthreads();
  const int K = A.n_levels - 1;
  const int n_top = A.lev[K].L.n_u;
  float* col_out = A.batch_out + (size_t)blockIdx.x * n_top;
  for (int l = 0; l <= K; ++l)
    for (int i = threadIdx.x; i < A.lev[l].L.n_u; i += kABottomThreads) sm[A.lev[l].off[0] + i] = A.lev[l].dinv[i];
  for (int i = threadIdx.x; i < n_top; i += kABottomThreads)
    sm[A.lev[K].off[2] + i] = i == (int)blockIdx.x ? 1.0f : 0.0f;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int l = 0; l <= K; ++l) {
      ABottomLevel& V = A.lev[l];
      V.dinv = sm + V.off[0];
      V.sol = sm + V.off[1];
      V.def = sm + V.off[2];
      V.d = sm + V.off[3];
      V.t = sm + V.off[4];
      V.E = sm + V.off[5];
    }
  }
  __syncthreads();
  // down: levels K .. 1 (one smoothing step each on the A block)
  for (int l = K; l >= 1; --l) {
    const ABottomLevel& V = A.lev[l];
    const ABottomLevel& C = A.lev[l - 1];
    bottom_a_chebyshev<per_q>(V, true);
    GatherArgs<float> a{};
    a.x = V.sol;
    a.b = V.def;
    a.y = V.t;
    bottom_a_apply<per_q>(V, EPI_RESID, a);
    for (int i = threadIdx.x; i < C.L.n_u; i += kABottomThreads) C.def[i] = 0.0f;
    __syncthreads();
    bottom_a_spmv(V.pt_rows, V.pt_ptr, V.pt_col, V.pt_val, V.t, C.def, false);
  }
  bottom_a_chebyshev<per_q>(A.lev[0], true);  // the coarse solve: the smoother
  for (int l = 1; l <= K; ++l) {
    const ABottomLevel& V = A.lev[l];
    const ABottomLevel& C = A.lev[l - 1];
    bottom_a_spmv(V.p_rows, V.p_ptr, V.p_col, V.p_val, C.sol, V.sol, true);
    bottom_a_chebyshev<per_q>(V, false);
  }
  for (int i = threadIdx.x; i < n_top; i += kABottomThreads) col_out[i] = A.lev[K].sol[i];
}

}  // namespace

int a_bottom_layout(ABottomArgs& A) {
  long off = 0;
  auto take = [&](long n) {
    const long o = off;
    off += (n + 3) / 4 * 4;
    return (int)o;
  };
  for (int l = 0; l < A.n_levels; ++l) {
    ABottomLevel& V = A.lev[l];
    for (int k = 0; k < 5; ++k) V.off[k] = take(V.L.n_u);
    V.off[5] = take((long)V.L.n_cells * 81);
  }
  return (int)(off * sizeof(float));
}

int a_bottom_reserve() {
  constexpr int kMaxDevices = 64;
  static int limit[kMaxDevices];
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
  if (limit[dev] > 0) return limit[dev];
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  const int want = optin - (int)sizeof(ABottomArgs) - 1024;
  if (want <= 0 ||
      cudaFuncSetAttribute(a_vcycle_bottom<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, want) != cudaSuccess ||
      cudaFuncSetAttribute(a_vcycle_bottom<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, want) != cudaSuccess)
    return 0;
  limit[dev] = want;
  return want;
}

void launch_a_vcycle_bottom_batch(const ABottomArgs& A, int smem_bytes, int n_cols, cudaStream_t s) {
  if (n_cols <= 0 || !A.batch_out) return;
  if (A.eta_per_q) a_vcycle_bottom<true><<<n_cols, kABottomThreads, smem_bytes, s>>>(A);
  else a_vcycle_bottom<false><<<n_cols, kABottomThreads, smem_bytes, s>>>(A);
  GB_CUDA(cudaGetLastError());
}

}  // namespace gb
