// The lower levels of the FP32 pressure-mass (Schur complement) V-cycle in one
// kernel launch on one thread block.
//
// On the coarse lattice levels of the mass V-cycle (at most a few hundred
// pressure nodes) every Chebyshev step, residual and transfer is a launch that
// does almost no work, and the ~38 launches per level cost their launch and
// drain latency each. This kernel runs levels 0..K of the cycle (pre-smoothing,
// residual, restriction, the coarse Chebyshev solve, prolongation and
// post-smoothing, in the order of the multi-launch cycle) inside one block,
// with __syncthreads() between dependent steps. The levels' per-cell mass
// matrices, diagonals and work vectors (about 170 KB for levels 0-3 of a
// lattice hierarchy: 1, 8, 64, 512 cells) are staged in shared memory once, so
// each step costs shared-memory rather than L2 latency; only the transfer
// matrices are read from global memory. Each step uses the same per-element
// arithmetic as the multi-launch kernels (mass_lattice_task and the
// vector-kernel expressions), so both paths compute the same values.
#include "ops.cuh"
#include "mass_bottom.cuh"

namespace gb {
namespace {

constexpr int kBottomThreads = 1024;

__device__ __forceinline__ void bottom_mass(const MassBottomLevel& V, int epi, const GatherArgs<float>& a) {
  const long tasks = (long)V.L.n_p * 8;
  for (long base = 0; base < tasks; base += kBottomThreads) {
    const long t = base + threadIdx.x;
    if (epi == EPI_RESID) mass_lattice_task<float, 3, EPI_RESID>(V.L, V.Mc, a, t);
    else mass_lattice_task<float, 3, EPI_CHEB_OUT>(V.L, V.Mc, a, t);
  }
  __syncthreads();
}

// PreconditionChebyshev from a zero start (zero_start) or one more sweep from x;
// the iterate alternates between x and t because the mass operator reads
// neighbouring entries (the multi-launch path does the same)
__device__ void bottom_chebyshev(const MassBottomLevel& V, bool zero_start) {
  const int n = V.L.n_p;
  float* x = V.sol;
  float* cur = x;
  auto step = [&](float f1, float f2) {
    float* nxt = cur == x ? V.t : x;
    GatherArgs<float> a{};
    a.x = cur;
    a.y = nxt;
    a.b = V.def;
    a.dinv = V.dinv;
    a.d = V.d;
    a.f1 = f1;
    a.f2 = f2;
    bottom_mass(V, EPI_CHEB_OUT, a);
    cur = nxt;
  };
  if (zero_start) {
    for (int i = threadIdx.x; i < n; i += kBottomThreads) {
      const float v = V.inv_theta * V.dinv[i] * V.def[i];
      V.d[i] = v;
      x[i] = v;
    }
    __syncthreads();
  } else {
    step(0.0f, V.inv_theta);
  }
  for (int k = 1; k < V.degree; ++k) step(V.f1[k], V.f2[k]);
  if (cur != x) {
    for (int i = threadIdx.x; i < n; i += kBottomThreads) x[i] = cur[i];
    __syncthreads();
  }
}

__device__ void bottom_spmv_add(int rows, const int* __restrict__ ptr, const int* __restrict__ col,
                                const float* __restrict__ val, const float* x, float* y) {
  for (int r = threadIdx.x; r < rows; r += kBottomThreads) {
    float t = 0.0f;
    const int e = ptr[r + 1];
    for (int k = ptr[r]; k < e; ++k) t += val[k] * x[col[k]];
    y[r] += t;
  }
  __syncthreads();
}

__device__ void bottom_zero(int n, float* y) {
  for (int i = threadIdx.x; i < n; i += kBottomThreads) y[i] = 0.0f;
  __syncthreads();
}

// Levels 0..K of the cycle on this block (A in shared memory, sm the dynamic
// shared memory of the level copies); the input is lev[K].def, the output
// lev[K].sol, both in global memory.
__device__ void bottom_levels(MassBottomArgs& A, int K, float* sm) {
  float* sol_out = A.lev[K].sol;
  // stage the mass matrices and diagonals of all levels and the top level's defect
  for (int l = 0; l <= K; ++l) {
    const MassBottomLevel& V = A.lev[l];
    const int n4 = V.L.n_cells * 16;  // 64 floats per cell
    const float4* src = reinterpret_cast<const float4*>(V.Mc);
    float4* dst = reinterpret_cast<float4*>(sm + V.off[0]);
    for (int i = threadIdx.x; i < n4; i += kBottomThreads) dst[i] = src[i];
    for (int i = threadIdx.x; i < V.L.n_p; i += kBottomThreads) sm[V.off[1] + i] = V.dinv[i];
  }
  // (past L1: in the cluster variant other blocks of the cluster wrote this defect)
  for (int i = threadIdx.x; i < A.lev[K].L.n_p; i += kBottomThreads) sm[A.lev[K].off[3] + i] = __ldcg(A.lev[K].def + i);
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int l = 0; l <= K; ++l) {
      MassBottomLevel& V = A.lev[l];
      V.gsol = V.sol;
      V.gdef = V.def;
      V.gd = V.d;
      V.gt = V.t;
      V.gMc = V.Mc;
      V.gdinv = V.dinv;
      V.Mc = sm + V.off[0];
      V.dinv = sm + V.off[1];
      V.sol = sm + V.off[2];
      V.def = sm + V.off[3];
      V.d = sm + V.off[4];
      V.t = sm + V.off[5];
    }
  }
  __syncthreads();
  // down: levels K .. 1
  for (int l = K; l >= 1; --l) {
    const MassBottomLevel& V = A.lev[l];
    const MassBottomLevel& C = A.lev[l - 1];
    bottom_chebyshev(V, true);
    for (int k = 1; k < V.steps; ++k) bottom_chebyshev(V, false);
    {
      GatherArgs<float> a{};
      a.x = V.sol;
      a.b = V.def;
      a.y = V.t;
      bottom_mass(V, EPI_RESID, a);
    }
    bottom_zero(C.L.n_p, C.def);
    bottom_spmv_add(V.pt_rows, V.pt_ptr, V.pt_col, V.pt_val, V.t, C.def);
    bottom_zero(C.L.n_p, C.sol);
  }
  // coarse level: the Chebyshev smoother as the coarse solver
  {
    const MassBottomLevel& V = A.lev[0];
    bottom_chebyshev(V, true);
    for (int k = 1; k < V.steps; ++k) bottom_chebyshev(V, false);
  }
  // up: levels 1 .. K
  for (int l = 1; l <= K; ++l) {
    const MassBottomLevel& V = A.lev[l];
    const MassBottomLevel& C = A.lev[l - 1];
    bottom_spmv_add(V.p_rows, V.p_ptr, V.p_col, V.p_val, C.sol, V.sol);
    for (int k = 0; k < V.steps; ++k) bottom_chebyshev(V, false);
  }
  for (int i = threadIdx.x; i < A.lev[K].L.n_p; i += kBottomThreads) sol_out[i] = A.lev[K].sol[i];
  __syncthreads();
  if (threadIdx.x == 0) {  // back to the global vectors for the caller
    for (int l = 0; l <= K; ++l) {
      MassBottomLevel& V = A.lev[l];
      V.sol = V.gsol;
      V.def = V.gdef;
      V.d = V.gd;
      V.t = V.gt;
      V.Mc = V.gMc;
      V.dinv = V.gdinv;
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBottomThreads) mass_vcycle_bottom(const MassBottomArgs args) {
  pdl_wait();
  // levels are indexed at run time: keep the arguments in shared memory rather
  // than a per-thread local copy of the parameter block
  __shared__ MassBottomArgs A;
  extern __shared__ float4 dyn4[];
  if (threadIdx.x == 0) A = args;
  __syncthreads();
  bottom_levels(A, A.n_levels - 1, reinterpret_cast<float*>(dyn4));
}

// ---------------------------------------------------------------------------
// Levels 0..K with the upper ones (Kb+1..K, a few thousand pressure nodes each)
// spread over a cluster of kClusterBlocks blocks: each Chebyshev step, residual
// and transfer is a loop over all the cluster's threads followed by a cluster
// barrier (barrier.cluster, release/acquire: the hardware barrier of the
// cluster, no spinning), with the level vectors in global memory (L2); loads of
// vectors that other blocks of the cluster wrote bypass L1 (ld.global.cg).
// Levels 0..Kb then run on block 0 alone (bottom_levels) while the others wait
// at the next cluster barrier. Per node the same arithmetic as the multi-launch
// kernels (row dot, lane reduction and epilogue of mass_lattice_task), so both
// paths give the same values. This replaces 37 launches per upper level.
constexpr int kClusterBlocks = 8;
constexpr int kClusterThreads = kClusterBlocks * kBottomThreads;

__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ int cluster_thread() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return (int)r * kBottomThreads + threadIdx.x;
}

template <int epi>
__device__ __forceinline__ void cluster_mass_task(const LevelView<float>& L, const float* __restrict__ Mc,
                                                  const GatherArgs<float>& a, long t) {
  constexpr int np = 8;
  const long g = t / np;
  const int s = (int)(t % np);
  const bool node_ok = g < L.n_p;
  const int node = node_ok ? (int)g : 0;
  const int gc[3] = {node % L.Np[0], (node / L.Np[0]) % L.Np[1], node / (L.Np[0] * L.Np[1])};
  int c[3] = {0, 0, 0}, l = 0;
  bool ok = node_ok;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int bit = (s >> d) & 1;
    c[d] = gc[d] - 1 + bit;
    ok = ok && c[d] >= 0 && c[d] < L.nc[d];
    l += (bit ? 0 : 1) << d;
  }
  float sum = 0.0f;
  if (ok) {
    const int cell = (c[2] * L.nc[1] + c[1]) * L.nc[0] + c[0];
    float r[np];
    load_row<float, np>(Mc + ((size_t)cell * np + l) * np, r);
    const int p0 = (c[2] * L.Np[1] + c[1]) * L.Np[0] + c[0];
#pragma unroll
    for (int j = 0; j < np; ++j) sum += r[j] * __ldcg(a.x + p0 + structured_pnode_offset<3>(L.Np, j));
  }
#pragma unroll
  for (int o = 1; o < np; o <<= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (node_ok && s == 0) {
    if (epi == EPI_RESID) {
      a.y[g] = __ldcg(a.b + g) - sum;
    } else {  // EPI_CHEB_OUT
      const float xg = __ldcg(a.x + g);
      const float dn = a.f1 * __ldcg(a.d + g) + a.f2 * a.dinv[g] * (__ldcg(a.b + g) - sum);
      a.d[g] = dn;
      a.y[g] = xg + dn;
    }
  }
}

__device__ void cluster_mass(const MassBottomLevel& V, int epi, const GatherArgs<float>& a) {
  const long tasks = (long)V.L.n_p * 8;
  const int gt = cluster_thread();
  for (long base = 0; base < tasks; base += kClusterThreads) {
    if (epi == EPI_RESID) cluster_mass_task<EPI_RESID>(V.L, V.Mc, a, base + gt);
    else cluster_mass_task<EPI_CHEB_OUT>(V.L, V.Mc, a, base + gt);
  }
  cluster_sync();
}

__device__ void cluster_chebyshev(const MassBottomLevel& V, bool zero_start) {
  const int n = V.L.n_p;
  const int gt = cluster_thread();
  float* x = V.sol;
  float* cur = x;
  auto step = [&](float f1, float f2) {
    float* nxt = cur == x ? V.t : x;
    GatherArgs<float> a{};
    a.x = cur;
    a.y = nxt;
    a.b = V.def;
    a.dinv = V.dinv;
    a.d = V.d;
    a.f1 = f1;
    a.f2 = f2;
    cluster_mass(V, EPI_CHEB_OUT, a);
    cur = nxt;
  };
  if (zero_start) {
    for (int i = gt; i < n; i += kClusterThreads) {
      const float v = V.inv_theta * V.dinv[i] * __ldcg(V.def + i);
      V.d[i] = v;
      x[i] = v;
    }
    cluster_sync();
  } else {
    step(0.0f, V.inv_theta);
  }
  for (int k = 1; k < V.degree; ++k) step(V.f1[k], V.f2[k]);
  if (cur != x) {
    for (int i = gt; i < n; i += kClusterThreads) x[i] = __ldcg(cur + i);
    cluster_sync();
  }
}

__device__ void cluster_spmv_add(int rows, const int* __restrict__ ptr, const int* __restrict__ col,
                                 const float* __restrict__ val, const float* x, float* y) {
  for (int r = cluster_thread(); r < rows; r += kClusterThreads) {
    float t = 0.0f;
    const int e = ptr[r + 1];
    for (int k = ptr[r]; k < e; ++k) t += val[k] * __ldcg(x + col[k]);
    y[r] = __ldcg(y + r) + t;
  }
  cluster_sync();
}

__device__ void cluster_zero(int n, float* y) {
  for (int i = cluster_thread(); i < n; i += kClusterThreads) y[i] = 0.0f;
  cluster_sync();
}

__global__ void __cluster_dims__(kClusterBlocks, 1, 1) __launch_bounds__(kBottomThreads)
    mass_vcycle_cluster(const MassBottomArgs args, int Kb) {
  pdl_wait();
  __shared__ MassBottomArgs A;
  extern __shared__ float4 dyn4[];
  if (threadIdx.x == 0) A = args;
  __syncthreads();
  const int K = A.n_levels - 1;
  for (int l = K; l > Kb; --l) {
    const MassBottomLevel& V = A.lev[l];
    const MassBottomLevel& C = A.lev[l - 1];
    cluster_chebyshev(V, true);
    for (int k = 1; k < V.steps; ++k) cluster_chebyshev(V, false);
    {
      GatherArgs<float> a{};
      a.x = V.sol;
      a.b = V.def;
      a.y = V.t;
      cluster_mass(V, EPI_RESID, a);
    }
    cluster_zero(C.L.n_p, C.def);
    cluster_spmv_add(V.pt_rows, V.pt_ptr, V.pt_col, V.pt_val, V.t, C.def);
    cluster_zero(C.L.n_p, C.sol);
  }
  unsigned rank;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
  if (rank == 0) bottom_levels(A, Kb, reinterpret_cast<float*>(dyn4));
  cluster_sync();
  for (int l = Kb + 1; l <= K; ++l) {
    const MassBottomLevel& V = A.lev[l];
    const MassBottomLevel& C = A.lev[l - 1];
    cluster_spmv_add(V.p_rows, V.p_ptr, V.p_col, V.p_val, C.sol, V.sol);
    for (int k = 0; k < V.steps; ++k) cluster_chebyshev(V, false);
  }
}

}  // namespace

int mass_bottom_layout(MassBottomArgs& A) {
  long off = 0;
  auto take = [&](long n) {
    const long o = off;
    off += (n + 3) / 4 * 4;  // 16-byte aligned pieces
    return (int)o;
  };
  for (int l = 0; l < A.n_levels; ++l) {
    MassBottomLevel& V = A.lev[l];
    V.off[0] = take((long)V.L.n_cells * 64);
    for (int k = 1; k < 6; ++k) V.off[k] = take(V.L.n_p);
  }
  return (int)(off * sizeof(float));
}

int mass_bottom_reserve() {
  constexpr int kMaxDevices = 64;
  static int limit[kMaxDevices];  // per device; 0 = not set yet
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
  if (limit[dev] > 0) return limit[dev];
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  const int want = optin - (int)sizeof(MassBottomArgs) - 1024;
  if (want <= 0 ||
      cudaFuncSetAttribute(mass_vcycle_bottom, cudaFuncAttributeMaxDynamicSharedMemorySize, want) != cudaSuccess)
    return 0;
  limit[dev] = want;
  return want;
}

void launch_mass_vcycle_bottom(const MassBottomArgs& A, int smem_bytes, cudaStream_t s) {
  mass_vcycle_bottom<<<1, kBottomThreads, smem_bytes, s>>>(A);
}

int mass_cluster_reserve() {
  constexpr int kMaxDevices = 64;
  static int limit[kMaxDevices];  // per device; 0 = not set yet, -1 = unavailable
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
  if (limit[dev] != 0) return limit[dev] > 0 ? limit[dev] : 0;
  const int want = mass_bottom_reserve();
  if (want <= 0 ||
      cudaFuncSetAttribute(mass_vcycle_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, want) != cudaSuccess) {
    limit[dev] = -1;
    return 0;
  }
  limit[dev] = want;
  return want;
}

void launch_mass_vcycle_cluster(const MassBottomArgs& A, int bottom_top, int smem_bytes, cudaStream_t s) {
  mass_vcycle_cluster<<<kClusterBlocks, kBottomThreads, smem_bytes, s>>>(A, bottom_top);
}

}  // namespace gb
