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

__global__ void __launch_bounds__(kBottomThreads) mass_vcycle_bottom(const MassBottomArgs args) {
  pdl_wait();
  // levels are indexed at run time: keep the arguments in shared memory rather
  // than a per-thread local copy of the parameter block
  __shared__ MassBottomArgs A;
  extern __shared__ float4 dyn4[];
  float* sm = reinterpret_cast<float*>(dyn4);
  if (threadIdx.x == 0) A = args;
  __syncthreads();
  const int K = A.n_levels - 1;
  const int n_top = A.lev[K].L.n_p;
  float* sol_out = A.batch_out ? A.batch_out + (size_t)blockIdx.x * n_top : A.lev[K].sol;
  // stage the mass matrices and diagonals of all levels and the top level's defect
  for (int l = 0; l <= K; ++l) {
    const MassBottomLevel& V = A.lev[l];
    const int n4 = V.L.n_cells * 16;  // 64 floats per cell
    const float4* src = reinterpret_cast<const float4*>(V.Mc);
    float4* dst = reinterpret_cast<float4*>(sm + V.off[0]);
    for (int i = threadIdx.x; i < n4; i += kBottomThreads) dst[i] = src[i];
    for (int i = threadIdx.x; i < V.L.n_p; i += kBottomThreads) sm[V.off[1] + i] = V.dinv[i];
  }
  for (int i = threadIdx.x; i < n_top; i += kBottomThreads)
    sm[A.lev[K].off[3] + i] = A.batch_out ? (i == (int)blockIdx.x ? 1.0f : 0.0f) : A.lev[K].def[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int l = 0; l <= K; ++l) {
      MassBottomLevel& V = A.lev[l];
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

void launch_mass_vcycle_bottom_batch(const MassBottomArgs& A, int smem_bytes, int n_cols, cudaStream_t s) {
  if (n_cols <= 0 || !A.batch_out) return;
  mass_vcycle_bottom<<<n_cols, kBottomThreads, smem_bytes, s>>>(A);
  GB_CUDA(cudaGetLastError());
}

namespace {
// 32 rows per block, the columns split over 16 warps: lane = row, warp = slice of
// columns; the 16 partial sums of a row are added in slice order
constexpr int kGemvSlices = 16;
constexpr int kGemvBatch = 16;
__global__ void __launch_bounds__(32 * kGemvSlices) dense_gemv_colmajor(int n, const float* __restrict__ B,
                                                                       const float* __restrict__ x,
                                                                       float* __restrict__ y) {
  __shared__ float part[kGemvSlices][32];
  const int lane = threadIdx.x & 31, slice = threadIdx.x >> 5;
  const int row = blockIdx.x * 32 + lane;
  const int chunk = (n + kGemvSlices - 1) / kGemvSlices;
  const int j0 = slice * chunk, j1 = min(n, j0 + chunk);
  // The matrix entries are loaded kGemvBatch at a time before they are added
  // (in column order, as one at a time would), so a thread keeps kGemvBatch
  // loads in flight; the matrix is fixed over a V-cycle, so the first batch is
  // loaded before pdl_wait and overlaps the preceding kernel.
  float bv[kGemvBatch];
  const bool first = row < n && j0 + kGemvBatch <= j1;
  if (first) {
#pragma unroll
    for (int u = 0; u < kGemvBatch; ++u) bv[u] = B[(size_t)(j0 + u) * n + row];
  }
  pdl_wait();
  float acc = 0.0f;
  if (row < n) {
    int j = j0;
    if (first) {
#pragma unroll
      for (int u = 0; u < kGemvBatch; ++u) acc += bv[u] * x[j0 + u];
      j += kGemvBatch;
    }
    for (; j + kGemvBatch <= j1; j += kGemvBatch) {
#pragma unroll
      for (int u = 0; u < kGemvBatch; ++u) bv[u] = B[(size_t)(j + u) * n + row];
#pragma unroll
      for (int u = 0; u < kGemvBatch; ++u) acc += bv[u] * x[j + u];
    }
    for (; j < j1; ++j) acc += B[(size_t)j * n + row] * x[j];
  }
  part[slice][lane] = acc;
  __syncthreads();
  if (slice == 0 && row < n) {
    float t = 0.0f;
#pragma unroll
    for (int k = 0; k < kGemvSlices; ++k) t += part[k][lane];
    y[row] = t;
  }
}
}  // namespace

namespace {
template <int epi>
__global__ void __launch_bounds__(kMassLatticeThreads) k_mass_lattice_batched(LevelView<float> L,
                                                                              const float* __restrict__ Mc,
                                                                              GatherArgs<float> a) {
  const size_t off = (size_t)blockIdx.y * L.n_p;
  a.x += off;
  if (a.y) a.y += off;
  if (a.b) a.b += off;
  if (a.d) a.d += off;
  mass_lattice_task<float, 3, epi>(L, Mc, a, blockIdx.x * (long)blockDim.x + threadIdx.x);
}
__global__ void k_cheb_first_batched(long n, long total, const float* __restrict__ b, const float* __restrict__ dinv,
                                     float f2, float* __restrict__ d, float* __restrict__ x) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const float v = f2 * dinv[i % n] * b[i];
    d[i] = v;
    x[i] = v;
  }
}
__global__ void k_copy_batched(long total, const float* __restrict__ x, float* __restrict__ y) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) y[i] = x[i];
}
__global__ void k_unit_columns(long n, long total, float* __restrict__ x) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
    x[i] = (i % n) == (i / n) ? 1.0f : 0.0f;
}
__global__ void k_spmv_batched(int rows, const int* __restrict__ ptr, const int* __restrict__ col,
                               const float* __restrict__ val, const float* __restrict__ x, long nx,
                               float* __restrict__ y, long ny, int add) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const float* xc = x + (size_t)blockIdx.y * nx;
  float t = 0.0f;
  for (int k = ptr[r]; k < ptr[r + 1]; ++k) t += val[k] * xc[col[k]];
  float* yc = y + (size_t)blockIdx.y * ny;
  yc[r] = add ? yc[r] + t : t;
}
int flat_grid(long total) {
  long b = (total + 255) / 256;
  if (b > 152L * 32) b = 152L * 32;
  return (int)(b < 1 ? 1 : b);
}
}  // namespace

void launch_mass_lattice_batched(const LevelView<float>& L, const float* Mc, int epi, const GatherArgs<float>& a,
                                 int m, cudaStream_t s) {
  const long tasks = (long)L.n_p * 8;
  const dim3 g((unsigned)((tasks + kMassLatticeThreads - 1) / kMassLatticeThreads), (unsigned)m);
  if (epi == EPI_RESID) k_mass_lattice_batched<EPI_RESID><<<g, kMassLatticeThreads, 0, s>>>(L, Mc, a);
  else k_mass_lattice_batched<EPI_CHEB_OUT><<<g, kMassLatticeThreads, 0, s>>>(L, Mc, a);
  GB_CUDA(cudaGetLastError());
}
void launch_cheb_first_batched(long n, int m, const float* b, const float* dinv, float f2, float* d, float* x,
                               cudaStream_t s) {
  const long total = n * m;
  k_cheb_first_batched<<<flat_grid(total), 256, 0, s>>>(n, total, b, dinv, f2, d, x);
}
void launch_copy_batched(long n, int m, const float* x, float* y, cudaStream_t s) {
  k_copy_batched<<<flat_grid(n * m), 256, 0, s>>>(n * m, x, y);
}
void launch_unit_columns(long n, int m, float* x, cudaStream_t s) {
  k_unit_columns<<<flat_grid(n * m), 256, 0, s>>>(n, n * m, x);
}
void launch_spmv_batched(int rows, const int* ptr, const int* col, const float* val, const float* x, long nx,
                         float* y, long ny, int m, bool add, cudaStream_t s) {
  if (rows <= 0 || m <= 0) return;
  const dim3 g((unsigned)((rows + 255) / 256), (unsigned)m);
  k_spmv_batched<<<g, 256, 0, s>>>(rows, ptr, col, val, x, nx, y, ny, add ? 1 : 0);
  GB_CUDA(cudaGetLastError());
}

void launch_dense_gemv_colmajor(int n, const float* B, const float* x, float* y, cudaStream_t s) {
  if (n <= 0) return;
  dense_gemv_colmajor<<<(n + 31) / 32, 32 * kGemvSlices, 0, s>>>(n, B, x, y);
}

}  // namespace gb
