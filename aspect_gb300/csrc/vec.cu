// Vector kernels: grid-stride, vectorisable element-wise updates and
// deterministic fixed-grid reductions.
#include "vec.cuh"

namespace gb {

namespace {
constexpr int kThreads = 256;
inline int grid_for(long n) {
  long b = (n + kThreads - 1) / kThreads;
  if (b > 152L * 16) b = 152L * 16;
  return (int)(b < 1 ? 1 : b);
}
inline void count() { ++VecCounter::launches(); }
}  // namespace

template <typename T>
__global__ void k_axpby(long n, T a, const T* __restrict__ x, T b, T* __restrict__ y) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}
template <typename T>
void v_axpby(long n, T a, const T* x, T b, T* y, cudaStream_t s) {
  if (n <= 0) return;
  k_axpby<<<grid_for(n), kThreads, 0, s>>>(n, a, x, b, y);
  count();
}

template <typename T>
void v_copy(long n, const T* x, T* y, cudaStream_t s) {
  if (n <= 0) return;
  GB_CUDA(cudaMemcpyAsync(y, x, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
}

template <typename T>
__global__ void k_scale(long n, T a, T* __restrict__ y) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] *= a;
}
template <typename T>
void v_scale(long n, T a, T* y, cudaStream_t s) {
  if (n <= 0) return;
  k_scale<<<grid_for(n), kThreads, 0, s>>>(n, a, y);
  count();
}

template <typename T>
__global__ void k_zero(long n, T* __restrict__ y) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] = T(0);
}
template <typename T>
void v_zero(long n, T* y, cudaStream_t s) {
  if (n <= 0) return;
  k_zero<<<grid_for(n), kThreads, 0, s>>>(n, y);
  count();
}

template <typename Ts, typename Td>
__global__ void k_cast(long n, const Ts* __restrict__ x, Td* __restrict__ y) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = (Td)x[i];
}
template <typename Ts, typename Td>
void v_cast(long n, const Ts* x, Td* y, cudaStream_t s) {
  if (n <= 0) return;
  k_cast<<<grid_for(n), kThreads, 0, s>>>(n, x, y);
  count();
}

// The diagonal inverse (fixed over a V-cycle, written only by the
// preconditioner set-up) of the thread's first entry is loaded before pdl_wait,
// overlapping the preceding kernel under the V-cycle graphs' programmatic edges.
template <typename T>
__global__ void k_cheb_first(long n, const T* __restrict__ b, const T* __restrict__ dinv, T f2, T* __restrict__ d,
                             T* __restrict__ x) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const T d0 = i < n ? dinv[i] : T(0);
  pdl_wait();
  if (i < n) {
    const T v = f2 * d0 * b[i];
    d[i] = v;
    x[i] = v;
  }
  for (i += (long)gridDim.x * blockDim.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const T v = f2 * dinv[i] * b[i];
    d[i] = v;
    x[i] = v;
  }
}
template <typename T>
void v_cheb_first(long n, const T* b, const T* dinv, T f2, T* d, T* x, cudaStream_t s) {
  if (n <= 0) return;
  k_cheb_first<<<grid_for(n), kThreads, 0, s>>>(n, b, dinv, f2, d, x);
  count();
}

template <typename T>
__global__ void k_cheb_step(long n, const T* __restrict__ b, const T* __restrict__ t, const T* __restrict__ dinv,
                            T f1, T f2, T* __restrict__ d, T* __restrict__ x) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const T v = f1 * d[i] + f2 * dinv[i] * (b[i] - t[i]);
    d[i] = v;
    x[i] += v;
  }
}
template <typename T>
void v_cheb_step(long n, const T* b, const T* t, const T* dinv, T f1, T f2, T* d, T* x, cudaStream_t s) {
  if (n <= 0) return;
  k_cheb_step<<<grid_for(n), kThreads, 0, s>>>(n, b, t, dinv, f1, f2, d, x);
  count();
}

template <typename T>
__global__ void k_sub(long n, const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ o) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    o[i] = a[i] - b[i];
}
template <typename T>
void v_sub(long n, const T* a, const T* b, T* out, cudaStream_t s) {
  if (n <= 0) return;
  k_sub<<<grid_for(n), kThreads, 0, s>>>(n, a, b, out);
  count();
}

template <typename T>
__global__ void k_copy_indexed(long m, const int* __restrict__ idx, const T* __restrict__ src, T* __restrict__ dst) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += (long)gridDim.x * blockDim.x)
    dst[idx[i]] = src[idx[i]];
}
template <typename T>
void v_copy_indexed(long m, const int* idx, const T* src, T* dst, cudaStream_t s) {
  if (m <= 0) return;
  k_copy_indexed<<<grid_for(m), kThreads, 0, s>>>(m, idx, src, dst);
  count();
}
template <typename T>
__global__ void k_zero_indexed(long m, const int* __restrict__ idx, T* __restrict__ dst) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += (long)gridDim.x * blockDim.x)
    dst[idx[i]] = T(0);
}
template <typename T>
void v_zero_indexed(long m, const int* idx, T* dst, cudaStream_t s) {
  if (m <= 0) return;
  k_zero_indexed<<<grid_for(m), kThreads, 0, s>>>(m, idx, dst);
  count();
}

template <typename Ts, typename Td>
__global__ void k_perm_scatter(long n, const int* __restrict__ perm, const Ts* __restrict__ in, Td* __restrict__ out) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[perm[i]] = (Td)in[i];
}
template <typename Ts, typename Td>
void v_permute_scatter(long n, const int* perm, const Ts* in, Td* out, cudaStream_t s) {
  if (n <= 0) return;
  k_perm_scatter<<<grid_for(n), kThreads, 0, s>>>(n, perm, in, out);
  count();
}
template <typename Ts, typename Td>
__global__ void k_perm_gather(long n, const int* __restrict__ perm, const Ts* __restrict__ in, Td* __restrict__ out) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = (Td)in[perm[i]];
}
template <typename Ts, typename Td>
void v_permute_gather(long n, const int* perm, const Ts* in, Td* out, cudaStream_t s) {
  if (n <= 0) return;
  k_perm_gather<<<grid_for(n), kThreads, 0, s>>>(n, perm, in, out);
  count();
}

template <typename T>
__global__ void k_spmv_add(long rows, const int* __restrict__ ptr, const int* __restrict__ col,
                           const T* __restrict__ val, const T* __restrict__ x, T* __restrict__ y) {
  pdl_wait();
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < rows; r += (long)gridDim.x * blockDim.x) {
    T t = T(0);
    const int e = ptr[r + 1];
    for (int k = ptr[r]; k < e; ++k) t += val[k] * x[col[k]];
    y[r] += t;
  }
}
template <typename T>
void v_spmv_add(long rows, const int* ptr, const int* col, const T* val, const T* x, T* y, cudaStream_t s) {
  if (rows <= 0) return;
  k_spmv_add<<<grid_for(rows), kThreads, 0, s>>>(rows, ptr, col, val, x, y);
  count();
}

// y = A x on rows [0, rows), y = 0 on [rows, n): the zero fill and the product of
// a restriction in one launch (the same sums as v_zero then v_spmv_add)
template <typename T>
__global__ void k_spmv_set(long rows, long n, const int* __restrict__ ptr, const int* __restrict__ col,
                           const T* __restrict__ val, const T* __restrict__ x, T* __restrict__ y) {
  pdl_wait();
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    T t = T(0);
    if (r < rows) {
      const int e = ptr[r + 1];
      for (int k = ptr[r]; k < e; ++k) t += val[k] * x[col[k]];
    }
    y[r] = T(0) + t;
  }
}
template <typename T>
void v_spmv_set(long rows, long n, const int* ptr, const int* col, const T* val, const T* x, T* y, cudaStream_t s) {
  if (n <= 0) return;
  k_spmv_set<<<grid_for(n), kThreads, 0, s>>>(rows, n, ptr, col, val, x, y);
  count();
}

// ---------------------------------------------------------------- reductions
// Block sums of acc[0..K) into partial[i * slot_stride + blockIdx.x] for output
// slots i < nk; slot i takes accumulator i, except that slot `moved` (when >= 0)
// takes accumulator K-1 (so callers never index acc at run time).
template <int K>
__device__ __forceinline__ void block_reduce_store(double (&acc)[K], int nk, double* partial, int slot_stride,
                                                   int moved = -1) {
  // Through shared memory rather than a shuffle tree per value: on this GPU the
  // FP64 additions are the cost, and a tree does five warp-wide additions per
  // value in every warp; here 8 segments of 32 threads are summed by nk x 8
  // threads, then each value's 8 segment sums by one thread (fixed order).
  __shared__ double sh[K][kDotThreads];
  __shared__ double seg[K][kDotThreads / 32];
#pragma unroll
  for (int j = 0; j < K; ++j) sh[j][threadIdx.x] = acc[j];
  __syncthreads();
  constexpr int nseg = kDotThreads / 32;
  if ((int)threadIdx.x < nk * nseg) {
    const int o = threadIdx.x / nseg, sg = threadIdx.x % nseg;
    const int src = o == moved ? K - 1 : o;
    double t = 0;
#pragma unroll 8
    for (int l = 0; l < 32; ++l) t += sh[src][sg * 32 + l];
    seg[src][sg] = t;
  }
  __syncthreads();
  if ((int)threadIdx.x < nk) {
    const int src = (int)threadIdx.x == moved ? K - 1 : (int)threadIdx.x;
    double t = 0;
#pragma unroll
    for (int w = 0; w < nseg; ++w) t += seg[src][w];
    partial[threadIdx.x * slot_stride + blockIdx.x] = t;
  }
}

// The block of a reduction that arrives last (a counter per chunk, reset by
// that block) sums the per-block partials itself, in the same fixed order a
// separate finishing launch would: lane l of a warp adds blocks l, l+32, ...,
// then lane 0 adds the 32 lane sums in lane order. Deterministic, one launch.
__device__ __forceinline__ bool arrive_last(unsigned* counter) {
  __shared__ bool last;
  __threadfence();  // this block's partials are visible before its arrival counts
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}
__device__ __forceinline__ void finish_partials(const double* part, int nk, double* out, unsigned* counter,
                                                int nb = kDotBlocks) {
  __shared__ double sh[kDotThreads / 32][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = wid; j < nk; j += kDotThreads / 32) {
    // lane l adds blocks l, l + 32, ... in that order; eight loads are issued
    // before they are added, so the finishing block does not wait on one load
    // at a time
    double t = 0;
    const double* pj = part + (size_t)j * nb;
    int b = lane;
    for (; b + 7 * 32 < nb; b += 8 * 32) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = __ldcg(pj + b + u * 32);
#pragma unroll
      for (int u = 0; u < 8; ++u) t += v[u];
    }
    for (; b < nb; b += 32) t += __ldcg(pj + b);
    sh[wid][lane] = t;
    __syncwarp();
    if (lane == 0) {
      double v = 0;
      for (int l = 0; l < 32; ++l) v += sh[wid][l];
      out[j] = v;
    }
    __syncwarp();
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// blockIdx.y = chunk of kDotChunk vectors; the chunk that ends at k also forms
// <w, w>. gridDim.x blocks per chunk (chosen so that all chunks run in about
// one wave); each thread takes two elements per step, so eighteen independent
// loads are in flight per thread. FP64 BLAS-1 on this GPU is bound by the
// FP64 pipe (one FMA per basis entry), not by HBM, so keeping it fed is what
// matters.
__global__ void __launch_bounds__(kDotThreads, 3) k_multidot(long n, const double* __restrict__ w,
                                                          const double* __restrict__ V, long ld, int k,
                                                          int with_norm, double* __restrict__ out,
                                                          double* __restrict__ partial, unsigned* counters,
                                                          const int* __restrict__ active) {
  pdl_wait();
  if (active && *active == 0) return;
  const int nb = gridDim.x;
  const int chunk = blockIdx.y;
  const int j0 = chunk * kDotChunk;
  const int kk = k - j0 < kDotChunk ? k - j0 : kDotChunk;
  const int norm = (with_norm && j0 + kk == k) ? 1 : 0;
  const double* __restrict__ Vc = V + (size_t)j0 * ld;
  double acc[kDotChunk + 1];
#pragma unroll
  for (int j = 0; j <= kDotChunk; ++j) acc[j] = 0;
  const long stride = (long)nb * blockDim.x;
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {
    const double wa = w[i], wb = w[i + stride];
    double va[kDotChunk], vb[kDotChunk];
#pragma unroll
    for (int j = 0; j < kDotChunk; ++j)
      if (j < kk) {
        va[j] = Vc[j * ld + i];
        vb[j] = Vc[j * ld + i + stride];
      }
#pragma unroll
    for (int j = 0; j < kDotChunk; ++j)
      if (j < kk) {
        acc[j] += wa * va[j];
        acc[j] += wb * vb[j];
      }
    if (norm) {
      acc[kDotChunk] += wa * wa;
      acc[kDotChunk] += wb * wb;
    }
  }
  if (i < n) {
    const double wi = w[i];
#pragma unroll
    for (int j = 0; j < kDotChunk; ++j)
      if (j < kk) acc[j] += wi * Vc[j * ld + i];
    if (norm) acc[kDotChunk] += wi * wi;
  }
  double* part = partial + (size_t)chunk * (kDotChunk + 1) * nb;
  block_reduce_store<kDotChunk + 1>(acc, kk + norm, part, nb, norm ? kk : -1);
  if (arrive_last(counters + chunk))
    finish_partials(part, kk + norm, out + j0, counters + chunk, nb);
}

// Blocks per chunk: all chunks together about 3 x kDotBlocks blocks (three
// resident per SM at 70 registers), at most kDotBlocks per chunk. FP64
// arithmetic (one FMA per basis entry) bounds the multi-dot on this GPU, so the
// grid aims at an even share of it per SM.
int multidot_blocks(int chunks) {
  int nb = 3 * kDotBlocks / (chunks > 0 ? chunks : 1);
  if (nb > kDotBlocks) nb = kDotBlocks;
  if (nb < 1) nb = 1;
  return nb;
}

void v_multidot(long n, const double* w, const double* V, long ld, int k, bool with_norm, double* out_dev,
                double* partial, cudaStream_t s, const int* active) {
  unsigned* counters = reinterpret_cast<unsigned*>(partial + kDotPartialDoubles);
  if (k == 0) {
    if (!with_norm) return;
    k_multidot<<<dim3(kDotBlocks, 1), kDotThreads, 0, s>>>(n, w, V, ld, 0, 1, out_dev, partial, counters, active);
    VecCounter::launches() += 1;
    return;
  }
  constexpr int per_launch = kDotMaxChunks * kDotChunk;
  for (int done = 0; done < k; done += per_launch) {
    const int kl = k - done < per_launch ? k - done : per_launch;
    const int norm = (with_norm && done + kl == k) ? 1 : 0;
    const int chunks = (kl + kDotChunk - 1) / kDotChunk;
    k_multidot<<<dim3(multidot_blocks(chunks), chunks), kDotThreads, 0, s>>>(n, w, V + (size_t)done * ld, ld, kl,
                                                                             norm, out_dev + done, partial,
                                                                             counters, active);
    VecCounter::launches() += 1;
  }
}

// exponent of the power-of-two scale for the float-pair passes of the next
// Arnoldi step: that of |w before| of this step
__device__ __forceinline__ int gs_shift_of(double norm) {
  const int e = norm > 0 && isfinite(norm) ? ilogb(norm) : 0;
  return e < -1000 ? -1000 : (e > 1000 ? 1000 : e);
}

// One classical Gram-Schmidt pass of Arnoldi step j after its multi-dot
// (dots[0..j] = V^T w, and for pass 0 dots[j+1] = <w, w> before): w -= V dots
// with <w, w> after formed in the same sweep (fixed-grid reduction); the block
// that finishes the reduction also does the step's bookkeeping:
//   pass 0: h[0..j] = dots, arn[1] = |w before|; pass 1: h[0..j] += dots;
//   h[j+1] = |w| and arn[2] = 1 / |w| (1 when |w| = 0);
//   pass 0: *need2 = 1 when |w| <= 0.7 |w before| (the second pass runs).
// Pass 1 does nothing when *need2 == 0. kCgsPerThread elements per thread in
// full warps (a partly filled warp costs the FP64 pipe as much as a full one);
// the coefficients are read from shared memory and subtracted (no negated copy).
constexpr int kCgsPerThread = 4;
constexpr int kCgsCached = 1024;
__global__ void __launch_bounds__(kDotThreads) k_cgs_update(long n, int j, int pass, const double* __restrict__ dots,
                                                            const double* __restrict__ V, long ld,
                                                            double* __restrict__ w, double* __restrict__ h,
                                                            double* __restrict__ arn, int* __restrict__ need2,
                                                            double* __restrict__ partial, unsigned* counter,
                                                            int* __restrict__ shift) {
  pdl_wait();
  if (pass == 1 && *need2 == 0) return;
  const int k = j + 1;
  const int kc = k < kCgsCached ? k : kCgsCached;
  __shared__ double c[kCgsCached];
  for (int i = threadIdx.x; i < kc; i += blockDim.x) c[i] = dots[i];
  __syncthreads();
  double acc[1] = {0};
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride) {
    double t = w[i];
    int q = 0;
    for (; q + 8 <= kc; q += 8) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = V[(size_t)(q + u) * ld + i];
#pragma unroll
      for (int u = 0; u < 8; ++u) t -= c[q + u] * v[u];
    }
    for (; q < kc; ++q) t -= c[q] * V[(size_t)q * ld + i];
    for (; q < k; ++q) t -= dots[q] * V[(size_t)q * ld + i];
    w[i] = t;
    acc[0] += t * t;
  }
  block_reduce_store<1>(acc, 1, partial, gridDim.x);
  if (!arrive_last(counter)) return;
  finish_partials(partial, 1, arn, counter, gridDim.x);  // arn[0] = <w, w>
  for (int i = threadIdx.x; i < k; i += blockDim.x) h[i] = pass == 0 ? dots[i] : h[i] + dots[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    if (pass == 0) arn[1] = sqrt(dots[k]);
    if (pass == 0 && shift) *shift = gs_shift_of(arn[1]);
    const double nw = sqrt(arn[0]);
    h[k] = nw;
    arn[2] = 1.0 / (nw > 0 ? nw : 1.0);
    if (pass == 0) *need2 = nw > 0.7 * arn[1] ? 0 : 1;
  }
}

void v_cgs_update(long n, int j, int pass, const double* dots, const double* V, long ld, double* w, double* h,
                  double* arn, int* need2, double* partial, cudaStream_t s, int* shift) {
  unsigned* counter = reinterpret_cast<unsigned*>(partial + kDotPartialDoubles) + kDotMaxChunks;
  long nb = (n + (long)kDotThreads * kCgsPerThread - 1) / ((long)kDotThreads * kCgsPerThread);
  const long max_nb = kDotPartialDoubles;  // one partial per block
  if (nb > max_nb) nb = max_nb;
  if (nb < 1) nb = 1;
  k_cgs_update<<<(int)nb, kDotThreads, 0, s>>>(n, j, pass, dots, V, ld, w, h, arn, need2, partial, counter, shift);
  VecCounter::launches() += 1;
}

// ---------------------------------------------------------------- double-float Gram-Schmidt
// The same classical Gram-Schmidt passes with the k n multiply-adds of a step on
// the FP32 pipe. Each basis vector is kept twice: in FP64 (what the preconditioner
// reads) and as a pair of floats (h, l) per entry whose sum is exactly the FP64
// entry (df_split_basis canonicalises the FP64 entry to that sum when the vector
// is formed). w is split the same way after an exact power-of-two scaling by the
// previous step's |w| (so its entries stay far inside the FP32 range), and
// products and sums are carried as unevaluated float pairs: Dekker's product
// through an FMA and Knuth's TwoSum (about 46 significant bits; the cross term
// l l' of a product, 2^-48 relative, is dropped). On this GPU the FP64 pipe
// retires about two FMAs per clock per SM and the FP32 pipe 128, so the passes
// run at the HBM rate of the float-pair basis (8 bytes per entry) instead of at
// the FP64 FMA rate. Block partials are converted to FP64 and summed from there
// on in FP64, in the fixed order of the FP64 kernels (deterministic).

// x 2^-sh as h + l: h = x 2^-sh with its binary64 significand truncated to 24
// bits, l = the next 23 bits (truncated), so |x 2^-sh - (h + l)| < 2^-46 |x 2^-sh|.
// Integer operations on the binary64 fields only (no FP64 instruction). With e
// the binary32 biased exponent of x 2^-sh: e >= 255 gives h = +-inf (an entry
// 2^127 times the scale: the products turn non-finite and the solver reports a
// breakdown), e <= 0 gives h = l = 0 and 0 < e < 24 gives l = 0 (errors below
// 2^-126 absolute, against a scale near 1).
__device__ __forceinline__ int df_exponent(unsigned hi, int sh) { return (int)((hi >> 20) & 0x7FFu) - 896 - sh; }
__device__ __forceinline__ void df_split(double x, int sh, float& h, float& l) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = df_exponent(hi, sh);
  // exponent field minus (896 + sh): the binary32 exponent e when 0 < e < 256
  const unsigned hj = hi - ((unsigned)(896 + sh) << 20);
  const unsigned hb = (__funnelshift_l(lo, hj, 3) & 0x7FFFFFFFu) | (hi & 0x80000000u);
  // l = (2^(e-23) with the 23 next significand bits) - 2^(e-23): one unit of h's
  // last place as the base, exact subtraction (same exponent)
  const unsigned base = (hb & 0xFF800000u) - (23u << 23);
  const float lf = __fsub_rn(__uint_as_float(base | ((lo >> 6) & 0x007FFFFFu)), __uint_as_float(base));
  h = e >= 255 ? __uint_as_float((hi & 0x80000000u) | 0x7F800000u) : (e > 0 ? __uint_as_float(hb) : 0.0f);
  l = (e >= 24 && e < 255) ? lf : 0.0f;
}
// df_split with sh = 0, returning h + l as a binary64 (exact: x with the
// significand bits that the pair does not hold cleared)
__device__ __forceinline__ double df_split_canonical(double x, float& h, float& l) {
  df_split(x, 0, h, l);
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = df_exponent(hi, 0);
  if (e >= 255) return x;
  if (e <= 0) return 0.0;
  return __hiloint2double((int)hi, (int)(lo & (e >= 24 ? 0xFFFFFFC0u : 0xE0000000u)));
}
// (sh, sl) += (ah + al)(bh + bl). The _rn intrinsics keep every rounding
// explicit (no addition contracted into an FMA, which would break TwoSum).
__device__ __forceinline__ void df_fma(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  const float t = __fadd_rn(sh, p);
  const float z = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z));
  sl = __fadd_rn(sl, __fadd_rn(err, e));
  sh = t;
}
__device__ __forceinline__ void df_add(float& ah, float& al, float bh, float bl) {
  const float t = __fadd_rn(ah, bh);
  const float z = __fsub_rn(t, ah);
  const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(t, z)), __fsub_rn(bh, z));
  al = __fadd_rn(al, __fadd_rn(bl, err));
  ah = t;
}

// exact 2^e for |e| <= 1000 (the shifts are clamped to that range)
__device__ __forceinline__ double pow2(int e) { return __hiloint2double((e + 1023) << 20, 0); }

// Float-pair sum over the 32 lanes of a warp in a fixed shuffle tree (lane 0
// holds the sum); FP32 operations only.
__device__ __forceinline__ void warp_sum_df(float& h, float& l) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, h, o), ol = __shfl_down_sync(0xffffffffu, l, o);
    df_add(h, l, oh, ol);
  }
}
// Block sums of float-pair accumulators into float-pair partials: slot i <
// nk of block b at part[i * slot_stride + b] takes accumulator i, except slot
// `moved` (when >= 0), which takes accumulator K-1. Warp trees, then the 8 warp
// sums in order; no FP64 instruction (the FP64 pipe of this GPU would make the
// reduction the tail of the launch).
template <int K>
__device__ __forceinline__ void block_reduce_store_df(float (&ah)[K], float (&al)[K], int nk, float2* part,
                                                      int slot_stride, int moved) {
  __shared__ float2 seg[K][kDotThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < K; ++j) {
    warp_sum_df(ah[j], al[j]);
    if (lane == 0) seg[j][wid] = make_float2(ah[j], al[j]);
  }
  __syncthreads();
  if ((int)threadIdx.x < nk) {
    const int src = (int)threadIdx.x == moved ? K - 1 : (int)threadIdx.x;
    float th = 0.0f, tl = 0.0f;
#pragma unroll
    for (int w = 0; w < kDotThreads / 32; ++w) df_add(th, tl, seg[src][w].x, seg[src][w].y);
    part[threadIdx.x * slot_stride + blockIdx.x] = make_float2(th, tl);
  }
}
// The float-pair passes stream the basis through a per-thread ring of
// asynchronous copies (cp.async, global -> shared): an item is kRingGroup
// basis entries of one entry pair (16 bytes each) plus, at a pair's first item,
// the pair of w; kRingStages items are in flight per thread, about 160 KB per SM
// at two blocks per SM, which is what keeps HBM busy (register-staged loads of
// the same kernels reached about 3.8 TB/s). Each thread reads back only its own
// slots, so the ring needs no block barrier; cp.async.wait_group is the
// hardware wait for the thread's own copies.
constexpr int kRingThreads = 256;
constexpr int kRingGroup = 4;                  // basis vectors per item
constexpr int kRingSlots = kRingGroup + 1;     // + the w pair
constexpr int kRingStages = 5;                 // items in flight per thread
constexpr int kRingBytes = kRingStages * kRingSlots * kRingThreads * 16;  // 102,400 (dynamic)
static_assert(kRingThreads == kDotThreads, "the block reductions assume kDotThreads");
static_assert(kDfChunk % kRingGroup == 0, "chunk of whole items");

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Issue cursor of a thread's items: pairs q0, q0 + step, ...; ng items per pair.
struct RingCursor {
  long q;
  int g, stage;
};
// Copies item (c.q, c.g) into stage c.stage (basis columns col0 + g*kRingGroup + b
// of Vc below kk; zero-fill beyond) and advances; always commits one group so
// that the wait count stays uniform.
__device__ __forceinline__ void ring_issue(float4* ring, RingCursor& c, long np, long step, int ng, int kk,
                                           const float2* __restrict__ Vc, long lds, const double* __restrict__ w) {
  if (c.q < np) {
    float4* dst = ring + (c.stage * kRingSlots) * kRingThreads + threadIdx.x;
#pragma unroll
    for (int b = 0; b < kRingGroup; ++b) {
      const int u = c.g * kRingGroup + b;
      const bool ok = u < kk;
      cp_async16(dst + b * kRingThreads, Vc + (size_t)(ok ? u : 0) * lds + 2 * c.q, ok ? 16 : 0);
    }
    if (c.g == 0) cp_async16(dst + kRingGroup * kRingThreads, w + 2 * c.q, 16);
    if (++c.g == ng) {
      c.g = 0;
      c.q += step;
    }
  }
  cp_async_commit();
  if (++c.stage == kRingStages) c.stage = 0;
}

template <int G>
__device__ __forceinline__ void multidot_group(float (&ah)[kDfChunk + 1], float (&al)[kDfChunk + 1],
                                               const float4* src, int kk, float a0, float b0, float a1, float b1) {
#pragma unroll
  for (int b = 0; b < kRingGroup; ++b) {
    constexpr int base = G * kRingGroup;
    if (base + b < kk) {
      const float4 v = src[b * kRingThreads];
      df_fma(ah[base + b], al[base + b], v.x, v.y, a0, b0);
      df_fma(ah[base + b], al[base + b], v.z, v.w, a1, b1);
    }
  }
}

// ---- one Arnoldi step on the float-pair basis
//
// Classical Gram-Schmidt with the conditional second pass in five launches,
// none with a cross-block finishing phase: a launch writes per-block float-pair
// partial sums, and the launch that needs their totals reduces them itself in
// its prologue (every block, in the same fixed order, so every block obtains
// the same values). This removes the fences, the arrival atomics and the single
// finishing block of the FP64 kernels, a tail that cost about as much as the
// pass itself at k ~ 30. The launches are queued with programmatic stream
// serialisation (each begins with pdl_wait, which returns once its predecessor
// has completed and its writes are visible).
//   dots, pass 0:   P1[j] = <w, V_j> (j < k), P1[k] = <w, w>
//   update, pass 0: w -= V c1, c1 = totals of P1; Q1 = <w, w>;
//                   block 0: h[0..k) = c1, arn[1] = |w before|
//   dots, pass 1:   need2 from P1[k], Q1 (block 0 stores it); if need2: P2
//   update, pass 1: if need2: w -= V c2; Q2 = <w, w>; block 0: h[0..k) += c2
//   basis:          v = w / |w| and its float pair (|w| from Q2 or Q1);
//                   block 0: h[k] = |w|, arn[2] = 1 / |w|, the next step's
//                   scale exponent
// need2 = |w after pass 0| <= 0.7 |w before| (the criterion of k_cgs_update).
// Partials are float pairs of the 2^-sh scaled sums; totals are unscaled when
// converted to FP64. Workspace (in the reduction workspace): P1, P2 (kGsStage
// pairs each), Q1, Q2 (kDotBlocks pairs each).
constexpr int kGsStage = (kDfChunk + 1) * kDotBlocks;  // partial pairs of one dots launch, at most
static_assert(2 * kGsStage + 2 * kDotBlocks <= kDotPartialDoubles, "float-pair partials fit the workspace");
static_assert((size_t)kGsStage * sizeof(float2) <= (size_t)kRingBytes, "partials staged in the ring");

__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// float-pair total of stage[0..nb) by one warp: lane l adds l, l + 32, ... then the tree
__device__ __forceinline__ void warp_total_df(const float2* stage, int nb, float& h, float& l) {
  h = l = 0.0f;
  for (int b = threadIdx.x & 31; b < nb; b += 32) {
    const float2 x = stage[b];
    df_add(h, l, x.x, x.y);
  }
  warp_sum_df(h, l);
}
__device__ __forceinline__ double df_to_double(float h, float l, int e) {
  return ((double)h + (double)l) * pow2(e);
}

// res[v] = (sum over b < nb of P[v * nb + b]) x 2^sh (x 2^(2 sh) for v ==
// norm_slot), v < nv, nv * nb <= kGsStage, by all threads of the block: the
// partials are copied into `stage` (shared) with every copy in flight at once,
// then warp w sums values w, w + 8, ... and converts to FP64.
__device__ void gs_totals(const float2* __restrict__ P, int nv, int nb, float2* stage, double* res, int sh,
                          int norm_slot) {
  const int total = nv * nb;
  for (int i = threadIdx.x; i < total; i += blockDim.x) cp_async8(stage + i, P + i);
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  for (int v = threadIdx.x >> 5; v < nv; v += blockDim.x / 32) {
    float h, l;
    warp_total_df(stage + v * nb, nb, h, l);
    if ((threadIdx.x & 31) == 0) res[v] = df_to_double(h, l, v == norm_slot ? 2 * sh : sh);
  }
  __syncthreads();
}
// need2 of the step from |w before|^2 (P1k = P1 + k nbp, nbp partials) and
// |w after pass 0|^2 (Q1, nbq partials), both staged in one round of copies
__device__ bool gs_need2(const float2* P1k, int nbp, const float2* Q1, int nbq, float2* stage, int sh) {
  __shared__ double r[2];
  for (int i = threadIdx.x; i < nbp; i += blockDim.x) cp_async8(stage + i, P1k + i);
  for (int i = threadIdx.x; i < nbq; i += blockDim.x) cp_async8(stage + nbp + i, Q1 + i);
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int wid = threadIdx.x >> 5;
  if (wid < 2) {
    float h, l;
    warp_total_df(wid == 0 ? stage : stage + nbp, wid == 0 ? nbp : nbq, h, l);
    if ((threadIdx.x & 31) == 0) r[wid] = df_to_double(h, l, 2 * sh);
  }
  __syncthreads();
  return !(sqrt(r[1]) > 0.7 * sqrt(r[0]));
}

// dots of pass `pass` (0: with <w, w>); blockIdx.y = chunk, the k vectors
// spread evenly over the chunks (at most kDfChunk each)
__global__ void __launch_bounds__(kRingThreads, 2) k_gs_dots_df(long n, const double* __restrict__ w,
                                                             const float2* __restrict__ Vs, long lds, int k, int pass,
                                                             const int* __restrict__ shift, float2* P1, float2* P2,
                                                             const float2* Q1, int nbq, int* __restrict__ need2) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ float4 ring[];
  const int sh = *shift;
  const int nb = gridDim.x;
  if (pass == 1) {
    const bool n2 = gs_need2(P1 + (size_t)k * nb, nb, Q1, nbq, reinterpret_cast<float2*>(ring), sh);
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *need2 = n2 ? 1 : 0;
    if (!n2) return;
  }
  const int chunks = gridDim.y, chunk = blockIdx.y;
  const int per = k / chunks, rem = k % chunks;
  const int kk = per + (chunk < rem ? 1 : 0);
  const int j0 = chunk * per + (chunk < rem ? chunk : rem);
  const int norm = (pass == 0 && chunk == chunks - 1) ? 1 : 0;
  const int ng = (kk + kRingGroup - 1) / kRingGroup;
  const float2* __restrict__ Vc = Vs + (size_t)j0 * lds;
  float ah[kDfChunk + 1], al[kDfChunk + 1];
#pragma unroll
  for (int j = 0; j <= kDfChunk; ++j) ah[j] = al[j] = 0.0f;
  const long np = n >> 1;
  const long step = (long)nb * kRingThreads;
  RingCursor is{blockIdx.x * (long)kRingThreads + threadIdx.x, 0, 0};
#pragma unroll 1
  for (int s = 0; s < kRingStages - 1; ++s) ring_issue(ring, is, np, step, ng, kk, Vc, lds, w);
  long q = blockIdx.x * (long)kRingThreads + threadIdx.x;
  int g = 0, stage = 0;
  float a0 = 0.0f, b0 = 0.0f, a1 = 0.0f, b1 = 0.0f;
  while (q < np) {
    ring_issue(ring, is, np, step, ng, kk, Vc, lds, w);
    cp_async_wait<kRingStages - 1>();
    const float4* src = ring + (stage * kRingSlots) * kRingThreads + threadIdx.x;
    if (g == 0) {
      const double2 wv = *reinterpret_cast<const double2*>(src + kRingGroup * kRingThreads);
      df_split(wv.x, sh, a0, b0);
      df_split(wv.y, sh, a1, b1);
      if (norm) {
        df_fma(ah[kDfChunk], al[kDfChunk], a0, b0, a0, b0);
        df_fma(ah[kDfChunk], al[kDfChunk], a1, b1, a1, b1);
      }
    }
    switch (g) {
      case 0: multidot_group<0>(ah, al, src, kk, a0, b0, a1, b1); break;
      case 1: multidot_group<1>(ah, al, src, kk, a0, b0, a1, b1); break;
      case 2: multidot_group<2>(ah, al, src, kk, a0, b0, a1, b1); break;
      default: multidot_group<3>(ah, al, src, kk, a0, b0, a1, b1); break;
    }
    static_assert(kDfChunk / kRingGroup == 4, "one case per item of a chunk");
    if (++stage == kRingStages) stage = 0;
    if (++g == ng) {
      g = 0;
      q += step;
    }
  }
  cp_async_wait<0>();
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {  // the last entry of an odd length
    float c0, d0;
    df_split(w[n - 1], sh, c0, d0);
#pragma unroll
    for (int j = 0; j < kDfChunk; ++j)
      if (j < kk) {
        const float2 v = Vc[(size_t)j * lds + n - 1];
        df_fma(ah[j], al[j], v.x, v.y, c0, d0);
      }
    if (norm) df_fma(ah[kDfChunk], al[kDfChunk], c0, d0, c0, d0);
  }
  float2* P = (pass == 0 ? P1 : P2) + (size_t)j0 * nb;
  block_reduce_store_df<kDfChunk + 1>(ah, al, kk + norm, P, nb, norm ? kk : -1);
}

// update of pass `pass`: w -= sum_j c_j V_j with c the totals of the pass's dots
__global__ void __launch_bounds__(kRingThreads, 2) k_gs_update_df(long n, int k, int pass,
                                                               const float2* __restrict__ Vs, long lds,
                                                               double* __restrict__ w, const int* __restrict__ shift,
                                                               const float2* P1, const float2* P2, int nbp,
                                                               float2* Q1, float2* Q2, const int* __restrict__ need2,
                                                               double* __restrict__ h, double* __restrict__ arn) {
  pdl_wait();
  pdl_trigger();
  if (pass == 1 && *need2 == 0) return;
  extern __shared__ float4 ring[];
  __shared__ double res[kGsMaxK + 1];
  __shared__ float2 c[kGsMaxK];
  const int sh = *shift;
  gs_totals(pass == 0 ? P1 : P2, pass == 0 ? k + 1 : k, nbp, reinterpret_cast<float2*>(ring), res, sh,
            pass == 0 ? k : -1);
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    float a, b;
    df_split(res[i], sh, a, b);
    c[i] = make_float2(a, b);
    if (blockIdx.x == 0) h[i] = pass == 0 ? res[i] : h[i] + res[i];
  }
  if (pass == 0 && blockIdx.x == 0 && threadIdx.x == 0) arn[1] = sqrt(res[k]);
  __syncthreads();
  const double up = pow2(sh);
  float nh = 0.0f, nl = 0.0f;  // <w, w> after, 2^-2sh scaled
  const long np = n >> 1;
  const long step = (long)gridDim.x * kRingThreads;
  const int ng = (k + kRingGroup - 1) / kRingGroup;
  RingCursor is{blockIdx.x * (long)kRingThreads + threadIdx.x, 0, 0};
#pragma unroll 1
  for (int s = 0; s < kRingStages - 1; ++s) ring_issue(ring, is, np, step, ng, k, Vs, lds, w);
  long q = blockIdx.x * (long)kRingThreads + threadIdx.x;
  int g = 0, stage_i = 0;
  float s0h = 0.0f, s0l = 0.0f, s1h = 0.0f, s1l = 0.0f;
  double2 wv = make_double2(0.0, 0.0);
  while (q < np) {
    ring_issue(ring, is, np, step, ng, k, Vs, lds, w);
    cp_async_wait<kRingStages - 1>();
    const float4* src = ring + (stage_i * kRingSlots) * kRingThreads + threadIdx.x;
    if (g == 0) wv = *reinterpret_cast<const double2*>(src + kRingGroup * kRingThreads);
#pragma unroll
    for (int b = 0; b < kRingGroup; ++b) {
      const int u = g * kRingGroup + b;
      if (u < k) {
        const float2 cc = c[u];
        const float4 v = src[b * kRingThreads];
        df_fma(s0h, s0l, cc.x, cc.y, v.x, v.y);
        df_fma(s1h, s1l, cc.x, cc.y, v.z, v.w);
      }
    }
    if (++stage_i == kRingStages) stage_i = 0;
    if (++g == ng) {
      wv.x = fma(-up, (double)s0h, wv.x);
      wv.x = fma(-up, (double)s0l, wv.x);
      wv.y = fma(-up, (double)s1h, wv.y);
      wv.y = fma(-up, (double)s1l, wv.y);
      reinterpret_cast<double2*>(w)[q] = wv;
      float a, bb;
      df_split(wv.x, sh, a, bb);
      df_fma(nh, nl, a, bb, a, bb);
      df_split(wv.y, sh, a, bb);
      df_fma(nh, nl, a, bb, a, bb);
      s0h = s0l = s1h = s1l = 0.0f;
      g = 0;
      q += step;
    }
  }
  cp_async_wait<0>();
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {  // the last entry of an odd length
    float t0h = 0.0f, t0l = 0.0f;
    for (int u = 0; u < k; ++u) {
      const float2 v = Vs[(size_t)u * lds + n - 1];
      df_fma(t0h, t0l, c[u].x, c[u].y, v.x, v.y);
    }
    double t = w[n - 1];
    t = fma(-up, (double)t0h, t);
    t = fma(-up, (double)t0l, t);
    w[n - 1] = t;
    float a, bb;
    df_split(t, sh, a, bb);
    df_fma(nh, nl, a, bb, a, bb);
  }
  float nha[1] = {nh}, nla[1] = {nl};
  block_reduce_store_df<1>(nha, nla, 1, pass == 0 ? Q1 : Q2, 1, -1);
}

// v = w / |w| canonicalised to its float pair (vs); block 0 writes h[k] = |w|,
// arn[2] = 1 / |w| and *shift_next (from arn[1] = |w before|).
__global__ void __launch_bounds__(kRingThreads) k_gs_basis_df(long n, int k, const int* __restrict__ shift,
                                                           int* __restrict__ shift_next, const float2* Q1,
                                                           const float2* Q2, int nbq, const int* __restrict__ need2,
                                                           const double* __restrict__ w, double* __restrict__ v,
                                                           float2* __restrict__ vs, double* __restrict__ h,
                                                           double* __restrict__ arn) {
  pdl_wait();
  pdl_trigger();
  __shared__ float2 gstage[kDotBlocks];
  __shared__ double r[1];
  const int sh = *shift;
  gs_totals(*need2 ? Q2 : Q1, 1, nbq, gstage, r, sh, 0);
  const double nw = sqrt(r[0]);
  const double sc = 1.0 / (nw > 0 ? nw : 1.0);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float a, b;
    v[i] = df_split_canonical(sc * w[i], a, b);
    vs[i] = make_float2(a, b);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    h[k] = nw;
    arn[2] = sc;
    *shift_next = gs_shift_of(arn[1]);
  }
}

// kernel launch with programmatic stream serialisation
template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, int threads, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  GB_CUDA(cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...));
}

// the ring's dynamic shared memory, granted once per device
void ring_reserve() {
  constexpr int kMaxDevices = 64;
  static bool done[kMaxDevices];
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < kMaxDevices && done[dev]) return;
  GB_CUDA(cudaFuncSetAttribute(k_gs_dots_df, cudaFuncAttributeMaxDynamicSharedMemorySize, kRingBytes));
  GB_CUDA(cudaFuncSetAttribute(k_gs_update_df, cudaFuncAttributeMaxDynamicSharedMemorySize, kRingBytes));
  if (dev >= 0 && dev < kMaxDevices) done[dev] = true;
}

void v_arnoldi_step_df(long n, int j, const float2* Vs, long lds, double* w, double* vnext, float2* vsnext,
                       double* h, double* arn, int* need2, const int* shift, int* shift_next, double* workspace,
                       cudaStream_t s) {
  const int k = j + 1;
  GB_CHECK(k >= 1 && k <= kGsMaxK, 2, "float-pair Arnoldi step: 1 <= j + 1 <= 128");
  ring_reserve();
  float2* P1 = reinterpret_cast<float2*>(workspace);
  float2* P2 = P1 + kGsStage;
  float2* Q1 = P2 + kGsStage;
  float2* Q2 = Q1 + kDotBlocks;
  const int chunks = (k + kDfChunk - 1) / kDfChunk;
  const int nbp = kDotBlocks / chunks;
  for (int pass = 0; pass < 2; ++pass) {
    launch_pdl(k_gs_dots_df, dim3(nbp, chunks), kRingThreads, kRingBytes, s, n, w, Vs, lds, k, pass, shift, P1, P2,
               Q1, kDotBlocks, need2);
    launch_pdl(k_gs_update_df, dim3(kDotBlocks), kRingThreads, kRingBytes, s, n, k, pass, Vs, lds, w, shift, P1, P2,
               nbp, Q1, Q2, need2, h, arn);
  }
  launch_pdl(k_gs_basis_df, dim3(kDotBlocks), kRingThreads, 0, s, n, k, shift, shift_next, Q1, Q2, kDotBlocks, need2,
             w, vnext, vsnext, h, arn);
  VecCounter::launches() += 5;
}

// v = sc w in FP64 canonicalised to the float pair, and the pair into vs;
// sc = *sc_dev when sc_dev is given (the reciprocal of |w| that k_cgs_update
// formed), else sc_host
__global__ void k_basis_df(long n, const double* __restrict__ sc_dev, double sc_host, const double* __restrict__ w,
                           double* __restrict__ v, float2* __restrict__ vs) {
  pdl_wait();
  const double sc = sc_dev ? *sc_dev : sc_host;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float a, b;
    v[i] = df_split_canonical(sc * w[i], a, b);
    vs[i] = make_float2(a, b);
  }
}
void v_basis_df(long n, const double* sc_dev, double sc_host, const double* w, double* v, float2* vs,
                cudaStream_t s) {
  if (n <= 0) return;
  k_basis_df<<<grid_for(n), kThreads, 0, s>>>(n, sc_dev, sc_host, w, v, vs);
  count();
}

template <typename T>
__global__ void __launch_bounds__(kDotThreads) k_dot(long n, const T* __restrict__ a, const T* __restrict__ b,
                                                     double* __restrict__ out, double* __restrict__ partial,
                                                     unsigned* counter, const int* __restrict__ active) {
  pdl_wait();
  if (active && *active == 0) return;
  double acc[1] = {0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    acc[0] += (double)a[i] * (double)b[i];
  block_reduce_store<1>(acc, 1, partial, kDotBlocks);
  if (arrive_last(counter)) finish_partials(partial, 1, out, counter);
}
template <typename T>
void v_dot(long n, const T* a, const T* b, double* out_dev, double* partial, cudaStream_t s, const int* active) {
  unsigned* counter = reinterpret_cast<unsigned*>(partial + kDotPartialDoubles) + kDotMaxChunks;
  k_dot<T><<<kDotBlocks, kDotThreads, 0, s>>>(n, a, b, out_dev, partial, counter, active);
  VecCounter::launches() += 1;
}

// ---------------------------------------------------------------- eigenvalue-estimate CG
// The CG of PreconditionChebyshev's eigenvalue estimate with every scalar on the
// device: per step, besides the level operator, four launches, each fusing a
// vector update, a reduction with k_dot's grid and order and the step's scalar
// bookkeeping in the block that finishes the reduction. The vector updates are
// written as k_axpby and k_cheb_first write theirs (runtime coefficients), so
// the iterates, dots and alpha/beta history equal those of the host-driven loop.
//   s: [0] r.z, [1] p.Ap, [2] r.r, [3] new r.z, [4] alpha, [5] beta,
//      [kEigHist ..) alphas, [kEigHist + its ..) betas
//   f: [0] running, [1] alphas stored, [2] betas stored
// A step that finds p.Ap <= 0 stops before storing alpha, one that finds
// |r| < 1e-2 after storing alpha (SolverControl(its, 1e-2), absolute); later
// launches see f[0] = 0 and return.
template <typename T>
__global__ void __launch_bounds__(kDotThreads) k_eig_pap(long n, const T* __restrict__ p, const T* __restrict__ Ap,
                                                         double* s, int* f, double* partial, unsigned* counter) {
  pdl_wait();
  if (f[0] == 0) return;
  double acc[1] = {0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    acc[0] += (double)p[i] * (double)Ap[i];
  block_reduce_store<1>(acc, 1, partial, kDotBlocks);
  if (!arrive_last(counter)) return;
  finish_partials(partial, 1, s + 1, counter);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double pAp = s[1];
    if (!(pAp > 0)) {
      f[0] = 0;
    } else {
      const double alpha = s[0] / pAp;
      s[4] = alpha;
      s[kEigHist + f[1]] = alpha;
      f[1] += 1;
    }
  }
}
// r = (-alpha) Ap + b r (b = 1) and r.r
template <typename T>
__global__ void __launch_bounds__(kDotThreads) k_eig_r(long n, const T* __restrict__ Ap, T* __restrict__ r, T b,
                                                       double* s, int* f, double* partial, unsigned* counter) {
  pdl_wait();
  if (f[0] == 0) return;
  const T a = (T)(-s[4]);
  double acc[1] = {0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const T v = a * Ap[i] + b * r[i];
    r[i] = v;
    acc[0] += (double)v * (double)v;
  }
  block_reduce_store<1>(acc, 1, partial, kDotBlocks);
  if (!arrive_last(counter)) return;
  finish_partials(partial, 1, s + 2, counter);
  __syncthreads();
  if (threadIdx.x == 0 && sqrt(s[2]) < 1e-2) f[0] = 0;
}
// z = f2 dinv r (f2 = 1) and r.z; beta = new r.z / r.z
template <typename T>
__global__ void __launch_bounds__(kDotThreads) k_eig_z(long n, const T* __restrict__ r, const T* __restrict__ dinv,
                                                       T f2, T* __restrict__ z, double* s, int* f, int its,
                                                       double* partial, unsigned* counter) {
  pdl_wait();
  if (f[0] == 0) return;
  double acc[1] = {0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const T v = f2 * dinv[i] * r[i];
    z[i] = v;
    acc[0] += (double)r[i] * (double)v;
  }
  block_reduce_store<1>(acc, 1, partial, kDotBlocks);
  if (!arrive_last(counter)) return;
  finish_partials(partial, 1, s + 3, counter);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double beta = s[3] / s[0];
    s[5] = beta;
    s[kEigHist + its + f[2]] = beta;
    f[2] += 1;
    s[0] = s[3];
  }
}
// p = a z + beta p (a = 1)
template <typename T>
__global__ void k_eig_p(long n, T a, const T* __restrict__ z, T* __restrict__ p, const double* s, const int* f) {
  pdl_wait();
  if (f[0] == 0) return;
  const T b = (T)s[5];
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    p[i] = a * z[i] + b * p[i];
}
__global__ void k_eig_start(int* f) {
  f[0] = 1;
  f[1] = 0;
  f[2] = 0;
}

void v_eig_start(int* f, cudaStream_t st) {
  k_eig_start<<<1, 1, 0, st>>>(f);
  count();
}
template <typename T>
void v_eig_step(long n, T* p, const T* Ap, T* r, T* z, const T* dinv, double* s, int* f, int its,
                double* partial, cudaStream_t st) {
  unsigned* counter = reinterpret_cast<unsigned*>(partial + kDotPartialDoubles) + kDotMaxChunks;
  k_eig_pap<T><<<kDotBlocks, kDotThreads, 0, st>>>(n, p, Ap, s, f, partial, counter);
  k_eig_r<T><<<kDotBlocks, kDotThreads, 0, st>>>(n, Ap, r, T(1), s, f, partial, counter);
  k_eig_z<T><<<kDotBlocks, kDotThreads, 0, st>>>(n, r, dinv, T(1), z, s, f, its, partial, counter);
  k_eig_p<T><<<grid_for(n), kThreads, 0, st>>>(n, T(1), z, p, s, f);
  VecCounter::launches() += 4;
}
template void v_eig_step<float>(long, float*, const float*, float*, float*, const float*, double*, int*, int,
                                double*, cudaStream_t);
template void v_eig_step<double>(long, double*, const double*, double*, double*, const double*, double*, int*, int,
                                 double*, cudaStream_t);

// w += V coef. The basis entries of a row are loaded eight at a time before
// they are summed (in order j = 0, 1, ...), so eight independent loads per
// thread are in flight instead of one dependent load per step; the sums are
// the same as the one-at-a-time loop's.
constexpr int kAxpyBatch = 8;
__global__ void __launch_bounds__(kThreads) k_multiaxpy(long n, int k, const double* __restrict__ coef,
                                                        const double* __restrict__ V, long ld,
                                                        double* __restrict__ w, const int* __restrict__ active) {
  pdl_wait();
  if (active && *active == 0) return;
  constexpr int kCached = 256;
  __shared__ double c[kCached];
  for (int j = threadIdx.x; j < k && j < kCached; j += blockDim.x) c[j] = coef[j];
  __syncthreads();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double t = w[i];
    int j = 0;
    for (; j + kAxpyBatch <= k; j += kAxpyBatch) {
      double v[kAxpyBatch];
#pragma unroll
      for (int u = 0; u < kAxpyBatch; ++u) v[u] = V[(size_t)(j + u) * ld + i];
#pragma unroll
      for (int u = 0; u < kAxpyBatch; ++u) t += (j + u < kCached ? c[j + u] : coef[j + u]) * v[u];
    }
    for (; j < k; ++j) t += (j < kCached ? c[j] : coef[j]) * V[(size_t)j * ld + i];
    w[i] = t;
  }
}
void v_multiaxpy(long n, int k, const double* coef_dev, const double* V, long ld, double* w, cudaStream_t s,
                 const int* active) {
  if (n <= 0 || k <= 0) return;
  k_multiaxpy<<<grid_for(n), kThreads, 0, s>>>(n, k, coef_dev, V, ld, w, active);
  count();
}

__global__ void k_symv_dense(long n, const double* __restrict__ S, const double* __restrict__ x,
                             double* __restrict__ y) {
  pdl_wait();
  const long row = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  // S is symmetric: row `row` is read as column `row` (contiguous)
  const double* col = S + row * n;
  double t = 0;
  for (long i = lane; i < n; i += 32) t += col[i] * x[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) y[row] = t;
}
void v_symv_dense(long n, const double* S, const double* x, double* y, cudaStream_t s) {
  if (n <= 0) return;
  k_symv_dense<<<ceil_div(n * 32, 256), 256, 0, s>>>(n, S, x, y);
  count();
}

template <typename T>
__global__ void k_check_finite(long n, const T* __restrict__ x, int* flag) {
  pdl_wait();
  int bad = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    if (!isfinite(x[i])) bad = 1;
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}
template <typename T>
void v_check_finite(long n, const T* x, int* flag, cudaStream_t s) {
  if (n <= 0) return;
  k_check_finite<<<grid_for(n), kThreads, 0, s>>>(n, x, flag);
  count();
}

#define INST(T)                                                                                    \
  template void v_axpby<T>(long, T, const T*, T, T*, cudaStream_t);                               \
  template void v_copy<T>(long, const T*, T*, cudaStream_t);                                      \
  template void v_scale<T>(long, T, T*, cudaStream_t);                                            \
  template void v_zero<T>(long, T*, cudaStream_t);                                                \
  template void v_cheb_first<T>(long, const T*, const T*, T, T*, T*, cudaStream_t);               \
  template void v_cheb_step<T>(long, const T*, const T*, const T*, T, T, T*, T*, cudaStream_t);   \
  template void v_sub<T>(long, const T*, const T*, T*, cudaStream_t);                             \
  template void v_copy_indexed<T>(long, const int*, const T*, T*, cudaStream_t);                  \
  template void v_zero_indexed<T>(long, const int*, T*, cudaStream_t);                            \
  template void v_spmv_add<T>(long, const int*, const int*, const T*, const T*, T*, cudaStream_t); \
  template void v_spmv_set<T>(long, long, const int*, const int*, const T*, const T*, T*, cudaStream_t); \
  template void v_dot<T>(long, const T*, const T*, double*, double*, cudaStream_t, const int*);               \
  template void v_check_finite<T>(long, const T*, int*, cudaStream_t);
INST(float)
INST(double)
#undef INST
template void v_cast<double, float>(long, const double*, float*, cudaStream_t);
template void v_cast<float, double>(long, const float*, double*, cudaStream_t);
template void v_permute_scatter<double, double>(long, const int*, const double*, double*, cudaStream_t);
template void v_permute_scatter<double, float>(long, const int*, const double*, float*, cudaStream_t);
template void v_permute_gather<double, double>(long, const int*, const double*, double*, cudaStream_t);
template void v_permute_gather<float, double>(long, const int*, const float*, double*, cudaStream_t);

}  // namespace gb
