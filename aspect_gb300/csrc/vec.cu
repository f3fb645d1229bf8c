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

template <typename T>
__global__ void k_cheb_first(long n, const T* __restrict__ b, const T* __restrict__ dinv, T f2, T* __restrict__ d,
                             T* __restrict__ x) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
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
  if (arrive_last(counters + chunk)) finish_partials(part, kk + norm, out + j0, counters + chunk, nb);
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
                                                            double* __restrict__ partial, unsigned* counter) {
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
    const double nw = sqrt(arn[0]);
    h[k] = nw;
    arn[2] = 1.0 / (nw > 0 ? nw : 1.0);
    if (pass == 0) *need2 = nw > 0.7 * arn[1] ? 0 : 1;
  }
}

void v_cgs_update(long n, int j, int pass, const double* dots, const double* V, long ld, double* w, double* h,
                  double* arn, int* need2, double* partial, cudaStream_t s) {
  unsigned* counter = reinterpret_cast<unsigned*>(partial + kDotPartialDoubles) + kDotMaxChunks;
  long nb = (n + (long)kDotThreads * kCgsPerThread - 1) / ((long)kDotThreads * kCgsPerThread);
  const long max_nb = kDotPartialDoubles;  // one partial per block
  if (nb > max_nb) nb = max_nb;
  if (nb < 1) nb = 1;
  k_cgs_update<<<(int)nb, kDotThreads, 0, s>>>(n, j, pass, dots, V, ld, w, h, arn, need2, partial, counter);
  VecCounter::launches() += 1;
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
