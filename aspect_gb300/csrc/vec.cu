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
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] *= a;
}
template <typename T>
void v_scale(long n, T a, T* y, cudaStream_t s) {
  if (n <= 0) return;
  k_scale<<<grid_for(n), kThreads, 0, s>>>(n, a, y);
  count();
}

template <typename Ts, typename Td>
__global__ void k_cast(long n, const Ts* __restrict__ x, Td* __restrict__ y) {
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

// ---------------------------------------------------------------- reductions
template <int K>
__device__ __forceinline__ void block_reduce_store(double (&acc)[K], int nk, double* partial, int slot_stride) {
  __shared__ double sh[K][kDotThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < K; ++j) {
    double v = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[j][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < nk) {
    double t = 0;
    for (int w = 0; w < kDotThreads / 32; ++w) t += sh[threadIdx.x][w];
    partial[threadIdx.x * slot_stride + blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(kDotThreads) k_multidot(long n, const double* __restrict__ w,
                                                          const double* __restrict__ V, long ld, int k,
                                                          int with_norm, double* __restrict__ partial,
                                                          const int* __restrict__ active) {
  if (active && *active == 0) return;
  double acc[kDotChunk + 1];
#pragma unroll
  for (int j = 0; j <= kDotChunk; ++j) acc[j] = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double wi = w[i];
#pragma unroll
    for (int j = 0; j < kDotChunk; ++j)
      if (j < k) acc[j] += wi * V[j * ld + i];
    if (with_norm) acc[kDotChunk] += wi * wi;
  }
  if (with_norm) acc[k] = acc[kDotChunk];
  block_reduce_store<kDotChunk + 1>(acc, k + with_norm, partial, kDotBlocks);
}

__global__ void k_finish(const double* __restrict__ partial, int nk, double* __restrict__ out,
                         const int* __restrict__ active) {
  if (active && *active == 0) return;
  const int j = blockIdx.x;
  if (j >= nk) return;
  __shared__ double sh[32];
  double t = 0;
  for (int b = threadIdx.x; b < kDotBlocks; b += 32) t += partial[j * kDotBlocks + b];
  sh[threadIdx.x] = t;
  __syncwarp();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int l = 0; l < 32; ++l) s += sh[l];
    out[j] = s;
  }
}

void v_multidot(long n, const double* w, const double* V, long ld, int k, bool with_norm, double* out_dev,
                double* partial, cudaStream_t s, const int* active) {
  if (k == 0) {
    if (!with_norm) return;
    k_multidot<<<kDotBlocks, kDotThreads, 0, s>>>(n, w, V, ld, 0, 1, partial, active);
    k_finish<<<1, 32, 0, s>>>(partial, 1, out_dev, active);
    VecCounter::launches() += 2;
    return;
  }
  for (int done = 0; done < k; done += kDotChunk) {
    const int kk = k - done < kDotChunk ? k - done : kDotChunk;
    const int norm = (with_norm && done + kk == k) ? 1 : 0;
    k_multidot<<<kDotBlocks, kDotThreads, 0, s>>>(n, w, V + done * ld, ld, kk, norm, partial, active);
    k_finish<<<kk + norm, 32, 0, s>>>(partial, kk + norm, out_dev + done, active);
    VecCounter::launches() += 2;
  }
}

template <typename T>
__global__ void __launch_bounds__(kDotThreads) k_dot(long n, const T* __restrict__ a, const T* __restrict__ b,
                                                     double* __restrict__ partial, const int* __restrict__ active) {
  if (active && *active == 0) return;
  double acc[1] = {0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    acc[0] += (double)a[i] * (double)b[i];
  block_reduce_store<1>(acc, 1, partial, kDotBlocks);
}
template <typename T>
void v_dot(long n, const T* a, const T* b, double* out_dev, double* partial, cudaStream_t s, const int* active) {
  k_dot<T><<<kDotBlocks, kDotThreads, 0, s>>>(n, a, b, partial, active);
  k_finish<<<1, 32, 0, s>>>(partial, 1, out_dev, active);
  VecCounter::launches() += 2;
}

__global__ void k_multiaxpy(long n, int k, const double* __restrict__ coef, const double* __restrict__ V, long ld,
                            double* __restrict__ w, const int* __restrict__ active) {
  if (active && *active == 0) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double t = w[i];
    for (int j = 0; j < k; ++j) t += coef[j] * V[j * ld + i];
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
  template void v_cheb_first<T>(long, const T*, const T*, T, T*, T*, cudaStream_t);               \
  template void v_cheb_step<T>(long, const T*, const T*, const T*, T, T, T*, T*, cudaStream_t);   \
  template void v_sub<T>(long, const T*, const T*, T*, cudaStream_t);                             \
  template void v_copy_indexed<T>(long, const int*, const T*, T*, cudaStream_t);                  \
  template void v_zero_indexed<T>(long, const int*, T*, cudaStream_t);                            \
  template void v_spmv_add<T>(long, const int*, const int*, const T*, const T*, T*, cudaStream_t); \
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
