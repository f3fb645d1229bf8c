// Measured arithmetic peaks of the CUDA cores, for the rooflines of the FP64
// and FP32 cell kernels (libgb_probe.so, separate from the solver library).
//
// Each thread runs kChains independent FMA chains of kSteps dependent FMAs, so
// the pipe sees kChains independent instructions per thread and warp; the grid
// fills every SM several times over. The result is folded into one store per
// thread so nothing is optimised away. Time with CUDA events around one launch
// after a warm-up launch; flops = 2 x threads x kChains x kSteps.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;
constexpr int kSteps = 2048;
constexpr int kThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kThreads) fma_chains(T a, T b, T* out) {
  T x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = T(threadIdx.x + c) * T(1e-3);
#pragma unroll 8
  for (int s = 0; s < kSteps; ++s)
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = x[c] * a + b;
  T t = T(0);
#pragma unroll
  for (int c = 0; c < kChains; ++c) t += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = t;
}

template <typename T>
int measure(double* tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  const int blocks = sms * 16;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * (size_t)blocks * kThreads) != cudaSuccess) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // a and b keep the chains bounded: x -> b / (1 - a)
  const T a = T(0.999), b = T(1e-3);
  fma_chains<T><<<blocks, kThreads>>>(a, b, out);
  cudaEventRecord(e0);
  fma_chains<T><<<blocks, kThreads>>>(a, b, out);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return 1;
  *tflops = 2.0 * blocks * kThreads * (double)kChains * kSteps / (ms * 1e-3) / 1e12;
  return 0;
}

}  // namespace

extern "C" int gb_probe_fp64_fma_tflops(double* tflops) { return measure<double>(tflops); }
extern "C" int gb_probe_fp32_fma_tflops(double* tflops) { return measure<float>(tflops); }
