// Shared host/device helpers of the GB300 GMG Stokes library.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace gb {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define GB_CUDA(x)                                                                     \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess)                                                             \
      throw ::gb::Error(3, std::string("CUDA error ") + cudaGetErrorString(e_) + " at " + \
                               __FILE__ + ":" + std::to_string(__LINE__) + " (" #x ")"); \
  } while (0)

#define GB_CHECK(cond, code, msg)                    \
  do {                                               \
    if (!(cond)) throw ::gb::Error((code), (msg));   \
  } while (0)

// Plain device buffer; allocation happens only in set-up calls.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    n = count;
    if (count) GB_CUDA(cudaMalloc(&p, count * sizeof(T)));
  }
  void zero(cudaStream_t s) {
    if (n) GB_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  // Host copies are set-up operations and are ordered against ALL device work:
  // the library's streams are non-blocking, so a plain cudaMemcpy (legacy
  // stream) neither waits for their kernels nor, from pageable memory, is
  // guaranteed to have landed before a kernel launched next on them reads it.
  void upload(const T* h, size_t count) {
    alloc(count);
    if (!count) return;
    GB_CUDA(cudaDeviceSynchronize());  // no kernel still reads the old contents
    GB_CUDA(cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice));
    GB_CUDA(cudaDeviceSynchronize());  // the DMA has landed before later launches
  }
  void upload(const std::vector<T>& h) { upload(h.data(), h.size()); }
  std::vector<T> download() const {
    std::vector<T> h(n);
    if (!n) return h;
    GB_CUDA(cudaDeviceSynchronize());  // producers on any stream have finished
    GB_CUDA(cudaMemcpy(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost));
    return h;
  }
  size_t bytes() const { return n * sizeof(T); }
};

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// Every kernel of the library starts with this wait. Inside the captured
// V-cycle graphs consecutive kernels are joined by programmatic edges, so a
// kernel's blocks may be resident before its predecessor has finished; the
// wait returns once every predecessor grid has completed and its memory
// operations are visible. Launched any other way (no programmatic edge) it
// returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

}  // namespace gb
