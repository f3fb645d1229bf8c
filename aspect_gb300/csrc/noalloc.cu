// Allocation-free application of the FP32 velocity-block (A) operator on a
// uniform lattice box level.
//
// Some callers cannot call cudaMalloc at the moment they need an operator
// application: code that runs under a fixed device-memory budget owned by
// another allocator (a framework's caching allocator, a pre-reserved pool), or
// code on a path that must never block on the driver's allocator. The
// handle-based entry points allocate their per-cell scratch when the handle is
// set up; this entry point instead keeps that scratch in a file-scope device
// array that exists for the life of the library, so a call allocates nothing:
// the caller passes the lattice description, the viscosity table, the input and
// the output, all in device memory.
//
// Limits and sharing rules:
//  * at most kNoallocMaxCells cells (16^3 = 4096 in 3D, 64^2 = 4096 in 2D);
//    larger levels are rejected with GB_GMG_EXCEEDS_STATIC_SCRATCH;
//  * every GPU that loads the library holds the array (1.33 MB) until exit;
//  * all calls share the one array: calls whose kernels overlap on the GPU
//    (different streams, or different host threads on one device) race on it
//    and must be serialised by the caller;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and keeps it for later
//    calls; make that first call before any stream capture. The kept address
//    belongs to the device's primary context: after cudaDeviceReset (or any
//    other teardown of that context) the library must be reloaded before this
//    entry point is called again.
// Each call overwrites, for every cell, the whole part of the array that it
// later reads, so nothing has to start at zero and a call's result does not
// depend on what an earlier call left behind.
#include <mutex>

#include "../../include/gb_gmg.h"
#include "ops.cuh"

namespace gb {
namespace {

constexpr int kNoallocMaxCells = GB_GMG_NOALLOC_MAX_CELLS;
constexpr int kMaxDevices = 64;

// per-cell contributions of pass 1: up to kNoallocMaxCells cells x 81 values
static __device__ __align__(256) float g_noalloc_scratch[kNoallocMaxCells * 81];

std::mutex g_lock;
float* g_scratch_ptr[kMaxDevices] = {nullptr};

// Launches through cudaLaunchKernel, whose return value is this launch's own
// status: an error left behind by unrelated earlier work is neither reported as
// this call's failure nor cleared.
template <int dim>
cudaError_t run(const LevelView<float>& L, float* scratch, const float* src, float* dst, cudaStream_t s) {
  const int cells_per_block = 4 * Shape<dim>::cpw;  // 128 threads
  LevelView<float> Lv = L;
  const float* su = src;
  const float* sp = nullptr;
  float* eu = scratch;
  float* ep = nullptr;
  void* cell_args[] = {&Lv, &su, &sp, &eu, &ep};
  cudaError_t e = cudaLaunchKernel((const void*)velocity_cell_kernel<float, dim, OPK_A>,
                                   dim3(ceil_div(L.n_cells, cells_per_block)), dim3(128), cell_args, 0, s);
  if (e != cudaSuccess) return e;
  GatherArgs<float> a{};
  a.E = scratch;
  a.x = const_cast<float*>(src);
  a.y = dst;
  a.cs = dim == 3 ? 3 * 27 : 2 * 9;  // the shared-thread kernel writes cell-major
  a.ss = 1;
  void* gather_args[] = {&Lv, &a};
  return cudaLaunchKernel((const void*)velocity_gather_structured<float, dim, EPI_STORE>,
                          dim3(ceil_div(L.n_u, 256)), dim3(256), gather_args, 0, s);
}

}  // namespace
}  // namespace gb

extern "C" int gb_gmg_ablock_apply_lattice_noalloc(int dim, const int32_t* n_cells_dir, const double* cell_size,
                                                   uint32_t zero_faces, int eta_per_cell, const float* d_eta,
                                                   const float* d_src, float* d_dst, void* stream) {
  using namespace gb;
  if ((dim != 2 && dim != 3) || !n_cells_dir || !cell_size || !d_eta || !d_src || !d_dst)
    return GB_GMG_INVALID_ARGUMENT;
  const int nq = dim == 3 ? 27 : 9;
  if (eta_per_cell != 1 && eta_per_cell != nq) return GB_GMG_INVALID_ARGUMENT;
  for (int d = 0; d < dim; ++d)
    if (n_cells_dir[d] < 1 || !(cell_size[d] > 0)) return GB_GMG_INVALID_ARGUMENT;
  // every factor is checked against the limit before it is multiplied in, so
  // the running product stays below kNoallocMaxCells^2 and cannot overflow
  long n_cells = 1;
  for (int d = 0; d < dim; ++d) {
    if (n_cells_dir[d] > kNoallocMaxCells) return GB_GMG_EXCEEDS_STATIC_SCRATCH;
    n_cells *= n_cells_dir[d];
    if (n_cells > kNoallocMaxCells) return GB_GMG_EXCEEDS_STATIC_SCRATCH;
  }

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GB_GMG_CUDA_ERROR;
  float* scratch;
  {
    std::lock_guard<std::mutex> lk(g_lock);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GB_GMG_CUDA_ERROR;
      g_scratch_ptr[dev] = static_cast<float*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }

  LevelView<float> L{};
  L.deg = 2;
  L.dim = dim;
  L.n_cells = (int)n_cells;
  L.structured = 1;
  double det = 1;
  for (int d = 0; d < 3; ++d) {
    const int nc = d < dim ? n_cells_dir[d] : 1;
    L.nc[d] = nc;
    L.Nn[d] = d < dim ? 2 * nc + 1 : 1;
    L.Np[d] = d < dim ? nc + 1 : 1;
    L.inv_h[d] = d < dim ? (float)(1.0 / cell_size[d]) : 1.0f;
    if (d < dim) det *= cell_size[d];
  }
  L.det = (float)det;
  L.n_nodes = L.Nn[0] * L.Nn[1] * L.Nn[2];
  L.n_u = dim * L.n_nodes;
  L.n_p = L.Np[0] * L.Np[1] * L.Np[2];
  L.zero_faces = zero_faces;
  L.geom = GEOM_CART;
  L.eta = d_eta;
  L.eta_n = eta_per_cell;
  L.s = 1.0f;
  L.compressible = 0;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  const cudaError_t e = dim == 3 ? run<3>(L, scratch, d_src, d_dst, s) : run<2>(L, scratch, d_src, d_dst, s);
  return e == cudaSuccess ? GB_GMG_OK : GB_GMG_CUDA_ERROR;
}
