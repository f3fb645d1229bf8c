// FP32 velocity-block (A) operator of large 3D lattice levels in one pass over
// the cells, with the gather and the epilogue (store, residual or Chebyshev
// step) fused in: the two-pass form writes 81 contributions per cell to memory
// and reads them back, more traffic than the operator's own vectors.
//
// Tiling: a thread block owns a tile of kTX x kTY cells in x and y and tz cell
// layers in z, one thread per cell of a layer, and marches through the layers.
// Per layer:
//   1. each thread computes its cell's 81 contributions in registers
//      (lattice_cell_f32, the cell pass of the two-pass form) and stores them to
//      shared memory, slot-major;
//   2. after a block barrier, the block sums them into the three node planes of
//      the layer, every node in a fixed order (lower cell first in y, then x);
//      the lowest plane also adds the top plane the previous layer left in
//      shared memory, and the top plane is kept for the next layer;
//   3. nodes strictly inside the tile are complete: their epilogue runs here
//      (no other block's cell touches them, so the Chebyshev step may update the
//      iterate in place). Nodes on the tile's faces are also touched by
//      neighbouring tiles: the block writes its partial sums there to a face
//      buffer (per tile, in a fixed face order).
// A second kernel visits every node on a tile face, adds the partial sums of
// the (two to eight) tiles that share it in a fixed tile order and runs the
// epilogue. Every sum has a fixed order, so results are bit-reproducible.
// Tile-interior nodes never lie on the domain boundary, so they are never
// constrained; constrained (Dirichlet) nodes are always face nodes.
//
// Measured on one GB300 (sinker workload, CUDA events): 64^3, 127 us against
// 119 us for the two-pass form (cell pass 66 us). The cell arithmetic (about 35
// flop per compulsory byte, above the FP32 ridge of ~10) dominates, and with one
// thread per cell (234 registers, two blocks per SM) the block's summation phase
// does not overlap its arithmetic phase, so removing the contribution round trip
// does not pay. The library therefore keeps it off by default
// (gb_gmg_options::fused_a_min_cells = 0); it is tested for parity.
#include "ops.cuh"

namespace gb {
namespace {

constexpr int kTX = 16, kTY = 8;          // cells per tile in x and y
constexpr int kFT = kTX * kTY;            // threads per block: one cell of a layer each
constexpr int kBX = 2 * kTX + 1;          // node box of a tile in x (33)
constexpr int kBY = 2 * kTY + 1;          // ... and in y (17)
constexpr int kPlane = kBX * kBY;         // nodes of one node plane of a tile (561)
constexpr int kSmemFloats = 81 * kFT + 2 * 3 * kPlane;

// Boundary nodes of a tile's node box kBX x kBY x (2 tz + 1), in the order:
// plane lz = 0, plane lz = 2 tz, then for 0 < lz < 2 tz: row ly = 0, row
// ly = kBY - 1, column lx = 0, column lx = kBX - 1.
__host__ __device__ inline int face_count(int tz) {
  const int inner = 2 * tz - 1;
  return 2 * kPlane + 2 * kBX * inner + 2 * (kBY - 2) * inner;
}
__device__ inline int face_index(int lx, int ly, int lz, int tz) {
  const int inner = 2 * tz - 1;
  if (lz == 0) return ly * kBX + lx;
  if (lz == 2 * tz) return kPlane + ly * kBX + lx;
  int base = 2 * kPlane;
  if (ly == 0) return base + (lz - 1) * kBX + lx;
  base += kBX * inner;
  if (ly == kBY - 1) return base + (lz - 1) * kBX + lx;
  base += kBX * inner;
  if (lx == 0) return base + (lz - 1) * (kBY - 2) + (ly - 1);
  return base + (kBY - 2) * inner + (lz - 1) * (kBY - 2) + (ly - 1);
}

template <int epi, bool eta_per_q>
__global__ void __launch_bounds__(kFT, 2) ablock_fused_f32(LevelView<float> L, GatherArgs<float> a,
                                                            float* __restrict__ F, int tz) {
  pdl_wait();
  extern __shared__ float4 smem4[];
  float* C = reinterpret_cast<float*>(smem4);  // [81][kFT] contributions of the layer's cells
  float* const carry = C + 81 * kFT;  // two buffers of 3 x kPlane: top plane of the previous layer
  const int ntx = L.nc[0] / kTX, nty = L.nc[1] / kTY;
  const int tile = blockIdx.x;
  const int tx = tile % ntx, ty = (tile / ntx) % nty, tzi = tile / (ntx * nty);
  const int t = threadIdx.x;
  const int i = tx * kTX + t % kTX, j = ty * kTY + t / kTX;
  const int nb = face_count(tz);
  float* Ft = F + (size_t)tile * 3 * nb;
  for (int e = t; e < 3 * kPlane; e += kFT) carry[e] = 0.0f;
  int cur = 0;
  for (int kl = 0; kl < tz; ++kl) {
    const int k = tzi * tz + kl;
    {
      float V[3][27], YP[8];
      lattice_cell_f32<OPK_A, eta_per_q>(L, a.x, nullptr, (k * L.nc[1] + j) * L.nc[0] + i, V, YP);
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int n = 0; n < 27; ++n) C[(c * 27 + n) * kFT + t] = V[c][n];
    }
    __syncthreads();
    const float* cin = carry + cur * 3 * kPlane;
    float* cout = carry + (cur ^ 1) * 3 * kPlane;
    // one item per node column (lx, ly) of the tile: its 3 planes x 3 components
    for (int p = t; p < kPlane; p += kFT) {
      const int ly = p / kBX, lx = p - ly * kBX;
      // cells of the layer around (lx, ly), per direction the lower one (candidate
      // 0) first: an odd node lies inside one cell, an even one between two
      const bool ox = lx & 1, oy = ly & 1;
      const int cx0 = ox ? lx >> 1 : (lx >> 1) - 1, px0 = ox ? 1 : 2;
      const int cy0 = oy ? ly >> 1 : (ly >> 1) - 1, py0 = oy ? 1 : 2;
      const bool vx0 = ox || lx > 0, vx1 = !ox && lx < kBX - 1;
      const bool vy0 = oy || ly > 0, vy1 = !oy && ly < kBY - 1;
      // shared-memory offsets of the (up to) four contributions, slot 0 of each
      const int o00 = (px0 + 3 * py0) * kFT + cy0 * kTX + cx0;
      const int o01 = (3 * py0) * kFT + cy0 * kTX + (lx >> 1);
      const int o10 = px0 * kFT + (ly >> 1) * kTX + cx0;
      const int o11 = (ly >> 1) * kTX + (lx >> 1);
      const bool xy_face = lx == 0 || lx == kBX - 1 || ly == 0 || ly == kBY - 1;
      const long node0 = ((long)(2 * k) * L.Nn[1] + 2 * ty * kTY + ly) * L.Nn[0] + 2 * tx * kTX + lx;
      const long plane = (long)L.Nn[0] * L.Nn[1];
#pragma unroll
      for (int nz = 0; nz < 3; ++nz) {
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
          const float* Cc = C + (comp * 27 + 9 * nz) * kFT;
          float v = nz == 0 ? cin[comp * kPlane + p] : 0.0f;
          if (vy0 && vx0) v += Cc[o00];
          if (vy0 && vx1) v += Cc[o01];
          if (vy1 && vx0) v += Cc[o10];
          if (vy1 && vx1) v += Cc[o11];
          if (nz == 2 && kl < tz - 1) {  // kept for the next layer
            cout[comp * kPlane + p] = v;
            continue;
          }
          const int lz = 2 * kl + nz;
          if (xy_face || lz == 0 || lz == 2 * tz) {
            Ft[(size_t)comp * nb + face_index(lx, ly, lz, tz)] = v;
            continue;
          }
          gather_epilogue<float, epi>(a, (long)comp * L.n_nodes + node0 + nz * plane, v, false);
        }
      }
    }
    cur ^= 1;
    __syncthreads();
  }
}

// The nodes on tile faces: sum the partial sums of the tiles that share the
// node (z, then y, then x: lower tile first) and run the epilogue.
template <int epi>
__global__ void __launch_bounds__(256) ablock_fused_faces(LevelView<float> L, GatherArgs<float> a,
                                                          const float* __restrict__ F, int tz) {
  pdl_wait();
  const int node = blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= L.n_nodes) return;
  const int nxy = L.Nn[0] * L.Nn[1];
  const int gz = node / nxy;
  const int rem = node - gz * nxy;
  const int gy = rem / L.Nn[0];
  const int gx = rem - gy * L.Nn[0];
  const int g3[3] = {gx, gy, gz};
  const int span[3] = {2 * kTX, 2 * kTY, 2 * tz};
  const int ntiles[3] = {L.nc[0] / kTX, L.nc[1] / kTY, L.nc[2] / tz};
  int tl[3][2], lc[3][2], cnt[3];
  bool on_face = false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int q = g3[d] / span[d], r = g3[d] - q * span[d];
    cnt[d] = 0;
    if (r == 0) {
      on_face = true;
      if (q > 0) { tl[d][cnt[d]] = q - 1; lc[d][cnt[d]] = span[d]; ++cnt[d]; }
      if (q < ntiles[d]) { tl[d][cnt[d]] = q; lc[d][cnt[d]] = 0; ++cnt[d]; }
    } else {
      tl[d][0] = q; lc[d][0] = r; cnt[d] = 1;
    }
  }
  if (!on_face) return;
  const int nb = face_count(tz);
  float sum[3] = {0.0f, 0.0f, 0.0f};
  for (int bz = 0; bz < cnt[2]; ++bz)
    for (int by = 0; by < cnt[1]; ++by)
      for (int bx = 0; bx < cnt[0]; ++bx) {
        const int tile = (tl[2][bz] * ntiles[1] + tl[1][by]) * ntiles[0] + tl[0][bx];
        const int f = face_index(lc[0][bx], lc[1][by], lc[2][bz], tz);
        const float* Ft = F + (size_t)tile * 3 * nb;
#pragma unroll
        for (int c = 0; c < 3; ++c) sum[c] += Ft[(size_t)c * nb + f];
      }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    bool z = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (g3[d] == 0 && ((L.zero_faces >> ((2 * d) * 3 + c)) & 1u)) z = true;
      if (g3[d] == L.Nn[d] - 1 && ((L.zero_faces >> ((2 * d + 1) * 3 + c)) & 1u)) z = true;
    }
    gather_epilogue<float, epi>(a, (long)c * L.n_nodes + node, sum[c], z);
  }
}

template <int epi>
void launch_epi(const LevelView<float>& L, const GatherArgs<float>& a, float* F, int tz, cudaStream_t s) {
  const int blocks = (L.nc[0] / kTX) * (L.nc[1] / kTY) * (L.nc[2] / tz);
  const size_t smem = sizeof(float) * kSmemFloats;
  if (L.eta_n != 1) ablock_fused_f32<epi, true><<<blocks, kFT, smem, s>>>(L, a, F, tz);
  else ablock_fused_f32<epi, false><<<blocks, kFT, smem, s>>>(L, a, F, tz);
  ablock_fused_faces<epi><<<ceil_div(L.n_nodes, 256), 256, 0, s>>>(L, a, F, tz);
}

template <int epi, bool pq>
bool set_smem_attribute() {
  return cudaFuncSetAttribute(ablock_fused_f32<epi, pq>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(float) * kSmemFloats)) == cudaSuccess;
}

}  // namespace

int fused_a_tile_layers(const LevelView<float>& L, int n_sm, long min_cells) {
  if (L.dim != 3 || !L.structured || L.n_cells < min_cells) return 0;
  if (L.nc[0] % kTX != 0 || L.nc[1] % kTY != 0) return 0;
  const long tiles_xy = (long)(L.nc[0] / kTX) * (L.nc[1] / kTY);
  // the most layers per tile that still gives two blocks per SM
  int best = 0;
  for (int tz = 1; tz <= L.nc[2]; ++tz) {
    if (L.nc[2] % tz != 0) continue;
    if (tiles_xy * (L.nc[2] / tz) >= 2L * n_sm || best == 0) best = tz;
  }
  return best;
}

size_t fused_a_face_floats(const LevelView<float>& L, int tz) {
  const size_t tiles = (size_t)(L.nc[0] / kTX) * (L.nc[1] / kTY) * (L.nc[2] / tz);
  return tiles * 3 * (size_t)face_count(tz);
}

bool fused_a_prepare() {
  constexpr int kMaxDevices = 64;
  static signed char state[kMaxDevices];  // per device: 0 not tried, 1 ready, -1 failed
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return false;
  if (state[dev] == 0)
    state[dev] = (set_smem_attribute<EPI_STORE, false>() && set_smem_attribute<EPI_STORE, true>() &&
                  set_smem_attribute<EPI_RESID, false>() && set_smem_attribute<EPI_RESID, true>() &&
                  set_smem_attribute<EPI_CHEB, false>() && set_smem_attribute<EPI_CHEB, true>())
                     ? 1
                     : -1;
  return state[dev] == 1;
}

void launch_fused_a(const LevelView<float>& L, int epi, const GatherArgs<float>& a, float* F, int tz,
                    cudaStream_t s) {
  switch (epi) {
    case EPI_STORE: launch_epi<EPI_STORE>(L, a, F, tz, s); break;
    case EPI_RESID: launch_epi<EPI_RESID>(L, a, F, tz, s); break;
    default: launch_epi<EPI_CHEB>(L, a, F, tz, s); break;
  }
}

}  // namespace gb
