// Vector kernels (HBM-bound) of the GMG V-cycle and the FP64 Krylov solver.
#pragma once
#include "common.cuh"

namespace gb {

// Fixed reduction grid: partial sums are formed per block in a fixed order and
// summed in a fixed order, so every dot product is bit-reproducible.
constexpr int kDotBlocks = 304;  // 2 x 152 SMs
constexpr int kDotThreads = 256;
constexpr int kDotChunk = 8;     // vectors per multi-dot block
constexpr int kDotMaxChunks = 16;  // chunks per multi-dot launch (128 vectors)
// reduction workspace: per-block partials, then the arrival counters (kDotMaxChunks
// for the multi-dot chunks and one for dots) in the following kDotCounterDoubles;
// allocate kDotWorkspaceDoubles and zero it once
constexpr long kDotPartialDoubles = (long)kDotMaxChunks * (kDotChunk + 1) * kDotBlocks;
constexpr long kDotCounterDoubles = kDotMaxChunks + 1;
constexpr long kDotWorkspaceDoubles = kDotPartialDoubles + kDotCounterDoubles;

struct VecCounter {
  static long long& launches() {
    static long long n = 0;
    return n;
  }
};

template <typename T>
void v_axpby(long n, T a, const T* x, T b, T* y, cudaStream_t s);  // y = a x + b y
template <typename T>
void v_copy(long n, const T* x, T* y, cudaStream_t s);
template <typename T>
void v_scale(long n, T a, T* y, cudaStream_t s);
// y = 0 by a kernel (not a memset node, so captured kernel chains stay kernel-to-kernel)
template <typename T>
void v_zero(long n, T* y, cudaStream_t s);
template <typename Ts, typename Td>
void v_cast(long n, const Ts* x, Td* y, cudaStream_t s);
// Chebyshev: zero start  d = f2 * dinv * b, x = d
template <typename T>
void v_cheb_first(long n, const T* b, const T* dinv, T f2, T* d, T* x, cudaStream_t s);
// Chebyshev step: d = f1 d + f2 dinv (b - t), x += d
template <typename T>
void v_cheb_step(long n, const T* b, const T* t, const T* dinv, T f1, T f2, T* d, T* x, cudaStream_t s);
// out = a - b
template <typename T>
void v_sub(long n, const T* a, const T* b, T* out, cudaStream_t s);
// dst[idx[k]] = src[idx[k]]
template <typename T>
void v_copy_indexed(long m, const int* idx, const T* src, T* dst, cudaStream_t s);
template <typename T>
void v_zero_indexed(long m, const int* idx, T* dst, cudaStream_t s);
// out[perm[i]] = in[i] (scatter) or out[i] = in[perm[i]] (gather); Ts -> Td
template <typename Ts, typename Td>
void v_permute_scatter(long n, const int* perm, const Ts* in, Td* out, cudaStream_t s);
template <typename Ts, typename Td>
void v_permute_gather(long n, const int* perm, const Ts* in, Td* out, cudaStream_t s);
// y += A x (CSR)
template <typename T>
void v_spmv_add(long rows, const int* ptr, const int* col, const T* val, const T* x, T* y, cudaStream_t s);
// y[r] = (A x)[r] for r < rows, 0 for rows <= r < n
template <typename T>
void v_spmv_set(long rows, long n, const int* ptr, const int* col, const T* val, const T* x, T* y, cudaStream_t s);
// The reductions and the multi-axpy take an optional device flag `active`: when
// it points to 0 the launches return at once (a step that the device decided to
// skip without a round trip to the host).
// out[j] = <w, V_j> for j < k (V rows of stride ld), plus out[k] = <w, w> if with_norm
// partial: the reduction workspace (kDotWorkspaceDoubles, zeroed once)
void v_multidot(long n, const double* w, const double* V, long ld, int k, bool with_norm, double* out_dev,
                double* partial, cudaStream_t s, const int* active = nullptr);
// one classical Gram-Schmidt pass of an Arnoldi step after its multi-dot (see vec.cu);
// pass 0 also sets *shift (when given) for the float-pair passes of the next step
void v_cgs_update(long n, int j, int pass, const double* dots, const double* V, long ld, double* w, double* h,
                  double* arn, int* need2, double* partial, cudaStream_t s, int* shift = nullptr);
// One Arnoldi step (classical Gram-Schmidt with the conditional second pass,
// the next basis vector and the Hessenberg column h[0..j+1]) on the float-pair
// copy Vs of the basis (entries (h, l) with h + l the FP64 entry; column stride
// lds even, 16-byte aligned columns): five launches, the partial sums of each
// reduced by the next (see vec.cu). w is scaled by 2^-(*shift) while it is split;
// the step writes the next step's exponent to *shift_next (another address) and
// whether the second pass ran to *need2. j + 1 <= 128.
constexpr int kDfChunk = 16;     // vectors per block of the dots launch
constexpr int kDfMaxChunks = 8;  // chunks of one step
constexpr int kGsMaxK = kDfMaxChunks * kDfChunk;  // basis vectors of one float-pair step, at most (128)
void v_arnoldi_step_df(long n, int j, const float2* Vs, long lds, double* w, double* vnext, float2* vsnext,
                       double* h, double* arn, int* need2, const int* shift, int* shift_next, double* workspace,
                       cudaStream_t s);
// v = sc w canonicalised to its float pair, the pair into vs (sc = *sc_dev if given)
void v_basis_df(long n, const double* sc_dev, double sc_host, const double* w, double* v, float2* vs,
                cudaStream_t s);
template <typename T>
void v_dot(long n, const T* a, const T* b, double* out_dev, double* partial, cudaStream_t s,
           const int* active = nullptr);
// Eigenvalue-estimate CG with device scalars (see vec.cu): s holds kEigHist +
// 2 its doubles (r.z in s[0] before the first step), f three ints.
constexpr int kEigHist = 8;
void v_eig_start(int* f, cudaStream_t st);
// one step after Ap = A p: alpha, r, |r|, z = D^-1 r, beta, p
template <typename T>
void v_eig_step(long n, T* p, const T* Ap, T* r, T* z, const T* dinv, double* s, int* f, int its,
                double* partial, cudaStream_t st);
// w += sum_j coef[j] V_j  (coef on the device)
void v_multiaxpy(long n, int k, const double* coef_dev, const double* V, long ld, double* w, cudaStream_t s,
                 const int* active = nullptr);
// y = S x for a dense symmetric n x n matrix S (FP64), one warp per row
void v_symv_dense(long n, const double* S, const double* x, double* y, cudaStream_t s);
// NaN / Inf check: flag[0] |= 1 if any non-finite entry
template <typename T>
void v_check_finite(long n, const T* x, int* flag, cudaStream_t s);

}  // namespace gb
