// FP64-accurate solves on top of the low-precision factor: the pieces of the refinement loop.
//
//   gbx_spotri_diag   inverses of the FP32 diagonal factor tiles (one op_trsm per 128 columns)
//   gbx_sprecond      z := (L L^T)^{-1} r with the FP32 tiled factor; FP64 vectors in and out,
//                     FP32 arithmetic inside; a forward and a backward sweep over tile columns,
//                     each step one diagonal-inverse product and one column update
//   gbx_dsymm_tiled   Y := alpha A X + beta Y with A the FP64 tile-major lower matrix (symmetric)
//   gbx_dposv_mixed   low-precision factor + preconditioned CG in FP64 until the normwise
//                     backward error max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf)
//                     reaches the tolerance
// The right-hand sides are column-major N x nrhs (leading dimension N).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "block_ops.cuh"
#include "gbx_common.cuh"
#include "gbx_potrf.h"

namespace gbx {
namespace mixed {
int plan_batch(int batch, const int* n, int NB, void* work, size_t work_bytes, cudaStream_t s, int sched);
int run_batch(int batch, const int* n, int NB, float* W, int prec, double fp64_cond, const int* dsel, void* work,
              size_t work_bytes, cudaStream_t s);
// device addresses of a batched factorisation's results in its workspace
struct InfoPtrs {
  const DagState* st;
  const int* minfo;
  const float* cond;
  const int* nfp64;
};
InfoPtrs info_ptrs(int batch, const int* n, int NB, const void* work);
}  // namespace mixed
}  // namespace gbx

namespace gbx {
namespace refine {

constexpr int kMaxRhs = 16;

__device__ __forceinline__ long long slot_of(int m, int n, int NT) {
  return (long long)n * NT - (long long)n * (n - 1) / 2 + (m - n);
}
__host__ __device__ __forceinline__ int tdim(int t, int N, int NB, int NT) { return t == NT - 1 ? N - (NT - 1) * NB : NB; }

// One matrix of a batched call: its tiles start at tile slot slot0 of A (FP64) and W (FP32), its
// diagonal-tile inverses at tile inv0 of Inv, its vectors (N x nrhs, column-major, leading
// dimension N) at element vec0 of every vector array. A single matrix is the table {0, 0, 0, N, NT}.
struct RMat {
  long long slot0, inv0, vec0;
  int N, NT;
};

// Every kernel body below works on one matrix (pointers already offset to it); the single-matrix
// kernels call it directly, the batched kernels with matrix list[1 + blockIdx.z] of the table. A
// list lives in device memory as {count, table index, ...}: launches cover the largest possible
// count in z and the slices at or past the current count return at once, so the lists can change
// on the device between launches of a captured graph.
#define GBX_MAT_OF_BLOCK()                       \
  if ((int)blockIdx.z >= list[0]) return;        \
  const RMat& mt = mats[list[1 + blockIdx.z]]

// Out = L_KK^{-T} (column-major), i.e. row r of Out holds column r of L_KK^{-1}; 128 rows per CTA
__device__ void diag_inverse_body(const float* W, float* Inv, int N, int NB, int NT, float* sm) {
  const int K = blockIdx.x, r0 = blockIdx.y * kBlk;
  if (K >= NT) return;
  const int n = tdim(K, N, NB, NT);
  if (r0 >= n) return;
  const int m = min(kBlk, n - r0);
  float* out = Inv + (long long)K * NB * NB;
  for (int idx = threadIdx.x; idx < kBlk * NB; idx += blockDim.x) {  // rows r0.. of the identity
    const int r = idx % kBlk, c = idx / kBlk;
    if (r < m) out[(r0 + r) + (long long)c * NB] = (r0 + r == c) ? 1.f : 0.f;
  }
  __syncthreads();
  // row r of L^{-T} is zero left of column r: rows r0.. solve against the trailing L(r0:, r0:) only
  const float* L = W + slot_of(K, K, NT) * (long long)NB * NB + r0 + (long long)r0 * NB;
  op_trsm<float, true>(L, NB, out + r0 + (long long)r0 * NB, NB, m, n - r0, sm);
}
__global__ void __launch_bounds__(kThreads, 1) diag_inverse_kernel(const float* W, float* Inv, int N, int NB, int NT) {
  extern __shared__ __align__(16) float sm_f[];
  diag_inverse_body(W, Inv, N, NB, NT, sm_f);
}
__global__ void __launch_bounds__(kThreads, 1)
    diag_inverse_batched(const RMat* mats, const int* list, const float* W, float* Inv, int NB) {
  extern __shared__ __align__(16) float sm_f[];
  GBX_MAT_OF_BLOCK();
  diag_inverse_body(W + mt.slot0 * NB * NB, Inv + mt.inv0 * NB * NB, mt.N, NB, mt.NT, sm_f);
}

// forward step, diagonal part: y_K = L_KK^{-1} x_K (Out^T x_K), in place in x
// one warp per output element c (lanes over r), all right-hand sides
__device__ void fwd_diag_body(const float* Inv, const float* X, float* Y, int N, int NB, int NT, int K, int nrhs,
                              float* xs_f) {
  if (K >= NT) return;
  const int n = tdim(K, N, NB, NT);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (blockIdx.x * nw >= n) return;
  const float* out = Inv + (long long)K * NB * NB;
  for (int idx = threadIdx.x; idx < n * nrhs; idx += blockDim.x) {
    const int r = idx % n, j = idx / n;
    xs_f[j * NB + r] = X[(long long)j * N + (long long)K * NB + r];
  }
  __syncthreads();
  for (int c = blockIdx.x * nw + warp; c < n; c += gridDim.x * nw) {
    float acc[kMaxRhs];
    for (int j = 0; j < nrhs; ++j) acc[j] = 0.f;
    for (int r = lane; r <= c; r += 32) {  // L^{-1} is lower: (L^{-1})(c, r) = Out(r, c), r <= c
      const float v = out[r + (long long)c * NB];
      for (int j = 0; j < nrhs; ++j) acc[j] = fmaf(v, xs_f[j * NB + r], acc[j]);
    }
    for (int j = 0; j < nrhs; ++j) {
      float a = acc[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0) Y[(long long)j * N + (long long)K * NB + c] = a;
    }
  }
}
__global__ void fwd_diag_kernel(const float* Inv, const float* X, float* Y, int N, int NB, int NT, int K, int nrhs) {
  extern __shared__ float xs_f[];  // [nrhs][NB]
  fwd_diag_body(Inv, X, Y, N, NB, NT, K, nrhs, xs_f);
}

// forward step, column update: x_M -= L_MK y_K for every M > K; thread per row, y_K in smem
__device__ void fwd_update_body(const float* W, const float* Y, float* X, int N, int NB, int NT, int K, int nrhs,
                                float* ys_f) {
  const long long row0 = (long long)(K + 1) * NB + (long long)blockIdx.x * blockDim.x;
  if (K >= NT || row0 >= N) return;  // whole CTA past the matrix
  const int kn = tdim(K, N, NB, NT);
  for (int idx = threadIdx.x; idx < kn * nrhs; idx += blockDim.x) {
    const int r = idx % kn, j = idx / kn;
    ys_f[j * NB + r] = Y[(long long)j * N + (long long)K * NB + r];
  }
  __syncthreads();
  const long long row = row0 + threadIdx.x;  // global row
  if (row >= N) return;
  const int M = (int)(row / NB), i = (int)(row % NB);
  const float* L = W + slot_of(M, K, NT) * (long long)NB * NB;
  float acc[kMaxRhs];
  for (int j = 0; j < nrhs; ++j) acc[j] = 0.f;
  int c = 0;
  for (; c + 8 <= kn; c += 8) {  // eight independent loads in flight per thread
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldg(L + i + (long long)(c + u) * NB);
#pragma unroll
    for (int u = 0; u < 8; ++u)
      for (int j = 0; j < nrhs; ++j) acc[j] = fmaf(v[u], ys_f[j * NB + c + u], acc[j]);
  }
  for (; c < kn; ++c) {
    const float v = __ldg(L + i + (long long)c * NB);
    for (int j = 0; j < nrhs; ++j) acc[j] = fmaf(v, ys_f[j * NB + c], acc[j]);
  }
  for (int j = 0; j < nrhs; ++j) X[(long long)j * N + row] -= acc[j];
}
__global__ void fwd_update_kernel(const float* W, const float* Y, float* X, int N, int NB, int NT, int K, int nrhs) {
  extern __shared__ float ys_f[];  // [nrhs][NB]
  fwd_update_body(W, Y, X, N, NB, NT, K, nrhs, ys_f);
}

// backward step, diagonal part: z_K = L_KK^{-T} y_K. A CTA owns 32 output rows (lanes, coalesced
// over i); its 8 warps split the column range and reduce through shared memory.
__device__ void bwd_diag_body(const float* Inv, const float* Y, float* X, int N, int NB, int NT, int K, int nrhs,
                              float* ys_f) {
  if (K >= NT) return;
  const int n = tdim(K, N, NB, NT);
  if (blockIdx.x * 32 >= n) return;
  const float* out = Inv + (long long)K * NB * NB;
  for (int idx = threadIdx.x; idx < n * nrhs; idx += blockDim.x) {
    const int r = idx % n, j = idx / n;
    ys_f[j * NB + r] = Y[(long long)j * N + (long long)K * NB + r];
  }
  __syncthreads();
  float* part = ys_f + nrhs * NB;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  float acc[kMaxRhs];
  for (int j = 0; j < nrhs; ++j) acc[j] = 0.f;
  if (i < n) {
    const int span = (n - i + nw - 1) / nw;
    const int cb = i + warp * span, ce = min(n, cb + span);
    for (int c = cb; c < ce; ++c) {  // L^{-T} upper: (L^{-T})(i, c) = Out(i, c), c >= i
      const float v = __ldg(out + i + (long long)c * NB);
      for (int j = 0; j < nrhs; ++j) acc[j] = fmaf(v, ys_f[j * NB + c], acc[j]);
    }
  }
  for (int j = 0; j < nrhs; ++j) part[(warp * nrhs + j) * 32 + lane] = acc[j];
  __syncthreads();
  if (warp == 0 && i < n)
    for (int j = 0; j < nrhs; ++j) {
      float s = 0.f;
      for (int w = 0; w < nw; ++w) s += part[(w * nrhs + j) * 32 + lane];
      X[(long long)j * N + (long long)K * NB + i] = s;
    }
}
__global__ void bwd_diag_kernel(const float* Inv, const float* Y, float* X, int N, int NB, int NT, int K, int nrhs) {
  extern __shared__ float ys_f[];  // [nrhs][NB] then [8 warps][nrhs][32] partial sums
  bwd_diag_body(Inv, Y, X, N, NB, NT, K, nrhs, ys_f);
}

// backward step, column update: y_J -= L_KJ^T z_K for every J < K; warp per output element c
__device__ void bwd_update_body(const float* W, const float* X, float* Y, int N, int NB, int NT, int K, int nrhs,
                                float* zs_f) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const long long total = (long long)K * NB;  // rows of y_0 .. y_{K-1}
  if (K >= NT || (long long)blockIdx.x * nw >= total) return;
  const int kn = tdim(K, N, NB, NT);
  for (int idx = threadIdx.x; idx < kn * nrhs; idx += blockDim.x) {
    const int r = idx % kn, j = idx / kn;
    zs_f[j * NB + r] = X[(long long)j * N + (long long)K * NB + r];
  }
  __syncthreads();
  for (long long g = (long long)blockIdx.x * nw + warp; g < total; g += (long long)gridDim.x * nw) {
    const int J = (int)(g / NB), c = (int)(g % NB);
    const float* L = W + slot_of(K, J, NT) * (long long)NB * NB;
    float acc[kMaxRhs];
    for (int j = 0; j < nrhs; ++j) acc[j] = 0.f;
    for (int r = lane; r < kn; r += 32) {
      const float v = __ldg(L + r + (long long)c * NB);
      for (int j = 0; j < nrhs; ++j) acc[j] = fmaf(v, zs_f[j * NB + r], acc[j]);
    }
    for (int j = 0; j < nrhs; ++j) {
      float a = acc[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0) Y[(long long)j * N + g] -= a;
    }
  }
}
__global__ void bwd_update_kernel(const float* W, const float* X, float* Y, int N, int NB, int NT, int K, int nrhs) {
  extern __shared__ float zs_f[];  // [nrhs][NB]
  bwd_update_body(W, X, Y, N, NB, NT, K, nrhs, zs_f);
}

__global__ void d2s_kernel(const double* in, float* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}
__global__ void s2d_kernel(const float* in, double* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

// tile (m, n) of lower slot `slot` (column-major slot order); false past the last slot
__device__ __forceinline__ bool slot_tile(int slot, int NT, int& m, int& n) {
  if (slot >= NT * (NT + 1) / 2) return false;
  n = 0;
  long long first = 0;
  while (first + (NT - n) <= slot) {
    first += NT - n;
    ++n;
  }
  m = n + (int)(slot - first);
  return true;
}

// ---- FP64 symmetric product Y := alpha A X + beta Y (A lower tiles) -----------------------------
// part 1: Y_m += A_mn X_n over the stored lower part (thread per row); diagonal tiles use j <= i
// part 2: Y_n += A_mn^T X_m over the strictly lower part (warp per column)
__device__ void symm_rows_body(const double* A, const double* X, double* Y, int N, int NB, int NT, int nrhs,
                               double alpha, double* xs_d) {
  const int slot = blockIdx.x, rb = blockIdx.y;
  int m, n;
  if (!slot_tile(slot, NT, m, n)) return;
  const int mrows = tdim(m, N, NB, NT), ncols = tdim(n, N, NB, NT);
  if (rb * (int)blockDim.x >= mrows) return;
  const int i = rb * blockDim.x + threadIdx.x;
  const double* T = A + (long long)slot * NB * NB;
  double acc[kMaxRhs];
  for (int j = 0; j < nrhs; ++j) acc[j] = 0.0;
  for (int c0 = 0; c0 < ncols; c0 += 512) {
    const int cw = min(512, ncols - c0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < cw * nrhs; idx += blockDim.x) {
      const int c = idx % cw, j = idx / cw;
      xs_d[j * 512 + c] = X[(long long)j * N + (long long)n * NB + c0 + c];
    }
    __syncthreads();
    if (i < mrows) {
      const int cend = (m == n) ? min(cw, i - c0 + 1) : cw;
      for (int c = 0; c < cend; ++c) {
        const double v = T[i + (long long)(c0 + c) * NB];
        for (int j = 0; j < nrhs; ++j) acc[j] = fma(v, xs_d[j * 512 + c], acc[j]);
      }
    }
  }
  if (i < mrows)
    for (int j = 0; j < nrhs; ++j) atomicAdd(Y + (long long)j * N + (long long)m * NB + i, alpha * acc[j]);
}
__global__ void symm_rows_kernel(const double* A, const double* X, double* Y, int N, int NB, int NT, int nrhs,
                                 double alpha) {
  extern __shared__ double xs_d[];  // [nrhs][512]
  symm_rows_body(A, X, Y, N, NB, NT, nrhs, alpha, xs_d);
}

__device__ void symm_cols_body(const double* A, const double* X, double* Y, int N, int NB, int NT, int nrhs,
                               double alpha, double* xs_d) {
  const int slot = blockIdx.x;
  int m, n;
  if (!slot_tile(slot, NT, m, n)) return;
  const int mrows = tdim(m, N, NB, NT), ncols = tdim(n, N, NB, NT);
  const double* T = A + (long long)slot * NB * NB;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if ((int)blockIdx.y * nw >= ncols) return;
  for (int r0 = 0; r0 < mrows; r0 += 512) {
    const int rw = min(512, mrows - r0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < rw * nrhs; idx += blockDim.x) {
      const int r = idx % rw, j = idx / rw;
      xs_d[j * 512 + r] = X[(long long)j * N + (long long)m * NB + r0 + r];
    }
    __syncthreads();
    for (int c = blockIdx.y * nw + warp; c < ncols; c += gridDim.y * nw) {
      double acc[kMaxRhs];
      for (int j = 0; j < nrhs; ++j) acc[j] = 0.0;
      for (int r = lane; r < rw; r += 32) {
        if (m == n && r0 + r <= c) continue;  // strictly lower part only
        const double v = T[(r0 + r) + (long long)c * NB];
        for (int j = 0; j < nrhs; ++j) acc[j] = fma(v, xs_d[j * 512 + r], acc[j]);
      }
      for (int j = 0; j < nrhs; ++j) {
        double a = acc[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) atomicAdd(Y + (long long)j * N + (long long)n * NB + c, alpha * a);
      }
    }
  }
}
__global__ void symm_cols_kernel(const double* A, const double* X, double* Y, int N, int NB, int NT, int nrhs,
                                 double alpha) {
  extern __shared__ double xs_d[];  // [nrhs][512]
  symm_cols_body(A, X, Y, N, NB, NT, nrhs, alpha, xs_d);
}

// ---- the same product in double-float arithmetic (FP32 pairs) for the refinement's residuals ----
// A = Ah + Al with Ah = fl32(A), Al = fl32(A - Ah) (48 significant bits, split once per solve), x split
// the same way per tile; a product a*x accumulates as the exact FP32 product pair of Ah*xh
// (TwoProduct by FMA) plus the cross terms Ah*xl + Al*xh, and the sum is carried as a TwoSum pair.
// Error about 2^-47 relative to sum |a x|, far below the 1e-14 backward-error target, at FP32 rates
// (GB300 runs FP32 FMAs ~67x faster than FP64 ones). Intrinsics keep the compiler from contracting
// the error-free transformations.
//
// The split by integer arithmetic on the bit pattern (IEEE-754 round to nearest, ties to even): with
// a = (2^52 + m) 2^(e-1075), hi keeps the top 23 bits of m, rounded on the low 29 bits, and
// a - hi = +-r 2^(e-1075) with |r| <= 2^28, so lo = fl32(r) 2^(e-1075) exactly. Bitwise equal to the
// FP64 route hi = fl32(a), lo = fl32(a - hi) whenever hi and lo are FP32 normal numbers (biased
// exponent e in [950, 1149]); other values (zero, tiny, huge, Inf, NaN) take the FP64 route, which
// costs four FP64-pipe operations per element and would bound a pass over A on this GPU.
__device__ __forceinline__ void split_f64(double a, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e >= 950 && e <= 1149) {
    const unsigned t = (unsigned)((b >> 29) & 0x7FFFFFu), rem = (unsigned)(b & 0x1FFFFFFFu);
    const bool up = rem > 0x10000000u || (rem == 0x10000000u && (t & 1u));
    const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
    hi = __uint_as_float(sgn | ((((unsigned)(e - 896) << 23) | t) + (up ? 1u : 0u)));
    int r = up ? (int)rem - (1 << 29) : (int)rem;
    if (sgn) r = -r;
    lo = __int2float_rn(r) * __uint_as_float((unsigned)(e - 948) << 23);  // r 2^(e-1075)
  } else {
    hi = __double2float_rn(a);
    lo = __double2float_rn(a - (double)hi);
  }
}

// One pass over the FP64 tiles of every listed matrix (one CTA per tile slot, padding included):
// W = fl32(A), the factor's working copy; Ah + Al = A, the split for the double-float residual
// products (both 0 outside the matrix's lower triangle); and the row sums of |A| for ||A||_inf,
// where the strictly lower part of each tile also counts for the rows of its columns. Thread t
// owns rows 2t, 2t + 1 and walks the columns, so a CTA reads each 4 KB column in one contiguous
// burst (16-byte loads, eight columns in flight per thread) and keeps its row sums in registers;
// the column sums meet in warp shuffles and shared memory. The sums of |fl32(a)| are carried in FP32 over at most 8 terms per thread and column
// group and added up in FP64 (relative error about 1e-6, for a norm). NB <= 512.
__global__ void __launch_bounds__(256) prep_batched(const RMat* mats, const int* list, const double* A, float* W,
                                                    float* Ah, float* Al, double* rs, int NB, int nrhs) {
  GBX_MAT_OF_BLOCK();
  __shared__ float s_col[8][512];
  int m, n;
  if (!slot_tile(blockIdx.x, mt.NT, m, n)) return;
  const int mrows = tdim(m, mt.N, NB, mt.NT), ncols = tdim(n, mt.N, NB, mt.NT);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = 2 * threadIdx.x;  // rows i0, i0 + 1
  const bool diag = m == n, live = i0 < NB;
  const long long tb = (mt.slot0 + blockIdx.x) * (long long)NB * NB;
  double* rsm = rs + mt.vec0 / nrhs;
  double rsum0 = 0.0, rsum1 = 0.0;
  for (int c0 = 0; c0 < NB; c0 += 8) {
    double2 a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      a[u] = live ? __ldcs((const double2*)(A + tb + i0 + (long long)(c0 + u) * NB)) : make_double2(0.0, 0.0);
    float p0 = 0.f, p1 = 0.f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int c = c0 + u;
      // entries of the lower triangle inside the matrix; the rest (padding past N, the strict upper
      // part of diagonal tiles) is never read by the factorisation or the products and becomes 0
      const bool ok0 = c < ncols && i0 < mrows && (!diag || c <= i0);
      const bool ok1 = c < ncols && i0 + 1 < mrows && (!diag || c <= i0 + 1);
      float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
      if (ok0) split_f64(a[u].x, h0, l0);
      if (ok1) split_f64(a[u].y, h1, l1);
      if (live) {
        const long long e = tb + i0 + (long long)c * NB;
        *(float2*)(W + e) = make_float2(h0, h1);
        *(float2*)(Ah + e) = make_float2(h0, h1);
        *(float2*)(Al + e) = make_float2(l0, l1);
      }
      const float v0 = fabsf(h0), v1 = fabsf(h1);
      p0 += v0;
      p1 += v1;
      float cv = ((!diag || i0 != c) ? v0 : 0.f) + ((!diag || i0 + 1 != c) ? v1 : 0.f);  // strictly lower
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) cv += __shfl_xor_sync(0xffffffffu, cv, o);
      if (lane == 0) s_col[warp][c] = cv;
    }
    rsum0 += (double)p0;
    rsum1 += (double)p1;
  }
  if (i0 < mrows) atomicAdd(rsm + (long long)m * NB + i0, rsum0);
  if (i0 + 1 < mrows) atomicAdd(rsm + (long long)m * NB + i0 + 1, rsum1);
  __syncthreads();
  for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
    float t = 0.f;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += s_col[w][c];
    if (!diag || c + 1 < mrows) atomicAdd(rsm + (long long)n * NB + c, (double)t);
  }
}

// hi + lo = a elementwise (the split of the residual products, for vectors and for testing)
__global__ void split_f64_kernel(const double* __restrict__ A, float* __restrict__ hi, float* __restrict__ lo,
                                 long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float h, l;
    split_f64(__ldcs(A + i), h, l);
    hi[i] = h;
    lo[i] = l;
  }
}

__device__ __forceinline__ void df_fma(float& sh, float& sl, float ah, float al, float xh, float xl) {
  const float p = __fmul_rn(ah, xh);
  const float e = __fmaf_rn(ah, xh, -p);                        // ah*xh = p + e exactly
  const float c = __fmaf_rn(ah, xl, __fmaf_rn(al, xh, e));      // low-order part of the product
  const float t = __fadd_rn(sh, p);                             // TwoSum(sh, p) = t + err
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, c));
}

// x split once per product into FP32 pairs (same layout as x), then staged per tile
__global__ void split_vec_kernel(const double* X, float* xh, float* xl, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = X[i];
    const float h = __double2float_rn(v);
    xh[i] = h;
    xl[i] = __double2float_rn(v - (double)h);
  }
}
__device__ __forceinline__ void load_pair(const float* Xh, const float* Xl, int N, long long off, int w, int nrhs,
                                          float* xh, float* xl) {
  for (int idx = threadIdx.x; idx < w * nrhs; idx += blockDim.x) {
    const int c = idx % w, j = idx / w;
    xh[j * 512 + c] = Xh[(long long)j * N + off + c];
    xl[j * 512 + c] = Xl[(long long)j * N + off + c];
  }
}

// (sh, sl) += (th, tl) for double-float pairs (TwoSum on the high parts)
__device__ __forceinline__ void df_add(float& sh, float& sl, float th, float tl) {
  const float t = __fadd_rn(sh, th);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(th, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, tl));
}

// rows: thread per row; Y_m += A_mn X_n (diagonal tiles: columns <= row)
template <int NR>
__device__ void symm_rows_df_body(const float* Ah, const float* Al, const float* Xh, const float* Xl, double* Y, int N,
                                  int NB, int NT, int nrhs, double alpha, float* sm) {
  const int slot = blockIdx.x, rb = blockIdx.y;
  int m, n;
  if (!slot_tile(slot, NT, m, n)) return;
  const int mrows = tdim(m, N, NB, NT), ncols = tdim(n, N, NB, NT);
  if (rb * (int)blockDim.x >= mrows) return;
  float* xh = sm;
  float* xl = sm + nrhs * 512;
  const int i = rb * blockDim.x + threadIdx.x;
  const long long tb = (long long)slot * NB * NB;
  float sh[NR], sl[NR];
#pragma unroll
  for (int j = 0; j < NR; ++j) sh[j] = sl[j] = 0.f;
  for (int c0 = 0; c0 < ncols; c0 += 512) {
    const int cw = min(512, ncols - c0);
    __syncthreads();
    load_pair(Xh, Xl, N, (long long)n * NB + c0, cw, nrhs, xh, xl);
    __syncthreads();
    if (i < mrows) {
      const int cend = (m == n) ? min(cw, i - c0 + 1) : cw;
      int c = 0;
      for (; c + 4 <= cend; c += 4) {  // four independent load pairs in flight
        float ah[4], al[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const long long e = tb + i + (long long)(c0 + c + u) * NB;
          ah[u] = __ldg(Ah + e);
          al[u] = __ldg(Al + e);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int j = 0; j < NR; ++j)
            if (j < nrhs) df_fma(sh[j], sl[j], ah[u], al[u], xh[j * 512 + c + u], xl[j * 512 + c + u]);
      }
      for (; c < cend; ++c) {
        const long long e = tb + i + (long long)(c0 + c) * NB;
        const float ah = __ldg(Ah + e), al = __ldg(Al + e);
#pragma unroll
        for (int j = 0; j < NR; ++j)
          if (j < nrhs) df_fma(sh[j], sl[j], ah, al, xh[j * 512 + c], xl[j * 512 + c]);
      }
    }
  }
  if (i < mrows)
#pragma unroll
    for (int j = 0; j < NR; ++j)
      if (j < nrhs) atomicAdd(Y + (long long)j * N + (long long)m * NB + i, alpha * ((double)sh[j] + (double)sl[j]));
}

// columns: warp per column over the strictly lower part; Y_n += A_mn^T X_m. The lane sums meet in
// double-float shuffles; each warp converts its columns' sums to FP64 together, once per 8 columns,
// so that the FP64 pipe (slow on this GPU) sees a handful of instructions per column.
template <int NR>
__device__ void symm_cols_df_body(const float* Ah, const float* Al, const float* Xh, const float* Xl, double* Y, int N,
                                  int NB, int NT, int nrhs, double alpha, float* sm) {
  const int slot = blockIdx.x;
  int m, n;
  if (!slot_tile(slot, NT, m, n)) return;
  const int mrows = tdim(m, N, NB, NT), ncols = tdim(n, N, NB, NT);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if ((int)blockIdx.y * nw >= ncols) return;
  float* xh = sm;
  float* xl = sm + nrhs * 512;
  float* res = sm + 2 * nrhs * 512 + warp * (8 * NR * 2);  // [8 columns][NR][hi, lo] per warp
  const long long tb = (long long)slot * NB * NB;
  for (int r0 = 0; r0 < mrows; r0 += 512) {
    const int rw = min(512, mrows - r0);
    __syncthreads();
    load_pair(Xh, Xl, N, (long long)m * NB + r0, rw, nrhs, xh, xl);
    __syncthreads();
    int q = 0, cfirst = -1;
    for (int c = blockIdx.y * nw + warp; c < ncols; c += gridDim.y * nw) {
      if (cfirst < 0) cfirst = c;
      float sh[NR], sl[NR];
#pragma unroll
      for (int j = 0; j < NR; ++j) sh[j] = sl[j] = 0.f;
      for (int r = lane; r < rw; r += 128) {  // rows r, r + 32, r + 64, r + 96: four load pairs in flight
        float ah[4], al[4];
        int xi[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int rr = r + 32 * u;
          const bool ok = rr < rw && !(m == n && r0 + rr <= c);  // strictly lower part only
          const long long e = tb + (r0 + rr) + (long long)c * NB;
          ah[u] = ok ? __ldg(Ah + e) : 0.f;  // a masked entry adds an exact zero
          al[u] = ok ? __ldg(Al + e) : 0.f;
          xi[u] = ok ? rr : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int j = 0; j < NR; ++j)
            if (j < nrhs) df_fma(sh[j], sl[j], ah[u], al[u], xh[j * 512 + xi[u]], xl[j * 512 + xi[u]]);
      }
#pragma unroll
      for (int j = 0; j < NR; ++j) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float th = __shfl_xor_sync(0xffffffffu, sh[j], o), tl = __shfl_xor_sync(0xffffffffu, sl[j], o);
          df_add(sh[j], sl[j], th, tl);
        }
      }
      if (lane == 0)
#pragma unroll
        for (int j = 0; j < NR; ++j) {
          res[(q * NR + j) * 2] = sh[j];
          res[(q * NR + j) * 2 + 1] = sl[j];
        }
      ++q;
      const int cnext = c + gridDim.y * nw;
      if (q == 8 || cnext >= ncols) {  // flush: every lane converts and adds a few of the results
        __syncwarp();
        const int stride = gridDim.y * nw;
        for (int e = lane; e < q * nrhs; e += 32) {
          const int qq = e / nrhs, j = e % nrhs;
          const double v = (double)res[(qq * NR + j) * 2] + (double)res[(qq * NR + j) * 2 + 1];
          atomicAdd(Y + (long long)j * N + (long long)n * NB + cfirst + qq * stride, alpha * v);
        }
        __syncwarp();
        q = 0;
        cfirst = -1;
      }
    }
  }
}

template <int NR>
__global__ void symm_rows_df_batched(const RMat* mats, const int* list, const float* Ah, const float* Al,
                                     const float* Xh, const float* Xl, double* Y, int NB, int nrhs, double alpha) {
  extern __shared__ float xsp_f[];  // [2][nrhs][512]
  GBX_MAT_OF_BLOCK();
  const long long o = mt.slot0 * NB * NB;
  symm_rows_df_body<NR>(Ah + o, Al + o, Xh + mt.vec0, Xl + mt.vec0, Y + mt.vec0, mt.N, NB, mt.NT, nrhs, alpha, xsp_f);
}
template <int NR>
__global__ void symm_cols_df_batched(const RMat* mats, const int* list, const float* Ah, const float* Al,
                                     const float* Xh, const float* Xl, double* Y, int NB, int nrhs, double alpha) {
  extern __shared__ float xsp_f[];  // [2][nrhs][512], then [8 warps][8 columns][NR][2] results
  GBX_MAT_OF_BLOCK();
  const long long o = mt.slot0 * NB * NB;
  symm_cols_df_body<NR>(Ah + o, Al + o, Xh + mt.vec0, Xl + mt.vec0, Y + mt.vec0, mt.N, NB, mt.NT, nrhs, alpha, xsp_f);
}
// launches the instantiation with the smallest NR >= nrhs
template <int NR>
int set_df_attrs(int big) {
  if (cudaFuncSetAttribute(symm_rows_df_batched<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(symm_cols_df_batched<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess)
    return GBX_ERR_CUDA;
  return GBX_OK;
}
template <int NR>
void launch_symm_df(dim3 gr, dim3 gc, size_t vs, cudaStream_t s, const RMat* mats, const int* list, const float* Ah,
                    const float* Al, const float* xh, const float* xl, double* y, int NB, int nrhs, double alpha) {
  symm_rows_df_batched<NR><<<gr, 128, vs, s>>>(mats, list, Ah, Al, xh, xl, y, NB, nrhs, alpha);
  symm_cols_df_batched<NR><<<gc, 256, vs + (size_t)8 * 8 * NR * 2 * sizeof(float), s>>>(mats, list, Ah, Al, xh, xl, y,
                                                                                        NB, nrhs, alpha);
}
// y += alpha A x with x split into FP32 pairs xh, xl beforehand
void symm_df(dim3 gr, dim3 gc, size_t vs, cudaStream_t s, const RMat* mats, const int* list, const float* Ah,
             const float* Al, const float* xh, const float* xl, double* y, int NB, int nrhs, double alpha) {
  if (nrhs <= 1) launch_symm_df<1>(gr, gc, vs, s, mats, list, Ah, Al, xh, xl, y, NB, nrhs, alpha);
  else if (nrhs <= 2) launch_symm_df<2>(gr, gc, vs, s, mats, list, Ah, Al, xh, xl, y, NB, nrhs, alpha);
  else if (nrhs <= 4) launch_symm_df<4>(gr, gc, vs, s, mats, list, Ah, Al, xh, xl, y, NB, nrhs, alpha);
  else if (nrhs <= 8) launch_symm_df<8>(gr, gc, vs, s, mats, list, Ah, Al, xh, xl, y, NB, nrhs, alpha);
  else launch_symm_df<16>(gr, gc, vs, s, mats, list, Ah, Al, xh, xl, y, NB, nrhs, alpha);
}

// ---- preconditioner sweeps as persistent launches ---------------------------------------------
// z := (L L^T)^{-1} r in two launches (forward L y = x, backward L^T z = y), each over an in-order
// list of tile tasks of every listed matrix:
//   forward  DIAG(K):   wait until the K updates of tile row K are in; y_K = L_KK^{-1} x_K; flag K
//            UPD(M, K): wait for flag K; x_M -= L_MK y_K (FP32 atomics); count one for row M
//   backward DIAG(K):   wait until the NT-1-K updates of row K are in; z_K = L_KK^{-T} y_K; flag K
//            UPD(M, K): wait for flag M; y_K -= L_MK^T z_M; count one for row K
// Every task waits only on tasks earlier in its list, so CTAs taking tasks in list order cannot
// deadlock; waits are bounded (the run state's status becomes GBX_ERR_TIMEOUT). x and y are the
// FP32 vectors at vec0 of each matrix (column j of a matrix at j * N); vectors written by other
// CTAs' atomics are read through L2.
struct SweepTask {
  int q;            // matrix (table index)
  short kind, sub;  // 0 diagonal / 1 off-diagonal tile; sub-task index
  int M, K;         // tile (M, K)
};
constexpr int kDiagSubs = 8;  // sub-tasks of a diagonal task: 64 output entries each
constexpr int kUpdSubs = 8;   // sub-tasks of an off-diagonal task: 64 rows (forward) / columns (backward)

// L2 prefetch of rows [r0, r1) of columns [c0, c1) of a column-major tile (one 128-byte line per
// instruction), spread over the CTA
__device__ __forceinline__ void prefetch_block(const float* T, int NB, int r0, int r1, int c0, int c1) {
  if (r1 <= r0 || c1 <= c0) return;
  const int nl = (r1 - r0 + 31) >> 5;
  for (int idx = threadIdx.x; idx < (c1 - c0) * nl; idx += blockDim.x) {
    const int c = c0 + idx / nl, l = idx % nl;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(T + r0 + 32 * l + (long long)c * NB));
  }
}

// 16-byte load of rows r..r+3 of column c of a tile; rows at or past `lim` read as zero (the tile slot
// holds NB rows, so a load that starts before `lim` stays inside it)
__device__ __forceinline__ float4 ld4_rows(const float* T, int r, long long c, int NB, int lim) {
  float4 v = r < lim ? __ldg((const float4*)(T + r + c * NB)) : make_float4(0, 0, 0, 0);
  if (r + 1 >= lim) v.y = 0.f;
  if (r + 2 >= lim) v.z = 0.f;
  if (r + 3 >= lim) v.w = 0.f;
  return v;
}

// vectors of tile row r0 (n entries, nrhs columns) into shared memory, zero past n
// (one pass of independent loads per thread: scalar, since column j starts at j * N, which need not be
// 16-byte aligned)
__device__ __forceinline__ void load_vec(const float* V, int N, long long r0, int n, int nrhs, float* vs) {
  float v[8];
  for (int base = 0; base < 512 * nrhs; base += 8 * 256) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = base + u * 256 + threadIdx.x, r = idx & 511, j = idx >> 9;
      v[u] = (idx < 512 * nrhs && r < n) ? __ldcg(V + (long long)j * N + r0 + r) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = base + u * 256 + threadIdx.x;
      if (idx < 512 * nrhs) vs[idx] = v[u];
    }
  }
  __syncthreads();
}

// warp-reduces acc[j] and, in lane 0, hands the sums to `put(j, sum)`
template <int NR, typename F>
__device__ __forceinline__ void warp_sums(float (&acc)[NR], int nrhs, F put) {
#pragma unroll
  for (int j = 0; j < NR; ++j) {
    float a = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0 && j < nrhs) put(j, a);
  }
}

// forward diagonal, sub-task s: y_c = sum_{r <= c} L^{-1}(c, r) x_r for c in [64 s, 64 s + 64), with
// L^{-1}(c, r) = out(r, c); a warp owns 8 columns, lanes four rows at a time
template <int NR>
__device__ void sweep_fwd_diag(const float* out, const float* X, float* Y, int N, int NB, int n, long long r0, int nrhs,
                               int sub, float* xs) {
  load_vec(X, N, r0, n, nrhs, xs);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int cc = 0; cc < 8; cc += 2) {
    const int c0 = 64 * sub + 8 * warp + cc;
    if (c0 >= n) break;
    float acc0[NR], acc1[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) acc0[j] = acc1[j] = 0.f;
    float4 v0[4], v1[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {  // out(r, c) for r <= c only
      const int r = 4 * lane + 128 * t;
      v0[t] = ld4_rows(out, r, c0, NB, min(n, c0 + 1));
      v1[t] = c0 + 1 < n ? ld4_rows(out, r, c0 + 1, NB, min(n, c0 + 2)) : make_float4(0, 0, 0, 0);
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int r = 4 * lane + 128 * t;
#pragma unroll
      for (int j = 0; j < NR; ++j)
        if (j < nrhs) {
          const float* x = xs + j * 512 + r;
          acc0[j] = fmaf(v0[t].x, x[0], fmaf(v0[t].y, x[1], fmaf(v0[t].z, x[2], fmaf(v0[t].w, x[3], acc0[j]))));
          acc1[j] = fmaf(v1[t].x, x[0], fmaf(v1[t].y, x[1], fmaf(v1[t].z, x[2], fmaf(v1[t].w, x[3], acc1[j]))));
        }
    }
    warp_sums<NR>(acc0, nrhs, [&](int j, float a) { Y[(long long)j * N + r0 + c0] = a; });
    if (c0 + 1 < n) warp_sums<NR>(acc1, nrhs, [&](int j, float a) { Y[(long long)j * N + r0 + c0 + 1] = a; });
  }
}

// forward update, sub-task s: x_M -= L_MK y_K on rows [64 s, 64 s + 64); a thread owns four
// consecutive rows and one sixteenth of the columns; the partial sums meet in shared memory
template <int NR>
__device__ void sweep_fwd_upd(const float* L, const float* Y, float* X, int N, int NB, int mrows, int kn, long long ry,
                              long long rx, int nrhs, int sub, float* ys) {
  load_vec(Y, N, ry, kn, nrhs, ys);
  const int rq = threadIdx.x & 15, g = threadIdx.x >> 4;
  const int i0 = 64 * sub + 4 * rq;
  float acc[4][NR];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[i][j] = 0.f;
  if (i0 < mrows) {
    const int span = (kn + 15) / 16, cb = g * span, ce = min(kn, cb + span);
    for (int c = cb; c < ce; c += 8) {
      float4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = c + u < ce ? ld4_rows(L, i0, c + u, NB, mrows) : make_float4(0, 0, 0, 0);
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int j = 0; j < NR; ++j)
          if (j < nrhs) {
            const float y = c + u < ce ? ys[j * 512 + c + u] : 0.f;
            acc[0][j] = fmaf(v[u].x, y, acc[0][j]);
            acc[1][j] = fmaf(v[u].y, y, acc[1][j]);
            acc[2][j] = fmaf(v[u].z, y, acc[2][j]);
            acc[3][j] = fmaf(v[u].w, y, acc[3][j]);
          }
    }
  }
  float* part = ys + NR * 512;  // [16 groups][NR][64 rows]
#pragma unroll
  for (int j = 0; j < NR; ++j)
#pragma unroll
    for (int i = 0; i < 4; ++i) part[(g * NR + j) * 64 + 4 * rq + i] = acc[i][j];
  __syncthreads();
  for (int idx = threadIdx.x; idx < 64 * nrhs; idx += blockDim.x) {
    const int r = idx & 63, j = idx >> 6;
    if (64 * sub + r >= mrows) continue;
    float sum = 0.f;
#pragma unroll
    for (int q = 0; q < 16; ++q) sum += part[(q * NR + j) * 64 + r];
    atomicAdd(X + (long long)j * N + rx + 64 * sub + r, -sum);
  }
}

// backward diagonal, sub-task s: z_i = sum_{c >= i} out(i, c) y_c for i in [64 s, 64 s + 64); a
// thread owns four consecutive rows and one sixteenth of the columns
template <int NR>
__device__ void sweep_bwd_diag(const float* out, const float* Y, float* X, int N, int NB, int n, long long r0, int nrhs,
                               int sub, float* ys) {
  load_vec(Y, N, r0, n, nrhs, ys);
  const int rq = threadIdx.x & 15, g = threadIdx.x >> 4;
  const int i0 = 64 * sub + 4 * rq;
  float acc[4][NR];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[i][j] = 0.f;
  if (i0 < n) {
    for (int c = i0 + g; c < n; c += 16 * 4) {  // columns c, c+16, c+32, c+48 of this group, from the diagonal on
      float4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int cu = c + 16 * u;
        v[u] = cu < n ? ld4_rows(out, i0, cu, NB, min(n, cu + 1)) : make_float4(0, 0, 0, 0);  // rows <= cu only
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int j = 0; j < NR; ++j)
          if (j < nrhs) {
            const float y = ys[j * 512 + min(c + 16 * u, 511)];
            acc[0][j] = fmaf(v[u].x, y, acc[0][j]);
            acc[1][j] = fmaf(v[u].y, y, acc[1][j]);
            acc[2][j] = fmaf(v[u].z, y, acc[2][j]);
            acc[3][j] = fmaf(v[u].w, y, acc[3][j]);
          }
    }
  }
  float* part = ys + NR * 512;  // [16 groups][NR][64 rows]
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NR; ++j)
#pragma unroll
    for (int i = 0; i < 4; ++i) part[(g * NR + j) * 64 + 4 * rq + i] = acc[i][j];
  __syncthreads();
  for (int idx = threadIdx.x; idx < 64 * nrhs; idx += blockDim.x) {
    const int r = idx & 63, j = idx >> 6;
    if (64 * sub + r >= n) continue;
    float sum = 0.f;
#pragma unroll
    for (int q = 0; q < 16; ++q) sum += part[(q * NR + j) * 64 + r];
    X[(long long)j * N + r0 + 64 * sub + r] = sum;
  }
}

// backward update, sub-task s: y_K -= L_MK^T z_M on columns [64 s, 64 s + 64): a warp owns 8
// columns, lanes four rows at a time
template <int NR>
__device__ void sweep_bwd_upd(const float* L, const float* X, float* Y, int N, int NB, int mrows, int kn, long long rz,
                              long long ry, int nrhs, int sub, float* zs) {
  load_vec(X, N, rz, mrows, nrhs, zs);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int cc = 0; cc < 8; cc += 2) {
    const int c0 = 64 * sub + 8 * warp + cc;
    if (c0 >= kn) break;
    float acc0[NR], acc1[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) acc0[j] = acc1[j] = 0.f;
    float4 v0[4], v1[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int r = 4 * lane + 128 * t;
      v0[t] = ld4_rows(L, r, c0, NB, mrows);
      v1[t] = c0 + 1 < kn ? ld4_rows(L, r, c0 + 1, NB, mrows) : make_float4(0, 0, 0, 0);
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int r = 4 * lane + 128 * t;
#pragma unroll
      for (int j = 0; j < NR; ++j)
        if (j < nrhs) {
          const float* z = zs + j * 512 + r;
          acc0[j] = fmaf(v0[t].x, z[0], fmaf(v0[t].y, z[1], fmaf(v0[t].z, z[2], fmaf(v0[t].w, z[3], acc0[j]))));
          acc1[j] = fmaf(v1[t].x, z[0], fmaf(v1[t].y, z[1], fmaf(v1[t].z, z[2], fmaf(v1[t].w, z[3], acc1[j]))));
        }
    }
    warp_sums<NR>(acc0, nrhs, [&](int j, float a) { atomicAdd(Y + (long long)j * N + ry + c0, -a); });
    if (c0 + 1 < kn) warp_sums<NR>(acc1, nrhs, [&](int j, float a) { atomicAdd(Y + (long long)j * N + ry + c0 + 1, -a); });
  }
}

template <int NR>
__global__ void __launch_bounds__(256) sweep_kernel(int dir, const RMat* mats, const SweepTask* tasks, int ntasks,
                                                    const int* active, const float* W, const float* Inv, float* Xf,
                                                    float* Yf, int NB, int nrhs, int* cnt, int* flag, DagState* st,
                                                    uint64_t timeout_ns) {
  extern __shared__ __align__(16) float vs_f[];  // [NR][512] vector, then [16][NR][64] partial sums
  __shared__ int s_t, s_ok;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      long long t = -1;
      if (!ld_volatile(&st->abort)) t = (long long)atomicAdd(&st->head, 1ULL);
      s_t = (t >= 0 && t < ntasks) ? (int)t : -1;
    }
    __syncthreads();
    if (s_t < 0) break;
    const SweepTask tk = tasks[s_t];
    // tasks of a matrix that is not in this sweep: skipped (no task of another matrix waits on them)
    if (active && !active[tk.q]) continue;
    const RMat& mt = mats[tk.q];
    const int N = mt.N, NT = mt.NT;
    int* c = cnt + mt.inv0;
    int* f = flag + mt.inv0;
    {  // the task's block of the factor does not depend on the wait: start fetching it into L2
      const int kn = tdim(tk.K, N, NB, NT), s64 = 64 * tk.sub;
      if (tk.kind == 0) {
        const float* out = Inv + (mt.inv0 + tk.K) * (long long)NB * NB;
        if (dir == 0) prefetch_block(out, NB, 0, min(kn, s64 + 64), s64, min(kn, s64 + 64));
        else prefetch_block(out, NB, s64, min(kn, s64 + 64), s64, kn);
      } else {
        const float* L = W + (mt.slot0 + slot_of(tk.M, tk.K, NT)) * (long long)NB * NB;
        const int mrows = tdim(tk.M, N, NB, NT);
        if (dir == 0) prefetch_block(L, NB, s64, min(mrows, s64 + 64), 0, kn);
        else prefetch_block(L, NB, 0, mrows, s64, min(kn, s64 + 64));
      }
    }
    if (threadIdx.x == 0) {
      bool ok;
      if (dir == 0)
        ok = tk.kind == 0 ? wait_geq(c + tk.K, kUpdSubs * tk.K, st, timeout_ns)
                          : wait_geq(f + tk.K, kDiagSubs, st, timeout_ns);
      else
        ok = tk.kind == 0 ? wait_geq(c + tk.K, kUpdSubs * (NT - 1 - tk.K), st, timeout_ns)
                          : wait_geq(f + tk.M, kDiagSubs, st, timeout_ns);
      s_ok = ok;
    }
    __syncthreads();
    if (!s_ok) break;
    float* X = Xf + mt.vec0;
    float* Y = Yf + mt.vec0;
    const int kn = tdim(tk.K, N, NB, NT);
    if (tk.kind == 0) {
      const float* out = Inv + (mt.inv0 + tk.K) * (long long)NB * NB;
      if (dir == 0) sweep_fwd_diag<NR>(out, X, Y, N, NB, kn, (long long)tk.K * NB, nrhs, tk.sub, vs_f);
      else sweep_bwd_diag<NR>(out, Y, X, N, NB, kn, (long long)tk.K * NB, nrhs, tk.sub, vs_f);
    } else {
      const float* L = W + (mt.slot0 + slot_of(tk.M, tk.K, NT)) * (long long)NB * NB;
      const int mrows = tdim(tk.M, N, NB, NT);
      if (dir == 0)
        sweep_fwd_upd<NR>(L, Y, X, N, NB, mrows, kn, (long long)tk.K * NB, (long long)tk.M * NB, nrhs, tk.sub, vs_f);
      else
        sweep_bwd_upd<NR>(L, X, Y, N, NB, mrows, kn, (long long)tk.M * NB, (long long)tk.K * NB, nrhs, tk.sub, vs_f);
    }
    __threadfence();  // this thread's results are visible before the completion is
    __syncthreads();
    if (threadIdx.x == 0) {
      if (tk.kind == 0) signal_done(f + tk.K);
      else signal_done(c + (dir == 0 ? tk.M : tk.K));
    }
  }
}

template <int NR>
int set_sweep_attrs(int big) {
  return cudaFuncSetAttribute(sweep_kernel<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) == cudaSuccess
             ? GBX_OK
             : GBX_ERR_CUDA;
}
// shared memory of a sweep CTA: the vector, then the partial sums
inline size_t sweep_smem(int NR) { return (size_t)NR * 512 * sizeof(float) + (size_t)16 * NR * 64 * sizeof(float); }
void launch_sweep(int dir, int grid, cudaStream_t s, const RMat* mats, const SweepTask* tasks, int ntasks,
                  const int* active, const float* W, const float* Inv, float* Xf, float* Yf, int NB, int nrhs,
                  int* cnt, int* flag, DagState* st, uint64_t timeout_ns) {
  const int NRb = nrhs <= 1 ? 1 : nrhs <= 2 ? 2 : nrhs <= 4 ? 4 : nrhs <= 8 ? 8 : 16;
  const size_t vs = sweep_smem(NRb);
#define GBX_SWEEP(NR)                                                                                          \
  sweep_kernel<NR><<<grid, 256, vs, s>>>(dir, mats, tasks, ntasks, active, W, Inv, Xf, Yf, NB, nrhs, cnt, flag, st, \
                                         timeout_ns)
  if (nrhs <= 1) GBX_SWEEP(1);
  else if (nrhs <= 2) GBX_SWEEP(2);
  else if (nrhs <= 4) GBX_SWEEP(4);
  else if (nrhs <= 8) GBX_SWEEP(8);
  else GBX_SWEEP(16);
#undef GBX_SWEEP
}

__global__ void scale_kernel(double* Y, long long n, double beta) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    Y[i] = beta == 0.0 ? 0.0 : Y[i] * beta;
}

// per right-hand side j: out[j*3 + q] = reduction q of the columns (0: dot(a,b), 1: max|a|, 2: max|b|)
__device__ void colstats_body(const double* a, const double* b, int N, double* out) {
  const int j = blockIdx.x;
  __shared__ double s_dot[256], s_ma[256], s_mb[256];
  double dot = 0, ma = 0, mb = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double x = a[(long long)j * N + i], y = b ? b[(long long)j * N + i] : 0.0;
    dot = fma(x, y, dot);
    ma = fmax(ma, fabs(x));
    mb = fmax(mb, fabs(y));
  }
  s_dot[threadIdx.x] = dot;
  s_ma[threadIdx.x] = ma;
  s_mb[threadIdx.x] = mb;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s_dot[threadIdx.x] += s_dot[threadIdx.x + o];
      s_ma[threadIdx.x] = fmax(s_ma[threadIdx.x], s_ma[threadIdx.x + o]);
      s_mb[threadIdx.x] = fmax(s_mb[threadIdx.x], s_mb[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[j * 3 + 0] = s_dot[0];
    out[j * 3 + 1] = s_ma[0];
    out[j * 3 + 2] = s_mb[0];
  }
}
// out: [matrix id][kMaxRhs][3]; `ncols` columns per matrix (nrhs, or 1 for the row-sum vector,
// whose vectors are at vec0 / nrhs)
__global__ void colstats_batched(const RMat* mats, const int* list, const double* a, const double* b, int nrhs,
                                 int ncols, double* out) {
  if ((int)blockIdx.z >= list[0]) return;
  const int id = list[1 + blockIdx.z];
  const RMat& mt = mats[id];
  const long long off = ncols == nrhs ? mt.vec0 : mt.vec0 / nrhs;
  colstats_body(a + off, b ? b + off : nullptr, mt.N, out + (long long)id * kMaxRhs * 3);
}

// y_j := y_j + coef_j * x_j  (coef from device memory)
__device__ void axpy_cols_body(double* y, const double* x, const double* coef, double sign, int N, int nrhs,
                               int xscale_mode) {
  const long long n = (long long)N * nrhs;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(i / N);
    if (xscale_mode == 0) y[i] += sign * coef[j] * x[i];  // y += s*c*x
    else if (xscale_mode == 1) y[i] = x[i] + coef[j] * y[i];  // y = x + c*y
    else y[i] = 0.0;                                          // y = 0
  }
}
// coef: [matrix id][kMaxRhs]
__global__ void axpy_cols_batched(const RMat* mats, const int* list, double* y, const double* x, const double* coef,
                                  double sign, int nrhs, int xscale_mode) {
  if ((int)blockIdx.z >= list[0]) return;
  const int id = list[1 + blockIdx.z];
  const RMat& mt = mats[id];
  axpy_cols_body(y + mt.vec0, x + mt.vec0, coef + (long long)id * kMaxRhs, sign, mt.N, nrhs, xscale_mode);
}
// y := x (the matrix's vectors)
__global__ void copy_vec_batched(const RMat* mats, const int* list, double* y, const double* x, int nrhs) {
  GBX_MAT_OF_BLOCK();
  const long long n = (long long)mt.N * nrhs;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[mt.vec0 + i] = x[mt.vec0 + i];
}

}  // namespace refine
}  // namespace gbx

using namespace gbx;
using namespace gbx::refine;

namespace {
int launch_ok() { return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA; }
int set_attrs() {
  static int done = 0;  // benign race: every caller sets the same values
  if (done) return GBX_OK;
  const int big = 96 * 1024;
  if (cudaFuncSetAttribute(fwd_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(fwd_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(bwd_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(bwd_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(symm_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(symm_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(diag_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(diag_inverse_batched, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      set_df_attrs<1>(big) || set_df_attrs<2>(big) || set_df_attrs<4>(big) || set_df_attrs<8>(big) ||
      set_df_attrs<16>(big) || set_sweep_attrs<1>(big) || set_sweep_attrs<2>(big) || set_sweep_attrs<4>(big) ||
      set_sweep_attrs<8>(big) || set_sweep_attrs<16>(big))
    return GBX_ERR_CUDA;
  done = 1;
  return GBX_OK;
}
}  // namespace

extern "C" int gbx_spotri_diag(int N, int NB, const float* W, float* Inv, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N <= 0 || NB <= 0 || NB > 1024 || !W || !Inv) return GBX_ERR_ARG;
  if (int e = set_attrs()) return e;
  const int NT = (N + NB - 1) / NB;
  const size_t smem = op_trsm_smem_elems<float>() * sizeof(float);
  dim3 grid(NT, (NB + kBlk - 1) / kBlk);
  diag_inverse_kernel<<<grid, kThreads, smem, (cudaStream_t)stream>>>(W, Inv, N, NB, NT);
  return launch_ok();
}

extern "C" int gbx_sprecond(int N, int NB, const float* W, const float* Inv, int nrhs, const double* R, double* Z,
                            float* tmp, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N <= 0 || NB <= 0 || NB > 1024 || nrhs <= 0 || nrhs > kMaxRhs || !W || !Inv || !R || !Z || !tmp)
    return GBX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (int e = set_attrs()) return e;
  const int NT = (N + NB - 1) / NB;
  const long long n = (long long)N * nrhs;
  const size_t vs = (size_t)nrhs * NB * sizeof(float);
  // two float buffers: X (rhs being reduced) and Y (solved blocks), so that no kernel reads a
  // block another CTA of the same launch writes
  float* X = tmp;
  float* Y = tmp + n;
  d2s_kernel<<<512, 256, 0, s>>>(R, X, n);
  for (int K = 0; K < NT; ++K) {  // L y = x
    const int kn = tdim(K, N, NB, NT);
    fwd_diag_kernel<<<(kn + 7) / 8, 256, vs, s>>>(Inv, X, Y, N, NB, NT, K, nrhs);
    const long long below = (long long)N - (long long)(K + 1) * NB;
    if (below > 0) fwd_update_kernel<<<(unsigned)((below + 127) / 128), 128, vs, s>>>(W, Y, X, N, NB, NT, K, nrhs);
  }
  for (int K = NT - 1; K >= 0; --K) {  // L^T z = y
    const int kn = tdim(K, N, NB, NT);
    bwd_diag_kernel<<<(kn + 31) / 32, 256, vs + (size_t)8 * nrhs * 32 * sizeof(float), s>>>(Inv, Y, X, N, NB, NT, K,
                                                                                           nrhs);
    if (K > 0) {
      const long long above = (long long)K * NB;
      bwd_update_kernel<<<(unsigned)std::min<long long>((above + 7) / 8, 4096), 256, vs, s>>>(W, X, Y, N, NB, NT, K,
                                                                                            nrhs);
    }
  }
  s2d_kernel<<<512, 256, 0, s>>>(X, Z, n);
  return launch_ok();
}

extern "C" int gbx_dsymm_tiled(int N, int NB, const double* A, int nrhs, double alpha, const double* X, double beta,
                               double* Y, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N <= 0 || NB <= 0 || nrhs <= 0 || nrhs > kMaxRhs || !A || !X || !Y) return GBX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (int e = set_attrs()) return e;
  const int NT = (N + NB - 1) / NB;
  const int nslots = NT * (NT + 1) / 2;
  const size_t vs = (size_t)nrhs * 512 * sizeof(double);
  if (beta != 1.0) scale_kernel<<<256, 256, 0, s>>>(Y, (long long)N * nrhs, beta);
  symm_rows_kernel<<<dim3(nslots, (NB + 127) / 128), 128, vs, s>>>(A, X, Y, N, NB, NT, nrhs, alpha);
  symm_cols_kernel<<<dim3(nslots, std::max(1, NB / 64)), 256, vs, s>>>(A, X, Y, N, NB, NT, nrhs, alpha);
  return launch_ok();
}

namespace {
// ---- the batched refinement: plan once, then a device-driven run ----------------------------------
// Per-matrix record kept on the device during a run; the host reads it once at the end.
struct DevRec {
  double shift, backward_error, anorm;
  float cond;
  int iterations, retries, fp64_tiles, piv;  // piv: first bad pivot of the last failed attempt, else 0
  int live;                                 // 1 when the matrix has a factor
  int pad;
};
// Run state of one workspace.
struct RunState {
  unsigned long long sig;  // signature of the plan in this workspace (written by the plan)
  int status;              // 0, GBX_ERR_ARG (exec does not match the plan) or GBX_ERR_TIMEOUT (factorisation)
  int attempt;             // factorisations launched
  int it;                  // CG iterations run (by any matrix)
  int pad;
  double shift;            // diagonal shift of the next factorisation attempt
};

// workspace of the batched refinement (the factor's workspace first)
struct BLayout {
  size_t fwork_bytes, inv, R, Z, P, Q, tmp, rowsum, stats, coef, mats, ahi, alo, sweep, tasks, rs, rec, fail, lists,
      flags, rz, norms, total;
  long long nf, nb;  // forward / backward sweep tasks
  long long nvec, sumN, sumNT;  // vector entries (sum of n * nrhs), sum of orders, sum of tile counts
  int maxNT, maxslots, maxN;
};
BLayout blayout(int batch, const int* n, int NB, int nrhs) {
  BLayout b;
  b.fwork_bytes = 0;
  gbx_potrf_mixed_batched_bufferSize(batch, n, NB, &b.fwork_bytes);
  long long sumNT = 0, sumN = 0, slots = 0;
  b.maxNT = b.maxslots = b.maxN = 0;
  b.nf = b.nb = 0;
  for (int k = 0; k < batch; ++k) {
    const long long nt = (n[k] + NB - 1) / NB;
    sumNT += nt;
    sumN += n[k];
    slots += nt * (nt + 1) / 2;
    b.maxNT = std::max(b.maxNT, (int)nt);
    b.maxslots = std::max(b.maxslots, (int)(nt * (nt + 1) / 2));
    b.maxN = std::max(b.maxN, n[k]);
    // forward: NT diagonal tasks + NT(NT-1)/2 updates; backward the same
    b.nf += nt * kDiagSubs + nt * (nt - 1) / 2 * kUpdSubs;
  }
  b.nb = b.nf;
  b.sumN = sumN;
  b.sumNT = sumNT;
  b.nvec = sumN * nrhs;
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t vec = (size_t)sumN * nrhs;
  size_t o = up(b.fwork_bytes);
  b.inv = o;
  o += up((size_t)sumNT * NB * NB * sizeof(float));
  b.R = o;
  o += up(vec * 8);
  b.Z = o;
  o += up(vec * 8);
  b.P = o;
  o += up(vec * 8);
  b.Q = o;
  o += up(vec * 8);
  b.tmp = o;
  o += up(2 * vec * 4);
  b.rowsum = o;
  o += up((size_t)sumN * 8);
  b.stats = o;  // two [batch][kMaxRhs][3] blocks
  o += up((size_t)2 * batch * kMaxRhs * 3 * 8);
  b.coef = o;  // alpha, beta: [2][batch][kMaxRhs]
  o += up((size_t)2 * batch * kMaxRhs * 8);
  b.mats = o;
  o += up((size_t)batch * sizeof(RMat));
  b.ahi = o;  // A split into FP32 pairs for the double-float residuals
  o += up((size_t)slots * NB * NB * sizeof(float));
  b.alo = o;
  o += up((size_t)slots * NB * NB * sizeof(float));
  b.sweep = o;  // two run states, then forward / backward row counters and flags
  o += up(2 * sizeof(DagState) + (size_t)4 * sumNT * sizeof(int));
  b.tasks = o;  // forward then backward task lists (sub-tasks of every tile of every matrix)
  o += up((size_t)(b.nf + b.nb) * sizeof(SweepTask));
  b.rs = o;
  o += up(sizeof(RunState));
  b.rec = o;
  o += up((size_t)batch * sizeof(DevRec));
  b.fail = o;  // per matrix: selected for the next factorisation attempt
  o += up((size_t)batch * sizeof(int));
  b.lists = o;  // five lists {count, entries}: all (largest first), live, active, true-residual, refactor
  o += up((size_t)5 * (batch + 1) * sizeof(int));
  b.flags = o;  // per matrix: live, active (the sweeps' selection)
  o += up((size_t)2 * batch * sizeof(int));
  b.rz = o;
  o += up((size_t)batch * kMaxRhs * 8);
  b.norms = o;  // anorm [batch], bnorm [batch][kMaxRhs], backward error [batch]
  o += up((size_t)batch * (2 + kMaxRhs) * 8);
  b.total = o + 4096;
  return b;
}

unsigned long long plan_signature(int batch, const int* n, int NB, int nrhs, int prec) {
  unsigned long long h = 1469598103934665603ull;  // FNV-1a over the plan's arguments
  auto mix = [&](unsigned long long v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (v >> (8 * i)) & 0xff;
      h *= 1099511628211ull;
    }
  };
  mix((unsigned long long)batch);
  mix((unsigned long long)NB);
  mix((unsigned long long)nrhs);
  mix((unsigned long long)prec);
  for (int k = 0; k < batch; ++k) mix((unsigned long long)n[k]);
  return h;
}

// ---- device side of the run ----------------------------------------------------------------------
struct RunPtrs {
  RunState* rs;
  DevRec* rec;
  int* fail;
  int *l_all, *l_live, *l_act, *l_true, *l_fail;
  int *live_flag, *act_flag;
  double *rz, *anorm, *bnorm, *be;
  double *stats, *stats_x, *coef, *coef_b;
  int batch, nrhs, maxiter, prec;
  double tol;
  unsigned long long sig;
};
__device__ __forceinline__ double st_at(const double* h, int k, int j, int q) { return h[((size_t)k * kMaxRhs + j) * 3 + q]; }

// normwise backward error of matrix k from the residual stats (max|r_j|) and the solution stats
__device__ double backward_of(const RunPtrs& p, int k) {
  double b = 0.0;
  for (int j = 0; j < p.nrhs; ++j) {
    const double den = p.anorm[k] * st_at(p.stats_x, k, j, 1) + p.bnorm[(size_t)k * kMaxRhs + j];
    b = fmax(b, den > 0 ? st_at(p.stats, k, j, 1) / den : 0.0);
  }
  return b;
}

// Order-preserving compaction by one CTA of kRunThreads threads: to = {count, the entries k of from
// (a list {count, entries}) with keep(k)}, in from's order. `to` may not alias `from`.
constexpr int kRunThreads = 256;
template <typename Keep>
__device__ void block_compact(const int* from, int* to, Keep keep) {
  __shared__ int s_warp[kRunThreads / 32];
  __shared__ int s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = from[0];
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  for (int c0 = 0; c0 < n; c0 += kRunThreads) {
    const int q = c0 + threadIdx.x;
    const int k = q < n ? from[1 + q] : -1;
    const bool f = q < n && keep(k);
    const unsigned m = __ballot_sync(0xffffffffu, f);
    if (lane == 0) s_warp[warp] = __popc(m);
    __syncthreads();
    int before = s_base;
    for (int w = 0; w < warp; ++w) before += s_warp[w];
    if (f) to[1 + before + __popc(m & ((1u << lane) - 1u))] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < kRunThreads / 32; ++w) t += s_warp[w];
      s_base += t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) to[0] = s_base;
  __syncthreads();
}

// start of a run: checks the plan signature; selects every matrix for the first factorisation
__global__ void run_init_kernel(RunPtrs p) {
  const bool ok = p.rs->sig == p.sig;
  __syncthreads();  // every thread has read the signature before thread 0 may change the state
  if (threadIdx.x == 0) {
    p.rs->status = ok ? 0 : GBX_ERR_ARG;
    p.rs->attempt = 0;
    p.rs->it = 0;
    p.rs->shift = 0.0;
    if (!ok) p.l_all[0] = 0;  // nothing runs; the result reports GBX_ERR_ARG
    p.l_live[0] = p.l_act[0] = p.l_true[0] = p.l_fail[0] = 0;
  }
  for (int k = threadIdx.x; k < p.batch; k += blockDim.x) {
    p.rec[k] = DevRec{0.0, INFINITY, 0.0, 0.f, 0, 0, 0, 0, 0, 0};
    p.fail[k] = ok ? 1 : 0;
    p.live_flag[k] = p.act_flag[k] = 0;
  }
}

// after a factorisation attempt: records the selected matrices' outcome, selects the failed ones for
// the next attempt (diagonal shift: about the operands' unit roundoff, then 4x per attempt) and sets
// the retry loop's condition; rebuilds the live list (matrices with a factor), largest first
__global__ void factor_check_kernel(RunPtrs p, const DagState* fst, const int* finfo, const float* fcond,
                                    const int* fnf, cudaGraphConditionalHandle retry) {
  __shared__ int s_any, s_status;
  RunState* rs = p.rs;
  if (threadIdx.x == 0) {
    s_any = 0;
    if (rs->status == 0 && fst->status < 0) rs->status = fst->status;  // a timed-out wait
    s_status = rs->status;
  }
  __syncthreads();
  const double shift = rs->shift;
  for (int k = threadIdx.x; k < p.batch; k += blockDim.x) {
    if (!p.fail[k]) continue;
    DevRec& r = p.rec[k];
    r.cond = fcond[k];
    r.fp64_tiles = fnf[k];
    r.shift = shift;
    if (finfo[k] != 0) {
      r.piv = finfo[k];
      ++r.retries;
      atomicAdd(&s_any, 1);
    } else {
      r.piv = 0;
      p.fail[k] = 0;
    }
  }
  __syncthreads();
  const bool ok = s_status == 0;
  for (int k = threadIdx.x; k < p.batch; k += blockDim.x) {
    const int live = ok && !p.fail[k];
    p.live_flag[k] = live;
    p.rec[k].live = live;
  }
  block_compact(p.l_all, p.l_live, [&](int k) { return ok && !p.fail[k]; });
  block_compact(p.l_all, p.l_fail, [&](int k) { return ok && p.fail[k] != 0; });
  if (threadIdx.x == 0) {
    ++rs->attempt;
    rs->shift = shift == 0.0 ? (p.prec == 1 ? 1.0 / 2048 : p.prec == 2 ? 1.0 / 32 : 1.0 / 256) : shift * 4;
    cudaGraphSetConditional(retry, (ok && s_any > 0 && rs->attempt < 8) ? 1u : 0u);
  }
}

// W = fl32(A) for the matrices of the refactorisation list, the diagonal scaled by (1 + shift)
__global__ void convert_shift_batched(const RMat* mats, const int* list, const double* A, float* W,
                                      const RunState* rs, int NB) {
  GBX_MAT_OF_BLOCK();
  int m, n;
  if (!slot_tile(blockIdx.x, mt.NT, m, n)) return;
  const long long base = (mt.slot0 + blockIdx.x) * (long long)NB * NB;
  const float f = (float)(1.0 + rs->shift);
  for (long long e = threadIdx.x; e < (long long)NB * NB; e += blockDim.x) {
    float v = (float)A[base + e];
    if (m == n && e % NB == e / NB) v *= f;
    W[base + e] = v;
  }
}

// ||A||_inf and ||b_j||_inf of the live matrices (from the row sums and the right-hand sides' stats)
__global__ void norms_kernel(RunPtrs p) {
  for (int q = threadIdx.x; q < p.l_live[0]; q += blockDim.x) {
    const int k = p.l_live[1 + q];
    p.anorm[k] = st_at(p.stats, k, 0, 1);
    for (int j = 0; j < p.nrhs; ++j) p.bnorm[(size_t)k * kMaxRhs + j] = st_at(p.stats_x, k, j, 1);
  }
}

// the active list: the matrices of `from` whose backward error is above the loop's target (half the
// tolerance, so that the final check on the true residual meets the tolerance itself) and which have
// iterations left; sets the CG loop's condition. Called by every thread of the CTA.
__device__ void select_active(const RunPtrs& p, const int* from, cudaGraphConditionalHandle loop) {
  auto go = [&](int k) { return p.be[k] > 0.5 * p.tol && p.rec[k].iterations < p.maxiter; };
  for (int q = threadIdx.x; q < from[0]; q += blockDim.x) {
    const int k = from[1 + q];
    p.act_flag[k] = go(k);
  }
  block_compact(from, p.l_act, go);
  if (threadIdx.x == 0) cudaGraphSetConditional(loop, p.l_act[0] > 0 ? 1u : 0u);
}

// start of CG: rz = r.z, the backward error of x0, the first active list
__global__ void pcg_start_kernel(RunPtrs p, cudaGraphConditionalHandle loop) {
  for (int q = threadIdx.x; q < p.l_live[0]; q += blockDim.x) {
    const int k = p.l_live[1 + q];
    for (int j = 0; j < p.nrhs; ++j) p.rz[(size_t)k * kMaxRhs + j] = st_at(p.stats, k, j, 0);
    p.be[k] = backward_of(p, k);
  }
  __syncthreads();
  if (threadIdx.x == 0) p.l_true[0] = 0;
  select_active(p, p.l_live, loop);
}

// alpha = (r.z) / (p.q); every 8th iteration the true residual replaces the recursive one
__global__ void pcg_alpha_kernel(RunPtrs p) {
  const int na = p.l_act[0];
  const bool due = (p.rs->it + 1) % 8 == 0;
  for (int q = threadIdx.x; q < na; q += blockDim.x) {
    const int k = p.l_act[1 + q];
    for (int j = 0; j < p.nrhs; ++j) {
      const double pq = st_at(p.stats, k, j, 0);
      p.coef[(size_t)k * kMaxRhs + j] = pq != 0.0 ? p.rz[(size_t)k * kMaxRhs + j] / pq : 0.0;
    }
    if (due) p.l_true[1 + q] = k;
  }
  if (threadIdx.x == 0) p.l_true[0] = due ? na : 0;
}

// after the preconditioner: the backward error, beta = (r.z)_new / (r.z)_old
__global__ void pcg_beta_kernel(RunPtrs p) {
  for (int q = threadIdx.x; q < p.l_act[0]; q += blockDim.x) {
    const int k = p.l_act[1 + q];
    ++p.rec[k].iterations;
    p.be[k] = backward_of(p, k);
    for (int j = 0; j < p.nrhs; ++j) {
      const double rz_new = st_at(p.stats, k, j, 0), old = p.rz[(size_t)k * kMaxRhs + j];
      p.coef_b[(size_t)k * kMaxRhs + j] = old != 0.0 ? rz_new / old : 0.0;
      p.rz[(size_t)k * kMaxRhs + j] = rz_new;
    }
  }
}

// end of a CG iteration: the next active list (a subset of the current one) and the loop condition
__global__ void pcg_select_kernel(RunPtrs p, cudaGraphConditionalHandle loop) {
  // the current list moves to l_true (free at this point of the iteration; the next alpha kernel
  // rebuilds it), and the next active list is compacted from there
  for (int q = threadIdx.x; q <= p.l_act[0]; q += blockDim.x) p.l_true[q] = p.l_act[q];
  if (threadIdx.x == 0) ++p.rs->it;
  __syncthreads();
  select_active(p, p.l_true, loop);
  if (threadIdx.x == 0) p.l_true[0] = 0;
}

// final check on the true residual of every live matrix
__global__ void pcg_final_kernel(RunPtrs p) {
  for (int q = threadIdx.x; q < p.l_live[0]; q += blockDim.x) {
    const int k = p.l_live[1 + q];
    p.rec[k].backward_error = backward_of(p, k);
    p.rec[k].anorm = p.anorm[k];
  }
}

// ---- host side ------------------------------------------------------------------------------------
struct DevStreams {
  cudaStream_t side = nullptr;  // capture stream of the CG loop's bodies and of uncaptured runs
  bool ready = false;
};
std::mutex g_run_mtx;
DevStreams g_run[64];

int run_streams(DevStreams*& d) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GBX_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_run_mtx);
  d = &g_run[dev];
  if (!d->ready) {
    if (cudaStreamCreateWithFlags(&d->side, cudaStreamNonBlocking) != cudaSuccess) return GBX_ERR_CUDA;
    d->ready = true;
  }
  return GBX_OK;
}

// Adds a WHILE conditional node (default condition 0, set by upstream kernels) at the capture
// position of the capturing stream `s`, and starts capturing its body on `body_s`.
int begin_while(cudaStream_t s, cudaStream_t body_s, cudaGraphConditionalHandle h, cudaGraphNode_t& node) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive)
    return GBX_ERR_CUDA;
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};  // the remaining fields zero
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &np) != cudaSuccess) return GBX_ERR_CUDA;
  if (cudaStreamBeginCaptureToGraph(body_s, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                    cudaStreamCaptureModeRelaxed) != cudaSuccess)
    return GBX_ERR_CUDA;
  return GBX_OK;
}
int end_while(cudaStream_t s, cudaStream_t body_s, cudaGraphNode_t node) {
  cudaGraph_t body = nullptr;
  if (cudaStreamEndCapture(body_s, &body) != cudaSuccess) return GBX_ERR_CUDA;
  return cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) == cudaSuccess
             ? GBX_OK
             : GBX_ERR_CUDA;
}
int conditional_handle(cudaStream_t s, cudaGraphConditionalHandle& h) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive)
    return GBX_ERR_CUDA;
  return cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) == cudaSuccess ? GBX_OK
                                                                                               : GBX_ERR_CUDA;
}

struct Run {
  int batch, NB, nrhs, prec;
  const int* n;
  const double *A, *B;
  double* X;
  float* W;
  char* base;
  size_t work_bytes;
  double fp64_cond;
  BLayout L;
  RunPtrs p;
  int sms;
  uint64_t tmo;
};

// z := M^{-1} r for the matrices flagged in `flags` (FP32 sweeps over the planned task lists of every
// matrix; the others' tasks are skipped)
int emit_precond(const Run& r, cudaStream_t s, const int* flags, const double* rv, double* z) {
  const BLayout& L = r.L;
  const long long nvec = L.nvec, sumNT = L.sumNT;
  float* xf = (float*)(r.base + L.tmp);
  float* yf = xf + nvec;
  DagState* sw_st = (DagState*)(r.base + L.sweep);
  int* sw_cnt = (int*)(r.base + L.sweep + 2 * sizeof(DagState));
  const SweepTask* tasks = (const SweepTask*)(r.base + L.tasks);
  const RMat* dmats = (const RMat*)(r.base + L.mats);
  const float* Inv = (const float*)(r.base + L.inv);
  d2s_kernel<<<512, 256, 0, s>>>(rv, xf, nvec);
  // fresh queue heads and counters; status and abort stay, so a wait that ran out is reported
  if (cudaMemsetAsync(&sw_st[0].head, 0, sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(&sw_st[1].head, 0, sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(sw_cnt, 0, (size_t)4 * sumNT * sizeof(int), s) != cudaSuccess)
    return GBX_ERR_CUDA;
  const int gf = (int)std::max(1LL, std::min<long long>(2 * r.sms, L.nf));
  const int gb = (int)std::max(1LL, std::min<long long>(2 * r.sms, L.nb));
  launch_sweep(0, gf, s, dmats, tasks, (int)L.nf, flags, r.W, Inv, xf, yf, r.NB, r.nrhs, sw_cnt, sw_cnt + sumNT,
               sw_st, r.tmo);
  launch_sweep(1, gb, s, dmats, tasks + L.nf, (int)L.nb, flags, r.W, Inv, xf, yf, r.NB, r.nrhs, sw_cnt + 2 * sumNT,
               sw_cnt + 3 * sumNT, sw_st + 1, r.tmo);
  s2d_kernel<<<512, 256, 0, s>>>(xf, z, nvec);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}
// y := y + alpha A x for the matrices of `list` (double-float arithmetic on the split A)
void emit_symm(const Run& r, cudaStream_t s, const int* list, double alpha, const double* x, double* y) {
  const BLayout& L = r.L;
  const long long nvec = L.nvec;
  const size_t vs = (size_t)2 * r.nrhs * 512 * sizeof(float);
  float* xh = (float*)(r.base + L.tmp);  // the preconditioner's FP32 buffers are free between its calls
  float* xl = xh + nvec;
  split_vec_kernel<<<512, 256, 0, s>>>(x, xh, xl, nvec);
  symm_df(dim3(L.maxslots, (r.NB + 127) / 128, r.batch), dim3(L.maxslots, std::max(1, r.NB / 64), r.batch), vs, s,
          (const RMat*)(r.base + L.mats), list, (const float*)(r.base + L.ahi), (const float*)(r.base + L.alo), xh, xl,
          y, r.NB, r.nrhs, alpha);
}
void emit_stats(const Run& r, cudaStream_t s, const int* list, const double* a, const double* b, double* out) {
  colstats_batched<<<dim3(r.nrhs, 1, (unsigned)r.batch), 256, 0, s>>>((const RMat*)(r.base + r.L.mats), list, a, b,
                                                                        r.nrhs, r.nrhs, out);
}
unsigned vec_grid(const Run& r) { return (unsigned)std::min<long long>(64, ((long long)r.L.maxN * r.nrhs + 255) / 256); }
void emit_copy(const Run& r, cudaStream_t s, const int* list, double* y, const double* x) {
  copy_vec_batched<<<dim3(vec_grid(r), 1, (unsigned)r.batch), 256, 0, s>>>((const RMat*)(r.base + r.L.mats), list, y,
                                                                             x, r.nrhs);
}
void emit_axpy(const Run& r, cudaStream_t s, const int* list, double* y, const double* x, const double* coef,
               double sign, int mode) {
  axpy_cols_batched<<<dim3(vec_grid(r), 1, (unsigned)r.batch), 256, 0, s>>>((const RMat*)(r.base + r.L.mats), list, y,
                                                                              x, coef, sign, r.nrhs, mode);
}

// The whole solve, emitted on the capturing stream `s` (its own capture, or the caller's).
int emit_run(Run& r, cudaStream_t s, cudaStream_t body_s) {
  const BLayout& L = r.L;
  RunPtrs& p = r.p;
  const RMat* dmats = (const RMat*)(r.base + L.mats);
  double* R = (double*)(r.base + L.R);
  double* Z = (double*)(r.base + L.Z);
  double* P = (double*)(r.base + L.P);
  double* Q = (double*)(r.base + L.Q);
  double* rowsum = (double*)(r.base + L.rowsum);
  float* Ahi = (float*)(r.base + L.ahi);
  float* Alo = (float*)(r.base + L.alo);
  float* Inv = (float*)(r.base + L.inv);
  void* fwork = r.base;
  // factorisation results in the factor's workspace
  const size_t fw = L.fwork_bytes;
  const gbx::mixed::InfoPtrs fi = gbx::mixed::info_ptrs(r.batch, r.n, r.NB, fwork);

  run_init_kernel<<<1, kRunThreads, 0, s>>>(p);
  // 0. one pass over A: W = fl32(A) for the first factorisation, the split of A for the residual
  //    products, and the row sums of |A|
  if (cudaMemsetAsync(rowsum, 0, (size_t)L.sumN * 8, s) != cudaSuccess) return GBX_ERR_CUDA;
  prep_batched<<<dim3(L.maxslots, 1, (unsigned)r.batch), 256, 0, s>>>(dmats, p.l_all, r.A, r.W, Ahi, Alo, rowsum, r.NB,
                                                                      r.nrhs);
  // 1. low-precision factorisation of every matrix; the ones that break down are factorised again,
  //    alone, with a growing diagonal shift (a WHILE node: at most 8 attempts in all)
  cudaGraphConditionalHandle h_retry, h_cg;
  if (int e = conditional_handle(s, h_retry)) return e;
  if (int e = conditional_handle(s, h_cg)) return e;
  if (int e = gbx::mixed::run_batch(r.batch, r.n, r.NB, r.W, r.prec, r.fp64_cond, p.fail, fwork, fw, s)) return e;
  factor_check_kernel<<<1, kRunThreads, 0, s>>>(p, fi.st, fi.minfo, fi.cond, fi.nfp64, h_retry);
  {
    cudaGraphNode_t node;
    if (int e = begin_while(s, body_s, h_retry, node)) return e;
    convert_shift_batched<<<dim3(L.maxslots, 1, (unsigned)r.batch), 256, 0, body_s>>>(dmats, p.l_fail, r.A, r.W, p.rs,
                                                                                     r.NB);
    if (int e = gbx::mixed::run_batch(r.batch, r.n, r.NB, r.W, r.prec, r.fp64_cond, p.fail, fwork, fw, body_s))
      return e;
    factor_check_kernel<<<1, kRunThreads, 0, body_s>>>(p, fi.st, fi.minfo, fi.cond, fi.nfp64, h_retry);
    if (int e = end_while(s, body_s, node)) return e;
  }
  // 2. the preconditioner's diagonal inverses; ||A||_inf and ||b_j||_inf
  diag_inverse_batched<<<dim3(L.maxNT, (r.NB + kBlk - 1) / kBlk, (unsigned)r.batch), kThreads,
                         op_trsm_smem_elems<float>() * sizeof(float), s>>>(dmats, p.l_live, r.W, Inv, r.NB);
  colstats_batched<<<dim3(1, 1, (unsigned)r.batch), 256, 0, s>>>(dmats, p.l_live, rowsum, nullptr, r.nrhs, 1, p.stats);
  emit_stats(r, s, p.l_live, r.B, nullptr, p.stats_x);
  norms_kernel<<<1, 256, 0, s>>>(p);
  // 3. x0 = M^{-1} b ; r = b - A x0 ; z = M^{-1} r ; p = z
  if (int e = emit_precond(r, s, p.live_flag, r.B, r.X)) return e;
  emit_copy(r, s, p.l_live, R, r.B);
  emit_symm(r, s, p.l_live, -1.0, r.X, R);
  if (int e = emit_precond(r, s, p.live_flag, R, Z)) return e;
  emit_copy(r, s, p.l_live, P, Z);
  emit_stats(r, s, p.l_live, R, Z, p.stats);
  emit_stats(r, s, p.l_live, r.X, nullptr, p.stats_x);
  pcg_start_kernel<<<1, kRunThreads, 0, s>>>(p, h_cg);
  // 4. preconditioned CG in FP64 (a WHILE node), each matrix until its own backward error meets
  //    the loop's target or it runs out of iterations
  {
    cudaGraphNode_t node;
    if (int e = begin_while(s, body_s, h_cg, node)) return e;
    cudaStream_t b = body_s;
    emit_axpy(r, b, p.l_act, Q, Q, p.coef, -1.0, 2);  // q = 0
    emit_symm(r, b, p.l_act, 1.0, P, Q);              // q = A p
    emit_stats(r, b, p.l_act, P, Q, p.stats);
    pcg_alpha_kernel<<<1, kRunThreads, 0, b>>>(p);
    emit_axpy(r, b, p.l_act, r.X, P, p.coef, 1.0, 0);
    emit_axpy(r, b, p.l_act, R, Q, p.coef, -1.0, 0);
    emit_copy(r, b, p.l_true, R, r.B);  // every 8th iteration: the true residual against drift
    emit_symm(r, b, p.l_true, -1.0, r.X, R);
    if (int e = emit_precond(r, b, p.act_flag, R, Z)) return e;
    emit_stats(r, b, p.l_act, R, Z, p.stats);
    emit_stats(r, b, p.l_act, r.X, nullptr, p.stats_x);
    pcg_beta_kernel<<<1, kRunThreads, 0, b>>>(p);
    emit_axpy(r, b, p.l_act, P, Z, p.coef_b, 1.0, 1);  // p = z + beta p
    pcg_select_kernel<<<1, kRunThreads, 0, b>>>(p, h_cg);
    if (int e = end_while(s, body_s, node)) return e;
  }
  // 5. final check on the true residual of every live matrix
  emit_copy(r, s, p.l_live, R, r.B);
  emit_symm(r, s, p.l_live, -1.0, r.X, R);
  emit_stats(r, s, p.l_live, R, nullptr, p.stats);
  emit_stats(r, s, p.l_live, r.X, nullptr, p.stats_x);
  pcg_final_kernel<<<1, 256, 0, s>>>(p);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

int check_args(int batch, const int* n, int NB, int nrhs, int prec) {
  if (batch <= 0 || !n || NB <= 0 || NB % 256 || NB > 512 || nrhs <= 0 || nrhs > kMaxRhs || prec < 0 || prec > 2)
    return GBX_ERR_ARG;
  for (int k = 0; k < batch; ++k)
    if (n[k] <= 0) return GBX_ERR_ARG;
  return GBX_OK;
}

int make_run(Run& r, int batch, const int* n, int NB, int nrhs, int prec, double fp64_cond, const double* A,
             const double* B, double* X, double tol, int maxiter, float* W, void* work, size_t work_bytes) {
  r.batch = batch;
  r.n = n;
  r.NB = NB;
  r.nrhs = nrhs;
  r.prec = prec;
  r.A = A;
  r.B = B;
  r.X = X;
  r.W = W;
  r.base = (char*)work;
  r.work_bytes = work_bytes;
  r.fp64_cond = fp64_cond;
  r.L = blayout(batch, n, NB, nrhs);
  r.tmo = gbx_get_wait_timeout_ns();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&r.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return GBX_ERR_CUDA;
  const BLayout& L = r.L;
  RunPtrs& p = r.p;
  char* base = r.base;
  p.rs = (RunState*)(base + L.rs);
  p.rec = (DevRec*)(base + L.rec);
  p.fail = (int*)(base + L.fail);
  int* lists = (int*)(base + L.lists);
  p.l_all = lists;
  p.l_live = lists + (batch + 1);
  p.l_act = lists + 2 * (batch + 1);
  p.l_true = lists + 3 * (batch + 1);
  p.l_fail = lists + 4 * (batch + 1);
  p.live_flag = (int*)(base + L.flags);
  p.act_flag = p.live_flag + batch;
  p.rz = (double*)(base + L.rz);
  p.anorm = (double*)(base + L.norms);
  p.bnorm = p.anorm + batch;
  p.be = p.bnorm + (size_t)batch * kMaxRhs;
  p.stats = (double*)(base + L.stats);
  p.stats_x = p.stats + (size_t)batch * kMaxRhs * 3;
  p.coef = (double*)(base + L.coef);
  p.coef_b = p.coef + (size_t)batch * kMaxRhs;
  p.batch = batch;
  p.nrhs = nrhs;
  p.maxiter = maxiter;
  p.prec = prec;
  p.tol = tol;
  p.sig = plan_signature(batch, n, NB, nrhs, prec);
  return GBX_OK;
}
}  // namespace

extern "C" int gbx_split_f64(const double* a, float* hi, float* lo, long long n, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (n < 0 || (n > 0 && (!a || !hi || !lo))) return GBX_ERR_ARG;
  if (n == 0) return GBX_OK;
  split_f64_kernel<<<(unsigned)std::min<long long>(4096, (n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, hi, lo, n);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

extern "C" int gbx_dposv_mixed_batched_bufferSize(int batch, const int* n, int NB, int nrhs, size_t* bytes) {
  if (!bytes || check_args(batch, n, NB, nrhs, 0)) return GBX_ERR_ARG;
  *bytes = blayout(batch, n, NB, nrhs).total;
  return GBX_OK;
}

extern "C" int gbx_dposv_mixed_batched_plan(int batch, const int* n, int NB, int nrhs, int prec, int sched, void* work,
                                            size_t work_bytes, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (check_args(batch, n, NB, nrhs, prec) || !work || sched < 0 || sched > 1) return GBX_ERR_ARG;
  const BLayout L = blayout(batch, n, NB, nrhs);
  if (work_bytes < L.total) return GBX_ERR_WORKSPACE;
  if (int e = set_attrs()) return e;
  DevStreams* ds = nullptr;
  if (int e = run_streams(ds)) return e;
  cudaStream_t s = (cudaStream_t)stream;
  char* base = (char*)work;
  // matrix table (batch order), the list of all matrices by decreasing tile count
  std::vector<RMat> mats(batch);
  long long slot = 0, invt = 0, vecn = 0;
  for (int k = 0; k < batch; ++k) {
    const int nt = (n[k] + NB - 1) / NB;
    mats[k] = RMat{slot, invt, vecn, n[k], nt};
    slot += (long long)nt * (nt + 1) / 2;
    invt += nt;
    vecn += (long long)n[k] * nrhs;
  }
  std::vector<int> all(batch + 1);
  all[0] = batch;
  for (int k = 0; k < batch; ++k) all[1 + k] = k;
  std::stable_sort(all.begin() + 1, all.end(), [&](int a, int b) { return mats[a].NT > mats[b].NT; });
  // the sweeps' task lists over every matrix, interleaved step by step (largest first); the run
  // skips the tasks of matrices that are not in a sweep
  std::vector<SweepTask> tf, tb;
  auto push = [](std::vector<SweepTask>& v, int q, int kind, int M, int K) {
    const int subs = kind == 0 ? kDiagSubs : kUpdSubs;
    for (int u = 0; u < subs; ++u) v.push_back(SweepTask{q, (short)kind, (short)u, M, K});
  };
  const int maxNT = L.maxNT;
  for (int K = 0; K < maxNT; ++K) {
    for (int i = 1; i <= batch; ++i)
      if (mats[all[i]].NT > K) push(tf, all[i], 0, K, K);
    for (int i = 1; i <= batch; ++i)  // the next step's own row first: it is on the critical path
      if (K + 1 < mats[all[i]].NT) push(tf, all[i], 1, K + 1, K);
    for (int i = 1; i <= batch; ++i)
      for (int M = K + 2; M < mats[all[i]].NT; ++M) push(tf, all[i], 1, M, K);
  }
  for (int st = 0; st < maxNT; ++st) {  // steps counted from each matrix's last tile row
    for (int i = 1; i <= batch; ++i)
      if (mats[all[i]].NT > st) push(tb, all[i], 0, mats[all[i]].NT - 1 - st, mats[all[i]].NT - 1 - st);
    for (int i = 1; i <= batch; ++i) {
      const int K = mats[all[i]].NT - 1 - st;
      if (K >= 1) push(tb, all[i], 1, K, K - 1);
    }
    for (int i = 1; i <= batch; ++i) {
      const int K = mats[all[i]].NT - 1 - st;
      for (int J = 0; J + 1 < K; ++J) push(tb, all[i], 1, K, J);
    }
  }
  if ((long long)tf.size() != L.nf || (long long)tb.size() != L.nb) return GBX_ERR_ARG;
  tf.insert(tf.end(), tb.begin(), tb.end());
  RunState rs;
  std::memset(&rs, 0, sizeof(rs));
  rs.sig = plan_signature(batch, n, NB, nrhs, prec);
  if (int e = gbx::mixed::plan_batch(batch, n, NB, work, L.fwork_bytes, s, sched)) return e;
  if (cudaMemcpyAsync(base + L.mats, mats.data(), batch * sizeof(RMat), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(base + L.lists, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(base + L.tasks, tf.data(), tf.size() * sizeof(SweepTask), cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(base + L.rs, &rs, sizeof(rs), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemsetAsync(base + L.sweep, 0, 2 * sizeof(DagState), s) != cudaSuccess)
    return GBX_ERR_CUDA;
  return cudaStreamSynchronize(s) == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

extern "C" int gbx_dposv_mixed_batched_exec(int batch, const int* n, int NB, const double* A, int nrhs,
                                            const double* B, double* X, int prec, double fp64_diag_cond, double tol,
                                            int maxiter, float* W, void* work, size_t work_bytes, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (check_args(batch, n, NB, nrhs, prec) || !A || !B || !X || !W || !work || maxiter < 0 || !(tol > 0.0) ||
      !(fp64_diag_cond >= 0.0))
    return GBX_ERR_ARG;
  if (work_bytes < blayout(batch, n, NB, nrhs).total) return GBX_ERR_WORKSPACE;
  if (int e = set_attrs()) return e;
  DevStreams* ds = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_run_mtx);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GBX_ERR_CUDA;
    ds = &g_run[dev];
    if (!ds->ready) return GBX_ERR_ARG;  // no plan was made in this process on this device
  }
  Run r;
  if (int e = make_run(r, batch, n, NB, nrhs, prec, fp64_diag_cond, A, B, X, tol, maxiter, W, work, work_bytes))
    return e;
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus cs;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return GBX_ERR_CUDA;
  if (cs == cudaStreamCaptureStatusActive) return emit_run(r, s, ds->side);  // into the caller's graph
  // not capturing: the run as a graph of its own, captured on a private stream and launched on `s`
  std::lock_guard<std::mutex> lk(g_run_mtx);  // one capture at a time on the private streams
  static cudaStream_t cap[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!cap[dev] && cudaStreamCreateWithFlags(&cap[dev], cudaStreamNonBlocking) != cudaSuccess) return GBX_ERR_CUDA;
  if (cudaStreamBeginCapture(cap[dev], cudaStreamCaptureModeRelaxed) != cudaSuccess) return GBX_ERR_CUDA;
  const int e = emit_run(r, cap[dev], ds->side);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(cap[dev], &g);
  if (e) {
    if (g) cudaGraphDestroy(g);
    return e;
  }
  if (ce != cudaSuccess || !g) return GBX_ERR_CUDA;
  cudaGraphExec_t ge = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) return GBX_ERR_CUDA;
  const cudaError_t le = cudaGraphLaunch(ge, s);
  cudaGraphExecDestroy(ge);  // released once the launch completes
  return le == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

extern "C" int gbx_dposv_mixed_batched_result(int batch, const int* n, int NB, int nrhs, double tol, const void* work,
                                              gbx_refine_info* info, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (check_args(batch, n, NB, nrhs, 0) || !work) return GBX_ERR_ARG;
  const BLayout L = blayout(batch, n, NB, nrhs);
  cudaStream_t s = (cudaStream_t)stream;
  const char* base = (const char*)work;
  std::vector<DevRec> rec(batch);
  RunState rs;
  DagState sw[2];
  if (cudaMemcpyAsync(rec.data(), base + L.rec, batch * sizeof(DevRec), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&rs, base + L.rs, sizeof(rs), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(sw, base + L.sweep, sizeof(sw), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return GBX_ERR_CUDA;
  bool ok = true;
  int first_bad = 0;
  for (int k = 0; k < batch; ++k) {
    const DevRec& d = rec[k];
    if (info) {
      info[k].iterations = d.iterations;
      info[k].factor_retries = d.retries;
      info[k].shift = d.shift;
      info[k].backward_error = d.live ? d.backward_error : INFINITY;
      info[k].anorm = d.anorm;
      info[k].cond_estimate = d.cond;
      info[k].fp64_diag_tiles = d.fp64_tiles;
    }
    if (!d.live) {
      ok = false;
      if (!first_bad) first_bad = d.piv;
    } else if (!(d.backward_error <= tol)) {
      ok = false;
    }
  }
  if (rs.status) return rs.status;
  if (sw[0].status || sw[1].status) return GBX_ERR_TIMEOUT;  // a sweep's wait ran out
  if (batch == 1 && first_bad > 0) return first_bad;
  return ok ? GBX_OK : GBX_ERR_NOCONV;
}

extern "C" int gbx_dposv_mixed_batched(int batch, const int* n, int NB, const double* A, int nrhs, const double* B,
                                       double* X, int prec, double fp64_diag_cond, double tol, int maxiter, float* W,
                                       void* work, size_t work_bytes, gbx_refine_info* info, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (int e = gbx_dposv_mixed_batched_plan(batch, n, NB, nrhs, prec, 0, work, work_bytes, stream)) return e;
  if (int e = gbx_dposv_mixed_batched_exec(batch, n, NB, A, nrhs, B, X, prec, fp64_diag_cond, tol, maxiter, W, work,
                                           work_bytes, stream))
    return e;
  return gbx_dposv_mixed_batched_result(batch, n, NB, nrhs, tol, work, info, stream);
}

extern "C" int gbx_dposv_mixed_bufferSize(int N, int NB, int nrhs, size_t* bytes) {
  if (N <= 0) return GBX_ERR_ARG;
  return gbx_dposv_mixed_batched_bufferSize(1, &N, NB, nrhs, bytes);
}

// one matrix: the batch of one
extern "C" int gbx_dposv_mixed(int N, int NB, const double* A, int nrhs, const double* B, double* X, int prec,
                               double fp64_diag_cond, double tol, int maxiter, float* W, void* work, size_t work_bytes,
                               gbx_refine_info* info, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N <= 0) return GBX_ERR_ARG;
  return gbx_dposv_mixed_batched(1, &N, NB, A, nrhs, B, X, prec, fp64_diag_cond, tol, maxiter, W, work, work_bytes,
                                 info, stream);
}
