// Inverse of an SPD matrix from its tiled Cholesky factor (the reference's POTRI chain,
// examples/potrf/potri.h:18-29: TRTRI of the lower factor, examples/potrf/trtri_L.h, then LAUUM,
// examples/potrf/lauum.h), FP64, in place on the tile-major lower storage.
//
//   TRTRI (L := L^{-1}), step k = 0 .. NT-1 (the tile algorithm of trtri_L.h's TRSMR / GEMM /
//   TRSML / TRTRI tasks):   A_mk := -A_mk L_kk^{-1}     (m > k)
//                           A_mn += A_mk A_kn            (m > k, n < k)
//                           A_kn := L_kk^{-1} A_kn       (n < k)
//                           A_kk := L_kk^{-1}
//   LAUUM (A := W^T W for the lower W = L^{-1}), step k (lauum.h's SYRK / GEMM / TRMM / LAUUM):
//                           A_mn += A_km^T A_kn          (n <= m < k)
//                           A_kn := A_kk^T A_kn          (n < k, A_kk lower)
//                           A_kk := A_kk^T A_kk          (lower)
// Every step is a few grid launches of one block product (one CTA per 128 x 128 output block):
// C = beta C + alpha op(A) op(B), where op transposes or not and a "lower" operand only counts
// the stored lower triangle of its tile. Outputs that overlap an operand go to a scratch row or
// column of tiles first. L_kk^{-1} comes from the FP64 block TRSM on the identity (its transpose,
// L^{-T}, is what the block TRSM produces).
#include <cuda_runtime.h>

#include <algorithm>

#include "block_ops.cuh"
#include "gbx_common.cuh"
#include "gbx_potrf.h"

namespace gbx {
namespace potri {

__host__ __device__ __forceinline__ long long slot_of(int m, int n, int NT) {
  return (long long)n * NT - (long long)n * (n - 1) / 2 + (m - n);
}
__host__ __device__ __forceinline__ int tdim(int t, int N, int NB, int NT) { return t == NT - 1 ? N - (NT - 1) * NB : NB; }

// one operand element as the product sees it: op(X)(r, c) = X(c, r) if transposed, else X(r, c);
// `rows` x `cols` is the stored extent from X; a lower operand reads zero above the diagonal of
// its tile, whose column index is sc + coff (X starts coff columns into the tile)
template <bool T, bool LOW>
__device__ __forceinline__ double ld_op(const double* X, int ld, int r, int c, int rows, int cols, int coff) {
  const int sr = T ? c : r, sc = T ? r : c;
  if (sr >= rows || sc >= cols || (LOW && sr < sc + coff)) return 0.0;
  return __ldcg(X + sr + (long long)sc * ld);
}

// acc (8 x 8 per thread: rows 4tx.., 64+4tx.., columns 4ty.., 64+4ty..) += sum over k < kd of
// op(A)(i, k) op(B)(k, j) for the m x n output block. A is stored m x kd (kd x m if TA), B kd x n
// (n x kd if TB). k is staged through shared memory 16 at a time; each operand is loaded with
// consecutive threads on its stored rows (coalesced).
template <bool TA, bool TB, bool LA, bool LB>
__device__ void gemm_gen_acc(double (&acc)[8][8], const double* A, int lda, const double* B, int ldb, int m, int n,
                             int kd, double* sm, int a_coff = 0, int b_coff = 0) {
  double* As = sm;              // [16][128]: As[kk * 128 + i] = op(A)(i, k0 + kk)
  double* Bs = sm + kKC * kBlk;  // [16][128]: Bs[kk * 128 + j] = op(B)(k0 + kk, j)
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int ar = TA ? kd : m, ac = TA ? m : kd;  // stored extents: op(A) is m x kd
  const int br = TB ? n : kd, bc = TB ? kd : n;  // op(B) is kd x n
  for (int k0 = 0; k0 < kd; k0 += kKC) {
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      if (!TA) {  // stored (i, k): threads along i
        const int i = tid & 127, kk = (tid >> 7) + 2 * s;
        As[kk * kBlk + i] = ld_op<false, LA>(A, lda, i, k0 + kk, ar, ac, a_coff);
      } else {  // stored (k, i): threads along k
        const int kk = tid & 15, i = (tid >> 4) + 16 * s;
        As[kk * kBlk + i] = ld_op<true, LA>(A, lda, i, k0 + kk, ar, ac, a_coff);
      }
      if (!TB) {  // stored (k, j): threads along k
        const int kk = tid & 15, j = (tid >> 4) + 16 * s;
        Bs[kk * kBlk + j] = ld_op<false, LB>(B, ldb, k0 + kk, j, br, bc, b_coff);
      } else {  // stored (j, k): threads along j
        const int j = tid & 127, kk = (tid >> 7) + 2 * s;
        Bs[kk * kBlk + j] = ld_op<true, LB>(B, ldb, k0 + kk, j, br, bc, b_coff);
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKC; ++kk) {
      double a0[4], a1[4], b0[4], b1[4];
      lds4(As + kk * kBlk + 4 * tx, a0);
      lds4(As + kk * kBlk + 64 + 4 * tx, a1);
      lds4(Bs + kk * kBlk + 4 * ty, b0);
      lds4(Bs + kk * kBlk + 64 + 4 * ty, b1);
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fma(i < 4 ? a0[i & 3] : a1[i & 3], j < 4 ? b0[j & 3] : b1[j & 3], acc[i][j]);
    }
  }
  __syncthreads();
}

// C(m x n block) := beta C + alpha acc
__device__ __forceinline__ void store_acc(const double (&acc)[8][8], double* C, int ldc, int m, int n, double alpha,
                                          double beta) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int col = (j < 4 ? 0 : 60) + 4 * ty + j;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int row = (i < 4 ? 0 : 60) + 4 * tx + i;
      if (row < m && col < n) {
        double* p = C + row + (long long)col * ldc;
        __stcg(p, beta == 0.0 ? alpha * acc[i][j] : fma(alpha, acc[i][j], __ldcg(p)));
      }
    }
  }
}

enum Op : int {
  TRSM_RIGHT = 0,  // S_m = -A_mk O^T         (m > k)        O = L_kk^{-T}
  GEMM_NN = 1,     // A_mn += A_mk A_kn        (m > k, n < k)
  TRSM_LEFT = 2,   // S_n = O^T A_kn           (n < k)
  LAUUM_UPD = 3,   // A_mn += A_km^T A_kn      (n <= m < k)
  TRMM = 4,        // S_n = A_kk^T A_kn        (n < k, A_kk lower)
  LAUUM_DIAG = 5,  // S_0 = A_kk^T A_kk        (both lower)
};

struct StepArgs {
  double* tiles;  // the tile-major lower storage
  double* S;      // scratch: a row / column of NT tiles
  const double* O;  // L_kk^{-T} (NB x NB, ld NB)
  int N, NB, NT, k;
};

// blockIdx.x: output tile (per op), blockIdx.y: 128 x 128 block of it (NB/128 x NB/128)
template <int OP>
__global__ void __launch_bounds__(kThreads, 1) step_kernel(StepArgs P) {
  extern __shared__ __align__(16) double smem[];
  const int NB = P.NB, NT = P.NT, N = P.N, k = P.k, r = NB / kBlk;
  const int bi = blockIdx.y % r, bj = blockIdx.y / r;
  const long long tl = (long long)NB * NB;
  auto T = [&](int a, int b) { return P.tiles + slot_of(a, b, NT) * tl; };
  const int kk = tdim(k, N, NB, NT);
  double acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0;
  int mrows, ncols;
  double* C;
  double alpha = 1.0, beta = 1.0;
  if (OP == TRSM_RIGHT) {
    const int m = k + 1 + blockIdx.x;
    mrows = tdim(m, N, NB, NT) - kBlk * bi;
    ncols = kk - kBlk * bj;
    if (mrows <= 0 || ncols <= 0) return;
    // rows bi of A_mk times columns bj of O^T: op(B)(p, j) = O(j, p)
    gemm_gen_acc<false, true, false, false>(acc, T(m, k) + kBlk * bi, NB, P.O + kBlk * bj, NB, min(mrows, kBlk),
                                            min(ncols, kBlk), kk, smem);
    C = P.S + (long long)blockIdx.x * tl + kBlk * bi + (long long)kBlk * bj * NB;
    alpha = -1.0;
    beta = 0.0;
  } else if (OP == GEMM_NN) {
    const int nk = k;  // outputs (m, n), m in (k, NT), n in [0, k)
    const int m = k + 1 + blockIdx.x / nk, n = blockIdx.x % nk;
    mrows = tdim(m, N, NB, NT) - kBlk * bi;
    ncols = tdim(n, N, NB, NT) - kBlk * bj;
    if (mrows <= 0 || ncols <= 0) return;
    gemm_gen_acc<false, false, false, false>(acc, T(m, k) + kBlk * bi, NB, T(k, n) + (long long)kBlk * bj * NB, NB,
                                             min(mrows, kBlk), min(ncols, kBlk), kk, smem);
    C = T(m, n) + kBlk * bi + (long long)kBlk * bj * NB;
  } else if (OP == TRSM_LEFT) {
    const int n = blockIdx.x;
    mrows = kk - kBlk * bi;
    ncols = tdim(n, N, NB, NT) - kBlk * bj;
    if (mrows <= 0 || ncols <= 0) return;
    // op(A)(i, p) = O(p, i) for rows bi: stored columns bi of O
    gemm_gen_acc<true, false, false, false>(acc, P.O + (long long)kBlk * bi * NB, NB, T(k, n) + (long long)kBlk * bj * NB,
                                            NB, min(mrows, kBlk), min(ncols, kBlk), kk, smem);
    C = P.S + (long long)n * tl + kBlk * bi + (long long)kBlk * bj * NB;
    beta = 0.0;
  } else if (OP == LAUUM_UPD) {
    int m = 0, rem = blockIdx.x;  // outputs (m, n), n <= m < k, packed row by row
    while (rem > m) {
      rem -= m + 1;
      ++m;
    }
    const int n = rem;
    mrows = NB - kBlk * bi;  // m, n < k: full tiles
    ncols = NB - kBlk * bj;
    // op(A)(i, p) = A_km(p, i): stored columns bi of A_km; op(B)(p, j) = A_kn(p, j)
    gemm_gen_acc<true, false, false, false>(acc, T(k, m) + (long long)kBlk * bi * NB, NB,
                                            T(k, n) + (long long)kBlk * bj * NB, NB, min(mrows, kBlk), min(ncols, kBlk),
                                            kk, smem);
    C = T(m, n) + kBlk * bi + (long long)kBlk * bj * NB;
  } else if (OP == TRMM) {
    const int n = blockIdx.x;
    mrows = kk - kBlk * bi;
    ncols = NB - kBlk * bj;
    if (mrows <= 0) return;
    // op(A)(i, p) = A_kk(p, i) over the stored lower triangle of A_kk (p >= i)
    const double* Akk = T(k, k);
    gemm_gen_acc<true, false, true, false>(acc, Akk + (long long)kBlk * bi * NB, NB, T(k, n) + (long long)kBlk * bj * NB,
                                           NB, min(mrows, kBlk), min(ncols, kBlk), kk, smem, kBlk * bi, 0);
    C = P.S + (long long)n * tl + kBlk * bi + (long long)kBlk * bj * NB;
    beta = 0.0;
  } else {  // LAUUM_DIAG
    mrows = kk - kBlk * bi;
    ncols = kk - kBlk * bj;
    if (mrows <= 0 || ncols <= 0 || bi < bj) return;  // the lower blocks of A_kk^T A_kk
    const double* Akk = T(k, k);
    gemm_gen_acc<true, false, true, true>(acc, Akk + (long long)kBlk * bi * NB, NB, Akk + (long long)kBlk * bj * NB, NB,
                                          min(mrows, kBlk), min(ncols, kBlk), kk, smem, kBlk * bi, kBlk * bj);
    C = P.S + kBlk * bi + (long long)kBlk * bj * NB;
    beta = 0.0;
  }
  store_acc(acc, C, NB, min(mrows, kBlk), min(ncols, kBlk), alpha, beta);
}

// O := L_kk^{-T} (column-major NB x NB): the block TRSM of 128 identity rows per CTA
__global__ void __launch_bounds__(kThreads, 1) diag_inverse64_kernel(const double* Lkk, double* O, int n, int NB) {
  extern __shared__ __align__(16) double smem[];
  const int r0 = blockIdx.x * kBlk;
  if (r0 >= n) return;
  const int m = min(kBlk, n - r0);
  for (int idx = threadIdx.x; idx < kBlk * NB; idx += blockDim.x) {
    const int r = idx % kBlk, c = idx / kBlk;
    if (r < m) O[(r0 + r) + (long long)c * NB] = (r0 + r == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  op_trsm<double>(Lkk, NB, O + r0, NB, m, n, smem);
}

// dst tile(s) := src tile(s), NB x NB each, cnt tiles; lower_only: the lower triangle only
__global__ void copy_tiles_kernel(const double* src, double* dst, long long cnt_elems, int NB, int lower_only) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt_elems;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % NB), j = (int)((e / NB) % NB);
    if (!lower_only || i >= j) dst[e] = src[e];
  }
}
// A_kk (lower) := O^T
__global__ void store_transpose_lower_kernel(const double* O, double* Akk, int n, int NB) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
    const int i = e % n, j = e / n;
    if (i >= j) Akk[i + (long long)j * NB] = O[j + (long long)i * NB];
  }
}

template <int OP>
int launch_step(const StepArgs& a, int ntiles, cudaStream_t s) {
  if (ntiles <= 0) return GBX_OK;
  const int r = a.NB / kBlk;
  const size_t smem = 2 * kKC * kBlk * sizeof(double);
  step_kernel<OP><<<dim3(ntiles, r * r), kThreads, smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

}  // namespace potri
}  // namespace gbx

using namespace gbx;
using namespace gbx::potri;

extern "C" int gbx_dpotri_tiled_bufferSize(int N, int NB, size_t* bytes) {
  if (N <= 0 || NB <= 0 || NB % kBlk || !bytes) return GBX_ERR_ARG;
  const long long NT = (N + NB - 1) / NB;
  *bytes = (size_t)(NT + 1) * NB * NB * sizeof(double) + 256;  // a row / column of tiles, then O
  return GBX_OK;
}

extern "C" int gbx_dpotri_tiled(int N, int NB, double* tiles, void* work, size_t work_bytes, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  size_t need = 0;
  if (int e = gbx_dpotri_tiled_bufferSize(N, NB, &need)) return e;
  if (!tiles) return GBX_ERR_ARG;
  if (!work || work_bytes < need) return GBX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  static int attr_done = 0;  // benign race: every caller sets the same value
  if (!attr_done) {
    if (cudaFuncSetAttribute(diag_inverse64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(op_trsm_smem_elems<double>() * sizeof(double))) != cudaSuccess)
      return GBX_ERR_CUDA;
    attr_done = 1;
  }
  const int NT = (N + NB - 1) / NB;
  const long long tl = (long long)NB * NB;
  double* S = (double*)work;
  double* O = S + (long long)NT * tl;
  StepArgs a;
  a.tiles = tiles;
  a.S = S;
  a.O = O;
  a.N = N;
  a.NB = NB;
  a.NT = NT;
  auto T = [&](int m, int n) { return tiles + slot_of(m, n, NT) * tl; };
  const int cgrid = 1024;
  // TRTRI: L := L^{-1}
  for (int k = 0; k < NT; ++k) {
    a.k = k;
    const int kk = tdim(k, N, NB, NT);
    diag_inverse64_kernel<<<(kk + kBlk - 1) / kBlk, kThreads, op_trsm_smem_elems<double>() * sizeof(double), s>>>(
        T(k, k), O, kk, NB);
    if (k + 1 < NT) {  // column below: S_m = -A_mk L_kk^{-1}, back into A_mk (the column is contiguous)
      if (int e = launch_step<TRSM_RIGHT>(a, NT - k - 1, s)) return e;
      copy_tiles_kernel<<<cgrid, 256, 0, s>>>(S, T(k + 1, k), (long long)(NT - k - 1) * tl, NB, 0);
    }
    if (k > 0 && k + 1 < NT)
      if (int e = launch_step<GEMM_NN>(a, (NT - k - 1) * k, s)) return e;
    if (k > 0) {  // row left of the diagonal: S_n = L_kk^{-1} A_kn
      if (int e = launch_step<TRSM_LEFT>(a, k, s)) return e;
      for (int n = 0; n < k; ++n)
        copy_tiles_kernel<<<64, 256, 0, s>>>(S + (long long)n * tl, T(k, n), tl, NB, 0);
    }
    store_transpose_lower_kernel<<<256, 256, 0, s>>>(O, T(k, k), kk, NB);
  }
  // LAUUM: A := W^T W for the lower W now in place
  for (int k = 0; k < NT; ++k) {
    a.k = k;
    if (k > 0) {
      if (int e = launch_step<LAUUM_UPD>(a, k * (k + 1) / 2, s)) return e;
      if (int e = launch_step<TRMM>(a, k, s)) return e;
      for (int n = 0; n < k; ++n)
        copy_tiles_kernel<<<64, 256, 0, s>>>(S + (long long)n * tl, T(k, n), tl, NB, 0);
    }
    if (int e = launch_step<LAUUM_DIAG>(a, 1, s)) return e;
    copy_tiles_kernel<<<64, 256, 0, s>>>(S, T(k, k), tl, NB, 1);
  }
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}
