// Tile kernels of the backward sweep of the tiled solve, FP64, column-major tiles.
//
// The right-hand sides of the solve flowgraph (ttg_gb300/potrf/potrs.h) are stored as tiles of
// nrhs rows by NB columns (one column per matrix row), so both sweeps are right-side operations on
// them: the forward sweep L Y = B is Y_k := B_k L_kk^{-T} and B_m -= Y_k L_mk^T (the TRSM and GEMM
// shapes of the factorisation, gbx_dtrsm_rlt_tile / gbx_dgemm_nt_tile), the backward sweep
// L^T X = Y is X_k := Y_k L_kk^{-1} and Y_m -= X_k L_km, the two kernels below.
#include <cuda_runtime.h>

#include "gbx_common.cuh"
#include "gbx_potrf.h"
#include "taskq.h"

namespace gbx {
namespace solve {

constexpr int kRowsPerCta = 8;  // one warp per row of B

// B(m x n) := B L^{-1}, L lower n x n (non-unit): one warp per row, columns from the last one down,
// x_c = (b_c - sum_{k > c} x_k L(k, c)) / L(c, c); the row lives in shared memory, the lanes split
// the sum over k (column c of L is contiguous below the diagonal).
__global__ void __launch_bounds__(32 * kRowsPerCta) trsm_rln_kernel(int m, int n, const double* __restrict__ L, int ldl,
                                                                      double* B, int ldb) {
  extern __shared__ double xs[];  // [kRowsPerCta][n]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kRowsPerCta + warp;
  double* x = xs + (size_t)warp * n;
  if (r < m)
    for (int c = lane; c < n; c += 32) x[c] = B[r + (long long)c * ldb];
  __syncwarp();
  if (r >= m) return;
  for (int c = n - 1; c >= 0; --c) {
    const double* Lc = L + (long long)c * ldl;
    double s = 0.0;
    for (int k = c + 1 + lane; k < n; k += 32) s = fma(x[k], Lc[k], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[c] = (x[c] - s) / Lc[c];
    __syncwarp();
  }
  for (int c = lane; c < n; c += 32) B[r + (long long)c * ldb] = x[c];
}

// C(m x n) -= A(m x k) B(k x n): one thread per element of C in 16 x 16 blocks, k staged through
// shared memory in chunks of 16 columns of A and rows of B
constexpr int kTile = 16;
__global__ void __launch_bounds__(kTile * kTile) gemm_nn_kernel(int m, int n, int k, const double* __restrict__ A, int lda,
                                                                const double* __restrict__ B, int ldb, double* C, int ldc) {
  __shared__ double As[kTile][kTile + 1], Bs[kTile][kTile + 1];
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int i = blockIdx.x * kTile + tx, j = blockIdx.y * kTile + ty;
  double acc = 0.0;
  for (int k0 = 0; k0 < k; k0 += kTile) {
    // As[q][tx] = A(i, k0 + q), Bs[ty][q] = B(k0 + q, j)
    const int q = ty;
    As[q][tx] = (i < m && k0 + q < k) ? A[i + (long long)(k0 + q) * lda] : 0.0;
    Bs[ty][tx] = (j < n && k0 + tx < k) ? B[(k0 + tx) + (long long)j * ldb] : 0.0;
    __syncthreads();
#pragma unroll
    for (int p = 0; p < kTile; ++p) acc = fma(As[p][tx], Bs[ty][p], acc);
    __syncthreads();
  }
  if (i < m && j < n) C[i + (long long)j * ldc] -= acc;
}

}  // namespace solve
}  // namespace gbx

extern "C" int gbx_dtrsm_rln_tile(int m, int n, const double* L, int ldl, double* B, int ldb, void* stream) {
  if (m < 0 || n < 0 || ldl < (n > 1 ? n : 1) || ldb < (m > 1 ? m : 1)) return GBX_ERR_ARG;
  if (m == 0 || n == 0) return GBX_OK;
  if (!L || !B) return GBX_ERR_ARG;
  if (auto* q = gbx::taskq::recorder(stream)) {  // a device task queue's stream: record, do not launch
    if (n > 2048) return GBX_ERR_ARG;
    return gbx::taskq::record(q, gbx::taskq::make_op(gbx::taskq::OP_TRSM_RLN, m, n, 0, L, nullptr, B, ldl, 0, ldb));
  }
  const size_t smem = (size_t)gbx::solve::kRowsPerCta * n * sizeof(double);
  if (smem > 48 * 1024) {
    if (smem > 200 * 1024) return GBX_ERR_ARG;  // n <= 3200
    if (cudaFuncSetAttribute(gbx::solve::trsm_rln_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return GBX_ERR_CUDA;
  }
  const int grid = (m + gbx::solve::kRowsPerCta - 1) / gbx::solve::kRowsPerCta;
  gbx::solve::trsm_rln_kernel<<<grid, 32 * gbx::solve::kRowsPerCta, smem, (cudaStream_t)stream>>>(m, n, L, ldl, B, ldb);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

extern "C" int gbx_dgemm_nn_tile(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C,
                                 int ldc, void* stream) {
  if (m < 0 || n < 0 || k < 0 || lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) || ldc < (m > 1 ? m : 1))
    return GBX_ERR_ARG;
  if (m == 0 || n == 0 || k == 0) return GBX_OK;
  if (!A || !B || !C) return GBX_ERR_ARG;
  if (auto* q = gbx::taskq::recorder(stream))
    return gbx::taskq::record(q, gbx::taskq::make_op(gbx::taskq::OP_GEMM_NN, m, n, k, A, B, C, lda, ldb, ldc));
  using gbx::solve::kTile;
  dim3 grid((m + kTile - 1) / kTile, (n + kTile - 1) / kTile);
  gbx::solve::gemm_nn_kernel<<<grid, kTile * kTile, 0, (cudaStream_t)stream>>>(m, n, k, A, lda, B, ldb, C, ldc);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}
