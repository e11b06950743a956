// Batched Cholesky solves of many independent SPD matrices of uneven sizes in ONE persistent
// launch (no host round trip, capturable in a CUDA graph).
//
// Each CTA takes matrices from a device-side queue in the order the caller gives (largest first is
// the longest-processing-time schedule) and for each matrix runs, on 256 threads:
//   plain (FP64):  left-looking Cholesky over 128-column panels with the FP64 block ops, then the
//                  forward/backward solve for its right-hand sides, all in place;
//   fp32 + IR:     FP32 copy factorised the same way, FP32 solve, then `refine` steps of FP64
//                  iterative refinement x += (L L^T)^{-1} (b - A x) with the residual in FP64.
// Matrix i is column-major n_i x n_i (leading dimension n_i) at A + offA[i] (only the lower
// triangle is read); its right-hand sides are column-major n_i x nrhs at B + offB[i] and are
// overwritten by the solution.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <numeric>
#include <vector>

#include "block_ops.cuh"
#include "gbx_common.cuh"
#include "gbx_potrf.h"

namespace gbx {
namespace batched {

constexpr int kMaxN = 1024;  // largest matrix order of the batched kernel (shared-memory vectors)

// in-place left-looking Cholesky of an n x n column-major matrix (ld), 128-column panels;
// returns 0 or the 1-based index of the first bad pivot
template <typename T>
__device__ int factor(T* A, int n, int ld, T* sm) {
  for (int p0 = 0; p0 < n; p0 += kBlk) {
    const int pb = min(kBlk, n - p0);
    if (p0 > 0)
      for (int r0 = p0; r0 < n; r0 += kBlk)
        op_gemm_nt<T>(A + r0, ld, A + p0, ld, A + r0 + (long long)p0 * ld, ld, min(kBlk, n - r0), pb, p0, r0 == p0,
                      sm);
    const int info = op_potrf<T>(A + p0 + (long long)p0 * ld, ld, pb, sm);
    if (info) return p0 + info;
    for (int r0 = p0 + kBlk; r0 < n; r0 += kBlk)
      op_trsm<T>(A + p0 + (long long)p0 * ld, ld, A + r0 + (long long)p0 * ld, ld, min(kBlk, n - r0), pb, sm);
  }
  return 0;
}

// x := (L L^T)^{-1} x for one right-hand side held in shared memory xs[0..n)
// forward and backward substitution by 32-column panels: warp 0 solves the panel's triangle
// (shuffle-free, __syncwarp), the whole CTA applies the panel to the remaining rows
template <typename T>
__device__ void solve_vec(const T* L, int n, int ld, T* xs) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int p0 = 0; p0 < n; p0 += 32) {  // L y = x
    const int pw = min(32, n - p0);
    if (warp == 0) {
      for (int c = 0; c < pw; ++c) {
        if (lane == c) xs[p0 + c] /= L[(p0 + c) + (long long)(p0 + c) * ld];
        __syncwarp();
        if (lane > c && lane < pw) xs[p0 + lane] -= L[(p0 + lane) + (long long)(p0 + c) * ld] * xs[p0 + c];
        __syncwarp();
      }
    }
    __syncthreads();
    for (int i = p0 + pw + tid; i < n; i += blockDim.x) {
      T s = T(0);
      for (int c = 0; c < pw; ++c) s += L[i + (long long)(p0 + c) * ld] * xs[p0 + c];
      xs[i] -= s;
    }
    __syncthreads();
  }
  const int last = ((n - 1) / 32) * 32;
  for (int p0 = last; p0 >= 0; p0 -= 32) {  // L^T x = y
    const int pw = min(32, n - p0);
    // contributions of the already solved rows below the panel: xs[r] -= sum_i L(i, r) x_i
    for (int r = warp; r < pw; r += blockDim.x / 32) {
      T s = T(0);
      for (int i = p0 + pw + lane; i < n; i += 32) s += L[i + (long long)(p0 + r) * ld] * xs[i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) xs[p0 + r] -= s;
    }
    __syncthreads();
    if (warp == 0) {
      for (int c = pw - 1; c >= 0; --c) {
        if (lane == c) xs[p0 + c] /= L[(p0 + c) + (long long)(p0 + c) * ld];
        __syncwarp();
        if (lane < c) xs[p0 + lane] -= L[(p0 + c) + (long long)(p0 + lane) * ld] * xs[p0 + c];
        __syncwarp();
      }
    }
    __syncthreads();
  }
}

struct Params {
  int batch;
  const int* n;
  const long long* offA;
  const long long* offB;
  const int* order;
  double* A;
  double* B;
  float* L32;    // fp32 factors (offA layout), fp32 + IR mode only
  int nrhs;
  int mode;      // 0 plain FP64, 1 fp32 + IR
  int refine;    // IR steps
  int* info;     // per matrix: 0 or first bad pivot
  unsigned long long* head;
};

__global__ void __launch_bounds__(kThreads, 1) batched_kernel(Params P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_idx;
  __shared__ double xd[kMaxN];  // FP64 vector (solution / residual)
  __shared__ float xf[kMaxN];   // FP32 correction
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned long long t = atomicAdd(P.head, 1ULL);
      s_idx = t < (unsigned long long)P.batch ? P.order[t] : -1;
    }
    __syncthreads();
    const int idx = s_idx;
    if (idx < 0) break;
    const int n = P.n[idx];
    if (n <= 0 || n > kMaxN) {
      if (threadIdx.x == 0) P.info[idx] = -1;
      continue;
    }
    double* A = P.A + P.offA[idx];
    double* B = P.B + P.offB[idx];
    if (P.mode == 0) {
      const int inf = factor<double>(A, n, n, (double*)smem_raw);
      if (threadIdx.x == 0) P.info[idx] = inf;
      if (inf) continue;
      for (int j = 0; j < P.nrhs; ++j) {
        double* b = B + (long long)j * n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) xd[i] = b[i];
        __syncthreads();
        solve_vec<double>(A, n, n, xd);
        for (int i = threadIdx.x; i < n; i += blockDim.x) b[i] = xd[i];
        __syncthreads();
      }
    } else {
      float* L = P.L32 + P.offA[idx];
      for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) L[e] = (float)A[e];
      __syncthreads();
      const int inf = factor<float>(L, n, n, (float*)smem_raw);
      if (threadIdx.x == 0) P.info[idx] = inf;
      if (inf) continue;
      for (int j = 0; j < P.nrhs; ++j) {
        double* b = B + (long long)j * n;
        // x0 = fp32 solve of b, kept in xd; b itself is read again for the residuals
        for (int i = threadIdx.x; i < n; i += blockDim.x) xf[i] = (float)b[i];
        __syncthreads();
        solve_vec<float>(L, n, n, xf);
        for (int i = threadIdx.x; i < n; i += blockDim.x) xd[i] = (double)xf[i];
        __syncthreads();
        for (int it = 0; it < P.refine; ++it) {
          // r = b - A x with A symmetric from its lower triangle, FP64; thread per row
          for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double s = b[i];
            for (int c = 0; c <= i; ++c) s -= A[i + (long long)c * n] * xd[c];
            for (int r = i + 1; r < n; ++r) s -= A[r + (long long)i * n] * xd[r];
            xf[i] = (float)s;
          }
          __syncthreads();
          solve_vec<float>(L, n, n, xf);
          for (int i = threadIdx.x; i < n; i += blockDim.x) xd[i] += (double)xf[i];
          __syncthreads();
        }
        for (int i = threadIdx.x; i < n; i += blockDim.x) b[i] = xd[i];
        __syncthreads();
      }
    }
  }
}

std::mutex g_mtx;
int g_sms = 0;
bool g_attr = false;

}  // namespace batched
}  // namespace gbx

using namespace gbx;
using namespace gbx::batched;

extern "C" int gbx_batched_order(int batch, const int* n_host, int* order_host) {
  if (batch < 0 || (batch > 0 && (!n_host || !order_host))) return GBX_ERR_ARG;
  std::vector<int> o(batch);
  std::iota(o.begin(), o.end(), 0);
  std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return n_host[a] > n_host[b]; });
  std::copy(o.begin(), o.end(), order_host);
  return GBX_OK;
}

extern "C" int gbx_dposv_batched(int batch, const int* n, const long long* offA, const long long* offB,
                                 const int* order, double* A, double* B, int nrhs, int mode, int refine, float* L32,
                                 int* info, void* work, size_t work_bytes, void* stream) {
  if (batch < 0 || nrhs < 1 || (mode != 0 && mode != 1) || refine < 0) return GBX_ERR_ARG;
  if (batch == 0) return GBX_OK;
  if (!n || !offA || !offB || !order || !A || !B || !info || (mode == 1 && !L32)) return GBX_ERR_ARG;
  if (!work || work_bytes < 256) return GBX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t smem = (size_t)kBlk * kBlk * sizeof(double) + 64;
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    if (!g_attr) {
      int dev = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBX_ERR_CUDA;
      if (cudaFuncSetAttribute(batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return GBX_ERR_CUDA;
      g_attr = true;
    }
  }
  if (cudaMemsetAsync(work, 0, 256, s) != cudaSuccess) return GBX_ERR_CUDA;
  Params P;
  P.batch = batch;
  P.n = n;
  P.offA = offA;
  P.offB = offB;
  P.order = order;
  P.A = A;
  P.B = B;
  P.L32 = L32;
  P.nrhs = nrhs;
  P.mode = mode;
  P.refine = refine;
  P.info = info;
  P.head = (unsigned long long*)work;
  const int grid = std::max(1, std::min(g_sms, batch));
  batched_kernel<<<grid, kThreads, smem, s>>>(P);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}
