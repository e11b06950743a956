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
  int refine;    // IR steps
  int* info;     // per matrix: 0 or first bad pivot
  unsigned long long* head;
};

// MODE 0: plain FP64 (one CTA per SM: 128 KB of shared memory for the FP64 block ops);
// MODE 1: fp32 + IR (64 KB of shared memory, two CTAs per SM)
template <int MODE>
__global__ void __launch_bounds__(kThreads, MODE == 0 ? 1 : 2) batched_kernel(Params P) {
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
    if constexpr (MODE == 0) {
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
constexpr size_t kSmem64 = (size_t)kBlk * kBlk * sizeof(double) + 64;
constexpr size_t kSmem32 = (size_t)kBlk * kBlk * sizeof(float) + 64;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform_elem(uint64_t seed, long long i, long long j) {
  const uint64_t r = mix64(mix64(seed) ^ (((uint64_t)i << 32) | (uint64_t)(uint32_t)j));
  return __dsub_rn(__dmul_rn((double)(r >> 11), 1.0 / 9007199254740992.0), 0.5);
}

// matrix k of the batch: (M + M^T)/2 + n*I with M_ij uniform in [-0.5, 0.5) from the counter-based
// generator with seed (seed + k * 0x9e3779b97f4a7c15); one CTA-strided loop per matrix
__global__ void gen_batch_kernel(int batch, const int* n, const long long* offA, unsigned long long seed, double* A) {
  for (int k = blockIdx.x; k < batch; k += gridDim.x) {
    const int nk = n[k];
    const uint64_t sk = seed + (uint64_t)k * 0x9e3779b97f4a7c15ULL;
    double* out = A + offA[k];
    for (long long e = threadIdx.x; e < (long long)nk * nk; e += blockDim.x) {
      const int i = (int)(e % nk), j = (int)(e / nk);
      double v;
      if (i == j) v = __dadd_rn(uniform_elem(sk, i, i), (double)nk);
      else v = __dmul_rn(0.5, __dadd_rn(uniform_elem(sk, i, j), uniform_elem(sk, j, i)));
      out[e] = v;
    }
  }
}

}  // namespace batched
}  // namespace gbx

using namespace gbx;
using namespace gbx::batched;

extern "C" int gbx_dgen_uniform_sym_batched(int batch, const int* n, const long long* offA, unsigned long long seed,
                                            double* A, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (batch < 0 || (batch > 0 && (!n || !offA || !A))) return GBX_ERR_ARG;
  if (batch == 0) return GBX_OK;
  gen_batch_kernel<<<std::min(batch, 4096), 256, 0, (cudaStream_t)stream>>>(batch, n, offA, seed, A);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

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
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  return gbx_dposv_batched_ex(batch, n, offA, offB, order, A, B, nrhs, mode, refine, L32, info, 0, work, work_bytes,
                              stream);
}

extern "C" int gbx_dposv_batched_ex(int batch, const int* n, const long long* offA, const long long* offB,
                                    const int* order, double* A, double* B, int nrhs, int mode, int refine, float* L32,
                                    int* info, int ctas, void* work, size_t work_bytes, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (batch < 0 || nrhs < 1 || (mode != 0 && mode != 1) || refine < 0 || ctas < 0) return GBX_ERR_ARG;
  if (batch == 0) return GBX_OK;
  if (!n || !offA || !offB || !order || !A || !B || !info || (mode == 1 && !L32)) return GBX_ERR_ARG;
  if (!work || work_bytes < 256) return GBX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    if (!g_attr) {
      int dev = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBX_ERR_CUDA;
      if (cudaFuncSetAttribute(batched_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem64) !=
              cudaSuccess ||
          cudaFuncSetAttribute(batched_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem32) !=
              cudaSuccess)
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
  P.refine = refine;
  P.info = info;
  P.head = (unsigned long long*)work;
  // default grid: every resident CTA slot (1 per SM in FP64, 2 per SM in fp32 + IR); `ctas` overrides it
  int grid = ctas > 0 ? ctas : (mode == 0 ? g_sms : 2 * g_sms);
  grid = std::max(1, std::min(grid, batch));
  if (mode == 0) batched_kernel<0><<<grid, kThreads, kSmem64, s>>>(P);
  else batched_kernel<1><<<grid, kThreads, kSmem32, s>>>(P);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}
