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
#include <vector>

#include "block_ops.cuh"
#include "gbx_common.cuh"
#include "gbx_potrf.h"

extern "C" int gbx_potrf_mixed_bufferSize(int N, int NB, size_t* bytes);
extern "C" int gbx_potrf_mixed(int N, int NB, const double* A, float* W, int prec, double shift, void* work,
                               size_t work_bytes, void* stream);
extern "C" int gbx_potrf_mixed_info(const void* work, int N, int NB, float* cond_est, void* stream);

namespace gbx {
namespace refine {

constexpr int kMaxRhs = 16;

__device__ __forceinline__ long long slot_of(int m, int n, int NT) {
  return (long long)n * NT - (long long)n * (n - 1) / 2 + (m - n);
}
__host__ __device__ __forceinline__ int tdim(int t, int N, int NB, int NT) { return t == NT - 1 ? N - (NT - 1) * NB : NB; }

// Out = L_KK^{-T} (column-major), i.e. row r of Out holds column r of L_KK^{-1}; 128 rows per CTA
__global__ void __launch_bounds__(kThreads, 1) diag_inverse_kernel(const float* W, float* Inv, int N, int NB, int NT) {
  extern __shared__ __align__(16) float sm_f[];
  const int K = blockIdx.x, r0 = blockIdx.y * kBlk;
  const int n = tdim(K, N, NB, NT);
  if (r0 >= n) return;
  const int m = min(kBlk, n - r0);
  float* out = Inv + (long long)K * NB * NB;
  for (int idx = threadIdx.x; idx < kBlk * NB; idx += blockDim.x) {  // rows r0.. of the identity
    const int r = idx % kBlk, c = idx / kBlk;
    if (r < m) out[(r0 + r) + (long long)c * NB] = (r0 + r == c) ? 1.f : 0.f;
  }
  __syncthreads();
  const float* L = W + slot_of(K, K, NT) * (long long)NB * NB;
  op_trsm<float>(L, NB, out + r0, NB, m, n, sm_f);
}

// forward step, diagonal part: y_K = L_KK^{-1} x_K (Out^T x_K), in place in x
// one warp per output element c (lanes over r), all right-hand sides
__global__ void fwd_diag_kernel(const float* Inv, const float* X, float* Y, int N, int NB, int NT, int K, int nrhs) {
  extern __shared__ float xs_f[];  // [nrhs][NB]
  const int n = tdim(K, N, NB, NT);
  const float* out = Inv + (long long)K * NB * NB;
  for (int idx = threadIdx.x; idx < n * nrhs; idx += blockDim.x) {
    const int r = idx % n, j = idx / n;
    xs_f[j * NB + r] = X[(long long)j * N + (long long)K * NB + r];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
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

// forward step, column update: x_M -= L_MK y_K for every M > K; thread per row, y_K in smem
__global__ void fwd_update_kernel(const float* W, const float* Y, float* X, int N, int NB, int NT, int K, int nrhs) {
  extern __shared__ float ys_f[];  // [nrhs][NB]
  const int kn = tdim(K, N, NB, NT);
  for (int idx = threadIdx.x; idx < kn * nrhs; idx += blockDim.x) {
    const int r = idx % kn, j = idx / kn;
    ys_f[j * NB + r] = Y[(long long)j * N + (long long)K * NB + r];
  }
  __syncthreads();
  const long long row = (long long)(K + 1) * NB + (long long)blockIdx.x * blockDim.x + threadIdx.x;  // global row
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

// backward step, diagonal part: z_K = L_KK^{-T} y_K. A CTA owns 32 output rows (lanes, coalesced
// over i); its 8 warps split the column range and reduce through shared memory.
__global__ void bwd_diag_kernel(const float* Inv, const float* Y, float* X, int N, int NB, int NT, int K, int nrhs) {
  extern __shared__ float ys_f[];  // [nrhs][NB] then [8 warps][nrhs][32] partial sums
  const int n = tdim(K, N, NB, NT);
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

// backward step, column update: y_J -= L_KJ^T z_K for every J < K; warp per output element c
__global__ void bwd_update_kernel(const float* W, const float* X, float* Y, int N, int NB, int NT, int K, int nrhs) {
  extern __shared__ float zs_f[];  // [nrhs][NB]
  const int kn = tdim(K, N, NB, NT);
  for (int idx = threadIdx.x; idx < kn * nrhs; idx += blockDim.x) {
    const int r = idx % kn, j = idx / kn;
    zs_f[j * NB + r] = X[(long long)j * N + (long long)K * NB + r];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const long long total = (long long)K * NB;  // rows of y_0 .. y_{K-1}
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

__global__ void d2s_kernel(const double* in, float* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}
__global__ void s2d_kernel(const float* in, double* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

// ---- FP64 symmetric product Y := alpha A X + beta Y (A lower tiles) -----------------------------
// part 1: Y_m += A_mn X_n over the stored lower part (thread per row); diagonal tiles use j <= i
// part 2: Y_n += A_mn^T X_m over the strictly lower part (warp per column)
__global__ void symm_rows_kernel(const double* A, const double* X, double* Y, int N, int NB, int NT, int nrhs,
                                 double alpha) {
  extern __shared__ double xs_d[];  // [nrhs][512]
  const int slot = blockIdx.x, rb = blockIdx.y;
  int n = 0;
  long long first = 0;
  while (first + (NT - n) <= slot) {
    first += NT - n;
    ++n;
  }
  const int m = n + (int)(slot - first);
  const int mrows = tdim(m, N, NB, NT), ncols = tdim(n, N, NB, NT);
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

__global__ void symm_cols_kernel(const double* A, const double* X, double* Y, int N, int NB, int NT, int nrhs,
                                 double alpha) {
  extern __shared__ double xs_d[];  // [nrhs][512]
  const int slot = blockIdx.x;
  int n = 0;
  long long first = 0;
  while (first + (NT - n) <= slot) {
    first += NT - n;
    ++n;
  }
  const int m = n + (int)(slot - first);
  const int mrows = tdim(m, N, NB, NT), ncols = tdim(n, N, NB, NT);
  const double* T = A + (long long)slot * NB * NB;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
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

__global__ void scale_kernel(double* Y, long long n, double beta) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    Y[i] = beta == 0.0 ? 0.0 : Y[i] * beta;
}

// row sums of |A| (for ||A||_inf)
__global__ void absrow_kernel(const double* A, double* rs, int N, int NB, int NT) {
  const int slot = blockIdx.x;
  int n = 0;
  long long first = 0;
  while (first + (NT - n) <= slot) {
    first += NT - n;
    ++n;
  }
  const int m = n + (int)(slot - first);
  const int mrows = tdim(m, N, NB, NT), ncols = tdim(n, N, NB, NT);
  const double* T = A + (long long)slot * NB * NB;
  for (int i = threadIdx.x; i < mrows; i += blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < ncols; ++c)
      if (m != n || c <= i) s += fabs(T[i + (long long)c * NB]);
    atomicAdd(rs + (long long)m * NB + i, s);
  }
  for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < mrows; ++r)
      if (m != n || r > c) s += fabs(T[r + (long long)c * NB]);
    atomicAdd(rs + (long long)n * NB + c, s);
  }
}

// per right-hand side j: out[j*k + q] = reduction q of the columns (0: dot(a,b), 1: max|a|, 2: max|b|)
__global__ void colstats_kernel(const double* a, const double* b, int N, int nrhs, double* out) {
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

// y_j := y_j + coef_j * x_j  (coef from device memory)
__global__ void axpy_cols_kernel(double* y, const double* x, const double* coef, double sign, int N, int nrhs,
                                 int xscale_mode) {
  const long long n = (long long)N * nrhs;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(i / N);
    if (xscale_mode == 0) y[i] += sign * coef[j] * x[i];  // y += s*c*x
    else y[i] = x[i] + coef[j] * y[i];                    // y = x + c*y
  }
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
      cudaFuncSetAttribute(diag_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess)
    return GBX_ERR_CUDA;
  done = 1;
  return GBX_OK;
}
}  // namespace

extern "C" int gbx_spotri_diag(int N, int NB, const float* W, float* Inv, void* stream) {
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

extern "C" int gbx_dposv_mixed_bufferSize(int N, int NB, int nrhs, size_t* bytes) {
  if (N <= 0 || NB <= 0 || nrhs <= 0 || nrhs > kMaxRhs || !bytes) return GBX_ERR_ARG;
  size_t f = 0;
  if (int e = gbx_potrf_mixed_bufferSize(N, NB, &f)) return e;
  const int NT = (N + NB - 1) / NB;
  const size_t vec = (size_t)N * nrhs * sizeof(double);
  *bytes = f + (size_t)NT * NB * NB * sizeof(float) + 4 * vec + 2 * (size_t)N * nrhs * sizeof(float) + N * sizeof(double) +
           64 * kMaxRhs * sizeof(double) + 4096;
  return GBX_OK;
}

extern "C" int gbx_dposv_mixed(int N, int NB, const double* A, int nrhs, const double* B, double* X, int prec,
                               double tol, int maxiter, float* W, void* work, size_t work_bytes, gbx_refine_info* info,
                               void* stream) {
  if (N <= 0 || NB <= 0 || nrhs <= 0 || nrhs > kMaxRhs || !A || !B || !X || !W || !work || maxiter < 0)
    return GBX_ERR_ARG;
  size_t need = 0;
  if (int e = gbx_dposv_mixed_bufferSize(N, NB, nrhs, &need)) return e;
  if (work_bytes < need) return GBX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  size_t fbytes = 0;
  gbx_potrf_mixed_bufferSize(N, NB, &fbytes);
  const int NT = (N + NB - 1) / NB;
  char* p = (char*)work;
  void* fwork = p;
  p += (fbytes + 255) / 256 * 256;
  float* Inv = (float*)p;
  p += ((size_t)NT * NB * NB * sizeof(float) + 255) / 256 * 256;
  const size_t vec = (size_t)N * nrhs;
  double* R = (double*)p;
  p += (vec * 8 + 255) / 256 * 256;
  double* Z = (double*)p;
  p += (vec * 8 + 255) / 256 * 256;
  double* P = (double*)p;
  p += (vec * 8 + 255) / 256 * 256;
  double* Q = (double*)p;
  p += (vec * 8 + 255) / 256 * 256;
  float* tmp = (float*)p;
  p += (2 * vec * 4 + 255) / 256 * 256;
  double* rowsum = (double*)p;
  p += ((size_t)N * 8 + 255) / 256 * 256;
  double* stats = (double*)p;  // [kMaxRhs*3] x2 + coefficients
  double* coef = stats + 6 * kMaxRhs;

  gbx_refine_info inf;
  std::memset(&inf, 0, sizeof inf);
  // 1. low-precision factorisation (shifted and retried if it breaks down)
  double shift = 0.0;
  int st = 0;
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (int e = gbx_potrf_mixed(N, NB, A, W, prec, shift, fwork, fbytes, stream)) return e;
    float cond = 0.f;
    st = gbx_potrf_mixed_info(fwork, N, NB, &cond, stream);
    inf.cond_estimate = cond;
    if (st == 0) break;
    if (st < 0) return st;
    shift = shift == 0.0 ? (prec == 1 ? 1.0 / 2048 : 1.0 / 256) : shift * 4;
    ++inf.factor_retries;
  }
  if (st != 0) return st;
  inf.shift = shift;
  if (int e = gbx_spotri_diag(N, NB, W, Inv, stream)) return e;
  // ||A||_inf
  cudaMemsetAsync(rowsum, 0, (size_t)N * 8, s);
  absrow_kernel<<<NT * (NT + 1) / 2, 256, 0, s>>>(A, rowsum, N, NB, NT);
  colstats_kernel<<<1, 256, 0, s>>>(rowsum, nullptr, N, 1, stats);
  double hs[6 * kMaxRhs];
  cudaMemcpyAsync(hs, stats, 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  const double anorm = hs[1];
  std::vector<double> bnorm(nrhs), rz(nrhs), hcoef(2 * kMaxRhs);
  colstats_kernel<<<nrhs, 256, 0, s>>>(B, nullptr, N, nrhs, stats);
  cudaMemcpyAsync(hs, stats, 3 * nrhs * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  for (int j = 0; j < nrhs; ++j) bnorm[j] = hs[3 * j + 1];

  // 2. x0 = M^{-1} b ; r = b - A x0
  if (int e = gbx_sprecond(N, NB, W, Inv, nrhs, B, X, tmp, stream)) return e;
  cudaMemcpyAsync(R, B, vec * 8, cudaMemcpyDeviceToDevice, s);
  if (int e = gbx_dsymm_tiled(N, NB, A, nrhs, -1.0, X, 1.0, R, stream)) return e;
  // z = M^{-1} r ; p = z
  if (int e = gbx_sprecond(N, NB, W, Inv, nrhs, R, Z, tmp, stream)) return e;
  cudaMemcpyAsync(P, Z, vec * 8, cudaMemcpyDeviceToDevice, s);
  colstats_kernel<<<nrhs, 256, 0, s>>>(R, Z, N, nrhs, stats);
  cudaMemcpyAsync(hs, stats, 3 * nrhs * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  for (int j = 0; j < nrhs; ++j) rz[j] = hs[3 * j];
  // backward error of x0
  auto backward = [&](const double* stat_r, const double* stat_x) {
    double be = 0.0;
    for (int j = 0; j < nrhs; ++j) {
      const double den = anorm * stat_x[3 * j + 1] + bnorm[j];
      be = std::max(be, den > 0 ? stat_r[3 * j + 1] / den : 0.0);
    }
    return be;
  };
  double hx[3 * kMaxRhs];
  colstats_kernel<<<nrhs, 256, 0, s>>>(X, nullptr, N, nrhs, stats + 3 * kMaxRhs);
  cudaMemcpyAsync(hx, stats + 3 * kMaxRhs, 3 * nrhs * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  double be = backward(hs, hx);
  int it = 0;
  // 3. preconditioned CG in FP64
  for (; it < maxiter && be > tol; ++it) {
    if (int e = gbx_dsymm_tiled(N, NB, A, nrhs, 1.0, P, 0.0, Q, stream)) return e;  // q = A p
    colstats_kernel<<<nrhs, 256, 0, s>>>(P, Q, N, nrhs, stats);
    cudaMemcpyAsync(hs, stats, 3 * nrhs * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
    for (int j = 0; j < nrhs; ++j) hcoef[j] = hs[3 * j] != 0.0 ? rz[j] / hs[3 * j] : 0.0;  // alpha_j
    cudaMemcpyAsync(coef, hcoef.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice, s);
    axpy_cols_kernel<<<512, 256, 0, s>>>(X, P, coef, 1.0, N, nrhs, 0);   // x += alpha p
    axpy_cols_kernel<<<512, 256, 0, s>>>(R, Q, coef, -1.0, N, nrhs, 0);  // r -= alpha q
    if ((it + 1) % 8 == 0) {  // replace the recursive residual by the true one against drift
      cudaMemcpyAsync(R, B, vec * 8, cudaMemcpyDeviceToDevice, s);
      if (int e = gbx_dsymm_tiled(N, NB, A, nrhs, -1.0, X, 1.0, R, stream)) return e;
    }
    if (int e = gbx_sprecond(N, NB, W, Inv, nrhs, R, Z, tmp, stream)) return e;  // z = M^{-1} r
    colstats_kernel<<<nrhs, 256, 0, s>>>(R, Z, N, nrhs, stats);
    colstats_kernel<<<nrhs, 256, 0, s>>>(X, nullptr, N, nrhs, stats + 3 * kMaxRhs);
    cudaMemcpyAsync(hs, stats, 6 * kMaxRhs * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
    be = backward(hs, hs + 3 * kMaxRhs);
    for (int j = 0; j < nrhs; ++j) {
      const double rz_new = hs[3 * j];
      hcoef[kMaxRhs + j] = rz[j] != 0.0 ? rz_new / rz[j] : 0.0;  // beta_j
      rz[j] = rz_new;
    }
    cudaMemcpyAsync(coef + kMaxRhs, hcoef.data() + kMaxRhs, nrhs * sizeof(double), cudaMemcpyHostToDevice, s);
    axpy_cols_kernel<<<512, 256, 0, s>>>(P, Z, coef + kMaxRhs, 1.0, N, nrhs, 1);  // p = z + beta p
  }
  // 4. final check on the true residual
  cudaMemcpyAsync(R, B, vec * 8, cudaMemcpyDeviceToDevice, s);
  if (int e = gbx_dsymm_tiled(N, NB, A, nrhs, -1.0, X, 1.0, R, stream)) return e;
  colstats_kernel<<<nrhs, 256, 0, s>>>(R, nullptr, N, nrhs, stats);
  colstats_kernel<<<nrhs, 256, 0, s>>>(X, nullptr, N, nrhs, stats + 3 * kMaxRhs);
  cudaMemcpyAsync(hs, stats, 6 * kMaxRhs * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  inf.backward_error = backward(hs, hs + 3 * kMaxRhs);
  inf.iterations = it;
  inf.anorm = anorm;
  if (info) *info = inf;
  return inf.backward_error <= tol ? GBX_OK : GBX_ERR_NOCONV;
}
