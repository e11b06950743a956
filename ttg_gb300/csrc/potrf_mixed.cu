// Mixed-precision tiled Cholesky for GB300 (sm_103a): the flowgraph of the reference's potrf
// example run by one persistent, warp-specialised kernel.
//
//   working matrix W   FP32 lower tiles (NB x NB column-major, the factor on exit)
//   operand copies Lb  every finished off-diagonal tile L_mk in bf16 or fp16, row-major (K-major
//                      for the tensor cores), each row scaled by a power of two (exponent in rowexp)
//   POTRF(K)           FP32 on the diagonal tile, one CTA, left-looking over 128-column panels
//   TRSM(M,K)          FP32, 128-row sub-tasks; writes L_MK and its scaled low-precision copy
//   SYRK(K,M), GEMM    tcgen05.mma (kind::f16) on 128 x 256 sub-tiles, K = NB, fp32 accumulators in
//                      TMEM; the epilogue applies the row scales and updates W in place
// Tasks follow the lookahead order of the FP64 executor at tile level; each tile task is split
// into a fixed number of CTA sub-tasks (unused sub-task slots are skipped) and completion counters
// per tile count finished sub-tasks.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "block_ops.cuh"
#include "gbx_common.cuh"
#include "gbx_potrf.h"
#include "tc_common.cuh"

namespace gbx {
namespace tc {
int make_tmap_kmajor_16b(CUtensorMap* map, const void* base, uint64_t rows, uint64_t k, uint64_t ld, uint32_t box_rows,
                         bool bf16);
}

namespace mixed {

using namespace gbx::tc;

constexpr int kThr = 256;            // 8 warps: 0 TMA, 1 MMA, 4..7 epilogue (tensor tasks); all (SIMT tasks)
constexpr int kSubM = 128, kSubN = 256, kBK = 64, kStages = 4;
constexpr uint32_t kABytes = kSubM * kBK * 2, kBBytes = kSubN * kBK * 2, kStageBytes = kABytes + kBBytes;
constexpr size_t kTcSmem = (size_t)kStages * kStageBytes;  // 192 KB (1024-aligned ring)
constexpr size_t kSimtSmem = (size_t)kBlk * kBlk * sizeof(float) + 64;
constexpr size_t kSmemBytes = (kTcSmem > kSimtSmem ? kTcSmem : kSimtSmem) + 1024;

enum : int { T_POTRF = 0, T_TRSM = 1, T_SYRK = 2, T_GEMM = 3 };

struct TileKey {
  int type, a, b, c;
};

__host__ __device__ __forceinline__ long long seg_prefix(long long k, long long R) {
  const long long s1 = k * R - k * (k - 1) / 2;
  const long long s2 = k * R * R - R * k * (k - 1) + (k - 1) * k * (2 * k - 1) / 6;
  return (3 * s1 + s2) / 2;
}
__host__ __device__ __forceinline__ long long num_tile_tasks(int NT) { return NT + seg_prefix(NT - 1, NT - 1); }

// the lookahead order of the tile flowgraph (same rule as the FP64 executor's block order)
__host__ __device__ inline TileKey decode(long long t, int NT) {
  if (t < NT) return t == 0 ? TileKey{T_POTRF, 0, 0, 0} : TileKey{T_TRSM, (int)t, 0, 0};
  const long long u = t - NT, R = NT - 1;
  int lo = 0, hi = NT - 2;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (seg_prefix(mid, R) <= u) lo = mid;
    else hi = mid - 1;
  }
  const int k = lo;
  const long long p = u - seg_prefix(k, R);
  const int r = NT - k - 1;
  if (p == 0) return TileKey{T_SYRK, k, k + 1, 0};
  if (p < r) return TileKey{T_GEMM, k + 1 + (int)p, k + 1, k};
  if (p == r) return TileKey{T_POTRF, k + 1, 0, 0};
  if (p < 2 * (long long)r) return TileKey{T_TRSM, k + 1 + (int)(p - r), k + 1, 0};
  const long long pp = p - 2 * (long long)r, q = r - 1;
  int clo = 0, chi = (int)q - 1;
  while (clo < chi) {
    const int mid = (clo + chi + 1) >> 1;
    const long long S = (long long)mid * q - (long long)mid * (mid - 1) / 2;
    if (S <= pp) clo = mid;
    else chi = mid - 1;
  }
  const long long o = pp - ((long long)clo * q - (long long)clo * (clo - 1) / 2);
  const int n = k + 2 + clo;
  if (o == 0) return TileKey{T_SYRK, k, n, 0};
  return TileKey{T_GEMM, n + (int)o, n, k};
}

struct Params {
  TraceBuf trace;
  float* W;
  void* Lb;  // bf16 or fp16, row-major per tile
  int* rowexp;
  int N, NB, NT;
  int f16;     // 1: fp16 operands, 0: bf16
  int sub_g;   // GEMM sub-tasks per tile = (NB/128)*(NB/256)
  int sub_t;   // TRSM sub-tasks per tile = NB/128
  int sub_s;   // SYRK sub-tasks per tile (lower 128 x 256 sub-tiles)
  long long ntasks;  // tile tasks * sub_g
  DagState* st;
  int* cnt;
  float* cond_est;  // max over diagonal tiles of (max L_ii / min L_ii)^2
  uint64_t timeout_ns;
};

__device__ __forceinline__ long long slot_of(int m, int n, int NT) {
  return (long long)n * NT - (long long)n * (n - 1) / 2 + (m - n);
}
__device__ __forceinline__ int tdim(int t, const Params& P) { return t == P.NT - 1 ? P.N - (P.NT - 1) * P.NB : P.NB; }

// i-th lower 128 x 256 sub-tile of a diagonal tile (rows 128*si, cols 256*sj with 256*sj < 128*(si+1))
__device__ __forceinline__ void syrk_sub(int idx, int NB, int& si, int& sj) {
  const int nr = NB / kSubM, nc = NB / kSubN;
  for (int j = 0; j < nc; ++j)
    for (int i = 0; i < nr; ++i)
      if (kSubN * j < kSubM * (i + 1)) {
        if (idx-- == 0) {
          si = i;
          sj = j;
          return;
        }
      }
  si = sj = -1;
}

__device__ __forceinline__ float pow2f(int e) {
  e = max(-126, min(127, e));
  return __int_as_float((e + 127) << 23);
}

// ---- FP32 SIMT tasks ---------------------------------------------------------------------------
__device__ int task_potrf(const Params& P, int K, float* sm) {
  const int n = tdim(K, P), NB = P.NB;
  float* A = P.W + slot_of(K, K, P.NT) * (long long)NB * NB;
  uint64_t ph[3] = {0, 0, 0};  // time in the three phases (tracing only)
  for (int p0 = 0; p0 < n; p0 += kBlk) {
    const int pb = min(kBlk, n - p0);
    uint64_t t = P.trace.buf ? globaltimer_ns() : 0;
    if (p0 > 0)
      for (int r0 = p0; r0 < n; r0 += kBlk)
        op_gemm_nt<float>(A + r0, NB, A + p0, NB, A + r0 + (long long)p0 * NB, NB, min(kBlk, n - r0), pb, p0,
                          r0 == p0, sm);
    if (P.trace.buf) {
      const uint64_t u = globaltimer_ns();
      ph[0] += u - t;
      t = u;
    }
    const int info = op_potrf<float>(A + p0 + (long long)p0 * NB, NB, pb, sm);
    if (info) return p0 + info;
    if (P.trace.buf) {
      const uint64_t u = globaltimer_ns();
      ph[1] += u - t;
      t = u;
    }
    for (int r0 = p0 + kBlk; r0 < n; r0 += kBlk)
      op_trsm<float>(A + p0 + (long long)p0 * NB, NB, A + r0 + (long long)p0 * NB, NB, min(kBlk, n - r0), pb, sm);
    if (P.trace.buf) ph[2] += globaltimer_ns() - t;
  }
  if (P.trace.buf && threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) trace_record(P.trace, globaltimer_ns() - ph[q], 4 + q, K, 0, 0, 0);
  // condition estimate of the diagonal tile from its factor's diagonal
  if (threadIdx.x == 0) {
    float mn = 3.0e38f, mx = 0.f;
    for (int i = 0; i < n; ++i) {
      const float d = __ldcg(A + i + (long long)i * NB);
      mn = fminf(mn, d);
      mx = fmaxf(mx, d);
    }
    const float est = (mx / mn) * (mx / mn);
    atomicMax((int*)P.cond_est, __float_as_int(est));  // positive floats order like their bits
  }
  __syncthreads();
  return 0;
}

__device__ void task_trsm(const Params& P, int M, int K, int rb, float* sm) {
  const int NB = P.NB, r0 = rb * kBlk, mrows = tdim(M, P), ncols = tdim(K, P);
  if (r0 >= mrows) return;
  const int m = min(kBlk, mrows - r0);
  const long long sM = slot_of(M, K, P.NT);
  float* B = P.W + sM * (long long)NB * NB;
  const float* L = P.W + slot_of(K, K, P.NT) * (long long)NB * NB;
  op_trsm<float>(L, NB, B + r0, NB, m, ncols, sm);
  // low-precision row-major copy with one power-of-two exponent per row: two threads per row,
  // column halves; loads coalesced across rows (column-major tile), 16-byte row-major stores
  __shared__ float s_half_max[kThr];
  const int t = threadIdx.x, i = t & (kBlk - 1), half = t >> 7;  // 128 rows x 2 halves
  const int r = r0 + i;
  const int cbeg = half * (NB / 2), cend = cbeg + NB / 2;
  float mx = 0.f;
  if (i < m)
    for (int c = cbeg; c < cend && c < ncols; ++c) mx = fmaxf(mx, fabsf(__ldcg(B + r + (long long)c * NB)));
  s_half_max[t] = mx;
  __syncthreads();
  mx = fmaxf(s_half_max[i], s_half_max[i + kBlk]);
  int e = 0;
  if (mx > 0.f) frexpf(mx, &e);  // mx * 2^-e in [0.5, 1)
  const float inv = pow2f(-e);
  if (i < m) {
    const long long base = sM * (long long)NB * NB + (long long)r * NB;
    for (int c0 = cbeg; c0 < cend; c0 += 8) {
      float v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = (c0 + j < ncols) ? __ldcg(B + r + (long long)(c0 + j) * NB) * inv : 0.f;
      uint4 pk;
      uint32_t* w = (uint32_t*)&pk;
      if (P.f16) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          __half2 h = __floats2half2_rn(v[2 * j], v[2 * j + 1]);
          w[j] = *(uint32_t*)&h;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
          w[j] = *(uint32_t*)&h;
        }
      }
      *(uint4*)((uint16_t*)P.Lb + base + c0) = pk;
    }
    if (half == 0) P.rowexp[sM * NB + r] = e;
  }
  __syncthreads();
}

// ---- the persistent kernel ------------------------------------------------------------------------
__global__ void __launch_bounds__(kThr, 1)
    potrf_mixed_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, Params P) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ long long s_task;
  __shared__ int s_go, s_info;
  __shared__ float s_colscale[kSubN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&done_bar), 1);
    mbar_fence_init();
  }
  if (warp == 1) tmem_alloc(smem_u32(&tmem_slot), kSubN);
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int NB = P.NB, NT = P.NT;
  const int nkb = NB / kBK;
  uint32_t prod_it = 0, cons_it = 0, acc_phase = 0;  // pipeline positions, identical in every role
  int* err = &P.st->status;

  for (;;) {
    __syncthreads();  // every thread has read the previous task index before it is overwritten
    if (threadIdx.x == 0) {
      long long t = -1;
      if (!ld_volatile(&P.st->abort)) t = (long long)atomicAdd(&P.st->head, 1ULL);
      s_task = (t >= 0 && t < P.ntasks) ? t : -1;
    }
    __syncthreads();
    const long long t = s_task;
    if (t < 0) break;
    const TileKey tk = decode(t / P.sub_g, NT);
    const int sub = (int)(t % P.sub_g);
    const int nsub = tk.type == T_POTRF ? 1 : tk.type == T_TRSM ? P.sub_t : tk.type == T_SYRK ? P.sub_s : P.sub_g;
    if (sub >= nsub) continue;  // unused slot of a task with fewer sub-tasks (uniform across the CTA)
    int* target = nullptr;
    if (threadIdx.x == 0) {
      bool ok = true;
      const int Sg = P.sub_g, St = P.sub_t, Ss = P.sub_s;
      switch (tk.type) {
        case T_POTRF:
          ok = wait_geq(P.cnt + tri_index(tk.a, tk.a, NT), Ss * tk.a, P.st, P.timeout_ns);
          break;
        case T_TRSM:
          ok = wait_geq(P.cnt + tri_index(tk.b, tk.b, NT), Ss * tk.b + 1, P.st, P.timeout_ns) &&
               wait_geq(P.cnt + tri_index(tk.a, tk.b, NT), Sg * tk.b, P.st, P.timeout_ns);
          break;
        case T_SYRK:
          ok = wait_geq(P.cnt + tri_index(tk.b, tk.a, NT), Sg * tk.a + St, P.st, P.timeout_ns) &&
               wait_geq(P.cnt + tri_index(tk.b, tk.b, NT), Ss * tk.a, P.st, P.timeout_ns);
          break;
        default:
          ok = wait_geq(P.cnt + tri_index(tk.a, tk.c, NT), Sg * tk.c + St, P.st, P.timeout_ns) &&
               wait_geq(P.cnt + tri_index(tk.b, tk.c, NT), Sg * tk.c + St, P.st, P.timeout_ns) &&
               wait_geq(P.cnt + tri_index(tk.a, tk.b, NT), Sg * tk.c, P.st, P.timeout_ns);
          break;
      }
      s_go = ok;
    }
    __syncthreads();
    if (!s_go) break;
    const uint64_t t_start = P.trace.buf ? globaltimer_ns() : 0;

    if (tk.type == T_POTRF) {
      const int info = task_potrf(P, tk.a, (float*)smem);
      if (threadIdx.x == 0) s_info = info;
      __syncthreads();
      if (s_info) {
        if (threadIdx.x == 0) {
          atomicCAS(&P.st->status, 0, tk.a * NB + s_info);
          atomicExch(&P.st->abort, 1);
        }
        break;
      }
      target = P.cnt + tri_index(tk.a, tk.a, NT);
    } else if (tk.type == T_TRSM) {
      task_trsm(P, tk.a, tk.b, sub, (float*)smem);
      target = P.cnt + tri_index(tk.a, tk.b, NT);
    } else {
      // tensor-core update of a 128 x 256 sub-tile of C = W(M,N) with L(M,K) L(N,K)^T
      int M, Nn, K, si, sj;
      if (tk.type == T_SYRK) {
        K = tk.a;
        M = Nn = tk.b;
        syrk_sub(sub, NB, si, sj);
      } else {
        M = tk.a;
        Nn = tk.b;
        K = tk.c;
        si = sub / (NB / kSubN);
        sj = sub % (NB / kSubN);
      }
      const int r0 = si * kSubM, c0 = sj * kSubN;
      const long long sA = slot_of(M, K, NT), sB = slot_of(Nn, K, NT), sC = slot_of(M, Nn, NT);
      if (warp == 0 && lane == 0) {
        // operands were written by other CTAs with ordinary stores: order them before the async-proxy reads
        asm volatile("fence.proxy.async.global;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // smem last written by SIMT tasks
        for (int kb = 0; kb < nkb; ++kb, ++prod_it) {
          const int s = prod_it % kStages;
          const uint32_t ph = (prod_it / kStages) & 1;
          if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1, err, P.timeout_ns)) break;
          const uint32_t dst = smem_u32(smem + (size_t)s * kStageBytes);
          mbar_arrive_expect_tx(smem_u32(&full_bar[s]), kStageBytes);
          tma_load_2d(dst, &tmA, smem_u32(&full_bar[s]), kb * kBK, (int)(sA * NB + r0));
          tma_load_2d(dst + kABytes, &tmB, smem_u32(&full_bar[s]), kb * kBK, (int)(sB * NB + c0));
        }
      } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_f16(kSubM, kSubN, !P.f16);
        for (int kb = 0; kb < nkb; ++kb, ++cons_it) {
          const int s = cons_it % kStages;
          const uint32_t ph = (cons_it / kStages) & 1;
          if (!mbar_wait(smem_u32(&full_bar[s]), ph, err, P.timeout_ns)) break;
          tc_fence_after();
          const uint32_t a_base = smem_u32(smem + (size_t)s * kStageBytes);
          const uint64_t ad = desc_kmajor_sw128(a_base), bd = desc_kmajor_sw128(a_base + kABytes);
#pragma unroll
          for (int k = 0; k < kBK / 16; ++k) umma_f16(tmem, ad + 2 * k, bd + 2 * k, idesc, (kb | k) != 0 ? 1u : 0u);
          umma_commit(smem_u32(&empty_bar[s]));
        }
        umma_commit(smem_u32(&done_bar));
      } else if (warp >= 4) {
        const int q = warp & 3;
        const int r = r0 + q * 32 + lane;  // row of C handled by this thread
        const int mrows = tdim(M, P), ncols = tdim(Nn, P);
        float* C = P.W + sC * (long long)NB * NB;
        // while the MMAs run: column scales of this sub-tile into shared memory, C lines into L2
        for (int c = (warp - 4) * 32 + lane; c < kSubN; c += 128)
          s_colscale[c] = (c0 + c < ncols) ? pow2f(__ldcg(P.rowexp + sB * NB + c0 + c)) : 0.f;
        if (r0 + q * 32 < mrows)
          for (int c = lane; c < kSubN && c0 + c < ncols; c += 32)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(C + (r0 + q * 32) + (long long)(c0 + c) * NB));
        asm volatile("bar.sync 1, 128;" ::: "memory");  // the four epilogue warps
        const float rscale = (r < mrows) ? pow2f(__ldcg(P.rowexp + sA * NB + r)) : 0.f;
        const bool row_ok = r < mrows;
        const bool syrk = tk.type == T_SYRK;
        if (mbar_wait(smem_u32(&done_bar), acc_phase, err, P.timeout_ns)) {
          tc_fence_after();
          float cur[16], nxt[16];
          auto load16 = [&](float (&dst)[16], int c) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int col = c0 + c + j;
              dst[j] = (row_ok && col < ncols) ? __ldcg(C + r + (long long)col * NB) : 0.f;
            }
          };
          load16(cur, 0);
          for (int c = 0; c < kSubN; c += 16) {
            uint32_t v[16];
            tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, v);
            if (c + 16 < kSubN) load16(nxt, c + 16);  // next chunk's loads are in flight during this chunk
            tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int col = c0 + c + j;
              if (row_ok && col < ncols && (!syrk || r >= col))
                __stcg(C + r + (long long)col * NB, cur[j] - __uint_as_float(v[j]) * (rscale * s_colscale[c + j]));
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) cur[j] = nxt[j];
          }
        }
      } else {
        // warps 2 and 3 (and the idle lanes of warps 0 and 1) skip the tensor part
      }
      if (warp == 0 && lane != 0) prod_it += nkb;
      if (warp != 0) prod_it += nkb;
      if (warp == 1 && lane != 0) cons_it += nkb;
      if (warp != 1) cons_it += nkb;
      acc_phase ^= 1;
      tc_fence_before();
      target = P.cnt + tri_index(M, Nn, NT);
    }
    __syncthreads();
    if (threadIdx.x == 0 && target) {
      signal_done(target);
      trace_record(P.trace, t_start, tk.type, tk.a, tk.b, tk.c, sub);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, kSubN);
  }
}

// W = fp32(A) on every tile slot
__global__ void convert_kernel(const double* __restrict__ A, float* __restrict__ W, long long n_elems) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n_elems; e += stride) W[e] = (float)A[e];
}
// diagonal of every diagonal tile scaled by (1 + shift): the shifted matrix factorised when the
// unshifted one breaks down in low precision
__global__ void shift_diag_kernel(float* W, int N, int NB, int NT, float shift) {
  const int K = blockIdx.x;
  const long long slot = (long long)K * NT - (long long)K * (K - 1) / 2;
  const int n = K == NT - 1 ? N - (NT - 1) * NB : NB;
  for (int i = threadIdx.x; i < n; i += blockDim.x) W[slot * NB * NB + i + (long long)i * NB] *= 1.f + shift;
}

struct Ws {  // workspace layout
  size_t state, cnt, cond, rowexp, lb, total;
};
inline Ws layout(int N, int NB) {
  const int NT = (N + NB - 1) / NB;
  const size_t nslots = (size_t)NT * (NT + 1) / 2;
  Ws w;
  w.state = 0;
  w.cnt = sizeof(DagState);
  w.cond = w.cnt + (((size_t)nslots * sizeof(int) + 255) / 256) * 256;
  w.rowexp = w.cond + 256;
  w.lb = w.rowexp + (((nslots * NB * sizeof(int)) + 1023) / 1024) * 1024;
  w.total = w.lb + nslots * (size_t)NB * NB * 2;
  return w;
}

std::mutex g_mtx;
bool g_attr = false;
int g_sms = 0;

}  // namespace mixed
}  // namespace gbx

using namespace gbx;
using namespace gbx::mixed;

extern "C" int gbx_potrf_mixed_bufferSize(int N, int NB, size_t* bytes) {
  if (N <= 0 || NB <= 0 || NB % 256 || NB > 1024 || !bytes) return GBX_ERR_ARG;
  *bytes = layout(N, NB).total;
  return GBX_OK;
}

extern "C" int gbx_potrf_mixed(int N, int NB, const double* A, float* W, int prec, double shift, void* work,
                               size_t work_bytes, void* stream) {
  if (N <= 0 || NB <= 0 || NB % 256 || NB > 1024 || !A || !W || !work || (prec != 0 && prec != 1))
    return GBX_ERR_ARG;
  const Ws w = layout(N, NB);
  if (work_bytes < w.total) return GBX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const int NT = (N + NB - 1) / NB;
  const long long nslots = (long long)NT * (NT + 1) / 2;
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    if (!g_attr) {
      int dev = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBX_ERR_CUDA;
      if (cudaFuncSetAttribute(potrf_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes) !=
          cudaSuccess)
        return GBX_ERR_CUDA;
      g_attr = true;
    }
  }
  char* base = (char*)work;
  if (cudaMemsetAsync(base, 0, w.rowexp, s) != cudaSuccess) return GBX_ERR_CUDA;  // state, counters, cond
  if (cudaMemsetAsync(base + w.lb, 0, w.total - w.lb, s) != cudaSuccess) return GBX_ERR_CUDA;
  const long long nel = nslots * (long long)NB * NB;
  convert_kernel<<<g_sms * 8, 256, 0, s>>>(A, W, nel);
  if (shift != 0.0) shift_diag_kernel<<<NT, 256, 0, s>>>(W, N, NB, NT, (float)shift);
  CUtensorMap ta, tb;
  const bool bf16 = prec == 0;
  if (int e = tc::make_tmap_kmajor_16b(&ta, base + w.lb, (uint64_t)nslots * NB, (uint64_t)NB, (uint64_t)NB, kSubM, bf16))
    return e;
  if (int e = tc::make_tmap_kmajor_16b(&tb, base + w.lb, (uint64_t)nslots * NB, (uint64_t)NB, (uint64_t)NB, kSubN, bf16))
    return e;
  Params P;
  P.W = W;
  P.Lb = base + w.lb;
  P.rowexp = (int*)(base + w.rowexp);
  P.N = N;
  P.NB = NB;
  P.NT = NT;
  P.f16 = prec == 1;
  P.sub_g = (NB / kSubM) * (NB / kSubN);
  P.sub_t = NB / kSubM;
  int ss = 0;
  for (int j = 0; j < NB / kSubN; ++j)
    for (int i = 0; i < NB / kSubM; ++i)
      if (kSubN * j < kSubM * (i + 1)) ++ss;
  P.sub_s = ss;
  P.ntasks = num_tile_tasks(NT) * P.sub_g;
  P.st = (DagState*)base;
  P.cnt = (int*)(base + w.cnt);
  P.cond_est = (float*)(base + w.cond);
  P.timeout_ns = gbx_get_wait_timeout_ns();
  P.trace = current_trace();
  potrf_mixed_kernel<<<g_sms, kThr, kSmemBytes, s>>>(ta, tb, P);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

extern "C" int gbx_potrf_mixed_info(const void* work, int N, int NB, float* cond_est, void* stream) {
  if (!work || N <= 0 || NB <= 0) return GBX_ERR_ARG;
  const Ws w = layout(N, NB);
  int st = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&st, work, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return GBX_ERR_CUDA;
  float c = 0.f;
  if (cudaMemcpyAsync(&c, (const char*)work + w.cond, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return GBX_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  if (cond_est) *cond_est = c;
  return st;
}
