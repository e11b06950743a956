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
#include <cuda_fp8.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <vector>

#include "block_ops.cuh"
#include "gbx_common.cuh"
#include "gbx_potrf.h"
#include "tc_common.cuh"

namespace gbx {
namespace tc {
int make_tmap_kmajor_16b(CUtensorMap* map, const void* base, uint64_t rows, uint64_t k, uint64_t ld, uint32_t box_rows,
                         bool bf16);
int make_tmap_kmajor_8b(CUtensorMap* map, const void* base, uint64_t rows, uint64_t k, uint64_t ld, uint32_t box_rows);
}

namespace mixed {

using namespace gbx::tc;

constexpr int kThr = 256;            // 8 warps: 0 TMA, 1 MMA, 4..7 epilogue (tensor tasks); all (SIMT tasks)
constexpr int kSubM = 128, kSubN = 256, kBK = 64, kStages = 4;
constexpr int kTrsmRows = 64;   // rows of a TRSM sub-task
constexpr int kMaxNB = 512;     // largest tile of the mixed path (the TRSM block lives in shared memory)
constexpr uint32_t kABytes = kSubM * kBK * 2, kBBytes = kSubN * kBK * 2, kStageBytes = kABytes + kBBytes;
constexpr size_t kTcSmem = (size_t)kStages * kStageBytes;  // 192 KB (1024-aligned ring)
constexpr size_t kSimtSmem = (size_t)kBlk * kBlk * sizeof(float) + 64;
constexpr size_t kTrsmSmem = (size_t)(kMaxNB * kTrsmRows + 32 * kMaxNB) * sizeof(float);
constexpr size_t kSmemBytes = std::max(std::max(kTcSmem, kSimtSmem), kTrsmSmem) + 1024;

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

// one matrix of the launch: its tile slots start at slot0 of the concatenated W / Lb / rowexp
// arrays, its completion counters at cnt0
struct MixMat {
  long long slot0;
  int N, NT, cnt0, id;  // id: index into the per-matrix info / condition arrays
  int dcnt0;            // first counter of the diagonal tiles' 128-block counters (NT * nb * nb)
  int dt0;              // first diagonal tile in the per-diagonal-tile arrays (FP64 scratch, route)
};
// a run of consecutive queue positions [start, next segment's start) holding, `mult` slots each,
// the tile tasks task0.. of one matrix's own task order. Segments are ordered by phase (phase p of a matrix: its
// tasks from POTRF(p) up to POTRF(p+1)), then by matrix, so the matrices of a batch advance side by
// side; every matrix still sees its own tasks in its own order, which keeps in-order grabbing free
// of deadlock.
struct MixSeg {
  long long start, task0;  // first queue position, first tile task (in the matrix's own order)
  int mat, mult;           // matrix; queue slots per tile task in this segment
  int sub0, pad;           // sub-task of the first slot (one-slot segments of POTRF mini-tasks)
};

struct Params {
  TraceBuf trace;
  float* W;
  void* Lb;  // bf16 or fp16, row-major per tile
  int* rowexp;
  int NB;
  int f16;     // 1: fp16 operands, 0: bf16 (or fp8, below)
  int fp8;     // 1: fp8 e4m3 operands (row-major, one byte per entry, rows scaled into [128, 256))
  int sub_g;   // GEMM sub-tasks per tile = (NB/128)*(NB/256)
  int sub_t;   // TRSM sub-tasks per tile = NB/64
  int nb;      // 128-blocks per tile edge (the diagonal tile's POTRF is a mini flowgraph of them)
  int npot;    // mini-tasks of a POTRF: per panel p, the block POTRF, nb-1-p TRSMs, their updates
  int* dcnt;   // completion counters of the diagonal tiles' 128-blocks
  int sub_s;   // SYRK sub-tasks per tile (lower 128 x 256 sub-tiles)
  long long ntasks;  // sub-task slots of all matrices
  const MixMat* mats;
  int nmats;
  const MixSeg* segs;  // ordered by start
  int nsegs;
  DagState* st;
  int* cnt;
  int* minfo;       // per matrix: 0 or the first bad pivot (1-based, global row)
  float* cond_est;  // per matrix: max over diagonal tiles of (max L_ii / min L_ii)^2
  double* D64;      // FP64 scratch tile of every diagonal tile (FP64 route), NB x NB each
  int* route;       // per diagonal tile: 1 when its POTRF took the FP64 route
  int* nfp64;       // per matrix: diagonal tiles factorised in FP64
  float fp64_cond;  // diagonal-ratio threshold of the FP64 route (+inf: never)
  const int* dsel;  // per matrix (device): factorise only the matrices with dsel[id] != 0; null: all
  uint64_t timeout_ns;
};

// the matrix a task belongs to, as every thread of the CTA sees it
struct Cur {
  long long slot0;
  int N, NT, id, dt0;  // dt0: index of its first diagonal tile in the per-diagonal-tile arrays
  int* cnt;
};

__device__ __forceinline__ long long slot_of(int m, int n, int NT) {
  return (long long)n * NT - (long long)n * (n - 1) / 2 + (m - n);
}
__device__ __forceinline__ int tdim(int t, const Cur& c, int NB) { return t == c.NT - 1 ? c.N - (c.NT - 1) * NB : NB; }

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
// POTRF(K) as a right-looking flowgraph of 128-blocks inside the diagonal tile, one queue slot per
// mini-task, in an order in which every mini-task waits only on earlier ones:
//   for each panel p:  PF(p): block (p,p) := chol(block (p,p))
//                      PT(p,i), i > p: block (i,p) := block (i,p) L_pp^{-T}
//                      PU(p,i,j), i >= j > p: block (i,j) -= block (i,p) block (j,p)^T
// Block counter (i,j) counts its finished writers (PU of panels < j, then PT/PF of panel j).
struct Mini {
  int kind, p, i, j;  // kind 0 PF, 1 PT, 2 PU
};
__host__ __device__ inline int panel_minis(int nb, int p) { return 1 + (nb - 1 - p) + (nb - 1 - p) * (nb - p) / 2; }
__device__ inline Mini mini_decode(int sub, int nb) {
  int p = 0;
  while (sub >= panel_minis(nb, p)) sub -= panel_minis(nb, p++);
  if (sub == 0) return Mini{0, p, p, p};
  if (sub - 1 < nb - 1 - p) return Mini{1, p, p + sub, p};
  int u = sub - 1 - (nb - 1 - p), j = p + 1;  // pairs i >= j > p, column by column
  while (u >= nb - j) u -= nb - j++;
  return Mini{2, p, j + u, j};
}

// Route of a diagonal tile's POTRF, chosen by its first mini-task PF(0) from the tile after all its
// SYRK updates: FP64 when the tile's condition estimate max_i a_ii / min_i a_ii (a lower bound of its
// 2-norm condition number) exceeds P.fp64_cond, or when a diagonal entry is not positive; else FP32.
// The FP64 route copies the tile's lower triangle into its FP64 scratch tile, runs the same
// mini-flowgraph in FP64 there (op_potrf / op_trsm / op_gemm_nt<double>), and each block's final
// writer (PF(j) for block (j,j), PT(j,i) for block (i,j)) also rounds the block into W.
__device__ bool choose_fp64_route(const Params& P, const float* A, int n, float* sm) {
  float mn = 3.0e38f, mx = 0.f;
  for (int i = threadIdx.x; i < n; i += kThr) {
    const float d = __ldcg(A + i + (long long)i * P.NB);
    mn = fminf(mn, d);
    mx = fmaxf(mx, d);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sm[warp] = mn;
    sm[8 + warp] = mx;
  }
  __syncthreads();
  mn = sm[0];
  mx = sm[8];
  for (int w = 1; w < kThr / 32; ++w) {
    mn = fminf(mn, sm[w]);
    mx = fmaxf(mx, sm[8 + w]);
  }
  __syncthreads();
  return !(mn > 0.f) || mx > P.fp64_cond * mn;
}

// (the FP64 scratch is read through L2 only: other CTAs wrote it, and L1 is not coherent)
__device__ void round_block_to_w(const double* D, float* A, int ld, int di, int dj, bool diag) {
  for (int idx = threadIdx.x; idx < kBlk * dj; idx += kThr) {
    const int i = idx & (kBlk - 1), j = idx >> 7;
    if (i < di && (!diag || i >= j)) A[i + (long long)j * ld] = (float)__ldcg(D + i + (long long)j * ld);
  }
}

// FP64 route block operations: plain loops through L2 with few live registers. The route is for
// the rare ill-conditioned diagonal tile; the register-blocked FP64 block ops of the FP64 executor
// would raise the persistent kernel's register peak and make it spill in its FP32 and tensor paths.
// Blocks are column-major with leading dimension ld; n, m <= 128.
// Cholesky of the lower n x n block in shared memory (right-looking, column by column); returns 0
// or the 1-based index of the first non-positive pivot. S: 128 x 128 doubles.
__device__ int f64_block_potrf(double* A, int ld, int n, double* S) {
  __shared__ int s_info;
  if (threadIdx.x == 0) s_info = 0;
#pragma unroll 1
  for (int idx = threadIdx.x; idx < kBlk * n; idx += kThr) {
    const int i = idx & (kBlk - 1), j = idx >> 7;
    S[idx] = (i < n && i >= j) ? __ldcg(A + i + (long long)j * ld) : 0.0;
  }
  __syncthreads();
#pragma unroll 1
  for (int j = 0; j < n; ++j) {
    if (threadIdx.x == 0) {
      const double d = S[j + kBlk * j];
      if (!(d > 0.0)) s_info = j + 1;
      else S[j + kBlk * j] = sqrt(d);
    }
    __syncthreads();
    if (s_info) break;
    const double piv = S[j + kBlk * j];
#pragma unroll 1
    for (int i = j + 1 + threadIdx.x; i < n; i += kThr) S[i + kBlk * j] /= piv;
    __syncthreads();
    const int w = n - j - 1;
#pragma unroll 1
    for (int idx = threadIdx.x; idx < w * w; idx += kThr) {
      const int i = j + 1 + idx % w, k = j + 1 + idx / w;
      if (i >= k) S[i + kBlk * k] -= S[i + kBlk * j] * S[k + kBlk * j];
    }
    __syncthreads();
  }
  const int info = s_info;
#pragma unroll 1
  for (int idx = threadIdx.x; idx < kBlk * n; idx += kThr) {
    const int i = idx & (kBlk - 1), j = idx >> 7;
    if (i < n && i >= j) A[i + (long long)j * ld] = S[idx];
  }
  __syncthreads();
  return info;
}
// B(m x n) := B L^{-T} (L lower n x n): one thread per row, forward substitution in place
__device__ void f64_block_trsm(const double* L, int ld, double* B, int m, int n) {
  const int r = threadIdx.x;
  if (r < m) {
#pragma unroll 1
    for (int c = 0; c < n; ++c) {
      double x = __ldcg(B + r + (long long)c * ld);
#pragma unroll 1
      for (int k = 0; k < c; ++k) x -= __ldcg(B + r + (long long)k * ld) * __ldcg(L + c + (long long)k * ld);
      B[r + (long long)c * ld] = x / __ldcg(L + c + (long long)c * ld);
    }
  }
  __syncthreads();
}
// C(m x n) -= A(m x k) B(n x k)^T, lower part only when `lower`
__device__ void f64_block_gemm(const double* A, const double* B, double* C, int ld, int m, int n, int k, bool lower) {
#pragma unroll 1
  for (int idx = threadIdx.x; idx < m * n; idx += kThr) {
    const int i = idx % m, j = idx / m;
    if (lower && i < j) continue;
    double acc = 0.0;
#pragma unroll 4
    for (int q = 0; q < k; ++q) acc = fma(__ldcg(A + i + (long long)q * ld), __ldcg(B + j + (long long)q * ld), acc);
    C[i + (long long)j * ld] = __ldcg(C + i + (long long)j * ld) - acc;
  }
  __syncthreads();
}

// One mini-task of the FP64 route on the tile's FP64 scratch D (NB x NB, column-major); the final
// writer of a block also rounds it into W (A).
__device__ int potrf_mini_fp64(double* D, float* A, int NB, int n, const Mini& mk, double* sm) {
  auto blk = [&](int i, int j) { return A + kBlk * i + (long long)kBlk * j * NB; };
  auto dblk = [&](int i, int j) { return D + kBlk * i + (long long)kBlk * j * NB; };
  auto bdim = [&](int i) { return min(kBlk, n - kBlk * i); };
  const int dp = bdim(mk.p);
  if (dp <= 0) return 0;
  if (mk.kind == 0) {
    const int info = f64_block_potrf(dblk(mk.p, mk.p), NB, dp, sm);
    round_block_to_w(dblk(mk.p, mk.p), blk(mk.p, mk.p), NB, dp, dp, true);
    return info;
  }
  const int di = bdim(mk.i);
  if (di <= 0) return 0;
  if (mk.kind == 1) {
    f64_block_trsm(dblk(mk.p, mk.p), NB, dblk(mk.i, mk.p), di, dp);
    round_block_to_w(dblk(mk.i, mk.p), blk(mk.i, mk.p), NB, di, dp, false);
    return 0;
  }
  const int dj = bdim(mk.j);
  if (dj > 0) f64_block_gemm(dblk(mk.i, mk.p), dblk(mk.j, mk.p), dblk(mk.i, mk.j), NB, di, dj, dp, mk.i == mk.j);
  return 0;
}

// returns 0 or the 1-based pivot index within the block (PF only)
__device__ int task_potrf_mini(const Params& P, const Cur& cm, int K, const Mini& mk, float* sm) {
  const int NB = P.NB, n = tdim(K, cm, NB);
  float* A = P.W + (cm.slot0 + slot_of(K, K, cm.NT)) * (long long)NB * NB;
  double* D = P.D64 + (cm.dt0 + K) * (long long)NB * NB;  // the tile's FP64 scratch
  int* route = P.route + cm.dt0 + K;
  auto blk = [&](int i, int j) { return A + kBlk * i + (long long)kBlk * j * NB; };
  auto bdim = [&](int i) { return min(kBlk, n - kBlk * i); };  // <= 0: past the ragged edge
  const int dp = bdim(mk.p);
  __shared__ int s_route;
  if (mk.kind == 0 && mk.p == 0) {  // PF(0) decides the tile's route for every later mini-task
    const bool f64 = choose_fp64_route(P, A, n, sm);
    if (f64) {
      for (long long idx = threadIdx.x; idx < (long long)n * NB; idx += kThr) {
        const int i = (int)(idx % NB), j = (int)(idx / NB);
        if (i < n && i >= j) D[idx] = (double)__ldcg(A + idx);
      }
      if (threadIdx.x == 0) atomicAdd(P.nfp64 + cm.id, 1);
    }
    if (threadIdx.x == 0) {
      *(volatile int*)route = f64 ? 1 : 0;  // made visible with the block's completion signal
      s_route = f64;
    }
    __syncthreads();
  } else {
    if (threadIdx.x == 0) s_route = ld_volatile(route);  // PF(0) precedes every mini-task of the tile
    __syncthreads();
  }
  const bool f64 = s_route != 0;
  if (f64 && mk.kind != 0) {
    potrf_mini_fp64(D, A, NB, n, mk, (double*)sm);
    __syncthreads();
    return 0;
  }
  if (mk.kind == 0) {
    if (dp <= 0) return 0;
    const int info = f64 ? potrf_mini_fp64(D, A, NB, n, mk, (double*)sm) : op_potrf<float>(blk(mk.p, mk.p), NB, dp, sm);
    __syncthreads();
    if (info == 0 && threadIdx.x == 0) {  // condition estimate of the block from its factor's diagonal
      float mn = 3.0e38f, mx = 0.f;
      for (int i = 0; i < dp; ++i) {
        const float d = __ldcg(blk(mk.p, mk.p) + i + (long long)i * NB);
        mn = fminf(mn, d);
        mx = fmaxf(mx, d);
      }
      const float est = (mx / mn) * (mx / mn);
      atomicMax((int*)(P.cond_est + cm.id), __float_as_int(est));  // positive floats order like their bits
    }
    __syncthreads();
    return info;
  }
  if (mk.kind == 1) {
    const int di = bdim(mk.i);
    if (di > 0 && dp > 0) op_trsm<float>(blk(mk.p, mk.p), NB, blk(mk.i, mk.p), NB, di, dp, sm);
    return 0;
  }
  const int di = bdim(mk.i), dj = bdim(mk.j);
  if (di > 0 && dj > 0 && dp > 0)
    op_gemm_nt<float>(blk(mk.i, mk.p), NB, blk(mk.j, mk.p), NB, blk(mk.i, mk.j), NB, di, dj, dp, mk.i == mk.j, sm);
  return 0;
}

// TRSM(M, K) sub-task rb: rows 64 rb .. 64 rb + 63 of W(M,K) := W(M,K) L_KK^{-T}, then their scaled
// low-precision row-major copy. The 64 x NB block stays in shared memory for the whole solve:
// per 32-column panel, each of 64 threads solves its row in registers against the panel's
// triangle (column-wise substitution), then all 256 threads apply the panel to the columns right of
// it (right-looking rank-32 update, 4 x 8 register micro-tiles with 16-byte shared loads). The next
// panel of L is loaded into registers while the current one is solved and applied.
// smem: block [NB][64] + L panel [32][512] = 192 KB for NB = 512
__device__ void task_trsm(const Params& P, const Cur& cm, int M, int K, int rb, float* sm) {
  const int NB = P.NB, r0 = rb * kTrsmRows, mrows = tdim(M, cm, NB), n = tdim(K, cm, NB);
  if (r0 >= mrows) return;
  const int m = min(kTrsmRows, mrows - r0);
  const long long sM = cm.slot0 + slot_of(M, K, cm.NT);
  float* B = P.W + sM * (long long)NB * NB + r0;
  const float* L = P.W + (cm.slot0 + slot_of(K, K, cm.NT)) * (long long)NB * NB;
  float* Bs = sm;                      // Bs[c * 64 + r]
  float* Ls = sm + kMaxNB * kTrsmRows;  // Ls[c * 512 + ii] = L(p0 + ii, p0 + c)
  const int tid = threadIdx.x;
  // the block into shared memory: 16-byte loads, eight in flight per thread; rows past the
  // matrix edge are zero (the tile slot holds NB rows, so the loads stay inside it)
  for (int f0 = 0; f0 < n * (kTrsmRows / 4); f0 += 8 * kThr) {
    float4 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int f = f0 + u * kThr + tid, c = f >> 4, r4 = (f & 15) * 4;
      v[u] = f < n * (kTrsmRows / 4) ? __ldcg((const float4*)(B + r4 + (long long)c * NB)) : make_float4(0, 0, 0, 0);
      if (r4 + 0 >= m) v[u].x = 0.f;
      if (r4 + 1 >= m) v[u].y = 0.f;
      if (r4 + 2 >= m) v[u].z = 0.f;
      if (r4 + 3 >= m) v[u].w = 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int f = f0 + u * kThr + tid;
      if (f < n * (kTrsmRows / 4)) *(float4*)(Bs + 4 * f) = v[u];
    }
  }
  const int tr = tid & 15, tc = tid >> 4;  // update micro-tile: rows 4tr.., columns 8tc.. of a 128-column chunk
  // the panel's columns of L, rows p0.. : sixteen 16-byte loads per thread, issued one panel ahead
  // so that they are in flight during the previous panel's update (not during the solve, which
  // needs the registers); rows past the edge stay inside the tile slot and are never read back
  float4 pre[16];
  auto load_panel = [&](int q0) {
    const int qw = min(32, n - q0), qspan = n - q0;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int f = u * kThr + tid, c = f >> 7, ii = (f & 127) * 4;
      if (c < qw && ii < qspan) pre[u] = __ldcg((const float4*)(L + (q0 + ii) + (long long)(q0 + c) * NB));
    }
  };
  load_panel(0);
  for (int p0 = 0; p0 < n; p0 += 32) {
    const int pw = min(32, n - p0), span = n - p0;
    __syncthreads();  // the previous panel's update is complete
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int f = u * kThr + tid, c = f >> 7, ii = (f & 127) * 4;
      if (c < pw && ii < span) *(float4*)(Ls + c * kMaxNB + ii) = pre[u];
    }
    __syncthreads();
    if (tid < kTrsmRows) {
      float x[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) x[c] = c < pw ? Bs[(p0 + c) * kTrsmRows + tid] : 0.f;
      if (pw == 32)
        col_solve32(x, Ls, kMaxNB);
      else
        row_solve32<float>(x, Ls, kMaxNB, pw);
#pragma unroll
      for (int c = 0; c < 32; ++c)
        if (c < pw) Bs[(p0 + c) * kTrsmRows + tid] = x[c];
    }
    __syncthreads();
    if (p0 + 32 < n) load_panel(p0 + 32);  // in flight during this panel's update
    // Bs(:, p0+jj) -= Bs(:, p0:p0+pw) * L(p0+jj, p0:p0+pw)^T for jj in [pw, span), chunks of 128
    // columns; a thread owns rows 4tr..4tr+3 x columns jj..jj+7 (three 16-byte loads per 32 FMAs)
    for (int j0 = pw; j0 < span; j0 += 128) {
      const int jj = j0 + 8 * tc;
      if (jj >= span) continue;
      float acc[4][8];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
      if (pw == 32 && jj + 8 <= span) {
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
          float a[4], b0[4], b1[4];
          lds4(Bs + (p0 + k) * kTrsmRows + 4 * tr, a);
          lds4(Ls + k * kMaxNB + jj, b0);
          lds4(Ls + k * kMaxNB + jj + 4, b1);
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              acc[i][j] = fmaf(a[i], b0[j], acc[i][j]);
              acc[i][j + 4] = fmaf(a[i], b1[j], acc[i][j + 4]);
            }
        }
      } else {  // ragged panel or chunk edge
        for (int k = 0; k < pw; ++k) {
          float a[4], b[8];
          lds4(Bs + (p0 + k) * kTrsmRows + 4 * tr, a);
#pragma unroll
          for (int j = 0; j < 8; ++j) b[j] = jj + j < span ? Ls[k * kMaxNB + jj + j] : 0.f;
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
      }
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (jj + j < span)
#pragma unroll
          for (int i = 0; i < 4; ++i) Bs[(p0 + jj + j) * kTrsmRows + 4 * tr + i] -= acc[i][j];
    }
  }
  __syncthreads();
  for (int idx = tid; idx < n * kTrsmRows; idx += kThr) {  // the solved block back to W
    const int r = idx & (kTrsmRows - 1), c = idx >> 6;
    if (r < m) __stcg(B + r + (long long)c * NB, Bs[idx]);
  }
  // low-precision row-major copy with one power-of-two exponent per row: four threads per row,
  // column quarters, 16-byte row-major stores
  __shared__ float s_q_max[kThr];
  const int r = tid & (kTrsmRows - 1), q = tid >> 6;
  const int cbeg = q * (NB / 4), cend = cbeg + NB / 4;
  float mx = 0.f;
  for (int c = cbeg; c < cend && c < n; ++c) mx = fmaxf(mx, fabsf(Bs[c * kTrsmRows + r]));
  s_q_max[tid] = mx;
  __syncthreads();
  mx = fmaxf(fmaxf(s_q_max[r], s_q_max[r + 64]), fmaxf(s_q_max[r + 128], s_q_max[r + 192]));
  int e = 0;
  if (mx > 0.f) frexpf(mx, &e);  // mx * 2^-e in [0.5, 1)
  if (P.fp8) e -= 8;              // fp8: the row into [128, 256), inside e4m3's range (448)
  const float inv = pow2f(-e);
  if (r < m) {
    const long long base = sM * (long long)NB * NB + (long long)(r0 + r) * NB;
    for (int c0 = cbeg; c0 < cend; c0 += 8) {
      float v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = (c0 + j < n) ? Bs[(c0 + j) * kTrsmRows + r] * inv : 0.f;
      if (P.fp8) {  // one byte per entry, rows of NB bytes
        uint2 p8;
        uint16_t* w8 = (uint16_t*)&p8;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          w8[j] = __nv_cvt_float2_to_fp8x2(make_float2(v[2 * j], v[2 * j + 1]), __NV_SATFINITE, __NV_E4M3);
        *(uint2*)((uint8_t*)P.Lb + base + c0) = p8;
        continue;
      }
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
    if (q == 0) P.rowexp[sM * NB + r0 + r] = e;
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
  __shared__ long long s_task, s_slot0;
  __shared__ int s_go, s_info, s_N, s_NT, s_cnt0, s_id, s_dcnt0, s_sub, s_dt0;
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
  const int NB = P.NB;
  const int kbk = P.fp8 ? 2 * kBK : kBK;  // elements per 128-byte operand row of a stage
  const int nkb = NB / kbk;
  uint32_t prod_it = 0, cons_it = 0, acc_phase = 0;  // pipeline positions, identical in every role
  int* err = &P.st->status;

  for (;;) {
    __syncthreads();  // every thread has read the previous task index before it is overwritten
    if (threadIdx.x == 0) {
      long long t = -1;
      if (!ld_volatile(&P.st->abort)) t = (long long)atomicAdd(&P.st->head, 1ULL);
      if (t >= 0 && t < P.ntasks) {
        int lo = 0, hi = P.nsegs - 1;  // last segment with start <= t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (P.segs[mid].start <= t) lo = mid;
          else hi = mid - 1;
        }
        const MixSeg sg = P.segs[lo];
        const MixMat mm = P.mats[sg.mat];
        s_task = sg.task0 + (t - sg.start) / sg.mult;
        s_sub = sg.sub0 + (int)((t - sg.start) % sg.mult);
        s_dcnt0 = mm.dcnt0;
        s_slot0 = mm.slot0;
        s_N = mm.N;
        s_NT = mm.NT;
        s_cnt0 = mm.cnt0;
        s_id = mm.id;
        s_dt0 = mm.dt0;
        // a matrix not selected for this launch: its whole task graph is skipped (tasks of one
        // matrix wait only on the same matrix's counters)
        if (P.dsel && !P.dsel[mm.id]) s_task = -2;
      } else {
        s_task = -1;
      }
    }
    __syncthreads();
    const long long t = s_task;
    if (t == -2) continue;
    if (t < 0) break;
    Cur cm;
    cm.slot0 = s_slot0;
    cm.N = s_N;
    cm.NT = s_NT;
    cm.id = s_id;
    cm.dt0 = s_dt0;
    cm.cnt = P.cnt + s_cnt0;
    const int NT = cm.NT;
    const TileKey tk = decode(t, NT);
    const int sub = s_sub;
    const int nsub =
        tk.type == T_POTRF ? P.npot : tk.type == T_TRSM ? P.sub_t : tk.type == T_SYRK ? P.sub_s : P.sub_g;
    if (sub >= nsub) continue;  // unused slot of a task with fewer sub-tasks (uniform across the CTA)
    Mini mk{0, 0, 0, 0};
    int* dc = nullptr;  // the diagonal tile's block counters (POTRF mini-tasks)
    if (tk.type == T_POTRF) {
      mk = mini_decode(sub, P.nb);
      dc = P.dcnt + s_dcnt0 + (long long)tk.a * P.nb * P.nb;
    }
    int* target = nullptr;
    int* target2 = nullptr;  // the tile counter, moved by the last mini-task of a POTRF
    if (threadIdx.x == 0) {
      bool ok = true;
      const int Sg = P.sub_g, St = P.sub_t, Ss = P.sub_s;
      int* cnt = cm.cnt;
      switch (tk.type) {
        case T_POTRF: {
          const int nb = P.nb;
          ok = wait_geq(cnt + tri_index(tk.a, tk.a, NT), Ss * tk.a, P.st, P.timeout_ns);
          if (mk.kind == 0)
            ok = ok && wait_geq(dc + mk.p * nb + mk.p, mk.p, P.st, P.timeout_ns);
          else if (mk.kind == 1)
            ok = ok && wait_geq(dc + mk.p * nb + mk.p, mk.p + 1, P.st, P.timeout_ns) &&
                 wait_geq(dc + mk.i * nb + mk.p, mk.p, P.st, P.timeout_ns);
          else
            ok = ok && wait_geq(dc + mk.i * nb + mk.p, mk.p + 1, P.st, P.timeout_ns) &&
                 wait_geq(dc + mk.j * nb + mk.p, mk.p + 1, P.st, P.timeout_ns) &&
                 wait_geq(dc + mk.i * nb + mk.j, mk.p, P.st, P.timeout_ns);
          break;
        }
        case T_TRSM:
          ok = wait_geq(cnt + tri_index(tk.b, tk.b, NT), Ss * tk.b + 1, P.st, P.timeout_ns) &&
               wait_geq(cnt + tri_index(tk.a, tk.b, NT), Sg * tk.b, P.st, P.timeout_ns);
          break;
        case T_SYRK:
          ok = wait_geq(cnt + tri_index(tk.b, tk.a, NT), Sg * tk.a + St, P.st, P.timeout_ns) &&
               wait_geq(cnt + tri_index(tk.b, tk.b, NT), Ss * tk.a, P.st, P.timeout_ns);
          break;
        default:
          ok = wait_geq(cnt + tri_index(tk.a, tk.c, NT), Sg * tk.c + St, P.st, P.timeout_ns) &&
               wait_geq(cnt + tri_index(tk.b, tk.c, NT), Sg * tk.c + St, P.st, P.timeout_ns) &&
               wait_geq(cnt + tri_index(tk.a, tk.b, NT), Sg * tk.c, P.st, P.timeout_ns);
          break;
      }
      s_go = ok ? (ld_volatile(P.minfo + cm.id) ? 2 : 1) : 0;  // 2: the matrix already failed, skip the work
    }
    __syncthreads();
    if (!s_go) break;
    if (s_go == 2) {  // a failed matrix: keep its counters moving so that its later tasks never wait
      __syncthreads();
      if (threadIdx.x == 0) {
        int* c = cm.cnt;
        if (tk.type == T_POTRF) {
          signal_done(dc + mk.i * P.nb + mk.j);
          if (mk.kind == 0 && mk.p == P.nb - 1) signal_done(c + tri_index(tk.a, tk.a, NT));
        } else if (tk.type == T_TRSM) signal_done(c + tri_index(tk.a, tk.b, NT));
        else if (tk.type == T_SYRK) signal_done(c + tri_index(tk.b, tk.b, NT));
        else signal_done(c + tri_index(tk.a, tk.b, NT));
      }
      continue;
    }
    const uint64_t t_start = P.trace.buf ? globaltimer_ns() : 0;

    if (tk.type == T_POTRF) {
      const int info = task_potrf_mini(P, cm, tk.a, mk, (float*)smem);
      if (threadIdx.x == 0) s_info = info;
      __syncthreads();
      if (s_info) {
        const int piv = tk.a * NB + kBlk * mk.p + s_info;  // 1-based row of the matrix
        if (P.nmats == 1) {  // one matrix: stop the whole launch
          if (threadIdx.x == 0) {
            atomicCAS(P.minfo + cm.id, 0, piv);
            atomicCAS(&P.st->status, 0, piv);
            atomicExch(&P.st->abort, 1);
          }
          break;
        }
        if (threadIdx.x == 0) atomicCAS(P.minfo + cm.id, 0, piv);  // others go on
      }
      target = dc + mk.i * P.nb + mk.j;
      if (mk.kind == 0 && mk.p == P.nb - 1) target2 = cm.cnt + tri_index(tk.a, tk.a, NT);
    } else if (tk.type == T_TRSM) {
      task_trsm(P, cm, tk.a, tk.b, sub, (float*)smem);
      target = cm.cnt + tri_index(tk.a, tk.b, NT);
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
      const long long sA = cm.slot0 + slot_of(M, K, NT), sB = cm.slot0 + slot_of(Nn, K, NT),
                      sC = cm.slot0 + slot_of(M, Nn, NT);
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
          tma_load_2d(dst, &tmA, smem_u32(&full_bar[s]), kb * kbk, (int)(sA * NB + r0));
          tma_load_2d(dst + kABytes, &tmB, smem_u32(&full_bar[s]), kb * kbk, (int)(sB * NB + c0));
        }
      } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_f16(kSubM, kSubN, !P.f16 && !P.fp8);  // e4m3: format fields 0 as for fp16
        for (int kb = 0; kb < nkb; ++kb, ++cons_it) {
          const int s = cons_it % kStages;
          const uint32_t ph = (cons_it / kStages) & 1;
          if (!mbar_wait(smem_u32(&full_bar[s]), ph, err, P.timeout_ns)) break;
          tc_fence_after();
          const uint32_t a_base = smem_u32(smem + (size_t)s * kStageBytes);
          const uint64_t ad = desc_kmajor_sw128(a_base), bd = desc_kmajor_sw128(a_base + kABytes);
          // four instructions per 128-byte stage row: K = 16 (16-bit) or 32 (fp8), 32 bytes each
          if (P.fp8) {
#pragma unroll
            for (int k = 0; k < 4; ++k) umma_f8(tmem, ad + 2 * k, bd + 2 * k, idesc, (kb | k) != 0 ? 1u : 0u);
          } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) umma_f16(tmem, ad + 2 * k, bd + 2 * k, idesc, (kb | k) != 0 ? 1u : 0u);
          }
          umma_commit(smem_u32(&empty_bar[s]));
        }
        umma_commit(smem_u32(&done_bar));
      } else if (warp >= 4) {
        // while the MMAs run: column scales of this sub-tile into shared memory, C lines into L2
        const int ncols = tdim(Nn, cm, NB), mrows = tdim(M, cm, NB);
        const float* C = P.W + sC * (long long)NB * NB;
        const int q = warp & 3;
        for (int c = (warp - 4) * 32 + lane; c < kSubN; c += 128)
          s_colscale[c] = (c0 + c < ncols) ? pow2f(__ldcg(P.rowexp + sB * NB + c0 + c)) : 0.f;
        if (r0 + q * 32 < mrows)
          for (int c = lane; c < kSubN && c0 + c < ncols; c += 32)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(C + (r0 + q * 32) + (long long)(c0 + c) * NB));
      }
      __syncwarp();
      __syncthreads();  // column scales ready; warps 0 and 1 have issued their last TMA / MMA
      {
        // epilogue on all eight warps: warp w reads TMEM lanes 32 (w % 4) .. (its rows) for one half
        // of the 256 columns; C := C - (A B^T) scaled by the rows' and columns' powers of two
        const int q = warp & 3, h = warp >> 2;
        const int r = r0 + q * 32 + lane;  // row of C handled by this thread
        const int mrows = tdim(M, cm, NB), ncols = tdim(Nn, cm, NB);
        float* C = P.W + sC * (long long)NB * NB;
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
          const int cb = h * (kSubN / 2), ce = cb + kSubN / 2;
          load16(cur, cb);
          for (int c = cb; c < ce; c += 16) {
            uint32_t v[16];
            tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, v);
            if (c + 16 < ce) load16(nxt, c + 16);  // next chunk's loads are in flight during this chunk
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
      }
      if (warp == 0 && lane != 0) prod_it += nkb;
      if (warp != 0) prod_it += nkb;
      if (warp == 1 && lane != 0) cons_it += nkb;
      if (warp != 1) cons_it += nkb;
      acc_phase ^= 1;
      tc_fence_before();
      target = cm.cnt + tri_index(M, Nn, NT);
    }
    __syncthreads();
    if (threadIdx.x == 0 && target) {
      trace_record(P.trace, t_start, tk.type, tk.a, tk.b, tk.c, sub);  // end stamp before any waiter can start
      signal_done(target);
      if (target2) signal_done(target2);
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

// workspace layout for a batch (one matrix is the batch of one): run state, completion counters,
// per-matrix condition estimates and info, the matrix table, row exponents, low-precision copies
struct Ws {
  size_t state, cnt, dcnt, cond, minfo, nfp64, route, mats, segs, sel, rowexp, lb, d64, total;
  long long slots, cnts, nsegs, dcnts, dtiles;
};
inline size_t up(size_t x, size_t a) { return (x + a - 1) / a * a; }
int npot_of(int NB) {  // mini-tasks of one POTRF
  const int nb = NB / kBlk;
  int c = 0;
  for (int p = 0; p < nb; ++p) c += panel_minis(nb, p);
  return c;
}
inline Ws layout_batch(int batch, const int* n, int NB) {
  long long slots = 0, nsegs = 0, dcnts = 0, dtiles = 0;
  const long long nb = NB / kBlk;
  for (int k = 0; k < batch; ++k) {
    const long long nt = (n[k] + NB - 1) / NB;
    slots += nt * (nt + 1) / 2;
    nsegs += (4 + npot_of(NB)) * nt;  // queue segments: per phase, three groups + POTRF mini-tasks
    dcnts += nt * nb * nb;
    dtiles += nt;
  }
  Ws w;
  w.nsegs = nsegs;
  w.slots = slots;
  w.cnts = slots;  // one counter per tile
  w.dcnts = dcnts;
  w.dtiles = dtiles;
  w.state = 0;
  w.cnt = sizeof(DagState);
  w.dcnt = up(w.cnt + (size_t)w.cnts * sizeof(int), 256);
  w.cond = up(w.dcnt + (size_t)w.dcnts * sizeof(int), 256);
  w.minfo = up(w.cond + (size_t)batch * sizeof(float), 256);
  w.nfp64 = up(w.minfo + (size_t)batch * sizeof(int), 256);
  w.route = up(w.nfp64 + (size_t)batch * sizeof(int), 256);
  w.mats = up(w.route + (size_t)dtiles * sizeof(int), 256);
  w.segs = up(w.mats + (size_t)batch * sizeof(MixMat), 256);
  w.sel = up(w.segs + (size_t)nsegs * sizeof(MixSeg), 256);
  w.rowexp = up(w.sel + (size_t)batch * sizeof(int), 1024);
  w.lb = up(w.rowexp + (size_t)slots * NB * sizeof(int), 1024);
  w.d64 = up(w.lb + (size_t)slots * NB * NB * 2, 256);
  w.total = w.d64 + (size_t)dtiles * NB * NB * sizeof(double);
  return w;
}
inline Ws layout(int N, int NB) { return layout_batch(1, &N, NB); }

int sub_syrk(int NB) {
  int ss = 0;
  for (int j = 0; j < NB / kSubN; ++j)
    for (int i = 0; i < NB / kSubM; ++i)
      if (kSubN * j < kSubM * (i + 1)) ++ss;
  return ss;
}

std::mutex g_mtx;
bool g_attr = false;
int g_sms = 0;

}  // namespace mixed
}  // namespace gbx

using namespace gbx;
using namespace gbx::mixed;

namespace gbx {
namespace mixed {
// Host side of a batched launch in two parts.
// plan_batch: the matrix table and the queue segments of every matrix of the batch, uploaded into
//   the workspace (host to device copies; not capturable).
// run_batch: clears the run state and counters and launches the persistent kernel over the planned
//   queue (no host synchronisation, no host to device copy: capturable in a CUDA graph). dsel
//   (device, per matrix, may be null) selects the matrices to factorise; the others' tasks are
//   skipped. W must already hold the (shifted) FP32 copy of every selected matrix.
// A, W: the matrices' tile-major lower storage concatenated in batch order (matrix k's slots follow
// matrix k-1's). The queue puts larger matrices first so the longest critical paths start first.
struct Shape {
  int sub_g, sub_t, sub_s, nslot, nb, npot;
  long long ntasks, nsegs;
};
Shape shape_of(int batch, const int* n, int NB) {
  Shape h;
  h.sub_g = (NB / kSubM) * (NB / kSubN);
  h.sub_t = NB / kTrsmRows;
  h.sub_s = sub_syrk(NB);
  h.nslot = std::max(std::max(h.sub_g, h.sub_t), h.sub_s);
  h.nb = NB / kBlk;
  h.npot = npot_of(NB);
  h.ntasks = 0;
  h.nsegs = 0;
  for (int k = 0; k < batch; ++k) {  // queue slots of a matrix: one per POTRF mini-task, nslot per other task
    const long long nt = (n[k] + NB - 1) / NB;
    h.ntasks += nt * h.npot + (num_tile_tasks((int)nt) - nt) * h.nslot;
  }
  return h;
}

int set_kernel_attrs() {
  std::lock_guard<std::mutex> lk(g_mtx);
  if (g_attr) return GBX_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBX_ERR_CUDA;
  if (cudaFuncSetAttribute(potrf_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes) !=
      cudaSuccess)
    return GBX_ERR_CUDA;
  g_attr = true;
  return GBX_OK;
}

int plan_batch(int batch, const int* n, int NB, void* work, size_t work_bytes, cudaStream_t s, int sched) {
  const Ws w = layout_batch(batch, n, NB);
  if (work_bytes < w.total) return GBX_ERR_WORKSPACE;
  if (int e = set_kernel_attrs()) return e;
  const Shape h = shape_of(batch, n, NB);
  const int nb = h.nb, npot = h.npot, nslot = h.nslot;
  // matrix table: slot / counter offsets in batch order, queue order largest first
  std::vector<long long> slot0(batch), dcnt0(batch), dt0(batch);
  long long acc = 0, dacc = 0, tacc = 0;
  for (int k = 0; k < batch; ++k) {
    slot0[k] = acc;
    dcnt0[k] = dacc;
    dt0[k] = tacc;
    const long long nt = (n[k] + NB - 1) / NB;
    acc += nt * (nt + 1) / 2;
    dacc += nt * nb * nb;
    tacc += nt;
  }
  std::vector<int> order(batch);
  for (int k = 0; k < batch; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return n[a] > n[b]; });
  std::vector<MixMat> mats(order.size());
  int maxNT = 0;
  for (size_t q = 0; q < order.size(); ++q) {
    const int k = order[q];
    const int nt = (n[k] + NB - 1) / NB;
    mats[q].slot0 = slot0[k];
    mats[q].N = n[k];
    mats[q].NT = nt;
    mats[q].cnt0 = (int)slot0[k];
    mats[q].id = k;
    mats[q].dcnt0 = (int)dcnt0[k];
    mats[q].dt0 = (int)dt0[k];
    maxNT = std::max(maxNT, nt);
  }
  // queue: phase by phase (phase p of a matrix: the tasks between POTRF(p) and POTRF(p+1) in its
  // own order); within a phase, group by group: 1 the updates of column p by panel p-1, 2 POTRF(p),
  // then (schedule 0) 4 the trailing updates of the columns right of p by panel p-1 and 3 the TRSMs
  // of column p, or (schedule 1) 3 before 4; within a group the matrices largest first; the POTRF
  // group goes mini-task by mini-task across the matrices. The trailing updates do not depend on
  // POTRF(p): with schedule 0 CTAs work on them while the POTRF mini-flowgraph runs instead of
  // waiting on its TRSMs; schedule 1 starts the next panel's critical chain earlier. Every task's
  // predecessors stay earlier in the queue in both (group 4 of phase p needs TRSMs and updates of
  // phase p-1; group 3 needs groups 1 and 2 of phase p), so in-order grabbing cannot deadlock.
  std::vector<MixSeg> segs;
  long long task0 = 0;
  auto group_range = [&](int nt, int p, int g, long long& first, long long& last) {
    if (p == 0) {  // POTRF(0), then TRSM(m, 0)
      first = g == 2 ? 0 : g == 3 ? 1 : 0;
      last = g == 2 ? 1 : g == 3 ? nt : 0;
      return;
    }
    const long long k = p - 1, R = nt - 1, r = nt - k - 1;
    const long long base = nt + seg_prefix(k, R), len = seg_prefix(k + 1, R) - seg_prefix(k, R);
    const long long lo[5] = {0, 0, r, r + 1, 2 * r}, hi[5] = {0, r, r + 1, 2 * r, len};
    first = base + lo[g];
    last = base + hi[g];
  };
  const int group_order[4] = {1, 2, sched == 1 ? 3 : 4, sched == 1 ? 4 : 3};
  for (int p = 0; p < maxNT; ++p)
    for (int gi = 0; gi < 4; ++gi) {
      const int g = group_order[gi];
      if (g == 2)  // the single POTRF of this phase, one slot per mini-task
        for (int u = 0; u < npot; ++u)
          for (size_t q = 0; q < mats.size(); ++q) {
            if (mats[q].NT <= p) continue;
            long long first, last;
            group_range(mats[q].NT, p, 2, first, last);
            segs.push_back(MixSeg{task0, first, (int)q, 1, u, 0});
            task0 += 1;
          }
      for (size_t q = 0; q < mats.size(); ++q) {
        const int nt = mats[q].NT;
        if (nt <= p) continue;
        long long first, last;
        group_range(nt, p, g, first, last);
        if (last <= first) continue;
        if (g == 2) continue;  // (queued above, mini-task by mini-task)
        segs.push_back(MixSeg{task0, first, (int)q, nslot, 0, 0});
        task0 += (last - first) * nslot;
      }
    }
  if ((long long)segs.size() > w.nsegs || task0 != h.ntasks) return GBX_ERR_ARG;  // the tables must fit their space
  // the reserved segment slots past the last one start beyond every queue position, so that the
  // kernel's search over all w.nsegs slots finds the right segment
  segs.resize((size_t)w.nsegs, MixSeg{LLONG_MAX, 0, 0, 1, 0, 0});
  char* base = (char*)work;
  if (cudaMemcpyAsync(base + w.mats, mats.data(), mats.size() * sizeof(MixMat), cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(base + w.segs, segs.data(), segs.size() * sizeof(MixSeg), cudaMemcpyHostToDevice, s) !=
          cudaSuccess)
    return GBX_ERR_CUDA;
  return GBX_OK;
}

int run_batch(int batch, const int* n, int NB, float* W, int prec, double fp64_cond, const int* dsel, void* work,
              size_t work_bytes, cudaStream_t s) {
  const Ws w = layout_batch(batch, n, NB);
  if (work_bytes < w.total) return GBX_ERR_WORKSPACE;
  if (int e = set_kernel_attrs()) return e;
  const Shape h = shape_of(batch, n, NB);
  char* base = (char*)work;
  // run state, counters, condition estimates, info, FP64-route counts and routes of every matrix
  if (cudaMemsetAsync(base, 0, w.mats, s) != cudaSuccess) return GBX_ERR_CUDA;
  CUtensorMap ta, tb;
  const bool bf16 = prec == 0;
  const uint64_t lrows = (uint64_t)w.slots * NB;
  // rows of a ragged tile's low-precision copy past the matrix edge are never written; the tensor
  // cores read them, but they only reach rows / columns of C that the epilogue does not store
  if (prec == 2) {  // fp8: rows of NB bytes in the same buffer
    if (int e = tc::make_tmap_kmajor_8b(&ta, base + w.lb, lrows, (uint64_t)NB, (uint64_t)NB, kSubM)) return e;
    if (int e = tc::make_tmap_kmajor_8b(&tb, base + w.lb, lrows, (uint64_t)NB, (uint64_t)NB, kSubN)) return e;
  } else {
    if (int e = tc::make_tmap_kmajor_16b(&ta, base + w.lb, lrows, (uint64_t)NB, (uint64_t)NB, kSubM, bf16)) return e;
    if (int e = tc::make_tmap_kmajor_16b(&tb, base + w.lb, lrows, (uint64_t)NB, (uint64_t)NB, kSubN, bf16)) return e;
  }
  Params P;
  P.W = W;
  P.Lb = base + w.lb;
  P.rowexp = (int*)(base + w.rowexp);
  P.NB = NB;
  P.f16 = prec == 1;
  P.fp8 = prec == 2;
  P.sub_g = h.sub_g;
  P.sub_t = h.sub_t;
  P.nb = h.nb;
  P.npot = h.npot;
  P.dcnt = (int*)(base + w.dcnt);
  P.sub_s = h.sub_s;
  P.ntasks = h.ntasks;
  P.mats = (const MixMat*)(base + w.mats);
  P.nmats = batch;
  P.segs = (const MixSeg*)(base + w.segs);
  P.nsegs = (int)w.nsegs;
  P.st = (DagState*)base;
  P.cnt = (int*)(base + w.cnt);
  P.minfo = (int*)(base + w.minfo);
  P.cond_est = (float*)(base + w.cond);
  P.D64 = (double*)(base + w.d64);
  P.route = (int*)(base + w.route);
  P.nfp64 = (int*)(base + w.nfp64);
  P.fp64_cond = fp64_cond >= 3.0e38 ? INFINITY : (float)fp64_cond;
  P.dsel = dsel;
  P.timeout_ns = gbx_get_wait_timeout_ns();
  P.trace = current_trace();
  potrf_mixed_kernel<<<g_sms, kThr, kSmemBytes, s>>>(ta, tb, P);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

// device addresses of a batched factorisation's results in its workspace
struct InfoPtrs {
  const DagState* st;
  const int* minfo;
  const float* cond;
  const int* nfp64;
};
InfoPtrs info_ptrs(int batch, const int* n, int NB, const void* work) {
  const Ws w = layout_batch(batch, n, NB);
  const char* b = (const char*)work;
  return InfoPtrs{(const DagState*)b, (const int*)(b + w.minfo), (const float*)(b + w.cond), (const int*)(b + w.nfp64)};
}

// W = fl32(A) for the selected matrices (sel host array, null: all), the diagonal scaled by (1 + shift)
int convert_host_sel(int batch, const int* n, int NB, const double* A, float* W, double shift,
                     const unsigned char* sel, cudaStream_t s) {
  if (int e = set_kernel_attrs()) return e;
  long long slot0 = 0;
  for (int k = 0; k < batch; ++k) {
    const int nt = (n[k] + NB - 1) / NB;
    const long long nsl = (long long)nt * (nt + 1) / 2, nel = nsl * (long long)NB * NB;
    if (!sel || sel[k]) {
      convert_kernel<<<std::min<long long>(g_sms * 8, (nel + 255) / 256), 256, 0, s>>>(
          A + slot0 * (long long)NB * NB, W + slot0 * (long long)NB * NB, nel);
      if (shift != 0.0)
        shift_diag_kernel<<<nt, 256, 0, s>>>(W + slot0 * (long long)NB * NB, n[k], NB, nt, (float)shift);
    }
    slot0 += nsl;
  }
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}
}  // namespace mixed
}  // namespace gbx

extern "C" long long gbx_mixed_task(int NT, long long t, int* key) {
  if (NT <= 0) return GBX_ERR_ARG;
  const long long n = num_tile_tasks(NT);
  if (t >= n || (t >= 0 && !key)) return GBX_ERR_ARG;
  if (t >= 0) {
    const TileKey k = decode(t, NT);
    key[0] = k.type;
    key[1] = k.a;
    key[2] = k.b;
    key[3] = k.c;
  }
  return n;
}

extern "C" int gbx_potrf_mixed_bufferSize(int N, int NB, size_t* bytes) {
  if (N <= 0 || NB <= 0 || NB % 256 || NB > kMaxNB || !bytes) return GBX_ERR_ARG;
  *bytes = layout(N, NB).total;
  return GBX_OK;
}

extern "C" int gbx_potrf_mixed(int N, int NB, const double* A, float* W, int prec, double shift, double fp64_diag_cond,
                               void* work, size_t work_bytes, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N <= 0) return GBX_ERR_ARG;
  return gbx_potrf_mixed_batched(1, &N, NB, A, W, prec, shift, fp64_diag_cond, nullptr, work, work_bytes, stream);
}

extern "C" int gbx_potrf_mixed_batched_bufferSize(int batch, const int* n, int NB, size_t* bytes) {
  if (batch <= 0 || !n || NB <= 0 || NB % 256 || NB > kMaxNB || !bytes) return GBX_ERR_ARG;
  for (int k = 0; k < batch; ++k)
    if (n[k] <= 0) return GBX_ERR_ARG;
  *bytes = layout_batch(batch, n, NB).total;
  return GBX_OK;
}

extern "C" int gbx_potrf_mixed_batched(int batch, const int* n, int NB, const double* A, float* W, int prec,
                                       double shift, double fp64_diag_cond, const unsigned char* sel, void* work,
                                       size_t work_bytes, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  size_t need = 0;
  if (int e = gbx_potrf_mixed_batched_bufferSize(batch, n, NB, &need)) return e;
  if (!A || !W || !work || prec < 0 || prec > 2 || !(fp64_diag_cond >= 0.0)) return GBX_ERR_ARG;
  if (work_bytes < need) return GBX_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  if (int e = plan_batch(batch, n, NB, work, work_bytes, s, 0)) return e;
  if (int e = convert_host_sel(batch, n, NB, A, W, shift, sel, s)) return e;
  const int* dsel = nullptr;
  if (sel) {
    const Ws w = layout_batch(batch, n, NB);
    std::vector<int> hs(batch);
    for (int k = 0; k < batch; ++k) hs[k] = sel[k] ? 1 : 0;
    if (cudaMemcpyAsync((char*)work + w.sel, hs.data(), batch * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return GBX_ERR_CUDA;
    dsel = (const int*)((char*)work + w.sel);
  }
  return run_batch(batch, n, NB, W, prec, fp64_diag_cond, dsel, work, work_bytes, s);
}

extern "C" int gbx_potrf_mixed_batched_info(const void* work, int batch, const int* n, int NB, int* info,
                                            float* cond_est, int* fp64_tiles, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (!work || batch <= 0 || !n || NB <= 0) return GBX_ERR_ARG;
  const Ws w = layout_batch(batch, n, NB);
  cudaStream_t s = (cudaStream_t)stream;
  int st = 0;
  if (cudaMemcpyAsync(&st, work, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return GBX_ERR_CUDA;
  if (info && cudaMemcpyAsync(info, (const char*)work + w.minfo, batch * sizeof(int), cudaMemcpyDeviceToHost, s) !=
                  cudaSuccess)
    return GBX_ERR_CUDA;
  if (cond_est && cudaMemcpyAsync(cond_est, (const char*)work + w.cond, batch * sizeof(float), cudaMemcpyDeviceToHost,
                                  s) != cudaSuccess)
    return GBX_ERR_CUDA;
  if (fp64_tiles && cudaMemcpyAsync(fp64_tiles, (const char*)work + w.nfp64, batch * sizeof(int),
                                    cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return GBX_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  return st < 0 ? st : GBX_OK;  // < 0: the launch itself failed (timeout)
}

extern "C" int gbx_potrf_mixed_info(const void* work, int N, int NB, float* cond_est, int* fp64_tiles, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (!work || N <= 0 || NB <= 0) return GBX_ERR_ARG;
  const Ws w = layout(N, NB);
  int st = 0, nf = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&st, work, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return GBX_ERR_CUDA;
  float c = 0.f;
  if (cudaMemcpyAsync(&c, (const char*)work + w.cond, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&nf, (const char*)work + w.nfp64, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return GBX_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  if (cond_est) *cond_est = c;
  if (fp64_tiles) *fp64_tiles = nf;
  return st;
}
