// FP64 tiled Cholesky for GB300 (sm_103a): block kernels, the persistent flowgraph executor,
// the tile-level drop-in entry points, the tiled solve and the device-side generators.
//
// FP64 on GB300 runs at ~2 DFMA/clk/SM, so every kernel here is organised to keep the FP64
// pipe busy (enough independent FMAs per warp, operands staged in shared memory, L2-only loads)
// and the executor is organised to keep every SM busy (device-side ready queue, lookahead order,
// fine-grained 128 x 128 blocks, no host round trip per task).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "block_ops.cuh"
#include "emu_f64.cuh"
#include "gbx_common.cuh"
#include "gbx_potrf.h"
#include "plgsy.cuh"
#include "taskq.h"
#include "tc_common.cuh"

namespace gbx {
namespace tc {
int make_tmap_kmajor_bf16(CUtensorMap* map, const void* base, uint64_t rows, uint64_t k, uint64_t ld,
                          uint32_t box_rows);  // gemm_bf16.cu
}

constexpr size_t kDagSmemBytes = (size_t)kBlk * kBlk * sizeof(double) + 64;  // POTRF dominates

// ------------------------------------------------------------------------------------------------
// the device-side ready queue: task index -> flowgraph key, in lookahead order
//   prologue: POTRF(0), TRSM(m,0) m=1..
//   for k = 0 .. NTb-2:
//     panel part (column k+1): SYRK(k,k+1), GEMM(m,k+1,k) m>k+1, POTRF(k+1), TRSM(m,k+1) m>k+1
//     trailing part: for n = k+2..: SYRK(k,n), GEMM(m,n,k) m>n
// The TRSM of the block just below a diagonal block, TRSM(K+1,K), is on the critical path
// POTRF(K) -> TRSM(K+1,K) -> SYRK(K,K+1) -> POTRF(K+1): it runs as kTrsmParts row sub-tasks
// (key c = sub-task) on as many CTAs, and its block counts as final after all of them.
// Every task's predecessors come earlier in this order, so CTAs that take tasks in order and
// wait for their predecessors always make progress.
// ------------------------------------------------------------------------------------------------
enum : int { T_POTRF = 0, T_TRSM = 1, T_SYRK = 2, T_GEMM = 3 };
constexpr int kTrsmParts = 4;

struct TaskKey {
  int type, a, b, c;
};

// TRSM completions block (M,K) counts before it is final
__host__ __device__ __forceinline__ int trsm_parts(int M, int K) { return M == K + 1 ? kTrsmParts : 1; }

__host__ __device__ __forceinline__ long long seg_prefix(long long k, long long R) {
  // sum over j < k of seg(j) = 2 r + r (r-1) / 2 (+ kTrsmParts - 1 when r >= 2, the split TRSM)
  // with r = R - j
  const long long s1 = k * R - k * (k - 1) / 2;
  const long long s2 = k * R * R - R * k * (k - 1) + (k - 1) * k * (2 * k - 1) / 6;
  const long long split = k < R - 1 ? k : (R - 1 > 0 ? R - 1 : 0);  // steps j < k with R - j >= 2
  return (3 * s1 + s2) / 2 + (kTrsmParts - 1) * split;
}

__host__ __device__ __forceinline__ long long dag_prologue(int NTb) {
  return NTb + (NTb >= 2 ? kTrsmParts - 1 : 0);
}

__host__ __device__ __forceinline__ long long dag_num_tasks(int NTb) {
  return dag_prologue(NTb) + seg_prefix(NTb - 1, NTb - 1);
}

// lead > 0 (the emulated executor): the first `lead` tasks of each step's trailing part go ahead of
// that step's TRSMs, so that the CTAs which take the TRSMs find their POTRF done instead of waiting
// for it (the order stays topological: trailing tasks of step k need only TRSMs of step k - 1).
__host__ __device__ inline TaskKey dag_decode(long long t, int NTb, long long lead = 0) {
  const long long P0 = dag_prologue(NTb);
  if (t < P0) {
    if (t == 0) return TaskKey{T_POTRF, 0, 0, 0};
    if (t <= kTrsmParts) return TaskKey{T_TRSM, 1, 0, (int)(t - 1)};
    return TaskKey{T_TRSM, (int)(t - (kTrsmParts - 1)), 0, 0};
  }
  const long long u = t - P0, R = NTb - 1;
  int lo = 0, hi = NTb - 2;  // largest k with seg_prefix(k) <= u
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (seg_prefix(mid, R) <= u) lo = mid;
    else hi = mid - 1;
  }
  const int k = lo;
  const long long p = u - seg_prefix(k, R);
  const int r = NTb - k - 1;
  if (p == 0) return TaskKey{T_SYRK, k, k + 1, 0};
  if (p < r) return TaskKey{T_GEMM, k + 1 + (int)p, k + 1, k};
  if (p == r) return TaskKey{T_POTRF, k + 1, 0, 0};
  const long long q = r - 1;  // trailing columns n = k+2 .. NTb-1: q (q + 1) / 2 tasks
  const long long X = lead < q * (q + 1) / 2 ? lead : q * (q + 1) / 2;
  const long long nts = q + (q > 0 ? kTrsmParts - 1 : 0);  // TRSM slots: TRSM(k+2,k+1) split
  long long pp;
  if (p <= r + X) pp = p - r - 1;  // the leading trailing tasks
  else if (p < r + 1 + X + nts) {
    const long long s = p - (r + 1 + X);
    if (s < kTrsmParts) return TaskKey{T_TRSM, k + 2, k + 1, (int)s};
    return TaskKey{T_TRSM, k + 2 + (int)(s - (kTrsmParts - 1)), k + 1, 0};
  } else pp = p - (r + 1 + nts);
  int clo = 0, chi = (int)q - 1;                           // largest c with S(c) <= pp
  while (clo < chi) {
    const int mid = (clo + chi + 1) >> 1;
    const long long S = (long long)mid * q - (long long)mid * (mid - 1) / 2;
    if (S <= pp) clo = mid;
    else chi = mid - 1;
  }
  const long long o = pp - ((long long)clo * q - (long long)clo * (clo - 1) / 2);
  const int n = k + 2 + clo;
  if (o == 0) return TaskKey{T_SYRK, k, n, 0};
  return TaskKey{T_GEMM, n + (int)o, n, k};
}

struct DagParams {
  TraceBuf trace;
  BlockView V;
  int NTb;
  long long ntasks;
  DagState* st;
  int* cnt;            // packed lower per-block completion counters
  uint64_t timeout_ns;
  // tensor-core emulated updates (kEmu launches): digit planes and row exponents of every lower
  // block, indexed by tri_index (diagonal blocks unused)
  uint16_t* planes;
  int* rexp;
  long long lead;  // trailing tasks of a step queued ahead of its TRSMs (dag_decode)
};


// the counters a task waits on: up to three (counter, target) pairs
__device__ __forceinline__ int dag_deps(const DagParams& P, const TaskKey& k, const int** c, int* v) {
  const int NTb = P.NTb;
  switch (k.type) {
    case T_POTRF:
      c[0] = P.cnt + tri_index(k.a, k.a, NTb), v[0] = k.a;
      return 1;
    case T_TRSM:
      c[0] = P.cnt + tri_index(k.b, k.b, NTb), v[0] = k.b + 1;
      c[1] = P.cnt + tri_index(k.a, k.b, NTb), v[1] = k.b;
      return 2;
    case T_SYRK:
      c[0] = P.cnt + tri_index(k.b, k.a, NTb), v[0] = k.a + trsm_parts(k.b, k.a);
      c[1] = P.cnt + tri_index(k.b, k.b, NTb), v[1] = k.a;
      return 2;
    default:
      c[0] = P.cnt + tri_index(k.a, k.c, NTb), v[0] = k.c + trsm_parts(k.a, k.c);
      c[1] = P.cnt + tri_index(k.b, k.c, NTb), v[1] = k.c + trsm_parts(k.b, k.c);
      c[2] = P.cnt + tri_index(k.a, k.b, NTb), v[2] = k.c;
      return 3;
  }
}
// blocking (bounded) wait for every dependency; false when the run stopped
__device__ __forceinline__ bool dag_deps_wait(const DagParams& P, const TaskKey& k) {
  const int* c[3];
  int v[3];
  const int n = dag_deps(P, k, c, v);
  for (int i = 0; i < n; ++i)
    if (!wait_geq(c[i], v[i], P.st, P.timeout_ns)) return false;
  return true;
}
// one non-blocking look at every dependency: relaxed loads issued together (an acquire each would
// serialise them); the caller fences once they are all met
__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ bool dag_deps_ready(const DagParams& P, const TaskKey& k) {
  const int* c[3];
  int v[3];
  const int n = dag_deps(P, k, c, v);
  const int x0 = ld_relaxed_gpu(c[0]);
  const int x1 = n > 1 ? ld_relaxed_gpu(c[1]) : v[1 % n];
  const int x2 = n > 2 ? ld_relaxed_gpu(c[2]) : v[2 % n];
  return x0 >= v[0] && (n < 2 || x1 >= v[1]) && (n < 3 || x2 >= v[2]);
}

// ---- the emulated update task: C(M,N) -= L(M,K) L(N,K)^T on the tensor cores -----------------
// Two passes over the 64-column halves of C; each pass accumulates the 28 digit-plane products of
// the seven groups g = i + j <= 6 into seven 128 x 64 FP32 accumulators in TMEM (group g in columns
// 64 g .. 64 g + 63), over two 64-wide chunks of k, in two phases: A (groups 3-6, 22 of the 28
// plane pairs) and B (groups 0-2). As soon as phase A of a pass is done the epilogue folds its four
// groups into one 64-bit integer per element (L) and frees their columns, so the next pass's phase
// A runs while this pass's groups 0-2 are read; those are folded with L into one 64-bit X per
// element and freed in turn, and the subtraction of X 2^E from C runs beside the next pass's
// products (and beside the first phase of the next task, which the producer and the issuer start
// once this task's last products are out).
// The emulated executor runs 384 threads (twelve warps); its FP64 tasks use the first 256.
//   warp 8 lane 0  TMA producer: per phase and chunk the phase's B planes (64 rows each) into one
//                  of two buffers, then its A planes (128 rows each) through a ring of seven slots
//                  (which fills the 227 KB of shared memory a CTA can have)
//   warp 9 lane 0  MMA issuer: per phase and chunk, for each A plane i and k-step, one MMA of
//                  M128 x N(64 x planes) x K16 against all the B planes j of the phase's groups
//                  i + j: the B planes of a chunk are consecutive 64-row blocks of one K-major tile
//                  and the groups consecutive 64-column blocks of TMEM, so 10 instructions per
//                  k-step cover the 28 plane pairs (one thread issues a tcgen05.mma only every
//                  ~110 clocks; an N=64 product takes the tensor pipe ~35). Each A slot is
//                  released after its instructions, each B buffer after its chunk.
//   warp 10        the C block's lines into L2 ahead of the epilogue's reads; warp 11 has no part
//   warps 0-7      epilogue: TMEM lane quarter = warp % 4, column half = warp / 4; per element the
//                  integer group sums L (after phase A) and X (after phase B), the rounding of X
//                  and one FP64 subtraction from C
namespace emuk {
constexpr int kASlots = 7, kBBufs = 2;
constexpr uint32_t kABytes = 128 * 128, kBBytes = 64 * 128;  // one plane chunk: rows x 128 bytes
constexpr uint32_t kBSetBytes = emu::kSlices * kBBytes;
constexpr size_t kSmemBytes = (size_t)kBBufs * kBSetBytes + (size_t)kASlots * kABytes + 1024;
constexpr int kTmemCols = 512;
constexpr int kThreadsEmu = 384;
constexpr int kEpiWarps = 8, kProducerWarp = 8, kIssuerWarp0 = 9;
struct Bars {
  uint64_t a_full[kASlots], a_empty[kASlots], b_full[kBBufs], b_empty[kBBufs];
  uint64_t done_a, done_b;  // phase A / B products of a pass complete (issuer commit)
  uint64_t free_l, free_h;  // the epilogue has read groups 3-6 / 0-2 of a pass (eight warps)
  uint64_t decided;         // the producer has decided whether to start the next task early
  uint64_t fin;
};
struct Pipe {  // pipeline positions, each kept by the one thread that uses it
  uint32_t a_it = 0, b_it = 0;  // producer: plane chunks issued; MMA issuer: consumed (A ring, B buffers)
  uint32_t passes = 0;          // MMA issuer and epilogue threads: accumulator passes begun
  uint32_t tasks = 0;           // MMA issuer: update tasks done (parity of the `decided` barrier)
  int ahead = 0;                // producer / issuer: phases of the next task already out (0 or 1)
  bool mma_issued = false;
};
}  // namespace emuk

// The next task of the queue, taken while the current one runs (kEmu: by an epilogue warp while
// the first pass's products run, or by the producer warp, idle in an FP64 task): decoded, and its dependencies looked at once without blocking (thread 0
// waits for them, if they were not met, after the current task has signalled: a CTA never waits
// on the task it runs itself). Called from a branch that no lane of a pipeline role has to
// reconverge with before it finishes.
struct Prefetch {
  long long* next;  // -2 none taken, -1 queue empty, else the task index
  int* ok;          // its dependencies were all met
  TaskKey* key;
  int* done;        // the three above are written (set last)
  int* ahead;       // kEmu: the producer started the next task's first phase (emu_update)
};
__device__ __noinline__ void prefetch_next(const DagParams& P, long long cur, const Prefetch& pf) {
  if (cur + 1 >= P.ntasks) {
    *(volatile int*)pf.done = 1;
    return;
  }
  long long tn = -1;
  if (!ld_volatile(&P.st->abort)) tn = (long long)atomicAdd(&P.st->head, 1ULL);
  int ok = 0;
  if (tn >= 0 && tn < P.ntasks) {
    const TaskKey kn = dag_decode(tn, P.NTb, P.lead);
    *pf.key = kn;
    // one look (a polling loop here slowed the producer lane of the same warp more than it saved)
    if (dag_deps_ready(P, kn)) {
      __threadfence();  // acquire side of the producers' fence + counter increment
      ok = 1;
    }
  }
  *pf.ok = ok;
  *pf.next = (tn >= 0 && tn < P.ntasks) ? tn : -1;
  __threadfence_block();
  *(volatile int*)pf.done = 1;
}

__device__ __forceinline__ void emu_update(const CUtensorMap* tmA, const CUtensorMap* tmB, const DagParams& P,
                                           int M, int Nn, int K, bool syrk, uint8_t* smem, emuk::Bars& bars,
                                           emuk::Pipe& pp, uint32_t tmem, int* s_cexp, long long cur_task,
                                           const Prefetch& pf) {
  using namespace emuk;
  using namespace tc;
  const BlockView& V = P.V;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long tA = tri_index(M, K, P.NTb), tB = tri_index(Nn, K, P.NTb);
  int* err = &P.st->status;
  uint8_t* smB = smem;                               // [kBBufs][7][64 x 128 B]
  uint8_t* smA = smem + (size_t)kBBufs * kBSetBytes;  // [kASlots][128 x 128 B]
  // column exponents of this task (rows of L(N,K)), before the roles split; each epilogue thread's
  // row exponent (row of L(M,K)) is read beside them
  const int r_ep = threadIdx.x & (emu::kEdge - 1);
  const int ea_ld = (warp < kEpiWarps && r_ep < V.dim(M)) ? __ldcg(P.rexp + tA * emu::kEdge + r_ep) : emu::kEmptyRow;
  if (threadIdx.x < emu::kEdge) s_cexp[threadIdx.x] = __ldcg(P.rexp + tB * emu::kEdge + threadIdx.x);
  __syncthreads();
  // one phase of one pass: the producer's loads (per 64-wide chunk of k the phase's B planes, 64
  // rows each, into one of two buffers, then its A planes, 128 rows each, through the ring) and the
  // issuer's products. Phase A (ph 0): groups 3-6, all seven planes; phase B (ph 1): groups 0-2,
  // planes 0-2.
  auto load_phase = [&](long long ta, long long tb, int pass, int ph) -> bool {
    const int np = ph == 0 ? emu::kSlices : 3;
    for (int c = 0; c < 2; ++c) {
      const uint32_t bb = pp.b_it % kBBufs, bph = (pp.b_it / kBBufs) & 1;
      if (!mbar_wait(smem_u32(&bars.b_empty[bb]), bph ^ 1, err, P.timeout_ns)) return false;
      const uint32_t bdst = smem_u32(smB + (size_t)bb * kBSetBytes);
      mbar_arrive_expect_tx(smem_u32(&bars.b_full[bb]), np * kBBytes);
      for (int j = 0; j < np; ++j)
        tma_load_2d(bdst + j * kBBytes, tmB, smem_u32(&bars.b_full[bb]), c * 64,
                    (int)((tb * emu::kSlices + j) * emu::kEdge + pass * 64));
      ++pp.b_it;
      for (int i = 0; i < np; ++i) {
        const uint32_t sl = pp.a_it % kASlots, aph = (pp.a_it / kASlots) & 1;
        if (!mbar_wait(smem_u32(&bars.a_empty[sl]), aph ^ 1, err, P.timeout_ns)) return false;
        mbar_arrive_expect_tx(smem_u32(&bars.a_full[sl]), kABytes);
        tma_load_2d(smem_u32(smA + (size_t)sl * kABytes), tmA, smem_u32(&bars.a_full[sl]), c * 64,
                    (int)((ta * emu::kSlices + i) * emu::kEdge));
        ++pp.a_it;
      }
    }
    return true;
  };
  auto issue_phase = [&](int ph) -> bool {
    // phase A writes groups 3-6 (TMEM columns 192-447), phase B groups 0-2 (columns 0-191): each
    // waits until the epilogue has read its columns of the previous pass
    if (pp.passes > 0 &&
        !mbar_wait(smem_u32(ph == 0 ? &bars.free_l : &bars.free_h), (pp.passes - 1) & 1, err, P.timeout_ns))
      return false;
    tc_fence_after();
    const int np_a = ph == 0 ? emu::kSlices : 3;  // A planes of the phase
    for (int c = 0; c < 2; ++c) {
      const uint32_t bb = pp.b_it % kBBufs, bph = (pp.b_it / kBBufs) & 1;
      if (!mbar_wait(smem_u32(&bars.b_full[bb]), bph, err, P.timeout_ns)) return false;
      tc_fence_after();
      const uint32_t bbase = smem_u32(smB + (size_t)bb * kBSetBytes);
      for (int i = 0; i < np_a; ++i) {
        const uint32_t sl = pp.a_it % kASlots, aph = (pp.a_it / kASlots) & 1;
        if (!mbar_wait(smem_u32(&bars.a_full[sl]), aph, err, P.timeout_ns)) return false;
        tc_fence_after();
        const uint64_t ad = desc_kmajor_sw128(smem_u32(smA + (size_t)sl * kABytes));
        // A_i against its B planes j of the phase's groups g = i + j at once: the planes are
        // consecutive 64-row blocks of one K-major tile and the groups consecutive 64-column
        // blocks of TMEM. Phase A: g = max(i,3)..6 (N <= 256); phase B: g = i..2.
        const int g0 = ph == 0 ? (i > 3 ? i : 3) : i, g1 = ph == 0 ? 6 : 2;
        const int np = g1 - g0 + 1;
        const uint64_t bd = desc_kmajor_sw128(bbase + (uint32_t)(g0 - i) * kBBytes);
        const uint32_t d = tmem + (uint32_t)(g0 * 64), id = idesc_f16(128, 64 * np, true);
#pragma unroll
        for (int ks = 0; ks < 4; ++ks)  // i = 0 first touches every group of the phase
          umma_f16(d, ad + 2 * ks, bd + 2 * ks, id, (c | i | ks) != 0 ? 1u : 0u);
        pp.mma_issued = true;
        umma_commit(smem_u32(&bars.a_empty[sl]));
        ++pp.a_it;
      }
      umma_commit(smem_u32(&bars.b_empty[bb]));
      ++pp.b_it;
    }
    umma_commit(smem_u32(ph == 0 ? &bars.done_a : &bars.done_b));
    return true;
  };
  // the four phases of a task: (pass 0, A), (pass 0, B), (pass 1, A), (pass 1, B); the first is
  // already out when the previous task started it early (pp.ahead). (Starting the first two early
  // measured slower: the producer then stays in the task until ring slots free up.)
  if (warp == kProducerWarp) {
    if (lane == 0) {
      // the planes were written by other CTAs with ordinary stores, and this CTA's shared memory
      // last by its FP64 tasks: order both before the async-proxy accesses
      asm volatile("fence.proxy.async.global;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      for (int u = pp.ahead; u < 4; ++u)
        if (!load_phase(tA, tB, u >> 1, u & 1)) return;
      pp.ahead = 0;
      // start the next task's first phase now, while this task's last composition runs, if it is an
      // update task whose dependencies were met when it was taken (only its digit planes are read
      // before it starts; its C block waits for its own start)
      bool ahead = false;
      TaskKey kn{};
      if (*(volatile int*)pf.done && *(volatile long long*)pf.next >= 0 && *(volatile int*)pf.ok) {
        kn = *pf.key;
        ahead = kn.type == T_SYRK || kn.type == T_GEMM;
      }
      *(volatile int*)pf.ahead = ahead ? 1 : 0;
      mbar_arrive(smem_u32(&bars.decided));
      if (ahead) {
        const int m = kn.type == T_SYRK ? kn.b : kn.a, n = kn.b;  // SYRK(K, M): C(M,M); GEMM(M, N, K)
        const int k = kn.type == T_SYRK ? kn.a : kn.c;
        if (!load_phase(tri_index(m, k, P.NTb), tri_index(n, k, P.NTb), 0, 0)) return;
        pp.ahead = 1;
      }
    }
    return;
  }
  if (warp == kIssuerWarp0) {
    if (lane == 0) {
      // consumer positions: this thread's own copy of a_it / b_it, advanced through the same
      // sequence of plane chunks as the producer's
      for (int u = pp.ahead; u < 4; ++u) {
        if (!issue_phase(u & 1)) return;
        if (u & 1) ++pp.passes;
      }
      pp.ahead = 0;
      if (!mbar_wait(smem_u32(&bars.decided), pp.tasks & 1, err, P.timeout_ns)) return;
      ++pp.tasks;
      if (*(volatile int*)pf.ahead) {
        if (!issue_phase(0)) return;
        pp.ahead = 1;
      }
    }
    return;
  }
  if (warp == kIssuerWarp0 + 1) {
    // C(M,N) into L2 ahead of the epilogue's reads: every 128-byte line of its columns
    const int mrows = V.dim(M), ncols = V.dim(Nn);
    const double* C = V.ptr(M, Nn);
    for (int col = lane; col < ncols; col += 32) {
      const uintptr_t c0 = (uintptr_t)(C + (long long)col * V.ld + (syrk ? col : 0));
      const uintptr_t c1 = (uintptr_t)(C + (long long)col * V.ld + mrows);
      for (uintptr_t a = c0 & ~(uintptr_t)127; a < c1; a += 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
    }
    return;
  }
  if (warp > kIssuerWarp0) return;
  if (warp < kEpiWarps) {
    const int q = warp & 3, r = q * 32 + lane;  // TMEM lane quarter; row of C
    const int h = warp >> 2;                    // column half of each pass
    const int mrows = V.dim(M), ncols = V.dim(Nn);
    double* C = V.ptr(M, Nn);
    const int ea = ea_ld;  // (r = r_ep)
    const bool row_ok = r < mrows && ea != emu::kEmptyRow;
    // the next task, while the first pass's products run (this warp waits for them otherwise)
    if (warp == kEpiWarps - 1 && lane == 0) prefetch_next(P, cur_task, pf);
    __syncwarp();
    long long Xv[32];  // per column of the pass: L (groups 3-6), then X (all seven groups)
    for (int pass = 0; pass < 2; ++pass) {
      // phase A done: groups 3-6 -> L, then their TMEM columns go back to the issuer
      if (!mbar_wait(smem_u32(&bars.done_a), pp.passes & 1, err, P.timeout_ns)) return;
      tc_fence_after();
#pragma unroll
      for (int cc = 0; cc < 32; cc += 8) {
        uint32_t v[4][8];
#pragma unroll
        for (int g = 0; g < 4; ++g) tmem_ld8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)((g + 3) * 64 + h * 32 + cc), v[g]);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 8; ++j) Xv[cc + j] = emu::group_l(v[0][j], v[1][j], v[2][j], v[3][j]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bars.free_l));
      // phase B done: groups 0-2 -> H, folded with L into X; the columns go back at once, and the
      // rounding and the subtraction from C run beside the next pass's products
      if (!mbar_wait(smem_u32(&bars.done_b), pp.passes & 1, err, P.timeout_ns)) return;
      tc_fence_after();
      uint32_t smask = 0;  // bit c: X of column c held as X 2^-8 (emu::fold)
#pragma unroll
      for (int cc = 0; cc < 32; cc += 8) {
        uint32_t v[3][8];
#pragma unroll
        for (int g = 0; g < 3; ++g) tmem_ld8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(g * 64 + h * 32 + cc), v[g]);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          int sh;
          Xv[cc + j] = emu::fold(emu::group_h(v[0][j], v[1][j], v[2][j]), Xv[cc + j], sh);
          smask |= (uint32_t)(sh >> 3) << (cc + j);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bars.free_h));
      // per chunk of four columns: C (in L2 by then: warp 10) read, X 2^(s + ea + eb - 62) subtracted,
      // C stored
#pragma unroll
      for (int cc = 0; cc < 32; cc += 4) {
        const int c0 = pass * 64 + h * 32 + cc;
        const int4 eb = *(const int4*)(s_cexp + c0);
        const int ebv[4] = {eb.x, eb.y, eb.z, eb.w};
        double cv[4], res[4];
        bool in[4], odd = false;
        int sE[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          in[j] = row_ok && c0 + j < ncols && (!syrk || r >= c0 + j);
          cv[j] = in[j] ? __ldcg(C + r + (long long)(c0 + j) * V.ld) : 0.0;
          sE[j] = ea - 62 + ebv[j] + (int)((smask >> (cc + j)) & 1) * 8;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          bool o;
          res[j] = emu::sub_scaled(cv[j], Xv[cc + j], sE[j], &o);
          odd |= o && in[j];
        }
        if (odd) {  // extreme scales only
#pragma unroll
          for (int j = 0; j < 4; ++j) res[j] = emu::sub_wide(cv[j], Xv[cc + j], sE[j]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (in[j]) __stcg(C + r + (long long)(c0 + j) * V.ld, res[j]);
      }
      ++pp.passes;
    }
  }
}

// Persistent executor: one CTA per SM takes tasks from the ready queue in order.
// Counter protocol (writers of block (M,N) in order: GEMM(M,N,0..N-1), then TRSM(M,N), as
// p(M,N) = trsm_parts(M,N) sub-tasks; of (M,M): SYRK(0..M-1,M), then POTRF(M)):
//   POTRF(K):      cnt(K,K) >= K
//   TRSM(M,K):     cnt(K,K) >= K+1, cnt(M,K) >= K
//   SYRK(K,M):     cnt(M,K) >= K+p(M,K), cnt(M,M) >= K
//   GEMM(M,N,K):   cnt(M,K) >= K+p(M,K), cnt(N,K) >= K+p(N,K), cnt(M,N) >= K
// kEmu: SYRK and GEMM run on the tensor cores (emu_update) from the digit planes that each TRSM
// writes of its block before it signals; POTRF and TRSM stay FP64.
template <bool kEmu>
__global__ void __launch_bounds__(kEmu ? emuk::kThreadsEmu : kThreads, 1)
    potrf_dag_f64_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, DagParams P) {
  extern __shared__ __align__(1024) uint8_t dsmem_raw[];
  uint8_t* dsmem = kEmu ? (uint8_t*)(((uintptr_t)dsmem_raw + 1023) & ~(uintptr_t)1023) : dsmem_raw;
  double* smem = (double*)dsmem;
  __shared__ long long s_task, s_next;
  __shared__ int s_go, s_failed, s_next_ok, s_next_done, s_ahead;
  __shared__ TaskKey s_key, s_next_key;
  __shared__ __align__(8) emuk::Bars bars;
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(16) int s_aux[2 * kBlk];
  const BlockView& V = P.V;
  const int NTb = P.NTb;
  const int warp = threadIdx.x >> 5;
  emuk::Pipe pp;
  uint32_t tmem = 0;
  if (kEmu) {
    if (threadIdx.x == 0) {
      using namespace tc;
      for (int i = 0; i < emuk::kASlots; ++i) {
        mbar_init(smem_u32(&bars.a_full[i]), 1);
        mbar_init(smem_u32(&bars.a_empty[i]), 1);
      }
      for (int i = 0; i < emuk::kBBufs; ++i) {
        mbar_init(smem_u32(&bars.b_full[i]), 1);
        mbar_init(smem_u32(&bars.b_empty[i]), 1);
      }
      mbar_init(smem_u32(&bars.done_a), 1);
      mbar_init(smem_u32(&bars.done_b), 1);
      mbar_init(smem_u32(&bars.free_l), emuk::kEpiWarps);
      mbar_init(smem_u32(&bars.free_h), emuk::kEpiWarps);
      mbar_init(smem_u32(&bars.decided), 1);
      mbar_init(smem_u32(&bars.fin), 1);
      mbar_fence_init();
    }
    if (warp == emuk::kIssuerWarp0) tc::tmem_alloc(tc::smem_u32(&tmem_slot), emuk::kTmemCols);
    __syncthreads();
    tc::tc_fence_after();
    tmem = tmem_slot;
  }
  // kEmu: the next task is taken while the current one runs (prefetch_next)
  if (threadIdx.x == 0) s_next = -2;  // none prefetched
  const Prefetch pf{&s_next, &s_next_ok, &s_next_key, &s_next_done, &s_ahead};
  for (;;) {
    if (threadIdx.x == 0) {
      long long t = -1;
      bool ready = false;
      if (s_next != -2) {
        t = s_next;
        ready = s_next_ok != 0;
      } else if (!ld_volatile(&P.st->abort)) {
        t = (long long)atomicAdd(&P.st->head, 1ULL);
      }
      s_task = (t >= 0 && t < P.ntasks) ? t : -1;
      s_failed = 0;
      s_next = -2;
      s_next_done = 0;
      if (s_task >= 0) {
        const TaskKey k = ready ? s_next_key : dag_decode(s_task, NTb, P.lead);
        s_key = k;
        s_go = ready ? 1 : (dag_deps_wait(P, k) ? 1 : 0);
      }
    }
    __syncthreads();
    const long long t = s_task;
    if (t < 0) break;
    const TaskKey tk = s_key;
    int* target;
    if (!s_go) break;
    const uint64_t t_start = P.trace.buf ? globaltimer_ns() : 0;
    switch (tk.type) {
      case T_POTRF: {  // the first 256 threads (all of them in the FP64 form)
        const int K = tk.a;
        if (threadIdx.x < kThreads) {
          const int info = op_potrf<double, kEmu>(V.ptr(K, K), V.ld, V.dim(K), smem);
          if (info != 0 && threadIdx.x == 0) {
            atomicCAS(&P.st->status, 0, K * V.b + info);
            atomicExch(&P.st->abort, 1);
            s_failed = 1;
          }
        } else if (kEmu && threadIdx.x == 32 * emuk::kProducerWarp + 1) {
          prefetch_next(P, t, pf);  // the producer warp has no role in an FP64 task
        }
        target = P.cnt + tri_index(K, K, NTb);
        break;
      }
      case T_TRSM: {  // the whole block, or (TRSM(K+1,K)) rows r0 .. r0 + V.b / kTrsmParts of it
        const int M = tk.a, K = tk.b;
        const int parts = trsm_parts(M, K), rows = V.b / parts;
        const int r0 = tk.c * rows, mr = min(rows, V.dim(M) - r0);
        if (threadIdx.x < kThreads && mr > 0) {
          op_trsm<double, false, kEmu>(V.ptr(K, K), V.ld, V.ptr(M, K) + r0, V.ld, mr, V.dim(K), smem);
          if (kEmu) {
            // the rows are final in global memory (each thread's own writes before the barrier)
            asm volatile("bar.sync 1, 256;" ::: "memory");
            const long long tb = tri_index(M, K, NTb);
            if (parts == 1)
              emu::slice_block(V.ptr(M, K), V.ld, V.dim(M), V.dim(K), P.planes + tb * emu::kBlockElems,
                               P.rexp + tb * emu::kEdge, s_aux);
            else
              emu::slice_block<emu::kEdge / kTrsmParts>(V.ptr(M, K) + r0, V.ld, mr, V.dim(K),
                                                        P.planes + tb * emu::kBlockElems + (long long)r0 * emu::kEdge,
                                                        P.rexp + tb * emu::kEdge + r0, s_aux);
          }
        } else if (kEmu && threadIdx.x == 32 * emuk::kProducerWarp + 1) {
          prefetch_next(P, t, pf);
        }
        target = P.cnt + tri_index(M, K, NTb);
        break;
      }
      case T_SYRK: {
        const int K = tk.a, M = tk.b;
        const double* a = V.ptr(M, K);
        if (kEmu) emu_update(&tmA, &tmB, P, M, M, K, true, dsmem, bars, pp, tmem, s_aux, t, pf);
        else if (V.b <= 64) op_gemm_nt<double, true>(a, V.ld, a, V.ld, V.ptr(M, M), V.ld, V.dim(M), V.dim(M), V.dim(K), true, smem);
        else op_gemm_nt<double>(a, V.ld, a, V.ld, V.ptr(M, M), V.ld, V.dim(M), V.dim(M), V.dim(K), true, smem);
        target = P.cnt + tri_index(M, M, NTb);
        break;
      }
      default: {
        const int M = tk.a, Nn = tk.b, K = tk.c;
        if (kEmu)
          emu_update(&tmA, &tmB, P, M, Nn, K, false, dsmem, bars, pp, tmem, s_aux, t, pf);
        else if (V.b <= 64)
          op_gemm_nt<double, true>(V.ptr(M, K), V.ld, V.ptr(Nn, K), V.ld, V.ptr(M, Nn), V.ld, V.dim(M), V.dim(Nn),
                                   V.dim(K), false, smem);
        else
          op_gemm_nt<double>(V.ptr(M, K), V.ld, V.ptr(Nn, K), V.ld, V.ptr(M, Nn), V.ld, V.dim(M), V.dim(Nn), V.dim(K),
                             false, smem);
        target = P.cnt + tri_index(M, Nn, NTb);
        break;
      }
    }
    __syncthreads();
    if (s_failed) break;
    if (threadIdx.x == 0) {
      if (kEmu && ld_volatile(&P.st->status) != 0) {  // a pipeline wait gave up: stop the launch
        atomicExch(&P.st->abort, 1);  // (every thread leaves at the next fetch)
        continue;
      }
      trace_record(P.trace, t_start, tk.type, tk.a, tk.b, tk.c, 0);  // end stamp before any waiter can start
      signal_done(target);
    }
  }
  if (kEmu) {
    using namespace tc;
    // after an early stop: let this CTA's copies and products in flight land (bounded waits) before
    // the shared memory and the accumulators are released
    if (warp == emuk::kProducerWarp && (threadIdx.x & 31) == 0) {
      for (uint32_t sl = 0; sl < emuk::kASlots; ++sl)
        if (pp.a_it > sl) {
          const uint32_t last = sl + emuk::kASlots * ((pp.a_it - 1 - sl) / emuk::kASlots);
          mbar_wait(smem_u32(&bars.a_full[sl]), (last / emuk::kASlots) & 1, nullptr, P.timeout_ns);
        }
      for (uint32_t bb = 0; bb < emuk::kBBufs; ++bb)
        if (pp.b_it > bb) {
          const uint32_t last = bb + emuk::kBBufs * ((pp.b_it - 1 - bb) / emuk::kBBufs);
          mbar_wait(smem_u32(&bars.b_full[bb]), (last / emuk::kBBufs) & 1, nullptr, P.timeout_ns);
        }
    }
    if (warp == emuk::kIssuerWarp0 && (threadIdx.x & 31) == 0 && pp.mma_issued) {
      umma_commit(smem_u32(&bars.fin));
      mbar_wait(smem_u32(&bars.fin), 0, nullptr, P.timeout_ns);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == emuk::kIssuerWarp0) {
      tc_fence_after();
      tmem_dealloc(tmem, emuk::kTmemCols);
    }
  }
}

// ---- single-purpose grids for the tile-level entry points ------------------------------------
__global__ void __launch_bounds__(kThreads, 1)
    gemm_nt_grid_kernel(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc,
                        int lower) {
  extern __shared__ __align__(16) double smem[];
  int bi = blockIdx.x, bj = blockIdx.y;
  if (lower) {  // blockIdx.x enumerates the lower block pairs (bi >= bj)
    const int t = blockIdx.x;
    bj = 0;
    int rem = t;
    const int nb = (n + kBlk - 1) / kBlk;
    while (rem >= nb - bj) {
      rem -= nb - bj;
      ++bj;
    }
    bi = bj + rem;
  }
  const int r0 = bi * kBlk, c0 = bj * kBlk;
  op_gemm_nt<double>(A + r0, lda, B + c0, ldb, C + r0 + (long long)c0 * ldc, ldc, min(kBlk, m - r0), min(kBlk, n - c0), k,
             lower && bi == bj, smem);
}

__global__ void __launch_bounds__(kThreads, 1)
    trsm_rlt_grid_kernel(int m, int n, const double* L, int ldl, double* B, int ldb) {
  extern __shared__ __align__(16) double smem[];
  const int r0 = blockIdx.x * kBlk;
  op_trsm<double>(L, ldl, B + r0, ldb, min(kBlk, m - r0), n, smem);
}

__global__ void copy_info_kernel(const DagState* st, int* devInfo) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *devInfo = st->status;
}

__global__ void set_head_kernel(DagState* st, unsigned long long head) {
  if (threadIdx.x == 0 && blockIdx.x == 0) st->head = head;
}

// ---- tiled solve: forward (L y = b) and backward (L^T x = y) sweeps over b x b blocks ---------
// Each sweep is one persistent launch over an in-order task sequence, step s holding NTb - s tasks:
//   forward,  K = s:          DIAG(K): wait until the K updates of block row K are in, then
//                             y_K = L_KK^{-1} x_K by substitution; flag K
//                             UPD(K+j, K): wait for flag K; x_{K+j} -= L_{K+j,K} y_K (FP64 atomics);
//                             count one for row K+j
//   backward, K = NTb-1-s:    DIAG(K): wait until the NTb-1-K updates of row K are in, then
//                             z_K = L_KK^{-T} y_K; flag K
//                             UPD(K, K-j): wait for flag K; y_{K-j} -= L_{K,K-j}^T z_K; count row K-j
// Every task waits only on earlier tasks, so CTAs taking tasks in order cannot deadlock; waits are
// bounded (status GBX_ERR_TIMEOUT). Vectors other CTAs update atomically are read through L2.
__device__ __forceinline__ void solve_decode(long long t, int NTb, int& s, int& j) {
  int lo = 0, hi = NTb - 1;  // largest s with start(s) = s NTb - s (s - 1) / 2 <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((long long)mid * NTb - (long long)mid * (mid - 1) / 2 <= t) lo = mid;
    else hi = mid - 1;
  }
  s = lo;
  j = (int)(t - ((long long)lo * NTb - (long long)lo * (lo - 1) / 2));
}

template <int DIR>
__global__ void __launch_bounds__(kThreads) solve_sweep_kernel(BlockView V, int NTb, double* X, int ldx, int nrhs,
                                                               DagState* st, int* cnt, int* flag,
                                                               uint64_t timeout_ns) {
  __shared__ double xk[kBlk];
  __shared__ double part[kThreads];
  __shared__ long long s_t;
  __shared__ int s_ok;
  const long long ntasks = (long long)NTb * (NTb + 1) / 2;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) {
      long long t = -1;
      if (!ld_volatile(&st->abort)) t = (long long)atomicAdd(&st->head, 1ULL);
      s_t = (t >= 0 && t < ntasks) ? t : -1;
    }
    __syncthreads();
    if (s_t < 0) break;
    int sidx, j;
    solve_decode(s_t, NTb, sidx, j);
    const int K = DIR == 0 ? sidx : NTb - 1 - sidx;
    const int O = DIR == 0 ? K + j : K - j;  // the other block of an update task
    if (tid == 0) {
      s_ok = j == 0 ? wait_geq(cnt + K, DIR == 0 ? K : NTb - 1 - K, st, timeout_ns)
                    : wait_geq(flag + K, 1, st, timeout_ns);
    }
    __syncthreads();
    if (!s_ok) break;
    const int kb = V.dim(K);
    if (j == 0) {  // substitution in the diagonal block, one right-hand side at a time
      const double* L = V.ptr(K, K);
      for (int r = 0; r < nrhs; ++r) {
        double* x = X + (long long)r * ldx + (long long)K * V.b;
        for (int i = tid; i < kb; i += blockDim.x) xk[i] = __ldcg(x + i);
        __syncthreads();
        if (DIR == 0) fwd_solve<double>(L, kb, V.ld, xk);
        else bwd_solve<double>(L, kb, V.ld, xk);
        for (int i = tid; i < kb; i += blockDim.x) x[i] = xk[i];
        __syncthreads();
      }
    } else if (DIR == 0) {  // x_O -= L_OK y_K: rows split over two halves of the CTA along k
      const int ob = V.dim(O);
      const double* L = V.ptr(O, K);
      for (int r = 0; r < nrhs; ++r) {
        const double* y = X + (long long)r * ldx + (long long)K * V.b;
        for (int i = tid; i < kb; i += blockDim.x) xk[i] = __ldcg(y + i);
        __syncthreads();
        const int row = tid & (kBlk - 1), half = tid >> 7;
        double a = 0.0;
        if (row < ob) {
          double a2 = 0.0;  // two chains, eight loads in flight per thread
          int c = half;
          for (; c + 14 < kb; c += 16) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = __ldcg(L + row + (long long)(c + 2 * u) * V.ld);
#pragma unroll
            for (int u = 0; u < 8; u += 2) {
              a = fma(v[u], xk[c + 2 * u], a);
              a2 = fma(v[u + 1], xk[c + 2 * u + 2], a2);
            }
          }
          for (; c < kb; c += 2) a = fma(__ldcg(L + row + (long long)c * V.ld), xk[c], a);
          a += a2;
        }
        part[tid] = a;
        __syncthreads();
        if (half == 0 && row < ob) atomicAdd(X + (long long)r * ldx + (long long)O * V.b + row, -(part[row] + part[row + kBlk]));
        __syncthreads();
      }
    } else {  // y_O -= L_KO^T z_K: warp per column of L_KO
      const int ob = V.dim(O);
      const double* L = V.ptr(K, O);
      const int warp = tid >> 5, lane = tid & 31;
      for (int r = 0; r < nrhs; ++r) {
        const double* z = X + (long long)r * ldx + (long long)K * V.b;
        for (int i = tid; i < kb; i += blockDim.x) xk[i] = __ldcg(z + i);
        __syncthreads();
        for (int c = warp; c < ob; c += kThreads / 32) {
          double a = 0.0;
#pragma unroll 4
          for (int i = lane; i < kb; i += 32) a = fma(__ldcg(L + i + (long long)c * V.ld), xk[i], a);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
          if (lane == 0) atomicAdd(X + (long long)r * ldx + (long long)O * V.b + c, -a);
        }
        __syncthreads();
      }
    }
    __threadfence();  // this thread's results are visible before the completion is
    __syncthreads();
    if (tid == 0) signal_done(j == 0 ? flag + K : cnt + O);
  }
}

// ---- device generators ----------------------------------------------------------------------
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

// grid: x over the NB*NB elements of a tile, y = tile row m, z = tile column n (m >= n)
__global__ void gen_tiles_kernel(int N, int NB, int NT, int kind, double bump_or_shift, unsigned long long seed,
                                 double* tiles) {
  const int m = blockIdx.y, n = blockIdx.z;
  if (m < n) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)NB * NB) return;
  const int i = (int)(e % NB), j = (int)(e / NB);
  const long long slot = (long long)n * NT - (long long)n * (n - 1) / 2 + (m - n);
  double* out = tiles + slot * (long long)NB * NB + e;
  const long long gi = (long long)m * NB + i, gj = (long long)n * NB + j;
  if (gi >= N || gj >= N) {
    *out = 0.0;
    return;
  }
  double v;
  if (kind == 0) {  // PLASMA: lower entries at stream position gi + gj*N, mirrored above
    const long long hi = gi >= gj ? gi : gj, lo = gi >= gj ? gj : gi;
    v = plgsy_entry(lcg_jump_dev((unsigned long long)hi + (unsigned long long)lo * (unsigned long long)N, seed));
    if (gi == gj) v = __dadd_rn(v, bump_or_shift);
  } else {
    if (gi == gj) v = __dadd_rn(uniform_elem(seed, gi, gi), bump_or_shift);
    else v = __dmul_rn(0.5, __dadd_rn(uniform_elem(seed, gi, gj), uniform_elem(seed, gj, gi)));
  }
  *out = v;
}

// A = diag(lam) + low-rank symmetric part, the closed form of Q diag(lam) Q^T for
// Q = I - U V^T (compact WY form of a product of r Householder reflectors):
//   A_ij = lam_i d_ij - lam_j (U V^T)_ij - lam_i (V U^T)_ij + (U G U^T)_ij,  G = V^T diag(lam) V
// U, V: column-major N x r (r <= 8), G: r x r column-major; one element per thread.
__global__ void gen_lowrank_kernel(int N, int NB, int NT, const double* __restrict__ lam,
                                   const double* __restrict__ U, const double* __restrict__ V,
                                   const double* __restrict__ G, int r, double* tiles) {
  const int m = blockIdx.y, n = blockIdx.z;
  if (m < n) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)NB * NB) return;
  const int i = (int)(e % NB), j = (int)(e / NB);
  const long long slot = (long long)n * NT - (long long)n * (n - 1) / 2 + (m - n);
  double* out = tiles + slot * (long long)NB * NB + e;
  const long long gi = (long long)m * NB + i, gj = (long long)n * NB + j;
  if (gi >= N || gj >= N) {
    *out = 0.0;
    return;
  }
  double ui[8], uj[8];
  double uv = 0.0, vu = 0.0;
  for (int a = 0; a < r; ++a) {
    ui[a] = U[gi + (long long)a * N];
    uj[a] = U[gj + (long long)a * N];
    uv = fma(ui[a], V[gj + (long long)a * N], uv);
    vu = fma(V[gi + (long long)a * N], uj[a], vu);
  }
  double ugu = 0.0;
  for (int b = 0; b < r; ++b) {
    double t = 0.0;
    for (int a = 0; a < r; ++a) t = fma(ui[a], G[a + b * r], t);
    ugu = fma(t, uj[b], ugu);
  }
  const double li = lam[gi], lj = lam[gj];
  *out = (gi == gj ? li : 0.0) - lj * uv - li * vu + ugu;
}

// one tile of the PLASMA generator: x over the m*n elements
__global__ void plgsy_tile_kernel(double bump, int m, int n, double* A, int lda, int gM, int m0, int n0,
                                  unsigned long long seed) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)m * n) return;
  const int i = (int)(e % m), j = (int)(e / m);
  const long long gi = (long long)m0 + i, gj = (long long)n0 + j;
  const long long hi = gi >= gj ? gi : gj, lo = gi >= gj ? gj : gi;
  double v = plgsy_entry(lcg_jump_dev((unsigned long long)hi + (unsigned long long)lo * (unsigned long long)gM, seed));
  if (gi == gj) v = __dadd_rn(v, bump);
  A[i + (long long)j * lda] = v;
}

// ---- host side --------------------------------------------------------------------------------
struct DevInfo {
  int dev = 0;
  int sms = 0;
  int dag_blocks_per_sm = 0;
  bool attrs_set = false;
};
// run state of the solve sweeps, per device (gbx_dpotrs_tiled has no workspace argument)
struct SolveScratch {
  void* buf = nullptr;
  size_t bytes = 0;
  cudaEvent_t ev = nullptr;  // recorded after each use: the next call's stream waits on it
};
std::mutex g_solve_mtx;
SolveScratch g_solve[32];
std::mutex g_mtx;
std::vector<DevInfo> g_dev;
TraceBuf g_trace{nullptr, 0};
TraceBuf current_trace() {
  std::lock_guard<std::mutex> lk(g_mtx);
  return g_trace;
}
uint64_t g_timeout_ns = 20ull * 1000 * 1000 * 1000;

int device_info(DevInfo& out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBX_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_mtx);
  if ((int)g_dev.size() <= dev) g_dev.resize(dev + 1);
  DevInfo& d = g_dev[dev];
  d.dev = dev;
  if (dev >= 32) return GBX_ERR_CUDA;
  if (!d.attrs_set) {
    if (cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBX_ERR_CUDA;
    if (cudaFuncSetAttribute(potrf_dag_f64_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kDagSmemBytes) != cudaSuccess)
      return GBX_ERR_CUDA;
    if (cudaFuncSetAttribute(potrf_dag_f64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)emuk::kSmemBytes) != cudaSuccess)
      return GBX_ERR_CUDA;
    if (cudaFuncSetAttribute(gemm_nt_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(4 * kKC * kBlk * sizeof(double))) != cudaSuccess)
      return GBX_ERR_CUDA;
    if (cudaFuncSetAttribute(trsm_rlt_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(op_trsm_smem_elems<double>() * sizeof(double))) != cudaSuccess)
      return GBX_ERR_CUDA;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, potrf_dag_f64_kernel<false>, kThreads, kDagSmemBytes) !=
        cudaSuccess)
      return GBX_ERR_CUDA;
    d.dag_blocks_per_sm = std::max(1, occ);
    d.attrs_set = true;
  }
  out = d;
  return GBX_OK;
}

// block edge used inside NB x NB tiles: NB itself up to 128, else the largest of 128/64/32 dividing NB
int block_edge(int NB) {
  if (NB <= kBlk) return NB;
  for (int b : {128, 64, 32})
    if (NB % b == 0) return b;
  return 0;
}

// Block edge of the executor for an N x N matrix of NB tiles. A small matrix is bound by its chain
// of block steps (each a single-CTA FP64 POTRF, TRSM and update of one block), so up to a size it
// takes 64-blocks: twice the steps, each about a quarter as long; larger matrices are bound by the
// total work and keep 128-blocks, whose block GEMM runs the FP64 pipe best and which the
// tensor-core updates need. That size: N = 4096 with FP64 FMA updates, N = 2048 with the
// tensor-core updates (GB300, NB = 512: N=3072 11.7 ms with 128-blocks against 14.8 with 64,
// N=4096 15.7 against 28.3; N=2048 7.70 against 7.60).
extern int g_fp64_update;
int g_forced_edge = 0;  // gbx_set_dag_block_edge
int dag_block_edge(int N, int NB) {
  const int b = block_edge(NB);
  if (b == 0) return 0;
  if (g_forced_edge > 0) return (NB % g_forced_edge == 0 && g_forced_edge <= b) ? g_forced_edge : b;
  return (b == kBlk && N <= (g_fp64_update == 1 ? 2048 : 4096)) ? 64 : b;
}

size_t dag_workspace_bytes(int NTb) {
  const size_t counters = (size_t)NTb * (NTb + 1) / 2 * sizeof(int);
  return sizeof(DagState) + ((counters + 255) / 256) * 256;
}

// FP64 update mode of the tiled executor (gbx_set_fp64_update): 0 FP64 FMA block GEMMs, 1 the
// tensor-core emulation (128-blocks only; other block edges run the FP64 FMA form)
int g_fp64_update = 0;
long long g_dag_lead = -1;  // gbx_set_dag_lead: -1 automatic
bool emu_active(const BlockView& V) { return g_fp64_update == 1 && V.b == kBlk; }

// workspace of an emulated run, after the counters: row exponents (128 per lower block), then the
// digit planes (7 x 128 x 128 bf16 per lower block), both indexed by tri_index
size_t emu_rexp_offset(int NTb) { return (dag_workspace_bytes(NTb) + 1023) / 1024 * 1024; }
size_t emu_planes_offset(int NTb) {
  const size_t ntri = (size_t)NTb * (NTb + 1) / 2;
  return (emu_rexp_offset(NTb) + ntri * emu::kEdge * sizeof(int) + 1023) / 1024 * 1024;
}
size_t emu_workspace_bytes(int NTb) {
  const size_t ntri = (size_t)NTb * (NTb + 1) / 2;
  return emu_planes_offset(NTb) + ntri * (size_t)emu::kBlockElems * sizeof(uint16_t);
}
size_t executor_workspace_bytes(const BlockView& V, int NTb) {
  return emu_active(V) ? emu_workspace_bytes(NTb) : dag_workspace_bytes(NTb);
}

int launch_dag(const BlockView& V, int NTb, void* work, size_t work_bytes, cudaStream_t s, long long first_task,
               uint64_t timeout_ns, bool allow_emu = true) {
  const bool emu = allow_emu && emu_active(V);
  const size_t need = emu ? emu_workspace_bytes(NTb) : dag_workspace_bytes(NTb);
  if (work == nullptr || work_bytes < need) return GBX_ERR_WORKSPACE;
  DevInfo di;
  if (int e = device_info(di)) return e;
  if (cudaMemsetAsync(work, 0, dag_workspace_bytes(NTb), s) != cudaSuccess) return GBX_ERR_CUDA;
  DagState* st = (DagState*)work;
  if (first_task) set_head_kernel<<<1, 32, 0, s>>>(st, (unsigned long long)first_task);
  DagParams P;
  P.V = V;
  P.NTb = NTb;
  P.ntasks = dag_num_tasks(NTb);
  P.st = st;
  P.cnt = (int*)((char*)work + sizeof(DagState));
  P.timeout_ns = timeout_ns;
  P.trace = current_trace();
  P.planes = nullptr;
  P.rexp = nullptr;
  CUtensorMap ta, tb;
  memset(&ta, 0, sizeof(ta));
  memset(&tb, 0, sizeof(tb));
  if (emu) {
    P.rexp = (int*)((char*)work + emu_rexp_offset(NTb));
    P.planes = (uint16_t*)((char*)work + emu_planes_offset(NTb));
    const uint64_t rows = (uint64_t)NTb * (NTb + 1) / 2 * emu::kSlices * emu::kEdge;
    if (int e = tc::make_tmap_kmajor_bf16(&ta, P.planes, rows, emu::kEdge, emu::kEdge, 128)) return e;
    if (int e = tc::make_tmap_kmajor_bf16(&tb, P.planes, rows, emu::kEdge, emu::kEdge, 64)) return e;
  }
  long long grid = (long long)di.sms * (emu ? 1 : di.dag_blocks_per_sm);
  grid = std::max(1LL, std::min(grid, P.ntasks));
  // emulated updates: a POTRF (~350 us) takes about fourteen update tasks' time (~25 us); 16 tasks
  // per CTA ahead of each step's TRSMs measured best (N=32768: 8/CTA 629 ms, 12 617, 16 606, 24 608;
  // N=16384: 120, 117, 116, 118 ms). The FP64 FMA form keeps its order (its update tasks take
  // longer than a POTRF).
  P.lead = g_dag_lead >= 0 ? g_dag_lead : (emu ? 16 * grid : 0);
  if (emu) potrf_dag_f64_kernel<true><<<(unsigned)grid, emuk::kThreadsEmu, emuk::kSmemBytes, s>>>(ta, tb, P);
  else potrf_dag_f64_kernel<false><<<(unsigned)grid, kThreads, kDagSmemBytes, s>>>(ta, tb, P);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

BlockView tiled_view(int N, int NB, double* tiles) {
  BlockView V;
  V.base = tiles;
  V.N = N;
  V.b = dag_block_edge(N, NB);
  V.ld = NB;
  V.r = NB / V.b;
  V.NT = (N + NB - 1) / NB;
  V.tile_elems = (long long)NB * NB;
  return V;
}

BlockView plain_view(int n, double* A, int lda) {
  BlockView V;
  V.base = A;
  V.N = n;
  V.b = n <= kBlk ? std::max(n, 1) : kBlk;
  V.ld = lda;
  V.r = 1 << 30;
  V.NT = 1;
  V.tile_elems = 0;
  return V;
}

}  // namespace gbx

using namespace gbx;

extern "C" {

long long gbx_dag_task(int NTb, long long t, int* key) { return gbx_dag_task_lead(NTb, 0, t, key); }

long long gbx_dag_task_lead(int NTb, long long lead, long long t, int* key) {
  if (NTb <= 0 || lead < 0) return GBX_ERR_ARG;
  const long long n = dag_num_tasks(NTb);
  if (t >= n || (t >= 0 && !key)) return GBX_ERR_ARG;
  if (t >= 0) {
    const TaskKey k = dag_decode(t, NTb, lead);
    key[0] = k.type;
    key[1] = k.a;
    key[2] = k.b;
    key[3] = k.c;
  }
  return n;
}

int gbx_version(void) { return 100; }
int gbx_built_arch(void) {
#if defined(GBX_ARCH)
  return GBX_ARCH;
#else
  return 0;
#endif
}

void gbx_set_trace_buffer(unsigned long long* buf, int capacity) {
  std::lock_guard<std::mutex> lk(g_mtx);
  g_trace = TraceBuf{capacity > 0 ? buf : nullptr, capacity > 0 ? capacity : 0};
}

void gbx_set_wait_timeout_ns(uint64_t ns) {
  std::lock_guard<std::mutex> lk(g_mtx);
  g_timeout_ns = ns;
}
uint64_t gbx_get_wait_timeout_ns(void) {
  std::lock_guard<std::mutex> lk(g_mtx);
  return g_timeout_ns;
}

int gbx_dpotrf_tile_bufferSize(int n, int lda, size_t* bytes) {
  if (n < 0 || lda < std::max(1, n) || bytes == nullptr) return GBX_ERR_ARG;
  const int b = n <= kBlk ? std::max(n, 1) : kBlk;
  const int NTb = (n + b - 1) / b;
  *bytes = dag_workspace_bytes(std::max(NTb, 1));
  return GBX_OK;
}

int gbx_dpotrf_tile(int n, double* A, int lda, void* work, size_t work_bytes, int* devInfo, void* stream) {
  if (n < 0 || lda < std::max(1, n) || (n > 0 && A == nullptr) || devInfo == nullptr) return GBX_ERR_ARG;
  if (auto* q = taskq::recorder(stream))  // a device task queue's stream: record, do not launch
    return taskq::record(q, taskq::make_op(taskq::OP_POTRF, n, n, 0, nullptr, nullptr, A, 0, 0, lda, devInfo));
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) return cudaMemsetAsync(devInfo, 0, sizeof(int), s) == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
  const BlockView V = plain_view(n, A, lda);
  const int NTb = (n + V.b - 1) / V.b;
  if (int e = launch_dag(V, NTb, work, work_bytes, s, 0, gbx_get_wait_timeout_ns(), false))
    return e;
  copy_info_kernel<<<1, 32, 0, s>>>((const DagState*)work, devInfo);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

int gbx_dtrsm_rlt_tile(int m, int n, const double* L, int ldl, double* B, int ldb, void* stream) {
  if (m < 0 || n < 0 || ldl < std::max(1, n) || ldb < std::max(1, m)) return GBX_ERR_ARG;
  if (m == 0 || n == 0) return GBX_OK;
  if (!L || !B) return GBX_ERR_ARG;
  if (auto* q = taskq::recorder(stream))
    return taskq::record(q, taskq::make_op(taskq::OP_TRSM_RLT, m, n, 0, L, nullptr, B, ldl, 0, ldb));
  DevInfo di;
  if (int e = device_info(di)) return e;
  const size_t smem = op_trsm_smem_elems<double>() * sizeof(double);
  trsm_rlt_grid_kernel<<<(m + kBlk - 1) / kBlk, kThreads, smem, (cudaStream_t)stream>>>(m, n, L, ldl, B, ldb);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

int gbx_dsyrk_ln_tile(int n, int k, const double* A, int lda, double* C, int ldc, void* stream) {
  if (n < 0 || k < 0 || lda < std::max(1, n) || ldc < std::max(1, n)) return GBX_ERR_ARG;
  if (n == 0 || k == 0) return GBX_OK;
  if (!A || !C) return GBX_ERR_ARG;
  if (auto* q = taskq::recorder(stream))
    return taskq::record(q, taskq::make_op(taskq::OP_SYRK_LN, n, n, k, A, nullptr, C, lda, 0, ldc));
  DevInfo di;
  if (int e = device_info(di)) return e;
  const int nb = (n + kBlk - 1) / kBlk;
  const size_t smem = 4 * kKC * kBlk * sizeof(double);
  gemm_nt_grid_kernel<<<nb * (nb + 1) / 2, kThreads, smem, (cudaStream_t)stream>>>(n, n, k, A, lda, A, lda, C, ldc,
                                                                                  1);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

int gbx_dgemm_nt_tile(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc,
                      void* stream) {
  if (m < 0 || n < 0 || k < 0 || lda < std::max(1, m) || ldb < std::max(1, n) || ldc < std::max(1, m))
    return GBX_ERR_ARG;
  if (m == 0 || n == 0 || k == 0) return GBX_OK;
  if (!A || !B || !C) return GBX_ERR_ARG;
  if (auto* q = taskq::recorder(stream))
    return taskq::record(q, taskq::make_op(taskq::OP_GEMM_NT, m, n, k, A, B, C, lda, ldb, ldc));
  DevInfo di;
  if (int e = device_info(di)) return e;
  const size_t smem = 4 * kKC * kBlk * sizeof(double);
  dim3 grid((m + kBlk - 1) / kBlk, (n + kBlk - 1) / kBlk);
  gemm_nt_grid_kernel<<<grid, kThreads, smem, (cudaStream_t)stream>>>(m, n, k, A, lda, B, ldb, C, ldc, 0);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

int gbx_set_dag_block_edge(int b) {
  if (b != 0 && b != 32 && b != 64 && b != kBlk) return GBX_ERR_ARG;
  g_forced_edge = b;
  return GBX_OK;
}

int gbx_dpotrf_tiled_bufferSize(int N, int NB, size_t* bytes) {
  if (N < 0 || NB <= 0 || bytes == nullptr) return GBX_ERR_ARG;
  const int b = dag_block_edge(N, NB);
  if (b == 0) return GBX_ERR_ARG;
  const int NTb = std::max(1, (N + b - 1) / b);
  *bytes = executor_workspace_bytes(tiled_view(std::max(N, 1), NB, nullptr), NTb);
  return GBX_OK;
}

int gbx_set_fp64_update(int mode) {
  if (mode != 0 && mode != 1) return GBX_ERR_ARG;
  g_fp64_update = mode;
  return GBX_OK;
}
int gbx_get_fp64_update(void) { return g_fp64_update; }

int gbx_set_dag_lead(long long tasks) {
  if (tasks < -1) return GBX_ERR_ARG;
  g_dag_lead = tasks;
  return GBX_OK;
}

int gbx_dpotrf_tiled(int N, int NB, double* tiles, void* work, size_t work_bytes, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N < 0 || NB <= 0 || block_edge(NB) == 0) return GBX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (N == 0) {
    if (!work || work_bytes < sizeof(DagState)) return GBX_ERR_WORKSPACE;
    return cudaMemsetAsync(work, 0, sizeof(DagState), s) == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
  }
  if (!tiles) return GBX_ERR_ARG;
  const BlockView V = tiled_view(N, NB, tiles);
  const int NTb = (N + V.b - 1) / V.b;
  return launch_dag(V, NTb, work, work_bytes, s, 0, gbx_get_wait_timeout_ns());
}

int gbx_dpotrf_tiled_status(const void* work, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (!work) return GBX_ERR_ARG;
  int st = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&st, work, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return GBX_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return GBX_ERR_CUDA;
  return st;
}

int gbx_dpotrs_tiled(int N, int NB, const double* tiles, int nrhs, double* B, int ldb, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N < 0 || NB <= 0 || block_edge(NB) == 0 || nrhs < 0 || ldb < std::max(1, N)) return GBX_ERR_ARG;
  if (N == 0 || nrhs == 0) return GBX_OK;
  if (!tiles || !B) return GBX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const BlockView V = tiled_view(N, NB, const_cast<double*>(tiles));
  const int NTb = (N + V.b - 1) / V.b;
  DevInfo di;
  if (int e = device_info(di)) return e;
  // run state and counters of the two sweeps: a per-device buffer, serialised across calls (the
  // previous call's launches are done before this one clears it)
  std::lock_guard<std::mutex> lk(g_solve_mtx);
  SolveScratch& sc = g_solve[di.dev];
  const size_t need = 2 * sizeof(DagState) + (size_t)4 * NTb * sizeof(int);
  if (!sc.ev && cudaEventCreateWithFlags(&sc.ev, cudaEventDisableTiming) != cudaSuccess) return GBX_ERR_CUDA;
  if (sc.bytes < need) {
    if (sc.buf && (cudaEventSynchronize(sc.ev) != cudaSuccess || cudaFree(sc.buf) != cudaSuccess)) return GBX_ERR_CUDA;
    sc.buf = nullptr;
    sc.bytes = 0;
    if (cudaMalloc(&sc.buf, need) != cudaSuccess) return GBX_ERR_CUDA;
    sc.bytes = need;
  }
  if (cudaStreamWaitEvent(s, sc.ev, 0) != cudaSuccess) return GBX_ERR_CUDA;
  DagState* st = (DagState*)sc.buf;
  int* c = (int*)((char*)sc.buf + 2 * sizeof(DagState));
  if (cudaMemsetAsync(sc.buf, 0, need, s) != cudaSuccess) return GBX_ERR_CUDA;
  const long long ntasks = (long long)NTb * (NTb + 1) / 2;
  const int grid = (int)std::max(1LL, std::min<long long>(2LL * di.sms, ntasks));
  const uint64_t tmo = gbx_get_wait_timeout_ns();
  solve_sweep_kernel<0><<<grid, kThreads, 0, s>>>(V, NTb, B, ldb, nrhs, st, c, c + NTb, tmo);
  solve_sweep_kernel<1><<<grid, kThreads, 0, s>>>(V, NTb, B, ldb, nrhs, st + 1, c + 2 * NTb, c + 3 * NTb, tmo);
  if (cudaEventRecord(sc.ev, s) != cudaSuccess) return GBX_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

// ---- factorisation and solve from host buffers -------------------------------------------------
//   copy-in:  one cudaMemcpyAsync of the whole tile array, then one of the right-hand sides, both
//             on the caller's stream ahead of the executor launch (copies interleaved with other
//             stream operations ran many times slower on this platform than one large copy);
//   copy-out: one copy of the whole factor on a second stream once the executor has finished,
//             running beside the solve on the caller's stream (both only read L).
// Host copies of pinned memory run at ~200 GB/s here (4.4 GB of tiles in ~22 ms each way), so the
// copies are a few percent of the step. Streaming L out per column group while the factorisation
// runs, signalled through flags in mapped host memory, was measured slower: the flags became
// visible to the host a quarter of a second late, as stream memory operations did.
namespace {
struct HostCopies {
  cudaStream_t out = nullptr;
  cudaEvent_t ev_kernel = nullptr, ev_out = nullptr;
  int* status = nullptr;  // pinned host copy of the executor's status
  bool ready = false;
};
std::mutex g_host_mtx;
HostCopies g_host[32];

int host_copies(HostCopies*& ho) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 32) return GBX_ERR_CUDA;
  HostCopies& h = g_host[dev];
  ho = &h;
  if (h.ready) return GBX_OK;
  if (cudaStreamCreateWithFlags(&h.out, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h.ev_kernel, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h.ev_out, cudaEventDisableTiming) != cudaSuccess ||
      cudaHostAlloc((void**)&h.status, sizeof(int), cudaHostAllocDefault) != cudaSuccess)
    return GBX_ERR_CUDA;
  h.ready = true;
  return GBX_OK;
}
}  // namespace

int gbx_dposv_tiled_host_bufferSize(int N, int NB, size_t* bytes) {
  if (N <= 0 || NB <= 0 || block_edge(NB) == 0 || !bytes) return GBX_ERR_ARG;
  return gbx_dpotrf_tiled_bufferSize(N, NB, bytes);
}

int gbx_dposv_tiled_host(int N, int NB, const double* A_host, double* L_host, int nrhs, const double* B_host,
                         double* X_host, double* tiles, double* X, void* work, size_t work_bytes, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  size_t need = 0;
  if (int e = gbx_dposv_tiled_host_bufferSize(N, NB, &need)) return e;
  if (nrhs < 0 || !A_host || !L_host || !tiles || (nrhs > 0 && (!B_host || !X_host || !X))) return GBX_ERR_ARG;
  if (!work || work_bytes < need) return GBX_ERR_WORKSPACE;
  std::lock_guard<std::mutex> lk(g_host_mtx);  // one caller at a time on the shared copy stream and events
  HostCopies* h = nullptr;
  if (int e = host_copies(h)) return e;
  cudaStream_t s = (cudaStream_t)stream;
  const BlockView V = tiled_view(N, NB, tiles);
  const int NTb = (N + V.b - 1) / V.b, NT = V.NT;
  const size_t tile_bytes = ((size_t)NT * (NT + 1) / 2) * (size_t)NB * NB * sizeof(double);
  if (cudaMemcpyAsync(tiles, A_host, tile_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) return GBX_ERR_CUDA;
  if (nrhs > 0 &&
      cudaMemcpyAsync(X, B_host, (size_t)N * nrhs * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return GBX_ERR_CUDA;
  if (int e = launch_dag(V, NTb, work, need, s, 0, gbx_get_wait_timeout_ns())) return e;
  // the status first (behind the 4.4 GB copy of L it would wait ~20 ms for the copy engine)
  if (cudaMemcpyAsync(h->status, work, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaEventRecord(h->ev_kernel, s) != cudaSuccess)
    return GBX_ERR_CUDA;
  // L goes back on the copy stream as soon as the executor is done
  if (cudaStreamWaitEvent(h->out, h->ev_kernel, 0) != cudaSuccess ||
      cudaMemcpyAsync(L_host, tiles, tile_bytes, cudaMemcpyDeviceToHost, h->out) != cudaSuccess ||
      cudaEventRecord(h->ev_out, h->out) != cudaSuccess)
    return GBX_ERR_CUDA;
  // the factorisation's status decides on the solve: wait for the executor
  if (cudaEventSynchronize(h->ev_kernel) != cudaSuccess) return GBX_ERR_CUDA;
  const int st = *(volatile int*)h->status;
  if (st != 0) {  // bad pivot or timed-out wait: no solve on a partial factor; L_host gets it anyway
    if (cudaEventSynchronize(h->ev_out) != cudaSuccess) return GBX_ERR_CUDA;
    return st;
  }
  if (nrhs > 0) {
    if (int e = gbx_dpotrs_tiled(N, NB, tiles, nrhs, X, N, stream)) return e;
    if (cudaMemcpyAsync(X_host, X, (size_t)N * nrhs * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return GBX_ERR_CUDA;
  }
  return cudaStreamWaitEvent(s, h->ev_out, 0) == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

static int gen_tiles(int N, int NB, int kind, double v, unsigned long long seed, double* tiles, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N < 0 || NB <= 0) return GBX_ERR_ARG;
  if (N == 0) return GBX_OK;
  if (!tiles) return GBX_ERR_ARG;
  const int NT = (N + NB - 1) / NB;
  if (NT > 65535) return GBX_ERR_ARG;
  const long long per_tile = (long long)NB * NB;
  dim3 grid((unsigned)((per_tile + 255) / 256), NT, NT);
  gen_tiles_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(N, NB, NT, kind, v, seed, tiles);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

int gbx_dplgsy_tiled(int N, int NB, double bump, unsigned long long seed, double* tiles, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  return gen_tiles(N, NB, 0, bump, seed, tiles, stream);
}

int gbx_dgen_uniform_sym_tiled(int N, int NB, unsigned long long seed, double shift, double* tiles, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  return gen_tiles(N, NB, 1, shift, seed, tiles, stream);
}

int gbx_dplgsy_tile(double bump, int m, int n, double* A, int lda, int gM, int m0, int n0, unsigned long long seed,
                    void* stream) {
  if (m < 0 || n < 0 || lda < std::max(1, m) || m0 < 0 || n0 < 0 || gM < 0) return GBX_ERR_ARG;
  if (m == 0 || n == 0) return GBX_OK;
  if (!A) return GBX_ERR_ARG;
  if (auto* q = taskq::recorder(stream)) {  // a device task queue's stream: record, do not launch
    taskq::Op o = taskq::make_op(taskq::OP_PLGSY, m, n, 0, nullptr, nullptr, A, 0, 0, lda);
    o.gM = gM;
    o.g0 = m0;
    o.g1 = n0;
    o.bump = bump;
    o.seed = seed;
    return taskq::record(q, o);
  }
  const long long total = (long long)m * n;
  plgsy_tile_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(bump, m, n, A, lda, gM, m0, n0,
                                                                                       seed);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

int gbx_dgen_lowrank_sym_tiled(int N, int NB, const double* lam, const double* U, const double* V, const double* G,
                               int r, double* tiles, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N <= 0 || NB <= 0 || r < 0 || r > 8 || !lam || (r > 0 && (!U || !V || !G)) || !tiles) return GBX_ERR_ARG;
  const int NT = (N + NB - 1) / NB;
  if (NT > 65535) return GBX_ERR_ARG;
  dim3 grid((unsigned)(((long long)NB * NB + 255) / 256), NT, NT);
  gen_lowrank_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(N, NB, NT, lam, U, V, G, r, tiles);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

// ---- allocation-free variant of gbx_dpotrf_tiled ---------------------------------------------------
// Some callers cannot call cudaMalloc: code whose device memory belongs to another allocator or is
// budgeted up front (a host framework's caching allocator, a fixed memory reservation), and code on
// latency-critical paths where cudaMalloc/cudaFree's implicit device synchronisation is not
// acceptable. For them the executor's scratch (run header + one completion counter per 128 x 128
// block) lives in this file-scope device array instead of a caller workspace. Every GPU that loads
// the library holds it until the process exits.
}  // extern "C"

namespace gbx {
constexpr int kNoAllocMaxNTb = 512;  // at most 512 blocks per edge: N <= 65536 (blocks of 128)
constexpr size_t kNoAllocBytes = sizeof(DagState) + (size_t)kNoAllocMaxNTb * (kNoAllocMaxNTb + 1) / 2 * sizeof(int);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];  // 525,376 bytes

std::mutex g_noalloc_mtx;
std::vector<void*> g_noalloc_ptr;  // device address of g_noalloc_scratch, per device

// One-time set-up per device, with that device current: the symbol's device address. In host code
// the array's name is only a host-side stand-in and must never be passed to a kernel. The address
// is kept for the life of the process; a cudaDeviceReset of the device would make it stale.
int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBX_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_noalloc_mtx);
  if ((int)g_noalloc_ptr.size() <= dev) g_noalloc_ptr.resize(dev + 1, nullptr);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GBX_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return GBX_OK;
}
}  // namespace gbx

extern "C" {

int gbx_dpotrf_tiled_noalloc(int N, int NB, double* tiles, int* devInfo, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (N < 0 || NB <= 0 || block_edge(NB) == 0 || !devInfo || (N > 0 && !tiles)) return GBX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (N == 0) return cudaMemsetAsync(devInfo, 0, sizeof(int), s) == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
  const BlockView V = tiled_view(N, NB, tiles);
  const int NTb = (N + V.b - 1) / V.b;
  if (NTb > kNoAllocMaxNTb) return GBX_ERR_NOALLOC_LIMIT;
  void* scratch = nullptr;
  if (int e = noalloc_scratch(&scratch)) return e;
  // launch_dag clears the header and the counters this run uses (cudaMemsetAsync, no allocation)
  if (int e = launch_dag(V, NTb, scratch, kNoAllocBytes, s, 0, gbx_get_wait_timeout_ns(), false))
    return e;
  copy_info_kernel<<<1, 32, 0, s>>>((const DagState*)scratch, devInfo);
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

int gbx_dag_timeout_selftest(int NB, double* tiles, void* work, size_t work_bytes, uint64_t timeout_ns,
                             void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (NB <= 0 || NB > kBlk || !tiles) return GBX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const BlockView V = tiled_view(2 * NB, NB, tiles);
  // skip task 0 (POTRF(0)): TRSM(1,0) then waits for a counter nothing will ever move
  if (int e = launch_dag(V, 2, work, work_bytes, s, 1, timeout_ns, false)) return e;
  return gbx_dpotrf_tiled_status(work, stream);
}

}  // extern "C"
