// Device task queue: the persistent device-side ready queue behind the TTG API's device tasks.
//
// While a TTG device task body runs with a queue's recording stream as its current stream, the tile
// entry points (gbx_dpotrf_tile, gbx_dtrsm_rlt_tile, gbx_dsyrk_ln_tile, gbx_dgemm_nt_tile,
// gbx_dtrsm_rln_tile, gbx_dgemm_nn_tile) append their operation to the queue instead of launching a
// kernel. The dependencies come from the operands: an operation waits for the last writer of every
// tile it reads or writes and for the readers of every tile it writes since that writer (the
// buffers of the flowgraph's values are distinct allocations, so a tile is its base pointer).
// gbx_taskq_run launches ONE persistent kernel over everything recorded since the previous run:
// 152 CTAs take sub-tasks (128 x 128 blocks of an operation's output) from a device-side queue in
// recording order and wait, with a time limit, on per-operation completion counters. Recording order
// is a topological order (a task body runs only after its inputs were sent, and its operation is
// recorded before its own sends), so in-order grabbing cannot deadlock. This replaces the
// reference's per-task hand-off to PaRSEC's device manager (parsec/ttg.h:1521-1672, 2678-2727).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "block_ops.cuh"
#include "gbx_common.cuh"
#include "gbx_potrf.h"
#include "plgsy.cuh"
#include "taskq.h"

namespace gbx {
namespace taskq {

constexpr int kMaxQueues = 64;
constexpr int kRlnRows = 8;  // rows of a TRSM_RLN sub-task (one warp each)

struct Queue {
  int id = -1;
  std::mutex m;
  std::vector<Op> ops;                                   // recorded, not yet run
  long long first = 0;                                   // global index of ops[0]
  struct Tile {
    long long writer = -1;
    std::vector<long long> readers;
  };
  std::unordered_map<const void*, Tile> tiles;           // dependency state per tile (global op indices)
  std::vector<std::vector<long long>> preds;             // per recorded op, global predecessor indices
  // device side of the last run
  void* dbuf = nullptr;
  size_t dbytes = 0;
  cudaStream_t last_stream = nullptr;
  int sms = 0;
};

std::mutex g_reg_mtx;
Queue* g_queues[kMaxQueues] = {};
char g_tags[kMaxQueues];  // stream handles of the queues: addresses inside this array

Queue* recorder(const void* stream) {
  const char* p = static_cast<const char*>(stream);
  if (p < g_tags || p >= g_tags + kMaxQueues) return nullptr;
  return g_queues[p - g_tags];
}

int nsub_of(const Op& o) {
  const auto nb = [](int x) { return (x + kBlk - 1) / kBlk; };
  switch (o.type) {
    case OP_POTRF: return 1;
    case OP_TRSM_RLT: return nb(o.m);
    case OP_SYRK_LN: return nb(o.n) * (nb(o.n) + 1) / 2;
    case OP_GEMM_NT: return nb(o.m) * nb(o.n);
    case OP_TRSM_RLN: return (o.m + kRlnRows - 1) / kRlnRows;
    default: return nb(o.n);  // OP_GEMM_NN, OP_PLGSY: column blocks of C
  }
}

int record(Queue* q, const Op& op) {
  std::lock_guard<std::mutex> lk(q->m);
  const long long me = q->first + (long long)q->ops.size();
  std::vector<long long> pred;
  auto reads = [&](const void* p) {
    if (!p) return;
    auto& t = q->tiles[p];
    if (t.writer >= 0) pred.push_back(t.writer);
    t.readers.push_back(me);
  };
  auto writes = [&](const void* p) {
    auto& t = q->tiles[p];
    if (t.writer >= 0) pred.push_back(t.writer);
    for (long long r : t.readers)
      if (r != me) pred.push_back(r);
    t.readers.clear();
    t.writer = me;
  };
  reads(op.A);
  if (op.type == OP_GEMM_NT || op.type == OP_GEMM_NN) reads(op.B);
  writes(op.C);
  std::sort(pred.begin(), pred.end());
  pred.erase(std::unique(pred.begin(), pred.end()), pred.end());
  q->ops.push_back(op);
  q->preds.push_back(std::move(pred));
  return GBX_OK;
}

// ---- device side ----------------------------------------------------------------------------------
struct DevOp {
  Op op;
  int nsub, npred;
  long long sub0, pred0;  // first sub-task (queue position), first entry in the predecessor array
};

struct RunParams {
  const DevOp* ops;
  int nops;
  long long ntasks;
  const int* pred;  // predecessor op indices (within the run)
  int* done;        // per op: finished sub-tasks
  DagState* st;
  uint64_t timeout_ns;
};

// C (m x n) := C L^{-1} for rows [r0, r0 + 8) of C: one warp per row, columns from the last one down
__device__ void rln_rows(const Op& o, int r0, double* xs) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = r0 + warp;
  if (warp < kRlnRows && r < o.m) {
    double* x = xs + (size_t)warp * o.n;
    for (int c = lane; c < o.n; c += 32) x[c] = __ldcg(o.C + r + (long long)c * o.ldc);
    __syncwarp();
    for (int c = o.n - 1; c >= 0; --c) {
      const double* Lc = o.A + (long long)c * o.lda;
      double s = 0.0;
      for (int k = c + 1 + lane; k < o.n; k += 32) s = fma(x[k], __ldcg(Lc + k), s);
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) x[c] = (x[c] - s) / __ldcg(Lc + c);
      __syncwarp();
    }
    for (int c = lane; c < o.n; c += 32) o.C[r + (long long)c * o.ldc] = x[c];
  }
  __syncthreads();
}

// C(:, c0 : c0 + 128) -= A B(:, c0 : c0 + 128), every thread a strided set of elements
__device__ void gemm_nn_cols(const Op& o, int c0) {
  const int nc = min(kBlk, o.n - c0);
  for (int idx = threadIdx.x; idx < o.m * nc; idx += kThreads) {
    const int i = idx % o.m, j = c0 + idx / o.m;
    double acc = 0.0;
    for (int q = 0; q < o.k; ++q) acc = fma(__ldcg(o.A + i + (long long)q * o.lda), __ldcg(o.B + q + (long long)j * o.ldb), acc);
    o.C[i + (long long)j * o.ldc] = __ldcg(o.C + i + (long long)j * o.ldc) - acc;
  }
  __syncthreads();
}

// columns [c0, c0 + 128) of a tile of the PLASMA test matrix (gbx_dplgsy_tile's entries)
__device__ void plgsy_cols(const Op& o, int c0) {
  const int nc = min(kBlk, o.n - c0);
  for (int idx = threadIdx.x; idx < o.m * nc; idx += kThreads) {
    const int i = idx % o.m, j = c0 + idx / o.m;
    const long long gi = (long long)o.g0 + i, gj = (long long)o.g1 + j;
    const long long hi = gi >= gj ? gi : gj, lo = gi >= gj ? gj : gi;
    double v = plgsy_entry(lcg_jump_dev((unsigned long long)hi + (unsigned long long)lo * (unsigned long long)o.gM, o.seed));
    if (gi == gj) v = __dadd_rn(v, o.bump);
    o.C[i + (long long)j * o.ldc] = v;
  }
  __syncthreads();
}

// Cholesky of the whole tile on one CTA: right-looking over 128-block panels
__device__ void potrf_tile(const Op& o, double* sm) {
  const int n = o.n, nb = (n + kBlk - 1) / kBlk;
  double* A = o.C;
  const int ld = o.ldc;
  auto blk = [&](int i, int j) { return A + (long long)kBlk * i + (long long)kBlk * j * ld; };
  auto dim = [&](int i) { return min(kBlk, n - kBlk * i); };
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int p = 0; p < nb; ++p) {
    const int info = op_potrf<double>(blk(p, p), ld, dim(p), sm);
    if (threadIdx.x == 0) s_bad = info ? p * kBlk + info : 0;
    __syncthreads();
    if (s_bad) break;
    for (int i = p + 1; i < nb; ++i) {
      op_trsm<double>(blk(p, p), ld, blk(i, p), ld, dim(i), dim(p), sm);
      __syncthreads();
    }
    for (int j = p + 1; j < nb; ++j)
      for (int i = j; i < nb; ++i) {
        op_gemm_nt<double>(blk(i, p), ld, blk(j, p), ld, blk(i, j), ld, dim(i), dim(j), dim(p), i == j, sm);
        __syncthreads();
      }
  }
  if (threadIdx.x == 0 && o.info) *o.info = s_bad;
  __syncthreads();
}

__device__ void run_sub(const Op& o, int s, double* sm) {
  const auto nb = [](int x) { return (x + kBlk - 1) / kBlk; };
  switch (o.type) {
    case OP_POTRF:
      potrf_tile(o, sm);
      return;
    case OP_TRSM_RLT: {
      const int r0 = s * kBlk;
      op_trsm<double>(o.A, o.lda, o.C + r0, o.ldc, min(kBlk, o.m - r0), o.n, sm);
      __syncthreads();
      return;
    }
    case OP_SYRK_LN: {
      int j = 0, rem = s;  // the s-th lower block (i, j), column by column
      while (rem >= nb(o.n) - j) rem -= nb(o.n) - j++;
      const int i = j + rem;
      op_gemm_nt<double>(o.A + (long long)i * kBlk, o.lda, o.A + (long long)j * kBlk, o.lda,
                         o.C + (long long)i * kBlk + (long long)j * kBlk * o.ldc, o.ldc, min(kBlk, o.n - i * kBlk),
                         min(kBlk, o.n - j * kBlk), o.k, i == j, sm);
      __syncthreads();
      return;
    }
    case OP_GEMM_NT: {
      const int i = s % nb(o.m), j = s / nb(o.m);
      op_gemm_nt<double>(o.A + (long long)i * kBlk, o.lda, o.B + (long long)j * kBlk, o.ldb,
                         o.C + (long long)i * kBlk + (long long)j * kBlk * o.ldc, o.ldc, min(kBlk, o.m - i * kBlk),
                         min(kBlk, o.n - j * kBlk), o.k, false, sm);
      __syncthreads();
      return;
    }
    case OP_TRSM_RLN:
      rln_rows(o, s * kRlnRows, sm);
      return;
    case OP_PLGSY:
      plgsy_cols(o, s * kBlk);
      return;
    default:
      gemm_nn_cols(o, s * kBlk);
      return;
  }
}

__global__ void __launch_bounds__(kThreads, 1) taskq_kernel(RunParams P) {
  extern __shared__ __align__(16) double smem_d[];
  __shared__ long long s_t;
  __shared__ int s_op, s_ok;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      long long t = -1;
      if (!ld_volatile(&P.st->abort)) t = (long long)atomicAdd(&P.st->head, 1ULL);
      s_t = (t >= 0 && t < P.ntasks) ? t : -1;
      if (s_t >= 0) {
        int lo = 0, hi = P.nops - 1;  // the last operation with sub0 <= t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (P.ops[mid].sub0 <= t) lo = mid;
          else hi = mid - 1;
        }
        s_op = lo;
        bool ok = true;
        const DevOp& d = P.ops[lo];
        for (int q = 0; q < d.npred && ok; ++q) {
          const int p = P.pred[d.pred0 + q];
          ok = wait_geq(P.done + p, P.ops[p].nsub, P.st, P.timeout_ns);
        }
        s_ok = ok;
      }
    }
    __syncthreads();
    if (s_t < 0 || !s_ok) break;
    const DevOp& d = P.ops[s_op];
    run_sub(d.op, (int)(s_t - d.sub0), smem_d);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) signal_done(P.done + s_op);
  }
}

constexpr size_t kSmem = (size_t)kBlk * kBlk * sizeof(double) + 64;  // op_potrf<double>, the largest

}  // namespace taskq
}  // namespace gbx

using namespace gbx;
using namespace gbx::taskq;

extern "C" int gbx_taskq_create(void** q) {
  if (!q) return GBX_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_reg_mtx);
  for (int i = 0; i < kMaxQueues; ++i)
    if (!g_queues[i]) {
      Queue* nq = new Queue();
      nq->id = i;
      g_queues[i] = nq;
      *q = nq;
      return GBX_OK;
    }
  return GBX_ERR_ARG;  // too many live queues
}

extern "C" int gbx_taskq_destroy(void* q) {
  if (!q) return GBX_ERR_ARG;
  Queue* Q = static_cast<Queue*>(q);
  {
    std::lock_guard<std::mutex> lk(g_reg_mtx);
    if (Q->id < 0 || g_queues[Q->id] != Q) return GBX_ERR_ARG;
    g_queues[Q->id] = nullptr;
  }
  if (Q->dbuf) {
    if (Q->last_stream) cudaStreamSynchronize(Q->last_stream);
    cudaFree(Q->dbuf);
  }
  delete Q;
  return GBX_OK;
}

extern "C" void* gbx_taskq_stream(void* q) {
  Queue* Q = static_cast<Queue*>(q);
  return (Q && Q->id >= 0) ? (void*)(g_tags + Q->id) : nullptr;
}

extern "C" long long gbx_taskq_pending(void* q) {
  if (!q) return GBX_ERR_ARG;
  Queue* Q = static_cast<Queue*>(q);
  std::lock_guard<std::mutex> lk(Q->m);
  return (long long)Q->ops.size();
}

extern "C" int gbx_taskq_run(void* q, void* stream) {
  if (!q) return GBX_ERR_ARG;
  Queue* Q = static_cast<Queue*>(q);
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<Op> ops;
  std::vector<std::vector<long long>> preds;
  long long first = 0;
  {
    std::lock_guard<std::mutex> lk(Q->m);
    ops.swap(Q->ops);
    preds.swap(Q->preds);
    first = Q->first;
    Q->first += (long long)ops.size();
  }
  if (ops.empty()) return GBX_OK;
  if (!Q->sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&Q->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaFuncSetAttribute(taskq_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem) != cudaSuccess)
      return GBX_ERR_CUDA;
  }
  // the run's tables: operations with their sub-task ranges, predecessors within this run
  const int nops = (int)ops.size();
  std::vector<DevOp> d(nops);
  std::vector<int> pr;
  long long ntasks = 0;
  for (int j = 0; j < nops; ++j) {
    d[j].op = ops[j];
    d[j].nsub = nsub_of(ops[j]);
    d[j].sub0 = ntasks;
    d[j].pred0 = (long long)pr.size();
    ntasks += d[j].nsub;
    for (long long p : preds[j])
      if (p >= first) pr.push_back((int)(p - first));  // earlier runs are complete
    d[j].npred = (int)(pr.size() - d[j].pred0);
  }
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t o_ops = up(sizeof(DagState)), o_pred = o_ops + up(d.size() * sizeof(DevOp)),
               o_done = o_pred + up(std::max<size_t>(1, pr.size()) * sizeof(int)),
               total = o_done + up((size_t)nops * sizeof(int));
  if (total > Q->dbytes) {  // grow: the previous run may still read the old tables
    if (Q->dbuf) {
      if (Q->last_stream && cudaStreamSynchronize(Q->last_stream) != cudaSuccess) return GBX_ERR_CUDA;
      cudaFree(Q->dbuf);
      Q->dbuf = nullptr;
    }
    const size_t cap = std::max(total, 2 * Q->dbytes);
    if (cudaMalloc(&Q->dbuf, cap) != cudaSuccess) return GBX_ERR_CUDA;
    Q->dbytes = cap;
  }
  char* b = static_cast<char*>(Q->dbuf);
  if (cudaMemsetAsync(b, 0, sizeof(DagState), s) != cudaSuccess ||
      cudaMemsetAsync(b + o_done, 0, (size_t)nops * sizeof(int), s) != cudaSuccess ||
      cudaMemcpyAsync(b + o_ops, d.data(), d.size() * sizeof(DevOp), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      (!pr.empty() &&
       cudaMemcpyAsync(b + o_pred, pr.data(), pr.size() * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess))
    return GBX_ERR_CUDA;
  RunParams P;
  P.ops = (const DevOp*)(b + o_ops);
  P.nops = nops;
  P.ntasks = ntasks;
  P.pred = (const int*)(b + o_pred);
  P.done = (int*)(b + o_done);
  P.st = (DagState*)b;
  P.timeout_ns = gbx_get_wait_timeout_ns();
  const int grid = (int)std::max(1LL, std::min<long long>(Q->sms, ntasks));
  taskq_kernel<<<grid, kThreads, kSmem, s>>>(P);
  Q->last_stream = s;
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}

extern "C" int gbx_taskq_status(void* q, void* stream) {
  if (!q) return GBX_ERR_ARG;
  Queue* Q = static_cast<Queue*>(q);
  if (!Q->dbuf) return GBX_OK;
  int st = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&st, Q->dbuf, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return GBX_ERR_CUDA;
  return st;
}
