// Shared device helpers of the GB300 tiled-Cholesky library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbx_potrf.h"

namespace gbx {

namespace taskq {
struct Queue;
Queue* recorder(const void* stream);  // taskq.cu: the device task queue a stream handle records into
}
/// True for the recording stream handle of a device task queue: entry points that cannot record
/// reject it (it is not a CUDA stream).
inline bool recording_stream(const void* stream) { return taskq::recorder(stream) != nullptr; }

// ---- memory-model helpers -------------------------------------------------------------------
__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- run state shared by all CTAs of one executor launch (lives in the caller's workspace) ---
struct DagState {
  int status;              // 0, >0 first bad pivot (1-based global), or GBX_ERR_TIMEOUT
  int abort;               // set when any CTA must stop
  int pad[2];
  unsigned long long head; // next task index of the device ready queue
  unsigned long long pad2[5];
};
static_assert(sizeof(DagState) == 64, "DagState must stay one 64-byte header");

// Waits until *cnt >= target. Returns false when the run was aborted or the wait ran out of
// time (then status := GBX_ERR_TIMEOUT and abort := 1). Called by one thread of the CTA.
__device__ __forceinline__ bool wait_geq(const int* cnt, int target, DagState* st, uint64_t timeout_ns) {
  if (ld_acquire_gpu(cnt) >= target) return true;
  const uint64_t t0 = globaltimer_ns();
  // iteration cap as a second bound in case the timer misbehaves (~2^31 * >=32ns)
  for (uint32_t it = 0; it < 0x7fffffffu; ++it) {
    if (ld_acquire_gpu(cnt) >= target) return true;
    if (ld_volatile(&st->abort)) return false;
    if (globaltimer_ns() - t0 > timeout_ns) break;
    __nanosleep(it < 64 ? 32 : 256);
  }
  atomicCAS(&st->status, 0, GBX_ERR_TIMEOUT);
  atomicExch(&st->abort, 1);
  return false;
}

// Completion signal: every write of the CTA to the block is made visible before the counter moves.
__device__ __forceinline__ void signal_done(int* cnt) {
  __threadfence();
  atomicAdd(cnt, 1);
}

// ---- optional per-task timeline ----------------------------------------------------------------
// buf[0] counts records; record i (i >= 0) occupies buf[2 + 4i .. 5 + 4i]:
//   start ns, end ns (globaltimer), key = type << 60 | a << 40 | b << 20 | c, sub << 32 | cta
struct TraceBuf {
  unsigned long long* buf;
  int cap;
};
__device__ __forceinline__ void trace_record(const TraceBuf& tb, uint64_t t0, int type, int a, int b, int c, int sub) {
  if (!tb.buf) return;
  const unsigned long long i = atomicAdd(tb.buf, 1ULL);
  if (i >= (unsigned long long)tb.cap) return;
  unsigned long long* r = tb.buf + 2 + 4 * i;
  r[0] = t0;
  r[1] = globaltimer_ns();
  r[2] = ((unsigned long long)type << 60) | ((unsigned long long)(a & 0xFFFFF) << 40) |
         ((unsigned long long)(b & 0xFFFFF) << 20) | (unsigned long long)(c & 0xFFFFF);
  r[3] = ((unsigned long long)(unsigned)sub << 32) | (unsigned long long)blockIdx.x;
}
TraceBuf current_trace();  // set by gbx_set_trace_buffer (host)

// ---- addressing of b x b blocks inside NB x NB tiles of the tile-major lower storage ---------
// A plain column-major matrix is the special case of a single tile (NT = 1) whose leading
// dimension is the matrix's lda.
struct BlockView {
  double* base;
  int N;   // matrix order
  int b;   // block edge
  int ld;  // leading dimension inside a tile (NB for tiled storage, lda for a plain matrix)
  int r;   // blocks per tile edge (NB / b); huge for a plain matrix
  int NT;  // tiles per edge (1 for a plain matrix)
  long long tile_elems;  // elements per tile slot (NB*NB)

  __host__ __device__ __forceinline__ double* ptr(int I, int J) const {
    const int m = I / r, n = J / r;
    const long long slot = (long long)n * NT - (long long)n * (n - 1) / 2 + (m - n);
    return base + slot * tile_elems + (long long)(I % r) * b + (long long)(J % r) * b * (long long)ld;
  }
  __host__ __device__ __forceinline__ int dim(int I) const {
    const int d = N - I * b;
    return d < b ? d : b;
  }
};

__host__ __device__ __forceinline__ long long tri_index(int I, int J, int NTb) {
  // packed lower index of block (I,J), I >= J, column by column
  return (long long)J * NTb - (long long)J * (J - 1) / 2 + (I - J);
}

}  // namespace gbx
