// Internal interface of the device task queue (taskq.cu) to the tile entry points: a stream handle
// from gbx_taskq_stream makes a tile entry point record its operation instead of launching it.
#pragma once
#include <cuda_runtime.h>

namespace gbx {
namespace taskq {

enum OpType : int {
  OP_POTRF = 0,
  OP_TRSM_RLT = 1,
  OP_SYRK_LN = 2,
  OP_GEMM_NT = 3,
  OP_TRSM_RLN = 4,
  OP_GEMM_NN = 5,
  OP_PLGSY = 6
};

// One recorded tile operation (FP64, column-major tiles):
//   POTRF     C (n x n, ldc) := chol(C), *info := 0 or the first bad pivot
//   TRSM_RLT  C (m x n) := C A^{-T}, A lower n x n
//   SYRK_LN   C (n x n) -= A A^T (lower), A n x k
//   GEMM_NT   C (m x n) -= A B^T, A m x k, B n x k
//   TRSM_RLN  C (m x n) := C A^{-1}, A lower n x n
//   GEMM_NN   C (m x n) -= A B, A m x k, B k x n
//   PLGSY     C (m x n) := rows g0.., columns g1.. of the gM x gM PLASMA test matrix (seed), with
//             `bump` added to its diagonal (gbx_dplgsy_tile)
struct Op {
  int type, m, n, k;
  const double* A;
  const double* B;
  double* C;
  int lda, ldb, ldc, gM;
  int* info;
  double bump;
  unsigned long long seed;
  int g0, g1;
};

struct Queue;
/// The queue a stream handle records into, or null for an ordinary stream (never dereferenced).
Queue* recorder(const void* stream);
/// Appends an operation; returns GBX_OK or an error status.
int record(Queue* q, const Op& op);
/// An operation with only the fields of the first group set (the PLGSY fields zero).
inline Op make_op(int type, int m, int n, int k, const double* A, const double* B, double* C, int lda, int ldb, int ldc,
                  int* info = nullptr) {
  Op o{};
  o.type = type;
  o.m = m;
  o.n = n;
  o.k = k;
  o.A = A;
  o.B = B;
  o.C = C;
  o.lda = lda;
  o.ldb = ldb;
  o.ldc = ldc;
  o.info = info;
  return o;
}

}  // namespace taskq
}  // namespace gbx
