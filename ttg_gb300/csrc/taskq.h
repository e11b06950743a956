// Internal interface of the device task queue (taskq.cu) to the tile entry points: a stream handle
// from gbx_taskq_stream makes a tile entry point record its operation instead of launching it.
#pragma once
#include <cuda_runtime.h>

namespace gbx {
namespace taskq {

enum OpType : int { OP_POTRF = 0, OP_TRSM_RLT = 1, OP_SYRK_LN = 2, OP_GEMM_NT = 3, OP_TRSM_RLN = 4, OP_GEMM_NN = 5 };

// One recorded tile operation (FP64, column-major tiles):
//   POTRF     C (n x n, ldc) := chol(C), *info := 0 or the first bad pivot
//   TRSM_RLT  C (m x n) := C A^{-T}, A lower n x n
//   SYRK_LN   C (n x n) -= A A^T (lower), A n x k
//   GEMM_NT   C (m x n) -= A B^T, A m x k, B n x k
//   TRSM_RLN  C (m x n) := C A^{-1}, A lower n x n
//   GEMM_NN   C (m x n) -= A B, A m x k, B k x n
struct Op {
  int type, m, n, k;
  const double* A;
  const double* B;
  double* C;
  int lda, ldb, ldc, pad;
  int* info;
};

struct Queue;
/// The queue a stream handle records into, or null for an ordinary stream (never dereferenced).
Queue* recorder(const void* stream);
/// Appends an operation; returns GBX_OK or an error status.
int record(Queue* q, const Op& op);

}  // namespace taskq
}  // namespace gbx
