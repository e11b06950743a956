// The LAPACK/BLAS calls of the reference's host potrf bodies and of its checker, routed to the
// oracle's plain-loop tile kernels (oracle.cpp) — TEST INFRASTRUCTURE ONLY. Only the operand
// combinations the potrf example uses are provided; anything else aborts.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "oracle.h"

namespace blas {
enum class Layout { ColMajor, RowMajor };
enum class Side { Left, Right };
enum class Op { NoTrans, Trans, ConjTrans };
enum class Diag { NonUnit, Unit };
enum class Uplo { Lower, Upper, General };

[[noreturn]] inline void unsupported(const char* what) {
  std::fprintf(stderr, "lapack shim: unsupported %s\n", what);
  std::abort();
}

inline void trsm(Layout, Side side, Uplo uplo, Op op, Diag diag, int64_t m, int64_t n, double alpha, const double* A,
                 int64_t lda, double* B, int64_t ldb) {
  if (side != Side::Right || uplo != Uplo::Lower || op != Op::Trans || diag != Diag::NonUnit || alpha != 1.0)
    unsupported("trsm");
  orc_trsm_rlt_tile((int)m, (int)n, A, (int)lda, B, (int)ldb);
}
inline void syrk(Layout, Uplo uplo, Op op, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                 double beta, double* C, int64_t ldc) {
  if (uplo != Uplo::Lower || op != Op::NoTrans || alpha != -1.0 || beta != 1.0) unsupported("syrk");
  orc_syrk_ln_tile((int)n, (int)k, A, (int)lda, C, (int)ldc);
}
inline void gemm(Layout, Op opa, Op opb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
                 const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
  if (opa != Op::NoTrans || opb != Op::Trans || alpha != -1.0 || beta != 1.0) unsupported("gemm");
  orc_gemm_nt_tile((int)m, (int)n, (int)k, A, (int)lda, B, (int)ldb, C, (int)ldc);
}
// B := B * op(A), A lower, Right side (the checker's LL^T product, testing_dpotrf.cc:296-297)
inline void trmm(Layout, Side side, Uplo uplo, Op op, Diag diag, int64_t m, int64_t n, double alpha, const double* A,
                 int64_t lda, double* B, int64_t ldb) {
  if (side != Side::Right || uplo != Uplo::Lower || op == Op::NoTrans || diag != Diag::NonUnit) unsupported("trmm");
  // B(i,:) := alpha * B(i,:) * A^T ; A lower => (B A^T)(i,j) = sum_{k<=j} B(i,k) A(j,k)
  std::vector<double> row(n);
  for (int64_t i = 0; i < m; ++i) {
    for (int64_t j = 0; j < n; ++j) {
      double s = 0.0;
      for (int64_t k = 0; k <= j; ++k) s += B[i + k * ldb] * A[j + k * lda];
      row[j] = alpha * s;
    }
    for (int64_t j = 0; j < n; ++j) B[i + j * ldb] = row[j];
  }
}
inline double nrm2(int64_t n, const double* x, int64_t incx) {
  double s = 0;
  for (int64_t i = 0; i < n; ++i) s += x[i * incx] * x[i * incx];
  return std::sqrt(s);
}
}  // namespace blas

namespace lapack {
using blas::Uplo;
enum class Norm { One, Inf, Fro, Max };
inline int64_t potrf(Uplo uplo, int64_t n, double* A, int64_t lda) {
  if (uplo != Uplo::Lower) blas::unsupported("potrf");
  return orc_potrf_tile((int)n, A, (int)lda);
}
inline double lange(Norm norm, int64_t m, int64_t n, const double* A, int64_t lda) {
  if (norm != Norm::Inf) blas::unsupported("lange");
  double mx = 0;
  for (int64_t i = 0; i < m; ++i) {
    double s = 0;
    for (int64_t j = 0; j < n; ++j) s += std::fabs(A[i + j * lda]);
    mx = std::max(mx, s);
  }
  return mx;
}
}  // namespace lapack
