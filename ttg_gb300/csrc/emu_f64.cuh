// FP64 block products on the bf16 tensor cores (Ozaki-style splitting, Ozaki, Ogita, Oishi and Rump
// 2012): the building blocks the executor's emulated GEMM/SYRK tasks use.
//
// Splitting. Every row r of an FP64 block L (128 x 128) is scaled by its own power of two 2^e_r,
// with |L(r,k)| < 2^e_r for every k, and rounded to the fixed-point integer
//     F(r,k) = round(L(r,k) 2^(55 - e_r)),  |F| <= 2^55,
// which is then written as seven balanced base-256 digits,
//     F = sum_{i=0..6} d_i 256^(6-i),   d_i in [-128, 127] for i >= 1, |d_0| <= 128,
// each digit stored as a bf16 "slice" (an integer of at most 8 significant bits: exact). So
// L(r,k) = 2^(e_r - 55) sum_i d_i(r,k) 2^(8(6-i)) up to 2^-56 |2^e_r|.
//
// Products. For C(r,c) -= sum_k A(r,k) B(c,k), with digit planes a_i of A and b_j of B:
//     sum_k A B = 2^(eA_r + eB_c - 110) sum_g 2^(8(12-g)) acc_g,   acc_g = sum_{i+j=g} sum_k a_i b_j.
// The groups g = 0..6 are kept (the dropped ones are below 2^-56 of the leading term). Each acc_g is
// a sum of at most 7 * 128 products of magnitude <= 2^14: below 2^24 in magnitude, so the tensor
// cores' FP32 accumulation of these integers is exact. Then
//     sum_k A B = X 2^(eA_r + eB_c - 62),   X = sum_{g=0..6} acc_g 2^(8(6-g))   (an integer < 2^70),
// X formed in 64 bits (fold), rounded once to FP64 and subtracted from C by one FMA with the power
// of two (sub_scaled): two roundings in all, against k of them for the FP64 dot product.
//
// Costs on GB300 (measured per SM per clock): FP64 add/FMA and every conversion to or from FP64
// ~1.6-1.9, float->int ~15, integer ~60, FP32 ~113. Hence integer-only splitting and folding, and
// two FP64-pipe operations per element of C per task (the conversion of X and the FMA: a rounding
// of X in integer instructions measured slower, ~30 of them per element).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbx {
namespace emu {

constexpr int kSlices = 7;                                  // digit planes per block
constexpr int kEdge = 128;                                  // block edge of the emulated executor
constexpr long long kPlaneElems = (long long)kEdge * kEdge; // bf16 elements per plane
constexpr long long kBlockElems = kSlices * kPlaneElems;    // bf16 elements per block
constexpr int kEmptyRow = -4000;                            // exponent of an all-zero row

// float holding an integer of magnitude <= 2^22 -> its bf16 bit pattern (exact for |d| <= 256)
__device__ __forceinline__ uint32_t digit_bf16(int d) {
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;  // exact for |d| < 2^22
  return __float_as_uint(f) >> 16;
}

// Splits kRows rows of an FP64 block (m x n valid, m <= kRows, column-major, leading dimension ld)
// into kSlices bf16 digit planes S[i][r][k] (row-major, k contiguous, plane stride kPlaneElems,
// zero outside m x n) and the row exponents rexp[r]: the whole 128-row block, or (kRows = 32) the
// rows of one TRSM sub-task, leaving the other rows alone. Threads 0..255 of the CTA: thread t
// handles row t % kRows and part t / kRows of the 256 / kRows parts of k (synchronised with named
// barrier 1); s_exp: 256 ints of shared memory.
template <int kRows = kEdge>
__device__ __forceinline__ void slice_block(const double* __restrict__ L, int ld, int m, int n,
                                            uint16_t* __restrict__ S, int* __restrict__ rexp, int* s_exp) {
  constexpr int kParts = 256 / kRows, kSpan = kEdge / kParts;  // k-range parts, elements per part
  static_assert(kSpan % 8 == 0, "whole 16-byte stores");
  const int r = threadIdx.x % kRows, h = threadIdx.x / kRows;
  const int k0 = h * kSpan;
  // 1. largest biased exponent in the row (integer compare of the exponent fields)
  int mex = 0;
  if (r < m)
    for (int k = k0; k < min(k0 + kSpan, n); ++k) mex = max(mex, (__double2hiint(__ldcg(L + r + (long long)k * ld)) >> 20) & 0x7ff);
  s_exp[h * kRows + r] = mex;
  asm volatile("bar.sync 1, 256;" ::: "memory");
#pragma unroll
  for (int q = 0; q < kParts; ++q) mex = max(mex, s_exp[q * kRows + r]);
  asm volatile("bar.sync 1, 256;" ::: "memory");
  // every |L(r,k)| < 2^e (frexp exponent of the largest); rows of zeros and subnormals give no digits
  const int e = mex - 1022;
  if (h == 0) rexp[r] = (mex > 0) ? e : kEmptyRow;
  // 2. fixed point and digits, eight consecutive k per 16-byte store of each plane
  for (int kc = 0; kc < kSpan; kc += 8) {
    uint32_t pk[kSlices][4];
#pragma unroll
    for (int i = 0; i < kSlices; ++i)
#pragma unroll
      for (int w = 0; w < 4; ++w) pk[i][w] = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = k0 + kc + j;
      long long F = 0;
      if (mex > 0 && r < m && k < n) {
        const long long bits = __double_as_longlong(__ldcg(L + r + (long long)k * ld));
        const int ex = (int)((bits >> 52) & 0x7ff);
        if (ex > 0) {
          const long long mant = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
          const int sh = ex - 1020 - e;  // F = mant 2^sh, sh <= 2 because |L| < 2^e
          long long f = 0;
          if (sh >= 0) f = mant << sh;
          else if (sh > -60) f = (mant + (1LL << (-sh - 1))) >> (-sh);  // round half up
          F = bits < 0 ? -f : f;
        }
      }
#pragma unroll
      for (int i = kSlices - 1; i >= 1; --i) {
        const int d = (int)((F + 128) & 255) - 128;
        F = (F - d) >> 8;  // exact: F - d is a multiple of 256
        pk[i][j >> 1] |= digit_bf16(d) << (16 * (j & 1));
      }
      pk[0][j >> 1] |= digit_bf16((int)F) << (16 * (j & 1));
    }
#pragma unroll
    for (int i = 0; i < kSlices; ++i)
      *(uint4*)(S + (long long)i * kPlaneElems + (long long)r * kEdge + k0 + kc) =
          make_uint4(pk[i][0], pk[i][1], pk[i][2], pk[i][3]);
  }
}

// the integer group sums of one element: H = acc_0 2^16 + acc_1 2^8 + acc_2 (|H| < 2^38) and
// L = acc_3 2^24 + acc_4 2^16 + acc_5 2^8 + acc_6 (|L| < 2^49), from the exact FP32 values
__device__ __forceinline__ long long group_h(uint32_t a0, uint32_t a1, uint32_t a2) {
  return (long long)__float2int_rn(__uint_as_float(a0)) * 65536 + (long long)__float2int_rn(__uint_as_float(a1)) * 256 +
         (long long)__float2int_rn(__uint_as_float(a2));
}
__device__ __forceinline__ long long group_l(uint32_t a3, uint32_t a4, uint32_t a5, uint32_t a6) {
  return (long long)__float2int_rn(__uint_as_float(a3)) * 16777216 +
         (long long)__float2int_rn(__uint_as_float(a4)) * 65536 + (long long)__float2int_rn(__uint_as_float(a5)) * 256 +
         (long long)__float2int_rn(__uint_as_float(a6));
}

// X = H 2^32 + L = sum_g acc_g 2^(8(6-g)) in 64 bits, as X 2^-s: exactly (s = 0) while |H| < 2^30
// (|X| < 2^62 + 2^49), else with s = 8, which drops only bits below 2^-54 of |X| >= 2^62
__device__ __forceinline__ long long fold(long long H, long long L, int& s) {
  s = (H >= (1LL << 30) || H <= -(1LL << 30)) ? 8 : 0;
  return (long long)((unsigned long long)H << (32 - s)) + (L >> s);
}

// 2^k as FP64, -1022 <= k <= 1023
__device__ __forceinline__ double pow2(int k) { return __hiloint2double((k + 1023) << 20, 0); }

// c - X 2^sE: X rounded to FP64 (to nearest even), and the product with the power of two
// subtracted in one FMA (exact product: subnormal and overflowing results come out of the FMA
// rounded once). *odd is set when 2^sE is not a normal FP64 number itself (extreme scales only;
// see sub_wide).
__device__ __forceinline__ double sub_scaled(double c, long long X, int sE, bool* odd) {
  *odd = (unsigned)(sE + 1022) > 2045u;
  return fma(-__ll2double_rn(X), pow2(sE), c);
}

// the same for any sE: 2^sE as 2^a 2^b with both factors normal (X 2^a is exact for X != 0, as
// a >= -1022), exact again up to the FMA's rounding for |sE| <= 2044; beyond, the clamped factors
// still give the limit (a product far below the smallest subnormal, or an overflow)
__device__ __forceinline__ double sub_wide(double c, long long X, int sE) {
  const int a = min(max(sE / 2, -1022), 1023), b = min(max(sE - a, -1022), 1023);
  return fma(-__ll2double_rn(X) * pow2(a), pow2(b), c);
}

}  // namespace emu
}  // namespace gbx
