// The PLASMA test-matrix generator of the reference (examples/potrf/core_plgsy.h:64-150 with the
// LCG of examples/potrf/random.h:19-41) as device functions: the 64-bit LCG jumped to a linear index,
// and the entry `0.5f - ran * RndF_Mul` evaluated in float as the reference does (its bits are the
// test inputs, so the constants are the reference's).
#pragma once
#include <cuda_runtime.h>

namespace gbx {

__device__ __forceinline__ unsigned long long lcg_jump_dev(unsigned long long n, unsigned long long seed) {
  unsigned long long a = 6364136223846793005ULL, c = 1ULL, x = seed;
  while (n) {
    if (n & 1ULL) x = a * x + c;
    c *= (a + 1);
    a *= a;
    n >>= 1;
  }
  return x;
}

__device__ __forceinline__ double plgsy_entry(unsigned long long ran) {
  // `0.5f - ran * RndF_Mul` evaluated in float, as the reference generator does
  const float r = __ull2float_rn(ran);
  const float p = __fmul_rn(r, 5.4210108624275222e-20f);
  return (double)__fsub_rn(0.5f, p);
}

}  // namespace gbx
