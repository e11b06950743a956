// tcgen05 BF16 GEMM core for sm_103a: D(fp32, column-major) = A * B^T with A (M x K) and B (N x K)
// stored K-major (row-major, K contiguous). One CTA computes a 128 x BN tile:
//   warp 0      TMA producer: 4-stage ring of {A 128x64, B BNx64} bf16 tiles, 128B swizzle
//   warp 1      MMA issuer: one thread issues tcgen05.mma (kind::f16, M=128, N=BN, K=16) into a
//               TMEM accumulator and frees each stage with tcgen05.commit
//   warps 2..5  epilogue: tcgen05.ld of the accumulator (lane = row) and coalesced column-major
//               stores (consecutive lanes write consecutive rows)
// Every mbarrier wait has a time limit; a timeout sets *status = GBX_ERR_TIMEOUT and the CTA
// still releases its TMEM before returning.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>

#include "gbx_common.cuh"
#include "gbx_potrf.h"
#include "tc_common.cuh"

namespace gbx {
namespace tc {

constexpr int kBM = 128, kBK = 64, kStages = 4;

template <int BN>
struct GemmCfg {
  static constexpr uint32_t a_bytes = kBM * kBK * 2;
  static constexpr uint32_t b_bytes = BN * kBK * 2;
  static constexpr uint32_t stage_bytes = a_bytes + b_bytes;
  static constexpr size_t smem_bytes = (size_t)kStages * stage_bytes + 1024;
};

template <int BN>
__global__ void __launch_bounds__(192, 1)
    gemm_bf16_nt_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
                        int K, float* D, long long ldd, int* status, uint64_t timeout_ns) {
  using C = GemmCfg<BN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int err;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  const int nk = (K + kBK - 1) / kBK;
  if (threadIdx.x == 0) {
    err = 0;
    for (int s = 0; s < kStages; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&done_bar), 1);
    mbar_fence_init();
  }
  if (warp == 1) tmem_alloc(smem_u32(&tmem_slot), BN);
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0 && lane == 0) {
    tma_prefetch_desc(&tmA);
    tma_prefetch_desc(&tmB);
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStages;
      const uint32_t ph = (kb / kStages) & 1;
      if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1, &err, timeout_ns)) break;
      const uint32_t a_dst = smem_u32(smem + (size_t)s * C::stage_bytes);
      mbar_arrive_expect_tx(smem_u32(&full_bar[s]), C::stage_bytes);
      tma_load_2d(a_dst, &tmA, smem_u32(&full_bar[s]), kb * kBK, m0);
      tma_load_2d(a_dst + C::a_bytes, &tmB, smem_u32(&full_bar[s]), kb * kBK, n0);
    }
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = idesc_f16(kBM, BN, true);
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStages;
      const uint32_t ph = (kb / kStages) & 1;
      if (!mbar_wait(smem_u32(&full_bar[s]), ph, &err, timeout_ns)) break;
      tc_fence_after();
      const uint32_t a_base = smem_u32(smem + (size_t)s * C::stage_bytes);
      const uint64_t ad = desc_kmajor_sw128(a_base), bd = desc_kmajor_sw128(a_base + C::a_bytes);
#pragma unroll
      for (int k = 0; k < kBK / 16; ++k)
        umma_f16(tmem, ad + 2 * k, bd + 2 * k, idesc, (kb | k) != 0 ? 1u : 0u);
      umma_commit(smem_u32(&empty_bar[s]));
    }
    umma_commit(smem_u32(&done_bar));
  } else if (warp >= 2) {
    const int sub = warp & 3;  // TMEM lane quarter this warp may read
    const int row = m0 + sub * 32 + lane;
    if (mbar_wait(smem_u32(&done_bar), 0, &err, timeout_ns)) {
      tc_fence_after();
      for (int c = 0; c < BN; c += 16) {
        uint32_t r[16];
        tmem_ld16(tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)c, r);
        tmem_ld_wait();
        if (row < M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = n0 + c + j;
            if (col < N) D[(long long)row + (long long)col * ldd] = __uint_as_float(r[j]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, BN);
  }
  if (threadIdx.x == 0 && err && status) atomicCAS(status, 0, err);
}

// ---- host helpers --------------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

// 2D K-major bf16 operand: `rows` rows of `k` elements, row stride `ld` elements; box 64 x box_rows
int make_tmap_kmajor_bf16(CUtensorMap* map, const void* base, uint64_t rows, uint64_t k, uint64_t ld,
                          uint32_t box_rows) {
  auto enc = encode_fn();
  if (!enc) return GBX_ERR_CUDA;
  if (((uintptr_t)base & 15) || ((ld * 2) & 15) || rows == 0 || k == 0) return GBX_ERR_ARG;
  cuuint64_t dims[2] = {k, rows};
  cuuint64_t strides[1] = {ld * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? GBX_OK : GBX_ERR_ARG;
}

// same for fp16 (bf16 = false)
int make_tmap_kmajor_16b(CUtensorMap* map, const void* base, uint64_t rows, uint64_t k, uint64_t ld, uint32_t box_rows,
                         bool bf16) {
  auto enc = encode_fn();
  if (!enc) return GBX_ERR_CUDA;
  if (((uintptr_t)base & 15) || ((ld * 2) & 15) || rows == 0 || k == 0) return GBX_ERR_ARG;
  cuuint64_t dims[2] = {k, rows};
  cuuint64_t strides[1] = {ld * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                   const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? GBX_OK : GBX_ERR_ARG;
}

// 8-bit (fp8) K-major operand: `rows` rows of `k` one-byte elements, row stride `ld` bytes; box
// 128 x box_rows (128-byte rows, the same swizzled layout as the 16-bit box of 64)
int make_tmap_kmajor_8b(CUtensorMap* map, const void* base, uint64_t rows, uint64_t k, uint64_t ld, uint32_t box_rows) {
  auto enc = encode_fn();
  if (!enc) return GBX_ERR_CUDA;
  if (((uintptr_t)base & 15) || (ld & 15) || rows == 0 || k == 0) return GBX_ERR_ARG;
  cuuint64_t dims[2] = {k, rows};
  cuuint64_t strides[1] = {ld};
  cuuint32_t box[2] = {128, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? GBX_OK : GBX_ERR_ARG;
}

}  // namespace tc
}  // namespace gbx

using namespace gbx;
using namespace gbx::tc;

extern "C" int gbx_gemm_bf16_nt_f32(int M, int N, int K, const void* A, int lda, const void* B, int ldb, float* D,
                                    int ldd, int* status, void* stream) {
  if (gbx::recording_stream(stream)) return GBX_ERR_ARG;  // not a CUDA stream
  if (M < 0 || N < 0 || K < 0 || lda < K || ldb < K || ldd < M || (lda % 8) || (ldb % 8)) return GBX_ERR_ARG;
  if (M == 0 || N == 0) return GBX_OK;
  if (!A || !B || !D) return GBX_ERR_ARG;
  constexpr int BN = 256;
  CUtensorMap ta, tb;
  if (int e = make_tmap_kmajor_bf16(&ta, A, (uint64_t)M, (uint64_t)K, (uint64_t)lda, kBM)) return e;
  if (int e = make_tmap_kmajor_bf16(&tb, B, (uint64_t)N, (uint64_t)K, (uint64_t)ldb, BN)) return e;
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(gemm_bf16_nt_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)GemmCfg<BN>::smem_bytes);
  });
  if (attr_err != cudaSuccess) return GBX_ERR_CUDA;
  dim3 grid((M + kBM - 1) / kBM, (N + BN - 1) / BN);
  gemm_bf16_nt_kernel<BN><<<grid, 192, GemmCfg<BN>::smem_bytes, (cudaStream_t)stream>>>(
      ta, tb, M, N, K, D, (long long)ldd, status, gbx_get_wait_timeout_ns());
  return cudaGetLastError() == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}
