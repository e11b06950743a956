"""GPU tests of the tcgen05 (5th-generation tensor core) BF16 GEMM core, through the C ABI,
against a float64 product of the same bf16 inputs (tolerance: relative 1e-5 of sum |a||b| — the
fp32 accumulation error bound for K <= 4096)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (128, 256, 512), (256, 512, 1024), (200, 300, 136),
                                   (1000, 777, 4096), (64, 16, 8)])
def test_bf16_gemm_matches_fp64_product(gbx, cuda, M, N, K):
    import torch
    g = torch.Generator(device=cuda).manual_seed(M * 31 + N * 7 + K)
    A = torch.randn(M, K, device=cuda, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device=cuda, generator=g).to(torch.bfloat16)
    D = torch.full((N, M), float("nan"), device=cuda, dtype=torch.float32)  # column-major M x N
    st = torch.zeros(1, dtype=torch.int32, device=cuda)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    gbx.call("gbx_gemm_bf16_nt_f32", M, N, K, _vp(A), K, _vp(B), K, _vp(D), M, _vp(st), s)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.double() @ B.double().T
    bound = A.double().abs() @ B.double().abs().T
    err = (D.T.double() - ref).abs()
    assert torch.all(err <= 1e-5 * bound + 1e-30), (err / bound).max().item()


def test_bf16_gemm_rejects_bad_leading_dimension(gbx, cuda):
    assert gbx.lib().gbx_gemm_bf16_nt_f32(128, 128, 64, None, 66, None, 64, None, 128, None, None) == gbx.GBX_ERR_ARG
