"""The allocation-free factorisation entry point (gbx_dpotrf_tiled_noalloc).

Some callers cannot call cudaMalloc — their device memory belongs to another allocator or is
budgeted up front, or they sit on a latency-critical path where cudaMalloc's device
synchronisation is not acceptable. For them gbx_dpotrf_tiled_noalloc keeps its scratch in a
library-owned static device array. This file is collected last so that a failure here cannot stop
the other tests of a run that stops at the first failure; it passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("N,NB", [(2048, 512), (1000, 128)])
def test_noalloc_matches_workspace_entry_point_twice(gbx, cuda, N, NB):
    import torch
    A0 = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A0, N, NB, seed=42)
    ref = A0.clone()
    gbx.potrf_tiled(ref, N, NB)  # the entry point with a caller workspace
    refn = ref.cpu().numpy()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    info = torch.full((1,), -99, dtype=torch.int32, device=cuda)
    for _ in range(2):  # two calls in a row: the shared scratch must be reset by every call
        T = A0.clone()
        info.fill_(-99)
        st = gbx.lib().gbx_dpotrf_tiled_noalloc(N, NB, _vp(T), _vp(info), s)
        assert st == 0
        torch.cuda.synchronize()
        assert int(info.item()) == 0
        got = T.cpu().numpy()
        mx = np.abs(refn).max()
        assert np.abs(got - refn).max() <= 1e-12 * mx  # the tolerance of the FP64 parity tests


def test_noalloc_rejects_problems_beyond_its_scratch(gbx, cuda):
    import torch
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    t = torch.zeros(8, dtype=torch.float64, device=cuda)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # 65664 / 128 = 513 blocks per edge > 512; rejected before any access to `t`
    assert gbx.lib().gbx_dpotrf_tiled_noalloc(65664, 512, _vp(t), _vp(info), s) == gbx.GBX_ERR_NOALLOC_LIMIT


def test_noalloc_reports_first_bad_pivot_then_recovers(gbx, cuda):
    """The shared scratch keeps the last call's run header: after a call that stopped at a bad pivot,
    the next call on an SPD matrix must start from a cleared status and abort word."""
    import torch
    N, NB = 1000, 128
    A0 = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A0, N, NB, seed=42)
    bad = A0.clone()
    nt = gbx.ntiles(N, NB)
    slot = 5 * nt - 5 * 4 // 2  # diagonal tile (5, 5)
    bad[slot * NB * NB + 60 + 60 * NB] = -1.0  # row 5 * 128 + 60 of the matrix
    ws_bad = bad.clone()
    work = gbx.potrf_tiled(ws_bad, N, NB, check=False)
    expect = gbx.potrf_status(work)  # the entry point with a caller workspace
    assert expect == 5 * NB + 60 + 1
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    info = torch.full((1,), -99, dtype=torch.int32, device=cuda)
    T = bad.clone()
    assert gbx.lib().gbx_dpotrf_tiled_noalloc(N, NB, _vp(T), _vp(info), s) == 0
    torch.cuda.synchronize()
    assert int(info.item()) == expect
    # the same scratch again, on the SPD matrix
    ref = A0.clone()
    gbx.potrf_tiled(ref, N, NB)
    T = A0.clone()
    info.fill_(-99)
    assert gbx.lib().gbx_dpotrf_tiled_noalloc(N, NB, _vp(T), _vp(info), s) == 0
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    refn, got = ref.cpu().numpy(), T.cpu().numpy()
    assert np.abs(got - refn).max() <= 1e-12 * np.abs(refn).max()
