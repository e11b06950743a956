"""GPU parity of the executor's tensor-core FP64 update mode (gbx_set_fp64_update(1)) against the CPU
oracle, at the FP64 bar of the plain path:
  * factor: max |L - L_ref| <= 1e-12 max |L_ref| and, elementwise, |L_ij - L_ref_ij| <= 1e-12 |L_ref_ij|
    wherever |L_ref_ij| >= 1e-6 max |L_ref|;
  * ||A - L L^T||_F / (N ||A||_F) <= 1e-15 and the reference driver's check < 60;
  * the same first bad pivot as the oracle for a matrix that is not positive definite.
The mode needs 128-blocks: below the small-matrix threshold the tests force that edge.
"""
import ctypes

import numpy as np
import pytest

import oracle
from test_gpu_potrf import assert_factor_close, to_dev

pytestmark = pytest.mark.gpu


@pytest.fixture
def emu(gbx):
    L = gbx.lib()
    old_t = L.gbx_get_wait_timeout_ns()
    assert L.gbx_set_fp64_update(1) == 0
    assert L.gbx_set_dag_block_edge(128) == 0
    L.gbx_set_wait_timeout_ns(5 * 10**9)
    try:
        yield L
    finally:
        L.gbx_set_fp64_update(0)
        L.gbx_set_dag_block_edge(0)
        L.gbx_set_wait_timeout_ns(old_t)


def _oracle_factor(t0, N, NB):
    ref = t0.copy()
    assert oracle.potrf_tiled(ref, N, NB, nthreads=0, use_blas=oracle.load_openblas())[0] == 0
    return oracle.tiles_to_lower(ref, N, NB)


@pytest.mark.parametrize("gen,N,NB", [("uniform", 1024, 256), ("uniform", 1000, 256), ("plgsy", 1536, 384),
                                      ("uniform", 2048, 512), ("uniform", 2500, 512), ("uniform", 384, 128)])
def test_emulated_updates_match_oracle(gbx, cuda, emu, gen, N, NB):
    t0 = oracle.plgsy_tiles(N, NB, N, 3872) if gen == "plgsy" else oracle.uniform_sym_tiles(N, NB, 42)
    t = to_dev(t0, cuda)
    work = gbx.potrf_tiled(t, N, NB)
    assert gbx.potrf_status(work) == 0
    L = oracle.tiles_to_lower(t.cpu().numpy(), N, NB)
    assert_factor_close(L, _oracle_factor(t0, N, NB))
    A0 = oracle.tiles_to_lower(t0, N, NB)
    A0 = A0 + np.tril(A0, -1).T
    assert oracle.check_dpotrf(L, A0) < 60.0
    assert oracle.frob_residual(L, A0) <= 1e-15


@pytest.mark.parametrize("spread", [0.0, 2.5])
def test_emulated_updates_graded_scaling(gbx, cuda, emu, spread):
    """D A D with D = 10^U(-spread, spread): rows of L over five orders of magnitude (the per-row
    scales of the digit planes) and ill-conditioned diagonal blocks (condition ~1e5)."""
    N, NB = 1536, 384
    A = oracle.uniform_sym_full(N, 11)
    d = 10.0 ** np.random.default_rng(3).uniform(-spread, spread, N)
    A = A * d[:, None] * d[None, :]
    t0 = oracle.tiles_from_full(A, NB)
    t = to_dev(t0, cuda)
    work = gbx.potrf_tiled(t, N, NB)
    assert gbx.potrf_status(work) == 0
    L = oracle.tiles_to_lower(t.cpu().numpy(), N, NB)
    assert_factor_close(L, _oracle_factor(t0, N, NB))
    assert oracle.frob_residual(L, A) <= 1e-15


@pytest.mark.parametrize("lo,hi", [(-490, -490), (-490, -100)])
def test_emulated_updates_extreme_scales(gbx, cuda, emu, lo, hi):
    """D A D with D = 2^round(U(lo, hi)): update products near 1e-295, where the power of two 2^E
    that scales the digit-plane products lies below the normal FP64 range (the wide-range form of
    the subtraction), alone or beside ordinary scales. D is a power of two per row, so D^-1 L of the
    executor and of the oracle are the factors of A itself."""
    N, NB = 1024, 256
    A = oracle.uniform_sym_full(N, 5)
    d = 2.0 ** np.round(np.random.default_rng(4).uniform(lo, hi, N))
    t0 = oracle.tiles_from_full(A * d[:, None] * d[None, :], NB)
    t = to_dev(t0, cuda)
    work = gbx.potrf_tiled(t, N, NB)
    assert gbx.potrf_status(work) == 0
    L = oracle.tiles_to_lower(t.cpu().numpy(), N, NB) / d[:, None]
    assert np.isfinite(L).all()
    assert_factor_close(L, _oracle_factor(t0, N, NB) / d[:, None])
    assert oracle.frob_residual(L, A) <= 1e-15


def test_emulated_updates_8192(gbx, cuda, emu):
    """The checked size of the N=32768 configuration (128-blocks by default at this size)."""
    if not oracle.load_openblas():
        pytest.skip("OpenBLAS not found for the N=8192 oracle run")
    N, NB = 8192, 512
    assert emu.gbx_set_dag_block_edge(0) == 0
    t0 = oracle.uniform_sym_tiles(N, NB, 42)
    t = to_dev(t0, cuda)
    work = gbx.potrf_tiled(t, N, NB)
    assert gbx.potrf_status(work) == 0
    L = oracle.tiles_to_lower(t.cpu().numpy(), N, NB)
    assert_factor_close(L, _oracle_factor(t0, N, NB))
    A0 = oracle.tiles_to_lower(t0, N, NB)
    A0 = A0 + np.tril(A0, -1).T
    res = np.linalg.norm(A0 - L @ L.T) / (N * np.linalg.norm(A0))
    print("emulated N=8192 ||A - L L^T||_F / (N ||A||_F) = %.3g" % res)
    assert res <= 1e-15


def test_emulated_mode_reports_first_bad_pivot(gbx, cuda, emu):
    N, NB = 1000, 128
    A = oracle.uniform_sym_full(N, 9)
    A[700, 700] = -1.0
    t0 = oracle.tiles_from_full(A, NB)
    ref = t0.copy()
    st, info, _ = oracle.potrf_tiled(ref, N, NB, nthreads=1)  # failing tile (1-based), pivot in it
    expect = (st - 1) * NB + info
    assert expect == 701
    t = to_dev(t0, cuda)
    work = gbx.potrf_tiled(t, N, NB, check=False)
    assert gbx.potrf_status(work) == expect
    # the library stays usable: a good matrix next
    t0 = oracle.uniform_sym_tiles(N, NB, 3)
    t = to_dev(t0, cuda)
    assert gbx.potrf_status(gbx.potrf_tiled(t, N, NB)) == 0
    assert_factor_close(oracle.tiles_to_lower(t.cpu().numpy(), N, NB), _oracle_factor(t0, N, NB))


def test_emulated_mode_workspace(gbx, emu):
    a = ctypes.c_size_t(0)
    assert emu.gbx_dpotrf_tiled_bufferSize(4096, 512, ctypes.byref(a)) == 0
    emu.gbx_set_fp64_update(0)
    b = ctypes.c_size_t(0)
    assert emu.gbx_dpotrf_tiled_bufferSize(4096, 512, ctypes.byref(b)) == 0
    ntri = 32 * 33 // 2
    assert a.value - b.value >= ntri * (7 * 128 * 128 * 2 + 128 * 4)


def test_emulated_host_buffers_solve(gbx, cuda, emu):
    """gbx_dposv_tiled_host (pinned host in and out, copies overlapped) in the emulated mode."""
    import torch
    N, NB = 2048, 512
    t0 = oracle.uniform_sym_tiles(N, NB, 5)
    rng = np.random.default_rng(2)
    b = rng.uniform(-1, 1, N)
    A_host = torch.from_numpy(t0.copy()).pin_memory()
    L_host = torch.empty_like(A_host).pin_memory()
    B_host = torch.from_numpy(b.copy()).pin_memory()
    X_host = torch.empty_like(B_host).pin_memory()
    tiles = torch.empty(t0.size, dtype=torch.float64, device=cuda)
    X = torch.empty(N, dtype=torch.float64, device=cuda)
    need = ctypes.c_size_t(0)
    assert emu.gbx_dposv_tiled_host_bufferSize(N, NB, ctypes.byref(need)) == 0
    work = torch.empty(need.value, dtype=torch.uint8, device=cuda)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    vp = lambda x: ctypes.c_void_p(x.data_ptr())
    assert emu.gbx_dposv_tiled_host(N, NB, vp(A_host), vp(L_host), 1, vp(B_host), vp(X_host), vp(tiles), vp(X),
                                    vp(work), need.value, s) == 0
    torch.cuda.synchronize()
    Lref = _oracle_factor(t0, N, NB)
    assert_factor_close(oracle.tiles_to_lower(L_host.numpy(), N, NB), Lref)
    A0 = oracle.tiles_to_lower(t0, N, NB)
    A0 = A0 + np.tril(A0, -1).T
    x = X_host.numpy()
    berr = np.max(np.abs(A0 @ x - b)) / (np.max(np.sum(np.abs(A0), 1)) * np.max(np.abs(x)) + np.max(np.abs(b)))
    assert berr <= 1e-14
