"""GPU parity tests of the FP64 path, through the C ABI, against the CPU oracle.

Tolerances (FP64):
  * generators: bit-exact;
  * tile kernels: elementwise |C - C_ref| <= 4 k eps (|C0| + |A||B|^T) (the standard GEMM bound);
  * factorisations: max |L - L_ref| <= 1e-12 max |L_ref| and, elementwise, |L_ij - L_ref_ij| <=
    1e-12 |L_ref_ij| wherever |L_ref_ij| >= 1e-6 max|L_ref|; residual ||A - L L^T||_F / (N ||A||_F)
    <= 1e-15 and the reference driver's ||LL^T - A||_inf / (||A||_inf N eps) < 60.
"""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _s():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def to_dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def colmajor_dev(a, ld, cuda):
    """numpy (rows x cols) -> CUDA tensor holding it column-major with leading dimension ld."""
    import torch
    rows, cols = a.shape
    buf = np.full((cols, ld), np.nan)
    buf[:, :rows] = a.T
    return torch.from_numpy(buf).to(cuda)


def from_colmajor(t, rows):
    return t.cpu().numpy()[:, :rows].T.copy()


def assert_factor_close(L, Lref, tol=1e-12):
    mx = np.max(np.abs(Lref))
    d = np.abs(L - Lref)
    assert np.max(d) <= tol * mx, np.max(d) / mx
    big = np.abs(Lref) >= 1e-6 * mx
    rel = d[big] / np.abs(Lref[big])
    assert np.max(rel) <= tol, np.max(rel)


# ---- generators --------------------------------------------------------------------------------
@pytest.mark.parametrize("N,NB", [(160, 32), (1000, 128), (2048, 512)])
def test_device_plgsy_bit_exact(gbx, cuda, N, NB):
    import torch
    t = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.plgsy(t, N, NB, N, 3872)
    assert np.array_equal(t.cpu().numpy(), oracle.plgsy_tiles(N, NB, N, 3872))


@pytest.mark.parametrize("N,NB", [(777, 128), (1024, 512)])
def test_device_uniform_sym_bit_exact(gbx, cuda, N, NB):
    import torch
    t = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(t, N, NB, seed=42)
    assert np.array_equal(t.cpu().numpy(), oracle.uniform_sym_tiles(N, NB, 42))


# ---- tile kernels (drop-ins for the four library calls) ----------------------------------------
GEMM_SHAPES = [(512, 512, 512), (128, 128, 128), (100, 77, 33), (300, 200, 600), (1, 1, 1), (129, 257, 17)]


@pytest.mark.parametrize("m,n,k", GEMM_SHAPES)
def test_tile_dgemm_nt(gbx, cuda, m, n, k):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A, B, C = rng.uniform(-1, 1, (m, k)), rng.uniform(-1, 1, (n, k)), rng.uniform(-1, 1, (m, n))
    lda, ldb, ldc = m + 3, n + 1, m + 5
    dA, dB, dC = colmajor_dev(A, lda, cuda), colmajor_dev(B, ldb, cuda), colmajor_dev(C, ldc, cuda)
    gbx.call("gbx_dgemm_nt_tile", m, n, k, _vp(dA), lda, _vp(dB), ldb, _vp(dC), ldc, _s())
    got = from_colmajor(dC, m)
    Cref = np.asfortranarray(C.copy())
    oracle.lib().orc_gemm_nt_tile(m, n, k, oracle._p(np.asfortranarray(A)), m, oracle._p(np.asfortranarray(B)), n,
                                  oracle._p(Cref), m)
    bound = 4 * k * EPS * (np.abs(C) + np.abs(A) @ np.abs(B).T)
    assert np.all(np.abs(got - Cref) <= bound)
    # padding rows between m and ldc untouched
    assert np.all(np.isnan(dC.cpu().numpy()[:, m:ldc]))


@pytest.mark.parametrize("n,k", [(512, 512), (128, 128), (100, 33), (257, 129)])
def test_tile_dsyrk_ln(gbx, cuda, n, k):
    rng = np.random.default_rng(n + k)
    A, C = rng.uniform(-1, 1, (n, k)), rng.uniform(-1, 1, (n, n))
    dA, dC = colmajor_dev(A, n, cuda), colmajor_dev(C, n + 2, cuda)
    gbx.call("gbx_dsyrk_ln_tile", n, k, _vp(dA), n, _vp(dC), n + 2, _s())
    got = from_colmajor(dC, n)
    ref = C - A @ A.T
    bound = 4 * k * EPS * (np.abs(C) + np.abs(A) @ np.abs(A).T)
    low = np.tril(np.ones((n, n), dtype=bool))
    assert np.all(np.abs(got - ref)[low] <= bound[low])
    assert np.array_equal(got[~low], C[~low])  # strict upper untouched


def spd(n, seed):
    return oracle.uniform_sym_full(n, seed)


@pytest.mark.parametrize("m,n", [(512, 512), (128, 128), (100, 77), (300, 33), (5, 200)])
def test_tile_dtrsm_rlt(gbx, cuda, m, n):
    L = np.linalg.cholesky(spd(n, 5))
    rng = np.random.default_rng(m + n)
    B = rng.uniform(-1, 1, (m, n))
    dL, dB = colmajor_dev(L, n + 1, cuda), colmajor_dev(B, m + 2, cuda)
    gbx.call("gbx_dtrsm_rlt_tile", m, n, _vp(dL), n + 1, _vp(dB), m + 2, _s())
    got = from_colmajor(dB, m)
    ref = np.asfortranarray(B.copy())
    oracle.lib().orc_trsm_rlt_tile(m, n, oracle._p(np.asfortranarray(L)), n, oracle._p(ref), m)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("m,n", [(1, 512), (8, 512), (3, 100), (16, 129), (40, 33)])
def test_tile_dtrsm_rln(gbx, cuda, m, n):
    """B := B L^{-1} (the backward sweep of the solve flowgraph) against the oracle."""
    L = np.linalg.cholesky(spd(n, 7))
    rng = np.random.default_rng(m * 3 + n)
    B = rng.uniform(-1, 1, (m, n))
    dL, dB = colmajor_dev(L, n + 3, cuda), colmajor_dev(B, m + 1, cuda)
    gbx.call("gbx_dtrsm_rln_tile", m, n, _vp(dL), n + 3, _vp(dB), m + 1, _s())
    got = from_colmajor(dB, m)
    ref = np.asfortranarray(B.copy())
    oracle.lib().orc_trsm_rln_tile(m, n, oracle._p(np.asfortranarray(L)), n, oracle._p(ref), m)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    assert np.all(np.isnan(dB.cpu().numpy()[:, m:m + 1]))  # padding rows untouched


@pytest.mark.parametrize("m,n,k", [(1, 512, 512), (8, 512, 300), (5, 37, 129), (16, 16, 16)])
def test_tile_dgemm_nn(gbx, cuda, m, n, k):
    """C := C - A B against the oracle, within the standard GEMM bound."""
    rng = np.random.default_rng(m + 5 * n + k)
    A, B, C = rng.uniform(-1, 1, (m, k)), rng.uniform(-1, 1, (k, n)), rng.uniform(-1, 1, (m, n))
    dA, dB, dC = colmajor_dev(A, m + 2, cuda), colmajor_dev(B, k + 1, cuda), colmajor_dev(C, m + 3, cuda)
    gbx.call("gbx_dgemm_nn_tile", m, n, k, _vp(dA), m + 2, _vp(dB), k + 1, _vp(dC), m + 3, _s())
    got = from_colmajor(dC, m)
    ref = np.asfortranarray(C.copy())
    oracle.lib().orc_gemm_nn_tile(m, n, k, oracle._p(np.asfortranarray(A)), m, oracle._p(np.asfortranarray(B)), k,
                                  oracle._p(ref), m)
    bound = 4 * k * EPS * (np.abs(C) + np.abs(A) @ np.abs(B))
    assert np.all(np.abs(got - ref) <= bound)


@pytest.mark.parametrize("n", [1, 31, 128, 129, 512, 1000])
def test_tile_dpotrf(gbx, cuda, n):
    import torch
    A = spd(n, n)
    lda = n + 4
    dA = colmajor_dev(A, lda, cuda)
    ws = ctypes.c_size_t(0)
    gbx.call("gbx_dpotrf_tile_bufferSize", n, lda, ctypes.byref(ws))
    work = torch.empty(ws.value, dtype=torch.uint8, device=cuda)
    info = torch.full((1,), -7, dtype=torch.int32, device=cuda)
    gbx.call("gbx_dpotrf_tile", n, _vp(dA), lda, _vp(work), ws.value, _vp(info), _s())
    assert int(info.item()) == 0
    got = from_colmajor(dA, n)
    ref = np.asfortranarray(A.copy())
    assert oracle.lib().orc_potrf_tile(n, oracle._p(ref), n) == 0
    assert_factor_close(np.tril(got), np.tril(ref))
    assert np.array_equal(np.triu(got, 1), np.triu(A, 1))  # upper untouched, like cuSOLVER


@pytest.mark.parametrize("n,bad", [(64, 40), (300, 170)])
def test_tile_dpotrf_reports_pivot(gbx, cuda, n, bad):
    import torch
    A = spd(n, 1)
    A[bad, bad] = -5.0  # makes the leading (bad+1) minor indefinite
    dA = colmajor_dev(A, n, cuda)
    ws = ctypes.c_size_t(0)
    gbx.call("gbx_dpotrf_tile_bufferSize", n, n, ctypes.byref(ws))
    work = torch.empty(ws.value, dtype=torch.uint8, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    gbx.call("gbx_dpotrf_tile", n, _vp(dA), n, _vp(work), ws.value, _vp(info), _s())
    ref = np.asfortranarray(A.copy())
    assert int(info.item()) == oracle.lib().orc_potrf_tile(n, oracle._p(ref), n) == bad + 1


# ---- the whole flowgraph on the device ---------------------------------------------------------
def run_dag(gbx, cuda, N, NB, tiles_np):
    import torch
    t = to_dev(tiles_np, cuda)
    gbx.potrf_tiled(t, N, NB)
    return t.cpu().numpy()


CASES = [("plgsy", 160, 32), ("plgsy", 1000, 128), ("uniform", 2048, 128), ("uniform", 2048, 512),
         ("uniform", 1536, 384), ("uniform", 700, 96), ("uniform", 2500, 512), ("uniform", 64, 64)]


@pytest.mark.parametrize("gen,N,NB", CASES)
def test_dag_potrf_matches_oracle(gbx, cuda, gen, N, NB):
    t0 = oracle.plgsy_tiles(N, NB, N, 3872) if gen == "plgsy" else oracle.uniform_sym_tiles(N, NB, 42)
    got = run_dag(gbx, cuda, N, NB, t0)
    ref = t0.copy()
    if oracle.load_openblas():
        st, _, _ = oracle.potrf_tiled(ref, N, NB, nthreads=0, use_blas=True)
    else:
        st, _, _ = oracle.potrf_tiled(ref, N, NB, nthreads=0)
    assert st == 0
    L, Lref = oracle.tiles_to_lower(got, N, NB), oracle.tiles_to_lower(ref, N, NB)
    assert_factor_close(L, Lref)
    if N <= 2048:
        A0 = oracle.tiles_to_lower(t0, N, NB)
        A0 = A0 + np.tril(A0, -1).T
        assert oracle.check_dpotrf(L, A0) < 60.0
        assert oracle.frob_residual(L, A0) <= 1e-15


@pytest.mark.parametrize("edge", [128, 64, 32])
def test_dag_block_edges_match_oracle(gbx, cuda, edge):
    """The executor's block edge (automatic: 64 up to N=4096, 128 above; forced here) changes only
    the order of the FP64 operations: the factor stays within the parity bar of the oracle."""
    N, NB = 2048, 128
    t0 = oracle.uniform_sym_tiles(N, NB, 42)
    assert gbx.lib().gbx_set_dag_block_edge(edge) == 0
    try:
        got = run_dag(gbx, cuda, N, NB, t0)
    finally:
        gbx.lib().gbx_set_dag_block_edge(0)
    ref = t0.copy()
    assert oracle.potrf_tiled(ref, N, NB, nthreads=0, use_blas=oracle.load_openblas())[0] == 0
    assert_factor_close(oracle.tiles_to_lower(got, N, NB), oracle.tiles_to_lower(ref, N, NB))


def test_dag_potrf_8192_vs_cpu_oracle(gbx, cuda):
    # the checked size of the N=32768 configuration
    N, NB = 8192, 512
    if not oracle.load_openblas():
        pytest.skip("OpenBLAS not found for the N=8192 oracle run")
    t0 = oracle.uniform_sym_tiles(N, NB, 42)
    got = run_dag(gbx, cuda, N, NB, t0)
    ref = t0.copy()
    assert oracle.potrf_tiled(ref, N, NB, nthreads=0, use_blas=True)[0] == 0
    L = oracle.tiles_to_lower(got, N, NB)
    assert_factor_close(L, oracle.tiles_to_lower(ref, N, NB))
    # the factorisation bar of the plain path at this size too: ||A - L L^T||_F / (N ||A||_F) <= 1e-15
    # (FP64 product on the host, numpy's multithreaded BLAS)
    A0 = oracle.tiles_to_lower(t0, N, NB)
    A0 = A0 + np.tril(A0, -1).T
    res = np.linalg.norm(A0 - L @ L.T) / (N * np.linalg.norm(A0))
    print("N=8192 ||A - L L^T||_F / (N ||A||_F) = %.3g" % res)
    assert res <= 1e-15


def test_dag_reports_first_bad_pivot(gbx, cuda):
    N, NB = 1000, 128
    A = oracle.uniform_sym_full(N, 9)
    A[700, 700] = -1.0
    t0 = oracle.tiles_from_full(A, NB)
    ref = t0.copy()
    st, info, _ = oracle.potrf_tiled(ref, N, NB, nthreads=1)
    expect = (st - 1) * NB + info
    assert expect == 701
    import torch
    t = to_dev(t0, cuda)
    with pytest.raises(gbx.NotPositiveDefinite) as e:
        gbx.potrf_tiled(t, N, NB)
    assert e.value.info == expect


def test_dag_wait_times_out_and_context_survives(gbx, cuda):
    import torch
    NB = 32
    tiles = torch.zeros(3 * NB * NB, dtype=torch.float64, device=cuda)
    need = gbx.potrf_workspace_bytes(2 * NB, NB)
    work = torch.empty(need, dtype=torch.uint8, device=cuda)
    st = gbx.lib().gbx_dag_timeout_selftest(NB, _vp(tiles), _vp(work), need, 200_000_000, _s())
    assert st == gbx.GBX_ERR_TIMEOUT
    # the context is still usable
    t0 = oracle.uniform_sym_tiles(256, 64, 1)
    got = run_dag(gbx, cuda, 256, 64, t0)
    ref = t0.copy()
    oracle.potrf_tiled(ref, 256, 64, nthreads=1)
    assert_factor_close(got, ref)


def test_dag_workspace_too_small(gbx, cuda):
    import torch
    t = torch.zeros(gbx.tiled_numel(512, 128), dtype=torch.float64, device=cuda)
    w = torch.empty(16, dtype=torch.uint8, device=cuda)
    st = gbx.lib().gbx_dpotrf_tiled(512, 128, _vp(t), _vp(w), 16, _s())
    assert st == gbx.GBX_ERR_WORKSPACE


# ---- solve ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("N,NB,nrhs", [(1000, 128, 1), (2048, 512, 8), (160, 32, 3)])
def test_potrs_matches_oracle(gbx, cuda, N, NB, nrhs):
    import torch
    A = oracle.uniform_sym_full(N, 42)
    t0 = oracle.tiles_from_full(A, NB)
    t = to_dev(t0, cuda)
    gbx.potrf_tiled(t, N, NB)
    rng = np.random.default_rng(42)
    B = rng.standard_normal((nrhs, N))
    dB = to_dev(B, cuda)
    gbx.potrs_tiled(t, N, NB, dB)
    X = dB.cpu().numpy()
    for r in range(nrhs):
        x = X[r]
        berr = np.linalg.norm(A @ x - B[r], np.inf) / (np.linalg.norm(A, np.inf) * np.linalg.norm(x, np.inf)
                                                      + np.linalg.norm(B[r], np.inf))
        assert berr <= 1e-14
    ref_f = t.cpu().numpy()
    Xref = oracle.potrs_tiled(ref_f, N, NB, B.T.copy())
    assert np.max(np.abs(X.T - Xref)) <= 1e-12 * np.max(np.abs(Xref))


def test_full_size_solve_backward_error(gbx, cuda):
    """N=16384: size-independent property — the solve's normwise backward error stays at FP64 level."""
    import torch
    N, NB = 16384, 512
    t = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(t, N, NB, seed=42)
    # dense copy of A for the residual (symmetric from the lower tiles)
    nt = gbx.ntiles(N, NB)
    A = torch.empty((N, N), dtype=torch.float64, device=cuda)
    tv = t.view(-1, NB, NB)
    for n in range(nt):
        for m in range(n, nt):
            s = oracle.tile_slot(m, n, nt)
            blk = tv[s].T  # tile is column-major: row index fastest
            A[m * NB:(m + 1) * NB, n * NB:(n + 1) * NB] = blk
            if m != n:
                A[n * NB:(n + 1) * NB, m * NB:(m + 1) * NB] = blk.T
    gbx.potrf_tiled(t, N, NB)
    g = torch.Generator(device=cuda).manual_seed(42)
    b = torch.randn(N, dtype=torch.float64, device=cuda, generator=g)
    x = b.clone()
    gbx.potrs_tiled(t, N, NB, x)
    r = A @ x - b
    berr = (r.abs().max() / (A.abs().sum(1).max() * x.abs().max() + b.abs().max())).item()
    assert berr <= 1e-14


@pytest.mark.parametrize("edge,ntb", [(128, 8), (0, 16)])
def test_task_timeline_trace(gbx, cuda, tmp_path, edge, ntb):
    """The per-task timeline records every executed task of the persistent executor (N=1024:
    eight 128-blocks when forced, sixteen 64-blocks by the automatic choice for small matrices)."""
    import json
    import torch
    N, NB = 1024, 256
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A, N, NB, seed=1)
    buf = torch.zeros(2 + 4 * 1000, dtype=torch.int64, device=cuda)
    gbx.lib().gbx_set_trace_buffer(_vp(buf), 1000)
    assert gbx.lib().gbx_set_dag_block_edge(edge) == 0
    try:
        gbx.potrf_tiled(A, N, NB)
    finally:
        gbx.lib().gbx_set_trace_buffer(None, 0)
        gbx.lib().gbx_set_dag_block_edge(0)
    recs = gbx.trace_records(buf)
    # every task once; TRSM(K+1,K) (on the critical path) as 4 row sub-tasks
    assert len(recs) == ntb + ntb * (ntb - 1) + ntb * (ntb - 1) * (ntb - 2) // 6 + 3 * (ntb - 1)
    assert all(r["end_ns"] >= r["start_ns"] for r in recs)
    pot = {r["a"]: r for r in recs if r["type"] == "POTRF"}
    trsm = [r for r in recs if r["type"] == "TRSM"]
    assert all(t["start_ns"] >= pot[t["b"]]["end_ns"] for t in trsm)  # dependency order is visible
    gbx.trace_to_chrome(recs, str(tmp_path / "t.json"))
    assert len(json.load(open(tmp_path / "t.json"))["traceEvents"]) == len(recs)


def _wait_stream(torch, seconds=60.0):
    """Polls the current stream with a deadline instead of blocking forever."""
    import time
    ev = torch.cuda.Event()
    ev.record()
    t0 = time.time()
    while not ev.query():
        assert time.time() - t0 < seconds, "stream did not finish"
        time.sleep(0.001)


@pytest.mark.parametrize("N,NB,nrhs", [(3000, 512, 2), (1000, 128, 1)])
def test_dposv_tiled_host_overlap(gbx, cuda, N, NB, nrhs):
    """Host buffers in, host buffers out, copies overlapped with the executor: the factor and the
    solution equal the device-resident path's bit for bit (both are deterministic)."""
    import torch
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A, N, NB, seed=11)
    B = torch.randn(nrhs, N, dtype=torch.float64, device=cuda)
    T = A.clone()
    gbx.potrf_tiled(T, N, NB)
    Xd = gbx.potrs_tiled(T, N, NB, B.clone())
    A_host = torch.empty(A.numel(), dtype=torch.float64, pin_memory=True)
    A_host.copy_(A)
    B_host = torch.empty(B.shape, dtype=torch.float64, pin_memory=True)
    B_host.copy_(B)
    L_host, X_host, _ = gbx.dposv_tiled_host(A_host, N, NB, B_host, check=False)
    _wait_stream(torch)
    assert torch.equal(L_host, T.cpu())
    assert torch.equal(X_host, Xd.cpu())


def test_dposv_tiled_host_non_spd_completes(gbx, cuda):
    """A breakdown stops the executor early; the copy-out stream is released and the call ends with
    the pivot status."""
    import ctypes
    import torch
    N, NB = 2048, 512
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A, N, NB, seed=3)
    A_host = torch.empty(A.numel(), dtype=torch.float64, pin_memory=True)
    A_host.copy_(A)
    slot = 2 * 4 - 2 * 1 // 2  # tile (2, 2) of NT = 4
    A_host[slot * NB * NB + 5 + 5 * NB] = -1e6  # row 1029 of the matrix
    B_host = torch.ones(1, N, dtype=torch.float64).pin_memory()
    need = ctypes.c_size_t(0)
    gbx.call("gbx_dposv_tiled_host_bufferSize", N, NB, ctypes.byref(need))
    work = torch.empty(need.value, dtype=torch.uint8, device=cuda)
    L_host, X_host, st0 = gbx.dposv_tiled_host(A_host, N, NB, B_host, work=work, check=False)
    assert st0 == 2 * NB + 5 + 1  # the call itself reports the pivot and skips the solve
    _wait_stream(torch)
    st = gbx.call("gbx_dpotrf_tiled_status", ctypes.c_void_p(work.data_ptr()),
                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 2 * NB + 5 + 1


@pytest.mark.parametrize("N,NB", [(1000, 128), (1800, 512), (512, 512)])
def test_potri_matches_oracle_and_inverse(gbx, cuda, N, NB):
    """Device TRTRI + LAUUM against the oracle's restatement (same factor) and numpy's inverse."""
    import torch
    A = oracle.uniform_sym_full(N, 33)
    t0 = oracle.tiles_from_full(A, NB)
    ref = t0.copy()
    assert oracle.potrf_tiled(ref, N, NB, nthreads=0)[0] == 0
    T = to_dev(ref, cuda)  # the same factor on both sides
    gbx.potri_tiled(T, N, NB)
    got = np.tril(oracle.tiles_to_lower(T.cpu().numpy(), N, NB))
    assert oracle.potri_tiled(ref, N, NB) == 0
    want = np.tril(oracle.tiles_to_lower(ref, N, NB))
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= 1e-13 * scale
    assert np.abs(got - np.tril(np.linalg.inv(A))).max() <= 1e-12 * scale
