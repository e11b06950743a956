"""GPU tests of the mixed-precision path (tensor-core low-precision factorisation + FP64
refinement), through the C ABI.

Tolerances:
  * factor: max |W - L64| / max |L64| <= 3e-2 (bf16 operands, unit roundoff 2^-8 x growth),
    <= 4e-3 (fp16, 2^-11) and <= 0.25 (fp8 e4m3, 2^-4), L64 from the CPU oracle;
  * solve: the target accuracy, normwise backward error max_j ||b_j - A x_j||_inf /
    (||A||_inf ||x_j||_inf + ||b_j||_inf) <= 1e-14, and the forward error against an FP64 solve of
    the same system bounded by kappa(A) * 1e-14.
"""
import numpy as np
import pytest

import oracle
from ttg_gb300 import workloads

pytestmark = pytest.mark.gpu


def dense_from_tiles(t, N, NB):
    L = oracle.tiles_to_lower(t, N, NB)
    return L + np.tril(L, -1).T


@pytest.mark.parametrize("N,NB,prec,tol", [(2048, 512, "bf16", 3e-2), (2048, 512, "fp16", 4e-3),
                                           (1800, 256, "bf16", 3e-2), (1024, 256, "fp16", 4e-3),
                                           (2048, 512, "fp8", 0.25), (1800, 256, "fp8", 0.25)])
def test_mixed_factor_close_to_fp64(gbx, cuda, N, NB, prec, tol):
    import torch
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A, N, NB, seed=42)
    W, work, st, cond = gbx.potrf_mixed(A, N, NB, prec=prec)
    assert st == 0
    ref = A.cpu().numpy().copy()
    oracle.load_openblas()
    assert oracle.potrf_tiled(ref, N, NB, nthreads=0, use_blas=oracle.lib().orc_blas_loaded())[0] == 0
    Lw = oracle.tiles_to_lower(W.double().cpu().numpy(), N, NB)
    L64 = oracle.tiles_to_lower(ref, N, NB)
    err = np.abs(Lw - L64).max() / np.abs(L64).max()
    print("factor %s N=%d NB=%d: max|W - L64| / max|L64| = %.3g" % (prec, N, NB, err))
    assert err <= tol, err
    assert 1.0 <= cond < 10.0  # diagonally dominant tiles


def solve_and_check(gbx, cuda, A, N, NB, nrhs, prec, kappa):
    import torch
    Bn = workloads.rhs(N, nrhs, seed=42)
    B = torch.from_numpy(Bn).to(cuda)
    X, info, st = gbx.dposv_mixed(A, N, NB, B, prec=prec, tol=1e-14, maxiter=300)
    assert st == 0, info
    assert info["backward_error"] <= 1e-14, info
    Ad = dense_from_tiles(A.cpu().numpy(), N, NB)
    Xn = X.cpu().numpy()
    # independent backward error on the host
    for j in range(nrhs):
        r = Bn[j] - Ad @ Xn[j]
        be = np.abs(r).max() / (np.abs(Ad).sum(1).max() * np.abs(Xn[j]).max() + np.abs(Bn[j]).max())
        assert be <= 1.5e-14, be
    Xref = np.linalg.solve(Ad, Bn.T).T
    fe = np.abs(Xn - Xref).max() / np.abs(Xref).max()
    assert fe <= kappa * 1e-14, fe
    return info


@pytest.mark.parametrize("prec", ["bf16", "fp16", "fp8"])
def test_dposv_mixed_well_conditioned(gbx, cuda, prec):
    import torch
    N, NB = 3000, 512
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A, N, NB, seed=42)
    info = solve_and_check(gbx, cuda, A, N, NB, 8, prec, kappa=10.0)
    print("dposv_mixed %s kappa~10: %s" % (prec, info))
    assert info["iterations"] <= (40 if prec == "fp8" else 10), info


@pytest.mark.parametrize("kappa,prec", [(1e4, "bf16"), (1e6, "bf16"), (1e6, "fp16")])
def test_dposv_mixed_householder(gbx, cuda, kappa, prec):
    N, NB = 2048, 512
    A = workloads.householder_tiles(N, NB, 4, kappa, 42, cuda)
    Ad = dense_from_tiles(A.cpu().numpy(), N, NB)
    Aref = workloads.householder_dense(N, 4, kappa, seed=42)
    assert np.abs(Ad - Aref).max() <= 1e-14  # device generator against the reflector products
    solve_and_check(gbx, cuda, A, N, NB, 8, prec, kappa=kappa)


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_dposv_mixed_householder_8192_fp64_checked(gbx, cuda, prec):
    """The mixed-precision configuration (A = H diag(lam) H^T, 4 reflectors, kappa = 1e6, 8 rhs) at
    N=8192: the solver's own backward error (double-float residual), the same figure from plain FP64
    products on the device (gbx_dsymm_tiled) and an FP64 residual on the host all meet 1e-14."""
    import torch
    N, NB, nrhs = 8192, 512, 8
    A = workloads.householder_tiles(N, NB, 4, 1e6, 42, cuda)
    Bn = workloads.rhs(N, nrhs, seed=42)
    B = torch.from_numpy(Bn).to(cuda)
    X, info, st = gbx.dposv_mixed(A, N, NB, B, prec=prec, tol=1e-14, maxiter=300)
    assert st == 0, info
    assert info["backward_error"] <= 1e-14, info
    dev = gbx.backward_error_fp64(A, N, NB, B, X)
    assert max(dev) <= 1e-14, dev
    Ad = dense_from_tiles(A.cpu().numpy(), N, NB)
    Xn = X.cpu().numpy()
    anorm = np.abs(Ad).sum(1).max()
    host = [np.abs(Bn[j] - Ad @ Xn[j]).max() / (anorm * np.abs(Xn[j]).max() + np.abs(Bn[j]).max())
            for j in range(nrhs)]
    print("N=8192 %s: solver %.3g, device FP64 %.3g, host FP64 %.3g" % (prec, info["backward_error"], max(dev),
                                                                       max(host)))
    assert max(host) <= 1e-14, host


def test_dsymm_tiled_matches_dense(gbx, cuda):
    import ctypes
    import torch
    N, NB, nrhs = 1100, 256, 3
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A, N, NB, seed=5)
    X = torch.randn(nrhs, N, dtype=torch.float64, device=cuda)
    Y = torch.randn(nrhs, N, dtype=torch.float64, device=cuda)
    Y0 = Y.clone()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    gbx.call("gbx_dsymm_tiled", N, NB, ctypes.c_void_p(A.data_ptr()), nrhs, -1.0, ctypes.c_void_p(X.data_ptr()), 2.0,
             ctypes.c_void_p(Y.data_ptr()), s)
    Ad = torch.from_numpy(dense_from_tiles(A.cpu().numpy(), N, NB)).to(cuda)
    ref = 2.0 * Y0 - (Ad @ X.T).T
    assert (Y - ref).abs().max().item() <= 1e-12 * ref.abs().max().item()


def batch_dense(A, sizes, NB, k):
    import numpy as np
    offs, _ = __import__("ttg_gb300").batched_tile_offsets(sizes, NB)
    n = int(sizes[k])
    nt = (n + NB - 1) // NB
    t = A[int(offs[k]):int(offs[k]) + nt * (nt + 1) // 2 * NB * NB].cpu().numpy()
    return dense_from_tiles(t, n, NB)


@pytest.mark.parametrize("prec", ["fp16", "bf16", "fp8"])
def test_dposv_mixed_batched_uneven(gbx, cuda, prec):
    """Uneven (ragged) orders in one batch, kappa = 1e4: every matrix to backward error 1e-14, and the
    factor of each matrix equal to the single-matrix launch's factor bit for bit (same tile order)."""
    import torch
    NB, nrhs = 256, 2
    sizes = np.array([700, 256, 1300, 1024, 90, 513])
    A, B = workloads.householder_batch(sizes, NB, 2, 1e4, 7, cuda, nrhs=nrhs)
    Wd = torch.empty(A.numel(), dtype=torch.float32, device=cuda)
    X, infos, st = gbx.dposv_mixed_batched(A, sizes, NB, B, nrhs, prec=prec, tol=1e-14, maxiter=300, W=Wd)
    assert st == 0, infos
    Xn, Bn = X.cpu().numpy(), B.cpu().numpy()
    off = 0
    for k, n in enumerate(sizes):
        n = int(n)
        Ad = batch_dense(A, sizes, NB, k)
        Xk = Xn[off:off + n * nrhs].reshape(nrhs, n)
        Bk = Bn[off:off + n * nrhs].reshape(nrhs, n)
        off += n * nrhs
        assert infos[k]["backward_error"] <= 1e-14, (k, infos[k])
        anorm = np.abs(Ad).sum(1).max()  # ||A||_inf from the single pass over A (FP32 partial sums)
        assert abs(infos[k]["anorm"] - anorm) <= 1e-5 * anorm, (k, infos[k]["anorm"], anorm)
        for j in range(nrhs):
            r = Bk[j] - Ad @ Xk[j]
            be = np.abs(r).max() / (np.abs(Ad).sum(1).max() * np.abs(Xk[j]).max() + np.abs(Bk[j]).max())
            assert be <= 1.5e-14, (k, be)
    # the batched factorisation against one launch per matrix
    offs, total = gbx.batched_tile_offsets(sizes, NB)
    Wb = torch.empty(total, dtype=torch.float32, device=cuda)
    n32 = np.ascontiguousarray(sizes.astype(np.int32))
    import ctypes
    need = ctypes.c_size_t(0)
    gbx.call("gbx_potrf_mixed_batched_bufferSize", len(sizes), n32.ctypes.data_as(ctypes.c_void_p), NB,
             ctypes.byref(need))
    work = torch.empty(need.value, dtype=torch.uint8, device=cuda)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    gbx.call("gbx_potrf_mixed_batched", len(sizes), n32.ctypes.data_as(ctypes.c_void_p), NB,
             ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(Wb.data_ptr()), gbx.PREC[prec], 0.0, gbx.FP64_DIAG_COND,
             None, ctypes.c_void_p(work.data_ptr()), need.value, s)
    info = np.zeros(len(sizes), dtype=np.int32)
    gbx.call("gbx_potrf_mixed_batched_info", ctypes.c_void_p(work.data_ptr()), len(sizes),
             n32.ctypes.data_as(ctypes.c_void_p), NB, info.ctypes.data_as(ctypes.c_void_p), None, None, s)
    assert not info.any()
    for k, n in enumerate(sizes):
        n = int(n)
        nt = (n + NB - 1) // NB
        o = int(offs[k])
        Ak = A[o:o + nt * (nt + 1) // 2 * NB * NB].clone()
        W1, _, st1, _ = gbx.potrf_mixed(Ak, n, NB, prec=prec)
        assert st1 == 0
        Wk = Wb[o:o + W1.numel()]
        Lb = oracle.tiles_to_lower(Wk.double().cpu().numpy(), n, NB)
        L1 = oracle.tiles_to_lower(W1.double().cpu().numpy(), n, NB)
        assert np.array_equal(Lb, L1), k
        # the solver's factor (W converted by its single pass over A) is the same factor
        Ld = oracle.tiles_to_lower(Wd[o:o + W1.numel()].double().cpu().numpy(), n, NB)
        assert np.array_equal(Ld, L1), k


def test_split_f64_bitwise(gbx, cuda):
    """The integer-arithmetic split hi + lo = a equals the FP64 conversions bit for bit:
    hi = fl32(a), lo = fl32(a - hi), over random exponents, rounding ties and special values."""
    import torch
    rng = np.random.default_rng(5)
    n = 1 << 20
    a = rng.standard_normal(n) * np.exp2(rng.integers(-160, 160, n).astype(np.float64))
    # halfway cases of the hi rounding (low 29 mantissa bits = 2^28, odd and even kept bit)
    bits = a[:4096].view(np.uint64)
    bits = (bits & ~np.uint64((1 << 29) - 1)) | np.uint64(1 << 28)
    a[:4096] = bits.view(np.float64)
    special = np.array([0.0, -0.0, 1.0, -1.0, 5e-324, -5e-324, 1e-310, 2.0 ** -126, 2.0 ** -149, 2.0 ** -150,
                        3.4028234663852886e38, 3.4028235677973366e38, 1e39, -1e300, np.inf, -np.inf, np.nan,
                        1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, 1.0 + 2.0 ** -52, 2.0 ** 127 * 1.9999999])
    a[4096:4096 + special.size] = special
    hi, lo = gbx.split_f64(torch.from_numpy(a).to(cuda))
    torch.cuda.synchronize()
    with np.errstate(over="ignore", invalid="ignore"):
        h_ref = a.astype(np.float32)
        l_ref = (a - h_ref.astype(np.float64)).astype(np.float32)
    h, l = hi.cpu().numpy(), lo.cpu().numpy()
    for got, ref in ((h, h_ref), (l, l_ref)):
        nan = np.isnan(ref)
        assert np.array_equal(np.isnan(got), nan)
        assert np.array_equal(got[~nan].view(np.uint32), ref[~nan].view(np.uint32))


def test_dposv_mixed_batched_reports_non_spd_member(gbx, cuda):
    """One indefinite matrix in the batch: it is reported (no factor after every shift), the others
    are solved."""
    import torch
    NB, nrhs = 256, 1
    sizes = np.array([512, 300, 600])
    A, B = workloads.householder_batch(sizes, NB, 2, 1e2, 3, cuda, nrhs=nrhs)
    offs, _ = gbx.batched_tile_offsets(sizes, NB)
    A[int(offs[1])] = -10.0  # A_00 of matrix 1
    X, infos, st = gbx.dposv_mixed_batched(A, sizes, NB, B, nrhs, prec="fp16", tol=1e-14)
    assert st == gbx.GBX_ERR_NOCONV
    assert infos[1]["backward_error"] == float("inf") and infos[1]["factor_retries"] == 8
    assert infos[0]["backward_error"] <= 1e-14 and infos[2]["backward_error"] <= 1e-14


def test_tune_mixed_batched_picks_a_converged_configuration(gbx, cuda):
    """The tuner times all twelve candidates (fp16, bf16, fp8 at NB 256 and 512, CTA schedules 0 and
    1; the 256 tiles made from the 512 ones on the device), each as a captured CUDA graph of the
    whole solve, and returns the fastest converged one."""
    from ttg_gb300 import autotune
    NB, nrhs = 512, 2
    sizes = np.array([700, 300, 1300])
    A, B = workloads.householder_batch(sizes, NB, 2, 1e3, 5, cuda, nrhs=nrhs)
    best = autotune.tune_mixed_batched(A, sizes, NB, B, nrhs, tol=1e-14, use_cache=False)
    assert best["ok"] and best["status"] == 0 and best["backward_error_max"] <= 1e-14, best
    assert {(c["prec"], c["NB"], c["sched"]) for c in best["candidates"]} == {
        (p, nb, sc) for p in ("fp16", "bf16", "fp8") for nb in (256, 512) for sc in (0, 1)}
    assert best["ms"] == min(c["ms"] for c in best["candidates"] if c["ok"])
    assert sum(c["ok"] for c in best["candidates"]) >= 8, best["candidates"]


# ---- FP64 route of the diagonal POTRF ------------------------------------------------------------
def test_fp64_diag_route_threshold(gbx, cuda):
    """Threshold 0 sends every diagonal tile to the FP64 POTRF, a huge one none; either factor stays
    within the bf16 tolerance of the FP64 factor."""
    import torch
    N, NB = 2048, 512
    A = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=cuda)
    gbx.gen_uniform_sym(A, N, NB, seed=42)
    ref = A.cpu().numpy().copy()
    oracle.load_openblas()
    assert oracle.potrf_tiled(ref, N, NB, nthreads=0, use_blas=oracle.lib().orc_blas_loaded())[0] == 0
    L64 = oracle.tiles_to_lower(ref, N, NB)
    for thr, expect in ((0.0, N // NB), (1e300, 0)):
        W, work, st, cond, nf = gbx.potrf_mixed(A, N, NB, prec="bf16", fp64_diag_cond=thr, with_fp64_tiles=True)
        assert st == 0 and nf == expect, (thr, st, nf)
        Lw = oracle.tiles_to_lower(W.double().cpu().numpy(), N, NB)
        assert np.abs(Lw - L64).max() / np.abs(L64).max() <= 3e-2


def test_fp64_diag_route_by_condition_estimate(gbx, cuda):
    """A diagonal tile scaled to a diagonal ratio of 1e6 (D A D, D = 10^(3 i / NB) on the first tile's
    rows) exceeds the default threshold and alone takes the FP64 route; the solve still reaches
    1e-14, and the FP64 route can be forced for every tile of the same system."""
    import torch
    N, NB, nrhs = 1536, 512, 2
    Ad = oracle.uniform_sym_full(N, 11)
    d = np.ones(N)
    d[:NB] = 10.0 ** (3.0 * np.arange(NB) / NB)
    Ad = Ad * d[:, None] * d[None, :]
    A = torch.from_numpy(np.ascontiguousarray(oracle.tiles_from_full(Ad, NB))).to(cuda)
    Bn = workloads.rhs(N, nrhs, seed=3)
    B = torch.from_numpy(Bn).to(cuda)
    for thr, expect in ((gbx.FP64_DIAG_COND, 1), (0.0, N // NB)):
        X, info, st = gbx.dposv_mixed(A, N, NB, B, prec="fp16", tol=1e-14, maxiter=300, fp64_diag_cond=thr)
        assert st == 0, info
        assert info["fp64_diag_tiles"] == expect, info
        assert info["backward_error"] <= 1e-14, info
        Xn = X.cpu().numpy()
        anorm = np.abs(Ad).sum(1).max()
        for j in range(nrhs):
            be = np.abs(Bn[j] - Ad @ Xn[j]).max() / (anorm * np.abs(Xn[j]).max() + np.abs(Bn[j]).max())
            assert be <= 1.5e-14, be


# ---- the batched solve as one CUDA graph -----------------------------------------------------------
def test_batched_mixed_solve_captured_in_cuda_graph(gbx, cuda):
    """Plan once, capture the run (factorisation with its retry loop, CG with device-side
    coefficients and convergence tests as WHILE nodes) in a torch CUDA graph, replay it twice on
    fresh right-hand sides: every matrix meets 1e-14 and the solution agrees with the uncaptured
    solve."""
    import torch
    NB, nrhs = 256, 2
    sizes = np.array([700, 256, 1300, 1024, 90, 513])
    A, B = workloads.householder_batch(sizes, NB, 2, 1e4, 7, cuda, nrhs=nrhs)
    X0, infos0, st0 = gbx.dposv_mixed_batched(A, sizes, NB, B, nrhs, prec="fp16", tol=1e-14, maxiter=300)
    assert st0 == 0
    solver = gbx.MixedBatchedSolver(sizes, NB, nrhs, prec="fp16", device=cuda)
    W = torch.empty(A.numel(), dtype=torch.float32, device=cuda)
    Bg = torch.zeros_like(B)
    X = torch.zeros_like(B)
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
        solver.run(A, Bg, X, W, tol=1e-14, maxiter=300, stream=side)
    for rep in range(2):
        Bg.copy_(B * (1 + rep))
        X.zero_()
        g.replay()
        torch.cuda.synchronize()
        infos, st = solver.result()
        assert st == 0, infos
        assert all(i["backward_error"] <= 1e-14 for i in infos), infos
        assert [i["iterations"] for i in infos] == [i["iterations"] for i in infos0] or rep == 1
        rel = ((X - X0 * (1 + rep)).abs().max() / (X0 * (1 + rep)).abs().max()).item()
        assert rel <= 1e4 * 1e-13, rel
