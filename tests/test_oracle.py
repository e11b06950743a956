"""CPU tests of the oracle: pinned against the reference's own generator and the golden fixtures,
cross-checked against numpy, and the restated flowgraph's scheduling rules."""
import hashlib
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "potrf_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_plgsy_matches_reference_generator_ragged(gold):
    # bit-exact against examples/potrf/core_plgsy.h compiled from the reference
    t = oracle.plgsy_tiles(100, 32, 100, 3872)
    assert np.array_equal(t, gold["plgsy_N100_NB32"])


@pytest.mark.parametrize("N,NB", [(160, 32), (1000, 128)])
def test_plgsy_matches_reference_generator_hash(gold, N, NB):
    t = oracle.plgsy_tiles(N, NB, N, 3872)
    h = np.frombuffer(hashlib.sha256(t.tobytes()).digest(), dtype=np.uint8)
    assert np.array_equal(h, gold["sha256_plgsy_N%d_NB%d" % (N, NB)])


def test_uniform_generator_golden(gold):
    vals = [oracle.lib().orc_uniform_elem(42, int(i), int(j)) for i, j in gold["uniform_seed42_idx"]]
    assert np.array_equal(np.array(vals), gold["uniform_seed42_val"])


def test_uniform_sym_properties():
    N = 300
    A = oracle.uniform_sym_full(N, 42)
    assert np.array_equal(A, A.T)
    off = A - np.diag(np.diag(A))
    assert np.abs(off).max() <= 0.5
    assert np.all(np.abs(np.diag(A) - N) <= 0.5)
    t = oracle.uniform_sym_tiles(N, 64, 42)
    assert np.array_equal(oracle.tiles_to_lower(t, N, 64), np.tril(A))


def test_factor_golden(gold):
    t = gold["plgsy_N100_NB32"].copy()
    st, info, _ = oracle.potrf_tiled(t, 100, 32, nthreads=3)
    assert st == 0
    # the flowgraph fixes the update order of every tile, so the factor is bit-reproducible
    assert np.array_equal(t, gold["factor_N100_NB32"])


@pytest.mark.parametrize("N,NB", [(160, 32), (100, 32), (257, 64), (64, 64), (1, 8)])
def test_oracle_vs_numpy_and_reference_check(N, NB):
    t = oracle.plgsy_tiles(N, NB, N, 3872)
    A0 = oracle.tiles_to_lower(t, N, NB)
    A0 = A0 + np.tril(A0, -1).T
    st, info, _ = oracle.potrf_tiled(t, N, NB, nthreads=4)
    assert st == 0
    L = oracle.tiles_to_lower(t, N, NB)
    Lr = np.linalg.cholesky(A0)
    assert np.max(np.abs(L - Lr)) <= 1e-12 * np.max(np.abs(Lr))
    # the reference driver's acceptance criterion (testing_dpotrf.cc:277-335)
    assert oracle.check_dpotrf(L, A0) < 60.0
    assert oracle.frob_residual(L, A0) <= 1e-15


def test_oracle_openblas_agrees():
    if not oracle.load_openblas():
        pytest.skip("no OpenBLAS shared library next to scipy")
    N, NB = 520, 128
    t = oracle.uniform_sym_tiles(N, NB, 42)
    t2 = t.copy()
    oracle.potrf_tiled(t, N, NB, nthreads=4, use_blas=False)
    oracle.potrf_tiled(t2, N, NB, nthreads=4, use_blas=True)
    assert np.max(np.abs(t - t2)) <= 1e-12 * np.max(np.abs(t))


def test_flowgraph_trace_is_a_valid_schedule():
    N, NB = 8 * 16, 16
    NT = 8
    t = oracle.uniform_sym_tiles(N, NB, 7)
    st, info, tr = oracle.potrf_tiled(t, N, NB, nthreads=3, trace=True)
    assert st == 0
    keys = [(int(x) >> 60, (int(x) >> 40) & 0xFFFFF, (int(x) >> 20) & 0xFFFFF, int(x) & 0xFFFFF) for x in tr]
    assert len(keys) == len(set(keys)) == NT + NT * (NT - 1) + NT * (NT - 1) * (NT - 2) // 6
    pos = {k: i for i, k in enumerate(keys)}
    for (ty, a, b, c), i in pos.items():
        if ty == 1:  # TRSM(M,K) after POTRF(K) and GEMM(M,K,K-1)
            assert pos[(0, b, 0, 0)] < i
            if b > 0:
                assert pos[(3, a, b, b - 1)] < i
        if ty == 3:  # GEMM(M,N,K) after TRSM(M,K), TRSM(N,K)
            assert pos[(1, a, c, 0)] < i and pos[(1, b, c, 0)] < i


def test_priorities_match_reference_formulas():
    nt = 10
    assert oracle.lib().orc_priority(0, nt, 3, 0, 0) == (nt - 3) ** 3
    assert oracle.lib().orc_priority(1, nt, 5, 2, 0) == (nt - 5) ** 3 + 3 * ((2 * nt) - 2 - 5 - 1) * (5 - 2)
    assert oracle.lib().orc_priority(2, nt, 2, 5, 0) == (nt - 2) ** 3 + 3 * (2 - 5)
    assert oracle.lib().orc_priority(3, nt, 7, 4, 1) == (nt - 7) ** 3 + 3 * ((2 * nt) - 7 - 4 - 3) * (7 - 4) + 6 * (7 - 1)


def test_non_spd_reports_failing_tile():
    N, NB = 96, 32
    A = oracle.uniform_sym_full(N, 3, shift=0.0)  # indefinite
    t = oracle.tiles_from_full(A, NB)
    st, info, _ = oracle.potrf_tiled(t, N, NB, nthreads=2)
    assert st >= 1 and info >= 1


def test_potrs_oracle():
    N, NB = 200, 64
    A = oracle.uniform_sym_full(N, 42)
    t = oracle.tiles_from_full(A, NB)
    oracle.potrf_tiled(t, N, NB, nthreads=2)
    b = np.random.default_rng(1).standard_normal(N)
    x = oracle.potrs_tiled(t, N, NB, b)[:, 0]
    assert np.linalg.norm(A @ x - b) / (np.linalg.norm(A) * np.linalg.norm(x)) < 1e-15


@pytest.mark.parametrize("use_blas", [False, True])
def test_batched_oracle_against_numpy(use_blas):
    if use_blas and not oracle.load_openblas():
        pytest.skip("no OpenBLAS")
    sizes = [1, 7, 32, 65, 96, 3, 128]
    nrhs = 2
    A = oracle.gen_uniform_sym_batched(sizes, seed=5)
    n, offA, offB = oracle.batched_offsets(sizes, nrhs)
    rng = np.random.default_rng(3)
    B = rng.standard_normal(int(offB[-1]))
    A0, B0 = A.copy(), B.copy()
    info = oracle.dposv_batched(sizes, A, B, nrhs=nrhs, nthreads=3, use_blas=use_blas)
    assert not info.any()
    for k, nk in enumerate(sizes):
        Ak = A0[offA[k]:offA[k + 1]].reshape(nk, nk).T
        assert np.array_equal(Ak, Ak.T)
        # generator: (M+M^T)/2 + n I from seed + k * golden-ratio constant
        sk = (5 + k * 0x9e3779b97f4a7c15) % 2 ** 64
        assert Ak[0, 0] == lib_elem(sk, 0, 0) + nk
        Bk = B0[offB[k]:offB[k + 1]].reshape(nrhs, nk).T
        Xk = B[offB[k]:offB[k + 1]].reshape(nrhs, nk).T
        assert np.allclose(Xk, np.linalg.solve(Ak, Bk), rtol=1e-12, atol=1e-14)
        Lk = np.tril(A[offA[k]:offA[k + 1]].reshape(nk, nk).T)
        assert np.allclose(Lk, np.linalg.cholesky(Ak), rtol=1e-12, atol=1e-14)


def lib_elem(seed, i, j):
    return oracle.lib().orc_uniform_elem(seed, i, j)


def test_batched_oracle_reports_bad_matrix():
    sizes = [4, 6]
    A = oracle.gen_uniform_sym_batched(sizes, seed=1)
    A[16 + 2 + 2 * 6] = -5.0  # diagonal entry (2,2) of matrix 1
    B = np.ones(10)
    info = oracle.dposv_batched(sizes, A, B)
    assert info[0] == 0 and info[1] == 3


@pytest.mark.parametrize("N,NB", [(700, 128), (300, 64), (128, 128)])
def test_potri_oracle_inverse(N, NB):
    """The restated TRTRI + LAUUM tile algorithm gives A^{-1} from the factor."""
    A = oracle.uniform_sym_full(N, 21)
    t = oracle.tiles_from_full(A, NB)
    assert oracle.potrf_tiled(t, N, NB, nthreads=2)[0] == 0
    assert oracle.potri_tiled(t, N, NB) == 0
    Ainv = np.tril(oracle.tiles_to_lower(t, N, NB))
    ref = np.tril(np.linalg.inv(A))
    assert np.abs(Ainv - ref).max() <= 1e-13 * np.abs(ref).max()


def test_backward_sweep_tile_ops_against_numpy():
    """The oracle's restatements of the solve flowgraph's backward-sweep tile operations:
    B L^{-1} (right, lower, non-transposed TRSM) and C - A B (non-transposed GEMM)."""
    rng = np.random.default_rng(3)
    n, m, k = 45, 4, 17
    L = np.linalg.cholesky(oracle.uniform_sym_full(n, 5))
    B = rng.standard_normal((m, n))
    X = np.asfortranarray(B.copy())
    oracle.lib().orc_trsm_rln_tile(m, n, oracle._p(np.asfortranarray(L)), n, oracle._p(X), m)
    assert np.abs(X @ L - B).max() <= 1e-13
    A2, B2, C = rng.standard_normal((m, k)), rng.standard_normal((k, n)), rng.standard_normal((m, n))
    Cf = np.asfortranarray(C.copy())
    oracle.lib().orc_gemm_nn_tile(m, n, k, oracle._p(np.asfortranarray(A2)), m, oracle._p(np.asfortranarray(B2)), k,
                                  oracle._p(Cf), m)
    assert np.abs(Cf - (C - A2 @ B2)).max() <= 1e-13
