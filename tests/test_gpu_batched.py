"""GPU tests of the batched persistent solver (one launch for many uneven SPD systems), through the
C ABI. Bars: FP64 mode — every solution's normwise backward error <= 1e-14 and factor info 0;
FP32 + 2 FP64 refinement steps — backward error <= 1e-14 as well (well-conditioned matrices);
FP32 without refinement — <= 1e-6 (single precision)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_batch(count, seed, sizes=None):
    rng = np.random.default_rng(seed)
    if sizes is None:
        sizes = 32 * rng.integers(1, 17, size=count)
    mats, rhs = [], []
    for n in sizes:
        M = rng.uniform(-0.5, 0.5, (n, n))
        mats.append((M + M.T) / 2 + n * np.eye(n))
        rhs.append(rng.standard_normal((1, n)))
    return mats, rhs


def berr(A, x, b):
    r = b - A @ x
    return np.abs(r).max() / (np.abs(A).sum(1).max() * np.abs(x).max() + np.abs(b).max())


@pytest.mark.parametrize("mode,refine,bar", [("fp64", 0, 1e-14), ("fp32", 2, 1e-14), ("fp32", 0, 1e-6)])
def test_batched_uneven_sizes(gbx, cuda, mode, refine, bar):
    mats, rhs = make_batch(96, seed=7)
    b = gbx.Batch(mats, rhs, cuda)
    b.solve(mode=mode, refine=refine)
    assert int(b.info.abs().sum().item()) == 0
    for A, r, x in zip(mats, rhs, b.solutions()):
        assert berr(A, x[0], r[0]) <= bar


def test_batched_edge_sizes_and_ragged_panels(gbx, cuda):
    mats, rhs = make_batch(0, seed=1, sizes=[1, 2, 31, 33, 127, 129, 255, 257, 512, 1000, 1024])
    b = gbx.Batch(mats, rhs, cuda)
    b.solve(mode="fp64")
    assert int(b.info.abs().sum().item()) == 0
    for A, r, x in zip(mats, rhs, b.solutions()):
        assert berr(A, x[0], r[0]) <= 1e-14


def test_batched_reports_non_spd_and_continues(gbx, cuda):
    mats, rhs = make_batch(0, seed=3, sizes=[64, 96, 64])
    mats[1] = mats[1].copy()
    mats[1][50, 50] = -1000.0
    b = gbx.Batch(mats, rhs, cuda)
    b.solve(mode="fp64")
    info = b.info.cpu().numpy()
    assert info[0] == 0 and info[2] == 0 and info[1] == 51
    xs = b.solutions()
    assert berr(mats[0], xs[0][0], rhs[0][0]) <= 1e-14


def test_batched_in_cuda_graph(gbx, cuda):
    import torch
    mats, rhs = make_batch(40, seed=11)
    b = gbx.Batch(mats, rhs, cuda)
    s = torch.cuda.Stream()
    b.solve(mode="fp32", refine=2)  # warm-up outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.solve(mode="fp32", refine=2, stream=s)
    for _ in range(2):
        b.reset()
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        for A, r, x in zip(mats, rhs, b.solutions()):
            assert berr(A, x[0], r[0]) <= 1e-14


def test_batched_device_generator_matches_oracle(gbx, cuda):
    import oracle
    sizes = [32, 100, 64]
    rhs = [np.ones((1, n)) for n in sizes]
    b = gbx.Batch(None, rhs, cuda, sizes=sizes, seed=42)
    A = b.A0.cpu().numpy()
    o = 0
    for k, n in enumerate(sizes):
        got = A[o:o + n * n].reshape(n, n).T  # column-major
        sk = (42 + k * 0x9E3779B97F4A7C15) % (1 << 64)
        ref = oracle.uniform_sym_full(n, sk, shift=n)
        assert np.array_equal(got, ref)
        o += n * n
