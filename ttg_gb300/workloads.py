"""Seeded synthetic workloads of the benchmark configurations.

* uniform: A = (M + M^T)/2 + shift*I, M_ij ~ U[-0.5, 0.5) from the counter-based generator keyed by
  (seed, i, j) (include/gbx_potrf.h, gbx_dgen_uniform_sym_tiled).
* householder: A = H diag(lam) H^T with H the product of r Householder reflectors
  H_k = I - tau_k v_k v_k^T, v_k ~ N(0, 1) i.i.d. (numpy default_rng(seed)), and lam log-spaced from
  1 down to 1/kappa, so that the condition number is kappa. H is passed to the device in
  compact-WY form H = I - U V^T (U = V T, LAPACK's dlarft recurrence for T), with G = V^T diag(lam) V.
* rhs: right-hand sides ~ N(0, 1) from numpy default_rng(seed + 1).
* householder batch: matrix k of a batch is the householder workload of order n_k with seed
  seed + k, right-hand sides rhs(n_k, nrhs, seed + k).
"""
import numpy as np


def householder_factors(N, r, kappa, seed=42):
    rng = np.random.default_rng(seed)
    V = rng.standard_normal((N, r))
    tau = 2.0 / np.einsum("ij,ij->j", V, V)
    T = np.zeros((r, r))
    for k in range(r):
        T[k, k] = tau[k]
        if k:
            T[:k, k] = -tau[k] * (T[:k, :k] @ (V[:, :k].T @ V[:, k]))
    U = V @ T
    lam = float(kappa) ** (-np.arange(N, dtype=np.float64) / max(N - 1, 1))
    G = V.T @ (lam[:, None] * V)
    return lam, U, V, G


def householder_dense(N, r, kappa, seed=42):
    """The same matrix built by applying the reflectors one by one (a cross-check for small N)."""
    rng = np.random.default_rng(seed)
    V = rng.standard_normal((N, r))
    lam = float(kappa) ** (-np.arange(N, dtype=np.float64) / max(N - 1, 1))
    Q = np.eye(N)
    for k in range(r):  # Q = H_1 H_2 ... H_r
        v = V[:, k]
        Q = Q - np.outer(Q @ v, v) * (2.0 / (v @ v))
    return (Q * lam) @ Q.T


def rhs(N, nrhs, seed=42):
    return np.random.default_rng(seed + 1).standard_normal((nrhs, N))


def householder_tiles(N, NB, r, kappa, seed, device):
    """FP64 tile-major lower tiles of the Householder workload, generated on `device`."""
    import torch

    import ttg_gb300 as gbx
    lam, U, V, G = householder_factors(N, r, kappa, seed)
    t = torch.empty(gbx.tiled_numel(N, NB), dtype=torch.float64, device=device)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
    gbx.gen_lowrank(t, N, NB, to(lam), to(U), to(V), to(G))
    return t


def batch_sizes(count, lo, hi, step, seed=42):
    """`count` orders drawn uniformly from step * {lo..hi} (numpy default_rng(seed))."""
    return step * np.random.default_rng(seed).integers(lo, hi + 1, size=count)


def householder_batch(sizes, NB, r, kappa, seed, device, nrhs=0):
    """Concatenated tile-major lower tiles of a batch of Householder matrices (matrix k with seed
    seed + k), generated on `device`; with nrhs > 0 also the concatenated column-major right-hand
    sides (CUDA float64). Returns (tiles, rhs or None)."""
    import torch

    import ttg_gb300 as gbx
    offs, total = gbx.batched_tile_offsets(sizes, NB)
    t = torch.empty(total, dtype=torch.float64, device=device)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
    for k, n in enumerate(sizes):
        n = int(n)
        lam, U, V, G = householder_factors(n, r, kappa, seed + k)
        view = t[int(offs[k]):]
        gbx.gen_lowrank(view, n, NB, to(lam), to(U), to(V), to(G))
    if nrhs <= 0:
        return t, None
    b = np.concatenate([rhs(int(n), nrhs, seed + k).ravel() for k, n in enumerate(sizes)])
    return t, to(b)
