"""CPU checks of the benchmark workload generators."""
import numpy as np
import pytest

from ttg_gb300 import workloads


@pytest.mark.parametrize("N,r,kappa", [(200, 4, 1e6), (257, 2, 1e4), (64, 1, 10.0)])
def test_householder_closed_form_matches_reflector_products(N, r, kappa):
    lam, U, V, G = workloads.householder_factors(N, r, kappa, seed=42)
    A_closed = np.diag(lam) - (U @ V.T) * lam[None, :] - lam[:, None] * (V @ U.T) + U @ G @ U.T
    A_ref = workloads.householder_dense(N, r, kappa, seed=42)
    assert np.abs(A_closed - A_ref).max() <= 1e-14
    assert np.allclose(A_ref, A_ref.T, atol=1e-15)
    w = np.linalg.eigvalsh(A_ref)
    assert w.min() > 0 and abs(w.max() / w.min() / kappa - 1) < 1e-6
