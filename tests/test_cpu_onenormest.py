"""The device 1-norm estimator (Higham & Tisseur's block algorithm, run
here on CPU torch tensors): never above the exact norm, exact for small
identity-sized problems, and close to scipy's onenormest on the same inputs."""
import numpy as np
import scipy.sparse as sp
import torch
from scipy.sparse.linalg import onenormest

from quspin_gb300.tools._onenormest import onenormest_device


def _ops(A):
    At = torch.tensor(A)
    return (lambda X: At @ X), (lambda X: At.conj().T @ X)


def test_estimate_bounds_and_agreement():
    rng = np.random.default_rng(0)
    exact_hits = 0
    for trial in range(20):
        n = 300
        A = sp.random(n, n, density=0.03, random_state=rng).toarray()
        A = A + 1j * sp.random(n, n, density=0.03, random_state=rng).toarray()
        exact = np.abs(A).sum(axis=0).max()
        np.random.seed(trial)
        mm, rmm = _ops(A)
        est = onenormest_device(mm, rmm, n, torch.complex128, "cpu", t=2)
        assert est <= exact * (1 + 1e-12)
        assert est >= 0.3 * exact
        np.random.seed(trial)
        sci = onenormest(sp.csr_matrix(A), t=2)
        assert est >= 0.5 * sci
        exact_hits += abs(est - exact) <= 1e-12 * exact
    assert exact_hits >= 10


def test_small_n_is_exact():
    A = np.arange(9, dtype=np.float64).reshape(3, 3) - 4
    mm, rmm = _ops(A.astype(np.complex128))
    assert abs(onenormest_device(mm, rmm, 3, torch.complex128, "cpu", t=4) - np.abs(A).sum(0).max()) < 1e-12
