"""The learned (m*, s) selection in the estimator branch of the reference's
partition (html expm_multiply_parallel_core.html:451-463, where onenormest
runs tens of products with the matrix): what it gains and how it falls back.

A NormRatioPredictor is trained on the GPU (csrc/mlp.cu) on the plain
selection's norm ratios of small J1-J2 chains (L = 12 .. 20, several J2 and
both spin-inversion sectors) and used on a chain it has not seen (L = 24,
J2 = 0.4) at t = 5, the benchmark's regime.  Compared with the plain selection on the
same operator: no products with the matrix for the selection, a comparable
Taylor cost, and the same state within 1e-12.  A predictor forced to predict
far too small norms triggers the fallback, which reproduces the plain
result."""
import time

import numpy as np
import pytest

from tests.models import chain_maps, j1j2_static

pytestmark = pytest.mark.gpu


def _j1j2(L, J2, z=0):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, pauli=0, kblock=(m["t"], 0), pblock=(m["p"], 0), zblock=(m["z"], z))
    return hamiltonian(j1j2_static(L, 1.0, J2), [], basis=b, dtype=np.float64).tocsr_gpu()


@pytest.fixture(scope="module")
def predictor(cuda):
    from quspin_gb300.learned import NormRatioPredictor, norm_ratio_training_set
    mats = [_j1j2(L, J2, z) for L in (12, 14, 16, 18, 20) for J2 in (0.0, 0.25, 0.5, 0.75, 1.0) for z in (0, 1)]
    f, r = norm_ratio_training_set(mats)
    pred = NormRatioPredictor(seed=0)
    hist = pred.fit(f, r, epochs=600)
    assert hist[-1] < 0.05 * hist[0]
    return pred


def test_learned_selection_makes_no_norm_products(cuda, predictor):
    from quspin_gb300.tools import ExpmMultiplyParallel
    A = _j1j2(24, 0.4)
    n = A.shape[0]
    rng = np.random.default_rng(0)
    v = rng.normal(size=n) + 1j * rng.normal(size=n)
    v /= np.linalg.norm(v)
    np.random.seed(0)
    t0 = time.perf_counter()
    plain = ExpmMultiplyParallel(A, a=-5j)
    t_plain = time.perf_counter() - t0
    assert plain.partition_source == "plain" and plain.norm_products > 0
    learned = ExpmMultiplyParallel(A, a=-5j)
    t0 = time.perf_counter()
    learned.set_predictor(predictor)
    t_learned = time.perf_counter() - t0
    assert learned.partition_source == "learned" and learned.norm_products == 0
    assert t_learned < t_plain
    w_plain = plain.dot(v)
    w_learned = learned.dot(v)
    assert learned.fallbacks == 0
    assert np.linalg.norm(w_learned - w_plain) <= 1e-12 * np.linalg.norm(w_plain)
    # the predicted (m*, s) costs at most 30% more Taylor terms than the plain one
    assert learned.m_star * learned.s <= 1.3 * plain.m_star * plain.s
    assert learned.terms_executed <= 1.3 * plain.terms_executed


def test_too_small_prediction_falls_back_to_plain(cuda, predictor):
    from quspin_gb300.learned import NormRatioPredictor
    from quspin_gb300.tools import ExpmMultiplyParallel

    class Tiny(NormRatioPredictor):
        def __init__(self, base):
            self.__dict__.update(base.__dict__)

        def predict_ratios(self, feats):
            return 1e-3 * super().predict_ratios(feats)

    A = _j1j2(18, 0.5)
    n = A.shape[0]
    rng = np.random.default_rng(1)
    v = rng.normal(size=n) + 1j * rng.normal(size=n)
    v /= np.linalg.norm(v)
    np.random.seed(0)
    plain = ExpmMultiplyParallel(A, a=-5j)
    w_plain = plain.dot(v)
    op = ExpmMultiplyParallel(A, a=-5j)
    op.set_predictor(Tiny(predictor))
    assert op.partition_source == "learned" and op.m_star * op.s < plain.m_star * plain.s
    np.random.seed(0)                     # the fallback's onenormest draws as the plain one did
    w = op.dot(v)
    assert op.fallbacks == 1 and op.partition_source == "plain"
    assert (op.m_star, op.s) == (plain.m_star, plain.s)
    assert np.array_equal(w.view(np.float64), w_plain.view(np.float64))
