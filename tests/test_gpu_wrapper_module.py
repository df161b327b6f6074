"""The native-layer drop-in: quspin_gb300.expm_multiply_parallel_wrapper
called exactly as the reference's ExpmMultiplyParallel body calls
parallel-sparse-tools' wrapper module
(docs/modules/parallel_sparse_tools/expm_multiply_parallel_core/
expm_multiply_parallel_core.html :96-103 and :248-272), on the inputs of the
committed reference run (tests/golden/c1_xxz_L20.npz): the shift, the 1-norm
and the evolved state reproduce the reference's values."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wrapper_functions_reproduce_reference_run(cuda):
    import quspin_gb300.expm_multiply_parallel_wrapper as W
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "c1_xxz_L20.npz"))
    indptr, indices, data = g["indptr"], g["indices"], g["data"]
    n = len(indptr) - 1
    # construction (html :96-103): mu = trace / n, 1-norm of A - mu I
    mu = np.array(W._wrapper_csr_trace(indptr, indices, data) / n, dtype=np.complex128)
    assert abs(complex(mu) - complex(g["mu"])) <= 1e-15 * max(1.0, abs(complex(g["mu"])))
    nrm = W._wrapper_csr_1_norm(indptr, indices, data, -mu)
    assert abs(nrm - float(g["A_1_norm"])) <= 1e-14 * float(g["A_1_norm"])
    # dot (html :241-260): in place on v, with the reference's s, m*, tol and mu
    tol = np.array(np.finfo(np.complex128).eps / 2, dtype=np.float64)
    a = np.array(-1j, dtype=np.complex128)
    mu_ref = np.array(complex(g["mu"]), dtype=np.complex128)
    ref = g["expm_ref"]
    old = W.PRECISION
    try:
        for prec in ("double", "ieee"):
            W.PRECISION = prec
            v = g["v"].copy()
            work = np.zeros(2 * v.size, dtype=np.complex128)
            W._wrapper_expm_multiply(indptr, indices, data, int(g["s"]), int(g["m_star"]), tol, mu_ref, a, v,
                                     work)
            assert np.linalg.norm(v - ref) <= 1e-12 * np.linalg.norm(ref), prec
            # the batch form on [n, 2] (html :261-272): both columns the same state
            V = np.ascontiguousarray(np.stack([g["v"], g["v"]], axis=1))
            W._wrapper_expm_multiply_batch(indptr, indices, data, int(g["s"]), int(g["m_star"]), tol, mu_ref, a,
                                           V, np.zeros((2 * n, 2), dtype=np.complex128))
            for c in range(2):
                assert np.linalg.norm(V[:, c] - ref) <= 1e-12 * np.linalg.norm(ref), prec
    finally:
        W.PRECISION = old
