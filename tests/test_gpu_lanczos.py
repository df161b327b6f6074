"""GPU Lanczos vs the oracle restatement of the reference's recurrence and
vs dense diagonalisation (test/test_Lanczos.py:8-78: m=20..50 steps, ground
energy within 1e-10 of eigsh; expm_lanczos vs scipy at 1e-10)."""
import numpy as np
import pytest
from scipy.sparse.linalg import eigsh, expm_multiply

from oracle import oracle as O
from tests.models import chain_maps, xxz_static

pytestmark = pytest.mark.gpu


def _H(L=14, dtype=np.float64):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, kblock=(m["t"], 0), pblock=(m["p"], 0), pauli=0)
    return hamiltonian(xxz_static(L), [], basis=b, dtype=dtype)


def test_lanczos_full_matches_oracle(cuda):
    from quspin_gb300.tools import lanczos_full
    H = _H()
    A = H.tocsr()
    rng = np.random.default_rng(0)
    v0 = rng.normal(size=H.Ns)
    E, V, Q = lanczos_full(H, v0, 20)
    Eo, Vo, Qo, ao, bo = O.lanczos_full(lambda x: A @ x, A.dtype, v0, 20)
    np.testing.assert_allclose(E, Eo, rtol=0, atol=1e-10)
    np.testing.assert_allclose(np.abs(Q), np.abs(Qo), rtol=0, atol=1e-8)


def test_lanczos_ground_state(cuda):
    from quspin_gb300.tools import lanczos_full, lanczos_iter, lin_comb_Q_T
    H = _H(20)
    A = H.tocsr()
    E_ex = eigsh(A, k=1, which="SA")[0][0]
    rng = np.random.default_rng(1)
    v0 = rng.normal(size=H.Ns)
    E, V, Q = lanczos_full(H, v0, 50)
    assert abs(E[0] - E_ex) < 1e-10
    E2, V2, Qit = lanczos_iter(H, v0, 50)
    assert abs(E2[0] - E_ex) < 1e-10
    g1 = lin_comb_Q_T(V[:, 0], Q)
    g2 = lin_comb_Q_T(V2[:, 0], Qit)
    # the iterator regenerates the same vectors with the same kernels
    np.testing.assert_allclose(g1, g2, rtol=0, atol=1e-13)
    g1 /= np.linalg.norm(g1)
    r = A @ g1 - E[0] * g1
    assert np.linalg.norm(r) < 1e-5


def test_expm_lanczos(cuda):
    from quspin_gb300.tools import expm_lanczos, lanczos_full
    H = _H(12)
    A = H.tocsr()
    rng = np.random.default_rng(2)
    v0 = rng.normal(size=H.Ns)
    v0 /= np.linalg.norm(v0)
    E, V, Q = lanczos_full(H, v0, 20)
    w = expm_lanczos(E, V, Q, a=-0.1j)
    ws = expm_multiply(-0.1j * A, v0)
    np.testing.assert_allclose(w, ws, rtol=0, atol=1e-10)


def test_full_ortho_and_reorth(cuda):
    from quspin_gb300.tools import lanczos_full
    H = _H()
    A = H.tocsr()
    E_ex = np.sort(eigsh(A, k=4, which="SA")[0])
    rng = np.random.default_rng(3)
    v0 = rng.normal(size=H.Ns)
    E, V, Q = lanczos_full(H, v0, 60, full_ortho=True)
    assert abs(E[0] - E_ex[0]) < 1e-10
    E, V, Q = lanczos_full(H, v0, 60, reorth=True)
    np.testing.assert_allclose(E[:3], E_ex[:3], rtol=0, atol=1e-9)
    G = Q @ Q.T
    assert np.abs(G - np.eye(len(E))).max() < 1e-12


def test_complex_start_vector(cuda):
    from quspin_gb300.tools import lanczos_full
    H = _H(12, dtype=np.complex128)
    A = H.tocsr()
    rng = np.random.default_rng(4)
    v0 = rng.normal(size=H.Ns) + 1j * rng.normal(size=H.Ns)
    E, V, Q = lanczos_full(H, v0, 12)
    Eo, Vo, Qo, ao, bo = O.lanczos_full(lambda x: A @ x, A.dtype, v0, 12)
    # early steps, before loss of orthogonality amplifies rounding differences
    np.testing.assert_allclose(E, Eo, rtol=0, atol=1e-10)
    np.testing.assert_allclose(np.abs(Q), np.abs(Qo), rtol=0, atol=1e-10)


def test_mixed_precision_lanczos(cuda):
    """complex64 / float32 matrix values with FP64 vectors and recurrence:
    ground energy within 1e-6 of the FP64 run."""
    from quspin_gb300.tools import lanczos_full
    H = _H(16)
    rng = np.random.default_rng(5)
    v0 = rng.normal(size=H.Ns)
    E64 = lanczos_full(H, v0, 60, reorth=True)[0]
    E32 = lanczos_full(H, v0, 60, reorth=True, precision="mixed")[0]
    assert abs(E64[0] - E32[0]) < 1e-6 * max(1.0, abs(E64[0]))


def test_ftlm_ltlm_against_reference_golden(cuda):
    """Device FTLM / LTLM iterations on the reference's own Lanczos data give
    the reference functions' results (tests/golden/thermal_xxz_L14.npz), with
    the operators as device matrices and Q_T on the device or as an
    iterator."""
    import os
    import torch
    import scipy.sparse as sp
    from quspin_gb300.sparse import DeviceCSR
    from quspin_gb300.tools import FTLM_static_iteration, LTLM_static_iteration
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "thermal_xxz_L14.npz"))
    n = g["v0"].size
    H = sp.csr_matrix((g["H_data"], g["H_indices"], g["H_indptr"]), shape=(n, n))
    C = sp.csr_matrix((g["C_data"], g["C_indices"], g["C_indptr"]), shape=(n, n))
    ops = {"H": DeviceCSR.from_scipy(H), "Czz": DeviceCSR.from_scipy(C)}
    Q = torch.tensor(g["Q_T"], device="cuda")
    Of, If = FTLM_static_iteration(ops, g["E"], g["V"], Q, beta=g["beta"])
    np.testing.assert_allclose(Of["H"], g["ftlm_H"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(Of["Czz"], g["ftlm_C"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(If, g["ftlm_I"], rtol=1e-12)
    Ol, Il = LTLM_static_iteration(ops, g["E"], g["V"], iter(list(Q)), beta=g["beta"])
    np.testing.assert_allclose(Ol["H"], g["ltlm_H"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(Ol["Czz"], g["ltlm_C"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(Il, g["ltlm_I"], rtol=1e-12)
