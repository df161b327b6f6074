"""Array equality with the oracle at the benchmark configurations' full sizes.

The GPU basis (states and orbit norms) and the canonical CSR the GPU builds
(indptr, column indices and values) are compared element for element with
the oracle's restatement of the reference's basis core and of
``_make_matrix`` (src/quspin/basis/basis_general/base_general.py:292-352,
817-899; src/quspin/basis/base.py:265-304), built on the host cores:

* the L=32 J1-J2 chain, Sz=0, k=0, p=+1, z=+1 (4,707,969 states, 159,282,583
  nonzeros) -- the benchmark matrix;
* four of the 26 momentum / reflection blocks of the L=24 mixed-field Ising
  chain: k=0 (p=+1) and k=12 (p=-1), real, and k=1, k=5, complex;
* the spinful Fermi-Hubbard 4x4 lattice, N_up = N_down = 5, (kx, ky) = (0, 0):
  complex CSR with fermion signs;
* the driven Ising chain L=26, k=0, p=+1: the diagonal static part (DIA) and
  the sigma^x drive (CSR).

The small configuration (XXZ chain L=20) is compared with the output of the
reference's own Python code run once (tests/golden/c1_xxz_L20.npz, made by
tests/golden/make_golden.py): the CSR, the (m*, s) selection, the evolved
state at 1e-12 relative and the converged 60-step Lanczos energies.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.models import chain_maps, hubbard_static, ising_static, j1j2_static, square_maps, xxz_static

pytestmark = pytest.mark.gpu


def _assert_csr_equal(Ag, Ao):
    """Device CSR Ag against scipy CSR Ao: same row pointers, column indices
    and value bits."""
    assert Ag.shape == Ao.shape
    ip = Ag.indptr.cpu().numpy().astype(np.int64)
    np.testing.assert_array_equal(ip, Ao.indptr.astype(np.int64))
    nnz = int(ip[-1])
    np.testing.assert_array_equal(Ag.indices[:nnz].cpu().numpy(), Ao.indices.astype(np.int32))
    dg = Ag.data[:nnz].cpu().numpy()
    do = Ao.data.astype(dg.dtype)
    # bit patterns, so that -0.0 / 0.0 and the last ulp count
    np.testing.assert_array_equal(dg.view(np.int64), do.view(np.int64))


def _assert_basis_equal(b, ob):
    assert b.Ns == ob.Ns
    np.testing.assert_array_equal(np.asarray(b.states).astype(np.uint64), ob.states)
    np.testing.assert_array_equal(np.asarray(b._n).astype(np.uint32), ob.norms)


def test_j1j2_L32_basis_and_csr_equal_oracle(cuda):
    from quspin_gb300 import hamiltonian, spin_basis_general
    L = 32
    m = chain_maps(L)
    blocks = dict(kblock=(m["t"], 0), pblock=(m["p"], 0), zblock=(m["z"], 0))
    b = spin_basis_general(L, Nup=L // 2, pauli=0, **blocks)
    H = hamiltonian(j1j2_static(L), [], basis=b, dtype=np.float64)
    Ag = H.tocsr_gpu()
    ob = O.OracleBasis(L, [(1, L // 2, 0)], pauli=0, **blocks)
    _assert_basis_equal(b, ob)
    Ao = ob.build_csr(O.consolidate_static(j1j2_static(L)), np.float64)
    assert Ao.nnz == 159282583
    _assert_csr_equal(Ag, Ao)


@pytest.mark.parametrize("k,p", [(0, 0), (12, 1), (1, None), (5, None)])
def test_ising_L24_blocks_equal_oracle(cuda, k, p):
    from quspin_gb300 import hamiltonian, spin_basis_general
    L = 24
    m = chain_maps(L)
    blocks = dict(kblock=(m["t"], k))
    if p is not None:
        blocks["pblock"] = (m["p"], p)
    dt = np.float64 if k in (0, 12) else np.complex128
    b = spin_basis_general(L, **blocks)
    Ag = hamiltonian(ising_static(L), [], basis=b, dtype=dt).tocsr_gpu()
    ob = O.OracleBasis(L, [(0, 0, 0)], pauli=1, **blocks)
    _assert_basis_equal(b, ob)
    _assert_csr_equal(Ag, ob.build_csr(O.consolidate_static(ising_static(L)), dt))


def test_hubbard_4x4_complex_csr_equal_oracle(cuda):
    from quspin_gb300 import hamiltonian, spinful_fermion_basis_general
    sq = square_maps(4, 4)
    b = spinful_fermion_basis_general(16, Nf=(5, 5), kx=(sq["tx"], 0), ky=(sq["ty"], 0))
    Ag = hamiltonian(hubbard_static(4, 4), [], basis=b, dtype=np.complex128).tocsr_gpu()
    tx, _ = O.process_spinful_map(16, sq["tx"], 0)
    ty, _ = O.process_spinful_map(16, sq["ty"], 0)
    ob = O.OracleBasis(32, [(2, 5, 5)], fermion=True, spinful=True, kx=(tx, 0), ky=(ty, 0))
    _assert_basis_equal(b, ob)
    Ao = ob.build_csr(O.consolidate_static(hubbard_static(4, 4)), np.complex128)
    assert np.iscomplexobj(Ao.data) and Ao.nnz == 36044706
    _assert_csr_equal(Ag, Ao)


def test_driven_L26_static_dia_and_drive_csr_equal_oracle(cuda):
    from quspin_gb300 import hamiltonian, spin_basis_general
    from quspin_gb300.sparse import DeviceCSR, DeviceDIA
    L = 26
    m = chain_maps(L)
    blocks = dict(kblock=(m["t"], 0), pblock=(m["p"], 0))
    static = [["zz", [[-1.0, i, (i + 1) % L] for i in range(L)]], ["z", [[-0.2, i] for i in range(L)]]]
    drive = [["x", [[-1.0, i] for i in range(L)], lambda t: np.cos(t), ()]]
    b = spin_basis_general(L, **blocks)
    H = hamiltonian(static, drive, basis=b, dtype=np.float64)
    ob = O.OracleBasis(L, [(0, 0, 0)], pauli=1, **blocks)
    _assert_basis_equal(b, ob)
    assert isinstance(H.static, DeviceDIA)
    diag_o = ob.build_csr(O.consolidate_static(static), np.float64).diagonal()
    dg = H.static.data.reshape(-1).cpu().numpy()
    np.testing.assert_array_equal(dg.view(np.int64), diag_o.view(np.int64))
    (Hd,) = H.dynamic.values()
    assert isinstance(Hd, DeviceCSR)
    _assert_csr_equal(Hd, ob.build_csr(O.consolidate_static([["x", [[-1.0, i] for i in range(L)]]]), np.float64))


def test_xxz_L20_against_reference_run_fixture(cuda):
    """GPU path vs outputs of the reference's own ExpmMultiplyParallel body and
    _lanczos_utils.lanczos_full (tests/golden/make_golden.py)."""
    import os
    from quspin_gb300 import hamiltonian, spin_basis_general
    from quspin_gb300.tools import ExpmMultiplyParallel, lanczos_full
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "c1_xxz_L20.npz"))
    L = 20
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, pauli=0, kblock=(m["t"], 0), pblock=(m["p"], 0))
    np.testing.assert_array_equal(np.asarray(b.states).astype(np.uint64), g["states"])
    H = hamiltonian(xxz_static(L, 1.0, 0.5), [], basis=b, dtype=np.float64)
    Ag = H.tocsr_gpu()
    np.testing.assert_array_equal(Ag.indptr.cpu().numpy(), g["indptr"])
    np.testing.assert_array_equal(Ag.indices.cpu().numpy(), g["indices"])
    np.testing.assert_array_equal(Ag.data.cpu().numpy().view(np.int64), g["data"].view(np.int64))
    np.random.seed(0)
    op = ExpmMultiplyParallel(Ag, a=-1j)
    assert (op.m_star, op.s) == (int(g["m_star"]), int(g["s"]))
    assert abs(complex(op._mu) - complex(g["mu"])) <= 1e-15 * max(1.0, abs(complex(g["mu"])))
    assert abs(op._A_1_norm - float(g["A_1_norm"])) <= 1e-14 * float(g["A_1_norm"])
    ref = g["expm_ref"]
    for prec, tol in (("double", 1e-12), ("ieee", 1e-12)):
        op.precision = prec
        w = op.dot(g["v"])
        assert np.linalg.norm(w - ref) <= tol * np.linalg.norm(ref), prec
    # 60 steps without reorthogonalisation: the two lowest Ritz values have
    # converged and agree; the others include rounding-dependent ghosts, which
    # differ between any two implementations
    E, V, Q = lanczos_full(H, g["v0"], 60)
    Er = g["lanczos_E"]
    np.testing.assert_allclose(E[:2], Er[:2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(E.min(), Er.min(), rtol=0, atol=1e-10)
