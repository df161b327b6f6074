"""GPU Hamiltonian construction and apply vs the CPU oracle.

Indices (indptr, indices) must be bit-exact; values too (the GPU arithmetic
is the oracle's, with the same term order); products within 1e-12 relative.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from tests.models import chain_maps, hubbard_static, ising_static, j1j2_static, square_maps, xxz_static

pytestmark = pytest.mark.gpu


def _cases():
    m = chain_maps(12)
    m10 = chain_maps(10)
    sq = square_maps(3, 3)
    return [
        ("xxz_k0p0", 12, 6, dict(kblock=(m["t"], 0), pblock=(m["p"], 0)), xxz_static(12), np.float64, 0),
        ("xxz_k0p1z0", 12, 6, dict(kblock=(m["t"], 0), pblock=(m["p"], 1), zblock=(m["z"], 0)), xxz_static(12),
         np.float64, 0),
        ("j1j2_k3", 12, 6, dict(kblock=(m["t"], 3)), j1j2_static(12), np.complex128, 0),
        ("j1j2_full", 10, 5, {}, j1j2_static(10), np.float64, 0),
        ("ising_k0p0", 10, None, dict(kblock=(m10["t"], 0), pblock=(m10["p"], 0)), ising_static(10), np.float64, 1),
        ("ising_k2", 10, None, dict(kblock=(m10["t"], 2)), ising_static(10), np.complex128, 1),
        ("ising_k5p1", 10, None, dict(kblock=(m10["t"], 5), pblock=(m10["p"], 1)), ising_static(10),
         np.complex64, 1),
        ("heis_sq", 9, 4, dict(tx=(sq["tx"], 1), ty=(sq["ty"], 0)),
         [["zz", [[1.0, i, sq["tx"][i]] for i in range(9)] + [[1.0, i, sq["ty"][i]] for i in range(9)]],
          ["+-", [[0.5, i, sq["tx"][i]] for i in range(9)] + [[0.5, i, sq["ty"][i]] for i in range(9)]],
          ["-+", [[0.5, i, sq["tx"][i]] for i in range(9)] + [[0.5, i, sq["ty"][i]] for i in range(9)]]],
         np.complex128, 0),
        ("xy_y", 8, None, {}, [["xy", [[0.3, i, (i + 1) % 8] for i in range(8)]],
                                ["yx", [[-0.3, i, (i + 1) % 8] for i in range(8)]]], np.complex128, 1),
    ]


@pytest.mark.parametrize("case", [c[0] for c in _cases()])
def test_csr_matches_oracle(cuda, case):
    from quspin_gb300 import hamiltonian, spin_basis_general
    name, L, Nup, blocks, static, dtype, pauli = [c for c in _cases() if c[0] == case][0]
    b = spin_basis_general(L, Nup=Nup, pauli=pauli, **blocks)
    ob = O.OracleBasis(L, [(1, Nup, 0)] if Nup is not None else [(0, 0, 0)], pauli=pauli, **blocks)
    H = hamiltonian(static, [], basis=b, dtype=dtype)
    Ho = O.make_static(ob, static, dtype)
    Hg = H.tocsr()
    Ho = sp.csr_matrix(Ho)
    np.testing.assert_array_equal(Hg.indptr, Ho.indptr)
    np.testing.assert_array_equal(Hg.indices, Ho.indices)
    np.testing.assert_array_equal(Hg.data, Ho.data)
    rng = np.random.default_rng(0)
    for shape in [(b.Ns,), (b.Ns, 3)]:
        v = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        y = H.dot(v)
        yo = Ho @ v
        assert np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)


def test_op_matches_oracle(cuda):
    from quspin_gb300 import spin_basis_general
    m = chain_maps(10)
    blocks = dict(kblock=(m["t"], 2), zblock=(m["z"], 1))
    b = spin_basis_general(10, Nup=5, pauli=0, **blocks)
    ob = O.OracleBasis(10, [(1, 5, 0)], pauli=0, **blocks)
    for opstr, indx in [("+-", [0, 1]), ("zz", [2, 5]), ("xy", [3, 4]), ("+-z", [1, 7, 2]), ("I", [0])]:
        ME, row, col = b.Op(opstr, indx, 0.7, np.complex128)
        MEo, rowo, colo = ob.Op(opstr, indx, 0.7, np.complex128)
        np.testing.assert_array_equal(row, rowo)
        np.testing.assert_array_equal(col, colo)
        np.testing.assert_array_equal(ME, MEo)


def test_hubbard_csr_and_known_energy(cuda):
    """4x4 Hubbard, Nf=(2,2), (kx,ky)=(0,0): CSR bit-exact vs the oracle and
    ground energy at U=4 equal to arXiv:cond-mat/0604319 (the known answer in
    the reference's test/test_FHM_energies_symm_adv.py:14-27) to 1e-12."""
    import scipy.sparse.linalg as sla
    from quspin_gb300 import hamiltonian, spinful_fermion_basis_general
    sq = square_maps(4, 4)
    b = spinful_fermion_basis_general(16, Nf=(2, 2), kx=(sq["tx"], 0), ky=(sq["ty"], 0))
    tx, _ = O.process_spinful_map(16, sq["tx"], 0)
    ty, _ = O.process_spinful_map(16, sq["ty"], 0)
    ob = O.OracleBasis(32, [(2, 2, 2)], fermion=True, spinful=True, kx=(tx, 0), ky=(ty, 0))
    st = hubbard_static(4, 4, t=1.0, U=4.0)
    H = hamiltonian(st, [], basis=b, dtype=np.float64)
    Ho = O.make_static(ob, st, np.float64)
    Hg = H.tocsr()
    np.testing.assert_array_equal(Hg.indptr, Ho.indptr)
    np.testing.assert_array_equal(Hg.indices, Ho.indices)
    np.testing.assert_array_equal(Hg.data, Ho.data)
    E0 = sla.eigsh(Hg, k=1, which="SA", tol=1e-14)[0][0]
    assert abs(E0 - (-11.5302924026297138)) < 1e-12


def test_dynamic_and_dia(cuda):
    """Diagonal-only static part is stored as DIA (base.py:299-304); dynamic
    part scaled by f(t) in dot (hamiltonian_core.py:769-772)."""
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(10)
    blocks = dict(kblock=(m["t"], 0), pblock=(m["p"], 0))
    b = spin_basis_general(10, **blocks)
    ob = O.OracleBasis(10, [(0, 0, 0)], pauli=1, **blocks)
    static = [["zz", [[-1.0, i, (i + 1) % 10] for i in range(10)]], ["z", [[-0.2, i] for i in range(10)]]]
    drive = lambda t, h0, A, w: h0 + A * np.cos(w * t)
    dyn = [["x", [[-1.0, i] for i in range(10)], drive, (0.8, 0.5, 2 * np.pi)]]
    H = hamiltonian(static, dyn, basis=b, dtype=np.float64)
    assert H.static.format == "dia"
    S = O.make_static(ob, static, np.float64)
    X = O.make_static(ob, [["x", [[-1.0, i] for i in range(10)]]], np.float64)
    np.testing.assert_array_equal(sp.dia_matrix(S).data.ravel(), H.static.tocsr().diagonal())
    rng = np.random.default_rng(3)
    v = rng.normal(size=b.Ns) + 1j * rng.normal(size=b.Ns)
    for t in (0.0, 0.37):
        y = H.dot(v, time=t)
        yo = S @ v + drive(t, 0.8, 0.5, 2 * np.pi) * (X @ v)
        assert np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)
        Hc = H.tocsr_gpu(t).tocsr()
        assert abs(Hc - (S + drive(t, 0.8, 0.5, 2 * np.pi) * X)).max() < 1e-14


def test_dot_out_semantics(cuda):
    import torch
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(10)
    b = spin_basis_general(10, Nup=5, kblock=(m["t"], 0))
    H = hamiltonian(xxz_static(10), [], basis=b, dtype=np.float64)
    Hs = H.tocsr()
    rng = np.random.default_rng(4)
    v = rng.normal(size=b.Ns)
    out = rng.normal(size=b.Ns)
    o2 = out.copy()
    H.dot(v, out=out, overwrite_out=False, a=0.5)
    np.testing.assert_allclose(out, o2 + 0.5 * (Hs @ v), rtol=0, atol=1e-12)
    vd = torch.tensor(v, device="cuda")
    yd = H.dot(vd)
    assert yd.is_cuda
    np.testing.assert_allclose(yd.cpu().numpy(), Hs @ v, rtol=0, atol=1e-12)
    with pytest.raises(ValueError):
        H.dot(np.zeros(b.Ns + 1))


def test_conj_transpose(cuda):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(10)
    b = spin_basis_general(10, kblock=(m["t"], 3))
    st = [["xy", [[0.3, i, (i + 1) % 10] for i in range(10)]], ["zz", [[0.7, i, (i + 2) % 10] for i in range(10)]],
          ["x", [[0.2, i] for i in range(10)]]]
    A = hamiltonian(st, [], basis=b, dtype=np.complex128).tocsr_gpu()
    AH = A.conj_transpose().tocsr()
    ref = sp.csr_matrix(A.tocsr().conj().T)
    ref.sort_indices()
    np.testing.assert_array_equal(AH.indptr, ref.indptr)
    np.testing.assert_array_equal(AH.indices, ref.indices)
    np.testing.assert_array_equal(AH.data, ref.data)


def test_conj_transpose_long_column(cuda):
    """A column with more than 512 entries (beyond the merge kernel's per-row
    sort) is transposed on the device by one sort of the (column, row) keys;
    the result equals scipy's conjugate transpose."""
    from quspin_gb300.sparse import DeviceCSR
    rng = np.random.default_rng(3)
    n = 5000
    A = sp.random(n, n, density=4.0 / n, random_state=4, format="lil", dtype=np.complex128)
    A[:, 17] = (rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1)))       # a full column
    A = sp.csr_matrix(A)
    A.sum_duplicates()
    A.eliminate_zeros()
    assert A.getcol(17).nnz > 512
    AH = DeviceCSR.from_scipy(A).conj_transpose().tocsr()
    ref = sp.csr_matrix(A.conj().T)
    ref.sort_indices()
    np.testing.assert_array_equal(AH.indptr, ref.indptr)
    np.testing.assert_array_equal(AH.indices, ref.indices)
    np.testing.assert_array_equal(AH.data, ref.data)
