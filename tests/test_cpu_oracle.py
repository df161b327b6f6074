"""CPU checks of the oracle (no GPU): known answers from the reference's own
tests, invariants, and the committed golden fixtures."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla
from scipy.sparse.linalg import expm_multiply

from oracle import oracle as O
from tests.models import chain_maps, hubbard_static, square_maps, xxz_static

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# arXiv:cond-mat/0604319 Sec. III A, as quoted by test/test_FHM_energies.py:20-33
E_PAPER = -np.array([12.0000000000000000, 11.9126285145094126, 11.8364690235642218, 11.7695877912829268,
                     11.7104580743242632, 11.6578605150913841, 11.6108110503797608, 11.5685079573602838,
                     11.5302924026297138])


def test_c1_dimension_and_golden_basis():
    m = chain_maps(20)
    ob = O.OracleBasis(20, [(1, 10, 0)], pauli=0, kblock=(m["t"], 0), pblock=(m["p"], 0))
    g = np.load(os.path.join(GOLD, "c1_xxz_L20.npz"))
    assert ob.Ns == 4752
    np.testing.assert_array_equal(ob.states, g["states"])
    np.testing.assert_array_equal(ob.norms, g["norms"])
    H = sp.csr_matrix(O.make_static(ob, xxz_static(20), np.float64))
    np.testing.assert_array_equal(H.indptr, g["indptr"])
    np.testing.assert_array_equal(H.indices, g["indices"])
    np.testing.assert_array_equal(H.data, g["data"])


def test_fhm_known_answers_symmetric_sector():
    """test/test_FHM_energies_symm_adv.py: kx=ky=0 sector, advanced maps."""
    N = 16
    sq = square_maps(4, 4)
    TX, TY = np.hstack((sq["tx"], sq["tx"] + N)), np.hstack((sq["ty"], sq["ty"] + N))
    ob = O.OracleBasis(2 * N, [(2, 2, 2)], fermion=True, spinful=True, ky=(TY, 0), kx=(TX, 0))
    Jp = [[1.0, i, TX[i]] for i in range(2 * N)] + [[1.0, i, TY[i]] for i in range(2 * N)]
    Jm = [[-1.0, i, TX[i]] for i in range(2 * N)] + [[-1.0, i, TY[i]] for i in range(2 * N)]
    H0 = O.make_static(ob, [["+-", Jp], ["-+", Jm]], np.float64)
    H1 = O.make_static(ob, [["nn", [[1.0, i, i + N] for i in range(N)]]], np.float64)
    E = [np.linalg.eigvalsh((H0 + U * H1).toarray())[0] for U in np.linspace(0.0, 4.0, 9)]
    np.testing.assert_allclose(E, E_PAPER, atol=1e-12)


def test_fhm_simple_symmetry_matches_advanced():
    sq = square_maps(4, 4)
    ob = O.OracleBasis(32, [(2, 2, 2)], fermion=True, spinful=True,
                       kx=O.process_spinful_map(16, sq["tx"], 0), ky=O.process_spinful_map(16, sq["ty"], 0))
    H = O.make_static(ob, hubbard_static(4, 4, 1.0, 4.0), np.float64)
    assert abs(np.linalg.eigvalsh(H.toarray())[0] - E_PAPER[-1]) < 1e-12


def test_sector_sums_and_spectra():
    """test/test_sq_lat_Heis.py:19-56 on a 3x3 lattice: Ns of all momentum x
    inversion blocks sums to the particle sector and the spectra agree."""
    sq = square_maps(3, 3)
    J = [[1.0, i, sq["tx"][i]] for i in range(9)] + [[1.0, i, sq["ty"][i]] for i in range(9)]
    st = [["zz", J], ["+-", J], ["-+", J]]
    for Nup in (3, 4):
        full = O.OracleBasis(9, [(1, Nup, 0)], pauli=1)
        Ef = np.linalg.eigvalsh(O.make_static(full, st, np.float64).toarray())
        tot, Es = 0, []
        for kx in range(3):
            for ky in range(3):
                b = O.OracleBasis(9, [(1, Nup, 0)], pauli=1, tx=(sq["tx"], kx), ty=(sq["ty"], ky))
                tot += b.Ns
                if b.Ns:
                    Es.append(np.linalg.eigvalsh(O.make_static(b, st, np.complex128).toarray()))
        assert tot == full.Ns
        np.testing.assert_allclose(np.sort(np.concatenate(Es)), Ef, atol=1e-12)


def test_oracle_expm_matches_golden_and_scipy():
    g = np.load(os.path.join(GOLD, "c1_xxz_L20.npz"))
    H = sp.csr_matrix((g["data"], g["indices"], g["indptr"]))
    np.random.seed(0)
    e = O.ExpmMultiplyParallelOracle(H, a=-1j)
    assert (e._m_star, e._s) == (int(g["m_star"]), int(g["s"]))
    w = e.dot(g["v"])
    np.testing.assert_allclose(w, g["expm_ref"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(w, g["expm_scipy"], rtol=0, atol=1e-14)
    r = np.load(os.path.join(GOLD, "random_complex_N3500.npz"))
    A = sp.csr_matrix((r["data"], r["indices"], r["indptr"]))
    y = O.ExpmMultiplyParallelOracle(A, a=-0.7j).dot(r["x"])
    np.testing.assert_allclose(y, r["expm_scipy"], rtol=0, atol=1e-15)


def test_oracle_lanczos_matches_reference_golden():
    g = np.load(os.path.join(GOLD, "c1_xxz_L20.npz"))
    H = sp.csr_matrix((g["data"], g["indices"], g["indptr"]))
    E = O.lanczos_full(lambda x: H @ x, H.dtype, g["v0"], 60)[0]
    np.testing.assert_allclose(E, g["lanczos_E"], rtol=0, atol=1e-12)
    assert abs(E[0] - sla.eigsh(H, k=1, which="SA")[0][0]) < 1e-10


def test_partition_restatement_matches_scipy():
    """quspin_gb300.tools._partition restates Al-Mohy & Higham Code Fragment
    3.1; compare with scipy's implementation, which the reference calls."""
    from scipy.sparse.linalg._expm_multiply import LazyOperatorNormInfo as SciInfo
    from scipy.sparse.linalg._expm_multiply import _fragment_3_1
    from quspin_gb300.tools import _partition as P
    rng = np.random.default_rng(0)
    for scale in (1e-3, 0.5, 3.0, 30.0, 80.0, 400.0):
        A = sp.random(200, 200, density=0.05, random_state=rng, format="csr") * scale
        A = A + A.T
        np.random.seed(5)
        ref = _fragment_3_1(SciInfo(A, A_1_norm=sla.norm(A, 1), ell=2), 1, 2.0 ** -53, ell=2)
        np.random.seed(5)
        info = P.LazyOperatorNormInfo(lambda v: A @ v, lambda v: A.T @ v, 200, sla.norm(A, 1), 1.0,
                                      np.dtype(np.float64))
        assert P.fragment_3_1(info, 1, 2.0 ** -53, ell=2) == ref


def test_oracle_taylor_vs_scipy_batch():
    m = chain_maps(12)
    ob = O.OracleBasis(12, [(1, 6, 0)], pauli=0, kblock=(m["t"], 0))
    H = sp.csr_matrix(O.make_static(ob, xxz_static(12), np.float64))
    rng = np.random.default_rng(1)
    V = rng.normal(size=(ob.Ns, 5)) + 1j * rng.normal(size=(ob.Ns, 5))
    V /= np.linalg.norm(V, axis=0)
    W = O.ExpmMultiplyParallelOracle(H, a=-2j).dot(V)
    np.testing.assert_allclose(W, expm_multiply(-2j * H, V), rtol=0, atol=5e-14)


def test_op_masks_and_pauli_scaling():
    m = chain_maps(8)
    b0 = O.OracleBasis(8, [(1, 4, 0)], pauli=0, kblock=(m["t"], 0))
    b1 = O.OracleBasis(8, [(1, 4, 0)], pauli=1, kblock=(m["t"], 0))
    ME0, r0, c0 = b0.Op("+-", [3, 4], 1.0, np.float64)
    ME1, r1, c1 = b1.Op("+-", [3, 4], 1.0, np.float64)
    np.testing.assert_array_equal(ME1, 4 * ME0)
    assert np.all(ME0 != 0)
    with pytest.raises(TypeError):
        O.make_static(O.OracleBasis(8, [(1, 4, 0)], pauli=0, kblock=(m["t"], 1)), xxz_static(8), np.float64)


def test_oracle_ftlm_ltlm_match_reference_golden():
    """FTLM / LTLM iterations restated in the oracle equal the reference's
    own functions (_FTLM.py, _LTLM.py run unmodified by
    tests/golden/make_golden.py) on the same Lanczos data."""
    g = np.load(os.path.join(GOLD, "thermal_xxz_L14.npz"))
    n = g["v0"].size
    H = sp.csr_matrix((g["H_data"], g["H_indices"], g["H_indptr"]), shape=(n, n))
    C = sp.csr_matrix((g["C_data"], g["C_indices"], g["C_indptr"]), shape=(n, n))
    ops = {"H": H, "Czz": C}
    Of, If = O.ftlm_static_iteration(ops, g["E"], g["V"], g["Q_T"], beta=g["beta"])
    np.testing.assert_allclose(Of["H"], g["ftlm_H"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(Of["Czz"], g["ftlm_C"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(If, g["ftlm_I"], rtol=1e-12)
    Ol, Il = O.ltlm_static_iteration(ops, g["E"], g["V"], g["Q_T"], beta=g["beta"])
    np.testing.assert_allclose(Ol["H"], g["ltlm_H"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(Ol["Czz"], g["ltlm_C"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(Il, g["ltlm_I"], rtol=1e-12)


def _proj_cases():
    """(N, sectors, fermion, blocks, static) of small sectors, complex momenta
    and fermion signs included."""
    m = chain_maps(8)
    xxz = xxz_static(8)
    hop = [["+-", [[-1.0, i, (i + 1) % 8] for i in range(8)]], ["-+", [[1.0, i, (i + 1) % 8] for i in range(8)]],
           ["nn", [[0.7, i, (i + 1) % 8] for i in range(8)]]]
    cases = []
    for k in (0, 1, 2, 3, 4):
        cases.append((8, [(1, 4, 0)], False, dict(kblock=(m["t"], k)), xxz))
    cases.append((8, [(1, 4, 0)], False, dict(kblock=(m["t"], 0), pblock=(m["p"], 1), zblock=(m["z"], 0)), xxz))
    cases.append((8, [(0, 0, 0)], False, dict(zblock=(m["z"], 1), kblock=(m["t"], 3)), xxz))
    for Nf, k in ((3, 1), (4, 0), (4, 2), (3, 5)):
        cases.append((8, [(1, Nf, 0)], True, dict(kblock=(m["t"], k)), hop))
    return cases


def test_oracle_projector_invariants():
    """P^dagger P = 1 and P^dagger H_full P = H_sector (the reference checks
    projected Hamiltonians this way: test/test_project_op.py,
    test/test_ham_project_to.py), with rows in the full space and in the
    particle-conserving basis."""
    for N, sectors, fermion, blocks, static in _proj_cases():
        ob = O.OracleBasis(N, sectors, fermion=fermion, pauli=0, **blocks)
        H = O.make_static(ob, static, np.complex128)
        full = O.OracleBasis(N, [(0, 0, 0)], fermion=fermion, pauli=0)
        pcon = O.OracleBasis(N, sectors, fermion=fermion, pauli=0)
        for rowb, P in ((full, ob.get_proj(np.complex128)), (pcon, ob.get_proj(np.complex128, pcon_basis=pcon))):
            assert P.shape == (rowb.Ns, ob.Ns)
            Ph = P.conj().T
            np.testing.assert_allclose((Ph @ P).toarray(), np.eye(ob.Ns), atol=1e-14)
            Hf = O.make_static(rowb, static, np.complex128)
            np.testing.assert_allclose((Ph @ Hf @ P).toarray(), H.toarray(), atol=1e-13)


def test_oracle_block_decomposition_of_evolution():
    """The identity block_ops rests on (tools/block_tools.py:618-795 in the
    reference): a state that breaks the translation symmetry evolves as the
    sum over momentum blocks of P_k e^{-itH_k} P_k^dagger psi.  Oracle
    projectors and sector matrices against the full-space evolution."""
    L = 8
    m = chain_maps(L)
    static = [["zz", [[1.0, i, (i + 1) % L] for i in range(L)]], ["x", [[0.7, i] for i in range(L)]]]
    full = O.OracleBasis(L, [(0, 0, 0)], pauli=1)
    Hf = O.make_static(full, static, np.complex128).tocsr()
    rng = np.random.default_rng(5)
    psi = rng.normal(size=2 ** L) + 1j * rng.normal(size=2 ** L)
    psi /= np.linalg.norm(psi)
    ref = expm_multiply(-1.3j * Hf, psi)
    out = np.zeros_like(psi)
    total = 0
    for k in range(L):
        b = O.OracleBasis(L, [(0, 0, 0)], pauli=1, kblock=(m["t"], k))
        P = b.get_proj(np.complex128)
        Hk = O.make_static(b, static, np.complex128).tocsr()
        out += P @ expm_multiply(-1.3j * Hk, P.conj().T @ psi)
        total += b.Ns
    assert total == 2 ** L
    np.testing.assert_allclose(out, ref, atol=1e-12)


def test_oracle_get_amp_matches_projector_entries():
    """get_amp's factor C (psi_s = C psi^sym_r) is the projector entry at row s
    of r's column, in both modes (test/test_get_amp.py checks the same through
    get_vec), complex momenta and fermion signs included."""
    for N, sectors, fermion, blocks, static in _proj_cases():
        ob = O.OracleBasis(N, sectors, fermion=fermion, pauli=0, **blocks)
        if ob.Ns == 0:
            continue
        pcon = O.OracleBasis(N, sectors, fermion=fermion, pauli=0)
        P = ob.get_proj(np.complex128, pcon_basis=pcon).tocsr()
        # representative mode: the representatives' own rows
        C, _ = ob.get_amp(ob.states, mode="representative")
        rows = pcon.index(ob.states)
        np.testing.assert_allclose(C, np.asarray(P[rows, np.arange(ob.Ns)]).ravel(), atol=1e-14)
        # full-basis mode: every state of the particle sector
        C, r = ob.get_amp(pcon.states, mode="full_basis")
        col = ob.index(r)
        inside = col >= 0
        expect = np.zeros(pcon.Ns, np.complex128)
        expect[inside] = np.asarray(P[np.arange(pcon.Ns)[inside], col[inside]]).ravel()
        np.testing.assert_allclose(np.where(inside, C, 0), expect, atol=1e-14)
        assert np.all(np.abs(C[~inside]) == 0)
