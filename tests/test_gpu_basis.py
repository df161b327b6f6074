"""GPU basis vs the CPU oracle: states, norms, blocks, index, representative
and normalization bit-exact (integer work), over spin chains with
translation / reflection / inversion, a 2-d square lattice and spinful
fermions with translations."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.models import chain_maps, square_maps

pytestmark = pytest.mark.gpu


def _spin_cases():
    cases = []
    for L in (8, 10, 12):
        m = chain_maps(L)
        cases.append((L, L // 2, dict(kblock=(m["t"], 0), pblock=(m["p"], 0))))
        cases.append((L, L // 2, dict(kblock=(m["t"], 0), pblock=(m["p"], 1), zblock=(m["z"], 0))))
        cases.append((L, None, dict(kblock=(m["t"], L // 2), pblock=(m["p"], 0))))
        for k in (1, 3):
            cases.append((L, L // 2, dict(kblock=(m["t"], k))))
            cases.append((L, None, dict(kblock=(m["t"], k), zblock=(m["z"], 1))))
        cases.append((L, L // 2 - 1, {}))
        cases.append((L, None, {}))
    sq = square_maps(4, 4)
    cases.append((16, 8, dict(tx=(sq["tx"], 0), ty=(sq["ty"], 0), px=(sq["px"], 0), z=(sq["z"], 0))))
    cases.append((16, 6, dict(tx=(sq["tx"], 1), ty=(sq["ty"], 2))))
    return cases


@pytest.mark.parametrize("case", range(len(_spin_cases())))
def test_spin_basis_matches_oracle(cuda, case):
    from quspin_gb300 import spin_basis_general
    L, Nup, blocks = _spin_cases()[case]
    b = spin_basis_general(L, Nup=Nup, **blocks)
    ob = O.OracleBasis(L, [(1, Nup, 0)] if Nup is not None else [(0, 0, 0)], **blocks)
    assert b.Ns == ob.Ns
    np.testing.assert_array_equal(b.states.astype(np.uint64), ob.states)
    np.testing.assert_array_equal(b._n.astype(np.uint32), ob.norms)
    assert b._N_p == ob.N_p
    if b._N_p:
        np.testing.assert_array_equal(b._basis_begin, ob.begin)
        np.testing.assert_array_equal(b._basis_end, ob.end)
    rng = np.random.default_rng(case)
    q = rng.integers(0, 2**L, size=500).astype(np.uint64)
    reps_g, g_g, s_g = b.representative(q, return_g=True, return_sign=True)
    reps_o, g_o, s_o = ob.representative(q)
    np.testing.assert_array_equal(reps_g.astype(np.uint64), reps_o)
    np.testing.assert_array_equal(g_g, g_o)
    np.testing.assert_array_equal(s_g, s_o)
    np.testing.assert_array_equal(np.atleast_1d(b.normalization(q)).astype(np.uint32), ob.normalization(q))
    idx = b.index(np.concatenate([b.states[:50], q.astype(b.dtype)]))
    np.testing.assert_array_equal(idx, ob.index(np.concatenate([ob.states[:50], q])))


def test_representative_sorted_unique_equals_states(cuda):
    """test/test_representative.py:118-153: unique representatives of the
    full particle sector with nonzero norm equal the basis states."""
    from quspin_gb300 import spin_basis_general
    sq = square_maps(4, 4)
    blocks = dict(tx=(sq["tx"], 0), ty=(sq["ty"], 0), px=(sq["px"], 0), z=(sq["z"], 0))
    full = spin_basis_general(16, Nup=8)
    b = spin_basis_general(16, Nup=8, **blocks)
    reps = np.unique(b.representative(full.states))[::-1]
    mask = b.normalization(reps) != 0
    np.testing.assert_array_equal(reps[mask], b.states)


@pytest.mark.parametrize("Nf,kx,ky", [((2, 2), 0, 0), ((2, 1), 1, 3), ((3, 2), 2, 0)])
def test_spinful_fermion_basis_matches_oracle(cuda, Nf, kx, ky):
    from quspin_gb300 import spinful_fermion_basis_general
    sq = square_maps(4, 4)
    b = spinful_fermion_basis_general(16, Nf=Nf, kx=(sq["tx"], kx), ky=(sq["ty"], ky))
    tx, _ = O.process_spinful_map(16, sq["tx"], kx)
    ty, _ = O.process_spinful_map(16, sq["ty"], ky)
    ob = O.OracleBasis(32, [(2, Nf[0], Nf[1])], fermion=True, spinful=True, kx=(tx, kx), ky=(ty, ky))
    assert b.Ns == ob.Ns
    np.testing.assert_array_equal(b.states.astype(np.uint64), ob.states)
    np.testing.assert_array_equal(b._n.astype(np.uint32), ob.norms)
    rng = np.random.default_rng(1)
    q = ob.states[rng.integers(0, ob.Ns, 200)]
    q = q ^ np.uint64(0b11)  # nearby words, mostly outside the basis
    rg, gg, sg = b.representative(q, return_g=True, return_sign=True)
    ro, go, so = ob.representative(q)
    np.testing.assert_array_equal(rg.astype(np.uint64), ro)
    np.testing.assert_array_equal(sg, so)


def test_c1_dimension(cuda):
    from quspin_gb300 import spin_basis_general
    m = chain_maps(20)
    b = spin_basis_general(20, Nup=10, kblock=(m["t"], 0), pblock=(m["p"], 0))
    assert b.Ns == 4752
