"""Projector to the full basis (basis.get_proj / project_from / project_to)
and the symmetry-block evolution tools (block_ops, block_diag_hamiltonian)
on the GPU, against the oracle and against evolution in the full space."""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.integrate import solve_ivp
from scipy.sparse.linalg import expm_multiply

from oracle import oracle as O
from tests.models import chain_maps, xxz_static

pytestmark = pytest.mark.gpu

qs = pytest.importorskip("quspin_gb300")
from quspin_gb300.basis import (spin_basis_1d, spin_basis_general, spinful_fermion_basis_general,  # noqa: E402
                                spinless_fermion_basis_general)
from quspin_gb300.operators import hamiltonian  # noqa: E402
from quspin_gb300.tools import block_diag_hamiltonian, block_ops  # noqa: E402


def _hop(L):
    return [["+-", [[-1.0, i, (i + 1) % L] for i in range(L)]], ["-+", [[1.0, i, (i + 1) % L] for i in range(L)]],
            ["nn", [[0.7, i, (i + 1) % L] for i in range(L)]]]


def _cases():
    m = chain_maps(8)
    out = []
    for k in (0, 1, 2, 3, 4):
        out.append(("spin", 4, dict(kblock=(m["t"], k))))
    out.append(("spin", 4, dict(kblock=(m["t"], 0), pblock=(m["p"], 1), zblock=(m["z"], 0))))
    out.append(("spin", None, dict(zblock=(m["z"], 1), kblock=(m["t"], 3))))
    for Nf, k in ((3, 1), (4, 0), (4, 2), (3, 5)):
        out.append(("fermion", Nf, dict(kblock=(m["t"], k))))
    return out


def _pair(kind, Np, blocks):
    if kind == "spin":
        gb = spin_basis_general(8, Nup=Np, pauli=0, **blocks)
        ob = O.OracleBasis(8, [(1, Np, 0)] if Np is not None else [(0, 0, 0)], pauli=0, **blocks)
        pb = O.OracleBasis(8, [(1, Np, 0)] if Np is not None else [(0, 0, 0)], pauli=0)
    else:
        gb = spinless_fermion_basis_general(8, Nf=Np, **blocks)
        ob = O.OracleBasis(8, [(1, Np, 0)], fermion=True, **blocks)
        pb = O.OracleBasis(8, [(1, Np, 0)], fermion=True)
    return gb, ob, pb


def _same(P, Q, tol=1e-14):
    P, Q = sp.csc_matrix(P), sp.csc_matrix(Q)
    P.sort_indices()
    Q.sort_indices()
    assert P.shape == Q.shape
    np.testing.assert_array_equal(P.indptr, Q.indptr)
    np.testing.assert_array_equal(P.indices, Q.indices)
    np.testing.assert_allclose(P.data, Q.data, rtol=0, atol=tol)


def test_get_proj_matches_oracle():
    """Rows in the full space and in the particle sector, complex momenta and
    fermion signs: structure exact, values within 1e-14."""
    for kind, Np, blocks in _cases():
        gb, ob, pb = _pair(kind, Np, blocks)
        _same(gb.get_proj(np.complex128), ob.get_proj(np.complex128))
        if Np is not None:
            _same(gb.get_proj(np.complex128, pcon=True), ob.get_proj(np.complex128, pcon_basis=pb))


def test_get_proj_spinful_matches_oracle():
    t = (np.arange(4) + 1) % 4
    for k in (0, 1, 2):
        gb = spinful_fermion_basis_general(4, Nf=(2, 1), kblock=(t, k))
        ob = O.OracleBasis(8, [(2, 2, 1)], fermion=True, spinful=True, kblock=O.process_spinful_map(4, t, k))
        pb = O.OracleBasis(8, [(2, 2, 1)], fermion=True, spinful=True)
        _same(gb.get_proj(np.complex128), ob.get_proj(np.complex128))
        _same(gb.get_proj(np.complex128, pcon=True), ob.get_proj(np.complex128, pcon_basis=pb))


def test_get_proj_noncommuting_maps_matches_oracle():
    """Reflection with a translation at k != 0, pi (maps that do not commute,
    as in the reference's test/test_project_to.py list): coset phases differ
    and summed images can cancel."""
    L = 10
    m = chain_maps(L)
    for q in (1, 3, L - 1):
        for Nup in (None, 4):
            blocks = dict(zb=(m["z"], 0), pb=(m["p"], 0), tb=(m["t"], q))
            if Nup is not None:
                blocks.pop("zb")
            gb = spin_basis_general(L, Nup=Nup, **blocks)
            ob = O.OracleBasis(L, [(1, Nup, 0)] if Nup is not None else [(0, 0, 0)], pauli=1, **blocks)
            if gb.Ns == 0:
                continue
            _same(gb.get_proj(np.complex128), ob.get_proj(np.complex128))


def test_get_amp_matches_oracle():
    """basis.get_amp in both modes against the oracle's restatement (whose
    factors equal the oracle projector's entries, tests/test_cpu_oracle.py)."""
    for kind, Np, blocks in _cases():
        gb, ob, pb = _pair(kind, Np, blocks)
        if gb.Ns == 0:
            continue
        C = gb.get_amp(gb.states.copy(), mode="representative")
        Co, _ = ob.get_amp(ob.states, mode="representative")
        np.testing.assert_allclose(np.atleast_1d(C), Co, rtol=0, atol=1e-15)
        full = pb.states.astype(gb.dtype)
        st = full.copy()
        C = gb.get_amp(st, mode="full_basis")
        Co, ro = ob.get_amp(pb.states, mode="full_basis")
        np.testing.assert_allclose(np.atleast_1d(C), Co, rtol=0, atol=1e-15)
        np.testing.assert_array_equal(st, ro.astype(gb.dtype))       # states replaced by representatives


def test_get_amp_round_trip():
    """test/test_get_amp.py on a 4x4 lattice sector: representative-mode
    factors turn symmetric amplitudes into the full-basis amplitudes that
    project_from gives; full-basis mode turns them back."""
    Lx = Ly = 4
    N = Lx * Ly
    s_ = np.arange(N)
    x, y = s_ % Lx, s_ // Lx
    tx, ty, z = (x + 1) % Lx + Lx * y, x + Lx * ((y + 1) % Ly), -(s_ + 1)
    for kx, ky in ((0, 0), (1, 0), (1, 2)):
        b = spin_basis_general(N, pauli=0, Nup=N // 2, kxblock=(tx, kx), kyblock=(ty, ky), zblock=(z, 0))
        bf = spin_basis_general(N, pauli=0, Nup=N // 2)
        rng = np.random.default_rng(kx + 10 * ky)
        v = rng.normal(size=b.Ns) + 1j * rng.normal(size=b.Ns)
        v /= np.linalg.norm(v)
        inds = bf.index(b.states)
        psi = v.copy()
        b.get_amp(b.states.copy(), amps=psi, mode="representative")
        full = b.project_from(v, pcon=True, sparse=False)
        np.testing.assert_allclose(psi, full[inds], atol=1e-14)
        states_full = bf.states.copy()
        amps = full.copy()
        with np.errstate(divide="ignore", invalid="ignore"):      # states outside the sector have C = 0
            b.get_amp(states_full, amps=amps, mode="full_basis")
        np.testing.assert_array_equal(states_full, b.representative(bf.states))
        np.testing.assert_allclose(amps[inds], v, atol=1e-13)


def test_project_to_from_match_projector():
    """test/test_project_to.py: P v == project_from(v) and P^dagger v_full ==
    project_to(v_full) for the reference's list of L=12 bases."""
    L = 12
    z = -(np.arange(L) + 1)
    p = np.arange(L)[::-1]
    t = (np.arange(L) + 1) % L
    bases = [
        spin_basis_general(L), spin_basis_general(L, Nup=L // 2),
        spin_basis_general(L, zb=(z, 0)), spin_basis_general(L, zb=(z, 1)),
        spin_basis_general(L, pb=(p, 0)), spin_basis_general(L, pb=(p, 1)),
        spin_basis_general(L, zb=(z, 0), pb=(p, 0)), spin_basis_general(L, zb=(z, 1), pb=(p, 1)),
        spin_basis_general(L, zb=(z, 0), pb=(t, 1)), spin_basis_general(L, zb=(z, 1), pb=(t, 0)),
        spin_basis_general(L, zb=(z, 0), pb=(p, 0), tb=(t, L - 1)),
        spin_basis_general(L, zb=(z, 1), pb=(p, 1), tb=(t, 0)),
        spin_basis_general(L, Nup=L // 2, pb=(p, 0), tb=(t, 0)),
        spin_basis_general(L, Nup=2, pb=(p, 0), tb=(t, L - 1)),
        spin_basis_general(L, Nup=1, pb=(p, 0), tb=(t, L - 2)),
        spin_basis_general(L, Nup=L // 2, pb=(p, 1), tb=(t, L - 1)),
    ]
    rng = np.random.default_rng(0)
    for b in bases:
        P = b.get_proj(np.complex128)
        Ns_full, Ns = P.shape
        assert Ns_full == 2 ** L and Ns == b.Ns
        v = rng.normal(size=Ns).astype(np.complex128)
        v /= np.linalg.norm(v)
        vf = rng.normal(size=Ns_full).astype(np.complex128)
        vf /= np.linalg.norm(vf)
        np.testing.assert_allclose(P.dot(v), b.project_from(v, sparse=False), atol=1e-10)
        np.testing.assert_allclose(P.conj().T.dot(vf), b.project_to(vf, sparse=False), atol=1e-10)
        np.testing.assert_allclose(b.project_from(v, sparse=True).toarray().ravel(), P.dot(v), atol=1e-14)
        V = rng.normal(size=(Ns, 3)) + 1j * rng.normal(size=(Ns, 3))
        np.testing.assert_allclose(b.project_from(V, sparse=False), P.dot(V), atol=1e-10)
        np.testing.assert_allclose(b.get_vec(V, sparse=False), P.dot(V), atol=1e-10)


def test_1d_and_general_projectors_agree():
    """test/test_general_spin_get_vec.py (spin-1/2, L=4)."""
    L = 4
    t = np.array([(i + 1) % L for i in range(L)])
    p = np.array([L - i - 1 for i in range(L)])
    z = np.array([-(i + 1) for i in range(L)])
    for Nup in (None, 2):
        for kblock in (None, 0, 1, 2, 3):
            for pblock in (None, 0, 1):
                for zblock in (None, 0, 1):
                    kw1, kw2 = {}, {}
                    dtype = np.complex128
                    if kblock in (0, 2) and pblock is not None:
                        dtype = np.float64
                        kw1["pblock"] = (-1) ** pblock
                        kw2["pblock"] = (p, pblock)
                    if zblock is not None:
                        kw1["zblock"] = (-1) ** zblock
                        kw2["zblock"] = (z, zblock)
                    if kblock is not None:
                        kw1["kblock"] = kblock
                        kw2["kblock"] = (t, kblock)
                    b1 = spin_basis_1d(L, Nup=Nup, pauli=0, **kw1)
                    b2 = spin_basis_general(L, Nup=Nup, pauli=0, **kw2)
                    if b1.Ns == 0:
                        continue
                    np.testing.assert_allclose((b1.get_proj(dtype) - b2.get_proj(dtype)).data, 0, atol=1e-14)
                    if Nup is not None:
                        np.testing.assert_allclose((b1.get_proj(dtype, pcon=True) - b2.get_proj(dtype, pcon=True)).data,
                                                   0, atol=1e-14)


def test_projection_identities_c1_sector():
    """L=20, Sz=0, k=0, p=+1 (4,752 states) against the Sz=0 sector (184,756
    states): project_to(project_from(v)) = v and P^dagger H_pcon P v =
    H_sector v."""
    L = 20
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, pauli=0, kblock=(m["t"], 0), pblock=(m["p"], 0))
    bp = spin_basis_general(L, Nup=L // 2, pauli=0)
    assert b.Ns == 4752
    rng = np.random.default_rng(1)
    v = rng.normal(size=b.Ns) + 1j * rng.normal(size=b.Ns)
    vf = b.project_from(v, sparse=False, pcon=True)
    assert vf.shape == (bp.Ns,)
    np.testing.assert_allclose(b.project_to(vf, sparse=False, pcon=True), v, atol=1e-12)
    H = hamiltonian(xxz_static(L), [], basis=b, dtype=np.float64)
    Hp = hamiltonian(xxz_static(L), [], basis=bp, dtype=np.float64)
    lhs = b.project_to(Hp.dot(vf), sparse=False, pcon=True)
    np.testing.assert_allclose(lhs, H.dot(v), atol=1e-11)


# ---------------------------------------------------------------------------
# block tools (test/test_block_tools.py, made exact: the reference's test is
# marked xfail)


def _drive(t, w):
    return np.sin(w * t) * t


def _ising_model(L):
    J = [[1.0, i, (i + 1) % L] for i in range(L)]
    h = [[1.0, i] for i in range(L)]
    return [["zz", J]], [["x", h, _drive, [1.3]]]


def test_block_diag_hamiltonian_spectrum():
    L = 8
    J = [[1.0, i, (i + 1) % L] for i in range(L)]
    h = [[1.0, i] for i in range(L)]
    static = [["xx", J], ["yy", J], ["zz", J]]
    dynamic = [["z", h, np.sin, ()]]
    blocks = [{"Nup": Nup} for Nup in range(L + 1)]
    P, Hb = block_diag_hamiltonian(blocks, static, dynamic, spin_basis_1d, (L,), np.float64)
    H = hamiltonian(static, dynamic, N=L, dtype=np.float64)
    for t in np.linspace(0, 2 * np.pi, 5):
        np.testing.assert_allclose(np.linalg.eigvalsh(Hb.toarray(time=t)), np.linalg.eigvalsh(H.toarray(time=t)),
                                   atol=1e-12)
        Hf = H.tocsr(time=t)
        np.testing.assert_allclose((P.T.conj() @ Hf @ P).toarray(), Hb.toarray(time=t), atol=1e-13)


def test_block_ops_expm_matches_full_space():
    L = 8
    static, dynamic = _ising_model(L)
    blocks = [{"kblock": k} for k in range(L)]
    bo = block_ops(blocks, static, dynamic, spin_basis_1d, (L,), np.complex128, compute_all_blocks=True)
    assert len(bo.P_dict) == L and len(bo.H_dict) == L
    H = hamiltonian(static, dynamic, N=L, dtype=np.complex128)
    rng = np.random.default_rng(2)
    psi0 = rng.random(2 ** L)
    psi0 /= np.linalg.norm(psi0)
    Ht = H.tocsr(time=0.3)
    start, stop, num = 0.0, 4.0, 6
    exact = expm_multiply(-1j * Ht, psi0, start=start, stop=stop, num=num, endpoint=True)
    got = bo.expm(psi0, H_time_eval=0.3, start=start, stop=stop, num=num, endpoint=True)
    assert got.shape == (2 ** L, num)
    np.testing.assert_allclose(got.T, exact, atol=1e-10)
    for g, e in zip(bo.expm(psi0, H_time_eval=0.3, start=start, stop=stop, num=num, endpoint=True, iterate=True),
                    exact):
        np.testing.assert_allclose(g, e, atol=1e-10)
    np.testing.assert_allclose(bo.expm(psi0, H_time_eval=0.3), expm_multiply(-1j * Ht, psi0), atol=1e-10)
    # imaginary time with a shift
    E0 = np.linalg.eigvalsh(Ht.toarray())[0]
    exact = expm_multiply(-(Ht - E0 * sp.identity(2 ** L)), psi0, start=0.5, stop=3.0, num=4, endpoint=True)
    got = bo.expm(psi0, H_time_eval=0.3, a=-1, shift=-E0, start=0.5, stop=3.0, num=4, endpoint=True)
    np.testing.assert_allclose(got.T, exact, atol=1e-9 * np.abs(exact).max())


def test_block_ops_evolve_matches_full_space():
    L = 8
    static, dynamic = _ising_model(L)
    blocks = [{"kblock": k} for k in range(L)]
    bo = block_ops(blocks, static, dynamic, spin_basis_1d, (L,), np.complex128)
    H = hamiltonian(static, dynamic, N=L, dtype=np.complex128)
    H0 = H.static.tocsr()
    Hd = list(H.dynamic.values())[0].tocsr()
    rng = np.random.default_rng(3)
    psi0 = rng.random(2 ** L) + 0j
    psi0 /= np.linalg.norm(psi0)
    times = np.linspace(0, 3.0, 5)
    ref = solve_ivp(lambda t, y: -1j * (H0 @ y + _drive(t, 1.3) * (Hd @ y)), (0, 3.0), psi0, method="DOP853",
                    t_eval=times, rtol=1e-12, atol=1e-12).y
    got = bo.evolve(psi0, 0.0, times, atol=1e-12, rtol=1e-12)
    assert got.shape == (2 ** L, len(times))
    np.testing.assert_allclose(got, ref, atol=1e-8)
    for g, r in zip(bo.evolve(psi0, 0.0, times, iterate=True, atol=1e-12, rtol=1e-12), ref.T):
        np.testing.assert_allclose(g, r, atol=1e-8)
    with pytest.raises(ValueError):
        bo.evolve(psi0, 0.0, times, imag_time=True)


def test_block_ops_no_projection_raises():
    L = 6
    static, dynamic = _ising_model(L)
    bo = block_ops([{"kblock": 0, "Nup": 0}], static, [], spin_basis_1d, (L,), np.complex128,
                   check_pcon=False, check_symm=False)
    psi0 = np.zeros(2 ** L)
    psi0[5] = 1.0      # a state with two up spins: no weight in Nup=0
    with pytest.raises(RuntimeError):
        bo.expm(psi0)
