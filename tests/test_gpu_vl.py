"""The many-vector Taylor term with the vectors across the lanes
(csrc/expm_vl.cu, launch shapes 1..3 with k > 1 vectors): whole evolutions of
k = 3, 8 and 12 vectors (a partly filled lane group; two sweeps of a row) for
one matrix, real and complex values, against the row hand-out kernel of
csrc/expm_lp.cu and scipy, and for a stack of sectors (MultiSectorExpm)
against per-sector evolutions: the float-pair form within 1e-12; the complex64
form no further from the float-pair result than the row hand-out kernel in
the same form (FP32 products), and within 1e-5."""
import numpy as np
import pytest

from tests.models import chain_maps, ising_static

pytestmark = pytest.mark.gpu


def _sector(L, k, p=None, dtype=np.complex128):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(L)
    blocks = dict(kblock=(m["t"], k))
    if p is not None:
        blocks["pblock"] = (m["p"], p)
    b = spin_basis_general(L, **blocks)
    return hamiltonian(ising_static(L), [], basis=b, dtype=dtype).tocsr_gpu()


def _evolve(M, V, code, precision="double"):
    from quspin_gb300 import _lib
    from quspin_gb300 import _device as D
    from quspin_gb300.tools import ExpmMultiplyParallel
    op = ExpmMultiplyParallel(M, a=-1.5j, precision=precision)
    k = V.shape[1]
    P, bt = op._operand(k)
    P.__dict__.setdefault("_tuned", {})[("taylor", k, bt)] = code
    return D.to_host(op.dot(D.to_device(V)))


@pytest.mark.parametrize("k", [3, 8, 12])
@pytest.mark.parametrize("kind", ["real", "complex"])
def test_vl_evolution_matches_row_handout(cuda, k, kind):
    from scipy.sparse.linalg import expm_multiply
    from quspin_gb300.tune import encode
    M = _sector(14, 0, 0, np.float64) if kind == "real" else _sector(14, 3)
    n = M.shape[0]
    rng = np.random.default_rng(k)
    V = rng.normal(size=(n, k)) + 1j * rng.normal(size=(n, k))
    V /= np.linalg.norm(V, axis=0)
    ref_lp = _evolve(M, V, encode(4, 1))
    ref = expm_multiply(-1.5j * M.tocsr(), V)
    assert np.linalg.norm(ref_lp - ref) <= 1e-12 * np.linalg.norm(ref)
    for shape in (1, 2, 3):
        W = _evolve(M, V, encode(2, 2) | (shape << 20))
        assert np.linalg.norm(W - ref_lp) <= 1e-12 * np.linalg.norm(ref_lp), shape
    # complex64 form: FP32 products, so compare its error with the row
    # hand-out kernel's error in the same form
    e_lp = np.linalg.norm(_evolve(M, V, encode(4, 1), precision="mixed") - ref_lp)
    e_vl = np.linalg.norm(_evolve(M, V, encode(2, 2) | (1 << 20), precision="mixed") - ref_lp)
    assert e_vl <= 2.0 * e_lp + 1e-7 * np.linalg.norm(ref_lp)
    assert e_vl <= 1e-5 * np.linalg.norm(ref_lp)


def test_vl_multi_sector(cuda):
    from quspin_gb300.tools import ExpmMultiplyParallel, MultiSectorExpm
    from quspin_gb300.tune import encode
    L = 12
    mats = []
    for kk in range(L):
        for p in ((0, 1) if kk in (0, L // 2) else (None,)):
            mats.append(_sector(L, kk, p, np.float64 if kk in (0, L // 2) else np.complex128))
    k = 5
    rng = np.random.default_rng(2)
    blocks = []
    for M in mats:
        V = rng.normal(size=(M.shape[0], k)) + 1j * rng.normal(size=(M.shape[0], k))
        blocks.append(V / np.linalg.norm(V, axis=0))
    for shape in (1, 3):
        ms = MultiSectorExpm(mats, a=-2j, nvec=k, graph=False)
        ms._group = encode(2, 2) | (shape << 20)
        out = ms.evolve(blocks)
        for M, V, W in zip(mats, blocks, out):
            ref = ExpmMultiplyParallel(M, a=-2j).dot(V)
            assert np.linalg.norm(W - ref) <= 1e-12 * np.linalg.norm(ref), shape
    out32 = {}
    for name, code in (("lp", 0), ("vl", encode(2, 2) | (1 << 20))):
        ms = MultiSectorExpm(mats, a=-2j, nvec=k, graph=False, precision="mixed")
        ms._group = code
        out32[name] = ms.evolve(blocks)
    for M, V, Wl, Wv in zip(mats, blocks, out32["lp"], out32["vl"]):
        ref = ExpmMultiplyParallel(M, a=-2j).dot(V)
        e_lp, e_vl = np.linalg.norm(Wl - ref), np.linalg.norm(Wv - ref)
        assert e_vl <= 2.0 * e_lp + 1e-7 * np.linalg.norm(ref)
        assert e_vl <= 1e-5 * np.linalg.norm(ref)
