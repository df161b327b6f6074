"""Many sectors in one launch sequence (MultiSectorExpm) vs per-sector
ExpmMultiplyParallel: FP64 form within 1e-12, mixed (complex64 Taylor
blocks) form within the stated 1e-6, for all momentum sectors of a
mixed-field Ising chain (reflection resolved at k = 0 and k = L/2) --
the shape of the L=24 multi-sector configuration, at L=12."""
import numpy as np
import pytest

from tests.models import chain_maps, ising_static

pytestmark = pytest.mark.gpu


def _sectors(L):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(L)
    out = []
    for k in range(L):
        ps = (0, 1) if k in (0, L // 2) else (None,)
        for p in ps:
            blocks = dict(kblock=(m["t"], k))
            if p is not None:
                blocks["pblock"] = (m["p"], p)
            b = spin_basis_general(L, **blocks)
            if b.Ns:
                dt = np.float64 if k in (0, L // 2) else np.complex128
                out.append(hamiltonian(ising_static(L), [], basis=b, dtype=dt).tocsr_gpu())
    return out


@pytest.mark.parametrize("graph", [False, True])
def test_multi_sector_matches_per_sector(cuda, graph):
    from quspin_gb300.tools import ExpmMultiplyParallel, MultiSectorExpm
    mats = _sectors(12)
    assert sum(M.shape[0] for M in mats) == 2 ** 12
    k = 3
    rng = np.random.default_rng(0)
    blocks = []
    for M in mats:
        V = rng.normal(size=(M.shape[0], k)) + 1j * rng.normal(size=(M.shape[0], k))
        blocks.append(V / np.linalg.norm(V, axis=0))
    ms = MultiSectorExpm(mats, a=-2j, nvec=k, graph=graph)
    out = ms.evolve(blocks)
    for M, V, W in zip(mats, blocks, out):
        ref = ExpmMultiplyParallel(M, a=-2j).dot(V)
        assert np.linalg.norm(W - ref) <= 1e-12 * np.linalg.norm(ref)
    # a second evolution reuses the captured sequence
    out2 = ms.evolve(blocks)
    for W, W2 in zip(out, out2):
        np.testing.assert_array_equal(W, W2)


def test_multi_sector_mixed_precision(cuda):
    from quspin_gb300.tools import MultiSectorExpm
    mats = _sectors(12)
    rng = np.random.default_rng(1)
    blocks = [rng.normal(size=(M.shape[0], 2)) + 1j * rng.normal(size=(M.shape[0], 2)) for M in mats]
    blocks = [V / np.linalg.norm(V, axis=0) for V in blocks]
    w64 = MultiSectorExpm(mats, a=-2j, nvec=2).evolve(blocks)
    w32 = MultiSectorExpm(mats, a=-2j, nvec=2, precision="mixed").evolve(blocks)
    num = np.sqrt(sum(np.linalg.norm(a - b) ** 2 for a, b in zip(w32, w64)))
    den = np.sqrt(sum(np.linalg.norm(b) ** 2 for b in w64))
    # complex64 terms with FP32 products and row sums: stated tolerance 5e-6
    assert num / den < 5e-6
