"""Benchmark-size checks through size-independent properties: sector
dimensions (Burnside counts), Hermitian structure of the CSR, norm
conservation and the group property of e^{-iHt}, the sector sum of the
many-sector workload, and the fermion basis against the oracle at full size."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.models import chain_maps, j1j2_static, square_maps

pytestmark = pytest.mark.gpu


def test_j1j2_L32_sector_and_evolution_properties(cuda):
    from quspin_gb300 import hamiltonian, spin_basis_general
    from quspin_gb300.tools import ExpmMultiplyParallel
    m = chain_maps(32)
    b = spin_basis_general(32, Nup=16, pauli=0, kblock=(m["t"], 0), pblock=(m["p"], 0), zblock=(m["z"], 0))
    assert b.Ns == 4707969
    H = hamiltonian(j1j2_static(32), [], basis=b, dtype=np.float64)
    A = H.tocsr_gpu()
    AT = A.conj_transpose()
    assert torch.equal(A.indptr, AT.indptr) and torch.equal(A.indices, AT.indices)
    rel = float((A.data - AT.data).abs().max() / A.data.abs().max())
    assert rel < 1e-15
    g = torch.Generator(device="cpu").manual_seed(0)
    v = torch.randn(b.Ns, dtype=torch.complex128, generator=g).to("cuda")
    v /= torch.linalg.vector_norm(v)
    w_full = ExpmMultiplyParallel(A, a=-2.0j).dot(v)
    half = ExpmMultiplyParallel(A, a=-1.0j)
    w_half = half.dot(half.dot(v))
    assert abs(float(torch.linalg.vector_norm(w_full)) - 1.0) < 1e-12
    assert float(torch.linalg.vector_norm(w_full - w_half)) < 1e-11


def test_ising_L24_sectors_sum_to_full_space(cuda):
    from quspin_gb300 import spin_basis_general
    m = chain_maps(24)
    tot = 0
    for k in range(24):
        for p in ((0, 1) if k in (0, 12) else (None,)):
            blocks = dict(kblock=(m["t"], k))
            if p is not None:
                blocks["pblock"] = (m["p"], p)
            tot += spin_basis_general(24, make_basis=True, **blocks).Ns
    assert tot == 2 ** 24


def test_driven_L26_dimension(cuda):
    from quspin_gb300 import spin_basis_general
    m = chain_maps(26)
    assert spin_basis_general(26, kblock=(m["t"], 0), pblock=(m["p"], 0)).Ns == 1296858


def test_hubbard_4x4_Nf55_k00_basis_matches_oracle(cuda):
    from quspin_gb300 import spinful_fermion_basis_general
    sq = square_maps(4, 4)
    b = spinful_fermion_basis_general(16, Nf=(5, 5), kx=(sq["tx"], 0), ky=(sq["ty"], 0))
    tx, _ = O.process_spinful_map(16, sq["tx"], 0)
    ty, _ = O.process_spinful_map(16, sq["ty"], 0)
    ob = O.OracleBasis(32, [(2, 5, 5)], fermion=True, spinful=True, kx=(tx, 0), ky=(ty, 0))
    assert b.Ns == ob.Ns
    np.testing.assert_array_equal(b.states.astype(np.uint64), ob.states)
    np.testing.assert_array_equal(b._n.astype(np.uint32), ob.norms)
