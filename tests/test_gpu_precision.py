"""The three arithmetic forms of the Taylor term against the oracle.

"double" (float-pair products, FP64 partial sums), "ieee" (IEEE double
products) and "mixed" (complex64 terms) on the same inputs; the tolerances are
the ones each form states: 1e-12 relative for the two double forms, 1e-5 for
the complex64 form.  Inputs scaled far outside the float range check the
power-of-two storage scale of the float forms."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from tests.models import chain_maps, j1j2_static, xxz_static

pytestmark = pytest.mark.gpu


def _j1j2(L=16):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, kblock=(m["t"], 0), pblock=(m["p"], 0), zblock=(m["z"], 0), pauli=0)
    return hamiltonian(j1j2_static(L), [], basis=b, dtype=np.float64)


def _state(n, seed, k=None):
    rng = np.random.default_rng(seed)
    shape = (n,) if k is None else (n, k)
    v = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    return v / np.linalg.norm(v, axis=0)


def _rel(x, y):
    return np.linalg.norm(x - y) / np.linalg.norm(y)


@pytest.mark.parametrize("a", [-5j, -1j, -0.3])
def test_forms_vs_oracle(cuda, a):
    from quspin_gb300.tools import ExpmMultiplyParallel
    H = _j1j2()
    A = H.tocsr()
    v = _state(A.shape[0], 3)
    np.random.seed(2)
    wo = O.ExpmMultiplyParallelOracle(A, a=a).dot(v)
    errs = {}
    for p in ("double", "ieee", "mixed"):
        np.random.seed(2)
        w = ExpmMultiplyParallel(H.tocsr_gpu(), a=a, precision=p).dot(v)
        errs[p] = _rel(w, wo)
    print("relative state error vs oracle:", errs)
    assert errs["ieee"] <= 1e-12
    assert errs["double"] <= 1e-12
    assert errs["mixed"] <= 1e-5


def test_forms_complex_matrix_and_batch(cuda):
    """Complex Hermitian values (the paired complex operand) and a block of
    right-hand sides (several vectors per row pass)."""
    from quspin_gb300.tools import ExpmMultiplyParallel
    rs = np.random.RandomState(5)
    N = 3000
    A = sp.random(N, N, density=np.log(N) / N, format="csr", random_state=rs) \
        + 1j * sp.random(N, N, density=np.log(N) / N, format="csr", random_state=rs)
    A = sp.csr_matrix((A + A.conj().T) / 2)
    for k in (None, 3, 8):
        V = _state(N, 11, k)
        np.random.seed(4)
        wo = O.ExpmMultiplyParallelOracle(A, a=-0.8j).dot(V)
        for p, tol in (("double", 1e-12), ("ieee", 1e-12), ("mixed", 1e-5)):
            np.random.seed(4)
            w = ExpmMultiplyParallel(A, a=-0.8j, precision=p).dot(V)
            assert _rel(w, wo) <= tol, (p, k, _rel(w, wo))


@pytest.mark.parametrize("scale", [1e-300, 1e-40, 1e40, 1e300])
def test_scaled_inputs(cuda, scale):
    """e^{aA}(c v) = c e^{aA} v for c far outside the float range."""
    from quspin_gb300.tools import ExpmMultiplyParallel
    H = _j1j2(14)
    A = H.tocsr()
    v = _state(A.shape[0], 6)
    np.random.seed(3)
    op = ExpmMultiplyParallel(H.tocsr_gpu(), a=-2j)
    w1 = op.dot(v)
    ws = op.dot(v * scale)
    assert np.all(np.isfinite(ws))
    assert _rel(ws / scale, w1) <= 1e-13
    op.precision = "mixed"
    wm = op.dot(v * scale)
    assert _rel(wm / scale, w1) <= 1e-5


def test_zero_and_single_nonzero(cuda):
    from quspin_gb300.tools import ExpmMultiplyParallel
    H = _j1j2(12)
    A = H.tocsr()
    n = A.shape[0]
    op = ExpmMultiplyParallel(H.tocsr_gpu(), a=-1j)
    assert np.all(op.dot(np.zeros(n, np.complex128)) == 0)
    e = np.zeros(n, np.complex128)
    e[n // 3] = 1.0
    np.random.seed(0)
    wo = O.ExpmMultiplyParallelOracle(A, a=-1j).dot(e)
    assert _rel(op.dot(e), wo) <= 1e-12


def test_multisector_forms(cuda):
    """The stacked-sector kernels in the three forms vs per-sector oracle
    evolutions (two momentum sectors of an XXZ chain, 4 states each)."""
    from quspin_gb300 import hamiltonian, spin_basis_general
    from quspin_gb300.tools import MultiSectorExpm
    L = 12
    m = chain_maps(L)
    mats, hosts = [], []
    for k in (0, 3):
        b = spin_basis_general(L, Nup=L // 2, kblock=(m["t"], k), pauli=0)
        H = hamiltonian(xxz_static(L), [], basis=b, dtype=np.complex128)
        mats.append(H.tocsr_gpu())
        hosts.append(H.tocsr())
    blocks = [_state(A.shape[0], 20 + i, 4) for i, A in enumerate(hosts)]
    for p, tol in (("double", 1e-12), ("ieee", 1e-12), ("mixed", 1e-5)):
        ms = MultiSectorExpm(mats, a=-1.5j, nvec=4, precision=p, graph=False)
        out = ms.evolve(blocks)
        for A, V, W in zip(hosts, blocks, out):
            ref = O.ExpmMultiplyParallelOracle(A, a=-1.5j).dot(V)
            assert _rel(W, ref) <= tol, (p, _rel(W, ref))


def test_chunk_outer_sweep_matches_row_order(cuda):
    """With more than 8 right-hand sides the float forms can sweep the rows
    once per chunk of 8 vectors (row sums carried in a scratch array); the
    result equals the one-sweep order to the stopping tolerance."""
    import torch
    from quspin_gb300 import _lib
    from quspin_gb300.sparse import DeviceCSR
    from quspin_gb300.tune import encode
    from quspin_gb300.tools import ExpmMultiplyParallel
    rng = np.random.default_rng(11)
    N = 70000
    r, c = rng.integers(0, N, 20 * N), rng.integers(0, N, 20 * N)
    A = sp.csr_matrix((rng.uniform(size=20 * N), (r, c)), shape=(N, N))
    A = sp.csr_matrix((A + A.T) * 0.5)
    V = _state(N, 12, 16)
    for prec, bt in (("double", _lib.CPF), ("mixed", _lib.C64)):
        res = []
        for chunk in (0, 1):
            op = ExpmMultiplyParallel(DeviceCSR.from_scipy(A), a=-0.5j, precision=prec)
            M, _ = op._operand(16)
            M.__dict__.setdefault("_tuned", {})[("taylor", 16, bt)] = encode(4, 1) | (chunk << 16)
            F = torch.tensor(V, device="cuda")
            op.run_device(F)
            res.append(F.cpu().numpy())
        assert _rel(res[1], res[0]) <= (1e-13 if prec == "double" else 1e-6), prec
    np.random.seed(1)
    wo = O.ExpmMultiplyParallelOracle(A, a=-0.5j).dot(V)
    assert _rel(res[0], wo) <= 1e-5
