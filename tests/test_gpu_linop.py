"""Matrix-free quantum_LinearOperator vs hamiltonian (the reference's
test/test_quantum_LinearOperator.py:8-74, atol 1e-10) and inplace_Op vs the
oracle (test/test_inplace_op.py)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.models import chain_maps, xxz_static

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_linop_equals_hamiltonian(cuda, dtype):
    from quspin_gb300 import hamiltonian, quantum_LinearOperator, spin_basis_general
    L = 10
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, pblock=(m["p"], 0), zblock=(m["z"], 0))
    static = xxz_static(L, J=1.0, Delta=0.7)
    H = hamiltonian(static, [], basis=b, dtype=dtype)
    Hop = quantum_LinearOperator(static, basis=b, dtype=dtype)
    rng = np.random.default_rng(0)
    for shape in [(b.Ns,), (b.Ns, 4)]:
        v = rng.normal(size=shape).astype(dtype)
        if np.dtype(dtype).kind == "c":
            v = v + 1j * rng.normal(size=shape)
        np.testing.assert_allclose(Hop.dot(v), H.dot(v), rtol=0, atol=1e-10)
        np.testing.assert_allclose(Hop.dot(v, a=0.3), H.dot(v, a=0.3), rtol=0, atol=1e-10)


def test_inplace_op_vs_oracle(cuda):
    from quspin_gb300 import spin_basis_general
    m = chain_maps(10)
    blocks = dict(kblock=(m["t"], 3))
    b = spin_basis_general(10, Nup=4, **blocks)
    ob = O.OracleBasis(10, [(1, 4, 0)], pauli=1, **blocks)
    rng = np.random.default_rng(1)
    v = rng.normal(size=(b.Ns, 2)) + 1j * rng.normal(size=(b.Ns, 2))
    ops = [["+-", [0, 3], 0.4], ["zz", [1, 2], -0.3], ["xy", [4, 5], 0.2]]
    for tr, cj in [(False, False), (True, False), (False, True), (True, True)]:
        r = b.inplace_Op(v, ops, np.complex128, transposed=tr, conjugated=cj, a=0.5)
        ro = ob.inplace_op(v, ops, np.complex128, transposed=tr, conjugated=cj, a=0.5)
        np.testing.assert_allclose(r, ro, rtol=0, atol=1e-12)
