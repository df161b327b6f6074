"""tools.matvec / get_matvec_function (the reference's
docs/modules/parallel_sparse_tools/matvec/matvec_core.html:105-201): CSR and
DIA operands, real and complex, numpy and CUDA-tensor vectors, one and two
columns, overwrite_out in both modes and the scale a, against scipy at 1e-13
relative."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

pytestmark = pytest.mark.gpu


def _mats(n=3000, seed=0):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=8 / n, format="csr", random_state=np.random.RandomState(seed))
    Ac = A + 1j * sp.random(n, n, density=8 / n, format="csr", random_state=np.random.RandomState(seed + 1))
    D_ = sp.dia_matrix((rng.normal(size=(3, n)), [0, 5, -7]), shape=(n, n))
    return {"csr_real": sp.csr_matrix(A), "csr_complex": sp.csr_matrix(Ac), "dia": D_}


@pytest.mark.parametrize("name", ["csr_real", "csr_complex", "dia"])
@pytest.mark.parametrize("ncol", [1, 2])
def test_matvec_modes_match_scipy(cuda, name, ncol):
    from quspin_gb300.tools.matvec import get_matvec_function, matvec
    A = _mats()[name]
    n = A.shape[0]
    rng = np.random.default_rng(3)
    shape = (n,) if ncol == 1 else (n, ncol)
    v = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    a = 0.7 - 0.2j
    ref = a * (A @ v)
    tol = lambda x: 1e-13 * np.abs(x).max()
    # overwrite: out = a A v (numpy in, numpy out)
    out = np.full(shape, 5.0 + 1j)
    res = matvec(A, v, overwrite_out=True, out=out, a=a)
    assert res is out and np.abs(out - ref).max() <= tol(ref)
    # accumulate: out += a A v
    out = np.full(shape, 5.0 + 1j)
    matvec(A, v, overwrite_out=False, out=out, a=a)
    assert np.abs(out - (5.0 + 1j + ref)).max() <= tol(ref)
    # no out: a new array
    assert np.abs(matvec(A, v, a=a) - ref).max() <= tol(ref)
    # the routine returned by get_matvec_function, device operands
    f = get_matvec_function(A)
    vd = torch.tensor(v, device="cuda")
    od = torch.zeros(shape, dtype=torch.complex128, device="cuda") + 2.0
    f(A, vd, overwrite_out=False, out=od, a=a)
    assert np.abs(od.cpu().numpy() - (2.0 + ref)).max() <= tol(ref)
    od = f(A, vd, a=a)
    assert torch.is_tensor(od) and np.abs(od.cpu().numpy() - ref).max() <= tol(ref)
