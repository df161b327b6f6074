"""The CSR product in its three arithmetic forms against scipy: float-pair
products for float64 / complex128 vectors (the default), IEEE double
products, and FP32 products for float32 / complex64 vectors; the _matvec
contract (y = a A x or y += a A x, matvec_core.html:146-201) for real and
complex matrices, one or several right-hand sides and extreme input scales."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def _mat(n, cplx, seed):
    rng = np.random.default_rng(seed)
    nnz = 30 * n
    r, c = rng.integers(0, n, nnz), rng.integers(0, n, nnz)
    v = rng.normal(size=nnz) + (1j * rng.normal(size=nnz) if cplx else 0)
    return sp.csr_matrix((v, (r, c)), shape=(n, n))


def _rel(x, y):
    return np.linalg.norm(x - y) / np.linalg.norm(y)


@pytest.mark.parametrize("cplx_A", [False, True])
@pytest.mark.parametrize("cplx_x", [False, True])
@pytest.mark.parametrize("k", [None, 3, 8])
def test_pair_and_ieee_forms(cuda, cplx_A, cplx_x, k):
    import torch
    from quspin_gb300 import _device as D
    from quspin_gb300.sparse import DeviceCSR
    n = 70000
    A = _mat(n, cplx_A, 1)
    M = DeviceCSR.from_scipy(A)
    rng = np.random.default_rng(2)
    shape = (n,) if k is None else (n, k)
    x = rng.normal(size=shape) + (1j * rng.normal(size=shape) if cplx_x else 0)
    dt = np.complex128 if (cplx_A or cplx_x) else np.float64
    a = 0.7 - 0.2j if dt == np.complex128 else 0.7
    ref = a * (A @ x)
    xd = D.to_device(x, dt)
    y0 = D.to_device(rng.normal(size=shape), dt)
    for prec in ("double", "ieee"):
        y = torch.empty_like(xd)
        M.matvec_into(xd, y, a=a, overwrite=True, precision=prec)
        assert _rel(D.to_host(y), ref) <= 1e-13, prec
        yacc = y0.clone()
        M.matvec_into(xd, yacc, a=a, overwrite=False, precision=prec)
        assert _rel(D.to_host(yacc), D.to_host(y0) + ref) <= 1e-13, prec


@pytest.mark.parametrize("scale", [1e-300, 1e-45, 1e45, 1e300])
def test_pair_form_scaled_inputs(cuda, scale):
    import torch
    from quspin_gb300 import _device as D
    from quspin_gb300.sparse import DeviceCSR
    n = 20000
    A = _mat(n, True, 3) * 0.5
    M = DeviceCSR.from_scipy(A)
    rng = np.random.default_rng(4)
    x1 = rng.normal(size=n) + 1j * rng.normal(size=n)
    xd = D.to_device(x1 * scale, np.complex128)
    y = torch.empty_like(xd)
    M.matvec_into(xd, y, precision="double")
    yh = D.to_host(y)
    assert np.all(np.isfinite(yh))
    # compare at unit scale (norms of the scaled vectors over/underflow)
    assert _rel(yh / scale, A @ x1) <= 1e-13


@pytest.mark.parametrize("cplx", [False, True])
def test_single_precision_form(cuda, cplx):
    import torch
    from quspin_gb300 import _device as D
    from quspin_gb300.sparse import DeviceCSR
    n = 50000
    A = _mat(n, cplx, 5)
    M = DeviceCSR.from_scipy(A).astype(np.complex64 if cplx else np.float32)
    rng = np.random.default_rng(6)
    x = rng.normal(size=(n, 4)) + 1j * rng.normal(size=(n, 4))
    xd = D.to_device(x, np.complex64)
    y = torch.empty_like(xd)
    M.matvec_into(xd, y, a=1.5)
    assert y.dtype == torch.complex64
    assert _rel(D.to_host(y), 1.5 * (A @ x)) <= 2e-6


def test_hamiltonian_dot_default_form(cuda):
    """hamiltonian.dot through the default (float-pair) product agrees with
    the IEEE product to 1e-13."""
    from quspin_gb300 import hamiltonian, spin_basis_general
    from quspin_gb300.sparse import set_spmv_precision
    from tests.models import chain_maps, j1j2_static
    L = 20
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, kblock=(m["t"], 0), pblock=(m["p"], 0), zblock=(m["z"], 0), pauli=0)
    H = hamiltonian(j1j2_static(L), [], basis=b, dtype=np.float64)
    rng = np.random.default_rng(7)
    v = rng.normal(size=H.Ns) + 1j * rng.normal(size=H.Ns)
    w = H.dot(v)
    old = set_spmv_precision("ieee")
    try:
        wi = H.dot(v)
    finally:
        set_spmv_precision(old)
    assert _rel(w, wi) <= 1e-13
    assert _rel(w, H.tocsr() @ v) <= 1e-13


def test_int64_indptr_paths_match_int32(cuda):
    """Matrices past 2^31 nonzeros carry an int64 indptr (src/quspin/basis/
    base.py:7-11 picks the index dtype by size); the int64 kernels give the
    same bits as the int32 ones on a small matrix stored both ways."""
    import torch
    from quspin_gb300 import _device as D
    from quspin_gb300.sparse import DeviceCSR
    from quspin_gb300.tools import ExpmMultiplyParallel
    n = 40000
    A = _mat(n, True, 9)
    A = sp.csr_matrix((A + A.conj().T) * 0.05)
    M32 = DeviceCSR.from_scipy(A)
    M64 = DeviceCSR(M32.indptr.to(torch.int64), M32.indices, M32.data, M32.shape, M32.dtype)
    assert M64.idx64 == 1 and M32.idx64 == 0
    rng = np.random.default_rng(10)
    x = D.to_device(rng.normal(size=n) + 1j * rng.normal(size=n), np.complex128)
    for prec in ("double", "ieee"):
        y32, y64 = torch.empty_like(x), torch.empty_like(x)
        M32.matvec_into(x, y32, precision=prec, group=0)
        M64.matvec_into(x, y64, precision=prec, group=0)
        assert torch.equal(y32, y64), prec
    for prec in ("double", "ieee", "mixed"):
        np.random.seed(0)
        w32 = ExpmMultiplyParallel(M32, a=-0.6j, precision=prec)
        np.random.seed(0)
        w64 = ExpmMultiplyParallel(M64, a=-0.6j, precision=prec)
        w64.set_partition(w32.m_star, w32.s)
        F32, F64 = x.clone(), x.clone()
        w32.run_device(F32)
        w64.run_device(F64)
        assert torch.linalg.vector_norm(F32 - F64) <= 1e-14 * torch.linalg.vector_norm(F32), prec


def test_empty_and_tiny_operators(cuda):
    """n = 0 and n = 1 operators through the product and the exponential."""
    import torch
    from quspin_gb300.sparse import DeviceCSR
    from quspin_gb300.tools import ExpmMultiplyParallel
    A1 = sp.csr_matrix(np.array([[2.0]]))
    w = ExpmMultiplyParallel(A1, a=-1j).dot(np.array([1.0 + 0j]))
    assert abs(w[0] - np.exp(-2j)) < 1e-14
    A0 = sp.csr_matrix((0, 0))
    M0 = DeviceCSR.from_scipy(A0)
    x0 = torch.zeros(0, dtype=torch.complex128, device="cuda")
    y0 = torch.empty_like(x0)
    M0.matvec_into(x0, y0)
    assert ExpmMultiplyParallel(A0, a=-1j).dot(np.zeros(0, np.complex128)).shape == (0,)


def test_coded_values_bit_identical(cuda):
    """Matrices with at most 256 distinct values keep one code byte per
    nonzero into a table of float pairs (also packed into the column words):
    products and whole evolutions are bit-identical to the
    one-pair-per-nonzero operand."""
    import torch
    from quspin_gb300 import hamiltonian, spin_basis_general
    from tests.models import chain_maps, xxz_static
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    from quspin_gb300.sparse import PairedCSR
    from quspin_gb300.tools import ExpmMultiplyParallel
    L = 20
    m = chain_maps(L)
    cases = [(spin_basis_general(L, Nup=L // 2, pauli=0, kblock=(m["t"], 0), pblock=(m["p"], 0)), np.float64),
             (spin_basis_general(L, Nup=L // 2, pauli=0, kblock=(m["t"], 3)), np.complex128)]
    rng = np.random.default_rng(7)
    for b, dt in cases:
        H = hamiltonian(xxz_static(L), [], basis=b, dtype=dt)
        A = H.tocsr_gpu()
        P1, P2 = PairedCSR(A, coded=True), PairedCSR(A, coded=False)
        assert P1.coded and not P2.coded and P1.distinct <= 256
        n = A.shape[0]
        x = D.to_device(rng.normal(size=(n, 3)) + 1j * rng.normal(size=(n, 3)))
        P3 = P1.packed()
        assert P3.vcode == (_lib.CPF8P if dt == np.complex128 else _lib.PF8P)
        xr = D.to_device(rng.normal(size=n))
        xs = torch.empty(2 * x.numel() * 2, dtype=torch.float32, device=x.device)
        nrm = torch.zeros(1, dtype=torch.int64, device=x.device)
        for xv, nv, xt, a_im in ((x, 3, _lib.C128, -0.25), (x[:, 0].contiguous(), 1, _lib.C128, -0.25),
                                 (xr, 1, _lib.F64, 0.0)):
            if xt == _lib.F64 and dt == np.complex128:
                continue
            ys = []
            for P in (P1, P2, P3):
                y = torch.empty_like(xv)
                for g in (0x202, 0x104, 0x408):
                    _lib.call("qs_csr_matvec_pairs", n, A.nnz, D.ptr(A.indptr), A.idx64, D.ptr(P.indices),
                              D.ptr(P.data), P.vcode, D.ptr(xv), xt, D.ptr(y), nv, 0.5, a_im, 1, g, D.ptr(xs),
                              D.ptr(nrm), D.stream())
                    ys.append(y.clone())
            for i in range(3):
                assert torch.equal(ys[i], ys[3 + i]) and torch.equal(ys[i], ys[6 + i]), (nv, xt, i)
            np.testing.assert_allclose(D.to_host(ys[0]), (0.5 + 1j * a_im) * (A.tocsr() @ D.to_host(xv)), rtol=0,
                                       atol=1e-12)
        v = rng.normal(size=n) + 1j * rng.normal(size=n)
        v /= np.linalg.norm(v)
        outs = []
        for coded in (True, False):
            op = ExpmMultiplyParallel(A, a=-2j)
            if not coded:
                op._Ad.__dict__["_paired_coded"] = PairedCSR(op._Ad, coded=False)
            outs.append(op.dot(D.to_device(v)))
        assert torch.equal(outs[0], outs[1])


def test_packed_vector_loads_spmv(cuda):
    """The packed operand read four column words per 16-byte load (launch
    shape 6, one complex vector): the same products as the one-word form in
    a different order within each lane; against scipy in float64 at the
    float-pair rounding of each row's sum of moduli, for 2 and 4 lanes per
    row, overwrite and accumulate."""
    import torch
    import scipy.sparse as sp
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    from quspin_gb300.sparse import DeviceCSR
    rng = np.random.default_rng(9)
    n = 40009
    A = sp.random(n, n, density=30.0 / n, random_state=3, format="csr")
    A.data = rng.choice(np.array([0.5, -1.0, 0.25, 2.0]), A.nnz)
    A = sp.csr_matrix(A + A.T)
    A.sum_duplicates()
    Ad = DeviceCSR.from_scipy(A)
    P = Ad.paired(coded=True)
    assert P.coded
    Pk = P.packed()
    assert Pk.padded
    xh = rng.normal(size=n) + 1j * rng.normal(size=n)
    x = D.to_device(xh)
    xs = torch.empty(4 * n, dtype=torch.float32, device="cuda")
    nrm = torch.zeros(1, dtype=torch.int64, device="cuda")
    scale = abs(A) @ abs(xh)
    for G in (2, 4):
        for ow in (1, 0):
            y = D.to_device(np.ones(n, np.complex128) * (0.5 - 0.5j))
            _lib.call("qs_csr_matvec_pairs", n, A.nnz, D.ptr(Ad.indptr), 0, D.ptr(Pk.indices), D.ptr(Pk.data),
                      Pk.vcode, D.ptr(x), _lib.C128, D.ptr(y), 1, 0.75, 0.25, ow, G | (1 << 8) | (6 << 20),
                      D.ptr(xs), D.ptr(nrm), D.stream())
            ref = (0.75 + 0.25j) * (A @ xh) + (0 if ow else (0.5 - 0.5j))
            err = np.abs(D.to_host(y) - ref)
            assert np.all(err <= 1e-13 * (scale + 1.0)), (G, ow)
