"""The single-vector Taylor terms of csrc/expm_st.cu (the 32-row kernel and
the persistent row-handout kernel) against the row-handout term of
csrc/expm_lp.cu on the same inputs: one term gives
bit-identical B, F and stopping-test norm for every value form (coded,
coded with the codes packed into the column words, one pair per nonzero,
complex coded, and the complex64 form) and every lane count, on a matrix
with an odd number of rows, empty rows and one long row; whole evolutions
through ExpmMultiplyParallel are bit-identical too."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

pytestmark = pytest.mark.gpu


def _matrix(n=70001, complex_vals=False, seed=0):
    """Hermitian matrix with few distinct values (so that it codes): unique
    upper-triangle pairs with values from a small set, their conjugate
    transposes and a diagonal from a small set; one empty row, one long row."""
    rng = np.random.default_rng(seed)
    m = 12 * n
    r, c = rng.integers(0, n, m), rng.integers(0, n, m)
    lo, hi = np.minimum(r, c), np.maximum(r, c)
    keep = lo < hi
    key = np.unique(lo[keep].astype(np.int64) * n + hi[keep])
    long_row = n // 2
    key = np.unique(np.concatenate([key, np.minimum(long_row, np.arange(0, n, 37)) * n
                                    + np.maximum(long_row, np.arange(0, n, 37))]))
    key = key[(key // n) < (key % n)]
    empty = n // 3
    key = key[(key // n != empty) & (key % n != empty)]
    rr, cc = key // n, key % n
    vals = np.array([0.5, -0.5, 0.25, 1.0, -1.5, 0.7071067811865476])
    if complex_vals:
        vals = vals * np.exp(1j * np.array([0.0, 0.5, 1.0, 0.5, 0.0, 1.0]))
    v = rng.choice(vals, key.size)
    d = rng.choice(np.array([0.0, 0.3, -1.2]), n)
    d[empty] = 0.0
    U = sp.csr_matrix((v, (rr, cc)), shape=(n, n))
    A = sp.csr_matrix(U + U.conj().T + sp.diags(d))
    A.eliminate_zeros()
    assert A[empty].nnz == 0 and A[long_row].nnz > 1000
    return A


def _term(M, code, B_in, F_in, btype):
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    n = M.shape[0]
    F = F_in.clone()
    Bout = torch.zeros_like(B_in)
    ctl = torch.zeros(_lib.load().qs_expm_ctl_bytes() // 8 + 1, dtype=torch.int64, device="cuda")
    coeff = torch.tensor([0.03 - 0.02j], dtype=torch.complex128, device="cuda")
    _lib.call("qs_taylor_term", n, M.nnz, D.ptr(M.indptr), M.idx64, D.ptr(M.indices), D.ptr(M.data), M.vcode,
              D.ptr(B_in), D.ptr(Bout), btype, D.ptr(F), 1, 0.37, 0.0, D.ptr(coeff), 0, 0.0, D.ptr(ctl), code,
              D.stream())
    torch.cuda.synchronize()
    assert int(ctl.view(torch.int32)[12].item()) == 0
    return Bout, F, float(ctl.view(torch.float64)[0].item())


def _same(a, b):
    return torch.equal(a.view(torch.int64) if a.dtype == torch.complex128 else a.view(torch.int32),
                       b.view(torch.int64) if b.dtype == torch.complex128 else b.view(torch.int32))


@pytest.mark.parametrize("complex_vals", [False, True])
def test_r32_term_bitwise_equal_to_row_handout(cuda, complex_vals):
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    from quspin_gb300.sparse import DeviceCSR
    from quspin_gb300.tune import encode
    A = _matrix(complex_vals=complex_vals)
    Ad = DeviceCSR.from_scipy(A)
    n = A.shape[0]
    g = torch.Generator(device="cpu").manual_seed(1)
    v = torch.randn(n, dtype=torch.complex128, generator=g).to("cuda")
    F0 = torch.randn(n, dtype=torch.complex128, generator=g).to("cuda")
    Bp = torch.empty(n, dtype=torch.complex128, device="cuda")          # float-pair storage, 16 bytes per element
    _lib.call("qs_split_pairs", 2 * n, D.ptr(v), D.ptr(Bp), D.stream())
    coded = Ad.paired(coded=True)
    assert coded.coded
    forms = [coded, coded.packed(), Ad.paired(coded=False)]
    for G, shape in ((4, 1), (2, 2), (8, 3), (2, 4), (4, 5)):
        ref = _term(coded, encode(G, 2), Bp, F0, _lib.CPF)
        for M in forms:
            for occ in (0, 1):
                out = _term(M, encode(G, 2) | (occ << 18) | (shape << 20), Bp, F0, _lib.CPF)
                assert _same(out[0], ref[0]) and _same(out[1], ref[1]), (G, M.vcode, occ)
                assert out[2] == ref[2]
    # complex64 form: float32 / complex64 values, complex64 B
    M32 = Ad.astype(np.complex64 if complex_vals else np.float32)
    B32 = v.to(torch.complex64)
    for G, shape in ((4, 1), (2, 2), (2, 4), (4, 5)):
        ref = _term(M32, encode(G, 2), B32, F0, _lib.C64)
        out = _term(M32, encode(G, 2) | (shape << 20), B32, F0, _lib.C64)
        assert _same(out[0], ref[0]) and _same(out[1], ref[1]) and out[2] == ref[2]


def test_r32_evolution_bitwise_equal(cuda):
    from quspin_gb300 import _lib
    from quspin_gb300.sparse import DeviceCSR
    from quspin_gb300.tools import ExpmMultiplyParallel
    from quspin_gb300.tune import encode
    A = _matrix(seed=3)
    n = A.shape[0]
    rng = np.random.default_rng(4)
    v = rng.normal(size=n) + 1j * rng.normal(size=n)
    v /= np.linalg.norm(v)
    out = []
    for packed, code in ((False, encode(4, 2)), (False, encode(4, 2) | (1 << 20)), (True, encode(4, 2) | (1 << 20)),
                         (True, encode(4, 2) | (5 << 20) | (1 << 18))):
        op = ExpmMultiplyParallel(DeviceCSR.from_scipy(A), a=-0.8j)
        P = op.A_device.paired()
        M = P.packed() if packed else P
        op._pick = M
        M.__dict__.setdefault("_tuned", {})[("taylor", 1, _lib.CPF)] = code
        F = torch.tensor(v, device="cuda")
        op.run_device(F)
        out.append(F.cpu().numpy())
    for o in out[1:]:
        assert np.array_equal(out[0].view(np.int64), o.view(np.int64))


@pytest.mark.parametrize("complex_vals", [False, True])
def test_rows_vector_loads_term(cuda, complex_vals):
    """Row hand-out term reading the packed column words four per 16-byte
    load (shapes 6 / 7): the same products as the one-word form (shapes
    4 / 5), summed in a different order within each lane, so the new term, F
    and the stopping-test norm agree to float-pair rounding; the
    register-cap variants of one shape are bit-identical."""
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    from quspin_gb300.sparse import DeviceCSR
    from quspin_gb300.tune import encode
    A = _matrix(n=50003, complex_vals=complex_vals, seed=5)
    Ad = DeviceCSR.from_scipy(A)
    n = A.shape[0]
    g = torch.Generator(device="cpu").manual_seed(2)
    v = torch.randn(n, dtype=torch.complex128, generator=g).to("cuda")
    F0 = torch.randn(n, dtype=torch.complex128, generator=g).to("cuda")
    Bp = torch.empty(n, dtype=torch.complex128, device="cuda")          # float-pair storage
    _lib.call("qs_split_pairs", 2 * n, D.ptr(v), D.ptr(Bp), D.stream())
    Pk = Ad.paired(coded=True).packed()
    assert Pk.padded and Pk.indices.numel() >= (Pk.nnz + 3) // 4 * 4 + 4

    def value(B):          # {re.hi, re.lo, im.hi, im.lo} -> complex128
        x = B.view(torch.float32).reshape(n, 2, 2).double().sum(-1)
        return torch.complex(x[:, 0], x[:, 1])

    # reordering a sum moves it by a small multiple of the unit roundoff times
    # the sum of the moduli of its terms: per-row scale |cf| (|A| |B| + |mu| |B|)
    vh = v.cpu().numpy()
    scale = abs(0.03 - 0.02j) * (abs(A) @ abs(vh) + 0.37 * abs(vh))
    scale_d = torch.tensor(scale, device="cuda")
    for G, shape_old, shape_new in ((2, 4, 6), (4, 5, 7)):
        ref = _term(Pk, encode(G, 2) | (shape_old << 20), Bp, F0, _lib.CPF)
        outs = [_term(Pk, encode(G, 2) | (occ << 18) | (shape_new << 20), Bp, F0, _lib.CPF) for occ in (0, 1, 2)]
        for o in outs[1:]:
            assert _same(o[0], outs[0][0]) and _same(o[1], outs[0][1]) and o[2] == outs[0][2]
        assert bool(((value(outs[0][0]) - value(ref[0])).abs() <= 1e-12 * scale_d).all()), G
        # F += the new term (in units 2^bexp of the control block: B's scale)
        assert float((outs[0][1] - ref[1]).abs().max()) <= 1e-12 * float(scale.max()), G
        assert abs(outs[0][2] - ref[2]) <= 1e-12 * abs(ref[2]), G


def test_rows_vector_loads_evolution(cuda):
    """A whole evolution on the four-words-per-load shape against the
    one-word shape: the same (m*, s) and states within 1e-13."""
    from quspin_gb300 import _lib
    from quspin_gb300.sparse import DeviceCSR
    from quspin_gb300.tools import ExpmMultiplyParallel
    from quspin_gb300.tune import encode
    A = _matrix(seed=6)
    n = A.shape[0]
    rng = np.random.default_rng(7)
    v = rng.normal(size=n) + 1j * rng.normal(size=n)
    v /= np.linalg.norm(v)
    out = []
    for code in (encode(2, 2) | (4 << 20) | (1 << 18), encode(2, 2) | (6 << 20), encode(4, 2) | (7 << 20) | (2 << 18)):
        op = ExpmMultiplyParallel(DeviceCSR.from_scipy(A), a=-0.8j)
        M = op.A_device.paired().packed()
        op._pick = M
        M.__dict__.setdefault("_tuned", {})[("taylor", 1, _lib.CPF)] = code
        F = torch.tensor(v, device="cuda")
        op.run_device(F)
        out.append(F.cpu().numpy())
    for o in out[1:]:
        assert np.linalg.norm(o - out[0]) <= 1e-13 * np.linalg.norm(out[0])
