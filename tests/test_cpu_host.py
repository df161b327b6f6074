"""Host-side logic that needs no GPU: the coded float-pair operand's value
table (csrc kernels read vals[codes] per nonzero) and the launch-code layout
of the tuner."""
import numpy as np
import torch

from quspin_gb300 import _lib
from quspin_gb300.sparse import value_codes
from quspin_gb300.tune import encode, occ_candidates


def test_value_codes_real_roundtrip():
    rng = np.random.default_rng(0)
    table = rng.normal(size=58)
    src = torch.tensor(table[rng.integers(0, 58, 10000)], dtype=torch.float64)
    vals, codes, distinct = value_codes(src)
    assert distinct == len(np.unique(src.numpy())) <= 58
    assert vals.shape == (256,) and codes.dtype == torch.uint8
    assert torch.equal(vals[codes.long()], src)           # exact, value by value


def test_value_codes_complex_roundtrip():
    rng = np.random.default_rng(1)
    base = rng.normal(size=40) + 1j * rng.normal(size=40)
    base[:5] = base[:5].real                              # some purely real entries
    src = torch.tensor(base[rng.integers(0, 40, 5000)], dtype=torch.complex128)
    vals, codes, distinct = value_codes(src)
    assert distinct <= 40 and vals.shape == (256, 2)
    dec = torch.view_as_complex(vals[codes.long()].contiguous())
    assert torch.equal(dec, src)


def test_value_codes_limits():
    assert value_codes(torch.arange(257, dtype=torch.float64)) is None          # one value too many
    assert value_codes(torch.arange(256, dtype=torch.float64)) is not None
    assert value_codes(torch.tensor([1.0, float("nan")], dtype=torch.float64)) is None
    assert value_codes(torch.zeros(0, dtype=torch.float64)) is None
    z = torch.complex(torch.arange(300, dtype=torch.float64) % 16, torch.arange(300, dtype=torch.float64) // 16)
    assert value_codes(z) is None                        # 300 distinct complex values


def test_launch_code_layout():
    assert encode(4, 2) == 4 | (2 << 8)
    code = encode(2, 1) | (1 << 18)
    assert code & 0xff == 2 and (code >> 8) & 0xff == 1 and (code >> 18) & 3 == 1
    M = type("M", (), {"idx64": 0})()
    assert occ_candidates(M, 1, _lib.CPF) == [(2, 1), (2, 2), (4, 1), (4, 2)]
    assert occ_candidates(M, 8, _lib.CPF) == []
    assert occ_candidates(M, 1, _lib.C128) == []
    M64 = type("M", (), {"idx64": 1})()
    assert occ_candidates(M64, 1, _lib.CPF) == []


def _powers_by_steps(map):
    """The reference's definition of the period (base_general.py:22-51),
    stepped one application at a time: labels move to map[i], an inverted
    site turns label x into -(x + 1); stop when the identity comes back."""
    m = np.asarray(map)
    dest = np.where(m < 0, -m - 1, m)
    sites = np.arange(len(m))
    start = sites.copy()
    seen = [tuple(sites)]
    while True:
        sites = np.where(m < 0, -sites - 1, sites)[dest]
        seen.append(tuple(int(x) for x in sites))
        if np.array_equal(sites, start):
            return len(seen) - 1, set(seen)


def test_process_map_period_and_group_match_stepwise_definition():
    import warnings
    from oracle import oracle as O
    from quspin_gb300.basis import GeneralBasisWarning, process_map
    rng = np.random.default_rng(3)
    L = 12
    s = np.arange(L)
    maps = [(s + 1) % L, s[::-1].copy(), -(s + 1), -(((s + 1) % L) + 1), np.where(s % 3 == 0, -(s[::-1] + 1), s[::-1])]
    for _ in range(40):
        perm = rng.permutation(L)
        flip = rng.random(L) < 0.3
        maps.append(np.where(flip, -(perm + 1), perm))
    for m in maps:
        out_map, per, q, group = process_map(m, 3)
        per_ref, group_ref = _powers_by_steps(m)
        assert per == per_ref == O.process_map(m, 3)[1]
        assert group == group_ref and q == 3 and out_map.dtype == np.int32
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        assert process_map(s, 0)[1] == 1
        assert any(issubclass(x.category, GeneralBasisWarning) for x in w)
    try:
        process_map(np.array([0, 0, 2]), 0)
    except ValueError as e:
        assert str(e) == "map must be a one-to-one site mapping."
    else:
        raise AssertionError("expected ValueError")


def test_consolidate_static_merges_bonds_and_drops_tiny_couplings():
    """_make_hamiltonian._consolidate_static (:19-41): repeated (opstr, sites)
    bonds are summed, couplings with |J| <= 10 eps are dropped."""
    from oracle import oracle as O
    from quspin_gb300.operators import _consolidate_static
    eps = np.finfo(np.float64).eps
    static = [["zz", [[1.0, 0, 1], [0.5, 1, 2], [0.25, 0, 1]]],
              ["+-", [[0.5, 0, 1], [5 * eps, 2, 3], [0.5, 1, 2]]],
              ["zz", [[-0.5, 1, 2], [2.0, 2, 3]]],
              ["x", [[1e-3, 0], [-1e-3, 0]]]]
    out = _consolidate_static(static)
    assert out == O.consolidate_static(static)
    d = {(o, tuple(ix)): J for o, ix, J in out}
    assert d[("zz", (0, 1))] == 1.25
    assert ("zz", (1, 2)) not in d                 # 0.5 - 0.5 = 0 dropped
    assert d[("zz", (2, 3))] == 2.0
    assert ("+-", (2, 3)) not in d                 # 5 eps <= 10 eps dropped
    assert ("x", (0,)) not in d                    # exact cancellation
    assert len(out) == 4


def test_r32_candidates_need_one_vector_float_forms():
    from quspin_gb300.tune import r32_candidates

    def M(vcode, idx64=0, padded=False):
        return type("M", (), {"idx64": idx64, "vcode": vcode, "padded": padded})()
    assert r32_candidates(M(_lib.PF8P), 1, _lib.CPF) == [(s, o) for s in (1, 2, 3, 4, 5) for o in (0, 1)]
    # the four-words-per-load shapes need the padded packed words
    assert r32_candidates(M(_lib.PF8P, padded=True), 1, _lib.CPF) == (
        [(s, o) for s in (1, 2, 3, 4, 5) for o in (0, 1)] + [(s, o) for s in (6, 7) for o in (0, 1, 2)])
    assert len(r32_candidates(M(_lib.PF8, padded=True), 1, _lib.CPF)) == 10
    assert len(r32_candidates(M(_lib.PF8), 1, _lib.CPF)) == 10
    assert r32_candidates(M(_lib.PF8), 2, _lib.CPF) == []
    assert r32_candidates(M(_lib.PF8), 1, _lib.C128) == []
    assert r32_candidates(M(_lib.PF8, idx64=1), 1, _lib.CPF) == []


def test_pair_split_reference_restates_the_definition():
    """The numpy restatement the bit-exact GPU test of qs_split_pairs_trunc
    compares with: hi has 24 significant bits, hi + lo has 48, the rest is
    below 2^-46 of x 2^-k, and both parts are truncations (|hi| <= |x|,
    |lo| <= |x 2^-k - hi|, same signs)."""
    from tests.test_gpu_pair_split import _reference
    rng = np.random.default_rng(0)
    x = rng.normal(size=50000) * np.exp(rng.uniform(-30, 30, 50000))
    for k in (0, 7, -5, 30):
        xs = x * 2.0 ** -k
        hi, lo = _reference(x, k)
        h, l_ = hi.astype(np.float64), lo.astype(np.float64)
        assert np.all(np.abs(xs - h - l_) <= 2.0 ** -46 * np.abs(xs))
        assert np.all(np.abs(h) <= np.abs(xs)) and np.all(np.abs(l_) <= np.abs(xs - h))
        assert np.all((h == 0) | (np.sign(h) == np.sign(xs)))
        assert np.all((l_ == 0) | (np.sign(l_) == np.sign(xs)))
        # 24 significant bits: the low 29 bits of the float64 pattern are zero
        assert np.all((h.view(np.uint64) & np.uint64((1 << 29) - 1)) == 0)


def test_sorted_conj_transpose_host_logic(monkeypatch):
    """The sort-based conjugate transpose (used for columns beyond the merge
    kernel's capacity) is plain torch code: run it on CPU tensors against
    scipy, with a full column and empty rows."""
    import scipy.sparse as sp
    from quspin_gb300 import _device as D
    from quspin_gb300.sparse import DeviceCSR
    monkeypatch.setattr(D, "device", lambda: torch.device("cpu"))
    rng = np.random.default_rng(5)
    n = 700
    A = sp.random(n, n, density=0.01, random_state=6, format="lil", dtype=np.complex128)
    A[:, 3] = rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1))
    A[10, :] = 0
    A = sp.csr_matrix(A)
    A.sum_duplicates()
    A.eliminate_zeros()
    M = DeviceCSR(torch.tensor(A.indptr.astype(np.int32)), torch.tensor(A.indices.astype(np.int32)),
                  torch.tensor(A.data), A.shape, np.complex128)
    T = M._conj_transpose_sorted()
    R = sp.csr_matrix(A.conj().T)
    R.sort_indices()
    np.testing.assert_array_equal(T.indptr.numpy(), R.indptr)
    np.testing.assert_array_equal(T.indices.numpy(), R.indices)
    np.testing.assert_array_equal(T.data.numpy(), R.data)
