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
