"""qs_split_pairs_trunc (csrc/expm_lp.cu, the float-pair split of the
many-vector stopping tests, formed with integer operations only) against a
numpy restatement of its definition in float64 arithmetic: hi = x 2^-k
truncated to 24 significant bits, lo = (x 2^-k - hi) truncated likewise,
zero below the normal float range.  Bit-exact."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

_TRUNC = np.uint64(~((1 << 29) - 1) & ((1 << 64) - 1))


def _trunc24(d):
    """float64 array -> float32 by truncation to 24 significant bits; values
    below the normal float32 range -> signed zero."""
    t = (d.view(np.uint64) & _TRUNC).view(np.float64)
    small = np.abs(t) < np.float64(np.finfo(np.float32).tiny)
    t = np.where(small, np.copysign(0.0, d), t)
    return t.astype(np.float32)


def _reference(x, k):
    xs = x * np.float64(2.0) ** -k                     # exact for the inputs below
    hi = _trunc24(xs)
    lo = _trunc24(xs - hi.astype(np.float64))
    return hi, lo


@pytest.mark.parametrize("k", [0, 7, -5, 30])
def test_split_pairs_trunc_bit_exact(cuda, k):
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    rng = np.random.default_rng(11 + k)
    x = np.concatenate([
        rng.normal(size=200000) * np.exp(rng.uniform(-30, 30, 200000)),
        rng.normal(size=1000).astype(np.float32).astype(np.float64),     # exact floats: lo = 0
        np.array([0.0, -0.0, 1.0, -1.0, 2.0 ** -100, -(2.0 ** -120), 1.0 + 2.0 ** -52, 3.0 - 2.0 ** -51]),
    ])
    xd = D.to_device(x)
    out = torch.empty(2 * x.size, dtype=torch.float32, device="cuda")
    _lib.call("qs_split_pairs_trunc", x.size, D.ptr(xd), k, D.ptr(out), D.stream())
    got = out.cpu().numpy().reshape(-1, 2)
    hi, lo = _reference(x, k)
    np.testing.assert_array_equal(got[:, 0].view(np.uint32), hi.view(np.uint32))
    # zero low parts may differ in sign only (the moduli square them)
    g_lo, r_lo = got[:, 1], lo
    both_zero = (g_lo == 0) & (r_lo == 0)
    np.testing.assert_array_equal(g_lo[~both_zero].view(np.uint32), r_lo[~both_zero].view(np.uint32))
    assert np.all(g_lo[both_zero] == 0)
