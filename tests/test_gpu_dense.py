"""qs_block_inner and qs_block_inner_dmma (csrc/dense.cu): the dense FP64
panels of the Lanczos tools, W[i, j] = sum_r op(Q[i, r]) X[r, j], against
numpy in float64 / complex128 at 1e-13 relative (FP64 products, a different
summation order), for the tiled shape (k > 2: FP64 FMAs, or FP64 tensor
instructions in the _dmma form) and the matrix-vector shape (k <= 2), with odd
sizes, row strides larger than n and both conjugation modes."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _inner(Q, X, conj, ldq=None, xrows=False, fn="qs_block_inner"):
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    m, nq = Q.shape
    k, n = X.shape if xrows else X.shape[::-1]
    cplx = int(Q.is_complex())
    ldq = nq if ldq is None else ldq
    W = torch.empty((m, k), dtype=Q.dtype, device="cuda")
    scr = torch.empty(int(_lib.load().qs_block_inner_scratch_doubles(n, m, k, cplx)), dtype=torch.float64,
                      device="cuda")
    _lib.call(fn, n, m, k, D.ptr(Q), ldq, D.ptr(X), X.shape[1], int(xrows), cplx, int(conj), D.ptr(W),
              D.ptr(scr), D.stream())
    return W.cpu().numpy()


@pytest.mark.parametrize("m,k,n", [(40, 40, 100003), (7, 13, 5000), (33, 3, 70001), (64, 64, 2000), (5, 1, 12345),
                                   (20, 2, 999)])
@pytest.mark.parametrize("cplx,conj", [(False, False), (True, False), (True, True)])
@pytest.mark.parametrize("fn", ["qs_block_inner", "qs_block_inner_dmma"])
def test_block_inner_matches_numpy(cuda, m, k, n, cplx, conj, fn):
    rng = np.random.default_rng(m * 1000 + k)
    Qh = rng.normal(size=(m, n + 5))
    Xh = rng.normal(size=(n, k))
    if cplx:
        Qh = Qh + 1j * rng.normal(size=Qh.shape)
        Xh = Xh + 1j * rng.normal(size=Xh.shape)
    Q = torch.tensor(Qh, device="cuda")
    X = torch.tensor(Xh, device="cuda")
    W = _inner(Q, X, conj, ldq=n + 5, fn=fn)
    Qn = Qh[:, :n].conj() if conj else Qh[:, :n]
    ref = Qn @ Xh
    scale = np.abs(Qn) @ np.abs(Xh)
    assert np.abs(W - ref).max() <= 1e-13 * scale.max()
    # the same vectors of X stored as rows
    Wr = _inner(Q, torch.tensor(np.ascontiguousarray(Xh.T), device="cuda"), conj, ldq=n + 5, xrows=True, fn=fn)
    assert np.abs(Wr - ref).max() <= 1e-13 * scale.max()
