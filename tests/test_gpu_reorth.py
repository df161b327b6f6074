"""qs_lanczos_reorth (csrc/lanczos.cu): classical Gram-Schmidt applied twice,
r -= Q[:nk]^T (conj(Q[:nk]) r), against numpy in float64 / complex128.

Covers row counts that leave partial row groups (the kernel takes 16 real or
8 complex rows per pass over the elements), vectors shorter than one block,
lengths that are not a multiple of the grid, and a row stride larger than n.
FP64 products in a different summation order: 1e-13 relative to the scale
of the projections."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _reorth(Qh, rh, n, passes=2):
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    L = _lib.load()
    nk, ldq = Qh.shape
    cplx = int(np.iscomplexobj(Qh))
    Q = torch.tensor(Qh, device="cuda")
    r = torch.tensor(rh, device="cuda")
    dv = (lambda t: D.ptr(torch.view_as_real(t))) if cplx else D.ptr
    scr = D.scratch_doubles(int(L.qs_lanczos_reorth_scratch_doubles(nk)))
    ctl = torch.zeros(int(L.qs_lanczos_ctl_bytes()), dtype=torch.uint8, device="cuda")
    _lib.check(L.qs_lanczos_reorth(n, cplx, nk, dv(Q), ldq, dv(r), passes, D.ptr(scr), D.ptr(ctl), D.stream()),
               "qs_lanczos_reorth")
    return r.cpu().numpy()


@pytest.mark.parametrize("nk,n", [(1, 1000), (7, 100), (8, 5000), (9, 100003), (16, 70001), (17, 33), (33, 200000),
                                  (50, 12345)])
@pytest.mark.parametrize("cplx", [False, True])
def test_reorth_matches_numpy(cuda, nk, n, cplx):
    rng = np.random.default_rng(nk * 7919 + n)
    Qh = rng.normal(size=(nk, n + 3))
    rh = rng.normal(size=n)
    if cplx:
        Qh = Qh + 1j * rng.normal(size=Qh.shape)
        rh = rh + 1j * rng.normal(size=n)
    # orthonormal rows, as the Lanczos vectors are
    q, _ = np.linalg.qr(Qh[:, :n].T)
    Qh[:, :n] = q.T
    out = _reorth(Qh, rh, n)
    ref = rh.copy()
    Qn = Qh[:, :n]
    for _ in range(2):
        ref = ref - Qn.T @ (Qn.conj() @ ref)
    scale = np.linalg.norm(rh)
    assert np.linalg.norm(out - ref) <= 1e-13 * scale
    # the result is orthogonal to every row
    assert np.abs(Qn.conj() @ out).max() <= 1e-13 * scale


def test_reorth_single_pass_removes_projection(cuda):
    """one pass on a vector built from the rows plus an orthogonal part leaves
    the orthogonal part"""
    rng = np.random.default_rng(11)
    n, nk = 40000, 21
    q, _ = np.linalg.qr(rng.normal(size=(n, nk + 1)))
    Qh = np.ascontiguousarray(q[:, :nk].T)
    c = rng.normal(size=nk)
    rh = Qh.T @ c + q[:, nk]
    out = _reorth(Qh, rh, n, passes=1)
    np.testing.assert_allclose(out, q[:, nk], rtol=0, atol=1e-13)


def _reorth_adaptive(Qh, rh, n, max_passes=2):
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    L = _lib.load()
    nk, ldq = Qh.shape
    cplx = int(np.iscomplexobj(Qh))
    Q = torch.tensor(Qh, device="cuda")
    r = torch.tensor(rh, device="cuda")
    dv = (lambda t: D.ptr(torch.view_as_real(t))) if cplx else D.ptr
    scr = D.scratch_doubles(int(L.qs_lanczos_reorth_scratch_doubles(nk)))
    ctl = torch.zeros(int(L.qs_lanczos_ctl_bytes()), dtype=torch.uint8, device="cuda")
    _lib.check(L.qs_lanczos_reorth_adaptive(n, cplx, nk, dv(Q), ldq, dv(r), max_passes, D.ptr(scr), D.ptr(ctl),
                                            D.stream()), "qs_lanczos_reorth_adaptive")
    return r.cpu().numpy()


@pytest.mark.parametrize("cplx", [False, True])
def test_reorth_adaptive_one_pass_when_norm_kept(cuda, cplx):
    """a random vector against 33 orthonormal rows keeps almost all of its
    norm: one pass, the same result as the fixed single pass"""
    rng = np.random.default_rng(21)
    n, nk = 50001, 33
    Qh = rng.normal(size=(nk, n)) + (1j * rng.normal(size=(nk, n)) if cplx else 0)
    q, _ = np.linalg.qr(Qh.T)
    Qh = np.ascontiguousarray(q.T)
    rh = rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
    out = _reorth_adaptive(Qh, rh, n)
    one = _reorth(Qh, rh, n, passes=1)
    np.testing.assert_array_equal(out, one)
    assert np.abs(Qh.conj() @ out).max() <= 1e-13 * np.linalg.norm(rh)


@pytest.mark.parametrize("cplx", [False, True])
def test_reorth_adaptive_second_pass_when_norm_lost(cuda, cplx):
    """a vector that lies almost in the span of the rows (orthogonal part
    1e-6 of it) loses its norm in the first pass, so a second pass runs and
    the result is orthogonal to the rows to working precision relative to
    its own norm, as the fixed two passes give"""
    rng = np.random.default_rng(22)
    n, nk = 40000, 21
    G = rng.normal(size=(n, nk + 1)) + (1j * rng.normal(size=(n, nk + 1)) if cplx else 0)
    q, _ = np.linalg.qr(G)
    Qh = np.ascontiguousarray(q[:, :nk].T)
    rh = Qh.T @ rng.normal(size=nk) + 1e-6 * q[:, nk]
    out = _reorth_adaptive(Qh, rh, n)
    two = _reorth(Qh, rh, n, passes=2)
    np.testing.assert_array_equal(out, two)
    assert np.abs(Qh.conj() @ out).max() <= 1e-12 * np.linalg.norm(out)
    np.testing.assert_allclose(out, 1e-6 * q[:, nk], rtol=0, atol=1e-15)
