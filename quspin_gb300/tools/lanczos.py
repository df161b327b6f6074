"""Lanczos tools with a device-resident recurrence.

Drop-in counterparts of QuSpin 1.0.1's ``lanczos_full``, ``lanczos_iter``,
``lin_comb_Q_T`` (src/quspin/tools/lanczos/_lanczos_utils.py:77-425) and
``expm_lanczos`` (src/quspin/tools/lanczos/_expm.py:7-52).  The recurrence
(scale, product, the two axpys, the dot product and the norm) runs on the
GPU with alpha/beta kept in device arrays; only the m x m tridiagonal
eigenproblem is solved on the host (scipy ``eigh_tridiagonal``), as in the
reference.  ``full_ortho=True`` keeps the reference's post-hoc
orthonormalisation + projection (:206-222), with the orthonormalisation by
classical Gram-Schmidt twice and the projection as one tiled FP64
block product (csrc/dense.cu); ``reorth=True`` is this package's per-step full
reorthogonalisation (classical Gram-Schmidt against every previous Lanczos
vector, repeated once only when the first pass removed more than
1 - 1/sqrt(2) of the norm, the criterion ARPACK applies), for long runs where
the plain recurrence loses orthogonality.
"""
from __future__ import annotations

import numpy as np
import torch
from scipy.linalg import eigh_tridiagonal

from .. import _device as D
from .. import _lib
from ..sparse import DeviceCSR, DeviceDIA, to_device_matrix

__all__ = ["lanczos_full", "lanczos_iter", "lin_comb_Q_T", "expm_lanczos", "FTLM_static_iteration",
           "LTLM_static_iteration"]


class _DeviceOp:
    """Uniform device product y = A x for the operators this package knows.
    precision="mixed" runs the product in single precision: x is rounded to
    float32 / complex64, multiplied by float32 / complex64 matrix values with
    FP32 row sums, and the result widened back into the FP64 vector y (the
    recurrence itself stays FP64)."""

    def __init__(self, A, precision="double"):
        from ..operators import hamiltonian, quantum_LinearOperator
        self._x32 = self._y32 = None
        if precision == "mixed":
            if isinstance(A, hamiltonian):
                A = A.tocsr_gpu()
            if isinstance(A, (DeviceCSR, DeviceDIA)):
                dt = np.dtype(A.dtype)
                A = A.astype(np.float32 if dt.kind == "f" else np.complex64)
                self.dtype = dt
            else:
                raise TypeError("precision='mixed' needs a hamiltonian or a device matrix")
            self.A = A
            self._f = self._single
            return
        self.A = A
        if isinstance(A, (DeviceCSR, DeviceDIA)):
            self._f = lambda x, y: A.matvec_into(x, y, overwrite=True)
        elif isinstance(A, hamiltonian):
            self._f = lambda x, y: A.dot(x, out=y)
        elif isinstance(A, quantum_LinearOperator):
            self._f = lambda x, y: A.dot(x, out=y)
        elif hasattr(A, "tocsr") or hasattr(A, "toarray") or isinstance(A, np.ndarray):
            import scipy.sparse as sp
            M = to_device_matrix(sp.csr_matrix(A))
            self.A = M
            self._f = lambda x, y: M.matvec_into(x, y, overwrite=True)
        else:
            raise TypeError("A must be a hamiltonian, quantum_LinearOperator or (sparse) matrix")
        self.dtype = np.dtype(A.dtype)

    def _single(self, x, y):
        st = torch.complex64 if x.is_complex() else torch.float32
        if self._x32 is None or self._x32.shape != x.shape or self._x32.dtype != st:
            self._x32 = torch.empty(x.shape, dtype=st, device=x.device)
            self._y32 = torch.empty(x.shape, dtype=st, device=x.device)
        self._x32.copy_(x)
        self.A.matvec_into(self._x32, self._y32, overwrite=True)
        y.copy_(self._y32)

    def __call__(self, x, y):
        self._f(x, y)


def _work_dtype(dtype):
    return np.dtype(np.complex128) if np.dtype(dtype).kind == "c" else np.dtype(np.float64)


def _recurrence(op, q0, m, eps, Q=None, reorth=False):
    """Runs the recurrence on the device.  q0: device vector (normalised).
    Q: optional device [m, n] tensor receiving the Lanczos vectors.  Returns
    (a, b, m_eff) with a, b host arrays."""
    n = q0.shape[0]
    cplx = int(q0.dtype == torch.complex128)
    n2 = n * (2 if cplx else 1)
    L = _lib.load()
    st = D.stream()
    ab = torch.zeros(2 * m + 1, dtype=torch.float64, device=D.device())
    a_d, b_d = ab[:m], ab[m:2 * m]
    scr = D.scratch_doubles(L.qs_lanczos_scratch_doubles())
    ctl = torch.zeros(2, dtype=torch.int32, device=D.device())
    ctl[1] = m
    rscr = D.scratch_doubles(L.qs_lanczos_reorth_scratch_doubles(m)) if reorth else None
    keep = Q is not None
    q = Q[0] if keep else torch.empty_like(q0)
    if not keep:
        q.copy_(q0)
    v = torch.zeros_like(q0)
    r = torch.zeros_like(q0)
    dv = lambda t: D.ptr(torch.view_as_real(t) if t.is_complex() else t)
    op(q, r)
    _lib.check(L.qs_lanczos_alpha(n, cplx, dv(r), None, None, dv(q), D.ptr(a_d[0:1]), D.ptr(scr), D.ptr(ctl), st),
               "qs_lanczos_alpha")
    if reorth:
        pass  # nothing earlier to project out
    _lib.check(L.qs_lanczos_beta(n2, dv(r), D.ptr(a_d[0:1]), dv(q), 1, D.ptr(b_d[0:1]), float(eps), 0,
                                 D.ptr(scr), D.ptr(ctl), st), "qs_lanczos_beta")
    for i in range(1, m):
        if keep:
            qi = Q[i]
            qprev = Q[i - 1]
        else:
            v.copy_(q)
            qi, qprev = q, v
        _lib.check(L.qs_lanczos_scale(n2, dv(r), D.ptr(b_d[i - 1:i]), dv(qi), D.ptr(ctl), st), "qs_lanczos_scale")
        op(qi, r)
        _lib.check(L.qs_lanczos_alpha(n, cplx, dv(r), dv(qprev), D.ptr(b_d[i - 1:i]), dv(qi), D.ptr(a_d[i:i + 1]),
                                      D.ptr(scr), D.ptr(ctl), st), "qs_lanczos_alpha")
        if reorth and keep:
            # r -= a_i q_i first, then project out Q[0..i] twice
            _lib.check(L.qs_lanczos_beta(n2, dv(r), D.ptr(a_d[i:i + 1]), dv(qi), 1, D.ptr(ab[2 * m:]), 0.0, i,
                                         D.ptr(scr), D.ptr(ctl), st), "qs_lanczos_beta")
            _lib.check(L.qs_lanczos_reorth_adaptive(n, cplx, i + 1, dv(Q), n, dv(r), 2, D.ptr(rscr), D.ptr(ctl),
                                                    st), "qs_lanczos_reorth_adaptive")
            _lib.check(L.qs_lanczos_beta(n2, dv(r), None, dv(qi), 0, D.ptr(b_d[i:i + 1]), float(eps), i,
                                         D.ptr(scr), D.ptr(ctl), st), "qs_lanczos_beta")
        else:
            _lib.check(L.qs_lanczos_beta(n2, dv(r), D.ptr(a_d[i:i + 1]), dv(qi), 1, D.ptr(b_d[i:i + 1]), float(eps),
                                         i, D.ptr(scr), D.ptr(ctl), st), "qs_lanczos_beta")
    m_eff = int(ctl[1].item())
    a = D.to_host(a_d)
    b = D.to_host(b_d)
    return a, b, m_eff, r, ab


def _start_vector(v0, dtype, eps):
    q = D.to_device(v0, _work_dtype(dtype)).reshape(-1).clone()
    nrm = float(torch.linalg.vector_norm(q).item())
    if np.abs(nrm - 1.0) > eps:
        q.div_(nrm)
    return q


def lanczos_full(A, v0, m, full_ortho=False, out=None, eps=None, reorth=False, precision="double"):
    """(E, V, Q_T) of an m-step Lanczos run (_lanczos_utils.py:77-227)."""
    host = not D.is_device_array(v0)
    v0a = np.asanyarray(v0) if host else v0
    n = v0a.shape[0] if v0a.ndim else 1
    vdt = v0a.dtype if host else D.np_dtype(v0a.dtype)
    op = _DeviceOp(A, precision)
    dtype = np.result_type(op.dtype, vdt)
    if v0a.ndim != 1:
        raise ValueError("expecting array with ndim=1 for initial Lanczos vector.")
    if m >= n:
        raise ValueError("Requested size of Lanczos basis must be smaller then size of original space (e.g. m < n).")
    if out is not None:
        if tuple(out.shape) != (m, n):
            raise ValueError("argument 'out' must have shape (m,n), see documentation.")
        odt = out.dtype if not D.is_device_array(out) else D.np_dtype(out.dtype)
        if odt != dtype:
            raise ValueError("argument 'out' has dtype {}, expecting dtype {}".format(odt, dtype))
    if eps is None:
        eps = np.finfo(dtype).eps
    wdt = _work_dtype(dtype)
    Q = torch.empty((m, n), dtype=D.torch_dtype(wdt), device=D.device())
    Q[0].copy_(_start_vector(v0, dtype, eps))
    a, b, m_eff, r, _ = _recurrence(op, Q[0], m, eps, Q=Q, reorth=reorth)
    m = m_eff
    if full_ortho:
        # orthonormalise Q[:m], then h[i, j] = <A q_i | q_j> (its upper
        # triangle is what the reference fills, :211-220) as one block
        # product of the rows R[i] = A q_i with the rows of Q
        _orthonormalize_rows(Q, m)
        R = torch.empty_like(Q[:m])
        for i in range(m):
            op(Q[i], R[i])
        h = D.to_host(_block_inner(R, Q[:m], conj=True, xrows=True).real)
        E, V = np.linalg.eigh(h, UPLO="U")
    else:
        E, V = eigh_tridiagonal(a[:m], b[:m - 1])
    Qm = Q[:m]
    if out is not None:
        if D.is_device_array(out):
            out[:m].copy_(Qm.to(out.dtype))
            return E, V, out[:m]
        out[:m] = D.to_host(Qm).astype(dtype, copy=False)
        return E, V, out[:m]
    if host:
        return E, V, D.to_host(Qm).astype(dtype, copy=False)
    return E, V, Qm.to(D.torch_dtype(dtype))


class _lanczos_vec_iter:
    """Regenerates the Lanczos vectors on demand (_lanczos_utils.py:15-74),
    with the same kernels and the stored device alpha / beta, so the vectors
    are bit-identical to the first pass."""

    def __init__(self, op, q0, ab, m, host, dtype):
        self._op, self._q0, self._ab, self._m = op, q0, ab, m
        self._host, self._dtype = host, dtype

    def __iter__(self):
        m = self._m
        M = (self._ab.shape[0] - 1) // 2
        a_d, b_d = self._ab[:M], self._ab[M:2 * M]
        q = self._q0.clone()
        v = torch.zeros_like(q)
        r = torch.zeros_like(q)
        n = q.shape[0]
        cplx = int(q.is_complex())
        n2 = n * (2 if cplx else 1)
        L = _lib.load()
        st = D.stream()
        scr = D.scratch_doubles(L.qs_lanczos_scratch_doubles())
        dummy = D.scratch_doubles(1)
        ctl = torch.zeros(2, dtype=torch.int32, device=D.device())
        dv = lambda t: D.ptr(torch.view_as_real(t) if t.is_complex() else t)
        out = lambda t: D.to_host(t).astype(self._dtype, copy=False) if self._host else t.clone()
        self._op(q, r)
        _lib.check(L.qs_lanczos_alpha(n, cplx, dv(r), None, None, dv(q), D.ptr(dummy), D.ptr(scr), D.ptr(ctl), st),
                   "qs_lanczos_alpha")
        _lib.check(L.qs_lanczos_beta(n2, dv(r), D.ptr(a_d[0:1]), dv(q), 1, D.ptr(dummy), 0.0, 0, D.ptr(scr),
                                     D.ptr(ctl), st), "qs_lanczos_beta")
        yield out(q)
        for i in range(1, m):
            v.copy_(q)
            _lib.check(L.qs_lanczos_scale(n2, dv(r), D.ptr(b_d[i - 1:i]), dv(q), D.ptr(ctl), st), "qs_lanczos_scale")
            self._op(q, r)
            _lib.check(L.qs_lanczos_alpha(n, cplx, dv(r), dv(v), D.ptr(b_d[i - 1:i]), dv(q), D.ptr(dummy),
                                          D.ptr(scr), D.ptr(ctl), st), "qs_lanczos_alpha")
            _lib.check(L.qs_lanczos_beta(n2, dv(r), D.ptr(a_d[i:i + 1]), dv(q), 1, D.ptr(dummy), 0.0, i,
                                         D.ptr(scr), D.ptr(ctl), st), "qs_lanczos_beta")
            yield out(q)


def lanczos_iter(A, v0, m, return_vec_iter=True, copy_v0=True, copy_A=False, eps=None):
    """(E, V[, Q_T iterator]) storing three vectors (_lanczos_utils.py:230-351)."""
    host = not D.is_device_array(v0)
    v0a = np.asanyarray(v0) if host else v0
    n = v0a.shape[0]
    vdt = v0a.dtype if host else D.np_dtype(v0a.dtype)
    op = _DeviceOp(A)
    dtype = np.result_type(op.dtype, vdt)
    if v0a.ndim != 1:
        raise ValueError("expecting array with ndim=1 for initial Lanczos vector.")
    if m >= n:
        raise ValueError("Requested size of Lanczos basis must be smaller then size of original space (e.g. m < n).")
    if eps is None:
        eps = np.finfo(dtype).eps
    q0 = _start_vector(v0, dtype, eps)
    a, b, m_eff, _, ab = _recurrence(op, q0, m, eps)
    m = m_eff
    E, V = eigh_tridiagonal(a[:m], b[:m - 1])
    if return_vec_iter:
        return E, V, _lanczos_vec_iter(op, q0, ab, m, host, dtype)
    return E, V


def lin_comb_Q_T(coeff, Q_T, out=None):
    """v = sum_i coeff[i] Q_T[i] (_lanczos_utils.py:366-425)."""
    coeff = np.asanyarray(coeff)
    if isinstance(Q_T, (np.ndarray, torch.Tensor)):
        host = not D.is_device_array(Q_T)
        qdt = Q_T.dtype if host else D.np_dtype(Q_T.dtype)
        dtype = np.result_type(qdt, coeff.dtype)
        Qd = D.to_device(Q_T, _work_dtype(qdt))
        nk, n = Qd.shape
        cc = int(np.iscomplexobj(coeff))
        cq = int(Qd.is_complex())
        c = D.to_device(np.ascontiguousarray(coeff[:nk], dtype=np.complex128 if cc else np.float64))
        res = torch.empty(n, dtype=torch.complex128 if (cc or cq) else torch.float64, device=D.device())
        dv = lambda t: D.ptr(torch.view_as_real(t) if t.is_complex() else t)
        _lib.call("qs_lanczos_lincomb", n, nk, dv(c), cc, dv(Qd), n, cq, dv(res), D.stream())
    else:
        it = iter(Q_T)
        q = next(it)
        host = not D.is_device_array(q)
        qdt = q.dtype if host else D.np_dtype(q.dtype)
        dtype = np.result_type(qdt, coeff.dtype)
        res = D.to_device(q, np.complex128 if dtype.kind == "c" else np.float64) * complex(coeff[0]) \
            if dtype.kind == "c" else D.to_device(q, np.float64) * float(coeff[0])
        for w, q in zip(coeff[1:], it):
            qd = D.to_device(q, np.complex128 if dtype.kind == "c" else np.float64)
            res.add_(qd, alpha=complex(w) if dtype.kind == "c" else float(w))
    if dtype.kind != "c" and res.is_complex():
        res = res.real
    if out is not None:
        odt = out.dtype if not D.is_device_array(out) else D.np_dtype(out.dtype)
        if odt != dtype:
            raise ValueError("argument 'out' has dtype {}, expecting dtype {}".format(odt, dtype))
        if D.is_device_array(out):
            out.copy_(res.to(out.dtype))
        else:
            out[...] = D.to_host(res).astype(dtype, copy=False)
        return out
    return D.to_host(res).astype(dtype, copy=False) if host else res.to(D.torch_dtype(dtype))


def expm_lanczos(E, V, Q_T, a=1.0, out=None):
    """exp(aA) v0 from a Lanczos decomposition (_expm.py:7-52)."""
    c = V.dot(np.exp(a * E) * V[0, :])
    return lin_comb_Q_T(c, Q_T, out=out)


def _q_block(Q_T):
    """Lanczos rows as one device tensor [m, n] (device tensor, array or an
    iterator of rows such as lanczos_iter's)."""
    if D.is_device_array(Q_T):
        return Q_T
    if isinstance(Q_T, np.ndarray):
        return D.to_device(Q_T)
    rows = [r if D.is_device_array(r) else D.to_device(np.asarray(r)) for r in Q_T]
    return torch.stack(rows, dim=0)


def _apply_block(A, X):
    """A X for a device block X [n, k] on the device: the package's operators
    and device matrices through their own dot, scipy / numpy matrices after
    conversion to a device CSR.  Anything else must return a CUDA tensor from
    ``dot`` of a CUDA tensor (no host round trip)."""
    from ..operators import hamiltonian, quantum_LinearOperator
    if isinstance(A, (hamiltonian, quantum_LinearOperator, DeviceCSR, DeviceDIA)):
        return A.dot(X)
    if isinstance(A, np.ndarray) or hasattr(A, "tocsr"):
        import scipy.sparse as sp
        return to_device_matrix(sp.csr_matrix(A)).dot(X)
    if hasattr(A, "dot"):
        Y = A.dot(X)
        if D.is_device_array(Y):
            return Y
    raise TypeError("operators must be a hamiltonian, quantum_LinearOperator, device or scipy/numpy matrix, "
                    "or an object whose dot maps CUDA tensors to CUDA tensors")


def _block_inner(Q, X, conj=True, xrows=False):
    """W = op(Q) X on the device (csrc/dense.cu, tiled FP64
    panels): Q [m, n] rows, X [n, k] C order or, with xrows, [k, n] rows;
    op = complex conjugate when conj.  Real operands stay real."""
    cplx = Q.is_complex() or X.is_complex()
    dt = torch.complex128 if cplx else torch.float64
    Q = Q.to(dt).contiguous()
    X = X.to(dt).contiguous()
    m, n = Q.shape
    k = X.shape[0] if xrows else X.shape[1]
    W = torch.empty((m, k), dtype=dt, device=D.device())
    scr = D.scratch_doubles(_lib.load().qs_block_inner_scratch_doubles(n, m, k, int(cplx)))
    dv = lambda t: D.ptr(torch.view_as_real(t) if t.is_complex() else t)
    _lib.call("qs_block_inner", n, m, k, dv(Q), n, dv(X), X.shape[1], int(xrows), int(cplx), int(conj), dv(W),
              D.ptr(scr), D.stream())
    return W


def _orthonormalize_rows(Q, m):
    """Q[:m] <- orthonormal rows spanning the same nested subspaces: classical
    Gram-Schmidt applied twice per row against the rows before it, then
    normalisation, on the device (csrc/lanczos.cu).  This is the QR step of
    full_ortho (_lanczos_utils.py:206-209); each row keeps the direction of
    its own component orthogonal to the earlier rows (R has a positive
    diagonal), where LAPACK's Householder QR may flip the sign of a row."""
    n = Q.shape[1]
    cplx = int(Q.is_complex())
    n2 = n * (2 if cplx else 1)
    L = _lib.load()
    st = D.stream()
    ctl = torch.zeros(2, dtype=torch.int32, device=D.device())
    ctl[1] = m
    scr = D.scratch_doubles(L.qs_lanczos_scratch_doubles())
    rscr = D.scratch_doubles(L.qs_lanczos_reorth_scratch_doubles(m))
    nrm = torch.zeros(1, dtype=torch.float64, device=D.device())
    dv = lambda t: D.ptr(torch.view_as_real(t) if t.is_complex() else t)
    for i in range(m):
        if i:
            _lib.check(L.qs_lanczos_reorth(n, cplx, i, dv(Q), n, dv(Q[i]), 2, D.ptr(rscr), D.ptr(ctl), st),
                       "qs_lanczos_reorth")
        _lib.check(L.qs_lanczos_beta(n2, dv(Q[i]), None, dv(Q[i]), 0, D.ptr(nrm), 0.0, i, D.ptr(scr), D.ptr(ctl),
                                     st), "qs_lanczos_beta")
        _lib.check(L.qs_lanczos_scale(n2, dv(Q[i]), D.ptr(nrm), dv(Q[i]), D.ptr(ctl), st), "qs_lanczos_scale")


def FTLM_static_iteration(O_dict, E, V, Q_T, beta=0):
    """One random start of the finite-temperature Lanczos method
    (src/quspin/tools/lanczos/_FTLM.py:10-109): with p(beta, j) = exp(-beta E_j)
    and c[a] = sum_j V[0, j] V[a, j] p(beta, j), returns
    ({key: sum_a c[a] <q_a | O q_0>}, c[0]) for every operator O of O_dict.
    The overlaps <q_a | O q_0> are one product and one block inner product
    per operator on the device."""
    E = np.asarray(D.to_host(E) if D.is_device_array(E) else E)
    V = np.asarray(D.to_host(V) if D.is_device_array(V) else V)
    Q = _q_block(Q_T)
    p = np.exp(-np.outer(np.atleast_1d(beta), E))
    c = np.einsum("j,aj,...j->a...", V[0, :], V, p)
    r = Q[0]
    res = {}
    for key, A in O_dict.items():
        Ar = _apply_block(A, r)
        ov = D.to_host(_block_inner(Q, Ar.reshape(-1, 1))[:, 0])   # <q_a | O q_0>, a = 0..m-1
        res[key] = np.squeeze(np.tensordot(ov, c[:ov.shape[0]], axes=(0, 0)))
    return res, np.squeeze(c[0, ...])


def LTLM_static_iteration(O_dict, E, V, Q_T, beta=0):
    """One random start of the low-temperature Lanczos method
    (src/quspin/tools/lanczos/_LTLM.py:9-139): Krylov states whose Boltzmann
    weight at the smallest beta is below machine epsilon are dropped (nv);
    the operator's matrix in the kept Lanczos basis, Ome[i, j] =
    <q_j | O q_i>, comes from one block product O Q^T (all nv columns in one
    sparse pass) and one dense [nv, n] x [n, nv] product on the device, is
    rotated to the Ritz basis and weighted by V[0, j] exp(-beta E_j / 2) on
    both sides; the identity term is sum_j V[0, j]^2 exp(-beta E_j)."""
    E = np.asarray(D.to_host(E) if D.is_device_array(E) else E)
    V = np.asarray(D.to_host(V) if D.is_device_array(V) else V)
    Q = _q_block(Q_T)
    nv = E.size
    beta = np.atleast_1d(beta)
    p = np.exp(-E * beta.min()) * np.abs(V[0, :]).max()
    mask = p < np.finfo(p.dtype).eps
    if np.any(mask):
        nv = int(np.argmax(mask))
    Qn = Q[:nv]
    X = Qn.transpose(0, 1).contiguous()                            # [n, nv]: columns q_i
    Vn = V[:nv, :nv].copy()
    pp = np.exp(-np.outer(E[:nv], beta / 2.0))
    cc = np.einsum("j,j...->j...", Vn[0, :], pp)
    res = {}
    for key, A in O_dict.items():
        AX = _apply_block(A, X)                                    # [n, nv]: columns O q_i
        Ome = D.to_host(_block_inner(Qn, AX).transpose(0, 1))     # [i, j] = <q_j | O q_i>
        A_diag = Vn.T.dot(Ome.dot(Vn))
        res[key] = np.squeeze(np.einsum("j...,l...,jl->...", cc, cc, A_diag))
    p = np.exp(-np.outer(E[:nv], beta))
    Id = np.einsum("j,j...->...", Vn[0, :] ** 2, p)
    return res, np.squeeze(Id)
