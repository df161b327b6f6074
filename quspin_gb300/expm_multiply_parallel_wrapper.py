"""GPU replacement for parallel-sparse-tools' ``expm_multiply_parallel_wrapper``.

QuSpin 1.0.1's ``ExpmMultiplyParallel`` (its Python body is the viewcode page
docs/modules/parallel_sparse_tools/expm_multiply_parallel_core/
expm_multiply_parallel_core.html) reaches native code through four functions
of the un-vendored ``parallel_sparse_tools.expm_multiply_parallel_core.
expm_multiply_parallel_wrapper`` module: the shift and norm at construction
(html :96-103) and the Taylor loop in ``dot`` (html :248-272).  This module
provides the same four functions with the same arguments, backed by
libqsgpu.so, so a maintainer who keeps QuSpin's Python and swaps only its
native layer installs it under that module name::

    import sys, quspin_gb300.expm_multiply_parallel_wrapper as w
    sys.modules["parallel_sparse_tools.expm_multiply_parallel_core."
                "expm_multiply_parallel_wrapper"] = w

Arguments are host numpy arrays, as the reference passes them; ``v`` is
updated in place.  The matrix is copied to the device once per distinct
(indptr, indices, data) triple (a small cache keyed by the arrays' identity
and shape), so repeated ``dot`` calls on one operator stream it from HBM; a
matrix whose arrays are changed in place needs ``clear_cache()`` first.
``PRECISION`` selects the Taylor-term arithmetic: ``"double"`` (float pairs,
the library default) or ``"ieee"`` (IEEE double products).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _device as D
from . import _lib
from .sparse import DeviceCSR

PRECISION = "double"
_CACHE = {}


def clear_cache():
    """Forget the device copies of the matrices seen so far."""
    _CACHE.clear()


def _device_csr(indptr, indices, data):
    key = (id(indptr), id(indices), id(data), len(indptr), len(indices), np.asarray(data).dtype.str)
    ent = _CACHE.get(key)
    if ent is not None and ent[0] is indptr and ent[1] is indices and ent[2] is data:
        return ent[3]
    data = np.asarray(data)
    dt = np.dtype(np.complex128 if np.iscomplexobj(data) else np.float64)
    n = len(indptr) - 1
    ip = D.to_device(np.ascontiguousarray(indptr, dtype=np.int32 if len(indices) < 2**31 - 1 else np.int64))
    M = DeviceCSR(ip, D.to_device(np.ascontiguousarray(indices, dtype=np.int32)),
                  D.to_device(np.ascontiguousarray(data, dtype=dt)), (n, n), dt)
    if len(_CACHE) >= 4:
        _CACHE.clear()
    _CACHE[key] = (indptr, indices, data, M)
    return M


def _wrapper_csr_trace(indptr, indices, data):
    """Trace of the CSR matrix (html :96-98)."""
    M = _device_csr(indptr, indices, data)
    t = M.trace()
    return t if np.iscomplexobj(np.asarray(data)) else float(np.real(t))


def _wrapper_csr_1_norm(indptr, indices, data, shift):
    """max_c sum_r |A + shift I|[r, c] (html :101-103)."""
    return _device_csr(indptr, indices, data).onenorm(complex(shift))


def _wrapper_expm_multiply(indptr, indices, data, s, m_star, tol, mu, a, v, work):
    """v <- e^{aA} v in place by s substeps of at most m_star Taylor terms with
    shift mu and stopping tolerance tol (html :248-260); v is [n] or [n, k]
    (C order); work (2 v.size elements) is accepted as the reference does and
    the device keeps its own term buffers."""
    M = _device_csr(indptr, indices, data)
    n = M.shape[0]
    v = np.asarray(v)
    if v.shape[0] != n:
        raise ValueError("dimension mismatch")
    nvec = 1 if v.ndim == 1 else v.shape[1]
    s, m_star = int(s), int(m_star)
    a, mu = complex(a), complex(mu)
    F = D.to_device(np.ascontiguousarray(v, dtype=np.complex128)).reshape(n, nvec).contiguous()
    if PRECISION == "ieee":
        op, btype = M, _lib.C128
    else:
        op, btype = M.paired(), _lib.CPF
    m = max(m_star, 1)
    consts = D.to_device(np.array([a / (s * (j + 1)) for j in range(m)] + [np.exp(a * mu / s), 1.0],
                                  dtype=np.complex128))
    wk = torch.empty(2 * n * nvec, dtype=torch.complex128, device=D.device())
    ctl = torch.zeros(_lib.load().qs_expm_ctl_bytes() // 8 + 1, dtype=torch.int64, device=D.device())
    from .tune import tune_taylor
    group = tune_taylor(op, nvec, btype)
    _lib.call("qs_expm_multiply", n, op.nnz, D.ptr(op.indptr), op.idx64, D.ptr(op.indices), D.ptr(op.data),
              op.vcode, D.ptr(F), nvec, s, m_star, float(tol), mu.real, mu.imag, D.ptr(consts[:m]),
              D.ptr(consts[m:m + 1]), D.ptr(consts[m + 1:]), D.ptr(wk), btype, D.ptr(ctl), group, D.stream())
    if int(ctl.view(torch.int32)[12].item()):
        raise RuntimeError("libqsgpu: a bounded device wait gave up in the Taylor loop")
    res = D.to_host(F).reshape(v.shape)
    v[...] = res if np.iscomplexobj(v) else res.real


_wrapper_expm_multiply_batch = _wrapper_expm_multiply
