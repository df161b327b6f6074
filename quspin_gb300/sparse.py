"""Device-resident sparse matrices (CSR and DIA) and their products.

``DeviceCSR`` holds the canonical CSR that the GPU Hamiltonian builder
produces (int32 or int64 ``indptr``, int32 ``indices``, values in one of
float32/float64/complex64/complex128) and applies it with the kernels of
``csrc/sparse.cu`` -- the GPU counterpart of parallel-sparse-tools' ``_matvec``
(docs/modules/parallel_sparse_tools/matvec/matvec_core.html:146-201 in the
reference).  ``DeviceDIA`` is the diagonal storage the reference uses when every
term of an operator is diagonal (src/quspin/basis/base.py:299-304).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from . import _device as D
from . import _lib


# Arithmetic of the CSR product for float64 / complex128 vectors: "double"
# (values and x as float pairs, FP32-instruction products with 48-bit
# significands, csrc/spmv_lp.cu; GB300's FP64 pipe is a small fraction of its
# FP32 rate) or "ieee" (IEEE double products, csrc/sparse.cu).  float32 /
# complex64 vectors always use FP32 products.
SPMV_PRECISION = "double"


def set_spmv_precision(precision):
    """Module default for DeviceCSR.matvec_into; returns the previous one."""
    global SPMV_PRECISION
    if precision not in ("double", "ieee"):
        raise ValueError("precision must be 'double' or 'ieee'")
    old, SPMV_PRECISION = SPMV_PRECISION, precision
    return old


def result_dtype(*dtypes):
    return np.result_type(*[np.dtype(d) for d in dtypes])


class DeviceCSR:
    format = "csr"
    # products after which matvec_into switches to the coded float-pair operand
    CODE_AFTER_PRODUCTS = 64

    def __init__(self, indptr, indices, data, shape, dtype):
        self.indptr = indptr
        self.indices = indices
        self.data = data
        self.shape = (int(shape[0]), int(shape[1]))
        self.dtype = np.dtype(dtype)
        self.idx64 = 1 if indptr.dtype == torch.int64 else 0
        self._nnz = None

    @property
    def nnz(self):
        if self._nnz is None:
            self._nnz = int(self.indptr[-1].item()) if self.shape[0] > 0 else 0
        return self._nnz

    @property
    def vcode(self):
        """Element type code of the values for the C ABI."""
        return D.code(self.dtype)

    def paired(self, coded=True):
        """The values split into float pairs (``PairedCSR``; coded when the
        matrix has at most 256 distinct values and ``coded``), cached."""
        key = "_paired_coded" if coded else "_paired"
        p = self.__dict__.get(key)
        if p is None:
            p = PairedCSR(self, coded=coded)
            self.__dict__[key] = p
        return p

    @classmethod
    def from_scipy(cls, A, dtype=None):
        A = sp.csr_matrix(A)
        if dtype is not None:
            A = A.astype(dtype)
        if not A.has_canonical_format:
            A = A.copy()
            A.sum_duplicates()
        dt = np.dtype(A.dtype)
        if dt not in D.SUPPORTED:
            dt = result_dtype(dt, np.float64)
            A = A.astype(dt)
        ip = A.indptr.astype(np.int32 if A.nnz < 2**31 - 1 else np.int64)
        return cls(D.to_device(ip), D.to_device(A.indices.astype(np.int32)), D.to_device(A.data),
                   A.shape, dt)

    def tocsr(self):
        """Host scipy.sparse.csr_matrix copy."""
        return sp.csr_matrix((D.to_host(self.data), D.to_host(self.indices), D.to_host(self.indptr)),
                             shape=self.shape)

    def astype(self, dtype):
        dtype = np.dtype(dtype)
        if dtype == self.dtype:
            return self
        return DeviceCSR(self.indptr, self.indices, self.data.to(D.torch_dtype(dtype)), self.shape, dtype)

    def _pair_scratch(self, count):
        """Device scratch for x split into float pairs (count doubles) and
        its norm word."""
        sc = self.__dict__.get("_xs")
        if sc is None or sc[0].numel() < 2 * count:
            sc = (torch.empty(max(2 * count, 2), dtype=torch.float32, device=D.device()),
                  torch.zeros(1, dtype=torch.int64, device=D.device()))
            self._xs = sc
        return sc

    def _spmv_operand(self):
        """The float-pair operand of the next product: plain pairs for the
        first CODE_AFTER_PRODUCTS products of a matrix, then the coded form
        (one sort of the values, worth it for a reused matrix; at once when
        a Taylor operand exists), with the codes packed into the column words
        where that applies."""
        P = self.__dict__.get("_paired_coded")
        if P is None:
            self._nprod = self.__dict__.get("_nprod", 0) + 1
            P = self.paired(coded=self._nprod > self.CODE_AFTER_PRODUCTS)
        Pk = P.packed() if P.coded else None
        return P if Pk is None else Pk

    def matvec_into(self, x, y, a=1.0, overwrite=True, group=None, precision=None, operand=None):
        """y (=|+=) a * A x on device tensors of the result dtype.  group:
        launch shape code (None: the autotuned one for this matrix and
        operand form); precision: "double" / "ieee" for float64 / complex128
        vectors (None: the module default); operand: the float-pair operand
        to use (None: the matrix's current one; the tuner pins it)."""
        n = self.shape[0]
        nvec = 1 if x.dim() == 1 else x.shape[1]
        xt = D.np_dtype(x.dtype)
        prec = SPMV_PRECISION if precision is None else precision
        paired = (prec == "double" and xt in (np.dtype(np.float64), np.dtype(np.complex128))
                  and not (self.dtype.kind == "c" and xt.kind != "c"))
        P = (operand if operand is not None else self._spmv_operand()) if paired else None
        if group is None:
            from .tune import tune_spmv
            group = tune_spmv(self, nvec, xt, prec, operand=P)
        a = complex(a)
        if paired:
            xs, nrm = self._pair_scratch(x.numel() * (2 if xt.kind == "c" else 1))
            _lib.call("qs_csr_matvec_pairs", n, self.nnz, D.ptr(self.indptr), self.idx64, D.ptr(P.indices),
                      D.ptr(P.data), P.vcode, D.ptr(x), D.code(xt), D.ptr(y), nvec, a.real, a.imag,
                      int(bool(overwrite)), int(group), D.ptr(xs), D.ptr(nrm), D.stream())
            return y
        _lib.call("qs_csr_matvec", n, self.nnz, D.ptr(self.indptr), self.idx64, D.ptr(self.indices),
                  D.ptr(self.data), D.code(self.dtype), D.ptr(x), D.code(xt), D.ptr(y), nvec, a.real, a.imag,
                  int(bool(overwrite)), int(group), D.stream())
        return y

    def dot(self, V, out=None, a=1.0, overwrite_out=True):
        return _apply(self, V, out, a, overwrite_out)

    def _conj_transpose_sorted(self):
        """A^H by one device sort of the (column, row) keys of the stored
        entries (canonical input: no duplicates to sum, no zeros to drop)."""
        n, nnz = self.shape[0], self.nnz
        dev = D.device()
        counts = (self.indptr[1:] - self.indptr[:-1]).to(torch.int64)
        rows = torch.repeat_interleave(torch.arange(n, dtype=torch.int64, device=dev), counts)
        cols = self.indices[:nnz].to(torch.int64)
        order = torch.argsort(cols * n + rows, stable=True)
        ccount = torch.bincount(cols, minlength=n)
        indptr = torch.zeros(n + 1, dtype=self.indptr.dtype, device=dev)
        indptr[1:] = torch.cumsum(ccount, 0).to(self.indptr.dtype)
        data = self.data[:nnz][order]
        if self.dtype.kind == "c":
            data = data.conj().resolve_conj()
        return DeviceCSR(indptr, rows[order].to(torch.int32), data.contiguous(), self.shape, self.dtype)

    def conj_transpose(self):
        """A^H as a canonical device CSR (built on the device)."""
        n = self.shape[0]
        if self.shape[0] != self.shape[1]:
            raise ValueError("square matrices only")
        L = _lib.load()
        st = D.stream()
        vt = D.code(self.dtype)
        cnt = torch.zeros(n + 1, dtype=torch.int64, device=D.device())
        _lib.call("qs_csr_t_count", n, D.ptr(self.indptr), self.idx64, D.ptr(self.indices), D.ptr(cnt), st)
        scr = torch.empty(max(L.qs_scan_scratch_elems(n), 1), dtype=torch.int64, device=D.device())
        _lib.call("qs_scan_inclusive_i64", D.ptr(cnt[1:]), n, D.ptr(scr), st)
        nnz = self.nnz
        keys = torch.empty(max(nnz, 1), dtype=torch.int64, device=D.device())
        vals = torch.empty(max(nnz, 1), dtype=D.torch_dtype(self.dtype), device=D.device())
        cursor = torch.zeros(n, dtype=torch.int64, device=D.device())
        _lib.call("qs_csr_t_fill", vt, n, D.ptr(self.indptr), self.idx64, D.ptr(self.indices), D.ptr(self.data),
                  D.ptr(cnt), D.ptr(cursor), D.ptr(keys), D.ptr(vals), st)
        mcount = torch.empty(n, dtype=torch.int64, device=D.device())
        err = D.err_flag()
        _lib.call("qs_csr_merge", vt, n, D.ptr(cnt), D.ptr(cursor), D.ptr(keys), D.ptr(vals), None, D.ptr(mcount),
                  D.ptr(err), st)
        if int(err.item()) & 8:
            # a column with more than 512 entries: the merge kernel's per-row
            # sort does not take it, so sort the (column, row) keys instead
            return self._conj_transpose_sorted()
        _lib.call("qs_scan_inclusive_i64", D.ptr(mcount), n, D.ptr(scr), st)
        nnz2 = int(mcount[-1].item()) if n else 0
        indptr = torch.empty(n + 1, dtype=self.indptr.dtype, device=D.device())
        indices = torch.empty(max(nnz2, 1), dtype=torch.int32, device=D.device())
        data = torch.empty(max(nnz2, 1), dtype=D.torch_dtype(self.dtype), device=D.device())
        _lib.call("qs_csr_compact", vt, n, D.ptr(cnt), D.ptr(keys), D.ptr(vals), D.ptr(mcount), D.ptr(indptr),
                  self.idx64, D.ptr(indices), D.ptr(data), st)
        return DeviceCSR(indptr, indices[:nnz2], data[:nnz2], self.shape, self.dtype)

    def trace(self):
        if self.dtype not in (np.dtype(np.float64), np.dtype(np.complex128)):
            return self.astype(result_dtype(self.dtype, np.float64)).trace()
        out = D.zeros(2, np.float64)
        scr = D.scratch_doubles(_lib.load().qs_reduce_scratch_doubles())
        _lib.call("qs_csr_trace", self.shape[0], D.ptr(self.indptr), self.idx64, D.ptr(self.indices),
                  D.ptr(self.data), int(self.dtype.kind == "c"), D.ptr(out), D.ptr(scr), D.stream())
        o = out.cpu().numpy()
        return complex(o[0], o[1]) if self.dtype.kind == "c" else float(o[0])

    def onenorm(self, shift=0.0):
        """max_c sum_r |A + shift I|[r, c]."""
        if self.dtype not in (np.dtype(np.float64), np.dtype(np.complex128)):
            return self.astype(result_dtype(self.dtype, np.float64)).onenorm(shift)
        shift = complex(shift)
        out = D.zeros(1, np.float64)
        col = D.scratch_doubles(self.shape[0])
        scr = D.scratch_doubles(_lib.load().qs_reduce_scratch_doubles())
        _lib.call("qs_csr_1_norm", self.shape[0], D.ptr(self.indptr), self.idx64, D.ptr(self.indices),
                  D.ptr(self.data), int(self.dtype.kind == "c"), shift.real, shift.imag, D.ptr(out), D.ptr(col),
                  D.ptr(scr), D.stream())
        return float(out.item())


class DeviceDIA:
    format = "dia"

    def __init__(self, offsets, data, shape, dtype):
        self.offsets = offsets      # int64 [ndiag] device
        self.data = data            # [ndiag, ldd] device
        self.shape = (int(shape[0]), int(shape[1]))
        self.dtype = np.dtype(dtype)

    @classmethod
    def from_diagonal(cls, diag, dtype):
        n = diag.shape[0]
        return cls(D.to_device(np.zeros(1, np.int64)), diag.reshape(1, n).contiguous(), (n, n), dtype)

    @classmethod
    def from_scipy(cls, A, dtype=None):
        A = sp.dia_matrix(A)
        if dtype is not None:
            A = A.astype(dtype)
        return cls(D.to_device(A.offsets.astype(np.int64)), D.to_device(np.ascontiguousarray(A.data)),
                   A.shape, A.dtype)

    @property
    def nnz(self):
        return int(self.data.numel())

    def tocsr(self):
        return sp.dia_matrix((D.to_host(self.data), D.to_host(self.offsets)), shape=self.shape).tocsr()

    def astype(self, dtype):
        dtype = np.dtype(dtype)
        if dtype == self.dtype:
            return self
        return DeviceDIA(self.offsets, self.data.to(D.torch_dtype(dtype)), self.shape, dtype)

    def matvec_into(self, x, y, a=1.0, overwrite=True, group=0):
        n = self.shape[0]
        nvec = 1 if x.dim() == 1 else x.shape[1]
        a = complex(a)
        _lib.call("qs_dia_matvec", n, int(self.offsets.numel()), D.ptr(self.offsets), int(self.data.shape[1]),
                  D.ptr(self.data), D.code(self.dtype), D.ptr(x), D.code(D.np_dtype(x.dtype)), D.ptr(y), nvec,
                  a.real, a.imag, int(bool(overwrite)), D.stream())
        return y

    def dot(self, V, out=None, a=1.0, overwrite_out=True):
        return _apply(self, V, out, a, overwrite_out)

    def trace(self):
        return self.tocsr().diagonal().sum()


def value_codes(src, table=256):
    """The coded form of a value array: (vals, codes, distinct) with vals the
    table padded with zeros to ``table`` entries (float64 [table], or
    [table, 2] real / imaginary parts for complex src), codes uint8 with
    vals[codes] == src exactly, or None when src has more than ``table``
    distinct values (or a NaN).  Only one-dimensional sorts: complex values
    are coded by the pair of their real- and imaginary-part codes."""
    if src.numel() == 0 or bool(torch.isnan(torch.view_as_real(src) if src.is_complex() else src).any()):
        return None
    if src.is_complex():
        ri = torch.view_as_real(src)
        ur, cr = torch.unique(ri[:, 0], return_inverse=True)
        ui, ci = torch.unique(ri[:, 1], return_inverse=True)
        if ur.numel() > table * table or ui.numel() > table * table:
            return None
        up, inv = torch.unique(cr.to(torch.int64) * ui.numel() + ci.to(torch.int64), return_inverse=True)
        if up.numel() > table:
            return None
        vals = torch.zeros(table, 2, dtype=torch.float64, device=src.device)
        vals[:up.numel(), 0] = ur[up // ui.numel()]
        vals[:up.numel(), 1] = ui[up % ui.numel()]
        distinct = int(up.numel())
    else:
        uniq, inv = torch.unique(src, return_inverse=True)
        if uniq.numel() > table:
            return None
        vals = torch.zeros(table, dtype=torch.float64, device=src.device)
        vals[:uniq.numel()] = uniq
        distinct = int(uniq.numel())
    return vals, inv.reshape(-1).to(torch.uint8), distinct


class PairedCSR:
    """A DeviceCSR whose values are kept as float pairs hi + lo, the operand
    form of the paired-single kernels (csrc/expm_lp.cu, csrc/spmv_lp.cu).
    Shares indptr and indices with its source.

    With ``coded`` (the default) and at most 256 distinct values (int32
    indices), the values are stored as a table of 256 pairs followed by one
    code byte per nonzero (type codes PF8 / CPF8): the kernels read 1 byte
    of value stream per nonzero instead of 8 or 16, with the same pairs and
    the same arithmetic, so the results are bit-identical.  Otherwise one
    pair per nonzero (PF / CPF)."""

    format = "csr"
    TABLE = 256

    def __init__(self, M, coded=True):
        self.indptr, self.indices, self.shape, self.idx64 = M.indptr, M.indices, M.shape, M.idx64
        self._nnz = M.nnz
        self.complex = M.dtype.kind == "c"
        self.dtype = np.dtype(np.complex128 if self.complex else np.float64)
        src = M.data.to(D.torch_dtype(self.dtype)).contiguous()
        self.coded = False
        if coded and not self.idx64 and src.numel() > 0 and self._encode(src):
            return
        self._plain(src)

    def _plain(self, src):
        count = src.numel() * (2 if self.complex else 1)
        self.data = torch.empty(max(2 * count, 2), dtype=torch.float32, device=D.device())
        if count:
            _lib.call("qs_split_pairs", count, D.ptr(src), D.ptr(self.data), D.stream())
        self.coded = False

    def _encode(self, src):
        coded = value_codes(src, self.TABLE)
        if coded is None:
            return False
        vals, codes, distinct = coded
        count = vals.numel()
        tbytes = count * 8                       # one float pair (8 bytes) per double
        buf = torch.empty(tbytes + ((src.numel() + 15) // 16) * 16, dtype=torch.uint8, device=D.device())
        _lib.call("qs_split_pairs", count, D.ptr(vals), D.ptr(buf), D.stream())
        buf[tbytes:tbytes + src.numel()].copy_(codes)
        self.data = buf
        self.coded = True
        self.distinct = distinct
        return True

    def packed(self):
        """The PackedCodedCSR form of this coded operand (cached), or None
        when it does not apply (plain values, int64 indices, >= 2^23 columns)."""
        if not self.coded or self.idx64 or self.shape[1] >= PackedCodedCSR.MAX_COLS:
            return None
        p = self.__dict__.get("_packed")
        if p is None:
            p = PackedCodedCSR(self)
            self._packed = p
        return p

    @property
    def nnz(self):
        return self._nnz

    @property
    def vcode(self):
        if self.coded:
            return _lib.CPF8 if self.complex else _lib.PF8
        return _lib.CPF if self.complex else _lib.PF

    @property
    def value_bytes(self):
        """Bytes of value stream per nonzero the kernels read."""
        return 1 if self.coded else (16 if self.complex else 8)

    def refresh(self, data):
        """Re-split new values (same pattern) into a one-pair-per-nonzero
        buffer (a coded operand becomes plain)."""
        src = data.to(D.torch_dtype(self.dtype)).contiguous()
        if self.coded:
            self._plain(src)
            return
        count = src.numel() * (2 if self.complex else 1)
        _lib.call("qs_split_pairs", count, D.ptr(src), D.ptr(self.data), D.stream())


class PackedCodedCSR:
    """A coded PairedCSR with each nonzero's code byte packed into the low 8
    bits of its column word (col << 8 | code, type codes PF8P / CPF8P): the
    single-vector Taylor term (csrc/expm_st.cu) and the SpMV then read one
    4-byte word per nonzero instead of a 4-byte index and a 1-byte code.
    ``data`` holds the 256-entry pair table only; ``indices`` is zero-padded
    to a multiple of four words plus four (``padded``), for the kernels that
    load the words four at a time.  Needs fewer than 2^23 columns and int32
    indices; built from a coded PairedCSR (``PairedCSR.packed()``)."""

    format = "csr"
    MAX_COLS = 1 << 23

    def __init__(self, P):
        if not P.coded or P.idx64 or P.shape[1] >= self.MAX_COLS:
            raise ValueError("the packed form needs a coded operand with int32 indices and < 2^23 columns")
        self.indptr, self.shape, self.idx64 = P.indptr, P.shape, 0
        self._nnz = P.nnz
        self.complex, self.dtype, self.distinct = P.complex, P.dtype, P.distinct
        tbytes = PairedCSR.TABLE * (16 if P.complex else 8)
        nnz = P.nnz
        codes = P.data[tbytes:tbytes + nnz].to(torch.int32)
        # zero words up to the next multiple of four and four more: the kernels
        # that read the words in aligned groups of four stay inside the buffer
        words = torch.zeros((nnz + 3) // 4 * 4 + 4, dtype=torch.int32, device=D.device())
        torch.bitwise_or(torch.bitwise_left_shift(P.indices[:nnz].to(torch.int32), 8), codes, out=words[:nnz])
        del codes
        self.indices = words
        self.padded = True
        self.data = P.data[:tbytes].clone()
        self.coded = True

    @property
    def nnz(self):
        return self._nnz

    @property
    def vcode(self):
        return _lib.CPF8P if self.complex else _lib.PF8P

    @property
    def value_bytes(self):
        """Bytes of value stream per nonzero beyond the 4-byte column word."""
        return 0


def to_device_matrix(A, dtype=None):
    if isinstance(A, (DeviceCSR, DeviceDIA)):
        return A if dtype is None else A.astype(dtype)
    if sp.issparse(A) and A.format == "dia":
        return DeviceDIA.from_scipy(A, dtype)
    return DeviceCSR.from_scipy(A, dtype)


def _apply(M, V, out, a, overwrite_out):
    """matvec with numpy-or-device operands; numpy in -> numpy out."""
    host = not D.is_device_array(V)
    rdt = result_dtype(M.dtype, V.dtype if host else D.np_dtype(V.dtype))
    if rdt not in D.SUPPORTED:
        rdt = result_dtype(rdt, np.float64)
    if np.iscomplexobj(np.zeros(1, rdt)) is False and np.iscomplexobj(a):
        rdt = result_dtype(rdt, np.complex64)
    x = D.to_device(V, rdt)
    if out is None:
        y = torch.empty_like(x)
        overwrite_out = True
    else:
        y = out if D.is_device_array(out) else D.to_device(out, rdt)
    M.matvec_into(x, y, a=a, overwrite=overwrite_out)
    if host:
        res = D.to_host(y)
        if out is not None and not D.is_device_array(out):
            out[...] = res
            return out
        return res
    return y
