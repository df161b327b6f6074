"""``ExpmMultiplyParallel``: e^{aA} v by the truncated Taylor method on the GPU.

Drop-in for QuSpin 1.0.1's ``quspin.tools.expm_multiply_parallel``
(src/quspin/tools/evolution.py:11-16 re-exports the class whose Python body is
docs/modules/parallel_sparse_tools/expm_multiply_parallel_core/
expm_multiply_parallel_core.html:115-463).  Same constructor, ``set_a``,
``dot`` and properties; the same dtype rule, tolerance (eps(dtype)/2),
shift mu = tr(A)/n, exact 1-norm of A - mu I and (m*, s) selection.  The
trace, 1-norm and every Taylor term run in ``csrc/sparse.cu`` /
``csrc/expm.cu`` / ``csrc/expm_lp.cu``; one ``dot`` issues about s (m* + 2)
launches and never synchronises with the host until the result is read.

``precision`` chooses the arithmetic of the Taylor terms; the partial sum F,
mu, the coefficients and the stopping test are IEEE double in all three:

* ``"double"`` (default): A's values and the term vectors B are float pairs
  hi + lo (48-bit significands) and every per-nonzero product runs in FP32
  instructions (csrc/pairf.cuh).  GB300's FP64 pipe is a small fraction of
  its FP32 rate, so this is the fast form of the double-precision method;
  its state error against IEEE double is of order 1e-14.
* ``"ieee"``: every product in IEEE double (the reference's arithmetic).
* ``"mixed"``: complex64 B and float32 / complex64 values with FP32 row
  sums (half the bytes per term); state error of order 1e-7.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from .. import _device as D
from .. import _lib
from ..sparse import DeviceCSR, DeviceDIA, to_device_matrix
from ._partition import LazyOperatorNormInfo, fragment_3_1


def _as_device_csr(A):
    from ..operators import hamiltonian
    if isinstance(A, hamiltonian):
        return A.tocsr_gpu()
    if isinstance(A, DeviceCSR):
        return A
    if isinstance(A, DeviceDIA):
        return DeviceCSR.from_scipy(A.tocsr(), A.dtype)
    if isinstance(A, np.ndarray):
        A = sp.csr_matrix(A)
    return to_device_matrix(sp.csr_matrix(A))


class ExpmMultiplyParallel:
    """Truncated-Taylor action of e^{aA} (html :115-260).  Beyond the
    reference's arguments: ``precision`` (see the module docstring) and
    ``predictor``, a learned.NormRatioPredictor for the (m*, s) selection
    (see ``set_predictor``)."""

    def __init__(self, A, a=1.0, dtype=None, copy=False, precision="double", predictor=None):
        if np.array(a).ndim == 0:
            self._a = a
        else:
            raise ValueError("a must be scalar value.")
        if A.shape[0] != A.shape[1]:
            raise ValueError("A must be a square matrix.")
        self._Ad = _as_device_csr(A)
        if copy:
            self._Ad = DeviceCSR(self._Ad.indptr.clone(), self._Ad.indices.clone(), self._Ad.data.clone(),
                                 self._Ad.shape, self._Ad.dtype)
        if precision not in ("double", "ieee", "mixed"):
            raise ValueError("precision must be 'double', 'ieee' or 'mixed'")
        self._precision = precision
        Adt = self._Ad.dtype
        a_dtype_min = np.min_scalar_type(self._a)
        if dtype is None:
            self._dtype = np.result_type(Adt, a_dtype_min, np.float64)
        else:
            min_dtype = np.result_type(Adt, a_dtype_min, np.float32)
            if not np.can_cast(min_dtype, dtype):
                raise ValueError("dtype not sufficient to represent a*A to at least float32 precision.")
            self._dtype = np.dtype(dtype)
        self._tol = np.array(np.finfo(self._dtype).eps / 2, dtype=np.finfo(self._dtype).eps.dtype)
        n = self._Ad.shape[0]
        tr = self._Ad.trace() if n else 0.0
        self._mu = np.array(tr / n if n else 0.0, dtype=self._dtype)
        self._A_1_norm = self._Ad.onenorm(-complex(self._mu)) if n else 0.0
        self._AH = None
        self._mixed = None
        self._bufs = {}
        self.fallbacks = 0
        self._predictor = predictor
        self._calculate_partition()

    @property
    def a(self):
        return self._a

    @property
    def precision(self):
        return self._precision

    @precision.setter
    def precision(self, p):
        if p not in ("double", "ieee", "mixed"):
            raise ValueError("precision must be 'double', 'ieee' or 'mixed'")
        self._precision = p

    @property
    def A(self):
        """Host scipy.sparse.csr_matrix copy of the exponentiated matrix."""
        return self._Ad.tocsr()

    @property
    def A_device(self):
        return self._Ad

    @property
    def m_star(self):
        return self._m_star

    @property
    def s(self):
        return self._s

    def set_a(self, a, dtype=None):
        """New scale a (html :216-260)."""
        if np.array(a).ndim == 0:
            self._a = a
            a_dtype_min = np.min_scalar_type(self._a)
            if dtype is None:
                self._dtype = np.result_type(self._Ad.dtype, a_dtype_min, np.float64)
            else:
                min_dtype = np.result_type(self._Ad.dtype, a_dtype_min, np.float32)
                if not np.can_cast(min_dtype, dtype):
                    raise ValueError("dtype not sufficient to represent a*A to at least float32 precision.")
                self._dtype = np.dtype(dtype)
            self._tol = np.array(np.finfo(self._dtype).eps / 2, dtype=np.finfo(self._dtype).eps.dtype)
            self._mu = np.array(self._mu, dtype=self._dtype)
            self._calculate_partition()
        else:
            raise ValueError("expecting 'a' to be scalar.")

    def set_partition(self, m_star, s):
        """Use an externally chosen (m*, s) (the learned predictor's entry)."""
        self._m_star, self._s = int(m_star), max(int(s), 1)

    # -- (m*, s) ---------------------------------------------------------------
    def _shifted_apply(self, conj):
        """Device map X -> a (A - mu I) X (or its adjoint) on [n, k] blocks."""
        a = complex(self._a)
        mu = complex(self._mu)
        if conj:
            a, mu = np.conj(a), np.conj(mu)
            if self._AH is None:
                self._AH = self._Ad.conj_transpose()
            M = self._AH
        else:
            M = self._Ad

        def f(X):
            x2 = X.reshape(X.shape[0], -1).to(torch.complex128).contiguous()
            y = torch.empty_like(x2)
            M.matvec_into(x2, y, a=a, overwrite=True)
            y.sub_(x2, alpha=a * mu)
            return y.reshape(X.shape)
        return f

    def set_predictor(self, predictor):
        """Choose (m*, s) with a learned.NormRatioPredictor whenever the
        estimator branch of the selection would run (None: always the plain
        onenormest selection).  A product whose Taylor loop then runs a
        substep through all m* terms without the stopping test firing is
        recomputed with the plain selection (``fallbacks`` counts these)."""
        self._predictor = predictor
        self._calculate_partition()

    @property
    def partition_source(self):
        """'plain' (exact norm or onenormest, as the reference) or 'learned'."""
        return self.__dict__.get("_partition_source", "plain")

    @property
    def norm_products(self):
        """Products with the matrix the last (m*, s) selection made."""
        info = self.__dict__.get("_norm_info")
        return 0 if info is None else int(getattr(info, "matvecs", 0))

    def _calculate_partition(self, plain=False):
        from ._partition import condition_3_13
        self._partition_source = "plain"
        if np.abs(self._a) * self._A_1_norm == 0:
            self._m_star, self._s = 0, 1
            self._norm_info = None
            return
        pred = None if plain else self.__dict__.get("_predictor")
        one = float(np.abs(self._a) * self._A_1_norm)
        if pred is not None and not condition_3_13(one, 1, 55, 2):
            from ..learned import FixedNormInfo
            f = pred.features(self._A_1_norm, self._Ad.shape[0], self._Ad.nnz, abs(complex(self._mu)))
            r = pred.predict_ratios(f)[0]
            self._norm_info = FixedNormInfo(one, {p: one * x for p, x in zip(pred.P, r)})
            self._m_star, self._s = fragment_3_1(self._norm_info, 1, self._tol, ell=2)
            self._partition_source = "learned"
            return
        self._norm_info = LazyOperatorNormInfo(self._shifted_apply(False), self._shifted_apply(True),
                                               self._Ad.shape[0], self._A_1_norm, self._a,
                                               np.dtype(np.complex128), ell=2,
                                               device=(torch.complex128, D.device()))
        self._m_star, self._s = fragment_3_1(self._norm_info, 1, self._tol, ell=2)

    # -- application -------------------------------------------------------------
    def _mixed_matrix(self):
        if self._mixed is None:
            A = self._Ad
            vt = np.dtype(np.float32) if A.dtype.kind == "f" else np.dtype(np.complex64)
            self._mixed = A.astype(vt)
        return self._mixed

    def _operand(self, nvec=1):
        """(matrix in the value form of the precision, B storage code).  For
        one vector in the float-pair form, the coded operand and its packed
        form (code bytes inside the column words) are both tuned once and the
        faster is kept."""
        if self._precision == "mixed":
            return self._mixed_matrix(), _lib.C64
        if self._precision == "ieee":
            return self._Ad, _lib.C128
        P = self._Ad.paired()
        if nvec != 1:
            return P, _lib.CPF
        pick = self.__dict__.get("_pick")
        if pick is None:
            pick = P
            Pk = P.packed() if P.shape[0] >= 65536 else None
            if Pk is not None:
                from ..tune import tune_taylor
                tune_taylor(P, 1, _lib.CPF)
                tune_taylor(Pk, 1, _lib.CPF)
                key = ("taylor", 1, _lib.CPF)
                t_plain = P.__dict__.get("_tuned_ms", {}).get(key)
                t_pack = Pk.__dict__.get("_tuned_ms", {}).get(key)
                if t_pack is not None and t_plain is not None and t_pack < t_plain:
                    pick = Pk
            self._pick = pick
        return pick, _lib.CPF

    def _buffers(self, n, nvec, btype):
        key = (n, nvec, btype)
        b = self._bufs.get(key)
        if b is None:
            esz_dt = torch.complex64 if btype == _lib.C64 else torch.complex128
            work = torch.empty(2 * n * nvec, dtype=esz_dt, device=D.device())
            ctl = torch.zeros(max(_lib.load().qs_expm_ctl_bytes() // 8, 1) + 1, dtype=torch.int64,
                              device=D.device())
            b = (work, ctl)
            self._bufs = {key: b}
        return b

    def _rownorm(self, n):
        """Row-sum scratch (n double pairs) of the chunk-outer Taylor sweep."""
        r = self.__dict__.get("_rown")
        if r is None or r.numel() < 2 * n:
            r = torch.empty(max(2 * n, 2), dtype=torch.float64, device=D.device())
            self._rown = r
        return r

    # below this many states x vectors a dot replays a captured launch
    # sequence (one graph launch instead of about s (m* + 2) kernel launches)
    GRAPH_MAX_ELEMS = 1 << 18

    def run_device(self, F, tol=None, work=None):
        """In place e^{aA} F for a complex128 device tensor F of shape (n,) or
        (n, k).  Returns F.  No host synchronisation, except with a learned
        (m*, s), where the substep counter is read once to decide on the
        fallback to the plain selection."""
        if self.partition_source != "learned":
            return self._run_device(F, tol, work)
        saved = F.clone()
        self._run_device(F, tol, work)
        if self.nonconverged_substeps:
            self.fallbacks = self.__dict__.get("fallbacks", 0) + 1
            self._calculate_partition(plain=True)
            F.copy_(saved)
            self._run_device(F, tol, work)
        return F

    def _run_device(self, F, tol=None, work=None):
        n = self._Ad.shape[0]
        nvec = 1 if F.dim() == 1 else F.shape[1]
        tol = float(self._tol if tol is None else tol)
        if (work is None and n * nvec <= self.GRAPH_MAX_ELEMS and F.is_contiguous()
                and not torch.cuda.is_current_stream_capturing()):
            return self._run_graph(F, tol)
        M, btype = self._operand(nvec)
        wbuf, ctl = self._buffers(n, nvec, btype)
        if work is not None and btype != _lib.C64:
            wbuf = work          # 16-byte elements: the caller's complex128 work array holds both B buffers
        self._consts = self._launch(F, tol, wbuf, ctl)     # kept alive until the stream reaches it
        self._last_ctl = ctl
        return F

    def _const_table(self):
        """Device table: the m* term coefficients a / (s (j+1)), eta, 1."""
        a = complex(self._a)
        mu = complex(self._mu)
        s, m = int(self._s), int(self._m_star)
        coeff = np.array([a / (s * (j + 1)) for j in range(max(m, 1))], dtype=np.complex128)
        eta = np.exp(a * mu / s)
        return D.to_device(np.concatenate([coeff, [eta, 1.0 + 0j]]).astype(np.complex128))

    def _launch(self, F, tol, wbuf, ctl, consts=None):
        """The launch sequence of one evolution of F (no host synchronisation;
        with a prepared consts table it issues device work only)."""
        n = self._Ad.shape[0]
        nvec = 1 if F.dim() == 1 else F.shape[1]
        mu = complex(self._mu)
        s, m = int(self._s), int(self._m_star)
        M, btype = self._operand(nvec)
        ctl.zero_()
        if consts is None:
            consts = self._const_table()
        cf = consts[:max(m, 1)]
        etap = consts[max(m, 1):max(m, 1) + 1]
        onep = consts[max(m, 1) + 1:]
        from ..tune import tune_taylor
        group = tune_taylor(M, nvec, btype)
        rown = self._rownorm(n) if (btype != _lib.C128 and nvec > 8) else None
        _lib.call("qs_expm_multiply_rows", n, M.nnz, D.ptr(M.indptr), M.idx64, D.ptr(M.indices), D.ptr(M.data),
                  M.vcode, D.ptr(F), nvec, s, m, tol, mu.real, mu.imag, D.ptr(cf), D.ptr(etap),
                  D.ptr(onep), D.ptr(wbuf), btype, D.ptr(ctl), group, D.ptr(rown), D.stream())
        return consts

    def _run_graph(self, F, tol):
        n = self._Ad.shape[0]
        nvec = 1 if F.dim() == 1 else F.shape[1]
        key = (tuple(F.shape), self._precision, tol, complex(self._a), int(self._s), int(self._m_star))
        graphs = self.__dict__.setdefault("_graphs", {})
        ent = graphs.get(key)
        if ent is None:
            _, btype = self._operand(nvec)
            Fg = F.clone()
            wbuf = torch.empty(2 * n * nvec, dtype=torch.complex64 if btype == _lib.C64 else torch.complex128,
                               device=F.device)
            ctl = torch.zeros(max(_lib.load().qs_expm_ctl_bytes() // 8, 1) + 1, dtype=torch.int64,
                              device=F.device)
            consts = self._const_table()
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                self._launch(Fg, tol, wbuf, ctl, consts)  # tuning and first launches outside the capture
            torch.cuda.current_stream().wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._launch(Fg, tol, wbuf, ctl, consts)
            ent = (g, Fg, wbuf, ctl, consts)
            graphs[key] = ent
        g, Fg, _, ctl, _ = ent
        Fg.copy_(F)
        g.replay()
        F.copy_(Fg)
        self._last_ctl = ctl
        return F

    @property
    def nonconverged_substeps(self):
        """Substeps of the last dot that used all m* terms without the
        stopping test firing (reads the device counter)."""
        c = getattr(self, "_last_ctl", None)
        return 0 if c is None else int(c.view(torch.int32)[10].item())

    @property
    def terms_executed(self):
        """Taylor terms executed by the last dot (reads the device counter)."""
        c = getattr(self, "_last_ctl", None)
        if c is None:
            return 0
        return int(c[4].item())

    def dot(self, v, work_array=None, overwrite_v=False, tol=None):
        """e^{aA} v (html :265-374); numpy in -> numpy out, CUDA tensor in ->
        CUDA tensor out (in place when overwrite_v)."""
        host = not D.is_device_array(v)
        if host:
            v = np.asarray(v)
        if v.ndim > 2:
            raise ValueError("array must have ndim <= 2.")
        if v.shape[0] != self._Ad.shape[1]:
            raise ValueError("dimension mismatch {}, {}".format(self._Ad.shape, v.shape))
        vdt = v.dtype if host else D.np_dtype(v.dtype)
        v_dtype = np.result_type(self._dtype, vdt)
        if overwrite_v:
            if v_dtype != vdt:
                raise ValueError("if overwrite_v is True, the input array must match correct output dtype for "
                                 "matrix multiplication.")
            if host and not v.flags["CARRAY"]:
                raise TypeError("input array must a contiguous and writable.")
        if work_array is not None:
            wsz = work_array.size if host or not D.is_device_array(work_array) else work_array.numel()
            vsz = v.size if host else v.numel()
            if wsz != 2 * vsz:
                raise ValueError("work_array must have twice the number of elements as in v.")
            wdt = work_array.dtype if not D.is_device_array(work_array) else D.np_dtype(work_array.dtype)
            if wdt != v_dtype:
                raise ValueError("work_array must be array of dtype which matches the result of the "
                                 "matrix-vector multiplication.")
        if tol is not None:
            tol = float(np.array(tol, dtype=np.array(self._mu).real.dtype))
        n = self._Ad.shape[0]
        if n == 0:
            return v if overwrite_v else v.copy() if host else v.clone()
        if not host and v.dtype == torch.complex128 and v.is_contiguous():
            F = v if overwrite_v else v.clone()
            wdev = work_array.view(-1) if (D.is_device_array(work_array) and
                                           work_array.dtype == torch.complex128) else None
            self.run_device(F, tol=tol, work=wdev)
            return F
        F = D.to_device(v, np.complex128).clone()
        self.run_device(F, tol=tol)
        if host:
            res = D.to_host(F)
            res = res.astype(v_dtype, copy=False) if v_dtype.kind == "c" else res.real.astype(v_dtype)
            if overwrite_v:
                v[...] = res
                return v
            return res
        res = F if v_dtype.kind == "c" else F.real
        res = res.to(D.torch_dtype(v_dtype))
        if overwrite_v:
            v.copy_(res)
            return v
        return res


expm_multiply_parallel = ExpmMultiplyParallel
