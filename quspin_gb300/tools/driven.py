"""Piecewise-constant evolution under a driven Hamiltonian.

The reference pattern for a time-dependent H(t) = H_0 + sum_k f_k(t) H_k
(examples/scripts/example22.py:84-98, application/quspin_app.py:166-179) is,
per step, ``H.tocsr(t)`` (a host CSR sum), a new ``ExpmMultiplyParallel``
(trace, exact 1-norm, fragment 3.1) and ``.dot(psi, overwrite_v=True)``.
``DrivenEvolution`` keeps that arithmetic on the device: the union sparsity
pattern of all parts is built once and each step forms the values of H(t) on
it, mu(t) from the precomputed per-part traces, and then either

* ``mode="plain"``: the exact 1-norm pass and the reference's (m*, s)
  selection, every step (one host round trip per step), or
* ``mode="learned"``: (m*, s) for every step of the trajectory from one
  batched forward of a ``PartitionPredictor``; no norm pass and no host round
  trip inside a segment.  A substep that exhausts its m* terms without the
  stopping test firing is counted on the device; such a segment is re-run
  with the plain selection (the fallback).

Many states evolve together as one [n, k] block.  ``precision`` selects the
Taylor-term arithmetic as for ``ExpmMultiplyParallel`` ("double": float-pair
products, "ieee": IEEE double products, "mixed": complex64 terms).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from .. import _device as D
from .. import _lib
from ..sparse import DeviceCSR
from ._partition import LazyOperatorNormInfo, fragment_3_1


class DrivenEvolution:
    def __init__(self, H, nvec=1, dtype=np.complex128, precision="double"):
        from ..operators import hamiltonian
        if not isinstance(H, hamiltonian):
            raise TypeError("H must be a hamiltonian")
        if precision not in ("double", "ieee", "mixed"):
            raise ValueError("precision must be 'double', 'ieee' or 'mixed'")
        self.precision = precision
        self.H = H
        self.nvec = int(nvec)
        parts = [H.static.tocsr()] + [Hd.tocsr() for Hd in H.dynamic.values()]
        self.funcs = list(H.dynamic.keys())
        pat = None
        for p in parts:
            q = sp.csr_matrix(p, dtype=np.float64, copy=True)
            q.data[:] = 1.0
            pat = q if pat is None else pat + q
        pat = sp.csr_matrix(pat)
        pat.sort_indices()
        vt = np.dtype(H.dtype)
        n = pat.shape[0]
        pat_keys = np.repeat(np.arange(n, dtype=np.int64), np.diff(pat.indptr)) * n + pat.indices
        self._vals = []
        for p in parts:
            pc = sp.csr_matrix(p, dtype=vt)
            pc.sum_duplicates()
            keys = np.repeat(np.arange(n, dtype=np.int64), np.diff(pc.indptr)) * n + pc.indices
            full = np.zeros(pat.nnz, vt)
            full[np.searchsorted(pat_keys, keys)] = pc.data
            self._vals.append(D.to_device(full))
        self.A = DeviceCSR.from_scipy(pat.astype(vt), vt)
        self.n = self.A.shape[0]
        self.traces = [complex(p.diagonal().sum()) for p in parts]
        self.part_norms = [DeviceCSR.from_scipy(sp.csr_matrix(p, dtype=vt), vt).onenorm(
            -(complex(p.diagonal().sum()) / self.n) if i == 0 else 0.0) for i, p in enumerate(parts)]
        self._data = torch.empty_like(self._vals[0])
        self._work = torch.empty(2 * self.n * self.nvec, dtype=torch.complex128, device=D.device())
        self._ctl = torch.zeros(8, dtype=torch.int64, device=D.device())
        self._op = None
        self.fallbacks = 0
        self.norm_passes = 0

    # -- per step ---------------------------------------------------------------
    def coeffs(self, t):
        return np.array([1.0] + [complex(f(t)).real if np.isrealobj(f(t)) else complex(f(t))
                                 for f in self.funcs])

    def _form(self, t):
        c = self.coeffs(t)
        self._data.copy_(self._vals[0])
        for v, ck in zip(self._vals[1:], c[1:]):
            self._data.add_(v, alpha=ck if self._data.is_complex() else float(np.real(ck)))
        mu = sum(ck * tr for ck, tr in zip(c, self.traces)) / self.n
        return DeviceCSR(self.A.indptr, self.A.indices, self._data, self.A.shape, self.A.dtype), complex(mu), c

    def norm_bound(self, t):
        c = self.coeffs(t)
        return float(sum(abs(ck) * nk for ck, nk in zip(c, self.part_norms)))

    def plain_partition(self, M, mu, a):
        """The reference's (m*, s): exact 1-norm pass + fragment 3.1."""
        self.norm_passes += 1
        A1 = M.onenorm(-mu)
        tol = np.finfo(np.complex128).eps / 2
        if abs(a) * A1 == 0:
            return 0, 1

        def apply(conj):
            aa, mm = (np.conj(a), np.conj(mu)) if conj else (a, mu)
            MM = M.conj_transpose() if conj else M

            def f(X):
                x2 = X.reshape(X.shape[0], -1).to(torch.complex128).contiguous()
                y = torch.empty_like(x2)
                MM.matvec_into(x2, y, a=aa, overwrite=True)
                y.sub_(x2, alpha=aa * mm)
                return y.reshape(X.shape)
            return f
        info = LazyOperatorNormInfo(apply(False), apply(True), self.n, A1, a, np.dtype(np.complex128),
                                    device=(torch.complex128, D.device()))
        return fragment_3_1(info, 1, tol, ell=2)

    def _operand(self, M):
        """M's values (formed on the device for this step) in the operand
        form of the precision, with the B storage code and launch shape."""
        from ..tune import tune_taylor
        if self.precision == "ieee":
            op, bt = M, _lib.C128
        elif self.precision == "mixed":
            vt = torch.float32 if M.dtype.kind == "f" else torch.complex64
            if self._op is None:
                self._op = DeviceCSR(M.indptr, M.indices, M.data.to(vt), M.shape, D.np_dtype(vt))
            self._op.data.copy_(M.data)
            op, bt = self._op, _lib.C64
        else:
            if self._op is None:
                self._op = M.paired(coded=False)      # values change every step
            else:
                self._op.refresh(M.data)
            op, bt = self._op, _lib.CPF
        return op, bt, tune_taylor(op, self.nvec, bt)

    def _taylor(self, F, M, mu, a, m, s):
        coeff = np.array([a / (s * (j + 1)) for j in range(max(m, 1))], np.complex128)
        consts = D.to_device(np.concatenate([coeff, [np.exp(a * mu / s), 1.0]]).astype(np.complex128))
        k = max(m, 1)
        op, bt, group = self._operand(M)
        if "_rown" not in self.__dict__:
            self._rown = torch.empty(2 * self.n, dtype=torch.float64, device=D.device())
        rown = self._rown if (bt != _lib.C128 and self.nvec > 8) else None
        _lib.call("qs_expm_multiply_rows", self.n, op.nnz, D.ptr(op.indptr), op.idx64, D.ptr(op.indices),
                  D.ptr(op.data), op.vcode, D.ptr(F), self.nvec, int(s), int(m), float(np.finfo(np.float64).eps / 2),
                  mu.real, mu.imag, D.ptr(consts[:k]), D.ptr(consts[k:k + 1]), D.ptr(consts[k + 1:]),
                  D.ptr(self._work), bt, D.ptr(self._ctl), group, D.ptr(rown), D.stream())
        self._keep = consts

    def run(self, F, t0, dt, nsteps, mode="plain", predictor=None, segment=50, record=None):
        """Evolve the device block F ([n, k] complex128) in place over nsteps
        steps of length dt, H evaluated at each step's midpoint."""
        a = -1j * dt
        ts = t0 + dt * (np.arange(nsteps) + 0.5)
        if mode == "learned":
            if predictor is None:
                raise ValueError("mode='learned' needs a predictor")
            feats = predictor.features(np.full(nsteps, abs(a)), np.array([self.norm_bound(t) for t in ts]),
                                       np.array([self.coeffs(t)[1:].real for t in ts]))
            m_pred, s_pred = predictor.predict(feats)
        done = 0
        while done < nsteps:
            seg = range(done, min(done + segment, nsteps))
            if mode == "learned":
                saved = F.clone()
                self._ctl.zero_()
                for i in seg:
                    M, mu, _ = self._form(ts[i])
                    self._taylor(F, M, mu, a, int(m_pred[i]), int(s_pred[i]))
                    if record is not None:
                        record.append((int(m_pred[i]), int(s_pred[i])))
                nonconv = int(self._ctl.view(torch.int32)[10].item())
                if nonconv:
                    self.fallbacks += 1
                    F.copy_(saved)
                    for i in seg:
                        M, mu, _ = self._form(ts[i])
                        m, s = self.plain_partition(M, mu, a)
                        self._taylor(F, M, mu, a, m, s)
            else:
                for i in seg:
                    M, mu, _ = self._form(ts[i])
                    m, s = self.plain_partition(M, mu, a)
                    if record is not None:
                        record.append((int(m), int(s)))
                    self._taylor(F, M, mu, a, m, s)
            done = seg.stop
        return F

    def training_set(self, t_values, dt_values):
        """(features, m*, s) of the plain selection at the given times and
        step lengths (the predictor's labels)."""
        feats, ms, ss = [], [], []
        for t, dt in zip(t_values, dt_values):
            a = -1j * dt
            M, mu, c = self._form(t)
            m, s = self.plain_partition(M, mu, a)
            feats.append([abs(a) * self.norm_bound(t), abs(a)] + list(c[1:].real))
            ms.append(m)
            ss.append(s)
        f = np.array(feats)
        from ..learned import PartitionPredictor
        return PartitionPredictor.features(f[:, 1], f[:, 0] / f[:, 1], f[:, 2:]), np.array(ms), np.array(ss)
