"""Many symmetry sectors and many states evolved together.

``MultiSectorExpm`` applies e^{a H_b} to a block of k states in every sector b
of a list of Hamiltonians (for instance all momentum sectors of a chain) in
one stacked launch sequence: the sector matrices are stacked
block-diagonally, every Taylor term of every sector is one launch of
``qs_taylor_multi_term`` (per-sector shift, factor and stopping test), and the
whole evolution is captured once in a CUDA graph and replayed.  This replaces
the reference's per-sector process fan-out (``block_tools.block_ops``,
src/quspin/tools/block_tools.py:135-220,618-795) for the expm_multiply path.

The schedule is common to all sectors: s = max_b s_b substeps of at most
m* = max_b m*_b terms, each sector's (m*_b, s_b) chosen as
``ExpmMultiplyParallel`` does; more substeps than a sector needs only
tightens its truncation, and each sector still stops on its own test.
``precision`` is as for ``ExpmMultiplyParallel``: "double" (float-pair
products, the default), "ieee" (IEEE double products) or "mixed" (complex64
term blocks and float32/complex64 values); F, shifts, coefficients and the
stopping tests stay in double precision.  The launch shape is autotuned on
the stacked matrix.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _device as D
from .. import _lib
from ..sparse import DeviceCSR
from .expm_multiply_parallel import ExpmMultiplyParallel, _as_device_csr


def _stack(mats):
    """Block-diagonal stack of device CSR matrices (int32 indices)."""
    offs = [0]
    for A in mats:
        offs.append(offs[-1] + A.shape[0])
    nnz_off = [0]
    for A in mats:
        nnz_off.append(nnz_off[-1] + A.nnz)
    if nnz_off[-1] >= 2**31 - 1 or offs[-1] >= 2**31 - 1:
        raise NotImplementedError("stacked sectors exceed 2^31 rows or nonzeros")
    ip = [torch.zeros(1, dtype=torch.int64, device=D.device())]
    ix, dt = [], []
    for b, A in enumerate(mats):
        ip.append(A.indptr[1:].to(torch.int64) + nnz_off[b])
        ix.append(A.indices + offs[b])
        dt.append(A.data)
    indptr = torch.cat(ip).to(torch.int32)
    dtype = np.result_type(*[A.dtype for A in mats])
    data = torch.cat([d.to(D.torch_dtype(dtype)) for d in dt])
    return DeviceCSR(indptr, torch.cat(ix).contiguous(), data, (offs[-1], offs[-1]), dtype), offs


class MultiSectorExpm:
    """e^{a H_b} V_b for every sector b in one graph-captured launch sequence."""

    def __init__(self, matrices, a, nvec=1, precision="double", graph=True):
        if precision not in ("double", "ieee", "mixed"):
            raise ValueError("precision must be 'double', 'ieee' or 'mixed'")
        if len(matrices) > _lib.load().qs_max_sectors():
            raise ValueError("at most {} sectors per launch".format(_lib.load().qs_max_sectors()))
        self._a = complex(a)
        self.nvec = int(nvec)
        self.precision = precision
        # an ExpmMultiplyParallel with the same a can be passed instead of a
        # matrix: its shift and (m*, s) are reused
        self._plain = [M if isinstance(M, ExpmMultiplyParallel) and complex(M.a) == self._a
                       else ExpmMultiplyParallel(M, a=a) for M in matrices]
        mats = [p.A_device for p in self._plain]
        self.sizes = [M.shape[0] for M in mats]
        self.m_star = max(p.m_star for p in self._plain)
        self.s = max(p.s for p in self._plain)
        self._tol = float(min(p._tol for p in self._plain))
        A, offs = _stack(mats)
        self._offs = offs
        if precision == "mixed":
            A = A.astype(np.float32 if A.dtype.kind == "f" else np.complex64)
            self._btype = _lib.C64
        elif precision == "ieee":
            self._btype = _lib.C128
        else:
            A = A.paired()
            self._btype = _lib.CPF
        self._A = A
        n, k = A.shape[0], self.nvec
        self.n = n
        dev = D.device()
        self.F = torch.zeros((n, k), dtype=torch.complex128, device=dev)
        bdt = torch.complex64 if self._btype == _lib.C64 else torch.complex128
        self._work = torch.empty(2 * n * k, dtype=bdt, device=dev)
        self._soff = torch.tensor(offs, dtype=torch.int64, device=dev)
        mus = np.array([complex(p._mu) for p in self._plain], np.complex128)
        etas = np.exp(self._a * mus / self.s)
        coeff = np.array([self._a / (self.s * (j + 1)) for j in range(max(self.m_star, 1))], np.complex128)
        self._mu = torch.tensor(mus, device=dev)
        self._eta = torch.tensor(etas, device=dev)
        self._coeff = torch.tensor(coeff, device=dev)
        nb = _lib.load().qs_multi_ctl_bytes()
        tmpl = np.zeros((nb + 7) // 8 * 2, np.int32)
        tmpl[1] = len(mats)
        self._ctl_tmpl = torch.tensor(tmpl, device=dev)
        self._ctl = self._ctl_tmpl.clone()
        self._group = self._tune()
        self._graph = None
        self._use_graph = graph

    @property
    def sector_offsets(self):
        return list(self._offs)

    def _term(self, j, bin_, bout, tol, group):
        A = self._A
        _lib.call("qs_taylor_multi_term", self.n, D.ptr(A.indptr), D.ptr(A.indices), D.ptr(A.data), A.vcode,
                  D.ptr(bin_), D.ptr(bout), self._btype, D.ptr(self.F), self.nvec, D.ptr(self._soff),
                  D.ptr(self._mu), D.ptr(self._coeff), j, tol, D.ptr(self._ctl), group, D.stream())

    def _rescale(self, use_eta):
        b0 = self._work[: self.n * self.nvec]
        _lib.call("qs_taylor_multi_rescale", self.n, self.nvec, D.ptr(self.F), D.ptr(b0), self._btype,
                  D.ptr(self._soff), D.ptr(self._eta), int(use_eta), D.ptr(self._ctl), D.stream())

    def _tune(self):
        from ..tune import _candidates, _time, encode, occ_candidates
        if self.n < 65536:
            return 0
        b0 = self._work[: self.n * self.nvec]
        b1 = self._work[self.n * self.nvec:]
        best, best_t = 0, None
        codes = [encode(G, U) for G, U in _candidates(self.n, self._A.nnz, self.nvec)
                 if not (self.nvec == 1 and U > 2)]
        codes += [encode(G, U) | (occ << 18) for G, U in occ_candidates(self._A, self.nvec, self._btype)
                  for occ in (1, 2)]
        if self.nvec > 1:      # the vectors-across-lanes kernel (csrc/expm_vl.cu), three shapes
            codes += [encode(2, 2) | (shape << 20) for shape in (1, 2, 3)]
        for code in codes:
            self._ctl.copy_(self._ctl_tmpl)
            t = _time(lambda: self._term(0, b0, b1, 0.0, code))
            if best_t is None or t < best_t:
                best, best_t = code, t
        self.F.zero_()
        return best

    def _sequence(self):
        """The full launch sequence of one evolution (F in place)."""
        nk = self.n * self.nvec
        b0, b1 = self._work[:nk], self._work[nk:]
        self._ctl.copy_(self._ctl_tmpl)
        self._rescale(False)
        for _ in range(self.s):
            for j in range(self.m_star):
                bi, bo = (b0, b1) if j % 2 == 0 else (b1, b0)
                self._term(j, bi, bo, self._tol, self._group)
            self._rescale(True)

    def run_device(self):
        """Evolve self.F in place (graph replay after the first call)."""
        if not self._use_graph:
            self._sequence()
            return self.F
        if self._graph is None:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            saved = self.F.clone()
            with torch.cuda.stream(side):
                self._sequence()              # warm-up outside capture
            torch.cuda.current_stream().wait_stream(side)
            self.F.copy_(saved)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._sequence()
            self._graph = g
        self._graph.replay()
        return self.F

    def load(self, blocks):
        """Copy per-sector state blocks ([n_b, k] each) into F."""
        for b, V in enumerate(blocks):
            v = D.to_device(V, np.complex128).reshape(self.sizes[b], self.nvec)
            self.F[self._offs[b]:self._offs[b + 1]].copy_(v)

    def blocks(self, host=True):
        out = [self.F[self._offs[b]:self._offs[b + 1]] for b in range(len(self.sizes))]
        return [D.to_host(o) for o in out] if host else out

    def evolve(self, blocks, host=True):
        """e^{a H_b} V_b for every sector; returns the list of blocks."""
        self.load(blocks)
        self.run_device()
        return self.blocks(host)

    @property
    def terms_executed(self):
        """Sector-terms executed by the last evolution (reads the device counter)."""
        return int(self._ctl.view(torch.int64)[1].item())
