"""Symmetry-reduced bases, built and queried on the GPU.

Drop-in counterparts of QuSpin 1.0.1's general bases for spin-1/2 and
fermions (reference paths relative to the project root):

* ``spin_basis_general`` -- src/quspin/basis/basis_general/spin.py:66-227
* ``spinless_fermion_basis_general`` / ``spinful_fermion_basis_general`` --
  src/quspin/basis/basis_general/fermion.py:69-283, :356-460, :722-727,
  :1080-1096
* ``spin_basis_1d`` -- src/quspin/basis/basis_1d/spin.py, which for spin-1/2
  gives the same states and matrix elements as the general basis with the
  translation / reflection / spin-inversion maps
  (test/test_general_spin_opstr.py:60-153).

The Python layer keeps the reference's map handling (``process_map``,
base_general.py:22-51; block ordering, :135-212) and its argument checks; the
enumeration, representative search, normalisation, index lookup, operator
strings and the canonical CSR assembly all run in ``csrc/basis.cu``.
"""
from __future__ import annotations

import ctypes
import warnings
from math import gcd

import numpy as np
import torch
from scipy.special import comb

from . import _device as D
from . import _lib
from .sparse import DeviceCSR, DeviceDIA


class GeneralBasisWarning(Warning):
    pass


def process_map(map, q):
    """Period of a symmetry map, with the reference's outputs and messages
    (src/quspin/basis/basis_general/base_general.py:22-51).

    ``map[i] = j >= 0`` sends site i to site j; ``map[i] = -(j + 1)`` sends it
    to site j and inverts it (spin inversion / particle-hole).  The map is a
    signed permutation g; its period is the order of g: along each cycle of
    the underlying permutation, a site comes back to itself after the cycle
    length l with the product of the inversions met on the way, so the cycle
    contributes l when it holds an even number of inverted sites and 2 l
    otherwise, and the period is the least common multiple of these.

    Returns (map as int32, period, q, set of the powers g^k, k = 0 .. period,
    each written as the tuple of signed site labels in the reference's
    notation)."""
    map = np.asarray(map, dtype=np.int32)
    inv = map < 0
    dest = np.where(inv, -map - 1, map).astype(np.int64)
    n = dest.size
    if not np.array_equal(np.sort(dest), np.arange(n)):
        raise ValueError("map must be a one-to-one site mapping.")
    per = 1
    seen = np.zeros(n, dtype=bool)
    for start in range(n):
        if seen[start]:
            continue
        length, flips, i = 0, 0, start
        while not seen[i]:
            seen[i] = True
            flips += int(inv[i])
            i = int(dest[i])
            length += 1
        cyc = length if flips % 2 == 0 else 2 * length
        per = per * cyc // gcd(per, cyc)
    if per == 1:
        warnings.warn("identity mapping found in set of transformations.", GeneralBasisWarning, stacklevel=5)
    # powers of g: position i of g^(k+1) holds the label of position dest[i]
    # of g^k, inverted once more when that site is an inverted one
    label = np.arange(n, dtype=np.int64)
    odd = np.zeros(n, dtype=bool)
    powers = set()
    for _ in range(per + 1):
        powers.add(tuple(int(x) for x in np.where(odd, -label - 1, label)))
        label, odd = label[dest], odd[dest] ^ inv[dest]
    return map, per, q, powers


def _phase_tables(L):
    p = np.arange(L)
    t = np.exp(-2j * np.pi * p / L)
    c = np.cos(2 * np.pi * p / L)
    for k in range(L):
        if k == 0:
            t[k], c[k] = 1.0, 1.0
        elif 4 * k == L:
            t[k], c[k] = -1j, 0.0
        elif 2 * k == L:
            t[k], c[k] = -1.0, -1.0
        elif 4 * k == 3 * L:
            t[k], c[k] = 1j, 0.0
    return (np.ascontiguousarray(t.real), np.ascontiguousarray(t.imag), np.ascontiguousarray(c))


_DIAG_CHARS = set("Izn")


class _TermTable:
    """Device term table: op characters, sites and couplings of op strings."""

    def __init__(self, terms):
        nop, off, chrs, sites, J = [], [], [], [], []
        o = 0
        for opstr, indx, Jt in terms:
            nop.append(len(opstr))
            off.append(o)
            chrs.extend(ord(c) for c in opstr)
            sites.extend(int(i) for i in indx)
            Jt = complex(Jt)
            J.extend([Jt.real, Jt.imag])
            o += len(opstr)
        self.T = len(terms)
        self.nop = D.to_device(np.asarray(nop if nop else [0], np.int32))
        self.off = D.to_device(np.asarray(off if off else [0], np.int32))
        self.chr = D.to_device(np.asarray(chrs if chrs else [0], np.int8))
        self.site = D.to_device(np.asarray(sites if sites else [0], np.int32))
        self.J = D.to_device(np.asarray(J if J else [0.0, 0.0], np.float64))

    def args(self):
        return (D.ptr(self.nop), D.ptr(self.off), D.ptr(self.chr), D.ptr(self.site), D.ptr(self.J))


class basis_general:
    """GPU general basis over spin-1/2 / fermion bits (common machinery).

    ``sectors`` is a list of (kind, p0, p1): kind 0 every word, 1 a fixed
    number p0 of set bits, 2 spinful (p0 up in the high half, p1 down in the
    low half).  ``blocks`` maps block names to (per-bit map, q).
    """

    _fermion = False
    _spinful = False
    _pauli = 0

    def _init_general(self, N, sectors, block_order=None, blocks=None):
        D.require_cuda()
        self._N = int(N)
        if self._N > 64:
            raise NotImplementedError("states wider than 64 bits are not supported")
        blocks = {k: v for k, v in (blocks or {}).items() if v is not None}
        if len(blocks) > 32:
            raise ValueError("general basis can only support up to 32 symmetries.")
        if any((type(m) is not tuple) and (len(m) != 2) for m in blocks.values()):
            raise ValueError("blocks must contain tuple: (map,q).")
        items = {k: process_map(*v) for k, v in blocks.items()}
        if block_order is None:
            sorted_items = sorted(items.items(), key=lambda x: x[1][1])
        else:
            block_order = list(block_order)
            missing = set(items) - set(block_order)
            if missing:
                raise ValueError("{} names found in block names but missing from block_order.".format(missing))
            missing = set(block_order) - set(items)
            if missing:
                raise ValueError("{} names found in block_order but missing from block names.".format(missing))
            block_order.reverse()
            sorted_items = [(k, items[k]) for k in block_order]
        self._blocks = {b: ((-1) ** q if per == 2 else q) for b, (_, per, q, _) in sorted_items}
        self._maps_dict = {b: m for b, (m, _, _, _) in sorted_items}
        remove_index = [i for i, it in enumerate(sorted_items[:-1]) if it[1][1] == 1]
        kept = [it for _, it in sorted_items]
        for i in sorted(remove_index):
            kept.pop(i)
        if kept:
            self._maps = np.ascontiguousarray(np.vstack([m for m, _, _, _ in kept]), dtype=np.int32)
            self._qs = np.asarray([q for _, _, q, _ in kept], dtype=np.int32)
            self._pers = np.asarray([p for _, p, _, _ in kept], dtype=np.int32)
            if any(m.shape[0] != self._N for m in self._maps):
                raise ValueError("size of map is not equal to N.")
        else:
            self._maps = np.zeros((0, self._N), dtype=np.int32)
            self._qs = np.zeros(0, dtype=np.int32)
            self._pers = np.zeros(0, dtype=np.int32)
        self._n_dtype = np.min_scalar_type(int(np.prod(self._pers, dtype=np.int64)) if len(self._pers) else 1)
        L = 1
        for p in self._pers:
            L = L // gcd(L, int(p)) * int(p)
        self._L = L
        self._phase_re, self._phase_im, self._costab = _phase_tables(L)
        self._sectors = list(sectors)
        self._basis_dtype = np.dtype(np.uint32) if self._N <= 32 else np.dtype(np.uint64)
        self._sbytes = self._basis_dtype.itemsize
        h = ctypes.c_void_p()
        maps = self._maps.reshape(-1) if self._maps.size else np.zeros(1, np.int32)
        pers = self._pers if self._pers.size else np.zeros(1, np.int32)
        qs = self._qs if self._qs.size else np.zeros(1, np.int32)
        rc = _lib.load().qs_sym_create(self._N, int(self._fermion), len(self._pers),
                                       maps.ctypes.data_as(ctypes.c_void_p), pers.ctypes.data_as(ctypes.c_void_p),
                                       qs.ctypes.data_as(ctypes.c_void_p),
                                       self._phase_re.ctypes.data_as(ctypes.c_void_p),
                                       self._phase_im.ctypes.data_as(ctypes.c_void_p),
                                       self._costab.ctypes.data_as(ctypes.c_void_p), L, ctypes.byref(h))
        if rc == -6:
            raise NotImplementedError("particle-hole type (negative) maps are not supported for fermion bases")
        _lib.check(rc, "qs_sym_create")
        self._sym = h
        self._made_basis = False
        self._states_host = None
        self._Ns = 0
        self._unique_me = True

    def __del__(self):
        h = getattr(self, "_sym", None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.qs_sym_destroy(h)
            except Exception:
                pass
            self._sym = None

    # -- construction ------------------------------------------------------
    def make(self, Ns_block_est=None, N_p=None):
        """Enumerate the sector on the GPU (base_general.py:817-899)."""
        L = _lib.load()
        st = D.stream()
        parts_s, parts_n = [], []
        sdt = self._basis_dtype
        for kind, p0, p1 in self._sectors:
            nch = L.qs_enum_num_chunks(self._N, kind, p0, p1)
            if nch < 0:
                raise ValueError("invalid particle sector")
            if nch == 0:
                continue
            off = torch.zeros(nch + 1, dtype=torch.int64, device=D.device())
            scr = torch.empty(max(L.qs_scan_scratch_elems(nch), 1), dtype=torch.int64, device=D.device())
            tot = ctypes.c_int64(0)
            _lib.check(L.qs_enum_count(self._sym, kind, p0, p1, D.ptr(off), nch, D.ptr(scr), ctypes.byref(tot), st),
                       "qs_enum_count")
            ns = int(tot.value)
            s = torch.empty(max(ns, 1), dtype=D.torch_dtype(sdt), device=D.device())
            n = torch.empty(max(ns, 1), dtype=torch.int32, device=D.device())
            if ns > 0:
                _lib.check(L.qs_enum_write(self._sym, kind, p0, p1, D.ptr(off), nch, D.ptr(s), D.ptr(n), st),
                           "qs_enum_write")
            parts_s.append(s[:ns])
            parts_n.append(n[:ns])
        if parts_s:
            states = torch.cat(parts_s)
            norms = torch.cat(parts_n)
        else:
            states = torch.empty(0, dtype=D.torch_dtype(sdt), device=D.device())
            norms = torch.empty(0, dtype=torch.int32, device=D.device())
        if len(parts_s) > 1:
            # several particle sectors: order the union descending (unsigned)
            key = states.to(torch.int64) if sdt == np.uint32 else states
            if sdt == np.uint32:
                key = key & 0xFFFFFFFF
                order = torch.argsort(key, descending=True, stable=True)
            else:
                order = torch.argsort(key ^ (-(2 ** 63)), descending=True, stable=True)
            states = states[order].contiguous()
            norms = norms[order].contiguous()
        self._basis = states
        self._n_dev = norms
        self._Ns = int(states.shape[0])
        self._states_host = None
        self._index_type = np.int32 if self._Ns < np.iinfo(np.int32).max else np.int64
        self._made_basis = True
        self.make_basis_blocks(N_p=N_p)
        return self._Ns

    def make_basis_blocks(self, N_p=None):
        """Prefix blocks for the index search (base_general.py:901-950)."""
        if not self._made_basis:
            raise ValueError("reference states are not constructed yet. basis must be constructed before "
                             "calculating blocks")
        if N_p is None:
            N_p = int(np.floor(np.log(self._Ns // 2 + 1) / np.log(2)))
        else:
            N_p = int(N_p)
        if len(self._pers) == 0 and all(k == 0 for k, _, _ in self._sectors):
            N_p = 0
        self._N_p = min(max(N_p, 0), self._N)
        if self._N_p > 0:
            nb = 1 << self._N_p
            self._begin = torch.empty(nb, dtype=torch.int64, device=D.device())
            self._end = torch.empty(nb, dtype=torch.int64, device=D.device())
            _lib.call("qs_make_blocks", self._N, self._sbytes, self._N_p, D.ptr(self._basis), self._Ns,
                      D.ptr(self._begin), D.ptr(self._end), D.stream())
        else:
            self._begin = torch.zeros(1, dtype=torch.int64, device=D.device())
            self._end = torch.zeros(1, dtype=torch.int64, device=D.device())

    # -- attributes mirroring the reference ----------------------------------
    @property
    def N(self):
        return self._N

    @property
    def Ns(self):
        return self._Ns

    @property
    def sps(self):
        return 2

    @property
    def dtype(self):
        return self._basis_dtype

    @property
    def states(self):
        if self._states_host is None:
            self._states_host = D.to_host(self._basis).view(self._basis_dtype)
        return self._states_host

    @property
    def _n(self):
        n = D.to_host(self._n_dev).view(np.uint32)
        if len(n):
            return n.astype(np.min_scalar_type(int(n.max())))
        return n.astype(self._n_dtype)

    @property
    def blocks(self):
        return dict(self._blocks)

    @property
    def _basis_begin(self):
        return D.to_host(self._begin) if self._N_p > 0 else np.array([], dtype=np.intp)

    @property
    def _basis_end(self):
        return D.to_host(self._end) if self._N_p > 0 else np.array([], dtype=np.intp)

    def _basis_args(self):
        return (D.ptr(self._basis), D.ptr(self._n_dev), self._Ns, self._N_p, D.ptr(self._begin), D.ptr(self._end))

    # -- queries --------------------------------------------------------------
    def index(self, s):
        """Position of state(s) in the basis (-1 if absent)."""
        if isinstance(s, str):
            s = int(s, 2)
        scalar = np.ndim(s) == 0
        q = np.atleast_1d(np.asarray(s)).astype(self._basis_dtype)
        qd = D.to_device(q)
        out = torch.empty(len(q), dtype=torch.int64, device=D.device())
        _lib.call("qs_index", self._N, self._sbytes, D.ptr(self._basis), self._Ns, self._N_p, D.ptr(self._begin),
                  D.ptr(self._end), D.ptr(qd), len(q), D.ptr(out), D.stream())
        r = D.to_host(out)
        return int(r[0]) if scalar else r

    def representative(self, states, out=None, return_g=False, return_sign=False):
        """Orbit representatives (base_general.py:1035-1117)."""
        s = np.atleast_1d(np.asarray(states, dtype=self._basis_dtype))
        if s.ndim != 1:
            raise TypeError("dimension of array_like states must not exceed 1.")
        sd = D.to_device(s)
        rd = torch.empty_like(sd)
        K = len(self._pers)
        g = torch.zeros((len(s), max(K, 1)), dtype=torch.int32, device=D.device()) if return_g else None
        sg = torch.zeros(len(s), dtype=torch.int8, device=D.device()) if return_sign else None
        if len(s):
            _lib.call("qs_representative", self._sym, D.ptr(sd), len(s), D.ptr(rd), D.ptr(g), D.ptr(sg),
                      D.stream())
        reps = D.to_host(rd).view(self._basis_dtype)
        extra = []
        if return_g:
            extra.append(D.to_host(g)[:, :K])
        if return_sign:
            extra.append(D.to_host(sg))
        if out is not None:
            if not isinstance(out, np.ndarray):
                raise TypeError("out must be a numpy.ndarray")
            if out.shape != s.shape:
                raise TypeError("states and out must have same shape.")
            if out.dtype != self._basis_dtype:
                raise TypeError("out must have same type as basis")
            out[...] = reps
            return tuple(extra) if len(extra) > 1 else (extra[0] if extra else None)
        return (reps, *extra) if extra else reps

    def normalization(self, states, out=None):
        """Norms of states as representatives, 0 outside the basis."""
        s = np.atleast_1d(np.asarray(states, dtype=self._basis_dtype))
        sd = D.to_device(s)
        nd = torch.empty(len(s), dtype=torch.int32, device=D.device())
        if len(s):
            _lib.call("qs_normalization", self._sym, D.ptr(sd), len(s), D.ptr(nd), D.stream())
        n = D.to_host(nd).view(np.uint32)
        if out is not None:
            if out.shape != s.shape:
                raise TypeError("states and out must have same shape.")
            if np.issubdtype(out.dtype, np.signedinteger):
                raise TypeError("out must have datatype numpy.uint8, numpy.uint16, numpy.uint32, or numpy.uint64.")
            out[...] = n
            return None
        return n.astype(np.min_scalar_type(int(n.max()) if len(n) else 0)).squeeze()

    # -- operator strings -------------------------------------------------------
    def _term(self, opstr, indx, J):
        """Validated (opstr, indx, J) in the per-bit form the kernels use."""
        indx = np.asarray(indx, dtype=np.int32).ravel()
        if self._spinful:
            if opstr.count("|") != 1 or "|" not in opstr:
                if opstr.count("|") == 0:
                    raise ValueError("missing '|' charactor in: {0}, {1}".format(opstr, indx))
                raise ValueError("only one '|' charactor allowed in: {0}, {1}".format(opstr, indx))
            i = opstr.index("|")
            left, right = opstr.split("|", 1)
            indx = np.concatenate([indx[:i], indx[i:] + self._N // 2]).astype(np.int32)
            opstr = left + right
        if len(opstr) != len(indx):
            raise ValueError("length of opstr does not match length of indx")
        if np.any(indx >= self._N) or np.any(indx < 0):
            raise ValueError("values in indx falls outside of system")
        extra = set(opstr) - self._allowed_ops
        if extra:
            raise ValueError("unrecognized characters {} in operator string.".format(extra))
        if len(opstr) > 16:
            raise NotImplementedError("operator strings longer than 16 sites are not supported")
        J = complex(J) * self._scale(opstr)
        return opstr, indx, J

    def _scale(self, opstr):
        return 1.0

    def _raw_op(self, opstr, indx, J):
        o, ix, Jc = self._term(opstr, indx, J)
        tt = _TermTable([(o, ix, Jc)])
        Ns = self._Ns
        row = torch.empty(max(Ns, 1), dtype=torch.int64, device=D.device())
        col = torch.empty(max(Ns, 1), dtype=torch.int64, device=D.device())
        me = torch.empty(max(Ns, 1), dtype=torch.complex128, device=D.device())
        err = D.err_flag()
        if Ns:
            _lib.call("qs_op", self._sym, *self._basis_args(), *tt.args(), D.ptr(row), D.ptr(col), D.ptr(me),
                      D.ptr(err), D.stream())
        if int(err.item()) & 1:
            raise ValueError("unrecognized characters in operator string {}".format(opstr))
        return me[:Ns], row[:Ns], col[:Ns]

    def Op(self, opstr, indx, J, dtype):
        """(ME, row, col) of one operator-string term (base_general.py:292-352)."""
        if not self._made_basis:
            raise AttributeError("this function requires the basis to be constructed first; use basis.make().")
        dtype = np.dtype(dtype)
        if self._Ns <= 0:
            return (np.array([], dtype=dtype), np.array([], dtype=self._index_type),
                    np.array([], dtype=self._index_type))
        me, row, col = self._raw_op(opstr, indx, J)
        ME = D.to_host(me)
        row = D.to_host(row).astype(self._index_type)
        col = D.to_host(col).astype(self._index_type)
        if dtype.kind != "c":
            bad = np.abs(ME.imag) > 1.1e-15 * np.maximum(1.0, np.abs(ME.real))
            if np.any(bad):
                raise TypeError("attemping to use real type for complex elements.")
            ME = ME.real.astype(dtype)
        else:
            ME = ME.astype(dtype)
        mask = ME != 0
        return ME[mask], row[mask], col[mask]

    def _make_matrix(self, op_list, dtype):
        """Canonical CSR (or DIA) of a list of terms (src/quspin/basis/base.py:265-304)."""
        return build_matrix(self, op_list, dtype)

    def inplace_Op(self, v_in, op_list, dtype, transposed=False, conjugated=False, v_out=None, a=1.0):
        """Matrix-free v_out += a * sum_t J_t op_t v_in (base_general.py:354-410)."""
        if not self._made_basis:
            raise AttributeError("this function requires the basis to be constructed first; use basis.make().")
        host = not D.is_device_array(v_in)
        vdt = np.asarray(v_in).dtype if host else D.np_dtype(v_in.dtype)
        rdt = np.result_type(vdt, dtype)
        shape = tuple(v_in.shape)
        if shape[0] != self._Ns:
            raise ValueError("dimension mismatch")
        x = D.to_device(v_in, np.complex128).reshape(self._Ns, -1).contiguous()
        if v_out is None:
            y = torch.zeros_like(x)
        else:
            if (np.asarray(v_out).dtype if not D.is_device_array(v_out) else D.np_dtype(v_out.dtype)) != rdt:
                raise TypeError("v_out does not have the correct data type.")
            if tuple(v_out.shape) != shape:
                raise ValueError("invalid shape for v_out and v_in: v_in.shape != v_out.shape")
            y = D.to_device(v_out, np.complex128).reshape(self._Ns, -1).clone()
        terms = [self._term(o, ix, Jt) for o, ix, Jt in op_list]
        tt = _TermTable(terms)
        err = D.err_flag()
        a = complex(a)
        if terms and self._Ns:
            _lib.call("qs_inplace_op", self._sym, *self._basis_args(), *tt.args(), tt.T, int(bool(transposed)),
                      int(bool(conjugated)), a.real, a.imag, D.ptr(x), D.ptr(y), x.shape[1], D.ptr(err), D.stream())
        if int(err.item()) & 1:
            raise ValueError("unrecognized characters in operator string")
        if rdt.kind != "c":
            y = y.real
        y = y.to(D.torch_dtype(rdt)).reshape(shape)
        if host:
            res = D.to_host(y)
            if v_out is not None:
                v_out[...] = res
                return v_out
            return res.squeeze()
        if v_out is not None:
            v_out.copy_(y)
            return v_out
        return y.squeeze()

    def get_amp(self, states, out=None, amps=None, mode="representative"):
        """Amplitude factor C with psi_s = C psi^sym_r between a state s of the
        full basis and its representative r (base_general.py:1183-1269), 0 for
        states outside the sector.  mode 'representative': states are
        representatives, amps (optional, symmetric-basis amplitudes) are
        multiplied by C in place; 'full_basis': states are full-basis states
        and are replaced in place by their representatives, amps (full-basis
        amplitudes) are divided by C in place.  C = sqrt(n_r / |G|) for a
        representative and sqrt(n_r / |G|) conj(chi(g)) sign(g) for the first
        group element g taking s to r -- the projector's entry at row s."""
        if mode not in ("representative", "full_basis"):
            raise ValueError("mode accepts only the values 'representative' and 'full_basis'.")
        caller = states
        states = np.atleast_1d(np.asarray(states, order="C", dtype=self._basis_dtype))
        shape = states.shape
        if out is not None:
            if shape != out.shape:
                raise TypeError("states and out must have same shape.")
            if out.dtype not in (np.float32, np.float64, np.complex64, np.complex128):
                raise TypeError("out must have datatype numpy.float32, numpy.float64, numpy.complex64, or "
                                "numpy.complex128.")
            if not out.flags["CARRAY"]:
                raise ValueError("out must be C-contiguous array.")
        elif amps is not None:
            out = np.zeros(shape, dtype=amps.dtype)
        else:
            out = np.zeros(shape, dtype=np.complex128)
        flat = states.reshape(-1)
        G = int(np.prod(self._pers, dtype=np.int64)) if len(self._pers) else 1
        if mode == "representative":
            n = np.atleast_1d(self.normalization(flat)).astype(np.float64)
            C = np.sqrt(n / G).astype(np.complex128)
        else:
            reps, g, sg = self.representative(flat, return_g=True, return_sign=True)
            n = np.atleast_1d(self.normalization(reps)).astype(np.float64)
            steps = np.asarray([(int(q) * (self._L // int(p))) % self._L for q, p in zip(self._qs, self._pers)],
                               np.int64)
            ph = (g.astype(np.int64) @ steps) % self._L if len(steps) else np.zeros(len(flat), np.int64)
            chi = self._phase_re[ph] + 1j * self._phase_im[ph]
            C = np.sqrt(n / G) * np.conj(chi) * sg
            flat[...] = reps
            if isinstance(caller, np.ndarray) and caller.dtype == self._basis_dtype and caller.flags["C_CONTIGUOUS"]:
                caller.reshape(-1)[...] = reps
        C = C.reshape(shape)
        if out.dtype.kind != "c":
            if np.any(np.abs(C.imag) > 1.1e-15):
                raise TypeError("attemping to use real type for complex elements.")
            C = C.real
        out[...] = C
        if amps is not None:
            if shape != amps.shape:
                raise TypeError("states and amps must have same shape.")
            if mode == "representative":
                amps *= out
            else:
                amps /= out
        return out.squeeze()

    # -- projector to the full / particle-conserving basis -------------------
    def _pcon_basis(self):
        """The same particle sector without symmetries (rows of the pcon
        projector), built once."""
        b = getattr(self, "_basis_pcon", None)
        if b is None:
            b = object.__new__(type(self))
            b._allowed_ops = getattr(self, "_allowed_ops", set())
            b._init_general(self._N, self._sectors, blocks=None)
            b.make()
            self._basis_pcon = b
        return b

    def _proj_device(self, pcon=False):
        """Device CSC of the projector: (colptr int64[Ns+1], rows int64,
        values complex128, Ns_full).  Built once per row space."""
        if not self._made_basis:
            raise AttributeError("this function requires the basis to be constructed first; use basis.make().")
        pcon = bool(pcon) and len(self._sectors) == 1 and self._sectors[0][0] != 0
        cache = self.__dict__.setdefault("_proj_cache", {})
        if pcon in cache:
            return cache[pcon]
        gsize = int(np.prod(self._pers, dtype=np.int64)) if len(self._pers) else 1
        Ns = self._Ns
        if pcon:
            pb = self._pcon_basis()
            Ns_full = pb.Ns
            pargs = (D.ptr(pb._basis), pb.Ns, pb._N_p, D.ptr(pb._begin), D.ptr(pb._end))
        else:
            if self._N > 62:
                raise NotImplementedError("the full space of more than 62 bits has no int64 index")
            Ns_full = 2 ** self._N
            pargs = (None, 0, 0, None, None)
        colptr = torch.zeros(Ns + 1, dtype=torch.int64, device=D.device())
        err = D.err_flag()
        base = (self._sym, D.ptr(self._basis), D.ptr(self._n_dev), Ns, gsize)
        if Ns:
            # pass 1: entries per column, then offsets
            _lib.call("qs_proj_fill", *base, 0, D.ptr(colptr), int(pcon), *pargs, None, None, D.ptr(err),
                      D.stream())
            torch.cumsum(colptr[1:].clone(), 0, out=colptr[1:])
        nnz = int(colptr[-1].item())
        rows = torch.empty(max(nnz, 1), dtype=torch.int64, device=D.device())
        vals = torch.empty(max(nnz, 1), dtype=torch.complex128, device=D.device())
        if Ns:
            _lib.call("qs_proj_fill", *base, 1, D.ptr(colptr), int(pcon), *pargs, D.ptr(rows), D.ptr(vals),
                      D.ptr(err), D.stream())
            e = int(err.item())
            if e:
                raise RuntimeError("projector construction failed (error bits {})".format(e))
        cache[pcon] = (colptr, rows[:nnz], vals[:nnz], Ns_full)
        return cache[pcon]

    def get_proj(self, dtype, pcon=False):
        """Projector from the symmetry-reduced to the full basis as a
        scipy.sparse.csc_matrix (base_general.py:521-582)."""
        import scipy.sparse as sp
        colptr, rows, vals, Ns_full = self._proj_device(pcon)
        dtype = np.dtype(dtype)
        v = D.to_host(vals)
        if dtype.kind != "c":
            if np.any(np.abs(v.imag) > 1.1e-15):
                raise TypeError("attemping to use real type for complex elements.")
            v = v.real
        index_type = np.result_type(np.min_scalar_type(-Ns_full), np.int32)
        return sp.csc_matrix((v.astype(dtype), D.to_host(rows).astype(index_type),
                              D.to_host(colptr).astype(index_type)), shape=(Ns_full, self._Ns))

    def _project(self, v0, direction, pcon):
        colptr, rows, vals, Ns_full = self._proj_device(pcon)
        host = not D.is_device_array(v0)
        vdt = np.asarray(v0).dtype if host else D.np_dtype(v0.dtype)
        squeeze = v0.ndim == 1
        n_in = self._Ns if direction == 0 else Ns_full
        n_out = Ns_full if direction == 0 else self._Ns
        x = D.to_device(v0, np.complex128).reshape(n_in, -1).contiguous()
        k = x.shape[1]
        y = torch.zeros((n_out, k), dtype=torch.complex128, device=D.device())
        if self._Ns and k:
            _lib.call("qs_proj_apply", direction, self._Ns, D.ptr(colptr), D.ptr(rows), D.ptr(vals), D.ptr(x), k,
                      D.ptr(y), D.stream())
        # the reference writes into an array of v0's dtype; a real v0 whose
        # image is complex (a complex projector) is promoted instead
        rdt = vdt
        if vdt.kind != "c":
            if bool(torch.any(y.imag.abs() > 1.1e-15)):
                rdt = np.result_type(vdt, np.complex64)
            else:
                y = y.real
        y = y.to(D.torch_dtype(rdt))
        if squeeze:
            y = y.reshape(-1)
        return D.to_host(y) if host else y

    def project_from(self, v0, sparse=True, pcon=False):
        """State(s) in the symmetry-reduced basis -> full basis, one state
        per column (base_general.py:696-777)."""
        import scipy.sparse as sp
        if not self._made_basis:
            raise AttributeError("this function requires the basis to be cosntructed first, see basis.make().")
        if not hasattr(v0, "shape"):
            v0 = np.asanyarray(v0)
        if v0.ndim not in (1, 2):
            raise ValueError("excpecting v0 to have ndim > 0 and at most 2")
        if v0.shape[0] != self._Ns:
            raise ValueError("v0 shape {0} not compatible with Ns={1}".format(v0.shape, self._Ns))
        if sp.issparse(v0):
            raise ValueError
        if sparse:
            vh = D.to_host(v0) if D.is_device_array(v0) else np.ascontiguousarray(v0)
            if vh.ndim == 1:
                vh = vh.reshape(-1, 1)
            return self.get_proj(vh.dtype, pcon=pcon).dot(sp.csc_matrix(vh))
        return self._project(v0, 0, pcon)

    def get_vec(self, v0, sparse=True, pcon=False):
        """Deprecated alias of project_from (base_general.py:685-694)."""
        return self.project_from(v0, sparse=sparse, pcon=pcon)

    def project_to(self, v0, sparse=True, pcon=False):
        """State(s) in the full basis -> symmetry-reduced basis, P^dagger v0
        (base_general.py:584-683).  As in the reference, the sparse form
        multiplies by the transpose P^T without conjugation."""
        import scipy.sparse as sp
        if not self._made_basis:
            raise AttributeError("this function requires the basis to be cosntructed first, see basis.make().")
        if not hasattr(v0, "shape"):
            v0 = np.asanyarray(v0)
        if v0.ndim not in (1, 2):
            raise ValueError("excpecting v0 to have ndim > 0 and at most 2")
        Ns_full = self._proj_device(pcon)[3]
        if v0.shape[0] != Ns_full:
            raise ValueError("v0 shape {0} not compatible with Ns_full={1}".format(v0.shape, Ns_full))
        if sp.issparse(v0):
            raise ValueError
        if sparse:
            vh = D.to_host(v0) if D.is_device_array(v0) else np.ascontiguousarray(v0)
            if vh.ndim == 1:
                vh = vh.reshape(-1, 1)
            return self.get_proj(vh.dtype, pcon=pcon).T.dot(sp.csr_matrix(vh))
        return self._project(v0, 1, pcon)

    def __repr__(self):
        return "<{} N={} Ns={} blocks={}>".format(type(self).__name__, self._N, self._Ns, self._blocks)


def build_matrix(basis, op_list, dtype):
    """GPU canonical assembly of sum_t J_t op_t (base.py:265-304).

    Off-diagonal terms are summed left to right in term order per entry,
    the diagonal array added last, exact zeros dropped -- the arithmetic of the
    reference's chain of scipy CSR additions.  Returns DeviceCSR or DeviceDIA.
    """
    dtype = np.dtype(dtype)
    if dtype not in D.SUPPORTED:
        raise TypeError("hamiltonian does not support type: " + str(dtype))
    Ns = basis.Ns
    vt = D.code(dtype)
    L = _lib.load()
    st = D.stream()
    terms = [basis._term(o, ix, J) for o, ix, J in op_list]
    is_diag = [set(o) <= _DIAG_CHARS for o, _, _ in terms]
    err = D.err_flag()
    off_idx = [i for i, d in enumerate(is_diag) if not d]
    # count pass (may reclassify terms whose every element sits on the diagonal)
    rowcnt = None
    while True:
        if not off_idx or Ns == 0:
            off_idx = []
            break
        tt = _TermTable([terms[i] for i in off_idx])
        rowcnt = torch.zeros(Ns + 1, dtype=torch.int64, device=D.device())
        flags = torch.zeros(len(off_idx), dtype=torch.int32, device=D.device())
        _lib.check(L.qs_csr_count(basis._sym, vt, *basis._basis_args(), *tt.args(), tt.T, D.ptr(rowcnt),
                                  D.ptr(flags), D.ptr(err), st), "qs_csr_count")
        e = int(err.item())
        if e & 1:
            raise ValueError("unrecognized characters in operator string")
        if e & 2:
            raise TypeError("attemping to use real type for complex elements.")
        fl = D.to_host(flags)
        moved = [off_idx[k] for k in range(len(off_idx)) if (fl[k] & 1) and not (fl[k] & 2)]
        dropped = [off_idx[k] for k in range(len(off_idx)) if not (fl[k] & 1)]
        if not moved and not dropped:
            break
        for i in moved:
            is_diag[i] = True
        off_idx = [i for i in off_idx if i not in moved and i not in dropped]
    diag_idx = [i for i, d in enumerate(is_diag) if d]
    diag = None
    if diag_idx and Ns:
        ttd = _TermTable([terms[i] for i in diag_idx])
        diag = torch.empty(Ns, dtype=D.torch_dtype(dtype), device=D.device())
        dflags = torch.zeros(len(diag_idx), dtype=torch.int32, device=D.device())
        _lib.check(L.qs_csr_diag(basis._sym, vt, *basis._basis_args(), *ttd.args(), ttd.T, D.ptr(diag),
                                 D.ptr(dflags), D.ptr(err), st), "qs_csr_diag")
        e = int(err.item())
        if e & 2:
            raise TypeError("attemping to use real type for complex elements.")
        if not np.any(D.to_host(dflags) & 1):
            diag = None
    if not off_idx:
        if diag is None:
            diag = torch.zeros(max(Ns, 0), dtype=D.torch_dtype(dtype), device=D.device())
            return DeviceDIA(D.to_device(np.zeros(0, np.int64)), diag.reshape(0, Ns), (Ns, Ns), dtype)
        return DeviceDIA.from_diagonal(diag, dtype)
    tt = _TermTable([terms[i] for i in off_idx])
    if diag is not None:
        rowcnt[1:] += 1          # a spare slot per row for a diagonal entry the merge may add
    scr = torch.empty(max(L.qs_scan_scratch_elems(Ns), 1), dtype=torch.int64, device=D.device())
    _lib.call("qs_scan_inclusive_i64", D.ptr(rowcnt[1:]), Ns, D.ptr(scr), st)
    nnz_pre = int(rowcnt[-1].item())
    keys = torch.empty(max(nnz_pre, 1), dtype=torch.int64, device=D.device())
    vals = torch.empty(max(nnz_pre, 1), dtype=D.torch_dtype(dtype), device=D.device())
    cursor = torch.zeros(Ns, dtype=torch.int64, device=D.device())
    _lib.check(L.qs_csr_fill(basis._sym, vt, *basis._basis_args(), *tt.args(), tt.T, D.ptr(rowcnt), D.ptr(cursor),
                             D.ptr(keys), D.ptr(vals), D.ptr(err), st), "qs_csr_fill")
    mcount = torch.empty(Ns, dtype=torch.int64, device=D.device())
    _lib.check(L.qs_csr_merge(vt, Ns, D.ptr(rowcnt), D.ptr(cursor), D.ptr(keys), D.ptr(vals), D.ptr(diag),
                              D.ptr(mcount), D.ptr(err), st), "qs_csr_merge")
    if int(err.item()) & 8:
        raise NotImplementedError("a matrix row collects more than 512 entries before merging")
    del cursor
    _lib.call("qs_scan_inclusive_i64", D.ptr(mcount), Ns, D.ptr(scr), st)
    nnz = int(mcount[-1].item())
    idx64 = nnz >= 2**31 - 1
    indptr = torch.empty(Ns + 1, dtype=torch.int64 if idx64 else torch.int32, device=D.device())
    indices = torch.empty(max(nnz, 1), dtype=torch.int32, device=D.device())
    data = torch.empty(max(nnz, 1), dtype=D.torch_dtype(dtype), device=D.device())
    _lib.check(L.qs_csr_compact(vt, Ns, D.ptr(rowcnt), D.ptr(keys), D.ptr(vals), D.ptr(mcount), D.ptr(indptr),
                                int(idx64), D.ptr(indices), D.ptr(data), st), "qs_csr_compact")
    del keys, vals, mcount, rowcnt
    return DeviceCSR(indptr, indices[:nnz], data[:nnz], (Ns, Ns), dtype)


# ---------------------------------------------------------------------------
# user-facing classes


class spin_basis_general(basis_general):
    """Spin-1/2 basis with user-defined symmetries (spin.py:66-227).

    Only S="1/2" is supported.  pauli: 1 Pauli matrices (default), 0 spin
    operators, -1 Pauli x/y/z with unit raising/lowering.
    """

    def __init__(self, N, Nup=None, m=None, S="1/2", pauli=1, Ns_block_est=None, make_basis=True,
                 block_order=None, **blocks):
        if S != "1/2":
            raise NotImplementedError("only S='1/2' is supported")
        self._S = S
        self._pauli = int(pauli)
        if self._pauli not in (-1, 0, 1):
            raise ValueError("Invalid value for optional argument pauli. Allowed values are the integers [-1,0,1].")
        blocks.pop("_Np", None)
        if Nup is not None and m is not None:
            raise ValueError("Cannot use Nup and m at the same time")
        if m is not None and Nup is None:
            if m < -0.5 or m > 0.5:
                raise ValueError("m must be between -S and S")
            Nup = int((m + 0.5) * N)
        try:
            Nup = [(N + (n + 1) if n < 0 else n) for n in iter(Nup)]
        except TypeError:
            if Nup is not None and Nup < 0:
                Nup = N + Nup + 1
        if Nup is None:
            sectors = [(0, 0, 0)]
        elif isinstance(Nup, list):
            for b in Nup:
                if b > N or b < 0:
                    raise ValueError("particle number Nb must satisfy: 0 <= Nb <= N")
            sectors = [(1, int(b), 0) for b in Nup]
        else:
            if Nup > N or Nup < 0:
                raise ValueError("particle number Nb must satisfy: 0 <= Nb <= N")
            sectors = [(1, int(Nup), 0)]
        self._Np = Nup
        self._allowed_ops = set(["I", "+", "-", "x", "y", "z"])
        self._init_general(N, sectors, block_order=block_order, blocks=blocks)
        if make_basis:
            self.make(Ns_block_est=Ns_block_est)

    def _scale(self, opstr):
        if self._pauli == 1:
            return float(1 << len(opstr.replace("I", "")))
        if self._pauli == -1:
            return float(1 << len(opstr.replace("I", "").replace("+", "").replace("-", "")))
        return 1.0


class spin_basis_1d(spin_basis_general):
    """Spin-1/2 chain basis (src/quspin/basis/basis_1d/spin.py) on the general
    machinery: kblock -> translation by a sites, pblock -> reflection,
    zblock -> spin inversion, pzblock -> reflection times inversion."""

    def __init__(self, L, Nup=None, m=None, S="1/2", pauli=1, a=1, kblock=None, pblock=None, zblock=None,
                 pzblock=None, Ns_block_est=None, make_basis=True, **kwargs):
        sites = np.arange(L)
        blocks = {}
        if kblock is not None:
            blocks["kblock"] = ((sites + a) % L, int(kblock) % (L // a))
        if pblock is not None:
            blocks["pblock"] = (L - 1 - sites, 0 if int(pblock) == 1 else 1)
        if zblock is not None:
            blocks["zblock"] = (-(sites + 1), 0 if int(zblock) == 1 else 1)
        if pzblock is not None:
            blocks["pzblock"] = (-(L - 1 - sites) - 1, 0 if int(pzblock) == 1 else 1)
        self._L = L
        spin_basis_general.__init__(self, L, Nup=Nup, m=m, S=S, pauli=pauli, Ns_block_est=Ns_block_est,
                                    make_basis=make_basis, **blocks)

    @property
    def L(self):
        return self._N


class spinless_fermion_basis_general(basis_general):
    """Spinless fermions with user-defined symmetries (fermion.py:69-230)."""

    _fermion = True

    def __init__(self, N, Nf=None, nf=None, Ns_block_est=None, make_basis=True, block_order=None, **blocks):
        blocks.pop("_Np", None)
        if Nf is not None and nf is not None:
            raise ValueError("cannot use 'nf' and 'Nf' simultaineously.")
        if Nf is None and nf is not None:
            Nf = int(nf * N)
        if Nf is None:
            sectors = [(0, 0, 0)]
        elif isinstance(Nf, (list, tuple)):
            sectors = [(1, int(b), 0) for b in Nf]
        else:
            sectors = [(1, int(Nf), 0)]
        self._Np = Nf
        self._allowed_ops = set(["I", "n", "+", "-", "z", "x", "y"])
        self._init_general(N, sectors, block_order=block_order, blocks=blocks)
        if make_basis:
            self.make(Ns_block_est=Ns_block_est)


def process_spinful_map(N, map, q):
    """Simple (length N) -> advanced (length 2N) map (fermion.py:274-283)."""
    map = np.asarray(map, dtype=np.int32)
    if len(map) == N:
        i_map = map.copy()
        i_map[map < 0] = -(i_map[map < 0] + 1) + N
        return np.hstack((i_map, (i_map + N) % (2 * N))), q
    return map, q


class spinful_fermion_basis_general(basis_general):
    """Spinful fermions, up on sites 0..N-1 (high bits), down on N..2N-1
    (fermion.py:285-460).  Simple symmetries use "|" operator strings."""

    _fermion = True

    def __init__(self, N, Nf=None, nf=None, Ns_block_est=None, simple_symm=True, make_basis=True,
                 block_order=None, double_occupancy=True, **blocks):
        if not double_occupancy:
            raise NotImplementedError("double_occupancy=False is not supported")
        blocks.pop("_Np", None)
        if Nf is not None and nf is not None:
            raise ValueError("cannot use 'nf' and 'Nf' simultaineously.")
        if Nf is None and nf is not None:
            Nf = (int(nf[0] * N), int(nf[1] * N))
        self._simple_symm = simple_symm
        blocks = {k: v for k, v in blocks.items() if v is not None}
        if any((type(m) is not tuple) and (len(m) != 2) for m in blocks.values()):
            raise ValueError("blocks must contain tuple: (map,q).")
        if simple_symm:
            if any(len(item[0]) != N for item in blocks.values()):
                raise ValueError("Simple symmetries must have mapping of length N.")
        else:
            if any(len(item[0]) != 2 * N for item in blocks.values()):
                raise ValueError("Advanced symmetries must have mapping of length 2*N.")
        blocks = {k: process_spinful_map(N, *v) for k, v in blocks.items()}
        if Nf is None:
            sectors = [(0, 0, 0)]
        elif isinstance(Nf, tuple) and len(Nf) == 2 and all(np.isscalar(x) for x in Nf):
            sectors = [(2, int(Nf[0]), int(Nf[1]))]
        else:
            sectors = [(2, int(a), int(b)) for a, b in Nf]
        for _, a, b in sectors:
            if a > N or a < 0 or b > N or b < 0:
                raise ValueError("particle number Nf must satisfy: 0 <= Nf <= N")
        self._Np = Nf
        self._spinful = bool(simple_symm)
        self._allowed_ops = set(["I", "n", "+", "-", "z", "x", "y"])
        self._init_general(2 * N, sectors, block_order=block_order, blocks=blocks)
        if make_basis:
            self.make(Ns_block_est=Ns_block_est)
