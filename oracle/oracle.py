"""CPU oracle for the QuSpin hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference leg import this module, and only as the comparison or the timed CPU
baseline.  The product package ``quspin_gb300`` never imports it.

It restates, on the CPU, the reference's algorithm for every step of the hot
path (QuSpin 1.0.1; paths are relative to the reference project root):

* basis construction -- ``src/quspin/basis/basis_general/base_general.py``
  (``process_map`` :22-51, block sorting :135-212, ``make`` :817-899,
  ``make_basis_blocks`` :901-950, ``_Op`` :292-352) and the native core it
  calls (quspin-extensions 0.1.8, restated in ``basis_oracle.c``);
* spin-1/2 Pauli rescaling -- ``basis_general/spin.py:216-227``;
* spinful-fermion map and operator-string handling --
  ``basis_general/fermion.py:274-283`` (``process_spinful_map``) and
  ``:1080-1096`` (``_simple_to_adv``);
* matrix assembly -- ``src/quspin/basis/base.py:265-304`` (``_make_matrix``,
  run with scipy exactly as the reference does) after
  ``src/quspin/operators/_make_hamiltonian.py:19-100`` (consolidation);
* ``ExpmMultiplyParallel`` -- the reference's Python body
  (``docs/modules/parallel_sparse_tools/expm_multiply_parallel_core/
  expm_multiply_parallel_core.html:150-463``) with the four native wrappers
  restated in ``sparse_oracle.c``, and scipy's ``_fragment_3_1`` for the
  (m*, s) choice, as the reference itself calls it;
* Lanczos -- ``src/quspin/tools/lanczos/_lanczos_utils.py:77-425`` and
  ``_expm.py:7-52`` restated with numpy.

Conventions pinned here (site <-> bit, map direction, representative,
norm, phase) are listed in the header of ``basis_oracle.c``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from math import gcd

import numpy as np
import scipy.sparse as sp

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")


def build():
    """Compile the oracle library (make in oracle/)."""
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                build()
            L = ctypes.CDLL(_LIB_PATH)
            c = ctypes
            sym = [c.c_int, c.c_int, c.c_int, _i32p, _i32p, _i32p]
            L.orc_make_basis.argtypes = sym + [c.c_int, c.c_int, c.c_int, _u64p, _u32p, c.c_int64]
            L.orc_make_basis.restype = c.c_int64
            L.orc_make_blocks.argtypes = [c.c_int, c.c_int, _u64p, c.c_int64, _i64p, _i64p]
            L.orc_make_blocks.restype = None
            L.orc_index_many.argtypes = [c.c_int, c.c_int, _u64p, c.c_int64, _i64p, _i64p,
                                         _u64p, c.c_int64, _i64p]
            L.orc_index_many.restype = None
            L.orc_representative.argtypes = sym + [_u64p, c.c_int64, _u64p, c.c_void_p, c.c_void_p]
            L.orc_representative.restype = c.c_int
            L.orc_normalization.argtypes = sym + [_u64p, c.c_int64, _u32p]
            L.orc_normalization.restype = c.c_int
            L.orc_orbit.argtypes = sym + [_u64p, c.c_int64, c.c_int64, _u64p, c.c_void_p, _i32p]
            L.orc_orbit.restype = c.c_int
            opargs = sym + [_f64p, _f64p, c.c_char_p, _i32p, c.c_int, c.c_double, c.c_double,
                            _u64p, _u32p, c.c_int64, c.c_int, _i64p, _i64p]
            L.orc_op.argtypes = opargs + [_i64p, _i64p, _f64p]
            L.orc_op.restype = c.c_int
            L.orc_inplace_op.argtypes = opargs + [c.c_int, c.c_int, _f64p, _f64p, c.c_int64]
            L.orc_inplace_op.restype = c.c_int
            L.orc_csr_matvec.argtypes = [_i64p, _i32p, _f64p, c.c_int, c.c_int64, c.c_int64,
                                         c.c_double, c.c_double, _f64p, _f64p, c.c_int]
            L.orc_csr_matvec.restype = None
            L.orc_csr_trace.argtypes = [_i64p, _i32p, _f64p, c.c_int, c.c_int64, _f64p]
            L.orc_csr_trace.restype = None
            L.orc_csr_1_norm.argtypes = [_i64p, _i32p, _f64p, c.c_int, c.c_int64, c.c_double, c.c_double]
            L.orc_csr_1_norm.restype = c.c_double
            L.orc_expm_multiply.argtypes = [_i64p, _i32p, _f64p, c.c_int, c.c_int64, c.c_int64,
                                            c.c_int, c.c_int, c.c_double,
                                            c.c_double, c.c_double, c.c_double, c.c_double,
                                            c.c_double, c.c_double, _f64p, _f64p]
            L.orc_expm_multiply.restype = c.c_int64
            L.orc_expm_substep.argtypes = L.orc_expm_multiply.argtypes
            L.orc_expm_substep.restype = c.c_int64
            L.orc_build_csr.argtypes = sym + [_f64p, _f64p, c.c_int, _i32p, _i32p, c.c_char_p, _i32p, _f64p, _i32p,
                                              _u64p, _u32p, c.c_int64, c.c_int, _i64p, _i64p, c.c_int,
                                              c.POINTER(c.c_void_p), c.POINTER(c.c_void_p),
                                              c.POINTER(c.c_void_p)]
            L.orc_build_csr.restype = c.c_int64
            L.orc_free.argtypes = [c.c_void_p]
            L.orc_free.restype = None
            L.orc_num_threads.argtypes = []
            L.orc_num_threads.restype = c.c_int
            _lib = L
    return _lib


# ---------------------------------------------------------------------------
# basis


def process_map(map, q):
    """Restates base_general.py:22-51: periodicity of a site map."""
    map = np.asarray(map, dtype=np.int32)
    i_map = map.copy()
    i_map[map < 0] = -(i_map[map < 0] + 1)
    s_map = map < 0
    sites = np.arange(len(map), dtype=np.int32)
    order = sites.copy()
    if np.any(np.sort(i_map) - order):
        raise ValueError("map must be a one-to-one site mapping.")
    per = 0
    while True:
        sites[s_map] = -(sites[s_map] + 1)
        sites = sites[i_map]
        per += 1
        if np.array_equal(order, sites):
            break
    return map, per, q


def process_spinful_map(N, map, q):
    """Restates fermion.py:274-283: simple (length N) -> advanced (2N) map."""
    map = np.asarray(map, dtype=np.int32)
    if len(map) == N:
        i_map = map.copy()
        i_map[map < 0] = -(i_map[map < 0] + 1) + N
        return np.hstack((i_map, (i_map + N) % (2 * N))), q
    return map, q


def phase_table(L):
    """exp(-2 pi i p / L), p = 0..L-1, exact on the quarter points."""
    p = np.arange(L)
    t = np.exp(-2j * np.pi * p / L)
    for k in range(L):
        if k == 0:
            t[k] = 1.0
        elif 4 * k == L:
            t[k] = -1j
        elif 2 * k == L:
            t[k] = -1.0
        elif 4 * k == 3 * L:
            t[k] = 1j
    return np.ascontiguousarray(t.real), np.ascontiguousarray(t.imag)


class OracleBasis:
    """CPU restatement of ``basis_general`` for spin-1/2 and fermions.

    sectors: list of (kind, p0, p1) -- kind 0 all words, 1 fixed popcount p0,
    2 spinful (p0 up in the high half, p1 down in the low half).
    blocks: name -> (map, q) with per-bit maps (spinful maps already in the
    advanced 2N form).
    """

    def __init__(self, N, sectors, fermion=False, block_order=None, N_p=None,
                 pauli=0, spinful=False, **blocks):
        self.N = N
        self.fermion = bool(fermion)
        self.pauli = pauli
        self.spinful = spinful
        blocks = {k: v for k, v in blocks.items() if v is not None}
        items = {k: process_map(*v) for k, v in blocks.items()}
        if block_order is None:
            sorted_items = sorted(items.items(), key=lambda x: x[1][1])
        else:
            bo = list(block_order)
            bo.reverse()
            sorted_items = [(k, items[k]) for k in bo]
        remove_index = [i for i, it in enumerate(sorted_items[:-1]) if it[1][1] == 1]
        kept = [it for _, it in sorted_items]
        for i in sorted(remove_index):
            kept.pop(i)
        if kept:
            self.maps = np.ascontiguousarray(np.vstack([m for m, _, _ in kept]), dtype=np.int32)
            self.pers = np.asarray([p for _, p, _ in kept], dtype=np.int32)
            self.qs = np.asarray([q for _, _, q in kept], dtype=np.int32)
        else:
            self.maps = np.zeros((0, N), dtype=np.int32)
            self.pers = np.zeros(0, dtype=np.int32)
            self.qs = np.zeros(0, dtype=np.int32)
        L = 1
        for p in self.pers:
            L = L // gcd(L, int(p)) * int(p)
        self.L = L
        self.phase_re, self.phase_im = phase_table(L)
        self.sectors = list(sectors)
        self._make(N_p)

    def _symargs(self):
        return (self.N, int(self.fermion), len(self.pers), self.maps.reshape(-1) if self.maps.size else
                np.zeros(1, np.int32), self.pers if self.pers.size else np.zeros(1, np.int32),
                self.qs if self.qs.size else np.zeros(1, np.int32))

    def _make(self, N_p):
        L = lib()
        all_s, all_n = [], []
        for kind, p0, p1 in self.sectors:
            cap = 1 << 16
            while True:
                st = np.zeros(cap, dtype=np.uint64)
                nm = np.zeros(cap, dtype=np.uint32)
                ns = L.orc_make_basis(*self._symargs(), kind, p0, p1, st, nm, cap)
                if ns == -2:
                    raise ValueError("unsupported symmetry map for this basis")
                if ns < -1:
                    cap = -1 - ns
                    continue
                break
            all_s.append(st[:ns])
            all_n.append(nm[:ns])
        states = np.concatenate(all_s) if all_s else np.zeros(0, np.uint64)
        norms = np.concatenate(all_n) if all_n else np.zeros(0, np.uint32)
        if len(self.sectors) > 1:
            order = np.argsort(states, kind="stable")[::-1]
            states, norms = states[order], norms[order]
        self.states = np.ascontiguousarray(states)
        self.norms = np.ascontiguousarray(norms)
        self.Ns = len(states)
        if N_p is None:
            N_p = int(np.floor(np.log(self.Ns // 2 + 1) / np.log(2)))
        if len(self.pers) == 0 and all(k == 0 for k, _, _ in self.sectors):
            N_p = 0
        self.N_p = min(max(int(N_p), 0), self.N)
        nb = 1 << self.N_p
        self.begin = np.zeros(nb, dtype=np.int64)
        self.end = np.zeros(nb, dtype=np.int64)
        if self.N_p > 0:
            L.orc_make_blocks(self.N, self.N_p, self.states, self.Ns, self.begin, self.end)

    # -- queries ---------------------------------------------------------
    def index(self, states):
        q = np.ascontiguousarray(np.atleast_1d(states), dtype=np.uint64)
        out = np.zeros(len(q), dtype=np.int64)
        lib().orc_index_many(self.N, self.N_p, self.states, self.Ns, self.begin, self.end, q, len(q), out)
        return out

    def representative(self, states):
        s = np.ascontiguousarray(np.atleast_1d(states), dtype=np.uint64)
        out = np.zeros_like(s)
        K = len(self.pers)
        g = np.zeros((len(s), max(K, 1)), dtype=np.int32)
        sg = np.zeros(len(s), dtype=np.int8)
        lib().orc_representative(*self._symargs(), s, len(s), out,
                                 g.ctypes.data_as(ctypes.c_void_p), sg.ctypes.data_as(ctypes.c_void_p))
        return out, g[:, :K], sg

    def normalization(self, states):
        s = np.ascontiguousarray(np.atleast_1d(states), dtype=np.uint64)
        out = np.zeros(len(s), dtype=np.uint32)
        lib().orc_normalization(*self._symargs(), s, len(s), out)
        return out

    def get_proj(self, dtype, pcon_basis=None):
        """Restates basis.get_proj (base_general.py:521-582): column i is
        sum_g chi(g) sign(g) |g s_i> / sqrt(n_i |G|), duplicate images summed
        (scipy CSC), images whose unit-phase sum is at most 1e-12 dropped.
        Rows: 2^N - 1 - state, or the index in pcon_basis."""
        G = int(np.prod(self.pers, dtype=np.int64)) if len(self.pers) else 1
        n = self.Ns
        images = np.zeros(n * G, np.uint64)
        signs = np.zeros(n * G, np.int8)
        phases = np.zeros(n * G, np.int32)
        rc = lib().orc_orbit(*self._symargs(), self.states, n, G, images, signs.ctypes.data_as(ctypes.c_void_p),
                             phases)
        if rc:
            raise ValueError("unsupported symmetry map")
        c = 1.0 / np.sqrt(self.norms.astype(np.float64) * G)
        unit = (self.phase_re[phases] + 1j * self.phase_im[phases]) * signs
        cols = np.repeat(np.arange(n), G)
        if pcon_basis is None:
            Ns_full = 2 ** self.N
            rows = (Ns_full - 1) - images.astype(np.int64)
        else:
            Ns_full = pcon_basis.Ns
            rows = pcon_basis.index(images)
        P = sp.csc_matrix((unit, (rows, cols)), shape=(Ns_full, n))
        P.sum_duplicates()
        # images whose summed unit phases cancel (maps that do not commute)
        P.data[np.abs(P.data) <= 1e-12] = 0.0
        P.eliminate_zeros()
        P = sp.csc_matrix(P @ sp.diags(c))
        dtype = np.dtype(dtype)
        return P.astype(dtype) if dtype.kind == "c" else sp.csc_matrix(P.real.astype(dtype))

    def get_amp(self, states, mode="representative"):
        """Restates basis.get_amp (base_general.py:1183-1269): the factor C with
        psi_s = C psi^sym_r for a state s and its representative r; 0 outside
        the sector.  'representative': states are representatives (C = sqrt(n/|G|));
        'full_basis': states are full-basis states, C = sqrt(n_r/|G|) conj(chi(g))
        sign(g) for the first group element g taking s to r.  Returns (C, r)."""
        s = np.ascontiguousarray(np.atleast_1d(states), dtype=np.uint64)
        G = int(np.prod(self.pers, dtype=np.int64)) if len(self.pers) else 1
        if mode == "representative":
            n = self.normalization(s).astype(np.float64)
            return np.sqrt(n / G).astype(np.complex128), s
        if mode != "full_basis":
            raise ValueError("mode accepts only the values 'representative' and 'full_basis'.")
        r, g, sg = self.representative(s)
        n = self.normalization(r).astype(np.float64)
        steps = np.asarray([(int(q) * (self.L // int(p))) % self.L for q, p in zip(self.qs, self.pers)], np.int64)
        ph = (g.astype(np.int64) @ steps) % self.L if len(steps) else np.zeros(len(s), np.int64)
        chi = self.phase_re[ph] + 1j * self.phase_im[ph]
        return np.sqrt(n / G) * np.conj(chi) * sg, r

    # -- operators -------------------------------------------------------
    def _prep(self, opstr, indx, J):
        indx = list(indx)
        if self.spinful and "|" in opstr:
            i = opstr.index("|")
            half = self.N // 2
            indx = indx[:i] + [j + half for j in indx[i:]]
            opstr = opstr.replace("|", "", 1)
        if not self.fermion and self.pauli == 1:
            J = J * (1 << len(opstr.replace("I", "")))
        elif not self.fermion and self.pauli == -1:
            J = J * (1 << len(opstr.replace("I", "").replace("+", "").replace("-", "")))
        return opstr, np.asarray(indx, dtype=np.int32), complex(J)

    def op_raw(self, opstr, indx, J):
        """(ME complex128[Ns], row int64[Ns], col int64[Ns]) before masking."""
        opstr, indx, J = self._prep(opstr, indx, J)
        if len(opstr) != len(indx):
            raise ValueError("length of opstr does not match length of indx")
        Ns = self.Ns
        row = np.zeros(Ns, dtype=np.int64)
        col = np.zeros(Ns, dtype=np.int64)
        me = np.zeros(2 * Ns, dtype=np.float64)
        rc = lib().orc_op(*self._symargs(), self.phase_re, self.phase_im, opstr.encode(), indx, len(indx),
                          J.real, J.imag, self.states, self.norms, Ns, self.N_p, self.begin, self.end,
                          row, col, me)
        if rc == -1:
            raise ValueError("unrecognized characters in operator string {}".format(opstr))
        return me.view(np.complex128), row, col

    def Op(self, opstr, indx, J, dtype):
        """Restates basis_general._Op (base_general.py:292-352) incl. masking."""
        ME, row, col = self.op_raw(opstr, indx, J)
        dtype = np.dtype(dtype)
        if not np.iscomplexobj(np.zeros(1, dtype)):
            if np.any(np.abs(ME.imag) > 1.1e-15 * np.maximum(1.0, np.abs(ME.real))):
                raise TypeError("attemping to use real type for complex matrix elements.")
            ME = ME.real.astype(dtype)
        else:
            ME = ME.astype(dtype)
        mask = ME != 0
        return ME[mask], row[mask], col[mask]

    def make_matrix(self, op_list, dtype):
        """Restates basis._make_matrix (base.py:265-304) with scipy."""
        off_diag = None
        diag = None
        Ns = self.Ns
        itype = np.int32 if Ns < np.iinfo(np.int32).max else np.int64
        for opstr, indx, J in op_list:
            ME, row, col = self.Op(opstr, indx, J, dtype)
            if len(ME) > 0:
                row = row.astype(itype)
                col = col.astype(itype)
                if np.array_equal(row, col):
                    if diag is None:
                        diag = np.zeros(Ns, dtype=dtype)
                    np.add.at(diag, row, ME)
                else:
                    m = sp.csr_matrix((ME, (row, col)), shape=(Ns, Ns), dtype=dtype)
                    off_diag = m if off_diag is None else off_diag + m
        if diag is not None and off_diag is not None:
            indptr = np.arange(Ns + 1)
            return off_diag + sp.csr_matrix((diag, indptr[:Ns], indptr), shape=(Ns, Ns), dtype=dtype)
        if off_diag is not None:
            return off_diag
        if diag is not None:
            return sp.dia_matrix((np.atleast_2d(diag), [0]), shape=(Ns, Ns), dtype=dtype)
        return sp.dia_matrix((Ns, Ns), dtype=dtype)

    def build_csr(self, op_list, dtype):
        """make_matrix without scipy's pairwise additions (same arithmetic;
        C + OpenMP), for large sectors.  float64 / complex128 only."""
        dtype = np.dtype(dtype)
        terms = [self._prep(o, ix, J) for o, ix, J in op_list]
        T = len(terms)
        nop = np.asarray([len(o) for o, _, _ in terms], np.int32)
        off = np.concatenate([[0], np.cumsum(nop)[:-1]]).astype(np.int32)
        chrs = "".join(o for o, _, _ in terms).encode()
        site = np.concatenate([ix for _, ix, _ in terms]).astype(np.int32) if T else np.zeros(1, np.int32)
        J = np.asarray([[complex(j).real, complex(j).imag] for _, _, j in terms], np.float64).reshape(-1)
        is_diag = np.asarray([int(set(o) <= set("Izn")) for o, _, _ in terms], np.int32)
        ip, ix_, dt = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        real = int(dtype.kind != "c")
        nnz = lib().orc_build_csr(*self._symargs(), self.phase_re, self.phase_im, T, nop, off, chrs, site, J,
                                  is_diag, self.states, self.norms, self.Ns, self.N_p, self.begin, self.end, real,
                                  ctypes.byref(ip), ctypes.byref(ix_), ctypes.byref(dt))
        if nnz < 0:
            raise ValueError("bad operator string or symmetry map")
        Ns = self.Ns
        indptr = np.ctypeslib.as_array(ctypes.cast(ip, ctypes.POINTER(ctypes.c_int64)), (Ns + 1,)).copy()
        indices = np.ctypeslib.as_array(ctypes.cast(ix_, ctypes.POINTER(ctypes.c_int32)), (max(nnz, 1),))[:nnz].copy()
        vals = np.ctypeslib.as_array(ctypes.cast(dt, ctypes.POINTER(ctypes.c_double)),
                                     ((1 if real else 2) * max(nnz, 1),)).copy()
        for p_ in (ip, ix_, dt):
            lib().orc_free(p_)
        data = vals[:nnz] if real else vals[:2 * nnz].view(np.complex128)
        itype = np.int32 if nnz < 2**31 - 1 else np.int64
        return sp.csr_matrix((data.astype(dtype), indices, indptr.astype(itype)), shape=(Ns, Ns))

    def inplace_op(self, v_in, op_list, dtype, transposed=False, conjugated=False, a=1.0):
        v = np.asarray(v_in)
        squeeze = v.ndim == 1
        v = v.reshape(self.Ns, -1).astype(np.complex128)
        out = np.zeros_like(v)
        vin = np.ascontiguousarray(v).view(np.float64).reshape(-1)
        vout = out.view(np.float64).reshape(-1)
        for opstr, indx, J in op_list:
            o, ix, Jc = self._prep(opstr, indx, a * J)
            rc = lib().orc_inplace_op(*self._symargs(), self.phase_re, self.phase_im, o.encode(), ix,
                                      len(ix), Jc.real, Jc.imag, self.states, self.norms, self.Ns,
                                      self.N_p, self.begin, self.end, int(transposed), int(conjugated),
                                      vin, vout, v.shape[1])
            if rc:
                raise ValueError("bad operator string")
        res = out.astype(np.result_type(dtype, v_in.dtype))
        return res.ravel() if squeeze else res


def consolidate_static(static_list):
    """Restates _make_hamiltonian._consolidate_static (:19-41)."""
    eps = 10 * np.finfo(np.float64).eps
    d = {}
    for opstr, bonds in static_list:
        dd = d.setdefault(opstr, {})
        for bond in bonds:
            J = bond[0]
            indx = tuple(bond[1:])
            dd[indx] = dd[indx] + J if indx in dd else J
    out = []
    for opstr, dd in d.items():
        for indx, J in dd.items():
            if np.abs(J) > eps:
                out.append((opstr, indx, J))
    return out


def make_static(basis, static_list, dtype):
    return basis.make_matrix(consolidate_static(static_list), dtype)


# ---------------------------------------------------------------------------
# sparse tools


def _csr_parts(A):
    A = sp.csr_matrix(A)
    indptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
    indices = np.ascontiguousarray(A.indices, dtype=np.int32)
    if np.iscomplexobj(A.data):
        data = np.ascontiguousarray(A.data, dtype=np.complex128).view(np.float64)
        cplx = 1
    else:
        data = np.ascontiguousarray(A.data, dtype=np.float64)
        cplx = 0
    return indptr, indices, data, cplx, A.shape[0]


def csr_matvec(A, x, a=1.0, out=None, overwrite=True):
    indptr, indices, data, cplx, n = _csr_parts(A)
    x = np.ascontiguousarray(x, dtype=np.complex128)
    nvec = 1 if x.ndim == 1 else x.shape[1]
    y = np.zeros_like(x) if out is None else out
    a = complex(a)
    lib().orc_csr_matvec(indptr, indices, data, cplx, n, nvec, a.real, a.imag,
                         x.view(np.float64).reshape(-1), y.view(np.float64).reshape(-1), int(overwrite))
    return y


def csr_trace(A):
    indptr, indices, data, cplx, n = _csr_parts(A)
    out = np.zeros(2)
    lib().orc_csr_trace(indptr, indices, data, cplx, n, out)
    return complex(out[0], out[1])


def csr_1_norm(A, shift):
    indptr, indices, data, cplx, n = _csr_parts(A)
    shift = complex(shift)
    return lib().orc_csr_1_norm(indptr, indices, data, cplx, n, shift.real, shift.imag)


def num_threads():
    return lib().orc_num_threads()


class ExpmMultiplyParallelOracle:
    """The reference's ExpmMultiplyParallel (expm_multiply_parallel_core.html
    :150-463) with its native wrappers restated in sparse_oracle.c."""

    def __init__(self, A, a=1.0, dtype=None):
        from scipy.sparse.linalg._expm_multiply import _fragment_3_1  # as the reference does
        self._fragment_3_1 = _fragment_3_1
        self._a = a
        self._A = sp.csr_matrix(A)
        a_dtype_min = np.min_scalar_type(self._a)
        if dtype is None:
            self._dtype = np.result_type(A.dtype, a_dtype_min, np.float64)
        else:
            self._dtype = dtype
        self._tol = np.finfo(self._dtype).eps / 2
        tr = csr_trace(self._A)
        if np.dtype(self._dtype).kind != "c":
            tr = tr.real
        self._mu = np.array(tr / self._A.shape[0], dtype=self._dtype)
        self._A_1_norm = csr_1_norm(self._A, -complex(self._mu))
        self._calculate_partition()

    def _calculate_partition(self):
        if np.abs(self._a) * self._A_1_norm == 0:
            self._m_star, self._s = 0, 1
        else:
            info = _LazyNormInfo(self._A, self._A_1_norm, self._a, self._mu, self._dtype)
            self._m_star, self._s = self._fragment_3_1(info, 1, self._tol, ell=2)

    def dot(self, v, tol=None):
        v = np.array(v, dtype=np.result_type(self._dtype, np.asarray(v).dtype), copy=True, order="C")
        out = np.ascontiguousarray(v, dtype=np.complex128)
        nvec = 1 if out.ndim == 1 else out.shape[1]
        work = np.zeros(2 * out.size, dtype=np.complex128)
        tol = self._tol if tol is None else tol
        indptr, indices, data, cplx, n = _csr_parts(self._A)
        a = complex(self._a)
        mu = complex(self._mu)
        eta = np.exp(a * mu / self._s)
        self.terms = lib().orc_expm_multiply(indptr, indices, data, cplx, n, nvec, int(self._s),
                                             int(self._m_star), float(tol), mu.real, mu.imag, a.real,
                                             a.imag, eta.real, eta.imag,
                                             out.view(np.float64).reshape(-1),
                                             work.view(np.float64).reshape(-1))
        return out.astype(v.dtype) if not np.iscomplexobj(v) else out


class _LazyNormInfo:
    """LazyOperatorNormInfo (html :399-463): onenormest of powers of a(A - mu)."""

    def __init__(self, A, A_1_norm, a, mu, dtype, ell=2):
        self._A, self._a, self._mu, self._dtype = A, a, mu, dtype
        self._A_1_norm = A_1_norm
        self._ell = ell
        self._d = {}
        self._op = None

    def onenorm(self):
        return np.abs(self._a) * self._A_1_norm

    def _linop(self):
        """a (A - mu I) and its adjoint, the products by the OpenMP CSR
        kernel of sparse_oracle.c (one or several columns)."""
        from scipy.sparse.linalg import LinearOperator
        if self._op is None:
            A, a, mu = self._A, complex(self._a), complex(self._mu)
            AH = sp.csr_matrix(A.transpose().conj())
            dt = np.result_type(self._dtype, np.complex128)

            def mv(M, c, m, v):
                v = np.asarray(v)
                y = csr_matvec(M, v)
                return c * (y - m * v.astype(dt))
            self._op = LinearOperator(A.shape, dtype=self._dtype, matvec=lambda v: mv(A, a, mu, v),
                                      matmat=lambda V: mv(A, a, mu, V),
                                      rmatvec=lambda v: mv(AH, np.conj(a), np.conj(mu), v),
                                      rmatmat=lambda V: mv(AH, np.conj(a), np.conj(mu), V))
        return self._op

    def d(self, p):
        from scipy.sparse.linalg import onenormest
        if p not in self._d:
            self._d[p] = onenormest(self._linop() ** p) ** (1.0 / p)
        return self._d[p]

    def alpha(self, p):
        return max(self.d(p), self.d(p + 1))


# ---------------------------------------------------------------------------
# Lanczos (restates _lanczos_utils.py:77-227, :230-351, :366-425, _expm.py:51-52)


def lanczos_full(A_dot, dtype_A, v0, m, full_ortho=False, eps=None):
    v0 = np.asanyarray(v0)
    n = v0.size
    dtype = np.result_type(dtype_A, v0.dtype)
    Q = np.zeros((m, n), dtype=dtype)
    Q[0, :] = v0[:]
    v = np.zeros_like(v0, dtype=dtype)
    r = np.zeros_like(v0, dtype=dtype)
    b = np.zeros((m,), dtype=v.real.dtype)
    a = np.zeros((m,), dtype=v.real.dtype)
    if eps is None:
        eps = np.finfo(dtype).eps
    q_norm = np.linalg.norm(Q[0, :])
    if np.abs(q_norm - 1.0) > eps:
        np.divide(Q[0, :], q_norm, out=Q[0, :])
    r[:] = A_dot(Q[0, :])
    a[0] = np.vdot(Q[0, :], r).real
    r += -a[0] * Q[0, :]
    b[0] = np.linalg.norm(r)
    for i in range(1, m):
        v[:] = Q[i - 1, :]
        np.divide(r, b[i - 1], out=Q[i, :])
        r[:] = A_dot(Q[i, :])
        r += -b[i - 1] * v
        a[i] = np.vdot(Q[i, :], r).real
        r += -a[i] * Q[i, :]
        b[i] = np.linalg.norm(r)
        if b[i] < eps:
            m = i
            break
    if full_ortho:
        q, _ = np.linalg.qr(Q[:m].T)
        Q[:m, :] = q.T[...]
        h = np.zeros((m, m), dtype=a.dtype)
        for i in range(m):
            r[:] = A_dot(Q[i, :])
            np.conj(r, out=r)
            h[i, i:] = np.dot(Q[i:m, :], r).real
        E, V = np.linalg.eigh(h, UPLO="U")
    else:
        from scipy.linalg import eigh_tridiagonal
        E, V = eigh_tridiagonal(a[:m], b[: m - 1])
    return E, V, Q[:m], a[:m], b[:m]


def lin_comb_Q_T(coeff, Q_T):
    out = np.multiply(Q_T[0], coeff[0])
    for w, q in zip(coeff[1:], Q_T[1:]):
        out += w * q
    return out


def expm_lanczos(E, V, Q_T, a=1.0):
    c = V.dot(np.exp(a * E) * V[0, :])
    return lin_comb_Q_T(c, Q_T)


def ftlm_static_iteration(O_dict, E, V, Q_T, beta=0):
    """Finite-temperature Lanczos, one random start (reference
    src/quspin/tools/lanczos/_FTLM.py:10-109): with p(beta, j) = exp(-beta E_j)
    and c[a] = sum_j V[0, j] V[a, j] p(beta, j), the iteration returns
    sum_a c[a] <q_a | O q_0> for every operator and the identity term c[0]."""
    E = np.asarray(E)
    V = np.asarray(V)
    Q = np.asarray(Q_T)
    p = np.exp(-np.outer(np.atleast_1d(beta), E))
    c = np.einsum("j,aj,...j->a...", V[0, :], V, p)
    r = Q[0]
    res = {}
    for key, A in O_dict.items():
        Ar = A @ r
        res[key] = np.squeeze(sum(c[i, ...] * np.vdot(Q[i], Ar) for i in range(Q.shape[0])))
    return res, np.squeeze(c[0, ...])


def ltlm_static_iteration(O_dict, E, V, Q_T, beta=0):
    """Low-temperature Lanczos, one random start (reference
    src/quspin/tools/lanczos/_LTLM.py:9-139): the Krylov states whose
    Boltzmann weight at the smallest beta is below machine epsilon are
    dropped (nv), the operator's matrix in the kept Lanczos basis,
    Ome[i, j] = <q_j | O q_i>, is rotated to the Ritz basis and weighted by
    c_j = V[0, j] exp(-beta E_j / 2) on both sides; the identity term is
    sum_j V[0, j]^2 exp(-beta E_j)."""
    E = np.asarray(E)
    V = np.asarray(V)
    Q = np.asarray(Q_T)
    nv = E.size
    beta = np.atleast_1d(beta)
    p = np.exp(-E * beta.min()) * np.abs(V[0, :]).max()
    mask = p < np.finfo(p.dtype).eps
    if np.any(mask):
        nv = int(np.argmax(mask))
    res = {}
    for key, A in O_dict.items():
        AQ = np.stack([A @ Q[i] for i in range(nv)], axis=0)          # rows: O q_i
        Ome = (AQ @ Q[:nv].conj().T)                                   # [i, j] = <q_j | O q_i>
        Vn = V[:nv, :nv]
        pp = np.exp(-np.outer(E[:nv], beta / 2.0))
        c = np.einsum("j,j...->j...", Vn[0, :], pp)
        A_diag = Vn.T.dot(Ome.dot(Vn))
        res[key] = np.squeeze(np.einsum("j...,l...,jl->...", c, c, A_diag))
    p = np.exp(-np.outer(E[:nv], beta))
    Id = np.einsum("j,j...->...", V[:nv, :nv][0, :] ** 2, p)
    return res, np.squeeze(Id)
