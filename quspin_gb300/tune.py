"""Launch-shape autotuner for the CSR kernels.

The SpMV and Taylor-term kernels take a launch shape (G lanes per row,
U entries in flight per lane).  The best shape depends on the row-length
distribution and on how the gathers of the vector spread over L2, so it is
measured: a handful of candidate shapes around the nnz/row heuristic are timed
with CUDA events on the actual matrix and the fastest is kept on the matrix
object.  Matrices smaller than ``MIN_ROWS`` keep the heuristic shape.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _device as D
from . import _lib

MIN_ROWS = 65536


def encode(G, U):
    return int(G) | (int(U) << 8)


def _candidates(n, nnz, nvec):
    """Shapes to time: 2, 4, 8 lanes per row (16 / 32 for long rows) x 1, 2, 4
    entries in flight (one column) -- gathers of random columns favour few
    lanes per row."""
    avg = nnz / max(n, 1)
    Gs = [2, 4, 8] + ([16] if avg >= 32 else []) + ([32] if avg >= 64 else [])
    Us = (1, 2, 4) if nvec == 1 else (1,)
    return [(G, U) for G in Gs for U in Us]


def occ_candidates(M, nvec, btype):
    """Shapes also timed with the registers capped for 6 / 8 resident blocks
    per SM (bits 18-19 of the launch code): single-vector float-pair terms
    with int32 indices."""
    if nvec != 1 or btype != _lib.CPF or getattr(M, "idx64", 0):
        return []
    return [(G, U) for G in (2, 4) for U in (1, 2)]


def r32_candidates(M, nvec, btype):
    """Shapes of the single-vector Taylor terms of csrc/expm_st.cu (bits 20-22
    of the launch code: 1..3 the 32-row kernel with 4, 2 or 8 lanes per row in
    the gather loop, 4..5 the persistent row-handout kernel with 2 or 4 lanes
    per row, 6..7 the same with the packed column words read four per load;
    bits 18-19: 0 / 1 for 4 / 6 resident blocks per SM, 2 for 5 in the
    row-handout kernel): one vector, float forms, int32 indices."""
    if nvec != 1 or btype == _lib.C128 or getattr(M, "idx64", 0):
        return []
    if M.vcode not in (_lib.PF8, _lib.CPF8, _lib.PF8P, _lib.CPF8P, _lib.PF, _lib.CPF, _lib.F32, _lib.C64):
        return []
    cands = [(shape, occ) for shape in (1, 2, 3, 4, 5) for occ in (0, 1)]
    if M.vcode in (_lib.PF8P, _lib.CPF8P) and getattr(M, "padded", False):
        cands += [(shape, occ) for shape in (6, 7) for occ in (0, 1, 2)]
    return cands


def _time(fn, reps=5):
    st = torch.cuda.current_stream()
    for _ in range(2):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        fn()
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_spmv(M, nvec=1, xdtype=np.complex128, precision="double", operand=None):
    """Fastest launch code for M.matvec_into with nvec columns of xdtype, on
    the given float-pair operand (plain, coded or packed; timed with that
    operand pinned, so the products of the tuning do not switch it)."""
    key = ("spmv", nvec, np.dtype(xdtype).str, precision, getattr(operand, "vcode", None))
    cache = M.__dict__.setdefault("_tuned", {})
    if key in cache:
        return cache[key]
    n = M.shape[0]
    if n < MIN_ROWS or getattr(M, "idx64", 0):
        cache[key] = 0
        return 0
    shape = (n,) if nvec == 1 else (n, nvec)
    x = torch.ones(shape, dtype=D.torch_dtype(xdtype), device=D.device())
    y = torch.empty_like(x)
    best, best_t = 0, None
    codes = [encode(G, U) for G, U in _candidates(n, M.nnz, nvec)]
    if (nvec == 1 and np.dtype(xdtype).kind == "c" and getattr(operand, "padded", False)
            and getattr(operand, "vcode", None) in (_lib.PF8P, _lib.CPF8P)):
        codes += [encode(G, 1) | (6 << 20) for G in (2, 4)]      # column words read four per load
    for code in codes:
        t = _time(lambda: M.matvec_into(x, y, group=code, precision=precision, operand=operand))
        if best_t is None or t < best_t:
            best, best_t = code, t
    cache[key] = best
    return best


def tune_taylor(M, nvec, btype):
    """Fastest launch code for the fused Taylor term on M (stopping test off)."""
    key = ("taylor", nvec, btype)
    cache = M.__dict__.setdefault("_tuned", {})
    if key in cache:
        return cache[key]
    n = M.shape[0]
    if n < MIN_ROWS or getattr(M, "idx64", 0):
        cache[key] = 0
        return 0
    bdt = torch.complex64 if btype == _lib.C64 else torch.complex128
    b0 = torch.ones(n * nvec, dtype=bdt, device=D.device())
    b1 = torch.empty_like(b0)
    F = torch.zeros(n * nvec, dtype=torch.complex128, device=D.device())
    ctl = torch.zeros(max(_lib.load().qs_expm_ctl_bytes() // 8, 1) + 1, dtype=torch.int64, device=D.device())
    coeff = torch.tensor([1e-3 + 0j], dtype=torch.complex128, device=D.device())
    best, best_t = 0, None
    cands = [(G, U, 0) for G, U in _candidates(n, M.nnz, nvec)]
    rown = None
    if btype != _lib.C128 and nvec > 8:
        # chunk-outer sweeps of 4 vectors keep a narrower slice of B in L2
        # (8-vector sweeps never beat the one-sweep order in measurements)
        cands += [(G, U, 3) for G, U, _ in cands]
        rown = torch.empty(2 * n, dtype=torch.float64, device=D.device())
    cands += [(G, U, occ << 2) for G, U in occ_candidates(M, nvec, btype) for occ in (1, 2)]
    if nvec > 1 and btype != _lib.C128:
        # the vectors-across-lanes kernel (csrc/expm_vl.cu), three shapes
        cands += [(2, 2, shape << 4) for shape in (1, 2, 3)]
    if getattr(M, "vcode", None) in (_lib.PF8P, _lib.CPF8P):
        cands = []                 # the packed form runs only in the single-vector kernels
    cands += [({1: 4, 2: 2, 3: 8, 4: 2, 5: 4, 6: 2, 7: 4}[shape], 2, (shape << 4) | (occ << 2))
              for shape, occ in r32_candidates(M, nvec, btype)]
    for G, U, ch in cands:
        code = encode(G, U) | (ch << 16)

        def run():
            _lib.call("qs_taylor_term_rows", n, M.nnz, D.ptr(M.indptr), M.idx64, D.ptr(M.indices), D.ptr(M.data),
                      M.vcode, D.ptr(b0), D.ptr(b1), btype, D.ptr(F), nvec, 0.0, 0.0, D.ptr(coeff), 0, 0.0,
                      D.ptr(ctl), code, D.ptr(rown), D.stream())
        t = _time(run)
        if best_t is None or t < best_t:
            best, best_t = code, t
    cache[key] = best
    M.__dict__.setdefault("_tuned_ms", {})[key] = best_t
    return best
