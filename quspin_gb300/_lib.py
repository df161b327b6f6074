"""ctypes binding of libqsgpu.so (the sm_103a kernels of this package).

The library is built in-tree by ``__graft_entry__.build()`` (``make`` in
``quspin_gb300/csrc``) into ``quspin_gb300/_lib/libqsgpu.so``.  There is no
CPU fallback: every public operation of the package runs through this
library and raises if it is missing or if no CUDA device is present.
"""
from __future__ import annotations

import ctypes
import os
import threading

_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
LIB_PATH = os.path.join(_DIR, "libqsgpu.so")

_lib = None
_lock = threading.Lock()

# element type codes shared with the C side
F32, F64, C64, C128, PF, CPF, PF8, CPF8, PF8P, CPF8P = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9

STATUS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "unrecognized character in operator string",
    -4: "complex matrix element in a real dtype",
    -5: "output buffer too small",
    -6: "unsupported configuration",
    -7: "iteration cap reached without convergence",
}

_vp = ctypes.c_void_p
_i = ctypes.c_int
_i64 = ctypes.c_int64
_d = ctypes.c_double

# name -> (restype, argtypes)
_SIGS = {
    "qs_sym_create": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, ctypes.POINTER(_vp)]),
    "qs_sym_destroy": (_i, [_vp]),
    "qs_scan_scratch_elems": (_i64, [_i64]),
    "qs_scan_inclusive_i64": (_i, [_vp, _i64, _vp, _vp]),
    "qs_enum_num_candidates": (_i64, [_i, _i, _i, _i]),
    "qs_enum_num_chunks": (_i64, [_i, _i, _i, _i]),
    "qs_enum_count": (_i, [_vp, _i, _i, _i, _vp, _i64, _vp, ctypes.POINTER(_i64), _vp]),
    "qs_enum_write": (_i, [_vp, _i, _i, _i, _vp, _i64, _vp, _vp, _vp]),
    "qs_make_blocks": (_i, [_i, _i, _i, _vp, _i64, _vp, _vp, _vp]),
    "qs_index": (_i, [_i, _i, _vp, _i64, _i, _vp, _vp, _vp, _i64, _vp, _vp]),
    "qs_representative": (_i, [_vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    "qs_normalization": (_i, [_vp, _vp, _i64, _vp, _vp]),
    "qs_op": (_i, [_vp, _vp, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qs_csr_count": (_i, [_vp, _i, _vp, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp]),
    "qs_csr_fill": (_i, [_vp, _i, _vp, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp,
                         _vp, _vp]),
    "qs_csr_diag": (_i, [_vp, _i, _vp, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp]),
    "qs_csr_merge": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qs_csr_compact": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp]),
    "qs_csr_t_count": (_i, [_i64, _vp, _i, _vp, _vp, _vp]),
    "qs_csr_t_fill": (_i, [_i, _i64, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qs_inplace_op": (_i, [_vp, _vp, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _d, _vp,
                           _vp, _i64, _vp, _vp]),
    "qs_proj_fill": (_i, [_vp, _vp, _vp, _i64, _i, _i, _vp, _i, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp,
                          _vp]),
    "qs_proj_apply": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _i64, _vp, _vp]),
    "qs_csr_matvec": (_i, [_i64, _i64, _vp, _i, _vp, _vp, _i, _vp, _i, _vp, _i64, _d, _d, _i, _i, _vp]),
    "qs_csr_matvec_pairs": (_i, [_i64, _i64, _vp, _i, _vp, _vp, _i, _vp, _i, _vp, _i64, _d, _d, _i, _i, _vp, _vp,
                                 _vp]),
    "qs_dia_matvec": (_i, [_i64, _i, _vp, _i64, _vp, _i, _vp, _i, _vp, _i64, _d, _d, _i, _vp]),
    "qs_reduce_scratch_doubles": (_i, []),
    "qs_vdot": (_i, [_i64, _vp, _vp, _i, _vp, _vp, _vp]),
    "qs_nrm2": (_i, [_i64, _vp, _vp, _vp, _vp]),
    "qs_csr_trace": (_i, [_i64, _vp, _i, _vp, _vp, _i, _vp, _vp, _vp]),
    "qs_csr_1_norm": (_i, [_i64, _vp, _i, _vp, _vp, _i, _d, _d, _vp, _vp, _vp, _vp]),
    "qs_expm_ctl_bytes": (_i, []),
    "qs_split_pairs": (_i, [_i64, _vp, _vp, _vp]),
    "qs_split_pairs_trunc": (_i, [_i64, _vp, _i, _vp, _vp]),
    "qs_rk_error_scratch_doubles": (_i, [_i64]),
    "qs_rk_combine": (_i, [_i64, _vp, _vp, _i, _vp, _d, _vp, _vp]),
    "qs_adjoint_axpy": (_i, [_i64, _vp, _vp, _d, _d, _i, _vp]),
    "qs_rk_error": (_i, [_i64, _vp, _vp, _vp, _i, _vp, _vp, _d, _d, _vp, _vp, _vp]),
    "qs_taylor_term": (_i, [_i64, _i64, _vp, _i, _vp, _vp, _i, _vp, _vp, _i, _vp, _i64, _d, _d, _vp, _i, _d, _vp,
                            _i, _vp]),
    "qs_taylor_term_rows": (_i, [_i64, _i64, _vp, _i, _vp, _vp, _i, _vp, _vp, _i, _vp, _i64, _d, _d, _vp, _i, _d, _vp,
                            _i, _vp, _vp]),
    "qs_taylor_rescale": (_i, [_i64, _i64, _vp, _vp, _i, _vp, _vp, _i, _vp]),
    "qs_expm_multiply": (_i, [_i64, _i64, _vp, _i, _vp, _vp, _i, _vp, _i64, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp,
                              _i, _vp, _i, _vp]),
    "qs_expm_multiply_rows": (_i, [_i64, _i64, _vp, _i, _vp, _vp, _i, _vp, _i64, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp,
                              _i, _vp, _i, _vp, _vp]),
    "qs_expm_noalloc_max_elems": (_i64, []),
    "qs_expm_multiply_noalloc": (_i, [_i64, _i64, _vp, _i, _vp, _vp, _i, _vp, _i64, _i, _i, _d, _d, _d, _d, _d,
                                      _i, _vp]),
    "qs_multi_ctl_bytes": (_i, []),
    "qs_max_sectors": (_i, []),
    "qs_taylor_multi_term": (_i, [_i64, _vp, _vp, _vp, _i, _vp, _vp, _i, _vp, _i64, _vp, _vp, _vp, _i, _d, _vp, _i,
                                  _vp]),
    "qs_taylor_multi_term_rows": (_i, [_i64, _vp, _vp, _vp, _i, _vp, _vp, _i, _vp, _i64, _vp, _vp, _vp, _i, _d, _vp, _i,
                                       _vp, _vp]),
    "qs_taylor_multi_rescale": (_i, [_i64, _i64, _vp, _vp, _i, _vp, _vp, _i, _vp, _vp]),
    "qs_mlp_dense_fwd": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "qs_mlp_dense_bwd": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qs_mlp_mse": (_i, [_i64, _i, _vp, _vp, _vp, ctypes.c_float, _vp, _vp, _i, _vp]),
    "qs_mlp_adam": (_i, [_i64, _vp, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                         ctypes.c_float, _i, _vp]),
    "qs_mlp_to_bf16": (_i, [_i64, _vp, _vp, _vp]),
    "qs_lanczos_ctl_bytes": (_i, []),
    "qs_lanczos_scratch_doubles": (_i, []),
    "qs_lanczos_reorth_scratch_doubles": (_i64, [_i]),
    "qs_lanczos_scale": (_i, [_i64, _vp, _vp, _vp, _vp, _vp]),
    "qs_lanczos_alpha": (_i, [_i64, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qs_lanczos_beta": (_i, [_i64, _vp, _vp, _vp, _i, _vp, _d, _i, _vp, _vp, _vp]),
    "qs_lanczos_reorth": (_i, [_i64, _i, _i, _vp, _i64, _vp, _i, _vp, _vp, _vp]),
    "qs_lanczos_reorth_adaptive": (_i, [_i64, _i, _i, _vp, _i64, _vp, _i, _vp, _vp, _vp]),
    "qs_lanczos_lincomb": (_i, [_i64, _i, _vp, _i, _vp, _i64, _i, _vp, _vp]),
    "qs_block_inner_scratch_doubles": (_i64, [_i64, _i, _i, _i]),
    "qs_block_inner": (_i, [_i64, _i, _i, _vp, _i64, _vp, _i64, _i, _i, _i, _vp, _vp, _vp]),
    "qs_block_inner_dmma": (_i, [_i64, _i, _i, _vp, _i64, _vp, _i64, _i, _i, _i, _vp, _vp, _vp]),
}


def exported_names():
    return list(_SIGS)


def load():
    """Load libqsgpu.so (raises RuntimeError when it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    "libqsgpu.so not found at {}; build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'`".format(LIB_PATH))
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class QsError(RuntimeError):
    pass


def check(rc, what):
    if rc != 0:
        raise QsError("{} failed: {} (status {})".format(what, STATUS.get(rc, "unknown"), rc))


def call(name, *args):
    rc = getattr(load(), name)(*args)
    check(rc, name)
    return rc
