"""Device plumbing: torch tensors as CUDA buffers, streams, dtype codes."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

_NP_TO_CODE = {
    np.dtype(np.float32): _lib.F32,
    np.dtype(np.float64): _lib.F64,
    np.dtype(np.complex64): _lib.C64,
    np.dtype(np.complex128): _lib.C128,
}
_NP_TO_TORCH = {
    np.dtype(np.float32): torch.float32,
    np.dtype(np.float64): torch.float64,
    np.dtype(np.complex64): torch.complex64,
    np.dtype(np.complex128): torch.complex128,
    np.dtype(np.int32): torch.int32,
    np.dtype(np.int64): torch.int64,
    np.dtype(np.int8): torch.int8,
    np.dtype(np.uint8): torch.uint8,
    np.dtype(np.uint32): torch.int32,     # reinterpreted bit patterns
    np.dtype(np.uint64): torch.int64,
}
_TORCH_TO_NP = {
    torch.float32: np.dtype(np.float32),
    torch.float64: np.dtype(np.float64),
    torch.complex64: np.dtype(np.complex64),
    torch.complex128: np.dtype(np.complex128),
    torch.int32: np.dtype(np.int32),
    torch.int64: np.dtype(np.int64),
    torch.int8: np.dtype(np.int8),
    torch.uint8: np.dtype(np.uint8),
}

SUPPORTED = (np.dtype(np.float32), np.dtype(np.float64), np.dtype(np.complex64), np.dtype(np.complex128))


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("quspin_gb300 needs a CUDA device (sm_103a); none is available")
    _lib.load()


def device():
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def code(dtype):
    return _NP_TO_CODE[np.dtype(dtype)]


def torch_dtype(dtype):
    return _NP_TO_TORCH[np.dtype(dtype)]


def np_dtype(tdtype):
    return _TORCH_TO_NP[tdtype]


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def empty(shape, dtype):
    return torch.empty(shape, dtype=torch_dtype(dtype), device=device())


def zeros(shape, dtype):
    return torch.zeros(shape, dtype=torch_dtype(dtype), device=device())


# Host arrays at least this large cross PCIe / C2C through a page-locked
# staging buffer (page-locked copies run at the link rate; pageable ones are
# staged by the driver in small pieces).
_STAGE_MIN_BYTES = 1 << 20
_STAGE_MAX_BYTES = 256 << 20          # larger transfers go through the page-locked buffer in chunks
_stage = {}


def _staging(nbytes):
    buf = _stage.get("buf")
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(nbytes, _STAGE_MIN_BYTES), dtype=torch.uint8, pin_memory=True)
        _stage["buf"] = buf
    return buf[:nbytes]


def _pinned(arr):
    try:
        return torch.from_numpy(arr).is_pinned()
    except (TypeError, RuntimeError):
        return False


def to_device(a, dtype=None):
    """Contiguous device tensor from a numpy array / torch tensor / scalar list."""
    if isinstance(a, torch.Tensor):
        t = a
        if dtype is not None and t.dtype != torch_dtype(dtype):
            t = t.to(torch_dtype(dtype))
        if not t.is_cuda:
            t = t.to(device(), non_blocking=False)
        return t.contiguous()
    arr = np.asarray(a)
    if dtype is not None:
        arr = arr.astype(dtype, copy=False)
    if arr.dtype == np.uint32:
        arr = arr.view(np.int32)
    elif arr.dtype == np.uint64:
        arr = arr.view(np.int64)
    arr = np.ascontiguousarray(arr)
    if arr.nbytes < _STAGE_MIN_BYTES or arr.dtype.kind not in "iufc" or _pinned(arr):
        return torch.from_numpy(arr).to(device())
    out = torch.empty(arr.shape, dtype=torch_dtype(arr.dtype), device=device())
    src, dst = arr.reshape(-1).view(np.uint8), out.view(-1).view(torch.uint8)
    step = min(arr.nbytes, _STAGE_MAX_BYTES)
    st = _staging(step)
    for o in range(0, arr.nbytes, step):
        k = min(step, arr.nbytes - o)
        st.numpy()[:k] = src[o:o + k]
        dst[o:o + k].copy_(st[:k])                     # synchronous: the staging buffer is free afterwards
    return out


def to_host(t, dtype=None):
    t = t.detach()
    nbytes = t.numel() * t.element_size()
    if t.is_cuda and nbytes >= _STAGE_MIN_BYTES and t.dtype in _TORCH_TO_NP:
        tc = t.contiguous()
        arr = np.empty(tuple(tc.shape), dtype=np_dtype(tc.dtype))
        src, dst = tc.view(-1).view(torch.uint8), arr.reshape(-1).view(np.uint8)
        step = min(nbytes, _STAGE_MAX_BYTES)
        st = _staging(step)
        for o in range(0, nbytes, step):
            k = min(step, nbytes - o)
            st[:k].copy_(src[o:o + k])                     # page-locked device-to-host copy
            torch.from_numpy(dst[o:o + k]).copy_(st[:k])   # host copy on torch's intra-op threads
    else:
        arr = t.cpu().numpy()
    if dtype is not None and arr.dtype != np.dtype(dtype):
        arr = arr.view(dtype) if arr.dtype.itemsize == np.dtype(dtype).itemsize and \
            arr.dtype.kind in "iu" and np.dtype(dtype).kind in "iu" else arr.astype(dtype)
    return arr


def is_device_array(x):
    return isinstance(x, torch.Tensor) and x.is_cuda


def scratch_doubles(n):
    return torch.empty(max(int(n), 1), dtype=torch.float64, device=device())


def err_flag():
    return torch.zeros(1, dtype=torch.int32, device=device())
