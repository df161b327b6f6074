"""``matvec`` / ``get_matvec_function`` on the GPU (the reference's
docs/modules/parallel_sparse_tools/matvec/matvec_core.html:105-201):
x (+)= a A v for CSR / DIA matrices, numpy or CUDA-tensor operands."""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from .. import _device as D
from ..sparse import DeviceCSR, DeviceDIA, _apply, to_device_matrix


def _dev(array):
    if isinstance(array, (DeviceCSR, DeviceDIA)):
        return array
    if isinstance(array, np.ndarray):
        return DeviceCSR.from_scipy(sp.csr_matrix(array))
    if sp.issparse(array):
        return to_device_matrix(array)
    raise TypeError("unsupported matrix type {}".format(type(array)))


def matvec(array, other, overwrite_out=False, out=None, a=1.0):
    """x = a A v (overwrite_out) or x += a A v; returns the result."""
    M = _dev(array)
    if out is None:
        overwrite_out = True
    return _apply(M, other, out, a, overwrite_out)


def get_matvec_function(array):
    """The product routine for ``array`` (a closure over its device copy)."""
    M = _dev(array)

    def f(arr, other, overwrite_out=False, out=None, a=1.0):
        return matvec(M, other, overwrite_out=overwrite_out, out=out, a=a)

    return f
