"""The allocation-free expm entry point (qs_expm_multiply_noalloc).

Some callers cannot allocate GPU memory: an application or plugin host that
reserves the device memory budget and hands out only its own buffers, or a
time-stepping loop that must not synchronise on cudaMalloc.  For them the
library takes its Taylor scratch from a static device array.  This test calls
that entry point through the C ABI, twice in a row (the second call finds the
previous call's scratch contents), and compares each result with the
allocating entry point qs_expm_multiply at the 1e-12 relative tolerance of the
other expm tests.  It is collected last so a failure here leaves every other
test already run.
"""
import numpy as np
import pytest

from tests.models import chain_maps, xxz_static

pytestmark = pytest.mark.gpu


def _problem():
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(20)
    b = spin_basis_general(20, Nup=10, pauli=0, kblock=(m["t"], 0), pblock=(m["p"], 0))
    return hamiltonian(xxz_static(20), [], basis=b, dtype=np.float64).tocsr_gpu()


def test_expm_noalloc_matches_allocating_entry_point(cuda):
    import torch
    from quspin_gb300 import _device as D
    from quspin_gb300 import _lib
    from quspin_gb300.tools import ExpmMultiplyParallel
    L = _lib.load()
    A = _problem()
    n, nvec = A.shape[0], 2
    op = ExpmMultiplyParallel(A, a=-1.3j)
    s, m, tol = int(op.s), int(op.m_star), float(op._tol)
    a, mu = complex(op.a), complex(op._mu)
    g = torch.Generator(device="cpu").manual_seed(5)
    v = torch.randn(n, nvec, dtype=torch.complex128, generator=g).to("cuda")
    v /= torch.linalg.vector_norm(v, dim=0)
    # allocating entry point: caller-owned scratch
    F_ref = v.clone()
    work = torch.empty(2 * n * nvec, dtype=torch.complex128, device="cuda")
    ctl = torch.zeros(8, dtype=torch.int64, device="cuda")
    consts = torch.tensor([a / (s * (j + 1)) for j in range(max(m, 1))] + [np.exp(a * mu / s), 1.0],
                          dtype=torch.complex128, device="cuda")
    k = max(m, 1)
    rc = L.qs_expm_multiply(n, A.nnz, D.ptr(A.indptr), A.idx64, D.ptr(A.indices), D.ptr(A.data), D.code(A.dtype),
                            D.ptr(F_ref), nvec, s, m, tol, mu.real, mu.imag, D.ptr(consts[:k]),
                            D.ptr(consts[k:k + 1]), D.ptr(consts[k + 1:]), D.ptr(work), _lib.C128, D.ptr(ctl), 0,
                            D.stream())
    assert rc == 0
    outs = [v.clone() for _ in range(2)]
    torch.cuda.synchronize()
    free_after_setup = None
    for i, F in enumerate(outs):
        rc = L.qs_expm_multiply_noalloc(n, A.nnz, D.ptr(A.indptr), A.idx64, D.ptr(A.indices), D.ptr(A.data),
                                        D.code(A.dtype), D.ptr(F), nvec, s, m, tol, mu.real, mu.imag, a.real, a.imag,
                                        0, D.stream())
        assert rc == 0
        torch.cuda.synchronize()
        if i == 0:
            # after the first (set-up) call on this device
            free_after_setup = torch.cuda.mem_get_info()[0]
        else:
            # the second call allocated no device memory (cudaMemGetInfo unchanged)
            assert torch.cuda.mem_get_info()[0] == free_after_setup
    for F in outs:
        err = (torch.linalg.vector_norm(F - F_ref) / torch.linalg.vector_norm(F_ref)).item()
        assert err <= 1e-12, err
    # sizes beyond the static scratch are rejected before any work
    too_many = L.qs_expm_noalloc_max_elems() // n + 1
    rc = L.qs_expm_multiply_noalloc(n, A.nnz, D.ptr(A.indptr), A.idx64, D.ptr(A.indices), D.ptr(A.data),
                                    D.code(A.dtype), D.ptr(v), too_many, s, m, tol, mu.real, mu.imag, a.real, a.imag,
                                    0, D.stream())
    assert rc == -5
