"""hamiltonian.evolve on the device against the reference's own integrator
(scipy's ode with DOP853 over the 2N real components, as
src/quspin/tools/evolution.py:300-345 sets it up) and against exact
exponentials: static and driven Hamiltonians, real and imaginary time, one or
several states, list and generator outputs."""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.integrate import ode
from scipy.sparse.linalg import expm_multiply

from tests.models import chain_maps, xxz_static

pytestmark = pytest.mark.gpu


def _xxz(L=12, dynamic=()):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, kblock=(m["t"], 0), pauli=0)
    return hamiltonian(xxz_static(L), list(dynamic), basis=b, dtype=np.complex128)


def _scipy_dop853(f, v0, t0, times, rtol, atol):
    """The reference's path: complex state as 2N reals through scipy's ode."""
    y0 = np.ascontiguousarray(v0, np.complex128).view(np.float64)
    solver = ode(lambda t, y: f(t, y.view(np.complex128)).view(np.float64))
    solver.set_integrator("dop853", rtol=rtol, atol=atol, nsteps=np.iinfo(np.int32).max)
    solver.set_initial_value(y0, t0)
    out = []
    for t in times:
        if t == t0:
            out.append(v0.copy())
            continue
        solver.integrate(t)
        assert solver.successful()
        out.append(solver._y.view(np.complex128).copy())
    return np.stack(out, axis=-1)


def _state(n, seed, k=None):
    rng = np.random.default_rng(seed)
    shape = (n,) if k is None else (n, k)
    v = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    return v / np.linalg.norm(v, axis=0)


def test_static_real_time(cuda):
    H = _xxz()
    A = H.tocsr()
    v0 = _state(H.Ns, 1)
    times = np.array([0.0, 0.5, 1.0, 2.5])
    vt = H.evolve(v0, 0.0, times)
    assert vt.shape == (H.Ns, len(times))
    exact = np.stack([expm_multiply(-1j * t * A, v0) for t in times], axis=-1)
    ref = _scipy_dop853(lambda t, y: -1j * (A @ y), v0, 0.0, times, 1e-9, 1e-9)
    assert np.abs(vt - exact).max() < 1e-6
    assert np.abs(vt - ref).max() < 1e-6
    tight = H.evolve(v0, 0.0, times, rtol=1e-12, atol=1e-12)
    assert np.abs(tight - exact).max() < 1e-9


def test_driven_against_reference_integrator(cuda):
    L = 12
    drive = lambda t, w: np.cos(w * t)
    dyn = [["zz", [[0.3, i, (i + 1) % L] for i in range(L)], drive, (2.0,)]]
    H = _xxz(L, dyn)
    A0 = _xxz(L).tocsr()
    A1 = (H.tocsr(time=0.0) - A0)            # cos(0) = 1
    v0 = _state(H.Ns, 2)
    times = np.linspace(0.0, 3.0, 7)
    vt = H.evolve(v0, 0.0, times, rtol=1e-10, atol=1e-10)
    ref = _scipy_dop853(lambda t, y: -1j * (A0 @ y + drive(t, 2.0) * (A1 @ y)), v0, 0.0, times, 1e-10, 1e-10)
    assert np.abs(vt - ref).max() < 1e-7
    # norm conservation of the unitary evolution
    assert np.abs(np.linalg.norm(vt, axis=0) - 1.0).max() < 1e-8


def test_imaginary_time_and_block(cuda):
    H = _xxz()
    A = H.tocsr()
    v0 = np.random.default_rng(3).normal(size=H.Ns).astype(np.complex128)
    n0 = np.linalg.norm(v0)
    vt = H.evolve(v0, 0.0, [1.0], imag_time=True, rtol=1e-11, atol=1e-11)
    ex = expm_multiply(-1.0 * A, v0)
    ex *= n0 / np.linalg.norm(ex)
    assert np.abs(vt[:, 0] - ex).max() < 1e-8
    V = _state(H.Ns, 4, k=3)
    Vt = H.evolve(V, 0.0, [0.0, 0.7], rtol=1e-11, atol=1e-11)
    assert Vt.shape == (H.Ns, 3, 2)
    assert np.abs(Vt[:, :, 1] - expm_multiply(-0.7j * A, V)).max() < 1e-8


def test_iterate_and_device_state(cuda):
    import torch
    H = _xxz()
    A = H.tocsr()
    v0 = _state(H.Ns, 5)
    gen = H.evolve(v0, 0.0, [0.3, 0.6], iterate=True, rtol=1e-11, atol=1e-11)
    outs = list(gen)
    assert len(outs) == 2
    assert np.abs(outs[1] - expm_multiply(-0.6j * A, v0)).max() < 1e-8
    vd = torch.tensor(v0, device="cuda")
    w = H.evolve(vd, 0.0, 0.6, rtol=1e-11, atol=1e-11)
    assert isinstance(w, torch.Tensor)
    assert np.abs(w.cpu().numpy() - outs[1]).max() < 1e-9
    with pytest.raises(ValueError):
        H.evolve(v0[:-1], 0.0, [1.0])


def test_liouville_evolution(cuda):
    """eom='LvNE': rho(t) = U rho0 U^dagger for a static H (dense exponential on
    a small sector) and the commutator equation integrated by scipy's ode for a
    driven H (the reference's own route, hamiltonian_core.py:1394-1420)."""
    from scipy.linalg import expm
    from quspin_gb300 import hamiltonian, spin_basis_general
    L = 10
    m = chain_maps(L)
    b = spin_basis_general(L, Nup=L // 2, kblock=(m["t"], 1), pauli=0)
    H = hamiltonian(xxz_static(L), [], basis=b, dtype=np.complex128)
    A = H.toarray() if hasattr(H, "toarray") else H.tocsr().toarray()
    n = A.shape[0]
    rng = np.random.default_rng(8)
    X = rng.normal(size=(n, 3)) + 1j * rng.normal(size=(n, 3))
    rho0 = X @ np.diag([0.5, 0.3, 0.2]) @ X.conj().T
    rho0 /= np.trace(rho0)
    times = [0.0, 0.4, 1.1]
    rt = H.evolve(rho0, 0.0, times, eom="LvNE", rtol=1e-11, atol=1e-11)
    assert rt.shape == (n, n, len(times))
    for k, t in enumerate(times):
        U = expm(-1j * t * A)
        assert np.abs(rt[:, :, k] - U @ rho0 @ U.conj().T).max() < 1e-9
    drive = lambda t, w: np.sin(w * t)
    Hd = hamiltonian(xxz_static(L), [["zz", [[0.4, i, (i + 1) % L] for i in range(L)], drive, (1.5,)]],
                     basis=b, dtype=np.complex128)
    A0 = A
    A1 = Hd.tocsr(time=np.pi / 3.0).toarray() - A0
    A1 = A1 / drive(np.pi / 3.0, 1.5)

    def f(t, y):
        R = y.reshape(n, n)
        Ht = A0 + drive(t, 1.5) * A1
        return (-1j * (Ht @ R - R @ Ht)).reshape(-1)
    ref = _scipy_dop853(f, rho0.reshape(-1), 0.0, [0.0, 0.9], 1e-11, 1e-11)
    got = Hd.evolve(rho0, 0.0, [0.0, 0.9], eom="LvNE", rtol=1e-11, atol=1e-11)
    assert np.abs(got[:, :, 1] - ref[:, 1].reshape(n, n)).max() < 1e-8
    with pytest.raises(NotImplementedError):
        H.evolve(rho0, 0.0, [1.0], eom="LvNE", imag_time=True)
