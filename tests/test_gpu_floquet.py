"""Floquet analysis with the evolution of the identity block on the device,
against dense products of exponentials and the reference's per-state ODE
route (scipy ode DOP853, src/quspin/tools/Floquet.py:21-62)."""
import numpy as np
import pytest
from scipy.integrate import ode
from scipy.linalg import expm, logm

from tests.models import chain_maps

pytestmark = pytest.mark.gpu


def _ising(L, hx, dynamic=()):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(L)
    b = spin_basis_general(L, kblock=(m["t"], 0))
    st = [["zz", [[-1.0, i, (i + 1) % L] for i in range(L)]], ["x", [[-hx, i] for i in range(L)]]]
    return hamiltonian(st, list(dynamic), basis=b, dtype=np.complex128)


def test_step_drive_lists(cuda):
    from quspin_gb300.tools import Floquet
    H1, H2 = _ising(8, 0.3), _ising(8, 1.7)
    A1, A2 = H1.tocsr().toarray(), H2.tocsr().toarray()
    dts = [0.4, 0.7]
    U = expm(-1j * dts[1] * A2) @ expm(-1j * dts[0] * A1)
    F = Floquet({"H_list": [H1, H2], "dt_list": dts}, UF=True, HF=True, thetaF=True, VF=True)
    assert F.T == pytest.approx(1.1)
    assert np.abs(F.UF - U).max() < 1e-12
    assert np.abs(F.HF - 1j / 1.1 * logm(U)).max() < 1e-10
    ev = np.linalg.eigvals(U)
    EF = np.sort(np.real(1j / 1.1 * np.log(ev)))
    assert np.abs(F.EF - EF).max() < 1e-10
    assert np.abs(F.VF.conj().T @ F.VF - np.eye(U.shape[0])).max() < 1e-9
    assert np.abs(np.abs(F.thetaF) - 1.0).max() < 1e-12


def test_time_list_drive(cuda):
    from quspin_gb300.tools import Floquet
    drive = lambda t, w: np.cos(w * t)
    H = _ising(8, 0.5, [["x", [[-0.6, i] for i in range(8)], drive, (2 * np.pi,)]])
    ts = np.linspace(0.0, 0.9, 10) + 0.05
    dts = np.full(10, 0.1)
    U = np.eye(H.Ns, dtype=complex)
    for t, dt in zip(ts, dts):
        U = expm(-1j * dt * H.tocsr(t).toarray()) @ U
    F = Floquet({"H": H, "t_list": ts, "dt_list": dts}, UF=True)
    assert np.abs(F.UF - U).max() < 1e-12


def test_continuous_drive_against_reference_route(cuda):
    from quspin_gb300.tools import Floquet
    drive = lambda t, w: np.cos(w * t)
    T = 1.0
    H = _ising(6, 0.5, [["x", [[-0.6, i] for i in range(6)], drive, (2 * np.pi / T,)]])
    F = Floquet({"H": H, "T": T}, UF=True)
    A0 = _ising(6, 0.5).tocsr().toarray()
    A1 = H.tocsr(0.0).toarray() - A0
    cols = []
    for i in range(H.Ns):
        e = np.zeros(H.Ns, complex)
        e[i] = 1.0
        s = ode(lambda t, y: (-1j * ((A0 + drive(t, 2 * np.pi / T) * A1) @ y.view(complex))).view(np.float64))
        s.set_integrator("dop853", atol=1e-12, rtol=1e-12, nsteps=10 ** 7)
        s.set_initial_value(e.view(np.float64), 0.0)
        s.integrate(T)
        cols.append(s._y.view(complex).copy())
    U = np.stack(cols, axis=1)
    assert np.abs(F.UF - U).max() < 1e-9
    with pytest.raises(TypeError):
        Floquet({"H": H, "T": 0.7})
