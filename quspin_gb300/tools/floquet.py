"""Floquet analysis of a periodic drive with the evolution on the device.

The reference's ``Floquet`` (src/quspin/tools/Floquet.py:142-437) builds the
one-period evolution operator U_F column by column -- one basis state at a
time, fanned out to joblib workers -- with scipy's ODE solver
(``_evolve_cont``, :21-62) or with ``scipy.sparse.linalg.expm_multiply``
over a list of constant steps (``_evolve_step_2/3``, :65-88), and then takes
the Floquet Hamiltonian, phases and states from dense linear algebra.  Here
all Ns basis states evolve together as one [Ns, Ns] block on the GPU:

* ``{"H", "T"[, "atol", "rtol"]}``: the device DOP853 of ``hamiltonian.evolve``
  on the identity block (rtol = atol = 1e-12 by default, as the reference);
* ``{"H", "t_list", "dt_list"[, "T"]}``: one ``ExpmMultiplyParallel`` per step
  on H(t_k), applied in place to the block;
* ``{"H_list", "dt_list"[, "T"]}``: the same with one matrix per step.

The dense post-processing (matrix logarithm, eigen-decomposition, the
orthonormalisation of degenerate Floquet states) runs on the host with scipy,
as in the reference.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as la
import torch

from .. import _device as D

__all__ = ["Floquet"]


def _check_periodic(H, T):
    """Every drive function must satisfy f(t) = f(t + T) at an irregular
    test time (the reference's periodicity check)."""
    t = np.cos((np.pi / np.exp(0)) ** (1.0 / np.euler_gamma))
    for fn in H.dynamic.keys():
        if abs(fn(t) - fn(t + T)) > 1e5 * np.finfo(np.complex128).eps:
            raise TypeError("Hamiltonian 'H' must be periodic with period 'T'!")


def _identity(Ns):
    return torch.eye(Ns, dtype=torch.complex128, device=D.device())


def _evolve_steps(mats, dts, Ns):
    from .expm_multiply_parallel import ExpmMultiplyParallel
    U = _identity(Ns)
    for M, dt in zip(mats, dts):
        ExpmMultiplyParallel(M, a=-1j * float(dt)).dot(U, overwrite_v=True)
    return U


class Floquet:
    """Floquet operator, Hamiltonian, quasi-energies, phases and states of a
    periodic evolution (same arguments and attributes as the reference)."""

    def __init__(self, evo_dict, HF=False, UF=False, thetaF=False, VF=False, n_jobs=1, force_ONB=False):
        from ..operators import hamiltonian
        if not isinstance(evo_dict, dict):
            raise ValueError("evo_dict={0} is not correct format.".format(evo_dict))
        if not isinstance(n_jobs, int):
            raise TypeError("expecting integer value for optional variable 'n_jobs'!")
        keys = set(evo_dict.keys())
        if keys in ({"H", "T"}, {"H", "T", "atol"}, {"H", "T", "rtol"}, {"H", "T", "atol", "rtol"}):
            H, T = evo_dict["H"], evo_dict["T"]
            atol = evo_dict.get("atol", 1e-12)
            rtol = evo_dict.get("rtol", 1e-12)
            if not isinstance(atol, float):
                raise ValueError("expecting float for 'atol'.")
            if not isinstance(rtol, float):
                raise ValueError("expecting float for 'rtol'.")
            if not isinstance(H, hamiltonian):
                raise ValueError("expecting hamiltonian object for 'H'.")
            if not np.isscalar(T):
                raise ValueError("expecting scalar object for 'T'.")
            if np.iscomplex(T):
                raise ValueError("expecting real value for 'T'.")
            _check_periodic(H, T)
            self._T = T
            U = H.evolve(_identity(H.Ns), 0.0, float(T), atol=atol, rtol=rtol)
        elif keys in ({"H", "t_list", "dt_list"}, {"H", "t_list", "dt_list", "T"}):
            H = evo_dict["H"]
            t_list = np.asarray(evo_dict["t_list"], dtype=np.float64)
            dt_list = np.asarray(evo_dict["dt_list"], dtype=np.float64)
            if t_list.ndim != 1:
                raise ValueError("t_list must be 1d array.")
            if dt_list.ndim != 1:
                raise ValueError("dt_list must be 1d array.")
            if not isinstance(H, hamiltonian):
                raise ValueError("expecting hamiltonian object for 'H'.")
            self._T = evo_dict["T"] if "T" in keys else dt_list.sum()
            U = _evolve_steps([H.tocsr_gpu(t) for t in t_list], dt_list, H.Ns)
        elif keys in ({"H_list", "dt_list"}, {"H_list", "dt_list", "T"}):
            H_list = evo_dict["H_list"]
            dt_list = np.asarray(evo_dict["dt_list"], dtype=np.float64)
            if dt_list.ndim != 1:
                raise ValueError("dt_list must be 1d array.")
            if type(H_list) not in (list, tuple):
                raise ValueError("expecting list/tuple for H_list.")
            if len(dt_list) != len(H_list):
                raise ValueError("Expecting arguments 'H_list' and 'dt_list' to have the same length!")
            self._T = evo_dict["T"] if "T" in keys else dt_list.sum()
            mats = [M.tocsr_gpu() if isinstance(M, hamiltonian) else M for M in H_list]
            U = _evolve_steps(mats, dt_list, mats[0].shape[0])
        else:
            raise ValueError("evo_dict={0} is not correct format.".format(evo_dict))
        UF_h = D.to_host(U)
        if UF:
            self._UF = np.copy(UF_h)
        if HF:
            self._HF = 1j / self._T * la.logm(UF_h)
        if VF:
            theta, V = la.eig(UF_h)
            if np.any(np.diff(np.sort(theta)) < 1e3 * np.finfo(theta.dtype).eps) or force_ONB:
                V, _ = la.qr(V)
            EF = np.real(1j / self._T * np.log(theta))
            order = np.argsort(EF)
            self._EF = np.array(EF[order])
            self._VF = np.array(V[:, order])
        else:
            theta = la.eigvals(UF_h)
            EF = np.real(1j / self._T * np.log(theta))
            order = np.argsort(EF)
            self._EF = np.array(EF[order])
        if thetaF:
            self._thetaF = np.array(theta[order])

    @property
    def T(self):
        return self._T

    @property
    def EF(self):
        return self._EF

    @property
    def HF(self):
        if hasattr(self, "_HF"):
            return self._HF
        raise AttributeError("missing atrribute 'HF'.")

    @property
    def UF(self):
        if hasattr(self, "_UF"):
            return self._UF
        raise AttributeError("missing atrribute 'UF'.")

    @property
    def thetaF(self):
        if hasattr(self, "_thetaF"):
            return self._thetaF
        raise AttributeError("missing atrribute 'thetaF'.")

    @property
    def VF(self):
        if hasattr(self, "_VF"):
            return self._VF
        raise AttributeError("missing atrribute 'VF'.")
