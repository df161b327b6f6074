"""Schroedinger evolution of a ``hamiltonian`` by an explicit 8th-order
Runge-Kutta method on the device.

The reference's ``hamiltonian.evolve`` (src/quspin/operators/
hamiltonian_core.py:1489-1630) hands the right-hand side -i H(t) v (or -H(t) v
for imaginary time) to scipy's ``ode`` wrapper around Hairer's DOP853
through ``tools.evolution.evolve`` (src/quspin/tools/evolution.py:144-470),
with rtol = atol = 1e-9 and an unbounded step count unless the caller says
otherwise.  Here the same method runs with the state resident on the GPU:

* right-hand side: ``hamiltonian.dot(v, time=t, a=-1j)``, the fused static +
  f_k(t)-weighted dynamic CSR products, no host CSR rebuild per step;
* stage and update combinations and the embedded error estimates:
  ``csrc/ode.cu`` (one pass over the stage block per stage);
* the Butcher tableau of DOP853 (Hairer, Noersett and Wanner, Solving
  Ordinary Differential Equations I, 2nd ed., section II.10) is taken from
  scipy's published coefficient tables;
* error norm and step-size control follow Hairer's DOP853 code as scipy's
  ``ode`` runs it (safety 0.9, growth at most 6, shrink at most 1/0.3 per
  step, exponent 1/8, the scaled 5th/3rd-order error combination, the
  initial-step heuristic), over the state viewed as 2N real components like
  scipy's complex wrapper.

Outputs follow the reference: an array of shape (Ns, len(times)) (or
(Ns, k, len(times))), a generator with ``iterate=True``, imaginary-time states
renormalised to the initial norm.  ``eom="LvNE"`` evolves a density matrix
with d rho / dt = -i [H(t), rho]; the commutator's right product comes from
the conjugate-transposed parts, rho H = (H^dagger rho^dagger)^dagger, with the
adjoints taken by a tiled transpose kernel (csrc/ode.cu).
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _device as D
from .. import _lib

_SAFE, _IFACTOR, _DFACTOR, _EXPO = 0.9, 6.0, 0.3, 1.0 / 8.0


def _tableau():
    from scipy.integrate._ivp import dop853_coefficients as c
    ns = c.N_STAGES
    return ns, np.asarray(c.A[:ns, :ns], np.float64), np.asarray(c.B, np.float64), \
        np.asarray(c.C[:ns], np.float64), np.asarray(c.E5, np.float64), np.asarray(c.E3, np.float64)


class DeviceDOP853:
    """Adaptive DOP853 on a device vector y (viewed as n2 real components)
    for y' = rhs(t, y, out)."""

    def __init__(self, rhs, y0, t0, rtol=1e-9, atol=1e-9, nsteps=None, max_step=0.0, first_step=0.0):
        self.ns, self.A, self.B, self.C, self.E5, self.E3 = _tableau()
        self._e5 = np.ascontiguousarray(self.E5[:self.ns + 1])
        self._e3 = np.ascontiguousarray(self.E3[:self.ns + 1])
        self.rhs = rhs
        self.y = y0.clone()
        self.t = float(t0)
        self.rtol, self.atol = float(rtol), float(atol)
        self.nsteps = int(np.iinfo(np.int32).max if nsteps is None else nsteps)
        self.max_step = float(max_step)
        self.h = float(first_step)
        self.shape = y0.shape
        self._real = self._r(self.y)
        self.n2 = self._real.numel()
        dev = y0.device
        self.K = torch.empty((self.ns + 1,) + tuple(self.y.shape), dtype=y0.dtype, device=dev)
        self.ytmp = torch.empty_like(self.y)
        self.ynew = torch.empty_like(self.y)
        L = _lib.load()
        self._scr = torch.zeros(max(L.qs_rk_error_scratch_doubles(self.n2), 1), dtype=torch.float64, device=dev)
        self._err = torch.zeros(2, dtype=torch.float64, device=dev)
        self.rhs(self.t, self.y, self.K[0])
        self.nfev, self.naccept, self.nreject = 1, 0, 0
        self._facold = 1e-4
        self._reject = False

    @staticmethod
    def _r(x):
        return torch.view_as_real(x).reshape(-1) if x.is_complex() else x.reshape(-1)

    def _combine(self, coef, nk, h, out):
        c = np.ascontiguousarray(coef[:nk], np.float64)
        _lib.call("qs_rk_combine", self.n2, D.ptr(self._r(self.y)), D.ptr(self.K), nk,
                  c.ctypes.data, h, D.ptr(self._r(out)), D.stream())

    def _sumsq(self, K, coef, nk):
        """sum_i ((sum_j coef_j K_j)_i / sk_i)^2 with sk = atol + rtol |y_i|
        (one pass of the error kernel with y as both end points)."""
        c = np.zeros(nk, np.float64)
        c[:] = coef
        y = D.ptr(self._r(self.y))
        _lib.call("qs_rk_error", self.n2, y, y, D.ptr(K), nk, c.ctypes.data, c.ctypes.data, self.atol, self.rtol,
                  D.ptr(self._scr), D.ptr(self._err), D.stream())
        return float(self._err[0].item())

    def _initial_step(self, hmax, direction):
        """Hairer's starting-step heuristic (HNW I, II.4) on the scaled norms."""
        dnf = self._sumsq(self.K[0], [1.0], 1)
        dny = self._sumsq(self.y, [1.0], 1)
        h = 1e-6 if (dnf <= 1e-10 or dny <= 1e-10) else 0.01 * np.sqrt(dny / dnf)
        h = min(h, hmax) * direction
        self._combine(np.array([1.0]), 1, h, self.ytmp)          # y + h f0
        self.rhs(self.t + h, self.ytmp, self.K[1])
        self.nfev += 1
        der2 = np.sqrt(self._sumsq(self.K, [-1.0, 1.0], 2)) / abs(h)
        der12 = max(abs(der2), np.sqrt(dnf))
        h1 = max(1e-6, abs(h) * 1e-3) if der12 <= 1e-15 else (0.01 / der12) ** (1.0 / 8.0)
        return min(100 * abs(h), h1, hmax) * direction

    def integrate(self, t_end):
        """Advance to t_end exactly (the last step is shortened)."""
        t_end = float(t_end)
        if t_end == self.t:
            return self.y
        direction = 1.0 if t_end > self.t else -1.0
        hmax = abs(self.max_step) if self.max_step else abs(t_end - self.t)
        if self.h == 0.0:
            self.h = self._initial_step(hmax, direction)
        h = direction * min(abs(self.h), hmax)
        uround = np.finfo(np.float64).eps
        steps = 0
        last = False
        while True:
            if steps > self.nsteps:
                raise RuntimeError("failed to evolve to time {0}, nsteps might be too small".format(t_end))
            if 0.1 * abs(h) <= abs(self.t) * uround:
                raise RuntimeError("failed to evolve to time {0}: step size too small".format(t_end))
            h_full = h
            if (self.t + 1.01 * h - t_end) * direction > 0:
                h = t_end - self.t
                last = True
            steps += 1
            for s in range(1, self.ns):
                self._combine(self.A[s], s, h, self.ytmp)
                self.rhs(self.t + self.C[s] * h, self.ytmp, self.K[s])
            self._combine(self.B, self.ns, h, self.ynew)
            self.rhs(self.t + h, self.ynew, self.K[self.ns])
            self.nfev += self.ns
            _lib.call("qs_rk_error", self.n2, D.ptr(self._r(self.y)), D.ptr(self._r(self.ynew)), D.ptr(self.K),
                      self.ns + 1, self._e5.ctypes.data, self._e3.ctypes.data, self.atol, self.rtol,
                      D.ptr(self._scr), D.ptr(self._err), D.stream())
            e5, e3 = self._err.tolist()
            if e5 == 0.0 and e3 == 0.0:
                err = 0.0
            else:
                deno = e5 + 0.01 * e3
                if deno <= 0.0:
                    deno = 1.0
                err = abs(h) * e5 / np.sqrt(deno * self.n2)
            fac11 = err ** _EXPO if err > 0 else 0.0
            fac = max(1.0 / _IFACTOR, min(1.0 / _DFACTOR, fac11 / _SAFE))
            hnew = h / fac
            if err <= 1.0:
                self._facold = max(err, 1e-4)
                self.naccept += 1
                self.t += h
                self.y, self.ynew = self.ynew, self.y
                self.K[0].copy_(self.K[self.ns])
                if abs(hnew) > hmax:
                    hnew = direction * hmax
                if self._reject:
                    hnew = direction * min(abs(hnew), abs(h))
                self._reject = False
                if last:
                    # the next interval starts from the step the controller
                    # proposed before this one was shortened to hit t_end
                    self.h = direction * max(abs(hnew), abs(h_full))
                    self.t = t_end
                    return self.y
            else:
                hnew = h / min(1.0 / _DFACTOR, fac11 / _SAFE)
                self._reject = True
                self.nreject += 1
                last = False
            h = hnew


def _dagger(M):
    """Device conjugate transpose of a static or dynamic part."""
    from ..sparse import DeviceCSR, DeviceDIA
    if isinstance(M, DeviceCSR):
        return M.conj_transpose()
    if isinstance(M, DeviceDIA) and bool((M.offsets == 0).all()):
        return DeviceDIA(M.offsets, M.data.conj().resolve_conj() if M.data.is_complex() else M.data, M.shape,
                         M.dtype)
    return DeviceCSR.from_scipy(M.tocsr().conj().T.tocsr(), M.dtype)


def _liouville_rhs(H):
    """rhs(t, rho, out): out = -i (H(t) rho - rho H(t)) with rho H =
    (H(t)^dagger rho^dagger)^dagger (hamiltonian_core.py:1394-1420)."""
    parts = [(None, _dagger(H._static))] + [(fn, _dagger(M)) for fn, M in H._dynamic.items()]
    buf = {}

    def rhs(t, rho, out):
        n = rho.shape[0]
        if "rd" not in buf:
            buf["rd"] = torch.empty_like(rho)
            buf["y"] = torch.empty_like(rho)
        rd, y = buf["rd"], buf["y"]
        H.dot(rho, time=t, out=out, a=-1j)                                   # -i H rho
        _lib.call("qs_adjoint_axpy", n, D.ptr(rho), D.ptr(rd), 1.0, 0.0, 0, D.stream())   # rho^dagger
        for k, (fn, Md) in enumerate(parts):
            c = 1.0 if fn is None else complex(np.conj(fn(t)))
            Md.matvec_into(rd, y, a=c, overwrite=(k == 0))                    # H^dagger rho^dagger
        _lib.call("qs_adjoint_axpy", n, D.ptr(y), D.ptr(out), 0.0, 1.0, 1, D.stream())     # += i (..)^dagger
    return rhs


def evolve_hamiltonian(H, v0, t0, times, eom="SE", solver_name="dop853", stack_state=False, verbose=False,
                       iterate=False, imag_time=False, **solver_args):
    """hamiltonian.evolve on the device (see the module docstring)."""
    if eom == "LvNE":
        return _evolve_lvne(H, v0, t0, times, solver_name, stack_state, verbose, iterate, imag_time,
                            **solver_args)
    if eom != "SE":
        raise ValueError("'{} equation' not recognized, must be 'SE' or 'LvNE'".format(eom))
    if solver_name not in ("dop853",):
        raise NotImplementedError("the GPU integrator is DOP853 (solver_name='dop853')")
    if imag_time and stack_state:
        raise NotImplementedError("stack state is not compatible with imaginary time evolution.")
    host = not D.is_device_array(v0)
    v0a = np.asanyarray(v0) if host else v0
    if np.iscomplexobj(np.asarray(times)):
        raise ValueError("times must be real number(s).")
    if v0a.ndim > 2:
        raise ValueError("v0 must have ndim <= 2")
    if v0a.shape[0] != H.Ns:
        raise ValueError("v0 must have {0} elements".format(H.Ns))
    if imag_time:
        dt = np.result_type(v0a.dtype if host else D.np_dtype(v0a.dtype), H.dtype, np.float64)
        a = -1.0
    else:
        dt = np.dtype(np.complex128)
        a = -1j
    y0 = D.to_device(v0a, dt).clone() if host else v0a.to(D.torch_dtype(dt)).clone()
    norm0 = torch.linalg.vector_norm(y0, dim=0)

    def rhs(t, y, out):
        H.dot(y, time=t, out=out, a=a)

    rtol = solver_args.pop("rtol", None)
    atol = solver_args.pop("atol", None)
    nsteps = solver_args.pop("nsteps", None)
    solver = DeviceDOP853(rhs, y0, t0, rtol=1e-9 if rtol is None else rtol, atol=1e-9 if atol is None else atol,
                          nsteps=nsteps, max_step=solver_args.pop("max_step", 0.0),
                          first_step=solver_args.pop("first_step", 0.0))

    def fmt(y):
        out = y.clone()
        if imag_time:
            out = out / (torch.linalg.vector_norm(out, dim=0) / norm0)
        if verbose:
            print("evolved to time {0}, norm of state(s) {1}".format(
                solver.t, D.to_host(torch.linalg.vector_norm(out, dim=0))))
        return D.to_host(out) if host else out

    if np.isscalar(times):
        return fmt(solver.integrate(times))

    def gen():
        for t in times:
            yield fmt(solver.integrate(t))
    if iterate:
        return gen()
    outs = [fmt(solver.integrate(t)) for t in times]
    if host:
        v = np.stack(outs, axis=0)
        return v.transpose() if v.ndim == 2 else v.transpose((1, 2, 0))
    v = torch.stack(outs, dim=0)
    return v.permute(1, 0) if v.dim() == 2 else v.permute(1, 2, 0)


def _evolve_lvne(H, rho0, t0, times, solver_name, stack_state, verbose, iterate, imag_time, **solver_args):
    """Liouville - von Neumann evolution d rho / dt = -i [H(t), rho] of a
    density matrix (hamiltonian_core.py:1598-1617 checks and right-hand side
    :1394-1420), integrated by the device DOP853 over the n^2 complex entries."""
    if solver_name not in ("dop853",):
        raise NotImplementedError("the GPU integrator is DOP853 (solver_name='dop853')")
    if imag_time:
        raise NotImplementedError("imaginary time not implemented for Liouville-von Neumann dynamics")
    if stack_state:
        raise NotImplementedError("stack_state not implemented for Liouville-von Neumann dynamics")
    host = not D.is_device_array(rho0)
    r0 = np.asanyarray(rho0) if host else rho0
    if r0.ndim != 2:
        raise ValueError("v0 must have ndim = 2")
    if tuple(r0.shape) != tuple(H._shape):
        raise ValueError("v0 must be same shape as Hamiltonian")
    y0 = (D.to_device(r0, np.complex128) if host else r0.to(torch.complex128)).contiguous().clone()
    rtol = solver_args.pop("rtol", None)
    atol = solver_args.pop("atol", None)
    solver = DeviceDOP853(_liouville_rhs(H), y0, t0, rtol=1e-9 if rtol is None else rtol,
                          atol=1e-9 if atol is None else atol, nsteps=solver_args.pop("nsteps", None),
                          max_step=solver_args.pop("max_step", 0.0), first_step=solver_args.pop("first_step", 0.0))

    def fmt(y):
        out = y.clone()
        if verbose:
            print("evolved to time {0}, trace of state {1}".format(solver.t, complex(torch.diagonal(out).sum())))
        return D.to_host(out) if host else out

    if np.isscalar(times):
        return fmt(solver.integrate(times))

    def gen():
        for t in times:
            yield fmt(solver.integrate(t))
    if iterate:
        return gen()
    outs = [fmt(solver.integrate(t)) for t in times]
    if host:
        return np.stack(outs, axis=0).transpose((1, 2, 0))
    return torch.stack(outs, dim=0).permute(1, 2, 0)
