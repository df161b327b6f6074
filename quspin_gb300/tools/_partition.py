"""Choice of the Taylor degree m* and substep count s for e^{aA} v.

The reference (ExpmMultiplyParallel._calculate_partition,
docs/modules/parallel_sparse_tools/expm_multiply_parallel_core/
expm_multiply_parallel_core.html:377-385) calls scipy's private
``_fragment_3_1`` with n0 = 1, ell = 2 and a lazy norm object whose
``d(p)`` estimates ||(a(A - mu I))^p||_1^(1/p) with ``onenormest``
(html :399-463).  This module restates that selection: Code Fragment 3.1
and conditions (3.11)-(3.13) of A. H. Al-Mohy and N. J. Higham, "Computing
the action of the matrix exponential, with an application to exponential
integrators", SIAM J. Sci. Comput. 33 (2011) 488-511, with the published
theta_m bounds for double precision (Higham, "Functions of Matrices",
Table A.3 for m <= 30, and Table 3.1 of the 2011 paper for m = 35..55).
The products inside ``onenormest`` run on the GPU.
"""
from __future__ import annotations

import numpy as np

# theta_m for u = 2^-53, in the table order the selection loop visits
THETA = {
    1: 2.29e-16, 2: 2.58e-8, 3: 1.39e-5, 4: 3.40e-4, 5: 2.40e-3, 6: 9.07e-3, 7: 2.38e-2, 8: 5.00e-2,
    9: 8.96e-2, 10: 1.44e-1, 11: 2.14e-1, 12: 3.00e-1, 13: 4.00e-1, 14: 5.14e-1, 15: 6.41e-1,
    16: 7.81e-1, 17: 9.31e-1, 18: 1.09, 19: 1.26, 20: 1.44, 21: 1.62, 22: 1.82, 23: 2.01, 24: 2.22,
    25: 2.43, 26: 2.64, 27: 2.86, 28: 3.08, 29: 3.31, 30: 3.54, 35: 4.7, 40: 6.0, 45: 7.2, 50: 8.5,
    55: 9.9,
}


def p_max(m_max):
    """Largest p with p (p - 1) <= m_max + 1."""
    lo = int(np.floor(np.sqrt(m_max)))
    hi = int(np.ceil(np.sqrt(m_max) + 1))
    return max(p for p in range(lo, hi + 1) if p * (p - 1) <= m_max + 1)


def condition_3_13(A_1_norm, n0, m_max, ell):
    """True when the exact 1-norm suffices (eq. 3.13)."""
    pm = p_max(m_max)
    return A_1_norm <= 2 * ell * pm * (pm + 3) * (THETA[m_max] / float(n0 * m_max))


def fragment_3_1(norm_info, n0, tol, m_max=55, ell=2):
    """(m*, s) minimising m s, Code Fragment 3.1."""
    if ell < 1:
        raise ValueError("expected ell to be a positive integer")
    best_m = best_s = None
    if condition_3_13(norm_info.onenorm(), n0, m_max, ell):
        for m, theta in THETA.items():
            s = int(np.ceil(norm_info.onenorm() / theta))
            if best_m is None or m * s < best_m * best_s:
                best_m, best_s = m, s
    else:
        for p in range(2, p_max(m_max) + 1):
            for m in range(p * (p - 1) - 1, m_max + 1):
                if m in THETA:
                    s = int(np.ceil(norm_info.alpha(p) / THETA[m]))
                    if best_m is None or m * s < best_m * best_s:
                        best_m, best_s = m, s
        best_s = max(best_s, 1)
    return best_m, best_s


class LazyOperatorNormInfo:
    """Exact 1-norm of a(A - mu I) and lazy 1-norm estimates of its powers
    (html :399-463).

    ``apply`` / ``apply_h`` map an [n, k] block to a (A - mu I) X and
    conj(a) (A^H - conj(mu) I) X.  With ``device`` (an [n, k] block dtype and
    torch device) the products and the estimator run on device tensors
    (``_onenormest.onenormest_device``); otherwise they take host arrays and
    scipy's ``onenormest`` drives them.
    """

    def __init__(self, apply, apply_h, n, A_1_norm, a, dtype, ell=2, device=None):
        self._apply = apply
        self._apply_h = apply_h
        self._n = n
        self._a = a
        self._dtype = dtype
        self._A_1_norm = A_1_norm
        self._ell = ell
        self._d = {}
        self._device = device
        self.matvecs = 0

    def onenorm(self):
        return np.abs(self._a) * self._A_1_norm

    def _linop(self):
        from scipy.sparse.linalg import LinearOperator

        def mv(v):
            self.matvecs += 1
            return self._apply(v)

        def rmv(v):
            self.matvecs += 1
            return self._apply_h(v)

        return LinearOperator((self._n, self._n), dtype=self._dtype, matvec=mv, rmatvec=rmv, matmat=mv,
                              rmatmat=rmv)

    def d(self, p):
        if p not in self._d:
            if self._device is not None:
                from ._onenormest import onenormest_device
                tdtype, dev = self._device

                def mm(X, f=self._apply):
                    for _ in range(p):
                        X = f(X)
                        self.matvecs += 1
                    return X

                def rmm(X, f=self._apply_h):
                    for _ in range(p):
                        X = f(X)
                        self.matvecs += 1
                    return X
                est = onenormest_device(mm, rmm, self._n, tdtype, dev, t=self._ell)
            else:
                from scipy.sparse.linalg import onenormest
                est = onenormest(self._linop() ** p)
            self._d[p] = est ** (1.0 / p)
        return self._d[p]

    def alpha(self, p):
        return max(self.d(p), self.d(p + 1))
