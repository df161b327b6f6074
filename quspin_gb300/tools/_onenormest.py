"""Block 1-norm estimator on device vectors.

The reference estimates ||(a(A - mu I))^p||_1 with scipy's ``onenormest``
(html expm_multiply_parallel_core.html:451-463), whose products, column sums,
sign vectors and row maxima all run on host numpy arrays.  This restates the
published algorithm -- N. J. Higham and F. Tisseur, "A block algorithm for
matrix 1-norm estimation, with an application to 1-norm pseudospectra",
SIAM J. Matrix Anal. Appl. 21 (2000) 1185-1201, Algorithm 2.4 with t
columns and at most itmax iterations -- on device tensors, so only a few
scalars per iteration cross to the host.  The random +-1 starting columns
come from numpy's global generator, like scipy's.
"""
from __future__ import annotations

import numpy as np
import torch


def _sign(Y):
    if Y.is_complex():
        a = Y.abs()
        return torch.where(a == 0, torch.ones_like(Y), Y / torch.where(a == 0, torch.ones_like(a), a))
    return torch.where(Y >= 0, torch.ones_like(Y), -torch.ones_like(Y))


def _random_pm1(n, t, dtype, device):
    return torch.tensor(np.random.randint(0, 2, size=(n, t)) * 2 - 1, dtype=dtype, device=device)


def _parallel_cols(S, T, n):
    """For each column of S, whether it is parallel to some column of T
    (entries are unit modulus, so parallel means |<s, t>| == n)."""
    if T is None or T.shape[1] == 0:
        return torch.zeros(S.shape[1], dtype=torch.bool, device=S.device)
    # inner products as broadcast products and column sums (a [1, n] x [n, m]
    # library GEMM with a long inner dimension is far slower on the device)
    G = (S.conj().unsqueeze(2) * T.unsqueeze(1)).sum(dim=0).abs()
    return (G >= n - 0.5).any(dim=1)


def onenormest_device(matmat, rmatmat, n, dtype, device, t=2, itmax=5):
    """Estimate of ||B||_1 for B given by matmat(X) = B X and
    rmatmat(X) = B^H X on device [n, t] blocks."""
    if t >= n:
        # exact: columns of the identity
        E = torch.eye(n, dtype=dtype, device=device)
        return float(matmat(E).abs().sum(dim=0).max())
    X = torch.ones((n, t), dtype=dtype, device=device)
    if t > 1:
        X[:, 1:] = _random_pm1(n, t - 1, dtype, device)
        for j in range(1, t):
            # resample columns parallel to an earlier column
            for _ in range(n):
                if not bool(_parallel_cols(X[:, j:j + 1], X[:, :j], n)[0]):
                    break
                X[:, j:j + 1] = _random_pm1(n, 1, dtype, device)
    X = X / n
    est_old = 0.0
    ind_hist = set()
    S_old = None
    ind_best = 0
    est = 0.0
    for k in range(1, itmax + 2):
        Y = matmat(X)
        norms = Y.abs().sum(dim=0)
        j = int(torch.argmax(norms))
        est = float(norms[j])
        if k >= 2 and est <= est_old:
            est = est_old
            break
        if est > est_old or k == 2:
            ind_best = int(ind_cols[j]) if k >= 2 else 0
        est_old = est
        if k > itmax:
            break
        S = _sign(Y)
        if S_old is not None and bool(_parallel_cols(S, S_old, n).all()):
            break
        if t > 1:
            for jj in range(t):
                for _ in range(n):
                    par = _parallel_cols(S[:, jj:jj + 1], torch.cat([S[:, :jj], S_old], 1) if S_old is not None
                                         else S[:, :jj], n)
                    if not bool(par[0]):
                        break
                    S[:, jj:jj + 1] = _random_pm1(n, 1, dtype, device)
        S_old = S
        Z = rmatmat(S)
        h = Z.abs().max(dim=1).values
        hmax = float(h.max())
        if k >= 2 and hmax == float(h[ind_best]):
            break
        order = torch.argsort(h, descending=True)[: t + len(ind_hist)].tolist()
        fresh = [i for i in order if i not in ind_hist]
        if t > 1 and len(fresh) == 0:
            break
        ind_cols = (fresh + [i for i in order if i in ind_hist])[:t]
        if all(i in ind_hist for i in ind_cols):
            break
        X = torch.zeros((n, t), dtype=dtype, device=device)
        for c, i in enumerate(ind_cols):
            X[i, c] = 1.0
        ind_hist.update(ind_cols)
    return est
