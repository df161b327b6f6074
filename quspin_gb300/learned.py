"""Learned choice of the Taylor degree m* and substep count s.

The reference picks (m*, s) for every ``ExpmMultiplyParallel`` with
Al-Mohy & Higham's fragment 3.1 (html expm_multiply_parallel_core.html
:377-463): an exact 1-norm pass over A - mu I and, when that norm is large,
``onenormest`` of powers of a(A - mu I) -- tens of matrix products.  In a
time-dependent evolution this runs at every step.  Here a small MLP
(3 dense layers, 64 hidden units, bfloat16 weights with FP32 accumulation,
``csrc/mlp.cu``) predicts (m*, s) from cheap features of the step; it is
trained on the GPU by the project's own forward / backward / Adam kernels on
(feature, m*, s) tuples that the plain selection generates.  The plain
selection stays the fallback and the arbiter: a step whose Taylor loop used
all m* terms of a substep without the stopping test firing is recomputed
with the plain (m*, s).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _device as D
from . import _lib
from .tools._partition import THETA

_M_KEYS = np.array(sorted(THETA.keys()))


def _bf16(t):
    out = torch.empty(t.shape, dtype=torch.bfloat16, device=t.device)
    _lib.call("qs_mlp_to_bf16", t.numel(), D.ptr(t), D.ptr(out), D.stream())
    return out


class MLP:
    """Dense ReLU network; every product runs in the kernels of csrc/mlp.cu."""

    def __init__(self, din, dout, hidden=64, layers=3, seed=0):
        D.require_cuda()
        dims = [din] + [hidden] * (layers - 1) + [dout]
        g = np.random.default_rng(seed)
        self.dims = dims
        self.W, self.b = [], []
        for i in range(layers):
            w = g.normal(0.0, np.sqrt(2.0 / dims[i]), size=(dims[i + 1], dims[i])).astype(np.float32)
            self.W.append(torch.tensor(w, device=D.device()))
            self.b.append(torch.zeros(dims[i + 1], dtype=torch.float32, device=D.device()))
        self.Wb = [_bf16(w) for w in self.W]
        self._adam = None
        self._step = 0

    @property
    def nparams(self):
        return sum(w.numel() + b.numel() for w, b in zip(self.W, self.b))

    def forward(self, X, keep=False):
        """X: device float32 [B, din] -> [B, dout]."""
        X = X.contiguous()
        B = X.shape[0]
        acts, zs = [X], []
        h = X
        for i, (wb, b) in enumerate(zip(self.Wb, self.b)):
            last = i == len(self.Wb) - 1
            z = torch.empty((B, self.dims[i + 1]), dtype=torch.float32, device=X.device)
            y = torch.empty_like(z)
            _lib.call("qs_mlp_dense_fwd", B, self.dims[i], self.dims[i + 1], D.ptr(h), D.ptr(wb), D.ptr(b),
                      D.ptr(z), D.ptr(y), 0 if last else 1, D.stream())
            zs.append(z)
            acts.append(y)
            h = y
        if keep:
            self._cache = (acts, zs)
        return h

    def backward(self, dY):
        """Gradients of the last forward(keep=True) for output gradient dY."""
        acts, zs = self._cache
        B = dY.shape[0]
        gW, gb = [None] * len(self.W), [None] * len(self.W)
        d = dY.contiguous()
        for i in reversed(range(len(self.W))):
            din, dout = self.dims[i], self.dims[i + 1]
            gw = torch.empty((dout, din), dtype=torch.float32, device=dY.device)
            gbi = torch.empty(dout, dtype=torch.float32, device=dY.device)
            dx = torch.empty((B, din), dtype=torch.float32, device=dY.device) if i > 0 else None
            zin = zs[i - 1] if i > 0 else None
            _lib.call("qs_mlp_dense_bwd", B, din, dout, D.ptr(d), D.ptr(self.Wb[i]), D.ptr(acts[i]), D.ptr(zin),
                      D.ptr(dx), D.ptr(gw), D.ptr(gbi), D.stream())
            gW[i], gb[i] = gw, gbi
            d = dx
        return gW, gb

    def mse(self, Y, T, colw=None):
        """(loss, dY) of the column-weighted mean squared error."""
        total = Y.numel()
        nb = 64
        dY = torch.empty_like(Y)
        part = torch.zeros(nb, dtype=torch.float32, device=Y.device)
        scale = 1.0 / total
        _lib.call("qs_mlp_mse", total, Y.shape[1], D.ptr(Y), D.ptr(T.contiguous()), D.ptr(colw), scale, D.ptr(dY),
                  D.ptr(part), nb, D.stream())
        return part.sum(), dY

    def adam(self, gW, gb, lr=3e-3, b1=0.9, b2=0.999, eps=1e-8):
        if self._adam is None:
            self._adam = [(torch.zeros_like(p), torch.zeros_like(p)) for p in self.W + self.b]
        self._step += 1
        params = self.W + self.b
        grads = gW + gb
        bf = self.Wb + [None] * len(self.b)
        for p, g, (m, v), wb in zip(params, grads, self._adam, bf):
            _lib.call("qs_mlp_adam", p.numel(), D.ptr(p), D.ptr(g), D.ptr(m), D.ptr(v), D.ptr(wb), lr, b1, b2, eps,
                      self._step, D.stream())

    def fit(self, X, T, epochs=400, lr=3e-3, batch=512, colw=None, seed=0):
        """Minibatch Adam on device tensors X [N, din], T [N, dout]."""
        N = X.shape[0]
        g = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(N, generator=g).to(X.device)
            tot = 0.0
            for s in range(0, N, batch):
                idx = perm[s:s + batch]
                Y = self.forward(X[idx], keep=True)
                loss, dY = self.mse(Y, T[idx], colw)
                gW, gb = self.backward(dY)
                self.adam(gW, gb, lr=lr)
                tot += float(loss) * len(idx)
            hist.append(tot / N)
        return hist

    def state(self):
        return {"dims": self.dims, "W": [D.to_host(w) for w in self.W], "b": [D.to_host(b) for b in self.b]}

    def load_state(self, st):
        self.W = [D.to_device(w.astype(np.float32)) for w in st["W"]]
        self.b = [D.to_device(b.astype(np.float32)) for b in st["b"]]
        self.Wb = [_bf16(w) for w in self.W]


class PartitionPredictor:
    """(m*, s) from step features, with the plain selection as fallback.

    Features of a step with generator a (A - mu I): log10 of |a| times an
    upper bound of ||A - mu I||_1 (the sum of the per-part norms weighted by
    the coefficients), log10 |a|, and the coefficients themselves.  Targets
    are m*/55 and log2 s of the plain selection.
    """

    MARGIN_M = 2          # extra Taylor terms over the prediction (the loop stops early anyway)

    def __init__(self, n_coeffs, hidden=64, seed=0):
        self.din = 2 + n_coeffs
        self.net = MLP(self.din, 2, hidden=hidden, layers=3, seed=seed)
        self.mu = np.zeros(self.din, np.float32)
        self.sd = np.ones(self.din, np.float32)

    @staticmethod
    def features(abs_a, norm_bound, coeffs):
        abs_a = np.atleast_1d(np.asarray(abs_a, np.float64))
        norm_bound = np.atleast_1d(np.asarray(norm_bound, np.float64))
        c = np.atleast_2d(np.asarray(coeffs, np.float64))
        if c.shape[0] != abs_a.shape[0]:
            c = c.T
        return np.column_stack([np.log10(abs_a * norm_bound + 1e-300), np.log10(abs_a + 1e-300), c]).astype(
            np.float32)

    @staticmethod
    def targets(m_star, s):
        return np.column_stack([np.asarray(m_star, np.float64) / 55.0,
                                np.log2(np.maximum(np.asarray(s, np.float64), 1.0))]).astype(np.float32)

    def fit(self, feats, m_star, s, epochs=400, lr=3e-3, batch=512, seed=0):
        self.mu = feats.mean(0)
        self.sd = feats.std(0) + 1e-6
        X = D.to_device((feats - self.mu) / self.sd)
        T = D.to_device(self.targets(m_star, s))
        return self.net.fit(X, T, epochs=epochs, lr=lr, batch=batch, seed=seed)

    def predict(self, feats):
        """Integer (m*, s) arrays; m* rounded up to a table degree plus a margin."""
        X = D.to_device(((feats - self.mu) / self.sd).astype(np.float32))
        Y = D.to_host(self.net.forward(X))
        m = np.ceil(Y[:, 0] * 55.0 - 1e-3).astype(np.int64) + self.MARGIN_M
        m = np.clip(m, 1, 55)
        s = np.maximum(np.ceil(2.0 ** Y[:, 1] - 0.25), 1).astype(np.int64)
        return m, s


class NormRatioPredictor:
    """Learned inputs of Code Fragment 3.1 for one operator (the estimator branch).

    When |a| ||A - mu I||_1 is too large for the exact-norm shortcut
    (condition 3.13 fails), the reference estimates
    d_p = ||(a (A - mu I))^p||_1^(1/p) for p = 2 .. 9 with ``onenormest``
    (html expm_multiply_parallel_core.html:451-463): tens of products with the
    full matrix.  The ratios d_p / (|a| ||A - mu I||_1) do not depend on a and
    lie in (0, 1]; this network predicts their logarithms from features that
    cost nothing beyond the exact 1-norm the constructor computes anyway
    (the 1-norm, the dimension, the stored entries per row and |mu|), and the
    selection then runs Code Fragment 3.1 on the predicted d_p.  The outputs
    are raised by ``MARGIN`` (in log10) so that errors fall on the side of
    more work.  The plain selection is the fallback: ExpmMultiplyParallel
    re-runs a product whose Taylor loop used all m* terms of a substep without
    the stopping test firing with the onenormest (m*, s).  Trained on the GPU
    by the kernels of csrc/mlp.cu on (features, ratios) of the plain
    selection over a family of operators (``training_pair``).
    """

    P = tuple(range(2, 10))
    MARGIN = 0.03

    def __init__(self, hidden=64, seed=0):
        self.net = MLP(4, len(self.P), hidden=hidden, layers=3, seed=seed)
        self.mu = np.zeros(4, np.float32)
        self.sd = np.ones(4, np.float32)

    @staticmethod
    def features(one_norm, n, nnz, abs_mu):
        """[B, 4] features of operators A - mu I: log10 of the exact 1-norm,
        log10 of the dimension, stored entries per row / 32, log10(1 + |mu|)."""
        one_norm, n, nnz, abs_mu = (np.atleast_1d(np.asarray(x, np.float64)) for x in (one_norm, n, nnz, abs_mu))
        return np.column_stack([np.log10(one_norm + 1e-300), np.log10(np.maximum(n, 1.0)),
                                nnz / np.maximum(n, 1.0) / 32.0, np.log10(1.0 + abs_mu)]).astype(np.float32)

    @classmethod
    def training_pair(cls, op):
        """(features [1, 4], log10 ratios [1, 8]) from an ExpmMultiplyParallel
        whose plain selection ran in the estimator branch."""
        info = op._norm_info
        base = info.onenorm()
        r = np.array([[np.log10(info.d(p) / base) for p in cls.P]], np.float32)
        A = op.A_device
        f = cls.features(op._A_1_norm, A.shape[0], A.nnz, abs(complex(op._mu)))
        return f, r

    def fit(self, feats, log_ratios, epochs=600, lr=3e-3, batch=64, seed=0):
        self.mu = feats.mean(0)
        self.sd = feats.std(0) + 1e-3
        X = D.to_device((feats - self.mu) / self.sd)
        T = D.to_device(np.asarray(log_ratios, np.float32))
        return self.net.fit(X, T, epochs=epochs, lr=lr, batch=batch, seed=seed)

    def predict_ratios(self, feats):
        """[B, 8] predicted d_p / (|a| ||A - mu I||_1), p = 2 .. 9, at most 1."""
        X = D.to_device(((np.atleast_2d(feats) - self.mu) / self.sd).astype(np.float32))
        Y = D.to_host(self.net.forward(X)).astype(np.float64)
        return np.minimum(10.0 ** (Y + self.MARGIN), 1.0)


class FixedNormInfo:
    """Norm information for Code Fragment 3.1 with given d_p (the learned
    selection): no matrix products."""

    def __init__(self, one_norm, d):
        self._one = float(one_norm)
        self._d = dict(d)
        self.matvecs = 0

    def onenorm(self):
        return self._one

    def d(self, p):
        return self._d[p]

    def alpha(self, p):
        return max(self.d(p), self.d(p + 1))


def norm_ratio_training_set(matrices, scale=100.0, seed=0):
    """(features, log10 ratios) of the plain selection for each device
    matrix: an ExpmMultiplyParallel with |a| ||A - mu I||_1 = scale (far in
    the estimator branch; the ratios do not depend on a), onenormest seeded
    with ``seed`` as the reference's global generator would be."""
    from .tools import ExpmMultiplyParallel
    feats, ratios = [], []
    for A in matrices:
        np.random.seed(seed)
        op = ExpmMultiplyParallel(A, a=-1j)
        if op._A_1_norm == 0:
            continue
        np.random.seed(seed)
        op.set_a(-1j * scale / op._A_1_norm)
        f, r = NormRatioPredictor.training_pair(op)
        feats.append(f)
        ratios.append(r)
    return np.concatenate(feats), np.concatenate(ratios)
