"""Learned (m*, s) predictor: the MLP kernels' gradients against a float64
CPU restatement of the same network (bfloat16 weights), training convergence,
and a driven evolution where learned partitions reproduce the plain
selection's states."""
import numpy as np
import pytest
import torch

from tests.models import chain_maps

pytestmark = pytest.mark.gpu


def _bf16_round(w):
    return torch.tensor(w).to(torch.bfloat16).to(torch.float64).numpy()


def test_mlp_gradients_match_cpu(cuda):
    from quspin_gb300.learned import MLP
    net = MLP(5, 2, hidden=64, layers=3, seed=3)
    rng = np.random.default_rng(0)
    B = 37
    X = rng.normal(size=(B, 5)).astype(np.float32)
    T = rng.normal(size=(B, 2)).astype(np.float32)
    Xd, Td = torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda")
    Y = net.forward(Xd, keep=True)
    loss, dY = net.mse(Y, Td)
    gW, gb = net.backward(dY)
    Ws = [_bf16_round(w.cpu().numpy()) for w in net.W]
    bs = [b.cpu().numpy().astype(np.float64) for b in net.b]
    h = [X.astype(np.float64)]
    zs = []
    for i, (W, b) in enumerate(zip(Ws, bs)):
        z = h[-1] @ W.T + b
        zs.append(z)
        h.append(z if i == len(Ws) - 1 else np.maximum(z, 0))
    np.testing.assert_allclose(Y.cpu().numpy(), h[-1], rtol=1e-5, atol=1e-5)
    d = 2 * (h[-1] - T) / T.size
    assert abs(float(loss) - np.mean((h[-1] - T) ** 2)) < 1e-5
    for i in reversed(range(len(Ws))):
        np.testing.assert_allclose(gW[i].cpu().numpy(), d.T @ h[i], rtol=1e-4, atol=1e-6)
        np.testing.assert_allclose(gb[i].cpu().numpy(), d.sum(0), rtol=1e-4, atol=1e-6)
        d = (d @ Ws[i]) * (zs[i - 1] > 0) if i > 0 else None


def test_mlp_training_reduces_loss(cuda):
    from quspin_gb300.learned import MLP
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, size=(2048, 3)).astype(np.float32)
    T = np.column_stack([np.sin(2 * X[:, 0]) + X[:, 1] ** 2, X[:, 2] * X[:, 0]]).astype(np.float32)
    net = MLP(3, 2, seed=0)
    hist = net.fit(torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda"), epochs=60, lr=3e-3, batch=256)
    assert hist[-1] < 0.05 * hist[0]


def _driven(L=10):
    from quspin_gb300 import hamiltonian, spin_basis_general
    m = chain_maps(L)
    b = spin_basis_general(L, kblock=(m["t"], 0), pblock=(m["p"], 0))
    static = [["zz", [[-1.0, i, (i + 1) % L] for i in range(L)]], ["z", [[-0.2, i] for i in range(L)]]]
    drive = lambda t, h0, A, w: h0 + A * np.cos(w * t)
    dyn = [["x", [[-1.0, i] for i in range(L)], drive, (0.8, 0.5, 2 * np.pi)]]
    return hamiltonian(static, dyn, basis=b, dtype=np.float64), drive


def test_driven_learned_matches_plain(cuda):
    from scipy.sparse.linalg import expm_multiply
    from quspin_gb300.learned import PartitionPredictor
    from quspin_gb300.tools.driven import DrivenEvolution
    H, drive = _driven()
    ev = DrivenEvolution(H, nvec=4)
    rng = np.random.default_rng(2)
    ts = rng.uniform(0, 3, 400)
    dts = 10 ** rng.uniform(-3, 0, 400)
    feats, ms, ss = ev.training_set(ts, dts)
    pred = PartitionPredictor(n_coeffs=1, seed=0)
    pred.fit(feats, ms, ss, epochs=150, lr=3e-3, batch=128)
    V = rng.normal(size=(H.Ns, 4)) + 1j * rng.normal(size=(H.Ns, 4))
    V /= np.linalg.norm(V, axis=0)
    dt, nsteps = 0.005, 60
    Fp = torch.tensor(V, device="cuda")
    Fl = Fp.clone()
    ev.run(Fp, 0.0, dt, nsteps, mode="plain")
    ev.run(Fl, 0.0, dt, nsteps, mode="learned", predictor=pred, segment=20)
    wp, wl = Fp.cpu().numpy(), Fl.cpu().numpy()
    assert np.linalg.norm(wl - wp) <= 1e-10 * np.linalg.norm(wp)
    # the plain path against scipy, step by step on the host
    W = V.copy()
    for i in range(nsteps):
        W = expm_multiply(-1j * dt * H.tocsr(time=dt * (i + 0.5)), W)
    assert np.linalg.norm(wp - W) <= 1e-12 * np.linalg.norm(W)


def test_driven_fallback_restores_plain(cuda):
    """A predictor that returns far too small (m*, s) makes the Taylor loop run
    substeps through all m* terms without the stopping test firing; every such
    segment is re-run from its saved state with the plain selection
    (tools/driven.py), so the result equals the plain run's."""
    from quspin_gb300.learned import PartitionPredictor
    from quspin_gb300.tools.driven import DrivenEvolution

    class TooSmall(PartitionPredictor):
        def predict(self, feats):
            k = np.atleast_2d(feats).shape[0]
            return np.full(k, 2, np.int64), np.ones(k, np.int64)

    H, _ = _driven()
    ev = DrivenEvolution(H, nvec=2)
    rng = np.random.default_rng(5)
    V = rng.normal(size=(H.Ns, 2)) + 1j * rng.normal(size=(H.Ns, 2))
    V /= np.linalg.norm(V, axis=0)
    dt, nsteps = 0.05, 20
    Fp = torch.tensor(V, device="cuda")
    Fl = Fp.clone()
    ev.run(Fp, 0.0, dt, nsteps, mode="plain")
    ev.fallbacks = 0
    ev.run(Fl, 0.0, dt, nsteps, mode="learned", predictor=TooSmall(n_coeffs=1), segment=10)
    assert ev.fallbacks == 2
    assert np.array_equal(Fl.cpu().numpy().view(np.float64), Fp.cpu().numpy().view(np.float64))
