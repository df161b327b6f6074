"""Generates tests/golden/*.npz (run once where a checkout of the reference
project is available; the fixtures are committed).

What runs from the reference itself:
  * src/quspin/tools/lanczos/_lanczos_utils.py and _expm.py, imported
    unmodified with a stand-in for numba.njit (numba is not installed);
  * the Python body of ExpmMultiplyParallel from the Sphinx viewcode page
    docs/modules/parallel_sparse_tools/expm_multiply_parallel_core/
    expm_multiply_parallel_core.html (text of its <pre> block), with its four
    native wrappers supplied by the oracle restatement (oracle/sparse_oracle.c);
  * scipy.sparse.linalg.expm_multiply, the arbiter of the reference's own
    tests (test/test_expm_multiply_parallel.py:65-74);
  * src/quspin/tools/lanczos/_FTLM.py and _LTLM.py, imported unmodified (their
    import of _get_first_lv resolved to the reference's own _lanczos_utils).
The basis and Hamiltonian come from the oracle restatement (the reference's
native basis core is not installable here).

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT
        (or set QUSPIN_REFERENCE_ROOT; REFERENCE_ROOT is the directory that
        holds the reference's src/, docs/ and test/ folders)
"""
import html
import importlib.util
import os
import re
import sys
import types

import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import expm_multiply

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QUSPIN_REFERENCE_ROOT", "")
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.models import chain_maps, xxz_static  # noqa: E402


def _numba_stub():
    def njit(*a, **k):
        if a and callable(a[0]):
            return a[0]
        return lambda f: f
    sys.modules["numba"] = types.SimpleNamespace(njit=njit)


def reference_lanczos():
    _numba_stub()
    path = os.path.join(REF, "src/quspin/tools/lanczos/_lanczos_utils.py")
    spec = importlib.util.spec_from_file_location("ref_lanczos_utils", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def reference_expm_class():
    page = os.path.join(REF, "docs/modules/parallel_sparse_tools/expm_multiply_parallel_core/"
                        "expm_multiply_parallel_core.html")
    text = open(page).read()
    src = re.search(r'<div class="highlight"><pre>(.*?)</pre>', text, re.S).group(1)
    src = html.unescape(re.sub(r"<[^>]+>", "", src)).replace("[docs]", "")
    src = src.replace("from .expm_multiply_parallel_wrapper import (", "from _golden_wrappers import (")
    wr = types.ModuleType("_golden_wrappers")

    def _trace(indptr, indices, data):
        A = sp.csr_matrix((data, indices, indptr))
        return O.csr_trace(A)

    def _one_norm(indptr, indices, data, shift):
        A = sp.csr_matrix((data, indices, indptr))
        return O.csr_1_norm(A, shift)

    def _expm(indptr, indices, data, s, m_star, tol, mu, a, v, work):
        A = sp.csr_matrix((data, indices, indptr), shape=(v.shape[0], v.shape[0]))
        x = np.ascontiguousarray(v, dtype=np.complex128)
        w = np.zeros(2 * x.size, np.complex128)
        ip, ix, dt, cp, n = O._csr_parts(A)
        a, mu = complex(a), complex(mu)
        eta = np.exp(a * mu / s)
        O.lib().orc_expm_multiply(ip, ix, dt, cp, n, 1 if x.ndim == 1 else x.shape[1], int(s), int(m_star),
                                  float(tol), mu.real, mu.imag, a.real, a.imag, eta.real, eta.imag,
                                  x.view(np.float64).reshape(-1), w.view(np.float64).reshape(-1))
        v[...] = x if np.iscomplexobj(v) else x.real

    wr._wrapper_csr_trace = _trace
    wr._wrapper_csr_1_norm = _one_norm
    wr._wrapper_expm_multiply = _expm
    wr._wrapper_expm_multiply_batch = _expm
    sys.modules["_golden_wrappers"] = wr
    ns = {}
    exec(compile(src, page, "exec"), ns)
    return ns["ExpmMultiplyParallel"]


def reference_thermal(lz):
    pkg = types.ModuleType("quspin")
    tools = types.ModuleType("quspin.tools")
    lanc = types.ModuleType("quspin.tools.lanczos")
    sys.modules.update({"quspin": pkg, "quspin.tools": tools, "quspin.tools.lanczos": lanc,
                        "quspin.tools.lanczos._lanczos_utils": lz})
    mods = []
    for name in ("_FTLM", "_LTLM"):
        path = os.path.join(REF, "src/quspin/tools/lanczos/{}.py".format(name))
        spec = importlib.util.spec_from_file_location("ref" + name, path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mods.append(mod)
    return mods[0].FTLM_static_iteration, mods[1].LTLM_static_iteration


def thermal_fixture(lz):
    """FTLM / LTLM iterations of the reference on an XXZ chain L=14 (k=0,
    p=+1), operators H and a nearest-neighbour zz correlator."""
    L = 14
    m = chain_maps(L)
    ob = O.OracleBasis(L, [(1, L // 2, 0)], pauli=0, kblock=(m["t"], 0), pblock=(m["p"], 0))
    H = sp.csr_matrix(O.make_static(ob, xxz_static(L, 1.0, 0.5), np.float64))
    Czz = sp.csr_matrix(O.make_static(ob, [["zz", [[1.0 / L, i, (i + 1) % L] for i in range(L)]]], np.float64))
    v0 = np.random.default_rng(7).normal(size=ob.Ns)
    E, V, Q_T = lz.lanczos_full(H, v0, 40)
    beta = np.linspace(0.0, 5.0, 11)
    ftlm, ltlm = reference_thermal(lz)
    Of, If = ftlm({"H": H, "Czz": Czz}, E, V, Q_T, beta=beta)
    Ol, Il = ltlm({"H": H, "Czz": Czz}, E, V, Q_T, beta=beta)
    np.savez_compressed(os.path.join(HERE, "thermal_xxz_L14.npz"), H_indptr=H.indptr, H_indices=H.indices,
                        H_data=H.data, C_indptr=Czz.indptr, C_indices=Czz.indices, C_data=Czz.data, v0=v0,
                        E=E, V=V, Q_T=Q_T, beta=beta, ftlm_H=Of["H"], ftlm_C=Of["Czz"], ftlm_I=If,
                        ltlm_H=Ol["H"], ltlm_C=Ol["Czz"], ltlm_I=Il)


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "src", "quspin")):
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set QUSPIN_REFERENCE_ROOT)")
    L = 20
    m = chain_maps(L)
    blocks = dict(kblock=(m["t"], 0), pblock=(m["p"], 0))
    ob = O.OracleBasis(L, [(1, L // 2, 0)], pauli=0, **blocks)
    H = sp.csr_matrix(O.make_static(ob, xxz_static(L, 1.0, 0.5), np.float64))
    rng = np.random.default_rng(2024)
    v = rng.normal(size=ob.Ns) + 1j * rng.normal(size=ob.Ns)
    v /= np.linalg.norm(v)
    v0 = np.random.default_rng(2025).normal(size=ob.Ns)

    EMP = reference_expm_class()
    np.random.seed(0)
    ref = EMP(H, a=-1j)
    w_ref = ref.dot(v.copy())
    w_scipy = expm_multiply(-1j * H, v)

    lz = reference_lanczos()
    thermal_fixture(lz)
    E, V, Q_T = lz.lanczos_full(H, v0, 60)
    E_iter, V_iter = lz.lanczos_iter(H, v0, 60, return_vec_iter=False)

    np.savez_compressed(os.path.join(HERE, "c1_xxz_L20.npz"), states=ob.states, norms=ob.norms,
                        indptr=H.indptr, indices=H.indices, data=H.data, v=v, v0=v0, expm_ref=w_ref,
                        expm_scipy=w_scipy, m_star=ref._m_star, s=ref._s, mu=complex(ref._mu),
                        A_1_norm=ref._A_1_norm, lanczos_E=E, lanczos_iter_E=E_iter)

    # the reference's random-matrix test shape (test_expm_multiply_parallel.py:52-75)
    rs = np.random.RandomState(0)
    N = 3500
    A = sp.random(N, N, density=np.log(N) / N, format="csr", random_state=rs) \
        + 1j * sp.random(N, N, density=np.log(N) / N, format="csr", random_state=rs)
    A = sp.csr_matrix((A + A.conj().T) / 2)
    x = rs.normal(0, 1, N) + 1j * rs.normal(0, 1, N)
    x /= np.linalg.norm(x)
    np.random.seed(0)
    y_ref = EMP(A, a=-0.7j).dot(x.copy())
    y_scipy = expm_multiply(-0.7j * A, x)
    np.savez_compressed(os.path.join(HERE, "random_complex_N3500.npz"), indptr=A.indptr, indices=A.indices,
                        data=A.data, x=x, expm_ref=y_ref, expm_scipy=y_scipy)
    print("Ns", ob.Ns, "nnz", H.nnz, "m*,s", ref._m_star, ref._s, "E0", E[0],
          "|ref-scipy|", np.abs(w_ref - w_scipy).max(), np.abs(y_ref - y_scipy).max())


if __name__ == "__main__":
    main()
