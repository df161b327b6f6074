"""Hamiltonians and symmetry maps of the benchmark configurations, shared by
the tests (the same site-coupling lists the reference's tests and examples
use: test/test_quantum_LinearOperator.py:20-24, test/test_FHM_energies.py:38-47)."""
import numpy as np


def chain_maps(L):
    s = np.arange(L)
    return dict(t=(s + 1) % L, p=s[::-1].copy(), z=-(s + 1))


def xxz_static(L, J=1.0, Delta=0.5, nn=1):
    bonds = [(i, (i + nn) % L) for i in range(L)]
    return [["+-", [[J / 2, i, j] for i, j in bonds]], ["-+", [[J / 2, i, j] for i, j in bonds]],
            ["zz", [[Delta, i, j] for i, j in bonds]]]


def j1j2_static(L, J1=1.0, J2=0.5):
    st = []
    for op in ("+-", "-+"):
        st.append([op, [[J1 / 2, i, (i + 1) % L] for i in range(L)] + [[J2 / 2, i, (i + 2) % L] for i in range(L)]])
    st.append(["zz", [[J1, i, (i + 1) % L] for i in range(L)] + [[J2, i, (i + 2) % L] for i in range(L)]])
    return st


def ising_static(L, hx=0.9, hz=0.5):
    return [["zz", [[-1.0, i, (i + 1) % L] for i in range(L)]], ["x", [[-hx, i] for i in range(L)]],
            ["z", [[-hz, i] for i in range(L)]]]


def square_maps(Lx, Ly):
    N = Lx * Ly
    s = np.arange(N)
    X, Y = s % Lx, s // Lx
    return dict(tx=(X + 1) % Lx + Y * Lx, ty=X + ((Y + 1) % Ly) * Lx, px=(Lx - X - 1) + Y * Lx,
                py=X + (Ly - Y - 1) * Lx, z=-(s + 1))


def hubbard_static(Lx, Ly, t=1.0, U=4.0):
    m = square_maps(Lx, Ly)
    N = Lx * Ly
    hop = [[-t, i, m["tx"][i]] for i in range(N)] + [[-t, i, m["ty"][i]] for i in range(N)]
    hopc = [[+t, i, m["tx"][i]] for i in range(N)] + [[+t, i, m["ty"][i]] for i in range(N)]
    return [["+-|", hop], ["-+|", hopc], ["|+-", hop], ["|-+", hopc], ["n|n", [[U, i, i] for i in range(N)]]]
