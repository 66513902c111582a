"""Product states on single strings, against dense matrices (host-side, no GPU):
the cases of the reference's state tests (test/state_test.py:6-70) for the
whole-space vectors, with the operators built here from Kronecker products."""
import itertools

import numpy as np

import fastfermion_gb300 as ff

I2 = np.eye(2, dtype=complex)
X = np.array([[0, 1], [1, 0]], dtype=complex)
Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
Z = np.array([[1, 0], [0, -1]], dtype=complex)


def kron_all(mats):
    out = np.ones((1, 1), dtype=complex)
    for m in mats:
        out = np.kron(out, m)
    return out


def subsets(items):
    items = list(items)
    for r in range(len(items) + 1):
        yield from itertools.combinations(items, r)


def test_basis_vectors():
    for cls in (ff.FockState, ff.QubitProductState):
        assert cls().vec(1) == [1, 0]
        assert cls([0]).vec(1) == [0, 1]
        assert cls([]).vec(2) == [1, 0, 0, 0]
        assert cls([1]).vec(2) == [0, 1, 0, 0]
        assert cls([0]).vec(2) == [0, 0, 1, 0]
        assert cls([0, 1]).vec(2) == [0, 0, 0, 1]


def test_fock_state_of_every_majorana_string():
    m = 4
    gam = []
    for i in range(2 * m):
        j, odd = divmod(i, 2)
        gam.append(kron_all([Z if k < j else ((Y if odd else X) if k == j else I2) for k in range(m)]))
    for S in subsets(range(2 * m)):
        M = np.eye(2 ** m, dtype=complex)
        for i in S:
            M = M @ gam[i]
        ms = ff.MajoranaString(list(S))
        for B in subsets(range(m)):
            st = ff.FockState(list(B))
            v = np.array(st.vec(m))
            assert abs(st(ms) - v @ M @ v) <= 1e-14, (S, B)


def test_qubit_state_of_every_pauli_string():
    n = 3
    single = {"I": I2, "X": X, "Y": Y, "Z": Z}
    for word in itertools.product("IXYZ", repeat=n):
        M = kron_all([single[a] for a in word])
        ps = ff.PauliString([(q, a) for q, a in enumerate(word) if a != "I"])
        for B in subsets(range(n)):
            st = ff.QubitProductState(list(B))
            v = np.array(st.vec(n))
            assert abs(st(ps) - v @ M @ v) <= 1e-14, (word, B)
