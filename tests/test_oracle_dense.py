"""The oracle against dense linear algebra: without truncation, the propagated
polynomial equals U^dagger O U; the Jordan-Wigner map and the sparse export give
the same operators as their dense matrices.

The reference's own circuit tests check propagation against the naive
product U^dagger O U (pauli_circuit_test.py:53-92, majorana_circuit_test.py:6-41).
These tests do the same for the oracle, so its pinning does not rest on the
reference's fixtures alone: every gate kind, both 64-bit key words (Pauli
qubits are spread over 0..127), complex coefficients, and Majorana strings
of every degree class (Hermitian or not).

Conventions (the reference's): circuit gate 0 acts on the state first, so
U = G_{m-1} ... G_0; ROT(P, theta) = exp(-i theta/2 P); a Majorana gate with
string A is exp(-i theta/2 i^r gamma_A), r = 1 when gamma_A is not Hermitian
(|A| mod 4 in {2, 3}); gamma_{2j} = Z..Z X_j and gamma_{2j+1} = Z..Z Y_j with
qubit 0 the leftmost tensor factor.
"""
import numpy as np
import pytest
from scipy.linalg import expm

from oracle import oracle as O

I2 = np.eye(2, dtype=complex)
X = np.array([[0, 1], [1, 0]], dtype=complex)
Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
Z = np.array([[1, 0], [0, -1]], dtype=complex)


def kron_all(mats):
    out = np.ones((1, 1), dtype=complex)
    for m in mats:
        out = np.kron(out, m)
    return out


def one_qubit(n, q, m):
    return kron_all([m if i == q else I2 for i in range(n)])


def pauli_matrix(key, qubits):
    """Dense matrix of the Pauli string with key planes (x0, x1, z0, z1)."""
    mats = []
    for q in qubits:
        w, b = divmod(q, 64)
        x = (int(key[w]) >> b) & 1
        z = (int(key[2 + w]) >> b) & 1
        mats.append([[I2, Z], [X, Y]][x][z])
    return kron_all(mats)


def polynomial_matrix(keys, re, im, qubits):
    dim = 2 ** len(qubits)
    out = np.zeros((dim, dim), dtype=complex)
    for t in range(keys.shape[1]):
        out += complex(re[t], im[t]) * pauli_matrix(keys[:, t], qubits)
    return out


def set_bit(key, q, plane):
    w, b = divmod(q, 64)
    key[plane * 2 + w] |= np.uint64(1) << np.uint64(b)


def random_pauli_key(rng, qubits, weight):
    key = np.zeros(4, dtype=np.uint64)
    for q in rng.choice(qubits, size=weight, replace=False):
        p = int(rng.integers(1, 4))  # 1 X, 2 Y, 3 Z
        if p in (1, 2):
            set_bit(key, int(q), 0)
        if p in (2, 3):
            set_bit(key, int(q), 1)
    return key


def clifford_matrix(kind, n, i, j):
    if kind == O.H:
        return one_qubit(n, i, np.array([[1, 1], [1, -1]], dtype=complex) / np.sqrt(2))
    if kind == O.S:
        return one_qubit(n, i, np.diag([1, 1j]))
    p0 = np.diag([1, 0]).astype(complex)
    p1 = np.diag([0, 1]).astype(complex)
    if kind == O.CNOT:
        return kron_all([p0 if k == i else I2 for k in range(n)]) + kron_all(
            [p1 if k == i else (X if k == j else I2) for k in range(n)])
    if kind == O.CZ:
        return kron_all([p0 if k == i else I2 for k in range(n)]) + kron_all(
            [p1 if k == i else (Z if k == j else I2) for k in range(n)])
    if kind == O.SWAP:
        return 0.5 * (np.eye(2 ** n) + one_qubit(n, i, X) @ one_qubit(n, j, X)
                      + one_qubit(n, i, Y) @ one_qubit(n, j, Y) + one_qubit(n, i, Z) @ one_qubit(n, j, Z))
    raise ValueError(kind)


@pytest.mark.parametrize("seed", range(6))
def test_pauli_oracle_equals_dense_heisenberg_product(seed):
    rng = np.random.default_rng(100 + seed)
    qubits = [0, 37, 63, 64, 100] if seed % 2 else [0, 1, 2, 3, 4]
    n = len(qubits)
    gates = np.zeros(40, dtype=O.PAULI_GATE)
    U = np.eye(2 ** n, dtype=complex)
    for g in gates:
        kind = int(rng.integers(0, 6)) if rng.random() < 0.4 else O.ROT
        if kind == O.ROT:
            key = random_pauli_key(rng, qubits, int(rng.integers(1, 4)))
            g["kind"] = O.ROT
            g["x"] = key[:2]
            g["z"] = key[2:]
            g["theta"] = rng.uniform(-np.pi, np.pi)
            G = expm(-0.5j * g["theta"] * pauli_matrix(key, qubits))
        else:
            a, b = rng.choice(n, size=2, replace=False)
            g["kind"], g["q0"], g["q1"] = kind, qubits[a], qubits[b]
            G = clifford_matrix(kind, n, int(a), int(b))
        U = G @ U
    nt = 5
    keys = np.stack([random_pauli_key(rng, qubits, int(rng.integers(1, n + 1))) for _ in range(nt)], axis=1)
    keys = np.unique(keys, axis=1)
    re = rng.normal(size=keys.shape[1])
    im = rng.normal(size=keys.shape[1])
    r = O.pauli_propagate(gates, keys, re, im, batched=bool(seed % 3))
    got = polynomial_matrix(r.keys, r.re, r.im, qubits)
    want = U.conj().T @ polynomial_matrix(keys, re, im, qubits) @ U
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
    # expectations in computational basis states: <b|O|b>, qubit 0 leftmost
    for _ in range(4):
        bits = rng.integers(0, 2, size=n)
        b = [0, 0]
        for q, v in zip(qubits, bits):
            b[q // 64] |= int(v) << (q % 64)
        idx = int("".join(str(int(v)) for v in bits), 2)
        assert abs(r.qubit_state(b[0], b[1]) - want[idx, idx]) <= 1e-12
    assert abs(r.overlapwithzero() - want[0, 0]) <= 1e-12


def gamma(n_modes, i):
    """Jordan-Wigner Majorana operator gamma_i on n_modes // 2 qubits."""
    nq = n_modes // 2
    j, odd = divmod(i, 2)
    return kron_all([Z if k < j else ((Y if odd else X) if k == j else I2) for k in range(nq)])


def majorana_matrix(key, n_modes):
    out = np.eye(2 ** (n_modes // 2), dtype=complex)
    for i in range(n_modes):
        if (int(key[i // 64]) >> (i % 64)) & 1:
            out = out @ gamma(n_modes, i)
    return out


@pytest.mark.parametrize("seed", range(6))
def test_majorana_oracle_equals_dense_heisenberg_product(seed):
    rng = np.random.default_rng(200 + seed)
    n_modes = 8
    gates = np.zeros(25, dtype=O.MAJORANA_GATE)
    U = np.eye(2 ** (n_modes // 2), dtype=complex)
    for g in gates:
        deg = int(rng.integers(1, 5))
        key = np.zeros(4, dtype=np.uint64)
        for i in rng.choice(n_modes, size=deg, replace=False):
            key[0] |= np.uint64(1) << np.uint64(int(i))
        g["alpha"] = key
        g["r"] = 1 if deg % 4 in (2, 3) else 0
        g["theta"] = rng.uniform(-np.pi, np.pi)
        H = (1j ** int(g["r"])) * majorana_matrix(key, n_modes)
        assert np.allclose(H, H.conj().T)
        U = expm(-0.5j * g["theta"] * H) @ U
    keys = np.zeros((4, 4), dtype=np.uint64)
    for t in range(4):
        for i in rng.choice(n_modes, size=int(rng.integers(1, n_modes)), replace=False):
            keys[0, t] |= np.uint64(1) << np.uint64(int(i))
    keys = np.unique(keys, axis=1)
    re = rng.normal(size=keys.shape[1])
    im = rng.normal(size=keys.shape[1])
    r = O.majorana_propagate(gates, keys, re, im)
    dim = 2 ** (n_modes // 2)
    got = np.zeros((dim, dim), dtype=complex)
    for t in range(r.keys.shape[1]):
        got += complex(r.re[t], r.im[t]) * majorana_matrix(r.keys[:, t], n_modes)
    obs = np.zeros((dim, dim), dtype=complex)
    for t in range(keys.shape[1]):
        obs += complex(re[t], im[t]) * majorana_matrix(keys[:, t], n_modes)
    want = U.conj().T @ obs @ U
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
    # Fock states: <b|O|b> with mode pair j on qubit j
    for occ in range(2 ** (n_modes // 2)):
        bits = [(occ >> j) & 1 for j in range(n_modes // 2)]
        idx = int("".join(str(v) for v in bits), 2)
        assert abs(r.fock_state(occ, 0) - want[idx, idx]) <= 1e-12


@pytest.mark.parametrize("seed", range(4))
def test_jordan_wigner_restatement_equals_dense_majorana_products(seed):
    """jw maps every Majorana string to the Pauli string of the same operator."""
    rng = np.random.default_rng(300 + seed)
    n_modes = 8
    keys = np.zeros((4, 6), dtype=np.uint64)
    for t in range(6):
        for i in rng.choice(n_modes, size=int(rng.integers(0, n_modes + 1)), replace=False):
            keys[0, t] |= np.uint64(1) << np.uint64(int(i))
    keys = np.unique(keys, axis=1)
    re = rng.normal(size=keys.shape[1])
    im = rng.normal(size=keys.shape[1])
    pk, pre, pim = O.jordan_wigner(keys, re, im)
    dim = 2 ** (n_modes // 2)
    want = np.zeros((dim, dim), dtype=complex)
    for t in range(keys.shape[1]):
        want += complex(re[t], im[t]) * majorana_matrix(keys[:, t], n_modes)
    got = polynomial_matrix(pk, pre, pim, list(range(n_modes // 2)))
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)


@pytest.mark.parametrize("seed", range(4))
def test_sparse_restatement_equals_dense_matrix(seed):
    """The CSC export is the dense matrix of the polynomial (qubit 0 leftmost)."""
    from scipy.sparse import csc_matrix
    rng = np.random.default_rng(400 + seed)
    n = 4
    keys = np.stack([random_pauli_key(rng, list(range(n)), int(rng.integers(1, n + 1))) for _ in range(8)], axis=1)
    keys = np.unique(keys, axis=1)
    re = rng.normal(size=keys.shape[1])
    im = rng.normal(size=keys.shape[1])
    indptr, indices, data = O.pauli_sparse(keys, re, im, n)
    got = csc_matrix((data, indices, indptr), shape=(2 ** n, 2 ** n)).toarray()
    np.testing.assert_allclose(got, polynomial_matrix(keys, re, im, list(range(n))), rtol=0, atol=1e-12)
