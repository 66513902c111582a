"""Conversions computed on the GPU: the Jordan-Wigner map of Majorana
polynomials (src/transforms.h:124-151) and sparse matrices of Pauli
polynomials (src/pauli/sparse.h:20-131).  Fixtures jw_*.npz and sparse_*.npz
are made by the reference itself (tests/golden/make_golden.py)."""
import numpy as np
import pytest

import fastfermion_gb300 as ff
from golden_io import assert_same_terms, load
from oracle import oracle as O

JW = ["jw_small", "jw_wide"]
SPARSE = ["sparse_random6", "sparse_propagated", "sparse_dropped_qubits"]


def pruned(indptr, indices, data, tol=1e-13):
    """CSC arrays without the entries of magnitude <= tol.  Within a group of
    terms with the same X mask the reference sums in the order its std::sort
    leaves ties in (which follows its hash-map iteration order), so where the
    terms cancel it can keep a residue of ~1e-17 where a fixed order gives an
    exact zero; structures are compared without such entries."""
    indptr = np.asarray(indptr, dtype=np.int64)
    keep = np.abs(data) > tol
    col = np.repeat(np.arange(indptr.size - 1), np.diff(indptr))
    counts = np.bincount(col[keep], minlength=indptr.size - 1)
    return np.concatenate([[0], np.cumsum(counts)]), np.asarray(indices)[keep], np.asarray(data)[keep]


def same_matrix(a, b):
    pa, pb = pruned(*a), pruned(*b)
    np.testing.assert_array_equal(pa[0], pb[0])
    np.testing.assert_array_equal(pa[1], pb[1])
    np.testing.assert_allclose(pa[2], pb[2], rtol=0, atol=1e-12)


# ---------------------------------------------------------------------------
# CPU: the oracle's restatements against the reference's outputs
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("name", JW)
def test_oracle_jw_matches_reference(name):
    fx = load(name)
    got = O.jordan_wigner(fx["obs_keys"], fx["obs_re"], fx["obs_im"])
    assert_same_terms(got, (fx["res_keys"], fx["res_re"], fx["res_im"]))


@pytest.mark.parametrize("name", SPARSE)
def test_oracle_sparse_matches_reference(name):
    fx = load(name)
    got = O.pauli_sparse(fx["obs_keys"], fx["obs_re"], fx["obs_im"], int(fx["n"]))
    same_matrix(got, (fx["indptr"], fx["indices"], fx["data"]))


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("name", JW)
def test_gpu_jw_matches_reference(name):
    fx = load(name)
    p = ff.jw(ff.MajoranaPolynomial.from_arrays(fx["obs_keys"], fx["obs_re"], fx["obs_im"]))
    assert_same_terms(p.arrays(), (fx["res_keys"], fx["res_re"], fx["res_im"]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", SPARSE)
def test_gpu_sparse_matches_reference(name):
    fx = load(name)
    p = ff.PauliPolynomial.from_arrays(fx["obs_keys"], fx["obs_re"], fx["obs_im"])
    m = p.sparse(int(fx["n"]))
    same_matrix((m.indptr.astype(np.int64), m.indices.astype(np.int64), m.data),
                (fx["indptr"], fx["indices"], fx["data"]))
    # against the oracle (same summation order): identical arrays
    indptr, indices, data = O.pauli_sparse(fx["obs_keys"], fx["obs_re"], fx["obs_im"], int(fx["n"]))
    np.testing.assert_array_equal(m.indptr, indptr)
    np.testing.assert_array_equal(m.indices, indices)
    assert np.array_equal(m.data, data)


@pytest.mark.gpu
def test_gpu_sparse_of_propagated_result_matches_dense():
    """A device-resident propagation result, n = 9: CSC against the oracle and
    against the dense matrix built from Kronecker products."""
    circ = ff.build_circuit(ff.workloads.chain_circuit(n=9, layers=4))
    res = ff.propagate(circ, ff.PauliString([(4, "Z")]), maxdegree=6, mincoeff=1e-8)
    k, re, im = res.arrays()
    m = res.sparse(9)
    indptr, indices, data = O.pauli_sparse(k, re, im, 9)
    np.testing.assert_array_equal(m.indptr, indptr)
    np.testing.assert_array_equal(m.indices, indices)
    assert np.array_equal(m.data, data)
    # dense check: qubit 0 is the leftmost factor
    P = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]), "Y": np.array([[0, -1j], [1j, 0]]),
         "Z": np.diag([1.0, -1.0])}
    dense = np.zeros((512, 512), dtype=complex)
    for t in range(re.size):
        mat = np.array([[1.0 + 0j]])
        for q in range(9):
            xb, zb = (int(k[0, t]) >> q) & 1, (int(k[2, t]) >> q) & 1
            mat = np.kron(mat, P["IZXY"[xb * 2 + zb]])
        dense += complex(re[t], im[t]) * mat
    np.testing.assert_allclose(m.toarray(), dense, rtol=0, atol=1e-12)


@pytest.mark.gpu
def test_gpu_jw_of_hubbard_result():
    """The 6x6 Hubbard propagation result (3 steps, device-resident) mapped to
    Pauli strings: the map is a bijection on strings, so the term count is kept
    (no coefficient is zero), and a sample of terms matches the oracle."""
    circ = ff.build_circuit(ff.workloads.hubbard_circuit(6, 6, steps=3))
    obs = ff.MajoranaPolynomial([], 0.5) + ff.MajoranaPolynomial([0, 1], 0.5j)
    res = ff.propagate(circ, obs, maxdegree=6, mincoeff=1e-7)
    k, re, im = res.arrays()
    p = ff.jw(ff.MajoranaPolynomial.from_arrays(k, re, im))
    assert len(p) == re.size
    sel = np.random.default_rng(0).choice(re.size, 3000, replace=False)
    want = O.jordan_wigner(k[:, sel], re[sel], im[sel])
    pk, pre, pim = p.arrays()
    at = {tuple(int(pk[w, i]) for w in range(4)): i for i in range(pre.size)}
    wk, wre, wim = want
    for t in range(wre.size):
        i = at[tuple(int(wk[w, t]) for w in range(4))]
        assert pre[i] == wre[t] and pim[i] == wim[t]
