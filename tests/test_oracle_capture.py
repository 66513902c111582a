"""The oracle's record of the partners that the degree filter drops: the
training data of the learned-correction form.

With no coefficient threshold the propagation is linear, and a maximum weight
W' > W satisfies, gate by gate (M' = M + the dropped partners of degree in
(W, W']),

    prod M' - prod M = sum over gates g of (prod_{after g} M') (M'_g - M_g) (prod_{before g} M)

so <O>_W' = <O>_W + the sum over dropped partners of their value propagated
at W' through the gates still to come.  That is the label each dropped term
gets; these tests pin it on the oracle.
"""
import numpy as np
import pytest

import fastfermion_gb300 as ff
from golden_io import load
from oracle import oracle as O


def _z(site):
    keys = np.zeros((4, 1), dtype=np.uint64)
    keys[2 + site // 64, 0] = np.uint64(1) << np.uint64(site % 64)
    return keys, np.ones(1), np.zeros(1)


def _degree(keys):
    x = keys[0] | keys[2]
    y = keys[1] | keys[3]
    return np.array([bin(int(a)).count("1") + bin(int(b)).count("1") for a, b in zip(x, y)])


def _labels(tab, d, wmax):
    out = np.zeros(len(d), dtype=complex)
    for i in range(len(d)):
        r = O.pauli_propagate(tab[: int(d.gate[i])], d.keys[:, i : i + 1], d.re[i : i + 1], d.im[i : i + 1],
                              maxdegree=wmax)
        out[i] = r.overlapwithzero()
    return out


CASES = [
    ("kicked_ising_3x3", lambda: ff.encode_pauli_circuit(ff.build_circuit(
        ff.workloads.kicked_ising_circuit(0.7, 3, 3, 2))), 4, 2, 5),
    ("chain_8", lambda: ff.encode_pauli_circuit(ff.build_circuit(
        ff.workloads.chain_circuit(8, 3))), 3, 2, 4),
]


@pytest.mark.parametrize("name,make,site,w,w2", CASES, ids=[c[0] for c in CASES])
def test_capture_leaves_the_result_unchanged(name, make, site, w, w2):
    tab = make()
    k, re, im = _z(site)
    plain = O.pauli_propagate(tab, k, re, im, maxdegree=w)
    cap, d = O.pauli_propagate_capture(tab, k, re, im, capdeg=w2, maxdegree=w)
    assert np.array_equal(plain.keys, cap.keys)
    assert np.array_equal(plain.re, cap.re) and np.array_equal(plain.im, cap.im)
    assert plain.apps == cap.apps
    deg = _degree(d.keys)
    assert len(d) > 0 and np.all(deg > w) and np.all(deg <= w2)
    assert np.all(tab["kind"][d.gate] == O.ROT)


@pytest.mark.parametrize("name,make,site,w,w2", CASES, ids=[c[0] for c in CASES])
def test_dropped_terms_account_for_the_truncation_error(name, make, site, w, w2):
    tab = make()
    k, re, im = _z(site)
    low, d = O.pauli_propagate_capture(tab, k, re, im, capdeg=w2, maxdegree=w)
    high = O.pauli_propagate(tab, k, re, im, maxdegree=w2)
    lab = _labels(tab, d, w2)
    f_low, f_high = low.overlapwithzero(), high.overlapwithzero()
    assert abs(f_high - f_low) > 1e-3  # the truncation error is not trivially zero
    assert abs(f_high - (f_low + lab.sum())) <= 1e-12


def test_identity_holds_through_clifford_segments():
    fx = load("ref_mixed_clifford")
    tab = fx["gates"]
    k, re, im = fx["obs_keys"], fx["obs_re"], fx["obs_im"]
    deg = int(_degree(np.asarray(k, dtype=np.uint64)).max())
    w, w2 = deg, deg + 2
    low, d = O.pauli_propagate_capture(tab, k, re, im, capdeg=w2, maxdegree=w)
    high = O.pauli_propagate(tab, k, re, im, maxdegree=w2)
    lab = _labels(tab, d, w2)
    assert abs(high.overlapwithzero() - low.overlapwithzero()) > 1e-3
    assert abs(high.overlapwithzero() - (low.overlapwithzero() + lab.sum())) <= 1e-12


def _label_job(args):
    tab, k, re, im, wmax, tau = args
    return O.pauli_propagate(tab, k, re, im, maxdegree=wmax, mincoeff=tau).overlapwithzero()


@pytest.mark.slow
def test_labels_with_a_coefficient_threshold_kicked_ising_10x10():
    """With the workload's threshold tau = 1e-6 the identity is approximate.
    On the 10x10 kicked-Ising circuit (theta_h = 0.3), the W=6 value plus the
    labels at W'=8 of the 909 dropped partners above tau comes within 1e-3 of
    the W=8 value, although the two values differ by 0.28 (about 4 minutes on
    8 cores)."""
    from multiprocessing import get_context
    tab = ff.encode_pauli_circuit(ff.build_circuit(ff.workloads.kicked_ising_circuit(0.3)))
    k, re, im = _z(55)
    tau = 1e-6
    low, d = O.pauli_propagate_capture(tab, k, re, im, capdeg=8, maxdegree=6, mincoeff=tau)
    high = O.pauli_propagate(tab, k, re, im, maxdegree=8, mincoeff=tau, n_threads=8)
    sel = np.nonzero(np.hypot(d.re, d.im) > tau)[0]
    jobs = [(tab[: int(d.gate[i])], d.keys[:, i : i + 1].copy(), d.re[i : i + 1].copy(), d.im[i : i + 1].copy(), 8,
             tau) for i in sel]
    with get_context("spawn").Pool(8) as pool:
        lab = np.array(pool.map(_label_job, jobs, chunksize=4))
    f_low, f_high = low.overlapwithzero(), high.overlapwithzero()
    assert abs(f_high - f_low) > 0.2
    assert abs(f_high - (f_low + lab.sum())) <= 1e-3
