"""The Python drop-in API on the GPU: same results as the reference fixtures
when circuits are built from this package's gate classes, and the reference's
error behaviour for bad input."""
import math

import numpy as np
import pytest

import fastfermion_gb300 as ff
from fastfermion_gb300 import _native
from golden_io import assert_same_terms, load

pytestmark = pytest.mark.gpu


def test_config1_through_python_api():
    fx = load("cfg1_chain")
    c = ff.build_circuit(ff.workloads.chain_circuit())
    r = ff.propagate(c, ff.PauliString("Z7"), maxdegree=6, mincoeff=1e-8)
    assert len(r) == 2646
    assert abs(r.overlapwithzero() - complex(*fx["overlap"])) < 1e-12
    k, a, b = r.arrays()
    assert_same_terms((k, a, b), (fx["res_keys"], fx["res_re"], fx["res_im"]))
    # terms dict view matches too
    assert len(r.terms) == 2646
    assert r.terms[ff.PauliString("Z7")] == complex(a[(k[2] == 1 << 7) & (k[0] == 0)][0], 0)


def test_unbatched_keyword_and_states():
    fx = load("cfg1_chain_unbatched")
    c = ff.build_circuit(ff.workloads.chain_circuit())
    r = ff.propagate(c, ff.PauliString("Z7"), maxdegree=6, mincoeff=1e-8, batched=False)
    assert len(r) == int(fx["n_terms"])
    s = ff.QubitProductState([1, 3])
    host = ff.PauliPolynomial.from_arrays(*r.arrays())
    assert abs(s(r) - s(host)) < 1e-12


def test_majorana_through_python_api():
    fx = load("ref_majorana_2")
    circ = [ff.MROT(ff.MajoranaString([0, 2]), 0.2j, 0.1), ff.MROT(ff.MajoranaString([0, 1, 2, 3]), 0.3, 0.1)]
    r = ff.propagate(circ, ff.poly("-1j*m2 + 2.1 m1 m0"))
    assert_same_terms(r.arrays(), (fx["res_keys"], fx["res_re"], fx["res_im"]))
    st = ff.FockState([0, 1])
    assert abs(st(r) - complex(*fx["state_values"][2])) < 1e-12


def test_hubbard_positional_majorana_args():
    fx = load("hubbard_6x6_2steps")
    c = ff.build_circuit(ff.workloads.hubbard_circuit(6, 6, steps=2))
    obs = ff.MajoranaPolynomial([], 0.5) + ff.MajoranaPolynomial([0, 1], 0.5j)
    r = ff.propagate(c, obs, 6, 1e-7)
    assert len(r) == int(fx["n_terms"])


def test_empty_observable_and_circuit():
    r = ff.propagate([], ff.PauliPolynomial())
    assert len(r) == 0 and r.overlapwithzero() == 0
    r = ff.propagate([], ff.PauliString("Z0"))
    assert len(r) == 1 and r.overlapwithzero() == 1


def test_duplicate_input_keys_rejected():
    ctx = _native.context(0)
    keys = np.zeros((4, 2), dtype=np.uint64)
    keys[2, :] = 1
    with pytest.raises(RuntimeError, match="duplicate"):
        ctx.pauli_propagate(keys, np.ones(2), None, np.zeros(0, dtype=_native.PAULI_GATE),
                            dict(maxdegree=128, topk=0, mincoeff=0.0, max_xweight=-1,
                                 xtrunc_period=1, batched=1, deterministic=0))
    # the context stays usable
    r = ff.propagate([ff.ROT("X", [0], 0.3)], ff.PauliString("Z0"))
    assert len(r) == 2


def test_bad_clifford_qubit_rejected():
    ctx = _native.context(0)
    g = np.zeros(1, dtype=_native.PAULI_GATE)
    g["kind"] = _native.CNOT
    g["q0"], g["q1"] = 0, 200
    keys = np.zeros((4, 1), dtype=np.uint64)
    with pytest.raises(RuntimeError, match="out of range"):
        ctx.pauli_propagate(keys, np.ones(1), None, g, dict(maxdegree=128, topk=0, mincoeff=0.0,
                                                            max_xweight=-1, xtrunc_period=1,
                                                            batched=1, deterministic=0))


def test_wide_register_and_complex_coefficients():
    """Qubits on both 64-bit words with complex coefficients: GPU = oracle."""
    from oracle import oracle as O
    rng = np.random.default_rng(3)
    qs = [0, 5, 63, 64, 70, 127]
    circ = []
    for _ in range(60):
        a, b = rng.choice(qs, 2, replace=False)
        circ.append(ff.ROT("XY"[rng.integers(2)] + "Z", [int(a), int(b)], float(rng.uniform(-2, 2))))
        if rng.random() < 0.3:
            circ.append(ff.CNOT(int(a), int(b)))
    obs = ff.PauliPolynomial(ff.PauliString([(127, "Z")]), 0.3 - 0.7j) + ff.PauliString([(0, "X"), (64, "Y")])
    r = ff.propagate(circ, obs, mincoeff=1e-9)
    k, a, b = obs.arrays()
    o = O.pauli_propagate(ff.encode_pauli_circuit(circ), k, a, b, mincoeff=1e-9)
    assert_same_terms(r.arrays(), (o.keys, o.re, o.im))


def test_reference_quirk_unknown_strategy_returns_input():
    obs = ff.PauliString("Z0")
    r = ff.propagate([ff.ROT("X", [0], 0.3)], obs, n_threads=4, parallel="bogus")
    assert len(r) == 1


def test_autotune_space_follows_the_circuit_kind():
    from fastfermion_gb300.autotune import DEFAULT_SPACE, MAJORANA_SPACE, _is_majorana
    from fastfermion_gb300 import _native
    assert _is_majorana(ff.build_circuit(ff.workloads.hubbard_circuit(2, 2, steps=1)))
    assert not _is_majorana(ff.build_circuit(ff.workloads.kicked_ising_circuit(0.5, 3, 3, 1)))
    assert not _is_majorana([])
    for space in (DEFAULT_SPACE, MAJORANA_SPACE):
        assert set(space) <= set(_native.Context.OPTIONS)


@pytest.mark.gpu
def test_engine_options_and_autotune():
    """Options change speed only; the tuner checks that and keeps the fastest."""
    from fastfermion_gb300 import _native
    ctx = _native.context(0)
    before = {k: ctx.get_option(k) for k in ctx.OPTIONS}
    with pytest.raises(RuntimeError):
        ctx.set_option("orbit_window", 99)
    with pytest.raises(RuntimeError):
        ctx.set_option("no_such_option", 1)
    circ = ff.build_circuit(ff.workloads.kicked_ising_circuit(0.5, 6, 6, 8))
    obs = ff.PauliString([(21, "Z")])
    ref = ff.propagate(circ, obs, maxdegree=6, mincoeff=1e-5)
    res = ff.autotune(circ, obs, repeats=1, maxdegree=6, mincoeff=1e-5)
    from fastfermion_gb300.autotune import DEFAULT_SPACE
    assert set(res["options"]) == set(DEFAULT_SPACE)
    assert len(res["timings"]) >= 5
    tuned = ff.propagate(circ, obs, maxdegree=6, mincoeff=1e-5)
    assert len(tuned) == len(ref) and tuned.overlapwithzero() == pytest.approx(ref.overlapwithzero(), abs=1e-12)
    for k, v in before.items():
        ctx.set_option(k, v)
