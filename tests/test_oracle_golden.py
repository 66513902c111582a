"""Pins the C oracle against fixtures produced by the reference implementation.

The serial oracle mirrors the reference map's iteration order, so term sets,
coefficients AND order-dependent sums (overlapwithzero, state expectations) are
compared bit for bit.  Large results are compared through a checksum of the
sorted term set.
"""
import numpy as np
import pytest

from golden_io import assert_same_terms, checksum, fixture_names, load
from oracle import oracle as O

SLOW = {n for n in fixture_names() if float(load(n)["ref_seconds"]) > 30.0}


def run_oracle(fx, n_threads=1):
    if str(fx["kind"]) == "pauli":
        return O.pauli_propagate(fx["gates"], fx["obs_keys"], fx["obs_re"], fx["obs_im"],
                                 maxdegree=int(fx["maxdegree"]), mincoeff=float(fx["mincoeff"]),
                                 topk=int(fx["topk"]), max_xweight=int(fx["max_xweight"]),
                                 xtrunc_period=int(fx["xtrunc_period"]),
                                 batched=bool(fx["batched"]), n_threads=n_threads)
    md = int(fx["maxdegree"]) if bool(fx["has_maxdegree"]) else None
    return O.majorana_propagate(fx["gates"], fx["obs_keys"], fx["obs_re"], fx["obs_im"],
                                maxdegree=md, mincoeff=float(fx["mincoeff"]))


def _params(names):
    return [pytest.param(n, marks=pytest.mark.slow) if n in SLOW else n for n in names]


@pytest.mark.parametrize("name", _params(fixture_names()))
def test_oracle_matches_reference(name):
    fx = load(name)
    r = run_oracle(fx)
    assert len(r) == int(fx["n_terms"])
    if "res_keys" in fx:
        assert_same_terms((r.keys, r.re, r.im), (fx["res_keys"], fx["res_re"], fx["res_im"]))
        # iteration order is the reference's too
        assert np.array_equal(r.keys, fx["res_keys"])
    assert checksum(r.keys, r.re, r.im) == str(fx["checksum"])
    for b, v in zip(fx["states"], fx["state_values"]):
        got = r.qubit_state(int(b[0]), int(b[1])) if str(fx["kind"]) == "pauli" else r.fock_state(int(b[0]), int(b[1]))
        assert got == complex(v[0], v[1]), (got, v)
    if str(fx["kind"]) == "pauli":
        assert r.overlapwithzero() == complex(*fx["overlap"])


SHARDABLE = [n for n in fixture_names("pauli") if n.startswith(("ref_", "rand_pauli", "cfg1"))
             and float(load(n)["ref_seconds"]) < 0.5]


@pytest.mark.parametrize("name", SHARDABLE)
def test_oracle_sharded_matches_serial(name):
    fx = load(name)
    a = run_oracle(fx, 1)
    b = run_oracle(fx, 3)
    assert_same_terms((a.keys, a.re, a.im), (b.keys, b.re, b.im))
    assert abs(a.overlapwithzero() - b.overlapwithzero()) < 1e-12
    assert a.apps == b.apps


def test_abs_is_hypot():
    rng = np.random.default_rng(1)
    for _ in range(1000):
        a, b = rng.normal(size=2) * 10.0 ** rng.integers(-12, 3)
        assert O.ffo_abs(a, b) == float(np.hypot(a, b))
