"""GPU parity: libffg (through its C ABI) against the reference's golden fixtures
and against the C oracle on the same inputs.

Bar: identical term sets and bit-identical coefficients (compared with ==, so
+0 and -0 are equal); expectation values within 1e-12 absolute (summation
order differs from the reference's hash-map order).
"""
import numpy as np
import pytest

from golden_io import assert_same_terms, checksum, fixture_names, load
from gpu_util import run_gpu, run_oracle

pytestmark = pytest.mark.gpu

ALL = fixture_names()
EXACT = [n for n in ALL if int(load(n).get("topk", 0)) == 0]
TOPK = [n for n in ALL if int(load(n).get("topk", 0)) > 0]


@pytest.mark.parametrize("name", EXACT)
def test_matches_reference_fixture(name):
    fx = load(name)
    r = run_gpu(fx)
    keys, re, im = r.copy()
    assert r.n == int(fx["n_terms"])
    if "res_keys" in fx:
        assert_same_terms((keys, re, im), (fx["res_keys"], fx["res_re"], fx["res_im"]))
    assert checksum(keys, re, im) == str(fx["checksum"])
    for b, v in zip(fx["states"], fx["state_values"]):
        if str(fx["kind"]) == "pauli":
            got = r.qubit_state(int(b[0]), int(b[1]))
        else:
            got = r.fock_state(int(b[0]), int(b[1]))
        assert abs(got - complex(v[0], v[1])) <= 1e-12 * max(1.0, abs(complex(v[0], v[1]))), (got, v)
    if str(fx["kind"]) == "pauli":
        ov = r.overlapwithzero()
        assert abs(ov - complex(*fx["overlap"])) <= 1e-12, (ov, fx["overlap"])


@pytest.mark.parametrize("name", [n for n in EXACT if float(load(n)["ref_seconds"]) < 2.0])
def test_matches_oracle(name):
    fx = load(name)
    g = run_gpu(fx)
    o = run_oracle(fx)
    assert_same_terms(g.copy(), (o.keys, o.re, o.im))


@pytest.mark.parametrize("name", TOPK)
def test_topk_magnitudes(name):
    """Top-k: the kept magnitudes equal the reference's (which strings survive
    among exactly tied magnitudes is implementation-defined)."""
    fx = load(name)
    keys, re, im = run_gpu(fx).copy()
    assert keys.shape[1] == int(fx["n_terms"])
    a = np.sort(np.hypot(re, im))
    b = np.sort(np.hypot(fx["res_re"], fx["res_im"]))
    assert np.array_equal(a, b)


def test_deterministic_mode_repeats():
    fx = load("cfg1_chain")
    r1 = run_gpu(fx, deterministic=1)
    r2 = run_gpu(fx, deterministic=1)
    k1, a1, b1 = r1.copy()
    k2, a2, b2 = r2.copy()
    assert np.array_equal(k1, k2) and np.array_equal(a1, a2)
    assert r1.overlapwithzero() == r2.overlapwithzero()
    order = np.lexsort(tuple(k1[w] for w in (3, 2, 1, 0)))
    assert np.array_equal(order, np.arange(k1.shape[1]))


def test_apps_counter_matches_oracle():
    from fastfermion_gb300 import _native
    for name in ("cfg1_chain", "cfg1_chain_unbatched", "ref_mixed_clifford", "rand_majorana_03", "rand_majorana_07",
                 "hubbard_3x3", "hubbard_6x6_3steps"):
        fx = load(name)
        run_gpu(fx)
        p = _native.context(0).profile()
        assert p["apps"] == run_oracle(fx).apps, name


SORT_MERGE = [n for n in EXACT if str(load(n)["kind"]) == "pauli" and float(load(n)["ref_seconds"]) < 2.0]


@pytest.mark.parametrize("name", SORT_MERGE)
def test_sort_merge_path_matches_reference(name):
    """The radix-sort + segmented-reduce merge (engine option merge_sort)
    reproduces the reference's term sets bit for bit, like the hash paths."""
    from fastfermion_gb300 import _native
    ctx = _native.context(0)
    ctx.set_option("merge_sort", 1)
    try:
        fx = load(name)
        r = run_gpu(fx)
        keys, re, im = r.copy()
        assert r.n == int(fx["n_terms"])
        assert checksum(keys, re, im) == str(fx["checksum"])
    finally:
        ctx.set_option("merge_sort", 0)
