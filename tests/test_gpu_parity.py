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


MAJORANA_ROUTE = [n for n in EXACT if str(load(n)["kind"]) == "majorana" and float(load(n)["ref_seconds"]) < 30.0]


@pytest.mark.parametrize("route", [1, 4, 8, 16, 1 << 20])
def test_majorana_routing_threshold_keeps_results(route):
    """Every |A| routing threshold of the Majorana orbit path (which groups the
    warp tier takes and which go straight to the team and block tiers) gives
    the reference's term sets bit for bit."""
    from fastfermion_gb300 import _native
    ctx = _native.context(0)
    before = ctx.get_option("morbit_route_big")
    ctx.set_option("morbit_route_big", route)
    try:
        for name in MAJORANA_ROUTE:
            fx = load(name)
            r = run_gpu(fx)
            keys, re, im = r.copy()
            assert r.n == int(fx["n_terms"]), name
            assert checksum(keys, re, im) == str(fx["checksum"]), name
    finally:
        ctx.set_option("morbit_route_big", before)


def _all_pauli_strings(nq):
    """Every non-identity Pauli string on nq qubits as (4, 4^nq - 1) key planes."""
    keys = []
    for code in range(1, 4 ** nq):
        x = z = 0
        for q in range(nq):
            p = (code >> (2 * q)) & 3  # 1 X, 2 Y, 3 Z
            if p in (1, 2):
                x |= 1 << q
            if p in (2, 3):
                z |= 1 << q
        keys.append((x, 0, z, 0))
    return np.array(keys, dtype=np.uint64).T.copy()


@pytest.mark.parametrize("batched", [True, False])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_exhaustive_three_qubit_pauli(seed, batched):
    """All 63 non-identity strings on 3 qubits with random complex coefficients
    through a random circuit of every gate type: GPU == oracle, bit for bit."""
    from fastfermion_gb300 import _native
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    keys = _all_pauli_strings(3)
    n = keys.shape[1]
    re, im = rng.normal(size=n), rng.normal(size=n) * (seed % 2)
    table = np.zeros(40, dtype=_native.PAULI_GATE)
    for i in range(40):
        kind = int(rng.integers(0, 6)) if rng.random() < 0.4 else 0
        table[i]["kind"] = kind
        if kind == 0:
            x = int(rng.integers(0, 8))
            z = int(rng.integers(0, 8))
            table[i]["x"] = (x, 0)
            table[i]["z"] = (z, 0)
            table[i]["theta"] = rng.uniform(-3, 3)
        else:
            a, b = rng.choice(3, 2, replace=False)
            table[i]["q0"], table[i]["q1"] = int(a), int(b)
    md = int(rng.integers(1, 4))
    p = dict(maxdegree=md, topk=0, mincoeff=1e-3 if seed == 2 else 0.0, max_xweight=-1, xtrunc_period=1,
             batched=int(batched), deterministic=0)
    g = _native.context(0).pauli_propagate(keys, re, im, table, dict(p))
    o = O.pauli_propagate(table, keys, re, im, maxdegree=md, mincoeff=p["mincoeff"], batched=batched)
    assert_same_terms(g.copy(), (o.keys, o.re, o.im))


@pytest.mark.parametrize("seed", [4, 5])
def test_exhaustive_four_mode_majorana(seed):
    """All 15 non-empty Majorana strings on 4 modes through random MROT
    circuits (odd and even degree): GPU == oracle, bit for bit."""
    from fastfermion_gb300 import _native
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    keys = np.zeros((4, 15), dtype=np.uint64)
    keys[0] = np.arange(1, 16, dtype=np.uint64)
    re, im = rng.normal(size=15), rng.normal(size=15)
    table = np.zeros(30, dtype=_native.MAJORANA_GATE)
    for i in range(30):
        a = int(rng.integers(1, 16))
        table[i]["alpha"] = (a, 0, 0, 0)
        table[i]["theta"] = rng.uniform(-2, 2)
        deg = bin(a).count("1")
        table[i]["r"] = 0 if deg % 4 in (0, 1) else 1
    pm = dict(has_maxdegree=1, maxdegree=3, mincoeff=1e-3, deterministic=0, pad=0)
    g = _native.context(0).majorana_propagate(keys, re, im, table, dict(pm))
    o = O.majorana_propagate(table, keys, re, im, maxdegree=3, mincoeff=1e-3)
    assert_same_terms(g.copy(), (o.keys, o.re, o.im))


def test_large_results_have_distinct_keys():
    """Size-independent invariants of large results: distinct keys (the merge
    left no duplicate), finite coefficients, above the threshold."""
    for name in ("cfg2_kicked_ising_0p5000", "hubbard_6x6_10steps", "cfg2w10_kicked_ising_0p3000"):
        fx = load(name)
        keys, re, im = run_gpu(fx).copy()
        k = np.ascontiguousarray(keys.T).view(np.dtype((np.void, 32))).ravel()
        assert np.unique(k).size == k.size, name
        assert np.all(np.isfinite(re)) and np.all(np.isfinite(im)), name
        tau = float(fx["mincoeff"])
        if tau > 0:
            assert np.all(np.hypot(re, im) > tau), name


ENGINE_PATHS = [("persistent", 0), ("orbit", 0), ("group_d", 2), ("group_d", 4), ("morbit", 0),
                ("persist_blocks_per_sm", 1)]
PATH_FIXTURES = ["ref_tfim", "ref_tfim_unbatched", "ref_mixed_clifford", "cfg1_chain", "rand_pauli_00",
                 "rand_pauli_05", "ref_heisenberg", "ref_majorana_1", "rand_majorana_03"]


@pytest.mark.gpu
@pytest.mark.parametrize("option,value", ENGINE_PATHS, ids=[f"{o}={v}" for o, v in ENGINE_PATHS])
def test_engine_paths_match_reference(option, value):
    """Every alternative engine path (one launch per op, no orbit path, fused
    rotation groups, the Majorana per-gate kernel, one persistent block per SM)
    gives the reference's term sets."""
    from fastfermion_gb300 import _native
    ctx = _native.context(0)
    old = ctx.get_option(option)
    try:
        ctx.set_option(option, value)
        for name in PATH_FIXTURES:
            fx = load(name)
            if str(fx["kind"]) == "pauli" and int(fx["topk"]) > 0:
                continue
            keys, re, im = run_gpu(fx).copy()
            if "res_keys" in fx:
                assert_same_terms((keys, re, im), (fx["res_keys"], fx["res_re"], fx["res_im"])), name
            else:
                assert checksum(keys, re, im) == str(fx["checksum"]), name
    finally:
        ctx.set_option(option, old)
