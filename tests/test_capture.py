"""Dropped-partner capture and per-instance active rotations: the data path of the
learned correction.

The GPU records every partner that the degree filter drops (key, value, gate)
while it propagates; those partners are then propagated at a higher cutoff,
each from the gate that created it, as instances of one batched propagation
whose rotations before that gate are inactive.  CPU cases pin the oracle's
restatement of the masked propagation; GPU cases compare the C ABI with the
oracle bit for bit.
"""
import numpy as np
import pytest

import fastfermion_gb300 as ff
from fastfermion_gb300 import _native
from golden_io import assert_same_terms
from oracle import oracle as O


def _z(site):
    keys = np.zeros((4, 1), dtype=np.uint64)
    keys[2 + site // 64, 0] = np.uint64(1) << np.uint64(site % 64)
    return keys, np.ones(1), np.zeros(1)


def _ki(theta, lx=3, ly=3, steps=2):
    return ff.encode_pauli_circuit(ff.build_circuit(ff.workloads.kicked_ising_circuit(theta, lx, ly, steps)))


def _random_circuit(seed, nq=8, ngates=40):
    rng = np.random.default_rng(seed)
    circ = []
    for _ in range(ngates):
        w = int(rng.integers(1, 3))
        qs = sorted(int(q) for q in rng.choice(nq, w, replace=False))
        circ.append(ff.ROT("".join("XYZ"[rng.integers(3)] for _ in qs), qs, float(rng.uniform(-1.5, 1.5))))
    return ff.encode_pauli_circuit(circ)


def _rot_index(tab):
    """circuit gate index -> rotation index (-1 for Clifford gates)"""
    r = np.cumsum(tab["kind"] == O.ROT) - 1
    return np.where(tab["kind"] == O.ROT, r, -1)


def _mask_before(tab, gate):
    """active rotations of a partner created by circuit gate `gate`: the
    rotations still to be applied to it, gates [0, gate)."""
    nrot = int(np.count_nonzero(tab["kind"] == O.ROT))
    words = max(1, (nrot + 63) // 64)
    m = np.zeros(words, dtype=np.uint64)
    nr = int(np.count_nonzero(tab["kind"][:gate] == O.ROT))
    for r in range(nr):
        m[r // 64] |= np.uint64(1) << np.uint64(r % 64)
    return m


def _sorted_drops(d):
    """oracle Dropped -> (keys, re, im, gate) sorted by gate, then key words"""
    order = np.lexsort((d.keys[3], d.keys[2], d.keys[1], d.keys[0], d.gate))
    return d.keys[:, order], d.re[order], d.im[order], d.gate[order]


# --------------------------------------------------------------------------- CPU


def test_oracle_mask_all_active_is_plain_propagation():
    tab = _random_circuit(1)
    k, re, im = _z(3)
    nrot = int(np.count_nonzero(tab["kind"] == O.ROT))
    full = np.array([(1 << 64) - 1] * max(1, (nrot + 63) // 64), dtype=np.uint64)
    a = O.pauli_propagate(tab, k, re, im, maxdegree=4, mincoeff=1e-3)
    b = O.pauli_propagate(tab, k, re, im, maxdegree=4, mincoeff=1e-3, active=full)
    assert_same_terms((a.keys, a.re, a.im), (b.keys, b.re, b.im))


def test_oracle_mask_skips_rotations():
    """Without truncation the batching does not matter: skipping rotations
    equals deleting them from the circuit, bit for bit."""
    tab = _random_circuit(2)
    k, re, im = _z(5)
    rng = np.random.default_rng(7)
    keep = rng.random(tab.size) < 0.6
    nrot = int(np.count_nonzero(tab["kind"] == O.ROT))
    m = np.zeros(max(1, (nrot + 63) // 64), dtype=np.uint64)
    for r, g in enumerate(np.nonzero(tab["kind"] == O.ROT)[0]):
        if keep[g]:
            m[r // 64] |= np.uint64(1) << np.uint64(r % 64)
    a = O.pauli_propagate(tab[keep], k, re, im, maxdegree=5)
    b = O.pauli_propagate(tab, k, re, im, maxdegree=5, active=m)
    assert_same_terms((a.keys, a.re, a.im), (b.keys, b.re, b.im))


def test_oracle_masked_labels_account_for_the_truncation_error():
    """<O>_W' = <O>_W + sum over dropped partners of their value propagated at
    W' from the gate that created them, here with the masked propagation."""
    tab = _ki(0.7)
    k, re, im = _z(4)
    low, d = O.pauli_propagate_capture(tab, k, re, im, capdeg=5, maxdegree=2)
    high = O.pauli_propagate(tab, k, re, im, maxdegree=5)
    lab = sum(O.pauli_propagate(tab, d.keys[:, i:i + 1], d.re[i:i + 1], d.im[i:i + 1], maxdegree=5,
                                active=_mask_before(tab, int(d.gate[i]))).overlapwithzero()
              for i in range(len(d)))
    assert abs(high.overlapwithzero() - low.overlapwithzero()) > 1e-3
    assert abs(high.overlapwithzero() - (low.overlapwithzero() + lab)) <= 1e-12


# --------------------------------------------------------------------------- GPU


def _gpu_params(maxdegree, mincoeff=0.0):
    return dict(maxdegree=maxdegree, topk=0, mincoeff=mincoeff, max_xweight=-1, xtrunc_period=1, batched=1,
                deterministic=0)


CAPTURE_CASES = [
    ("kicked_ising_3x3", lambda: _ki(0.7), 4, 2, 5, 0.0),
    ("chain_8", lambda: ff.encode_pauli_circuit(ff.build_circuit(ff.workloads.chain_circuit(8, 3))), 3, 2, 4, 0.0),
    ("random_8q", lambda: _random_circuit(3), 2, 3, 6, 1e-4),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,site,w,w2,tau", CAPTURE_CASES, ids=[c[0] for c in CAPTURE_CASES])
def test_gpu_capture_matches_oracle(name, make, site, w, w2, tau):
    tab = make()
    k, re, im = _z(site)
    ctx = _native.context(0)
    res, drops = ctx.pauli_propagate_capture(k, re, im, tab, _gpu_params(w, tau), capdeg=w2)
    o, d = O.pauli_propagate_capture(tab, k, re, im, capdeg=w2, maxdegree=w, mincoeff=tau)
    assert_same_terms(res.copy(), (o.keys, o.re, o.im))
    gk, gre, gim, gg = drops.copy()
    ok, ore, oim, og = _sorted_drops(d)
    assert len(d) > 0 and gk.shape == ok.shape
    assert np.array_equal(gg, og) and np.array_equal(gk, ok)
    assert np.array_equal(gre, ore) and np.array_equal(gim, oim)


@pytest.mark.gpu
def test_gpu_capture_kicked_ising_10x10_above_threshold():
    """W=6, tau=1e-6 on the 10x10 kicked-Ising circuit: the partners above tau
    that W=6 drops (degree 7..10), against the oracle's record."""
    tab = ff.encode_pauli_circuit(ff.build_circuit(ff.workloads.kicked_ising_circuit(0.3)))
    k, re, im = _z(55)
    ctx = _native.context(0)
    res, drops = ctx.pauli_propagate_capture(k, re, im, tab, _gpu_params(6, 1e-6), capdeg=10, min_abs=1e-6)
    o, d = O.pauli_propagate_capture(tab, k, re, im, capdeg=10, maxdegree=6, mincoeff=1e-6)
    assert_same_terms(res.copy(), (o.keys, o.re, o.im))
    sel = np.abs(d.re) > 1e-6
    ok, ore, oim, og = _sorted_drops(type(d)(d.keys[:, sel], d.re[sel], d.im[sel], d.gate[sel]))
    gk, gre, gim, gg = drops.copy()
    assert gk.shape[1] == ok.shape[1] > 100
    assert np.array_equal(gg, og) and np.array_equal(gk, ok) and np.array_equal(gre, ore)


@pytest.mark.gpu
def test_gpu_capture_survives_regrowth():
    """A tiny store with no headroom makes batches overflow their output store,
    so they run again after the store grows: the record keeps each
    (key, gate) once and the result is unchanged."""
    tab = ff.encode_pauli_circuit(ff.build_circuit(ff.workloads.chain_circuit()))  # 2646 terms at the end
    k, re, im = _z(7)
    ctx = _native.context(0)
    base_r, base_d = ctx.pauli_propagate_capture(k, re, im, tab, _gpu_params(6, 1e-8), capdeg=8)
    old = {n: ctx.get_option(n) for n in ("min_capacity", "store_headroom")}
    try:
        ctx.set_option("min_capacity", 64)
        ctx.set_option("store_headroom", 1)
        r, d = ctx.pauli_propagate_capture(k, re, im, tab, _gpu_params(6, 1e-8), capdeg=8)
        assert ctx.profile()["regrows"] > 0
    finally:
        for n, v in old.items():
            ctx.set_option(n, v)
    assert_same_terms(r.copy(), base_r.copy())
    a, b = d.copy(), base_d.copy()
    assert len(d) == len(base_d) > 0
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_gpu_instances_with_active_rotations_match_oracle(seed):
    """Instances with their own active rotations (random masks) against the
    oracle's masked propagation of each instance alone, with a threshold."""
    rng = np.random.default_rng(100 + seed)
    tab = _random_circuit(10 + seed, nq=10, ngates=60)
    nrot = int(np.count_nonzero(tab["kind"] == O.ROT))
    words = max(1, (nrot + 63) // 64)
    ninst = 5
    keys, res, off, masks = [], [], [0], np.zeros((ninst, words), dtype=np.uint64)
    for i in range(ninst):
        m = int(rng.integers(1, 4))
        kk = np.zeros((4, m), dtype=np.uint64)
        kk[2] = rng.choice(np.arange(1, 1 << 10), m, replace=False).astype(np.uint64)
        keys.append(kk)
        res.append(rng.normal(size=m))
        off.append(off[-1] + m)
        for r in range(nrot):
            if rng.random() < 0.7:
                masks[i, r // 64] |= np.uint64(1) << np.uint64(r % 64)
    K, R = np.concatenate(keys, axis=1), np.concatenate(res)
    ctx = _native.context(0)
    expect, b = ctx.pauli_propagate_instances(K, R, np.array(off), tab, None, _gpu_params(5, 1e-5), masks)
    gk, gre, ginst = b.copy()
    for i in range(ninst):
        o = O.pauli_propagate(tab, keys[i], res[i], None, maxdegree=5, mincoeff=1e-5, active=masks[i])
        sel = ginst == i
        assert_same_terms((gk[:, sel], gre[sel], np.zeros(int(sel.sum()))), (o.keys, o.re, o.im))
        assert abs(expect[i] - o.overlapwithzero().real) <= 1e-12


@pytest.mark.gpu
def test_gpu_labels_account_for_the_truncation_error():
    """End to end on the GPU: the W=2 value plus the labels of its dropped
    partners (each propagated at W'=5 from its gate, all in one batched launch)
    equals the W'=5 value (no threshold, so exactly up to rounding)."""
    tab = _ki(0.7)
    k, re, im = _z(4)
    ctx = _native.context(0)
    low, drops = ctx.pauli_propagate_capture(k, re, im, tab, _gpu_params(2), capdeg=5)
    high = ctx.pauli_propagate(k, re, im, tab, _gpu_params(5))
    dk, dre, _, dg = drops.copy()
    masks = np.stack([_mask_before(tab, int(g)) for g in dg])
    lab, _ = ctx.pauli_propagate_instances(dk, dre, np.arange(dre.size + 1), tab, None, _gpu_params(5), masks)
    f_low, f_high = low.overlapwithzero().real, high.overlapwithzero().real
    assert abs(f_high - f_low) > 1e-3
    assert abs(f_high - (f_low + lab.sum())) <= 1e-12


@pytest.mark.gpu
def test_gpu_barrier_timeout_reports_an_error_and_the_context_recovers():
    """Failure detection without a fault: with a 1000-cycle limit the blocks of
    the persistent kernel give up at a grid barrier; the call returns
    FFG_ERR_STATE instead of hanging, and the same context then propagates
    correctly with the default limit."""
    tab = ff.encode_pauli_circuit(ff.build_circuit(ff.workloads.chain_circuit()))
    k, re, im = _z(7)
    ctx = _native.context(0)
    p = dict(_gpu_params(6, 1e-8), batched=0)  # unbatched: one persistent launch runs the rotations
    old = ctx.get_option("barrier_limit_kcycles")
    try:
        ctx.set_option("barrier_limit_kcycles", 1)
        with pytest.raises(_native.FFGError, match="grid barrier timed out"):
            ctx.pauli_propagate(k, re, im, tab, p)
    finally:
        ctx.set_option("barrier_limit_kcycles", old)
    r = ctx.pauli_propagate(k, re, im, tab, p)
    o = O.pauli_propagate(tab, k, re, im, maxdegree=6, mincoeff=1e-8, batched=False)
    assert_same_terms(r.copy(), (o.keys, o.re, o.im))


@pytest.mark.gpu
def test_gpu_group_regions_grow_and_groups_run_again():
    """Groups too large for shared memory start in 64-member global-memory
    regions (option group_region_cap), outgrow them and run again in regions
    four times larger; the term set is unchanged (10x10 kicked Ising, W=10,
    theta_h=0.3, whose largest groups exceed the 4096-member shared-memory
    tier, against the reference's own result)."""
    from golden_io import load
    fx = load("cfg2w10_kicked_ising_0p3000")
    ctx = _native.context(0)
    p = _gpu_params(int(fx["maxdegree"]), float(fx["mincoeff"]))
    old = ctx.get_option("group_region_cap")
    try:
        ctx.set_option("group_region_cap", 64)
        r = ctx.pauli_propagate(fx["obs_keys"], fx["obs_re"], fx["obs_im"], fx["gates"], p)
        prof = ctx.profile()
    finally:
        ctx.set_option("group_region_cap", old)
    assert prof["orbit_max_group"] > 4096, prof["orbit_max_group"]  # some group used the global regions
    assert_same_terms(r.copy(), (fx["res_keys"], fx["res_re"], fx["res_im"]))
