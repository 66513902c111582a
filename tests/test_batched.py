"""Batched instances and the adjoint (ffg_pauli_propagate_batched, ffg_batch_adjoint).

Parity: every instance of a batched propagation must give the term set the
reference gives for that instance alone, bit for bit (golden fixtures made by
the reference: tests/golden/hea_50q_inst*.npz), and the oracle's per-instance
runs elsewhere.  Gradients: the adjoint must equal the reference's
parameter-shift derivatives where those are exact (no coefficient threshold:
the truncated map is then a first-degree trigonometric polynomial in each
angle; fixtures hea_shift_*.npz), central finite differences on the GPU
(h = 1e-5), and the linearity identity sum_t c_t dF/dc_t = F.
"""
import math

import numpy as np
import pytest

import fastfermion_gb300 as ff
from fastfermion_gb300 import _native
from fastfermion_gb300 import workloads as W
from golden_io import assert_same_terms, checksum, load
from oracle import oracle as O

# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------


def hea_table(n, layers):
    return ff.encode_pauli_circuit(ff.build_circuit(W.hea_circuit(n, layers)))


def with_angles(table, th):
    t = table.copy()
    t["theta"][t["kind"] == 0] = th
    return t


def concat(obs):
    keys = np.concatenate([o[0] for o in obs], axis=1)
    re = np.concatenate([o[1] for o in obs])
    off = np.cumsum([0] + [o[1].size for o in obs]).astype(np.int64)
    return keys, re, off


def params(maxdegree, mincoeff, batched=True):
    return dict(maxdegree=maxdegree, topk=0, mincoeff=mincoeff, max_xweight=-1, xtrunc_period=1,
                batched=int(batched), deterministic=0)


def run_batched(table, obs, thetas, maxdegree, mincoeff, batched=True, every=1):
    keys, re, off = concat(obs)
    ctx = _native.context(0)
    return ctx.pauli_propagate_batched(keys, re, off, table, thetas, params(maxdegree, mincoeff, batched), every)


# ---------------------------------------------------------------------------
# CPU: workload generator and fixtures
# ---------------------------------------------------------------------------


def test_hea_workload_shapes():
    th, obs = W.hea_instances(256)
    assert th.shape == (256, 400)
    assert np.all(np.abs(th) <= math.pi)
    counts = [o[1].size for o in obs]
    assert min(counts) >= 1 and max(counts) <= 64 and len(set(counts)) > 20
    for k, _ in obs[:20]:
        pairs = {(int(k[0, t]), int(k[2, t])) for t in range(k.shape[1])}
        assert len(pairs) == k.shape[1]  # distinct strings within an instance
        w = [bin(int(k[0, t]) | int(k[2, t])).count("1") for t in range(k.shape[1])]
        assert 1 <= min(w) and max(w) <= 4


@pytest.mark.parametrize("name", ["hea_50q_inst0", "hea_50q_inst1"])
def test_oracle_matches_reference_hea_instance(name):
    fx = load(name)
    o = O.pauli_propagate(fx["gates"], fx["obs_keys"], fx["obs_re"], fx["obs_im"], maxdegree=6, mincoeff=1e-7)
    assert len(o) == int(fx["n_terms"])
    assert checksum(o.keys, o.re, o.im) == str(fx["checksum"])


@pytest.mark.parametrize("name", ["hea_shift_10q", "hea_shift_10q_unbatched", "hea_shift_70q"])
def test_oracle_pins_parameter_shift_fixture(name):
    fx = load(name)
    n, layers = int(fx["n"]), int(fx["layers"])
    table = hea_table(n, layers)
    off = fx["offsets"]
    rng = np.random.default_rng(1)
    for i in range(off.size - 1):
        k = fx["obs_keys"][:, off[i]:off[i + 1]]
        re = fx["obs_re"][off[i]:off[i + 1]]

        def ev(th):
            r = O.pauli_propagate(with_angles(table, th), k, re, np.zeros(re.size), maxdegree=int(fx["maxdegree"]),
                                  batched=bool(fx["batched"]))
            return r.overlapwithzero().real
        th = fx["thetas"][i]
        assert abs(ev(th) - fx["expect"][i]) < 1e-12
        for r in rng.choice(th.size, 3, replace=False):
            tp, tm = th.copy(), th.copy()
            tp[r] += math.pi / 2
            tm[r] -= math.pi / 2
            assert abs(0.5 * (ev(tp) - ev(tm)) - fx["shift_grad"][i, r]) < 1e-12


# ---------------------------------------------------------------------------
# GPU: forward parity
# ---------------------------------------------------------------------------


def small_cases():
    # (n, layers, ninst, seed, maxdegree, mincoeff, batched)
    return [(12, 3, 5, 3, 4, 1e-5, True), (12, 3, 4, 4, 5, 0.0, False), (20, 4, 9, 5, 6, 1e-7, True),
            (70, 2, 3, 6, 4, 1e-6, True)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", small_cases())
def test_batched_instances_match_oracle(case):
    n, layers, ninst, seed, md, tau, batched = case
    th, obs = W.hea_instances(ninst, n=n, layers=layers, seed=seed, max_terms=12)
    table = hea_table(n, layers)
    expect, h = run_batched(table, obs, th, md, tau, batched, every=0)
    keys, re, inst = h.copy()
    for i in range(ninst):
        o = O.pauli_propagate(with_angles(table, th[i]), obs[i][0], obs[i][1], np.zeros(obs[i][1].size),
                              maxdegree=md, mincoeff=tau, batched=batched)
        sel = inst == i
        assert_same_terms((keys[:, sel], re[sel], np.zeros(int(sel.sum()))), (o.keys, o.re, o.im))
        assert abs(expect[i] - o.overlapwithzero().real) < 1e-12


@pytest.mark.gpu
def test_full_batched_ansatz_matches_reference_instances():
    """256 instances x 50 qubits, 8 layers, W=6, tau=1e-7 in one batched run;
    instances 0 and 1 against the reference's own runs of them."""
    th, obs = W.hea_instances(256)
    expect, h = run_batched(hea_table(50, 8), obs, th, 6, 1e-7, every=0)
    keys, re, inst = h.copy()
    for i in (0, 1):
        fx = load(f"hea_50q_inst{i}")
        sel = inst == i
        assert int(sel.sum()) == int(fx["n_terms"])
        assert checksum(keys[:, sel], re[sel], np.zeros(int(sel.sum()))) == str(fx["checksum"])
        assert abs(expect[i] - float(fx["overlap"][0])) < 1e-12
    # an instance the fixtures do not cover, against the oracle
    i = 200
    o = O.pauli_propagate(with_angles(hea_table(50, 8), th[i]), obs[i][0], obs[i][1], np.zeros(obs[i][1].size),
                          maxdegree=6, mincoeff=1e-7)
    sel = inst == i
    assert_same_terms((keys[:, sel], re[sel], np.zeros(int(sel.sum()))), (o.keys, o.re, o.im))


@pytest.mark.gpu
def test_batched_rejects_unsupported():
    th, obs = W.hea_instances(2, n=6, layers=1, seed=1, max_terms=3)
    keys, re, off = concat(obs)
    ctx = _native.context(0)
    table = hea_table(6, 1)
    for over in (dict(topk=5), dict(max_xweight=2)):
        p = params(4, 0.0)
        p.update(over)
        with pytest.raises(RuntimeError):
            ctx.pauli_propagate_batched(keys, re, off, table, th, p, 1)
    with pytest.raises(RuntimeError):
        ctx.pauli_propagate_batched(keys, re, np.array([0, 1], dtype=np.int64), table, th[:1], params(4, 0.0), 1)


# ---------------------------------------------------------------------------
# GPU: gradients
# ---------------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hea_shift_10q", "hea_shift_10q_unbatched", "hea_shift_70q"])
def test_adjoint_matches_reference_parameter_shift(name):
    fx = load(name)
    n, layers = int(fx["n"]), int(fx["layers"])
    off = fx["offsets"]
    obs = [(fx["obs_keys"][:, off[i]:off[i + 1]], fx["obs_re"][off[i]:off[i + 1]]) for i in range(off.size - 1)]
    expect, h = run_batched(hea_table(n, layers), obs, fx["thetas"], int(fx["maxdegree"]), 0.0,
                            bool(fx["batched"]))
    np.testing.assert_allclose(expect, fx["expect"], rtol=0, atol=1e-12)
    g, _ = h.adjoint(np.ones(off.size - 1))
    np.testing.assert_allclose(g, fx["shift_grad"], rtol=0, atol=1e-11)


@pytest.mark.gpu
def test_adjoint_matches_central_differences():
    n, layers, ninst = 16, 4, 3
    th, obs = W.hea_instances(ninst, n=n, layers=layers, seed=11, max_terms=8)
    table = hea_table(n, layers)
    _, h = run_batched(table, obs, th, 5, 0.0)
    w = np.array([1.0, -0.5, 2.0])
    g, _ = h.adjoint(w)
    hstep = 1e-5
    rng = np.random.default_rng(2)
    for i in range(ninst):
        for r in rng.choice(th.shape[1], 6, replace=False):
            tp, tm = th.copy(), th.copy()
            tp[i, r] += hstep
            tm[i, r] -= hstep
            fp, _ = run_batched(table, obs, tp, 5, 0.0, every=0)
            fm, _ = run_batched(table, obs, tm, 5, 0.0, every=0)
            fd = (w @ fp - w @ fm) / (2 * hstep)
            assert abs(fd - g[i, r]) < 1e-7 * max(1.0, abs(fd)), (i, r, fd, g[i, r])


@pytest.mark.gpu
def test_adjoint_full_size_linearity_and_checkpoints():
    """The full batched ansatz: sum_t c_t dF/dc_t = F per instance (the map is
    linear in the input coefficients for a fixed truncation pattern), and
    recomputing segments from sparser checkpoints gives the same gradient."""
    th, obs = W.hea_instances(256)
    table = hea_table(50, 8)
    keys, re, off = concat(obs)
    expect, h = run_batched(table, obs, th, 6, 1e-7, every=1)
    w = np.random.default_rng(3).normal(size=256)
    g1, gc = h.adjoint(w, with_coef=True)
    for i in range(256):
        lhs = float(gc[off[i]:off[i + 1]] @ re[off[i]:off[i + 1]])
        assert abs(lhs - w[i] * expect[i]) < 1e-10 * max(1.0, abs(w[i] * expect[i])), i
    assert np.all(np.isfinite(g1)) and np.any(g1 != 0)
    _, h3 = run_batched(table, obs, th, 6, 1e-7, every=5)
    g3, _ = h3.adjoint(w)
    np.testing.assert_allclose(g3, g1, rtol=1e-9, atol=1e-12)


@pytest.mark.gpu
def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    from fastfermion_gb300 import batched as B
    n, layers = 10, 2
    th, obs = W.hea_instances(4, n=n, layers=layers, seed=5, max_terms=5)
    circ = ff.build_circuit(W.hea_circuit(n, layers))
    polys = [ff.PauliPolynomial.from_arrays(k, r, np.zeros(r.size)) for k, r in obs]
    t = torch.tensor(th, dtype=torch.float64, requires_grad=True)
    e = B.expectation(circ, polys, t, maxdegree=4)
    w = torch.tensor([0.3, -1.0, 2.0, 0.5], dtype=torch.float64)
    (e * w).sum().backward()
    r = B.propagate_batched(circ, polys, th, maxdegree=4)
    # per-instance sums run in no fixed order: equal up to rounding
    np.testing.assert_allclose(e.detach().numpy(), r.expect, rtol=0, atol=1e-14)
    np.testing.assert_allclose(t.grad.numpy(), r.gradient(w.numpy()), rtol=1e-12, atol=1e-14)


@pytest.mark.gpu
def test_theta_sweep_as_instances_matches_reference_fixtures():
    """The headline theta_h sweep as instances of one batched propagation
    (per-instance angles, no checkpoints: orbit windows): every instance's
    term set equals the reference's own result for that theta_h."""
    from golden_io import assert_same_terms, load
    from fastfermion_gb300 import _native
    names = ["cfg2_kicked_ising_0p1000", "cfg2_kicked_ising_0p5000", "cfg2_kicked_ising_0p9000"]
    fxs = [load(n) for n in names]
    tabs = [fx["gates"] for fx in fxs]
    k = np.concatenate([fx["obs_keys"] for fx in fxs], axis=1)
    re = np.concatenate([fx["obs_re"] for fx in fxs])
    off = np.array([0, 1, 2, 3], dtype=np.int64)
    th = np.stack([t["theta"][t["kind"] == 0] for t in tabs])
    p = dict(maxdegree=int(fxs[0]["maxdegree"]), topk=0, mincoeff=float(fxs[0]["mincoeff"]), max_xweight=-1,
             xtrunc_period=1, batched=1, deterministic=0)
    ctx = _native.context(0)
    expect, h = ctx.pauli_propagate_batched(k, re, off, tabs[0], th, p, 0)
    keys, cre, inst = h.copy()
    for i, fx in enumerate(fxs):
        sel = inst == i
        assert_same_terms((keys[:, sel], cre[sel], np.zeros(int(sel.sum()))),
                          (fx["res_keys"], fx["res_re"], fx["res_im"]))
        assert abs(expect[i] - float(fx["overlap"][0])) <= 1e-12


@pytest.mark.gpu
def test_adjoint_full_size_matches_central_differences():
    """Config 4 at full size (256 instances x 50 qubits x 8 layers, W=6,
    tau=1e-7): the adjoint gradient of sum_i <O_i> against central differences
    (h=1e-5) at 20 sampled (instance, angle) pairs, each perturbed instance
    propagated alone.  The threshold makes the map piecewise; a sample whose
    +-h propagations change the truncation pattern shows up as a jump and is
    reported, and at least 18 of the 20 must agree to 1e-6."""
    th, obs = W.hea_instances(256)
    table = hea_table(50, 8)
    _, h = run_batched(table, obs, th, 6, 1e-7, every=1)
    g, _ = h.adjoint(np.ones(256))
    rng = np.random.default_rng(17)
    hstep, good, rows = 1e-5, 0, []
    for _ in range(20):
        i, r = int(rng.integers(256)), int(rng.integers(th.shape[1]))
        tp, tm = th[i:i + 1].copy(), th[i:i + 1].copy()
        tp[0, r] += hstep
        tm[0, r] -= hstep
        fp, _ = run_batched(table, [obs[i]], tp, 6, 1e-7, every=0)
        fm, _ = run_batched(table, [obs[i]], tm, 6, 1e-7, every=0)
        fd = (fp[0] - fm[0]) / (2 * hstep)
        ok = abs(fd - g[i, r]) <= 1e-6 * max(1.0, abs(fd))
        good += ok
        rows.append((i, r, fd, g[i, r], ok))
    print("\n".join(f"inst {i:3d} angle {r:3d}: fd {fd:+.10e} adjoint {a:+.10e} {'' if ok else 'JUMP'}"
                    for i, r, fd, a, ok in rows))
    assert good >= 18, rows
