"""The learned correction's network (tcgen05 BF16 GEMMs, FP32 accumulation) and
the features of dropped partners, against the CPU restatement in
oracle/surrogate_ref.py.

Tolerances: the GPU and the restatement round the same GEMM operands to BF16
and differ in the order of FP32 sums and in the GELU's tanh, which the GPU
takes from its hardware approximation (relative error about 2^-11) and the
restatement computes exactly.  Either can move an activation across a BF16
rounding boundary (2^-8 relative).  Outputs and gradients are therefore
compared with a norm-relative tolerance of 1e-2, the loss with 5e-3; the GEMM
self-test, whose inputs are exact BF16 values, with 1e-5.
"""
import numpy as np
import pytest

from oracle import surrogate_ref as R


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


# --------------------------------------------------------------------------- CPU


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = np.concatenate([rng.normal(size=4000).astype(np.float32) * 10 ** rng.uniform(-8, 8, 4000).astype(np.float32),
                        np.array([0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -(1.0 + 2 ** -8)], np.float32)])
    want = torch.from_numpy(a).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(R.bf16_bits(a), want)


def test_restated_backward_matches_finite_differences():
    """The float64 network (no BF16 rounding): analytic gradient against central
    differences of the loss, on a sample of parameters of every block."""
    rng = np.random.default_rng(1)
    p = R.init_params(3).astype(np.float64)
    p[R.HID * R.IN:R.HID * R.IN + R.HID] = rng.normal(scale=0.1, size=R.HID)  # b1 != 0
    x = rng.normal(size=(40, R.IN))
    t = rng.normal(size=40)
    w = rng.uniform(0.1, 1.0, size=40)
    g, _ = R.gradient(p, x, t, w, bf16_ops=False)
    h = 1e-6
    idx = np.concatenate([rng.choice(R.NPARAMS, 60, replace=False), [R.NPARAMS - 1, R.NPARAMS - 2]])
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (R.gradient(pp, x, t, w, bf16_ops=False)[1] - R.gradient(pm, x, t, w, bf16_ops=False)[1]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


# --------------------------------------------------------------------------- GPU


@pytest.fixture(scope="module")
def mlp():
    pytest.importorskip("torch")
    from fastfermion_gb300 import _native
    return _native.MLP(_native.context(0))


def _dev(torch, a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.cuda() if dtype is None else t.to(dtype).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("n,k", [(128, 32), (128, 128), (32, 128), (16, 16), (144, 64), (256, 128), (48, 128)])
def test_tensor_core_gemm_selftest(mlp, n, k):
    rng = np.random.default_rng(n * 1000 + k)
    a = R.bf16_bits(rng.normal(size=(128, k)).astype(np.float32))
    b = R.bf16_bits(rng.normal(size=(n, k)).astype(np.float32))
    d = mlp.selftest_gemm(a, b)
    want = R.from_bits(a).astype(np.float64) @ R.from_bits(b).astype(np.float64).T
    assert _rel(d, want) <= 1e-5
    assert np.max(np.abs(d - want)) <= 1e-4 * np.max(np.abs(want))


def _problem(seed, n):
    rng = np.random.default_rng(seed)
    p = R.init_params(seed)
    d = R.unpack(p)
    d["b1"] = rng.normal(scale=0.1, size=R.HID)
    d["b2"] = rng.normal(scale=0.1, size=R.HID)
    d["b3"] = rng.normal(scale=0.1, size=R.HID)
    d["b4"] = 0.05
    p = R.pack(d).astype(np.float32)
    xb = R.bf16_bits(rng.normal(size=(n, R.IN)).astype(np.float32))
    t = rng.normal(size=n).astype(np.float32)
    w = (rng.uniform(0.1, 1.0, size=n) / n).astype(np.float32)
    return p, xb, t, w


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 127, 128, 300, 5000, 150001])
def test_forward_matches_restatement(mlp, n):
    import torch
    p, xb, _, _ = _problem(n, n)
    mlp.set_params(p)
    x = _dev(torch, xb.view(np.int16))
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    mlp.forward(x, n, y)
    want = R.forward(p, R.from_bits(xb))
    assert _rel(y.cpu().numpy(), want) <= 1e-2
    assert np.allclose(mlp.get_params(), p)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [128, 1000, 40000])
def test_gradient_matches_restatement(mlp, n):
    import torch
    p, xb, t, w = _problem(7 + n, n)
    mlp.set_params(p)
    x = _dev(torch, xb.view(np.int16))
    g, loss = mlp.gradient(x, _dev(torch, t), _dev(torch, w), n)
    want, wloss = R.gradient(p, R.from_bits(xb), t.astype(np.float64), w.astype(np.float64))
    assert abs(loss - wloss) <= 5e-3 * abs(wloss)
    o = 0
    for name, size in (("W1", 4096), ("b1", 128), ("W2", 16384), ("b2", 128), ("W3", 16384), ("b3", 128),
                       ("w4", 128), ("b4", 1)):
        assert _rel(g[o:o + size], want[o:o + size]) <= 1e-2, name
        o += size


@pytest.mark.gpu
def test_adam_step_matches_restatement_and_training_reduces_the_loss(mlp):
    import torch
    n = 2048
    p, xb, t, w = _problem(11, n)
    t = (R.forward(p, R.from_bits(xb)) * 0.5 + 0.1).astype(np.float32)  # a reachable target
    mlp.set_params(p)
    x, tt, ww = _dev(torch, xb.view(np.int16)), _dev(torch, t), _dev(torch, w)
    g, l0 = mlp.gradient(x, tt, ww, n)
    mlp.adam_step(x, tt, ww, n, lr=1e-3)
    p1 = mlp.get_params()
    want, _, _ = R.adam(p.astype(np.float64), g.astype(np.float64), 0.0, 0.0, 1, 1e-3)
    assert np.max(np.abs(p1 - want)) <= 1e-6 + 1e-5 * np.max(np.abs(want))
    for _ in range(200):
        mlp.adam_step(x, tt, ww, n, lr=1e-3)
    _, l1 = mlp.gradient(x, tt, ww, n)
    assert l1 < 0.2 * l0, (l0, l1)


@pytest.mark.gpu
def test_drop_features_match_restatement():
    import torch

    import fastfermion_gb300 as ff
    from fastfermion_gb300 import _native, surrogate as S
    tab = ff.encode_pauli_circuit(ff.build_circuit(ff.workloads.kicked_ising_circuit(0.3)))
    keys = np.zeros((4, 1), dtype=np.uint64)
    keys[2, 0] = np.uint64(1) << np.uint64(55)
    ctx = _native.context(0)
    _, drops = ctx.pauli_propagate_capture(keys, np.ones(1), np.zeros(1), tab,
                                           dict(maxdegree=6, topk=0, mincoeff=1e-6, max_xweight=-1, xtrunc_period=1,
                                                batched=1, deterministic=0), capdeg=10, min_abs=1e-6)
    dk, dre, _, dg = drops.copy()
    n = dre.size
    bog, nb = S.batch_of_gate(tab)
    coords = S.lattice_coords(10, 10)
    feat = torch.zeros((n, 32), dtype=torch.float32, device="cuda")
    x = torch.zeros((n, 32), dtype=torch.int16, device="cuda")
    kd = _dev(torch, dk.view(np.int64))
    _native.drop_features(ctx, kd, n, _dev(torch, dre), _dev(torch, dg), n, tab, bog, nb, coords, 55, 6, feat, x)
    want = R.features(dk, dre, dg, tab, bog, nb, coords, 55, 6)
    got = feat.cpu().numpy()
    err = np.abs(got - want) / np.maximum(np.abs(want), 1.0)
    assert np.max(err) <= 1e-6, (np.argmax(np.max(err, axis=0)), np.max(err, axis=0))
    assert np.array_equal(x.cpu().numpy().view(np.uint16), R.bf16_bits(got))
    # standardised network input: bf16((f - shift) * scale) in FP32
    shift = want.mean(0).astype(np.float32)
    scale = (1.0 / (want.std(0) + 1e-3)).astype(np.float32)
    _native.drop_features(ctx, kd, n, _dev(torch, dre), _dev(torch, dg), n, tab, bog, nb, coords, 55, 6, None, x,
                          shift=shift, scale=scale)
    std = ((got - shift) * scale).astype(np.float32)
    assert np.array_equal(x.cpu().numpy().view(np.uint16), R.bf16_bits(std))


@pytest.mark.gpu
def test_set_targets_match_restatement_and_fit_set_totals(mlp):
    """Set-level training: the targets/weights written on the GPU against the
    restatement, and Adam steps on them drive every segment's total
    sum_r c_r y_r to its target."""
    import torch
    rng = np.random.default_rng(5)
    nseg, per = 12, 300
    n = nseg * per
    p, xb, _, _ = _problem(21, n)
    mlp.set_params(p)
    seg = np.arange(0, n + 1, per, dtype=np.int64)
    coef = rng.normal(size=n) * 10 ** rng.uniform(-4, -1, size=n)
    delta = rng.normal(scale=0.05, size=nseg)
    label = rng.normal(size=n).astype(np.float32)
    lw = (coef * coef / np.sum(coef * coef) * 0.1).astype(np.float32)
    x = _dev(torch, xb.view(np.int16))
    dc, ds, dd = _dev(torch, coef), _dev(torch, seg), _dev(torch, delta)
    dl, dlw = _dev(torch, label), _dev(torch, lw)
    t = torch.zeros(n, dtype=torch.float32, device="cuda")
    w = torch.zeros(n, dtype=torch.float32, device="cuda")
    l_set, l_lab = mlp.set_targets(x, n, dc, ds, dd, nseg, t, w, dl, dlw, want_loss=True)
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    mlp.forward(x, n, y)
    wt, ww, ws, wl = R.set_targets(y.cpu().numpy(), coef, seg, delta, label, lw)
    assert np.allclose(w.cpu().numpy(), ww, rtol=1e-6)
    assert np.allclose(t.cpu().numpy(), wt, rtol=1e-5, atol=1e-5 * np.max(np.abs(wt)))
    assert l_set == pytest.approx(ws, rel=1e-9) and l_lab == pytest.approx(wl, rel=1e-5)
    for _ in range(300):
        mlp.set_targets(x, n, dc, ds, dd, nseg, t, w)
        mlp.adam_step(x, t, w, n, lr=3e-4)
    l_end, _ = mlp.set_targets(x, n, dc, ds, dd, nseg, t, w, want_loss=True)
    assert l_end < 1e-2 * l_set, (l_set, l_end)
