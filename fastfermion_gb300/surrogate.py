"""Learned truncation correction: a surrogate for the partners that a low
weight cutoff drops.

No counterpart in the reference: its propagate (src/pauli/propagate.h:71-89)
discards every partner of weight above ``maxdegree``.  With the truncation
pattern fixed, the propagation is linear, so the value at a higher cutoff W'
is the low-cutoff value plus, for every partner dropped at gate g, its own
value propagated at W' through the gates still to come (gates [0, g)).  That
value divided by the partner's coefficient is the partner's *transfer*; the
network predicts it from 32 features of the partner, and the corrected
estimate is

    <O>_W + sum over dropped partners D of c_D * t(features(D)).

Everything runs on the GPU through the C ABI:
  * ``capture``    the W propagation, recording the dropped partners above the
                   coefficient threshold (ffg_pauli_propagate_capture);
  * ``labels``     the training targets: every dropped partner propagated at
                   W' from its gate, all of them as instances of one batched
                   propagation whose rotations before that gate are inactive
                   (ffg_pauli_propagate_instances);
  * features       ffg_drop_features;
  * the network    trained by ffg_mlp_adam_step (tcgen05 BF16 GEMMs, FP32
                   accumulation) and evaluated by ffg_mlp_correction.

Plain propagation at W' is the judge of the held-out error and the fallback:
``Surrogate.estimate`` returns the corrected W value only when the validated
held-out error is within the bound, and otherwise runs plain W'.  PyTorch
serves only as device memory (tensors passed by address) and for shuffling
rows between steps.
"""
import math
import time

import numpy as np

from . import _native


def batch_of_gate(tab):
    """(index of the commuting run of every circuit gate in application order,
    number of runs).  Rotations get their run; a Clifford gate gets the run of
    the next rotation applied after it."""
    tab = np.ascontiguousarray(tab, dtype=_native.PAULI_GATE)
    sizes = _native.pauli_schedule(tab, batched=True)
    rot = np.nonzero(tab["kind"] == _native.ROT)[0][::-1]  # application order
    out = np.zeros(tab.size, dtype=np.int32)
    pos = 0
    for b, s in enumerate(sizes):
        out[rot[pos:pos + s]] = b
        pos += s
    last = len(sizes) - 1 if sizes else 0
    for g in range(tab.size - 1, -1, -1):
        if tab["kind"][g] == _native.ROT:
            last = out[g]
        else:
            out[g] = last
    return out, max(1, len(sizes))


def lattice_coords(lx, ly):
    """[2][128] coordinates of the qubits of an lx-by-ly lattice, qubit ly*x + y."""
    c = np.zeros((2, 128), dtype=np.float32)
    for q in range(lx * ly):
        c[0, q], c[1, q] = q // ly, q % ly
    return c


def active_masks(tab, gates_of_drops):
    """[m][W] uint64 masks: the rotations before each drop's creating gate."""
    tab = np.ascontiguousarray(tab, dtype=_native.PAULI_GATE)
    is_rot = tab["kind"] == _native.ROT
    nrot = int(is_rot.sum())
    words = max(1, (nrot + 63) // 64)
    nbefore = np.concatenate([[0], np.cumsum(is_rot)])[np.asarray(gates_of_drops, dtype=np.int64)]
    m = np.zeros((nbefore.size, words), dtype=np.uint64)
    for wd in range(words):
        k = np.clip(nbefore - 64 * wd, 0, 64)
        full = k >= 64
        m[full, wd] = np.uint64(0xFFFFFFFFFFFFFFFF)
        part = ~full & (k > 0)
        m[part, wd] = (np.uint64(1) << k[part].astype(np.uint64)) - np.uint64(1)
    return m


def init_params(seed=0):
    """Kaiming-uniform weights, zero biases (FP32, the ffg_mlp layout)."""
    rng = np.random.default_rng(seed)
    parts = []
    for o, i in ((128, 32), (128, 128), (128, 128)):
        lim = math.sqrt(6.0 / i)
        parts += [rng.uniform(-lim, lim, size=o * i), np.zeros(o)]
    parts += [rng.uniform(-math.sqrt(3.0 / 128), math.sqrt(3.0 / 128), size=128), np.zeros(1)]
    return np.concatenate(parts).astype(np.float32)


def pauli_params(maxdegree, tau):
    return dict(maxdegree=int(maxdegree), topk=0, mincoeff=float(tau), max_xweight=-1, xtrunc_period=1,
                batched=1, deterministic=0)


def labels(ctx, tab, dk, dre, dg, maxdegree_hi, tau, chunk=4096):
    """Value of every dropped partner (keys dk [4][m], coefficient dre, creating
    gate dg) propagated at maxdegree_hi through the gates still to come."""
    m = dre.size
    out = np.zeros(m)
    for s in range(0, m, chunk):
        e = min(m, s + chunk)
        v, b = ctx.pauli_propagate_instances(dk[:, s:e], dre[s:e], np.arange(e - s + 1), tab, None,
                                             pauli_params(maxdegree_hi, tau), active_masks(tab, dg[s:e]))
        b.free()
        out[s:e] = v
    return out


class Workload:
    """A family of circuits (one per parameter value) on an lx-by-ly lattice
    with a single-site Z observable, a low cutoff `maxdegree`, the judge's
    cutoff `maxdegree_hi` and a coefficient threshold `tau`."""

    def __init__(self, make_table, lx, ly, obs_site, maxdegree, maxdegree_hi, tau):
        self.make_table = make_table
        self.lx, self.ly, self.obs_site = lx, ly, obs_site
        self.maxdegree, self.maxdegree_hi, self.tau = maxdegree, maxdegree_hi, tau
        self.coords = lattice_coords(lx, ly)
        self._cache = {}

    def observable(self):
        k = np.zeros((4, 1), dtype=np.uint64)
        k[2 + self.obs_site // 64, 0] = np.uint64(1) << np.uint64(self.obs_site % 64)
        return k, np.ones(1), np.zeros(1)

    def table(self, theta):
        if theta not in self._cache:
            tab = self.make_table(theta)
            self._cache[theta] = (tab, *batch_of_gate(tab))
        return self._cache[theta]

    def plain(self, ctx, theta, maxdegree=None):
        """<0|O|0> of the plain propagation (default: the judge's cutoff)."""
        tab = self.table(theta)[0]
        k, re, im = self.observable()
        r = ctx.pauli_propagate(k, re, im, tab, pauli_params(maxdegree or self.maxdegree_hi, self.tau))
        v = r.overlapwithzero().real
        r.free()
        return v


class Sample:
    """Dropped partners of one parameter value: device BF16 features x [n][32],
    device FP64 coefficients, and for training data the transfer targets and
    the sum of the labels."""

    def __init__(self, theta, low, x, coef, n, keep=None, target=None, label_sum=None):
        self.theta, self.low, self.x, self.coef, self.n = theta, low, x, coef, n
        self.keep, self.target, self.label_sum = keep, target, label_sum


def make_sample(ctx, wl, theta, with_labels=False):
    """The W propagation at theta with capture, and the features (with_labels:
    and the W' labels) of its dropped partners above tau."""
    import torch
    tab, bog, nb = wl.table(theta)
    k, re, im = wl.observable()
    res, drops = ctx.pauli_propagate_capture(k, re, im, tab, pauli_params(wl.maxdegree, wl.tau),
                                             capdeg=wl.maxdegree_hi, min_abs=wl.tau)
    low = res.overlapwithzero().real
    res.free()
    n = len(drops)
    x = torch.zeros((max(n, 1), 32), dtype=torch.int16, device="cuda")
    if not with_labels:
        if n:
            dk, stride, dre, _, dg = drops.device()
            _native.drop_features(ctx, dk, stride, dre, dg, n, tab, bog, nb, wl.coords, wl.obs_site,
                                  wl.maxdegree, None, x)
            return Sample(theta, low, x, dre, n, keep=drops)
        drops.free()
        return Sample(theta, low, x, None, 0)
    hk, hre, _, hg = drops.copy()
    drops.free()
    lab = labels(ctx, tab, hk, hre, hg, wl.maxdegree_hi, wl.tau) if n else np.zeros(0)
    coef = torch.from_numpy(hre.copy()).cuda()
    if n:
        kd = torch.from_numpy(hk.view(np.int64).copy()).cuda()
        gd = torch.from_numpy(hg.copy()).cuda()
        _native.drop_features(ctx, kd, n, coef, gd, n, tab, bog, nb, wl.coords, wl.obs_site, wl.maxdegree,
                              None, x)
    target = torch.from_numpy((lab / np.where(hre == 0, 1.0, hre)).astype(np.float32)).cuda()
    return Sample(theta, low, x, coef, n, target=target, label_sum=float(lab.sum()))


class Surrogate:
    """The trained network, its training history and its validated error."""

    def __init__(self, ctx, wl, seed=0):
        self.ctx, self.wl = ctx, wl
        self.mlp = _native.MLP(ctx)
        self.mlp.set_params(init_params(seed))
        self.seed = seed
        self.held_out_error = math.inf
        self.history = []

    def train(self, samples, steps=2000, batch=8192, lr=1e-3, lr_end=1e-5):
        """Adam on the coefficient-weighted squared error of the predicted
        contributions, sum_r c_r^2 (t_pred - t_r)^2 / sum_r c_r^2 over each
        minibatch; cosine learning-rate decay from lr to lr_end."""
        import torch
        xs = torch.cat([s.x[:s.n] for s in samples if s.n])
        ts = torch.cat([s.target[:s.n] for s in samples if s.n])
        cs = torch.cat([s.coef[:s.n] for s in samples if s.n])
        w_all = (cs * cs).float()
        n = xs.shape[0]
        g = torch.Generator(device="cuda")
        g.manual_seed(self.seed)
        b = min(batch, n)
        t0 = time.perf_counter()
        perm = torch.randperm(n, device="cuda", generator=g)
        pos = 0
        for step in range(steps):
            if pos + b > n:
                perm = torch.randperm(n, device="cuda", generator=g)
                pos = 0
            idx = perm[pos:pos + b]
            pos += b
            x = xs[idx].contiguous()
            t = ts[idx].contiguous()
            w = w_all[idx]
            w = (w / w.sum()).contiguous()
            rate = lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * step / max(steps - 1, 1)))
            loss = self.mlp.adam_step(x, t, w, b, rate, want_loss=(step % 200 == 0 or step == steps - 1))
            if loss is not None:
                self.history.append((step, loss))
        torch.cuda.synchronize()
        self.train_seconds = time.perf_counter() - t0
        self.rows = n
        return self

    def correction(self, sample):
        """sum over the sample's dropped partners of c * t_pred (device work)."""
        import torch
        if not sample.n:
            return 0.0
        t = torch.empty(sample.n, dtype=torch.float32, device="cuda")
        coef = sample.coef if isinstance(sample.coef, int) else sample.coef
        return self.mlp.correction(sample.x, coef, sample.n, t)

    def validate(self, held_out, judge_values, bound=1e-3):
        """Held-out |corrected - judge| for each sample; records the largest."""
        errs = []
        for s, j in zip(held_out, judge_values):
            errs.append(abs(s.low + self.correction(s) - j))
        self.held_out_error = max(errs) if errs else math.inf
        self.bound = bound
        return np.array(errs)

    def estimate(self, theta):
        """(value, seconds, path): the corrected W estimate when the validated
        held-out error is within the bound, else the plain W' propagation."""
        import torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if self.held_out_error <= getattr(self, "bound", 1e-3):
            s = make_sample(self.ctx, self.wl, theta)
            v = s.low + self.correction(s)
            path = "surrogate"
        else:
            v = self.wl.plain(self.ctx, theta)
            path = "fallback"
        torch.cuda.synchronize()
        return v, time.perf_counter() - t0, path
