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
serves only as device memory (tensors passed to the C ABI by address).

Training objective.  With the coefficient threshold on, the labels of single
partners do not add up to the W' value (a partner's descendants below tau are
erased alone, while in the joint W' run they merge with others), so the
network is trained on the set-level loss sum_theta (predicted correction -
(judge - low))^2 over the training parameter values, optionally with the
per-partner labels as a second term.
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


def kicked_ising_workload():
    """The learned-correction workload: the 10x10 kicked-Ising circuit (20
    steps, RZZ(-pi/2) on the 180 edges then RX(theta_h) on every site),
    observable Z at site (5,5), plain cutoff W=6 corrected towards the W'=10
    judge, threshold 1e-6."""
    from . import workloads as W
    from .propagation import encode_pauli_circuit

    def make(theta):
        from . import build_circuit
        return encode_pauli_circuit(build_circuit(W.kicked_ising_circuit(theta)))

    return Workload(make, 10, 10, 55, 6, 10, 1e-6)


class Sample:
    """Dropped partners of one parameter value: the W value `low`, the FP32
    features `feat` [n][32] and the device record of the drops (`drops`, kept
    alive for the network's input and coefficients)."""

    def __init__(self, theta, low, n, drops, feat, seconds):
        self.theta, self.low, self.n, self.drops, self.feat, self.seconds = theta, low, n, drops, feat, seconds
        self.x = None
        self.judge = self.judge_seconds = self.labels = None

    def coef(self):
        """device address of the coefficients (FP64 [n])"""
        return self.drops.device()[2]

    def inputs(self, ctx, wl, shift, scale):
        """BF16 network input [n][32] (standardised features)."""
        import torch
        self.x = torch.zeros((max(self.n, 1), 32), dtype=torch.int16, device="cuda")
        if self.n:
            tab, bog, nb = wl.table(self.theta)
            dk, stride, dre, _, dg = self.drops.device()
            _native.drop_features(ctx, dk, stride, dre, dg, self.n, tab, bog, nb, wl.coords, wl.obs_site,
                                  wl.maxdegree, x=self.x, shift=shift, scale=scale)
        return self.x


def make_sample(ctx, wl, theta, features=True):
    """The W propagation at theta recording its dropped partners above tau, and
    their FP32 features."""
    import torch
    tab, bog, nb = wl.table(theta)
    k, re, im = wl.observable()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res, drops = ctx.pauli_propagate_capture(k, re, im, tab, pauli_params(wl.maxdegree, wl.tau),
                                             capdeg=wl.maxdegree_hi, min_abs=wl.tau)
    low = res.overlapwithzero().real
    res.free()
    n = len(drops)
    feat = None
    if features:
        feat = torch.zeros((max(n, 1), 32), dtype=torch.float32, device="cuda")
        if n:
            dk, stride, dre, _, dg = drops.device()
            _native.drop_features(ctx, dk, stride, dre, dg, n, tab, bog, nb, wl.coords, wl.obs_site, wl.maxdegree,
                                  feat=feat)
    torch.cuda.synchronize()
    return Sample(theta, low, n, drops, feat, time.perf_counter() - t0)


def _f64(addr, n):
    """device FP64 [n] at addr, copied into a torch tensor"""
    import torch
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    _native.device_copy(out.data_ptr(), addr, 8 * n)
    return out


class Surrogate:
    """The network, trained on the corrections judge(theta) - low(theta) of a set
    of training parameter values (and, optionally, on per-partner labels), and
    validated on held-out values."""

    def __init__(self, ctx, wl, seed=0, members=1):
        self.ctx, self.wl, self.seed = ctx, wl, seed
        # an ensemble of `members` networks (seeds seed, seed+1, ...); the
        # correction is their mean
        self.mlps = [_native.MLP(ctx) for _ in range(members)]
        for i, m in enumerate(self.mlps):
            m.set_params(init_params(seed + i))
        self.mlp = self.mlps[0]
        self.shift = self.scale = None
        self.held_out_error = math.inf
        self.bound = 1e-3
        self.history = []

    def collect(self, thetas, labels_for=()):
        """A Sample per theta with the judge's value (plain W', timed) and, for
        thetas in labels_for, the W' labels of its dropped partners (in the
        device order of the record)."""
        import torch
        data = []
        for th in thetas:
            s = make_sample(self.ctx, self.wl, th)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.judge = self.wl.plain(self.ctx, th)
            torch.cuda.synchronize()
            s.judge_seconds = time.perf_counter() - t0
            if th in labels_for and s.n:
                dk, stride, dre, _, dg = s.drops.device()
                hk = np.stack([_native.device_view(dk + 8 * w * stride, (s.n,), "<u8").cpu().numpy()
                               for w in range(4)])
                hre = _native.device_view(dre, (s.n,), "<f8").cpu().numpy()
                hg = _native.device_view(dg, (s.n,), "<i4").cpu().numpy()
                s.labels = labels(self.ctx, self.wl.table(th)[0], hk, hre, hg, self.wl.maxdegree_hi, self.wl.tau)
            data.append(s)
        return data

    def fit(self, data, steps=6000, lr=3e-3, label_weight=0.0):
        """Adam on the set-level loss L = sum_theta (sum_D c_D t(x_D) - (judge -
        low))^2 (ffg_mlp_set_targets) plus label_weight times the normalised
        coefficient-weighted squared error of the transfers of partners with
        labels; the features are standardised with the training set's mean and
        deviation; constant rate for the first half of the steps, cosine decay
        to 1% in the second."""
        import torch
        live = [s for s in data if s.n]
        feats = torch.cat([s.feat[:s.n] for s in live])
        self.shift = feats.mean(0).cpu().numpy().astype(np.float32)
        self.scale = (1.0 / (feats.std(0) + 1e-3)).cpu().numpy().astype(np.float32)
        X = torch.cat([s.inputs(self.ctx, self.wl, self.shift, self.scale)[:s.n] for s in live]).contiguous()
        C = torch.cat([_f64(s.coef(), s.n) for s in live]).contiguous()
        seg = torch.tensor(np.cumsum([0] + [s.n for s in live]), dtype=torch.int64, device="cuda")
        delta = torch.tensor([s.judge - s.low for s in live], dtype=torch.float64, device="cuda")
        n, ns = X.shape[0], len(live)
        lab = lw = None
        if label_weight > 0 and any(s.labels is not None for s in live):
            c_h = C.cpu().numpy()
            lab_h, lw_h, pos = [], [], 0
            for s in live:
                c = c_h[pos:pos + s.n]
                pos += s.n
                if s.labels is None:
                    lab_h.append(np.zeros(s.n))
                    lw_h.append(np.zeros(s.n))
                else:
                    lab_h.append(s.labels / np.where(c == 0, 1.0, c))
                    lw_h.append(c * c)
            lw_all = np.concatenate(lw_h)
            lw_all *= label_weight / max(lw_all.sum(), 1e-300)
            lab = torch.from_numpy(np.concatenate(lab_h).astype(np.float32)).cuda()
            lw = torch.from_numpy(lw_all.astype(np.float32)).cuda()
        T = torch.empty(n, dtype=torch.float32, device="cuda")
        W = torch.empty(n, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        half = steps // 2
        for k, mlp in enumerate(self.mlps):
            for it in range(steps):
                rate = lr if it < half else lr * (0.01 + 0.5 * (1 + math.cos(math.pi * (it - half) /
                                                                           max(steps - half, 1))))
                want = it % 1000 == 0 or it == steps - 1
                loss = mlp.set_targets(X, n, C, seg, delta, ns, T, W, lab, lw, want_loss=want)
                mlp.adam_step(X, T, W, n, rate)
                if want:
                    self.history.append((k, it, loss[0], loss[1]))
        torch.cuda.synchronize()
        self.train_seconds = time.perf_counter() - t0
        self.rows, self.sets, self.steps = n, ns, steps
        return self

    def correction(self, sample):
        """sum over the sample's dropped partners of c * t(x), on the GPU."""
        import torch
        if not sample.n:
            return 0.0
        x = sample.inputs(self.ctx, self.wl, self.shift, self.scale)
        t = torch.empty(sample.n, dtype=torch.float32, device="cuda")
        return sum(m.correction(x, sample.coef(), sample.n, t) for m in self.mlps) / len(self.mlps)

    def predict(self, theta):
        """(corrected W value, seconds of W propagation with capture + features
        + network, plain W value)"""
        import torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s = make_sample(self.ctx, self.wl, theta, features=False)
        v = s.low + self.correction(s)
        torch.cuda.synchronize()
        return v, time.perf_counter() - t0, s.low

    def validate(self, held):
        """Held-out errors |corrected - judge|; records the largest as the
        validated error that decides between the surrogate and the fallback."""
        errs = np.array([abs(s.low + self.correction(s) - s.judge) for s in held])
        self.held_out_error = float(errs.max()) if errs.size else math.inf
        return errs

    def estimate(self, theta):
        """(value, seconds, path): the corrected W estimate when the validated
        held-out error is within the bound, else the plain W' propagation."""
        if self.held_out_error <= self.bound:
            v, sec, _ = self.predict(theta)
            return v, sec, "surrogate"
        import torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        v = self.wl.plain(self.ctx, theta)
        torch.cuda.synchronize()
        return v, time.perf_counter() - t0, "fallback"


def evaluate(sur, held, bound=1e-3, plain_cutoffs=(6, 7, 8, 9)):
    """Per held-out value: the error of the plain W value and of the corrected
    one against the judge, the time of the surrogate path (prediction, plus
    the fallback's W' run when the prediction misses the bound), and the time of
    the cheapest plain run within the bound (a cutoff from plain_cutoffs, else
    the judge's W' run)."""
    import torch
    rows = []
    for s in held:
        v, t_pred, low = sur.predict(s.theta)
        err = abs(v - s.judge)
        t_sur = t_pred + (s.judge_seconds if err > bound else 0.0)
        t_plain, w_plain = s.judge_seconds, sur.wl.maxdegree_hi
        for w in plain_cutoffs:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pv = sur.wl.plain(sur.ctx, s.theta, w)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            if abs(pv - s.judge) <= bound:
                t_plain, w_plain = dt, w
                break
        rows.append(dict(theta=s.theta, judge=s.judge, low=low, corrected=v, err_plain_w=abs(low - s.judge),
                         err_surrogate=err, t_predict=t_pred, t_surrogate=t_sur, t_plain=t_plain, w_plain=w_plain,
                         t_judge=s.judge_seconds, n_drops=s.n))
    return rows
