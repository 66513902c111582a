"""CPU restatement (numpy) of the learned correction's network and features.

TEST INFRASTRUCTURE ONLY: the checker of the GPU kernels in
fastfermion_gb300/csrc/ffg_mlp.cu (imported by the tests, never by the
fastfermion_gb300 package).  No counterpart in the reference, whose propagate
discards the partners that the degree filter drops
(src/pauli/propagate.h:71-89); these functions restate the GPU's own
definitions so that its kernels can be checked against them.

Network: 32 -> 128 -> 128 -> 128 -> 1, GELU after each hidden layer, in
the tanh form of Hendrycks and Gimpel (2016):
gelu(z) = z/2 (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))).  The GPU evaluates
that tanh with its hardware approximation (relative error about 2^-11); here
it is exact.  The GPU rounds the GEMM operands to BF16 (round to nearest
even) -- the weights W1..W3, the input x, the hidden activations H1, H2 and
the pre-activation gradients dZ1..dZ3 -- and accumulates in FP32; everything
else is FP32.  `forward`/`gradient` reproduce those roundings (accumulating in
float64, so only the order of the FP32 sums differs); with bf16=False they are
the exact float64 network, used to pin the backward pass by finite differences.

Parameter layout (flat, 37377 values): W1[128][32], b1[128], W2[128][128],
b2[128], W3[128][128], b3[128], w4[128], b4.
"""
import math

import numpy as np

IN, HID = 32, 128
NPARAMS = HID * IN + HID + 2 * (HID * HID + HID) + HID + 1


def bf16_bits(a):
    """float32 -> BF16 bit patterns (uint16), round to nearest even."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bits(b):
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def bf16(a):
    return from_bits(bf16_bits(a))


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (HID, IN)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)),
                        ("W3", (HID, HID)), ("b3", (HID,)), ("w4", (HID,)), ("b4", ())):
        size = int(np.prod(shape)) if shape else 1
        out[name] = p[o:o + size].reshape(shape) if shape else p[o]
        o += size
    return out


def pack(d):
    return np.concatenate([np.ravel(d[k]) for k in ("W1", "b1", "W2", "b2", "W3", "b3", "w4")] +
                          [np.array([d["b4"]])])


def init_params(seed=0):
    """Kaiming-uniform weights (GELU gain ~ ReLU's), zero biases."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, (o, i) in (("W1", (HID, IN)), ("W2", (HID, HID)), ("W3", (HID, HID))):
        lim = math.sqrt(6.0 / i)
        d[name] = rng.uniform(-lim, lim, size=(o, i))
    d["b1"], d["b2"], d["b3"] = np.zeros(HID), np.zeros(HID), np.zeros(HID)
    d["w4"] = rng.uniform(-math.sqrt(3.0 / HID), math.sqrt(3.0 / HID), size=HID)
    d["b4"] = 0.0
    return pack(d).astype(np.float32)


_GK = math.sqrt(2.0 / math.pi)
_GA = 0.044715


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(_GK * (z + _GA * z * z * z)))


def gelu_grad(z):
    t = np.tanh(_GK * (z + _GA * z * z * z))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _GK * (1.0 + 3.0 * _GA * z * z)


def _round(a, on):
    return bf16(a).astype(np.float64) if on else np.asarray(a, dtype=np.float64)


def _f32(a, on):
    return np.asarray(a, dtype=np.float32).astype(np.float64) if on else a


def forward(p, x, bf16_ops=True, cache=False):
    """y[n] for inputs x[n][32] (FP32 values; rounded to BF16 when bf16_ops)."""
    d = unpack(np.asarray(p, dtype=np.float32) if bf16_ops else p)
    on = bf16_ops
    X = _round(x, on)
    z1 = _f32(X @ _round(d["W1"], on).T, on)
    h1 = _round(gelu(z1 + d["b1"]), on)
    z2 = _f32(h1 @ _round(d["W2"], on).T, on)
    h2 = _round(gelu(z2 + d["b2"]), on)
    z3 = _f32(h2 @ _round(d["W3"], on).T, on)
    h3 = _f32(gelu(z3 + d["b3"]), on)
    y = h3 @ d["w4"] + d["b4"]
    if cache:
        return y, dict(X=X, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3, d=d)
    return y


def gradient(p, x, target, weight, bf16_ops=True):
    """(dL/dp flat, L) with L = sum_r weight_r (y_r - target_r)^2."""
    on = bf16_ops
    y, c = forward(p, x, bf16_ops, cache=True)
    d = c["d"]
    e = y - target
    loss = float(np.sum(weight * e * e))
    dy = _f32(2.0 * weight * e, on)
    g = {}
    g["w4"] = c["h3"].T @ dy
    g["b4"] = np.sum(dy)
    dz3 = _f32(dy[:, None] * d["w4"][None, :] * gelu_grad(c["z3"] + d["b3"]), on)
    g["b3"] = dz3.sum(axis=0)
    dz3r = _round(dz3, on)
    g["W3"] = dz3r.T @ c["h2"]
    dh2 = _f32(dz3r @ _round(d["W3"], on), on)
    dz2 = _f32(dh2 * gelu_grad(c["z2"] + d["b2"]), on)
    g["b2"] = dz2.sum(axis=0)
    dz2r = _round(dz2, on)
    g["W2"] = dz2r.T @ c["h1"]
    dh1 = _f32(dz2r @ _round(d["W2"], on), on)
    dz1 = _f32(dh1 * gelu_grad(c["z1"] + d["b1"]), on)
    g["b1"] = dz1.sum(axis=0)
    g["W1"] = _round(dz1, on).T @ c["X"]
    return pack(g), loss


def adam(p, g, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (the GPU's update, in float64): returns (p, m, v)."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    c1, c2 = 1 - beta1 ** step, 1 - beta2 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


# ---------------------------------------------------------------------------
# features of dropped partners (ffg_drop_features)
# ---------------------------------------------------------------------------
def features(keys, coef, gate, gates, batch_of_gate, nbatches, coords, obs, maxdegree):
    """[n][32] float64 features (the GPU computes them in FP32)."""
    keys = np.asarray(keys, dtype=np.uint64).reshape(4, -1)
    coords = np.asarray(coords, dtype=np.float64).reshape(2, 128)
    n = keys.shape[1]
    lx = max(1.0, float(np.max(coords[0] + 1.0)))
    ly = max(1.0, float(np.max(coords[1] + 1.0)))
    ng = len(gates)
    sup = np.zeros((ng, 2), dtype=np.uint64)
    abs_sin = np.zeros(ng)
    rot = np.zeros(ng, dtype=bool)
    for j, G in enumerate(gates):
        if int(G["kind"]) == 0:
            sup[j, 0] = int(G["x"][0]) | int(G["z"][0])
            sup[j, 1] = int(G["x"][1]) | int(G["z"][1])
            abs_sin[j] = float(np.float32(abs(math.sin(float(G["theta"])))))
            rot[j] = True
        else:
            qs = [int(G["q0"])] + ([int(G["q1"])] if int(G["kind"]) >= 3 else [])
            for q in qs:
                sup[j, q >> 6] |= np.uint64(1 << (q & 63))
    ox, oy = coords[0, obs], coords[1, obs]
    out = np.zeros((n, 32))
    span = lx + ly
    for i in range(n):
        x0, x1, z0, z1 = (int(keys[w, i]) for w in range(4))
        xb = x0 | (x1 << 64)
        zb = z0 | (z1 << 64)
        s = xb | zb
        qs = [q for q in range(128) if (s >> q) & 1]
        types = [(1 if ((xb >> q) & 1 and (zb >> q) & 1) else (0 if (xb >> q) & 1 else 2)) for q in qs]
        nx, ny, nz = types.count(0), types.count(1), types.count(2)
        w = nx + ny + nz
        qx = np.array([coords[0, q] for q in qs])
        qy = np.array([coords[1, q] for q in qs])
        dist = np.abs(qx - ox) + np.abs(qy - oy)
        near = [sum(1 for t, d in zip(types, dist) if t == k and d <= 1.0) for k in range(3)]
        mid = [sum(1 for t, d in zip(types, dist) if t == k and 1.0 < d <= 3.0) for k in range(3)]
        cx, cy = (qx.mean(), qy.mean()) if w else (0.0, 0.0)
        g = int(gate[i])
        c = s
        cone, sin_sum = 0, np.float32(0.0)
        for j in range(g - 1, -1, -1):  # FP32 sum in the GPU's order
            sj = int(sup[j, 0]) | (int(sup[j, 1]) << 64)
            if sj & c:
                cone += 1
                sin_sum = np.float32(sin_sum + np.float32(abs_sin[j]))
                c |= sj
        cg = float(coef[i])
        f = out[i]
        f[0], f[1], f[2], f[3] = w / 8, nx / 8, ny / 8, nz / 8
        f[4], f[5], f[6], f[7] = qx.min() / lx, qx.max() / lx, qy.min() / ly, qy.max() / ly
        f[8] = (qx.max() - qx.min() + 1) * (qy.max() - qy.min() + 1) / (lx * ly)
        f[9] = math.log10(abs(cg) + 1e-300) / 8 + 1
        f[10] = -1.0 if cg < 0 else 1.0
        f[11] = batch_of_gate[g] / nbatches
        f[12] = g / ng
        f[13] = cone / ng
        f[14] = np.float32(sin_sum / np.float32(cone)) if cone else 0.0
        f[15] = abs_sin[g]
        f[16] = math.sqrt(max(0.0, 1.0 - abs_sin[g] ** 2)) if rot[g] else 1.0
        f[17] = dist.min() / span
        f[18] = (abs(cx - ox) + abs(cy - oy)) / span
        f[19] = 1.0 if (s >> obs) & 1 else 0.0
        f[20] = (nx + ny) / 8
        f[21], f[22], f[23] = near[0] / 5, near[1] / 5, near[2] / 5
        f[24], f[25], f[26] = mid[0] / 8, mid[1] / 8, mid[2] / 8
        f[27] = (w - maxdegree) / 4
        f[28] = bin(c).count("1") / (lx * ly)
        f[29] = (nbatches - batch_of_gate[g]) / nbatches
        f[30] = (cx - ox) / lx
        f[31] = (cy - oy) / ly
    return out


def set_targets(y, coef, seg, delta, label=None, label_weight=None):
    """Per-row targets and weights whose weighted squared error has the gradient
    of the set-level loss (ffg_mlp_set_targets): returns (target, weight,
    set loss, label loss)."""
    y = np.asarray(y, np.float64)
    coef = np.asarray(coef, np.float64)
    seg = np.asarray(seg, np.int64)
    n, ns = y.size, seg.size - 1
    R = np.array([np.dot(coef[seg[s]:seg[s + 1]], y[seg[s]:seg[s + 1]]) - delta[s] for s in range(ns)])
    segid = np.repeat(np.arange(ns), np.diff(seg))
    g = R[segid] * coef
    w = np.full(n, np.float32(1.0 / n), dtype=np.float64)
    lab_loss = 0.0
    if label is not None:
        e = y - np.asarray(label, np.float64)
        lw = np.asarray(label_weight, np.float64)
        g = g + lw * e
        w = w + lw
        lab_loss = float(np.sum(lw * e * e))
    return y - g / w, w, float(np.sum(R * R)), lab_loss
