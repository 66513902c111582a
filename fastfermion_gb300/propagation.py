"""``propagate``: the drop-in entry point (src/python_bind.cpp:392-527).

Both reference overloads live under one name and are resolved the way the
binding resolves them (Pauli first): a circuit of H/S/CNOT/SWAP/CZ/ROT gates
with a Pauli observable runs Pauli propagation, a circuit of MROT gates with a
Majorana observable runs Majorana propagation.  Gates and observables of the
reference package itself are accepted too (converted by attribute access).

All propagation work runs on the GPU through libffg; ``n_threads`` and
``parallel`` are accepted for signature compatibility (every strategy of the
reference produces the same term set).
"""
import numpy as np

from . import _native
from .majorana import MROT, MajoranaPolynomial, MajoranaString
from .pauli import CNOT, CZ, H, ROT, S, SWAP, PauliPolynomial, PauliString

_KIND = {"ROT": 0, "H": 1, "S": 2, "CNOT": 3, "SWAP": 4, "CZ": 5}
_STRATEGIES = ("auto", "serial", "omp", "sharded")
_M64 = (1 << 64) - 1

_profile_enabled = False


def _pauli_masks_of(ps):
    if isinstance(ps, PauliString):
        return ps.x, ps.z
    x = z = 0  # a reference PauliString: use its index list
    for pos, a in ps.indices():
        if a in "XY":
            x |= 1 << pos
        if a in "YZ":
            z |= 1 << pos
    return x, z


def _maj_mask_of(ms):
    if isinstance(ms, MajoranaString):
        return ms.alpha
    a = 0
    for pos in ms.indices():
        a |= 1 << pos
    return a


def _is_pauli_gate(g):
    return type(g).__name__ in _KIND


def _is_majorana_gate(g):
    return type(g).__name__ == "MROT"


def encode_pauli_circuit(circuit):
    """Flat gate table (PAULI_GATE) of a Pauli circuit, in circuit order."""
    t = np.zeros(len(circuit), dtype=_native.PAULI_GATE)
    for i, g in enumerate(circuit):
        name = type(g).__name__
        t["kind"][i] = _KIND[name]
        if name == "ROT":
            x, z = _pauli_masks_of(g.axis)
            t["x"][i] = (x & _M64, x >> 64)
            t["z"][i] = (z & _M64, z >> 64)
            t["theta"][i] = g.theta
        else:
            q = list(g.qubits)
            t["q0"][i] = q[0]
            t["q1"][i] = q[1] if len(q) > 1 else 0
    return t


def encode_majorana_circuit(circuit):
    t = np.zeros(len(circuit), dtype=_native.MAJORANA_GATE)
    for i, g in enumerate(circuit):
        a = _maj_mask_of(g.axis)
        t["alpha"][i] = [(a >> (64 * w)) & _M64 for w in range(4)]
        t["theta"][i] = g.theta
        if hasattr(g, "_r"):
            t["r"][i] = int(bool(g._r))
        else:
            t["r"][i] = 0 if g.axis.is_hermitian() else 1
    return t


def _pauli_obs_arrays(obs):
    if isinstance(obs, (PauliString, PauliPolynomial)):
        p = obs if isinstance(obs, PauliPolynomial) else PauliPolynomial(obs)
        return p.arrays()
    # reference objects
    if hasattr(obs, "terms"):
        items = list(obs.terms.items())
    else:
        items = [(obs, 1 + 0j)]
    n = len(items)
    keys = np.zeros((4, n), dtype=np.uint64)
    re, im = np.zeros(n), np.zeros(n)
    for i, (s, c) in enumerate(items):
        x, z = _pauli_masks_of(s)
        keys[:, i] = (x & _M64, x >> 64, z & _M64, z >> 64)
        re[i], im[i] = c.real, c.imag
    return keys, re, im


def _maj_obs_arrays(obs):
    if isinstance(obs, (MajoranaString, MajoranaPolynomial)):
        p = obs if isinstance(obs, MajoranaPolynomial) else MajoranaPolynomial(obs)
        return p.arrays()
    items = list(obs.terms.items()) if hasattr(obs, "terms") else [(obs, 1 + 0j)]
    n = len(items)
    keys = np.zeros((4, n), dtype=np.uint64)
    re, im = np.zeros(n), np.zeros(n)
    for i, (s, c) in enumerate(items):
        a = _maj_mask_of(s)
        keys[:, i] = [(a >> (64 * w)) & _M64 for w in range(4)]
        re[i], im[i] = c.real, c.imag
    return keys, re, im


def _is_pauli_obs(o):
    return type(o).__name__ in ("PauliString", "PauliPolynomial")


def _is_majorana_obs(o):
    return type(o).__name__ in ("MajoranaString", "MajoranaPolynomial")


def _pauli_signature(circuit, observable, n_threads=1, maxdegree=None, mincoeff=None, topk=0,
                     max_xweight=-1, xtrunc_period=1, batched=True, parallel="auto", *,
                     deterministic=False, device=None):
    return locals()


def _majorana_signature(circuit, observable, maxdegree=None, mincoeff=0, *, deterministic=False,
                        device=None):
    return locals()


def propagate(circuit, observable, *args, **kwargs):
    """Heisenberg-picture propagation of ``observable`` through ``circuit``.

    Pauli form (src/pauli/propagate.h:297): ``propagate(circuit, observable,
    n_threads=1, maxdegree=None, mincoeff=None, topk=0, max_xweight=-1,
    xtrunc_period=1, batched=True, parallel="auto") -> PauliPolynomial``.

    Majorana form (src/majorana_propagation.h:35-55): ``propagate(circuit,
    observable, maxdegree=None, mincoeff=0) -> MajoranaPolynomial``.

    Extra keywords: ``deterministic`` (sorted-key result order and expectation
    sums) and ``device`` (CUDA device ordinal).
    """
    circuit = list(circuit)
    if all(_is_pauli_gate(g) for g in circuit) and _is_pauli_obs(observable):
        a = _pauli_signature(circuit, observable, *args, **kwargs)
        return _propagate_pauli(circuit, observable, a["n_threads"], a["maxdegree"], a["mincoeff"],
                                a["topk"], a["max_xweight"], a["xtrunc_period"], a["batched"],
                                a["parallel"], a["deterministic"], a["device"])
    if all(_is_majorana_gate(g) for g in circuit) and _is_majorana_obs(observable):
        a = _majorana_signature(circuit, observable, *args, **kwargs)
        return _propagate_majorana(circuit, observable, a["maxdegree"], a["mincoeff"] or 0.0,
                                   a["deterministic"], a["device"])
    raise TypeError("propagate(): incompatible function arguments (expected a Pauli circuit with a "
                    "Pauli observable, or an MROT circuit with a Majorana observable)")


def _propagate_pauli(circuit, observable, n_threads, maxdegree, mincoeff, topk, max_xweight,
                     xtrunc_period, batched, parallel, deterministic, device):
    if n_threads > 1 and parallel not in _STRATEGIES:
        # the reference returns the observable unchanged for an unknown strategy
        # name when n_threads > 1 (src/pauli/propagate.h:306-308, 492)
        return PauliPolynomial.from_arrays(*_pauli_obs_arrays(observable))
    keys, re, im = _pauli_obs_arrays(observable)
    table = encode_pauli_circuit(circuit)
    ctx = _native.context(device)
    ctx.set_profiling(_profile_enabled)
    params = dict(maxdegree=128 if maxdegree is None else int(maxdegree), topk=int(topk),
                  mincoeff=0.0 if mincoeff is None else float(mincoeff),
                  max_xweight=int(max_xweight), xtrunc_period=int(xtrunc_period),
                  batched=int(bool(batched)), deterministic=int(bool(deterministic)))
    res = ctx.pauli_propagate(keys, re, im, table, params)
    _record_profile(ctx)
    return PauliPolynomial._from_result(res)


def _propagate_majorana(circuit, observable, maxdegree, mincoeff, deterministic, device):
    keys, re, im = _maj_obs_arrays(observable)
    table = encode_majorana_circuit(circuit)
    ctx = _native.context(device)
    ctx.set_profiling(_profile_enabled)
    params = dict(has_maxdegree=int(maxdegree is not None),
                  maxdegree=0 if maxdegree is None else int(maxdegree),
                  mincoeff=float(mincoeff or 0.0), deterministic=int(bool(deterministic)), pad=0)
    res = ctx.majorana_propagate(keys, re, im, table, params)
    _record_profile(ctx)
    return MajoranaPolynomial._from_result(res)


# --------------------------------------------------------------------------
# profiling hooks (src/python_bind.cpp:428-446)
# --------------------------------------------------------------------------
_last_profile = {}
_accum = {}


def _record_profile(ctx):
    global _last_profile
    p = ctx.profile()
    _last_profile = p
    if _profile_enabled:
        for k, v in p.items():
            _accum[k] = _accum.get(k, 0) + v


def profile_reset():
    """Clears the accumulated per-phase times and enables collection."""
    global _profile_enabled
    _accum.clear()
    _profile_enabled = True


def profile_disable():
    global _profile_enabled
    _profile_enabled = False


def profile_get():
    """Accumulated per-phase timings.  The reference's keys are kept: ``emit``
    is rotation-kernel time (emission and merge are one fused pass on the GPU,
    so ``merge`` and ``snapshot`` stay 0); ``n_gates`` counts rotations.  The
    per-thread lists are empty and ``n_local``/``n_remote`` are 0 (no shards).
    GPU-specific counters follow under their own names."""
    a = dict(_accum)
    d = {"snapshot": 0.0, "emit": a.get("seconds_rotations", 0.0), "merge": 0.0,
         "n_gates": int(a.get("n_gates", 0)), "emit_per_thread": [], "merge_per_thread": [],
         "n_local": 0, "n_remote": 0}
    d.update({k: v for k, v in a.items()})
    return d


def last_profile():
    """Counters of the most recent propagation (whether or not profiling is on)."""
    return dict(_last_profile)


has_openmp = False
