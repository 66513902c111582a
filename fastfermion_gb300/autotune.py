"""Autotuner for the orbit engine's runtime options.

The engine's tuning knobs (``ffg_set_option``): the |A| threshold from which
a group skips the warp tier (``orbit_route_big`` for Pauli circuits,
``morbit_route_big`` for Majorana circuits), the 256-thread team tier
(``orbit_team``), orbit batches per host round trip (``orbit_window``),
programmatic dependent launch (``pdl``) and, for Majorana circuits, the
shortest commuting run sent to the orbit path (``morbit_min_gates``).  ``autotune`` times a propagation of
the caller's own circuit and observable under candidate settings (coordinate
descent over the space, best of ``repeats`` runs each), keeps the fastest
setting on the device's context and caches it per circuit, observable and
truncation parameters.  The options change speed only: every candidate must
give the same term count and expectation value, which the tuner checks.
"""
import hashlib
import time

import numpy as np

from . import _native

DEFAULT_SPACE = {
    "orbit_route_big": (6, 8, 10, 12),
    "orbit_team": (1, 0),
    "orbit_window": (16, 4),
    "pdl": (1, 0),
}

MAJORANA_SPACE = {
    "morbit_route_big": (12, 8, 10, 16),
    "morbit_min_gates": (2, 1, 4),
    "orbit_team": (1, 0),
    "orbit_window": (16, 4),
    "pdl": (1, 0),
}

_cache = {}


def _is_majorana(circuit):
    from .majorana import MROT
    return len(circuit) > 0 and all(isinstance(g, MROT) for g in circuit)


def _signature(circuit, observable, kwargs):
    from .propagation import encode_majorana_circuit, encode_pauli_circuit
    h = hashlib.sha256()
    try:
        h.update(encode_pauli_circuit(circuit).tobytes())
    except (KeyError, AttributeError, TypeError):
        h.update(encode_majorana_circuit(circuit).tobytes())
    for a in observable.arrays() if hasattr(observable, "arrays") else ():
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(repr(sorted(kwargs.items())).encode())
    return h.hexdigest()


def _run(circuit, observable, kwargs):
    from .propagation import propagate
    t0 = time.perf_counter()
    r = propagate(circuit, observable, **kwargs)
    dt = time.perf_counter() - t0
    return dt, len(r), complex(r.overlapwithzero()) if hasattr(r, "overlapwithzero") else complex(r.fock_state())


def autotune(circuit, observable, space=None, repeats=2, device=None, **kwargs):
    """Picks the fastest engine options for propagating ``observable`` through
    ``circuit`` with the truncation keywords ``kwargs`` (those of
    ``propagate``), applies them to the device's context and returns
    ``{"options": {...}, "seconds": best time, "timings": [(options, s), ...]}``."""
    ctx = _native.context(device)
    key = _signature(circuit, observable, kwargs)
    if key in _cache:
        for k, v in _cache[key]["options"].items():
            ctx.set_option(k, v)
        return _cache[key]
    if space is None:
        space = MAJORANA_SPACE if _is_majorana(circuit) else DEFAULT_SPACE
    space = dict(space)
    kwargs = dict(kwargs)
    if device is not None:
        kwargs["device"] = device
    best = {k: ctx.get_option(k) for k in space}
    for k, v in best.items():
        ctx.set_option(k, v)
    _run(circuit, observable, kwargs)  # warm-up: allocations, first-call set-up
    base = None
    timings = []

    def measure(opts):
        nonlocal base
        for k, v in opts.items():
            ctx.set_option(k, v)
        runs = [_run(circuit, observable, kwargs) for _ in range(max(1, repeats))]
        t = min(r[0] for r in runs)
        out = (runs[0][1], runs[0][2])
        if base is None:
            base = out
        elif out[0] != base[0] or abs(out[1] - base[1]) > 1e-12 * max(1.0, abs(base[1])):
            raise RuntimeError(f"engine options changed the result: {opts} gave {out}, expected {base}")
        timings.append((dict(opts), t))
        return t

    best_t = measure(best)
    for name, values in space.items():
        for v in values:
            if v == best[name]:
                continue
            trial = dict(best, **{name: v})
            t = measure(trial)
            if t < best_t:
                best, best_t = trial, t
    for k, v in best.items():
        ctx.set_option(k, v)
    res = {"options": best, "seconds": best_t, "timings": timings}
    _cache[key] = res
    return res
