"""Shared helpers for the GPU parity tests (run libffg through its C ABI)."""
import numpy as np

from fastfermion_gb300 import _native
from oracle import oracle as O


def pauli_params(fx, **over):
    p = dict(maxdegree=int(fx["maxdegree"]), topk=int(fx["topk"]), mincoeff=float(fx["mincoeff"]),
             max_xweight=int(fx["max_xweight"]), xtrunc_period=int(fx["xtrunc_period"]),
             batched=int(bool(fx["batched"])), deterministic=0)
    p.update(over)
    return p


def majorana_params(fx, **over):
    p = dict(has_maxdegree=int(bool(fx["has_maxdegree"])), maxdegree=int(fx["maxdegree"]),
             mincoeff=float(fx["mincoeff"]), deterministic=0, pad=0)
    p.update(over)
    return p


def run_gpu(fx, **over):
    ctx = _native.context(0)
    if str(fx["kind"]) == "pauli":
        return ctx.pauli_propagate(fx["obs_keys"], fx["obs_re"], fx["obs_im"], fx["gates"],
                                   pauli_params(fx, **over))
    return ctx.majorana_propagate(fx["obs_keys"], fx["obs_re"], fx["obs_im"], fx["gates"],
                                  majorana_params(fx, **over))


def run_oracle(fx):
    if str(fx["kind"]) == "pauli":
        return O.pauli_propagate(fx["gates"], fx["obs_keys"], fx["obs_re"], fx["obs_im"],
                                 maxdegree=int(fx["maxdegree"]), mincoeff=float(fx["mincoeff"]),
                                 topk=int(fx["topk"]), max_xweight=int(fx["max_xweight"]),
                                 xtrunc_period=int(fx["xtrunc_period"]), batched=bool(fx["batched"]))
    md = int(fx["maxdegree"]) if bool(fx["has_maxdegree"]) else None
    return O.majorana_propagate(fx["gates"], fx["obs_keys"], fx["obs_re"], fx["obs_im"],
                                maxdegree=md, mincoeff=float(fx["mincoeff"]))


def has_topk_tie(fx):
    """True when some top-k cut in the oracle run lands on tied magnitudes (the
    GPU's tie rule keeps the smallest keys; the reference keeps its hash-map
    iteration order)."""
    return int(fx["topk"]) > 0
