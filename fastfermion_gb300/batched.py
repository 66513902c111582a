"""Batched propagation and gradients.

Not in fastfermion: its ``propagate`` runs one observable through one circuit
and has no derivatives.  Here many observables (instances) that go through
the same circuit structure -- the same rotation axes and Clifford gates, with
their own rotation angles -- are propagated together in one term store on the
GPU (``ffg_pauli_propagate_batched``), and the adjoint kernel gives
d<0|O_i|0>/d theta for every rotation angle of every instance
(``ffg_batch_adjoint``).  ``expectation`` wraps both in a
``torch.autograd.Function``.

Truncation semantics are those of ``propagate`` for each instance alone
(``maxdegree``, ``mincoeff``, ``batched``); the derivative is that of the
truncated map with the truncation pattern of the forward pass held fixed.
"""
import numpy as np

from . import _native
from .pauli import PauliPolynomial, PauliString
from .propagation import encode_pauli_circuit


def _observable_arrays(observables):
    keys, res, offsets = [], [], [0]
    for o in observables:
        if isinstance(o, PauliString):
            o = PauliPolynomial(o)
        k, re, im = o.arrays()
        if np.any(im != 0):
            raise ValueError("batched propagation needs real coefficients")
        keys.append(k)
        res.append(re)
        offsets.append(offsets[-1] + re.size)
    keys = np.concatenate(keys, axis=1) if keys else np.zeros((4, 0), dtype=np.uint64)
    re = np.concatenate(res) if res else np.zeros(0)
    return keys, re, np.asarray(offsets, dtype=np.int64)


def _params(maxdegree, mincoeff, batched):
    return dict(maxdegree=128 if maxdegree is None else int(maxdegree), topk=0,
                mincoeff=0.0 if mincoeff is None else float(mincoeff), max_xweight=-1,
                xtrunc_period=1, batched=int(bool(batched)), deterministic=0)


class BatchedResult:
    """Outcome of ``propagate_batched``: per-instance expectations, final term
    sets and the adjoint."""

    def __init__(self, expect, handle):
        self.expect = expect
        self._h = handle

    @property
    def ninst(self):
        return self._h.ninst

    def terms(self):
        """(keys (4, n), re (n,), inst (n,)) of all instances' final terms."""
        return self._h.copy()

    def polynomials(self):
        """One PauliPolynomial per instance."""
        keys, re, inst = self._h.copy()
        out = []
        for i in range(self.ninst):
            sel = inst == i
            out.append(PauliPolynomial.from_arrays(keys[:, sel], re[sel], np.zeros(int(sel.sum()))))
        return out

    def gradient(self, weights=None, with_coef=False):
        """d(sum_i w_i <O_i>)/d theta as an (ninst, nrot) array (w = 1 by default);
        with_coef also returns the derivative by the input coefficients."""
        w = np.ones(self.ninst) if weights is None else np.asarray(weights, dtype=np.float64)
        g, gc = self._h.adjoint(w, with_coef=with_coef)
        return (g, gc) if with_coef else g


def propagate_batched(circuit, observables, thetas=None, maxdegree=None, mincoeff=None, batched=True,
                      checkpoint_every=1, device=None):
    """Propagates every observable of ``observables`` through ``circuit`` with
    its own rotation angles: row i of ``thetas`` (ninst x number of ROT gates,
    circuit order) replaces the ROT angles for instance i (None keeps the
    circuit's angles).  ``checkpoint_every = k`` keeps the term set entering
    every k-th step for the adjoint (0: no gradient)."""
    table = encode_pauli_circuit(circuit) if not isinstance(circuit, np.ndarray) else circuit
    keys, re, offsets = _observable_arrays(observables)
    ctx = _native.context(device)
    if thetas is not None:
        thetas = np.ascontiguousarray(thetas, dtype=np.float64)
        nrot = int(np.sum(table["kind"] == _native.ROT))
        if thetas.shape != (offsets.size - 1, nrot):
            raise ValueError(f"thetas must have shape ({offsets.size - 1}, {nrot})")
    expect, h = ctx.pauli_propagate_batched(keys, re, offsets, table, thetas,
                                            _params(maxdegree, mincoeff, batched), checkpoint_every)
    return BatchedResult(expect, h)


def _autograd_function():
    import torch

    class PropagateExpectation(torch.autograd.Function):
        """thetas (ninst, nrot) -> <0|O_i(thetas_i)|0> (ninst,), float64."""

        @staticmethod
        def forward(fctx, thetas, table, observables, maxdegree, mincoeff, batched, checkpoint_every):
            th = thetas.detach().to("cpu", torch.float64).numpy()
            r = propagate_batched(table, observables, th, maxdegree, mincoeff, batched,
                                  max(1, int(checkpoint_every)))
            fctx.result = r
            return torch.as_tensor(r.expect, dtype=torch.float64, device=thetas.device)

        @staticmethod
        def backward(fctx, grad_out):
            w = grad_out.detach().to("cpu", torch.float64).numpy()
            g = fctx.result.gradient(w)
            return (torch.as_tensor(g, dtype=torch.float64, device=grad_out.device),
                    None, None, None, None, None, None)

    return PropagateExpectation


_fn = None


def expectation(circuit, observables, thetas, maxdegree=None, mincoeff=None, batched=True, checkpoint_every=1):
    """Differentiable per-instance expectations <0|O_i|0> as a torch tensor;
    ``thetas`` is an (ninst, nrot) float64 tensor."""
    global _fn
    if _fn is None:
        _fn = _autograd_function()
    table = encode_pauli_circuit(circuit) if not isinstance(circuit, np.ndarray) else circuit
    return _fn.apply(thetas, table, observables, maxdegree, mincoeff, batched, checkpoint_every)
