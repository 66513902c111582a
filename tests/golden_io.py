"""Helpers shared by the tests: golden-fixture loading and term-set comparison."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture_names(kind=None, full_only=False):
    """Propagation fixtures (kind "pauli" or "majorana"; other kinds, such as the
    parameter-shift fixtures, are loaded by name)."""
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        with np.load(p) as z:
            if kind and str(z["kind"]) != kind:
                continue
            if not kind and str(z["kind"]) not in ("pauli", "majorana"):
                continue
            if full_only and "res_keys" not in z:
                continue
        out.append(os.path.basename(p)[:-4])
    return out


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def sort_terms(keys, re, im):
    keys = np.asarray(keys, dtype=np.uint64).reshape(4, -1)
    order = np.lexsort(tuple(keys[w] for w in (3, 2, 1, 0)))
    return keys[:, order], np.asarray(re)[order], np.asarray(im)[order]


def checksum(keys, re, im):
    import hashlib
    k, r, i = sort_terms(keys, re, im)
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(k).tobytes())
    h.update(np.ascontiguousarray(r + 0.0).tobytes())
    h.update(np.ascontiguousarray(i + 0.0).tobytes())
    return h.hexdigest()


def assert_same_terms(a, b, rtol=0.0, atol=0.0):
    """a, b: (keys, re, im).  Identical key sets; coefficients equal (== when
    rtol = atol = 0, which treats +0 and -0 as equal)."""
    ka, ra, ia = sort_terms(*a)
    kb, rb, ib = sort_terms(*b)
    assert ka.shape == kb.shape, f"term count {ka.shape[1]} != {kb.shape[1]}"
    assert np.array_equal(ka, kb), "key sets differ"
    if rtol == 0.0 and atol == 0.0:
        bad = np.nonzero((ra != rb) | (ia != ib))[0]
        assert bad.size == 0, f"{bad.size} coefficients differ, first at {bad[:5]}: {ra[bad[:3]]} vs {rb[bad[:3]]}"
    else:
        np.testing.assert_allclose(ra, rb, rtol=rtol, atol=atol)
        np.testing.assert_allclose(ia, ib, rtol=rtol, atol=atol)
