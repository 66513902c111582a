"""Generates the golden fixtures in tests/golden/ by running the reference
implementation (fastfermion) itself.

Run from the repository root in a container that holds the reference sources
and its built extension (``make -f oracle/ref.mk``):

    python tests/golden/make_golden.py [--ref /path/to/reference] [--only NAME]

Every fixture records the circuit as a flat gate table, the observable, the
propagation parameters and the reference's result: the full term set (in the
reference's serial iteration order) for small results, or a checksum of the
sorted term set for large ones, plus the expectation values.  The test-suite
only reads the .npz files; it never needs the reference at run time.
"""
import argparse
import hashlib
import importlib.util
import math
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from fastfermion_gb300 import workloads as W  # noqa: E402
from oracle.oracle import MAJORANA_GATE, PAULI_GATE  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
KIND = {"ROT": 0, "H": 1, "S": 2, "CNOT": 3, "SWAP": 4, "CZ": 5}
FULL_LIMIT = 20000  # store full term sets up to this many terms


def load_reference(ref):
    built = os.path.join(ROOT, "oracle", "_ref")
    spec = importlib.util.spec_from_file_location(
        "fastfermion", os.path.join(ref, "fastfermion", "__init__.py"),
        submodule_search_locations=[os.path.join(ref, "fastfermion"), built])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["fastfermion"] = mod
    spec.loader.exec_module(mod)
    return mod


# --------------------------------------------------------------------------
# conversions (reference objects -> flat arrays)
# --------------------------------------------------------------------------

def pauli_masks(ps):
    x = [0, 0]
    z = [0, 0]
    for pos, a in ps.indices():
        w, b = divmod(pos, 64)
        if a in "XY":
            x[w] |= 1 << b
        if a in "YZ":
            z[w] |= 1 << b
    return x, z


def maj_mask(ms):
    a = [0, 0, 0, 0]
    for pos in ms.indices():
        w, b = divmod(pos, 64)
        a[w] |= 1 << b
    return a


def pauli_table(circuit):
    g = np.zeros(len(circuit), dtype=PAULI_GATE)
    for i, gate in enumerate(circuit):
        name = type(gate).__name__
        g[i]["kind"] = KIND[name]
        if name == "ROT":
            x, z = pauli_masks(gate.axis)
            g[i]["x"] = x
            g[i]["z"] = z
            g[i]["theta"] = gate.theta
        else:
            q = list(gate.qubits)
            g[i]["q0"] = q[0]
            g[i]["q1"] = q[1] if len(q) > 1 else 0
    return g


def maj_table(circuit):
    g = np.zeros(len(circuit), dtype=MAJORANA_GATE)
    for i, gate in enumerate(circuit):
        g[i]["alpha"] = maj_mask(gate.axis)
        g[i]["theta"] = gate.theta
        g[i]["r"] = 0 if gate.axis.is_hermitian() else 1
    return g


def poly_arrays(poly, kind):
    items = list(poly.terms.items())
    n = len(items)
    keys = np.zeros((4, n), dtype=np.uint64)
    re = np.zeros(n)
    im = np.zeros(n)
    for i, (s, c) in enumerate(items):
        if kind == "pauli":
            x, z = pauli_masks(s)
            keys[:, i] = [x[0], x[1], z[0], z[1]]
        else:
            keys[:, i] = maj_mask(s)
        re[i] = c.real
        im[i] = c.imag
    return keys, re, im


def checksum(keys, re, im):
    """sha256 over the term set sorted by key; signed zeros are normalised."""
    order = np.lexsort(tuple(keys[w] for w in (3, 2, 1, 0)))
    k = np.ascontiguousarray(keys[:, order])
    r = re[order] + 0.0
    i = im[order] + 0.0
    h = hashlib.sha256()
    h.update(k.tobytes())
    h.update(np.ascontiguousarray(r).tobytes())
    h.update(np.ascontiguousarray(i).tobytes())
    return h.hexdigest()


# --------------------------------------------------------------------------
# case runners
# --------------------------------------------------------------------------

def mk(ff, spec):
    if spec[0] == "ROT":
        return ff.ROT(spec[1], list(spec[2]), spec[3])
    if spec[0] == "MROT":
        return ff.MROT(ff.MajoranaString(list(spec[1])), spec[2], spec[3])
    return getattr(ff, spec[0])(*spec[1:])


def save(name, **arrs):
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrs)


def pauli_case(ff, name, circuit, obs, states=((0, 0),), **kw):
    t0 = time.time()
    res = ff.propagate(circuit, obs, **kw)
    dt = time.time() - t0
    ok, ore, oim = poly_arrays(obs if hasattr(obs, "terms") else ff.PauliPolynomial(obs), "pauli")
    rk, rre, rim = poly_arrays(res, "pauli")
    ov = res.overlapwithzero()
    st = np.array([[b0, b1] for b0, b1 in states], dtype=np.uint64)
    sv = []
    for b0, b1 in states:
        up = [i for i in range(64) if (b0 >> i) & 1] + [64 + i for i in range(64) if (b1 >> i) & 1]
        sv.append(complex(ff.QubitProductState(up)(res)))
    arrs = dict(kind="pauli", gates=pauli_table(circuit), obs_keys=ok, obs_re=ore, obs_im=oim,
                maxdegree=kw.get("maxdegree") if kw.get("maxdegree") is not None else 128,
                mincoeff=kw.get("mincoeff") or 0.0, topk=kw.get("topk", 0),
                max_xweight=kw.get("max_xweight", -1), xtrunc_period=kw.get("xtrunc_period", 1),
                batched=kw.get("batched", True), n_terms=len(res),
                overlap=np.array([ov.real, ov.imag]), states=st,
                state_values=np.array([[v.real, v.imag] for v in sv]),
                checksum=checksum(rk, rre, rim), ref_seconds=dt)
    if len(res) <= FULL_LIMIT:
        arrs.update(res_keys=rk, res_re=rre, res_im=rim)
    save(name, **arrs)
    print(f"{name:32s} terms={len(res):8d} <O>={ov.real:+.15e} {dt:7.2f}s", flush=True)


def majorana_case(ff, name, circuit, obs, maxdegree=None, mincoeff=0.0, occs=((0, 0),)):
    t0 = time.time()
    res = ff.propagate(circuit, obs, maxdegree=maxdegree, mincoeff=mincoeff)
    dt = time.time() - t0
    ok, ore, oim = poly_arrays(obs, "majorana")
    rk, rre, rim = poly_arrays(res, "majorana")
    sv = []
    for b0, b1 in occs:
        occ = [i for i in range(64) if (b0 >> i) & 1] + [64 + i for i in range(64) if (b1 >> i) & 1]
        sv.append(complex(ff.FockState(occ)(res)))
    arrs = dict(kind="majorana", gates=maj_table(circuit), obs_keys=ok, obs_re=ore, obs_im=oim,
                has_maxdegree=maxdegree is not None, maxdegree=maxdegree or 0,
                mincoeff=mincoeff, n_terms=len(res),
                states=np.array([[b0, b1] for b0, b1 in occs], dtype=np.uint64),
                state_values=np.array([[v.real, v.imag] for v in sv]),
                checksum=checksum(rk, rre, rim), ref_seconds=dt)
    if len(res) <= FULL_LIMIT:
        arrs.update(res_keys=rk, res_re=rre, res_im=rim)
    save(name, **arrs)
    print(f"{name:32s} terms={len(res):8d} F={sv[0]:.12e} {dt:7.2f}s", flush=True)


# --------------------------------------------------------------------------
# circuits from the reference's own tests (test/omp_test.py, batched_test.py,
# sharded_test.py, pauli_circuit_test.py, majorana_circuit_test.py)
# --------------------------------------------------------------------------

def tfim(ff, n, dt):
    g = [ff.ROT("ZZ", [i, (i + 1) % n], -2 * dt) for i in range(n)]
    return g + [ff.ROT("X", [i], -2 * dt) for i in range(n)]


def heisenberg(ff, n, dt):
    g = []
    for i in range(n):
        j = (i + 1) % n
        g += [ff.ROT("XX", [i, j], 2 * dt), ff.ROT("YY", [i, j], 2 * dt), ff.ROT("ZZ", [i, j], 2 * dt)]
    return g


def random_pauli_circuit(ff, rng, qubits, ngates, p_clifford=0.3, wmax=3):
    out = []
    for _ in range(ngates):
        if rng.random() < p_clifford:
            name = ["H", "S", "CNOT", "SWAP", "CZ"][rng.integers(5)]
            if name in ("H", "S"):
                out.append(getattr(ff, name)(int(rng.choice(qubits))))
            else:
                i, j = rng.choice(qubits, size=2, replace=False)
                out.append(getattr(ff, name)(int(i), int(j)))
        else:
            w = int(rng.integers(1, wmax + 1))
            qs = sorted(int(q) for q in rng.choice(qubits, size=w, replace=False))
            ps = "".join("XYZ"[rng.integers(3)] for _ in qs)
            out.append(ff.ROT(ps, qs, float(rng.uniform(-math.pi, math.pi))))
    return out


def random_pauli_poly(ff, rng, qubits, nterms, complex_coef, wmax=3):
    p = ff.PauliPolynomial()
    for _ in range(nterms):
        w = int(rng.integers(1, wmax + 1))
        qs = sorted(int(q) for q in rng.choice(qubits, size=w, replace=False))
        s = ff.PauliString([(q, "XYZ"[rng.integers(3)]) for q in qs])
        c = complex(rng.normal(), rng.normal() if complex_coef else 0.0)
        p += ff.PauliPolynomial(s) * c
    return p


def random_maj_circuit(ff, rng, modes, ngates, dmax=4):
    out = []
    for _ in range(ngates):
        d = int(rng.integers(1, dmax + 1))
        supp = sorted(int(q) for q in rng.choice(modes, size=d, replace=False))
        herm = d % 4 in (0, 1)
        c = complex(rng.uniform(0.2, 1.5), 0.0) if herm else complex(0.0, rng.uniform(0.2, 1.5))
        out.append(ff.MROT(ff.MajoranaString(supp), c, float(rng.uniform(-1.5, 1.5))))
    return out


def random_maj_poly(ff, rng, modes, nterms, dmax=4):
    p = ff.MajoranaPolynomial()
    for _ in range(nterms):
        d = int(rng.integers(0, dmax + 1))
        supp = sorted(int(q) for q in rng.choice(modes, size=d, replace=False))
        p += ff.MajoranaPolynomial(supp, complex(rng.normal(), rng.normal()))
    return p


def cases(ff):
    P = ff.PauliString
    Z6 = P("Z" + "I" * 5)
    yield "ref_tfim", lambda: pauli_case(ff, "ref_tfim", tfim(ff, 6, 0.1) * 5, Z6)
    yield "ref_tfim_unbatched", lambda: pauli_case(ff, "ref_tfim_unbatched", tfim(ff, 6, 0.1) * 5, Z6, batched=False)
    yield "ref_tfim_threshold", lambda: pauli_case(ff, "ref_tfim_threshold", tfim(ff, 6, 0.1) * 5, Z6, mincoeff=1e-3)
    yield "ref_tfim_threshold_unbatched", lambda: pauli_case(ff, "ref_tfim_threshold_unbatched", tfim(ff, 6, 0.1) * 5, Z6, mincoeff=1e-3, batched=False)
    yield "ref_tfim_maxdegree", lambda: pauli_case(ff, "ref_tfim_maxdegree", tfim(ff, 6, 0.1) * 5, Z6, maxdegree=3)
    yield "ref_heisenberg", lambda: pauli_case(ff, "ref_heisenberg", heisenberg(ff, 4, 0.03) * 5, P("ZIII"))
    mixed = [ff.H(0), ff.ROT("Z", (0,), 0.5), ff.CNOT(0, 1), ff.ROT("XX", [0, 1], 0.3)]
    yield "ref_mixed_clifford", lambda: pauli_case(ff, "ref_mixed_clifford", mixed * 5, P("ZI"))
    yield "ref_mixed_clifford_unbatched", lambda: pauli_case(ff, "ref_mixed_clifford_unbatched", mixed * 5, P("ZI"), batched=False)
    yield "ref_polynomial_obs", lambda: pauli_case(
        ff, "ref_polynomial_obs", tfim(ff, 4, 0.05) * 10,
        ff.PauliPolynomial(P("ZI")) + ff.PauliPolynomial(P("IZ")))
    yield "ref_single_gate", lambda: pauli_case(ff, "ref_single_gate", [ff.ROT("X", (0,), 0.3)], P("Z"))
    yield "ref_empty_circuit", lambda: pauli_case(ff, "ref_empty_circuit", [], P("Z"))
    yield "ref_identity_rotation", lambda: pauli_case(ff, "ref_identity_rotation", [ff.ROT("X", (0,), 0.0)] * 10, P("Z"))
    yield "ref_all_commuting", lambda: pauli_case(ff, "ref_all_commuting", [ff.ROT("ZZ", [0, 1], 0.3)] * 10, P("ZI"))
    yield "ref_clifford_only", lambda: pauli_case(ff, "ref_clifford_only", [ff.H(0), ff.CNOT(0, 1)], P("ZI"))
    yield "ref_x_batch", lambda: pauli_case(ff, "ref_x_batch", [ff.ROT("X", [i], 0.1) for i in range(6)] * 3, Z6)
    yield "ref_no_commuting", lambda: pauli_case(ff, "ref_no_commuting", [ff.ROT("ZZ", [i, (i + 1) % 4], 0.1) for i in range(4)] * 3, P("ZIII"))
    # exact zeros stay in the term set (mincoeff = 0)
    yield "exact_zero_kept", lambda: pauli_case(ff, "exact_zero_kept", [ff.ROT("X", [0], 0.3), ff.ROT("X", [0], -0.3)], P("Z"), batched=False)
    # maxdegree filters only emitted partners; heavy terms stay
    yield "maxdegree_keeps_heavy", lambda: pauli_case(ff, "maxdegree_keeps_heavy", [ff.ROT("X", [5], 0.4)], P("ZZZZ"), maxdegree=2)
    # pauli_circuit_test.py:53-92 circuits x observables
    circs = [[ff.H(0)], [ff.S(0)], [ff.CNOT(0, 1)],
             [ff.H(0), ff.CNOT(0, 1), ff.S(1), ff.CNOT(1, 2), ff.H(2)],
             [ff.ROT("I", 0.3)], [ff.ROT("XX", 0.34)],
             [ff.H(0), ff.CNOT(0, 1), ff.ROT("XY", 0.23), ff.ROT("ZZ", 0.78), ff.S(1), ff.CNOT(1, 2), ff.H(2)]]
    obss = ["X0 Z1", "X0Z1Y2", "-Z2+3*X0"]
    for ci, c in enumerate(circs):
        for oi, o in enumerate(obss):
            nm = f"ref_circuit_{ci}_{oi}"
            yield nm, (lambda nm=nm, c=c, o=o: pauli_case(ff, nm, c, ff.poly(o)))
    # the benchmark configurations (16-qubit chain, 10x10 kicked Ising)
    yield "cfg1_chain", lambda: pauli_case(ff, "cfg1_chain", [mk(ff, s) for s in W.chain_circuit()], P("Z7"), maxdegree=6, mincoeff=1e-8, states=((0, 0), (0b1010110011, 0)))
    yield "cfg1_chain_unbatched", lambda: pauli_case(ff, "cfg1_chain_unbatched", [mk(ff, s) for s in W.chain_circuit()], P("Z7"), maxdegree=6, mincoeff=1e-8, batched=False)
    for th in W.KICKED_ISING_THETAS:
        nm = "cfg2_kicked_ising_%s" % ("%.4f" % th).replace(".", "p")
        yield nm, (lambda nm=nm, th=th: pauli_case(
            ff, nm, [mk(ff, s) for s in W.kicked_ising_circuit(th)], P([(55, "Z")]),
            maxdegree=8, mincoeff=1e-6))
    # the large-N variant: W = 10 (peak ~4e8 terms inside a batch; ~15 min on 8 cores)
    yield "cfg2w10_kicked_ising_0p3000", lambda: pauli_case(
        ff, "cfg2w10_kicked_ising_0p3000", [mk(ff, s) for s in W.kicked_ising_circuit(0.3)], P([(55, "Z")]),
        maxdegree=10, mincoeff=1e-6, n_threads=os.cpu_count(), parallel="sharded")
    # smaller kicked-Ising variants with large in-batch growth
    yield "ki_6x6_w6", lambda: pauli_case(ff, "ki_6x6_w6", [mk(ff, s) for s in W.kicked_ising_circuit(0.7, 6, 6, 8)], P([(21, "Z")]), maxdegree=6, mincoeff=1e-5)
    yield "ki_8x8_w6_unbatched", lambda: pauli_case(ff, "ki_8x8_w6_unbatched", [mk(ff, s) for s in W.kicked_ising_circuit(0.4, 8, 8, 6)], P([(27, "Z")]), maxdegree=6, mincoeff=1e-5, batched=False)
    # su4 example (examples/pauli_propagation.py with maxdegree as a keyword)
    def su4():
        sys.path.insert(0, os.path.join(REF, "examples"))
        from common import read_circuit
        c = read_circuit(os.path.join(REF, "examples", "data", "su4circuit-16.txt"))
        pauli_case(ff, "su4_example", c, ff.poly("Z15"), maxdegree=4)
    yield "su4_example", su4
    # randomised circuits: every gate type, words 0 and 1, complex coefficients,
    # truncation rules
    rng = np.random.default_rng(20261203)
    small = list(range(6))
    wide = [0, 1, 2, 61, 62, 63, 64, 65, 66, 125, 126, 127]
    for r in range(24):
        qs = small if r % 2 == 0 else wide
        cplx = r % 3 == 0
        kw = {}
        if r % 4 == 1:
            kw["maxdegree"] = 3
        if r % 5 == 2:
            kw["mincoeff"] = 1e-3
        if r % 6 == 3:
            kw["max_xweight"] = 2
            kw["xtrunc_period"] = 1 + r % 3
        if r % 7 == 4:
            kw["batched"] = False
        if r % 8 == 5:
            kw["topk"] = 40
        circ = random_pauli_circuit(ff, rng, qs, 40 + 5 * r)
        obs = random_pauli_poly(ff, rng, qs, 1 + r % 5, cplx)
        nm = f"rand_pauli_{r:02d}"
        yield nm, (lambda nm=nm, circ=circ, obs=obs, kw=kw: pauli_case(ff, nm, circ, obs, states=((0, 0), (0b101, 1 << 62)), **kw))
    # Majorana: reference tests
    mc = [ff.MROT(ff.MajoranaString([0, 2]), 0.2j, 0.1), ff.MROT(ff.MajoranaString([0, 1, 2, 3]), 0.3, 0.1)]
    for oi, o in enumerate(["m0 m1", "-m1 + m0m2", "-1j*m2 + 2.1 m1 m0"]):
        nm = f"ref_majorana_{oi}"
        yield nm, (lambda nm=nm, o=o: majorana_case(ff, nm, mc, ff.poly(o), occs=((0, 0), (0b1, 0), (0b11, 0))))
    # random Majorana circuits (odd/even degree, r = 0/1, wide indices)
    for r in range(12):
        modes = list(range(8)) if r % 2 == 0 else [0, 1, 2, 3, 62, 63, 64, 65, 126, 127, 128, 129, 200, 201, 254, 255]
        circ = random_maj_circuit(ff, rng, modes, 30 + 4 * r)
        obs = random_maj_poly(ff, rng, modes, 1 + r % 4)
        md = 4 if r % 3 == 1 else None
        mcf = 1e-3 if r % 4 == 2 else 0.0
        nm = f"rand_majorana_{r:02d}"
        yield nm, (lambda nm=nm, circ=circ, obs=obs, md=md, mcf=mcf: majorana_case(ff, nm, circ, obs, maxdegree=md, mincoeff=mcf, occs=((0, 0), (0b1011, 0), (1 << 63, 1))))
    # Fermi-Hubbard (config 3 family)
    def hub(nm, lx, ly, steps, md, mcf):
        c = [mk(ff, s) for s in W.hubbard_circuit(lx, ly, steps=steps)]
        obs = ff.MajoranaPolynomial([], 0.5) + ff.MajoranaPolynomial([0, 1], 0.5j)
        majorana_case(ff, nm, c, obs, maxdegree=md, mincoeff=mcf, occs=((0, 0), (0b0110100101, 0)))
    yield "hubbard_3x3", lambda: hub("hubbard_3x3", 3, 3, 10, 6, 1e-7)
    yield "hubbard_6x6_2steps", lambda: hub("hubbard_6x6_2steps", 6, 6, 2, 6, 1e-7)
    yield "hubbard_6x6_3steps", lambda: hub("hubbard_6x6_3steps", 6, 6, 3, 6, 1e-7)
    # the full 6x6 Hubbard workload: 10 steps, ~1.2e7 final terms, minutes on the reference
    yield "hubbard_6x6_10steps", lambda: hub("hubbard_6x6_10steps", 6, 6, 10, 6, 1e-7)


def obs_from_arrays(ff, keys, re):
    """Reference PauliPolynomial of the terms keys (4, m) / re (m,)."""
    p = ff.PauliPolynomial()
    for t in range(re.size):
        x = int(keys[0, t]) | (int(keys[1, t]) << 64)
        z = int(keys[2, t]) | (int(keys[3, t]) << 64)
        ops = []
        for q in range(128):
            a, b = (x >> q) & 1, (z >> q) & 1
            if a or b:
                ops.append((q, "X" if a and not b else ("Y" if a else "Z")))
        p += ff.PauliPolynomial(ff.PauliString(ops)) * float(re[t])
    return p


def hea_instance_circuit(ff, n, layers, th):
    spec = W.hea_circuit(n, layers)
    out, r = [], 0
    for s in spec:
        if s[0] == "ROT":
            out.append(ff.ROT(s[1], list(s[2]), float(th[r])))
            r += 1
        else:
            out.append(mk(ff, s))
    return out


def hea_cases(ff):
    """Batched-ansatz workload (256 instances x 50 qubits, 8 layers, W=6,
    tau=1e-7): instances 0 and 1 run alone through the reference, and
    parameter-shift derivatives of a small ansatz from the reference."""
    thetas, obs = W.hea_instances(256)
    for i in (0, 1):
        nm = f"hea_50q_inst{i}"
        yield nm, (lambda nm=nm, i=i: pauli_case(ff, nm, hea_instance_circuit(ff, 50, 8, thetas[i]),
                                                  obs_from_arrays(ff, *obs[i]), maxdegree=6, mincoeff=1e-7))

    def shift(nm, n, layers, ninst, seed, maxdegree, batched):
        th, ob = W.hea_instances(ninst, n=n, layers=layers, seed=seed, max_terms=6, max_weight=3)
        t0 = time.time()
        f = np.zeros(ninst)
        g = np.zeros_like(th)
        for i in range(ninst):
            o = obs_from_arrays(ff, *ob[i])

            def ev(t):
                return ff.propagate(hea_instance_circuit(ff, n, layers, t), o, maxdegree=maxdegree,
                                    batched=batched).overlapwithzero().real
            f[i] = ev(th[i])
            for r in range(th.shape[1]):
                tp, tm = th[i].copy(), th[i].copy()
                tp[r] += math.pi / 2
                tm[r] -= math.pi / 2
                g[i, r] = 0.5 * (ev(tp) - ev(tm))
        keys = np.concatenate([o[0] for o in ob], axis=1)
        re = np.concatenate([o[1] for o in ob])
        off = np.cumsum([0] + [o[1].size for o in ob]).astype(np.int64)
        save(nm, kind="hea_shift", n=n, layers=layers, seed=seed, maxdegree=maxdegree, batched=batched,
             thetas=th, obs_keys=keys, obs_re=re, offsets=off, expect=f, shift_grad=g)
        print(f"{nm:32s} ninst={ninst} angles={th.shape[1]} {time.time() - t0:7.2f}s", flush=True)
    yield "hea_shift_10q", lambda: shift("hea_shift_10q", 10, 3, 3, 7, 4, True)
    yield "hea_shift_10q_unbatched", lambda: shift("hea_shift_10q_unbatched", 10, 3, 2, 8, 5, False)
    yield "hea_shift_70q", lambda: shift("hea_shift_70q", 70, 2, 2, 9, 3, True)


def transform_cases(ff):
    """Jordan-Wigner maps of random Majorana polynomials and sparse matrices of
    Pauli polynomials, by the reference (kinds "jw" and "sparse")."""
    rng = np.random.default_rng(777)

    def jw_case(nm, modes, nterms, dmax):
        p = random_maj_poly(ff, rng, modes, nterms, dmax)
        ok, ore, oim = poly_arrays(p, "majorana")
        res = ff.jw(p)
        rk, rre, rim = poly_arrays(res, "pauli")
        save(nm, kind="jw", obs_keys=ok, obs_re=ore, obs_im=oim, res_keys=rk, res_re=rre, res_im=rim)
        print(f"{nm:32s} terms={len(res):8d}", flush=True)
    yield "jw_small", lambda: jw_case("jw_small", list(range(12)), 40, 5)
    yield "jw_wide", lambda: jw_case("jw_wide", [0, 1, 62, 63, 64, 65, 127, 128, 129, 200, 201, 254, 255], 60, 6)

    def sparse_case(nm, poly, n):
        ok, ore, oim = poly_arrays(poly, "pauli")
        m = poly.sparse(n)
        save(nm, kind="sparse", n=n, obs_keys=ok, obs_re=ore, obs_im=oim, indptr=m.indptr.astype(np.int64),
             indices=m.indices.astype(np.int64), data=np.asarray(m.data, dtype=complex))
        print(f"{nm:32s} nnz={m.nnz:8d}", flush=True)
    yield "sparse_random6", lambda: sparse_case("sparse_random6", random_pauli_poly(ff, rng, list(range(6)), 40, True, 4), 6)
    yield "sparse_propagated", lambda: sparse_case(
        "sparse_propagated", ff.propagate(tfim(ff, 6, 0.1) * 5, ff.PauliString("Z" + "I" * 5)), 6)
    yield "sparse_dropped_qubits", lambda: sparse_case("sparse_dropped_qubits", random_pauli_poly(ff, rng, list(range(7)), 25, True, 3), 5)


REF = os.environ.get("FFG_REFERENCE_SRC", "/root/reference")

if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=REF)
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    REF = a.ref
    ff = load_reference(REF)
    for name, fn in list(cases(ff)) + list(hea_cases(ff)) + list(transform_cases(ff)):
        if a.only and a.only not in name:
            continue
        fn()
