"""Synthetic circuits for the propagation workloads (gate specifications only).

Each generator returns a list of plain tuples so that the same circuit can be
instantiated with this package's gate classes (``build_circuit``) or with any
other implementation of the same gate types:

* ``("ROT", paulis, qubits, theta)``   Pauli rotation exp(-i theta/2 P)
* ``("H", q)``, ``("S", q)``, ``("CNOT", i, j)``, ``("SWAP", i, j)``, ``("CZ", i, j)``
* ``("MROT", support, coeff, t)``      Majorana rotation exp(-i t/2 coeff*gamma_S)

There is no dataset: every circuit is generated from its parameters and a seed.
"""
import math

import numpy as np


def chain_circuit(n=16, layers=10, seed=0, hi=math.pi / 8):
    """16-qubit open chain: per layer RZZ(theta) on bonds (i, i+1), then RX(phi) on
    every qubit; angles drawn in gate order from default_rng(seed).uniform(0, hi)."""
    ngates = layers * ((n - 1) + n)
    ang = np.random.default_rng(seed).uniform(0.0, hi, size=ngates)
    out, a = [], 0
    for _ in range(layers):
        for i in range(n - 1):
            out.append(("ROT", "ZZ", [i, i + 1], float(ang[a])))
            a += 1
        for i in range(n):
            out.append(("ROT", "X", [i], float(ang[a])))
            a += 1
    return out


def lattice_edges(lx=10, ly=10):
    """Open lx-by-ly square lattice, site index 10*x + y style (ly*x + y): the
    (x,y)-(x+1,y) edges first, then the (x,y)-(x,y+1) edges."""
    edges = []
    for x in range(lx - 1):
        for y in range(ly):
            edges.append((ly * x + y, ly * (x + 1) + y))
    for x in range(lx):
        for y in range(ly - 1):
            edges.append((ly * x + y, ly * x + y + 1))
    return edges


def kicked_ising_circuit(theta_h, lx=10, ly=10, steps=20, theta_zz=-math.pi / 2):
    """Kicked Ising: each step RZZ(theta_zz) on all lattice edges, then RX(theta_h)
    on every site."""
    edges = lattice_edges(lx, ly)
    step = [("ROT", "ZZ", [i, j], theta_zz) for i, j in edges]
    step += [("ROT", "X", [q], theta_h) for q in range(lx * ly)]
    return step * steps


KICKED_ISING_THETAS = (0.1, 0.3, 0.5, 0.7, 0.9, 1.1, math.pi / 2)


def learned_correction_thetas(seed=2024):
    """theta_h values of the learned-correction workload on the 10x10 kicked
    Ising circuit: a seeded training grid of 64 values in [0.05, pi/2] (64
    equal cells, one uniform draw in each) and 16 held-out values drawn
    uniformly from the same range."""
    rng = np.random.default_rng(seed)
    lo, hi = 0.05, math.pi / 2
    edges = np.linspace(lo, hi, 65)
    train = edges[:-1] + rng.uniform(0.0, 1.0, 64) * np.diff(edges)
    held = np.sort(rng.uniform(lo, hi, 16))
    return [float(t) for t in train], [float(t) for t in held]


def hubbard_step(lx=6, ly=6, t=1.0, u=4.0, dt=0.1):
    """One Trotter step of the spinful 2D Fermi-Hubbard model in Majorana form.

    Majorana index 4*site + 2*sigma + {0,1}, site = ly*x + y.  Hopping on the
    horizontal bonds, then the vertical bonds (for each bond and spin the
    normal-ordered strings of -0.5i*t*g_{4i+2s} g_{4j+2s+1} and
    -0.5i*t*g_{4j+2s} g_{4i+2s+1}), then per site the non-identity terms of
    0.25*U*(1 + i g0 g1)(1 + i g2 g3).  Every term becomes MROT(S, coeff, 2*dt).
    """
    def site(x, y):
        return ly * x + y

    horiz = [(site(x, y), site(x + 1, y)) for x in range(lx - 1) for y in range(ly)]
    vert = [(site(x, y), site(x, y + 1)) for x in range(lx) for y in range(ly - 1)]
    gates = []
    for i, j in horiz + vert:
        for s in (0, 1):
            for a, b in ((4 * i + 2 * s, 4 * j + 2 * s + 1), (4 * j + 2 * s, 4 * i + 2 * s + 1)):
                c = complex(0.0, -0.5 * t)
                if a > b:  # g_a g_b = -g_b g_a
                    a, b, c = b, a, -c
                gates.append(("MROT", [a, b], c, 2 * dt))
    if u != 0:
        for s in range(lx * ly):
            b0 = 4 * s
            gates.append(("MROT", [b0, b0 + 1], complex(0.0, 0.25 * u), 2 * dt))
            gates.append(("MROT", [b0 + 2, b0 + 3], complex(0.0, 0.25 * u), 2 * dt))
            gates.append(("MROT", [b0, b0 + 1, b0 + 2, b0 + 3], complex(-0.25 * u, 0.0), 2 * dt))
    return gates


def hubbard_circuit(lx=6, ly=6, t=1.0, u=4.0, dt=0.1, steps=10):
    return hubbard_step(lx, ly, t, u, dt) * steps


def hea_circuit(n=50, layers=8, theta=0.0):
    """Hardware-efficient ansatz on an open chain: per layer RY(theta) on every
    qubit, then CZ on the bonds (i, i+1).  Per-instance angles replace theta
    (row i of ``hea_instances``' thetas, ROT gates in circuit order)."""
    out = []
    for _ in range(layers):
        out += [("ROT", "Y", [q], theta) for q in range(n)]
        out += [("CZ", q, q + 1) for q in range(n - 1)]
    return out


def hea_instances(ninst=256, n=50, layers=8, seed=0, max_terms=64, max_weight=4):
    """Seeded instances of the batched ansatz workload: angles (ninst, layers*n)
    from uniform[-pi, pi], and one observable per instance with a term count
    drawn from 1..max_terms, each term a distinct random Pauli string of weight
    1..max_weight on random qubits with an N(0, 1) coefficient.

    Returns (thetas, [(keys (4, m) uint64, re (m,)) per instance])."""
    rng = np.random.default_rng(seed)
    thetas = rng.uniform(-math.pi, math.pi, size=(ninst, layers * n))
    obs = []
    for _ in range(ninst):
        m = int(rng.integers(1, max_terms + 1))
        seen = set()
        keys = np.zeros((4, m), dtype=np.uint64)
        re = rng.normal(size=m)
        t = 0
        while t < m:
            w = int(rng.integers(1, max_weight + 1))
            qs = rng.choice(n, size=w, replace=False)
            x = z = 0
            for q in qs:
                p = int(rng.integers(1, 4))  # 1 X, 2 Y, 3 Z
                if p in (1, 2):
                    x |= 1 << int(q)
                if p in (2, 3):
                    z |= 1 << int(q)
            if (x, z) in seen:
                continue
            seen.add((x, z))
            keys[0, t], keys[1, t] = x & (2**64 - 1), x >> 64
            keys[2, t], keys[3, t] = z & (2**64 - 1), z >> 64
            t += 1
        obs.append((keys, re))
    return thetas, obs
