"""ctypes wrapper around the C oracle (oracle/ffo.c).

TEST INFRASTRUCTURE ONLY: imported by the test-suite, by the smoke check and by
the CPU-baseline leg of bench.py, never by the fastfermion_gb300 package.

Gate tables use the numpy dtypes below; they have the same memory layout as the
structs in oracle/ffo.h.  Keys are uint64 arrays of shape (4, n).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libffo.so")

PAULI_GATE = np.dtype([("kind", "<i4"), ("q0", "<i4"), ("q1", "<i4"), ("pad", "<i4"),
                       ("x", "<u8", (2,)), ("z", "<u8", (2,)), ("theta", "<f8")])
MAJORANA_GATE = np.dtype([("alpha", "<u8", (4,)), ("theta", "<f8"), ("r", "<i4"), ("pad", "<i4")])
ROT, H, S, CNOT, SWAP, CZ = range(6)


class _Params(ctypes.Structure):
    _fields_ = [("maxdegree", ctypes.c_int32), ("topk", ctypes.c_int32),
                ("mincoeff", ctypes.c_double), ("max_xweight", ctypes.c_int32),
                ("xtrunc_period", ctypes.c_int32), ("batched", ctypes.c_int32),
                ("n_threads", ctypes.c_int32)]


def build(force=False):
    """Compile libffo.so from ffo.c (gcc, OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "ffo.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           src, "-o", LIB, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i64, dp = ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)
        L.ffo_pauli_propagate.restype = vp
        L.ffo_pauli_propagate.argtypes = [vp, i64, vp, vp, vp, i64, ctypes.POINTER(_Params)]
        L.ffo_majorana_propagate.restype = vp
        L.ffo_majorana_propagate.argtypes = [vp, i64, vp, vp, vp, i64, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_double]
        for f in ("ffo_size", "ffo_apps", "ffo_peak"):
            getattr(L, f).restype = i64
            getattr(L, f).argtypes = [vp]
        L.ffo_copy.argtypes = [vp, vp, vp, vp]
        L.ffo_free.argtypes = [vp]
        L.ffo_overlapwithzero.argtypes = [vp, dp, dp]
        L.ffo_qubit_state.argtypes = [vp, vp, dp, dp]
        L.ffo_fock_state.argtypes = [vp, vp, dp, dp]
        L.ffo_abs.restype = ctypes.c_double
        L.ffo_abs.argtypes = [ctypes.c_double, ctypes.c_double]
        L.ffo_pauli_propagate_capture.restype = vp
        L.ffo_pauli_propagate_capture.argtypes = [vp, i64, vp, vp, vp, i64, ctypes.POINTER(_Params),
                                                  ctypes.c_int32, ctypes.POINTER(vp)]
        L.ffo_pauli_propagate_masked.restype = vp
        L.ffo_pauli_propagate_masked.argtypes = [vp, i64, vp, vp, vp, i64, ctypes.POINTER(_Params), vp]
        L.ffo_drops_size.restype = i64
        L.ffo_drops_size.argtypes = [vp]
        L.ffo_drops_copy.argtypes = [vp, vp, vp, vp, vp]
        L.ffo_drops_free.argtypes = [vp]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None and a.size else None


class OraclePoly:
    """Result of an oracle propagation: keys (4, n), re, im in iteration order."""

    def __init__(self, handle):
        L = lib()
        self.h = handle
        n = L.ffo_size(handle)
        self.keys = np.zeros((4, n), dtype=np.uint64)
        self.re = np.zeros(n)
        self.im = np.zeros(n)
        if n:
            L.ffo_copy(handle, _ptr(self.keys), _ptr(self.re), _ptr(self.im))
        self.apps = L.ffo_apps(handle)
        self.peak = L.ffo_peak(handle)

    def __len__(self):
        return self.re.size

    def _pair(self, fn, *args):
        r, i = ctypes.c_double(), ctypes.c_double()
        fn(self.h, *args, ctypes.byref(r), ctypes.byref(i))
        return complex(r.value, i.value)

    def overlapwithzero(self):
        return self._pair(lib().ffo_overlapwithzero)

    def qubit_state(self, b0=0, b1=0):
        b = np.array([b0, b1], dtype=np.uint64)
        return self._pair(lib().ffo_qubit_state, _ptr(b))

    def fock_state(self, b0=0, b1=0):
        b = np.array([b0, b1], dtype=np.uint64)
        return self._pair(lib().ffo_fock_state, _ptr(b))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ffo_free(self.h)
            self.h = None


def pauli_propagate(gates, keys, re, im=None, maxdegree=128, mincoeff=0.0, topk=0,
                    max_xweight=-1, xtrunc_period=1, batched=True, n_threads=1, active=None):
    """active: None, or a uint64 mask over the rotations (bit r of word r // 64
    set = the r-th ROT gate in circuit order acts; the others are skipped, the
    batching and truncation points stay those of the whole circuit)."""
    gates = np.ascontiguousarray(gates, dtype=PAULI_GATE)
    keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
    re = np.ascontiguousarray(re, dtype=np.float64)
    im = None if im is None else np.ascontiguousarray(im, dtype=np.float64)
    p = _Params(int(maxdegree), int(topk), float(mincoeff), int(max_xweight),
                int(xtrunc_period), int(bool(batched)), int(n_threads))
    if active is not None:
        nrot = int(np.count_nonzero(gates["kind"] == ROT))
        active = np.ascontiguousarray(active, dtype=np.uint64).reshape(-1)
        assert active.size >= max(1, (nrot + 63) // 64)
        h = lib().ffo_pauli_propagate_masked(_ptr(gates), gates.size, _ptr(keys), _ptr(re), _ptr(im),
                                             re.size, ctypes.byref(p), _ptr(active))
    else:
        h = lib().ffo_pauli_propagate(_ptr(gates), gates.size, _ptr(keys), _ptr(re), _ptr(im),
                                      re.size, ctypes.byref(p))
    if not h:
        raise ValueError("oracle rejected the circuit")
    return OraclePoly(h)


class Dropped:
    """Partners dropped by the degree filter: keys (4, m), re, im and gate (the
    index of the gate that created each one; gates [0, gate) remain)."""

    def __init__(self, keys, re, im, gate):
        self.keys, self.re, self.im, self.gate = keys, re, im, gate

    def __len__(self):
        return self.re.size


def pauli_propagate_capture(gates, keys, re, im=None, capdeg=128, maxdegree=128, mincoeff=0.0, topk=0,
                            max_xweight=-1, xtrunc_period=1, batched=True):
    """Serial propagation that also returns the partners dropped by the degree
    filter with degree in (maxdegree, capdeg]: (OraclePoly, Dropped)."""
    L = lib()
    gates = np.ascontiguousarray(gates, dtype=PAULI_GATE)
    keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
    re = np.ascontiguousarray(re, dtype=np.float64)
    im = None if im is None else np.ascontiguousarray(im, dtype=np.float64)
    p = _Params(int(maxdegree), int(topk), float(mincoeff), int(max_xweight),
                int(xtrunc_period), int(bool(batched)), 1)
    d = ctypes.c_void_p()
    h = L.ffo_pauli_propagate_capture(_ptr(gates), gates.size, _ptr(keys), _ptr(re), _ptr(im),
                                      re.size, ctypes.byref(p), int(capdeg), ctypes.byref(d))
    if not h:
        raise ValueError("oracle rejected the circuit")
    m = L.ffo_drops_size(d)
    dk = np.zeros((4, m), dtype=np.uint64)
    dre, dim, dg = np.zeros(m), np.zeros(m), np.zeros(m, dtype=np.int64)
    if m:
        L.ffo_drops_copy(d, _ptr(dk), _ptr(dre), _ptr(dim), _ptr(dg))
    L.ffo_drops_free(d)
    return OraclePoly(h), Dropped(dk, dre, dim, dg)


def majorana_propagate(gates, keys, re, im=None, maxdegree=None, mincoeff=0.0):
    gates = np.ascontiguousarray(gates, dtype=MAJORANA_GATE)
    keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(4, -1)
    re = np.ascontiguousarray(re, dtype=np.float64)
    im = None if im is None else np.ascontiguousarray(im, dtype=np.float64)
    h = lib().ffo_majorana_propagate(_ptr(gates), gates.size, _ptr(keys), _ptr(re), _ptr(im),
                                     re.size, int(maxdegree is not None),
                                     int(maxdegree or 0), float(mincoeff))
    return OraclePoly(h)


def ffo_abs(re, im):
    return lib().ffo_abs(float(re), float(im))


# ---------------------------------------------------------------------------
# Conversions (pure Python restatements; small inputs only)
# ---------------------------------------------------------------------------

def _popc(v):
    return bin(v).count("1")


def _ipow(m):
    return (1 + 0j, 1j, -1 + 0j, -1j)[m % 4]


def jordan_wigner(keys, re, im=None):
    """Jordan-Wigner map of Majorana terms (keys (4, n), re, im) to Pauli terms
    (src/transforms.h:124-151): index i = 2j + r maps to Z_0..Z_{j-1} X_j (r = 0)
    or Z_0..Z_{j-1} Y_j (r = 1), multiplied in increasing index order with the
    phase bookkeeping of pauli_string_multiply (src/pauli/algebra.h:227-233);
    coefficient v * i^jpow; exact zeros dropped (compress(0)).  Returns
    (keys (4, m) uint64, re, im) in input order."""
    keys = np.asarray(keys, dtype=np.uint64).reshape(4, -1)
    re = np.asarray(re, dtype=np.float64)
    im = np.zeros_like(re) if im is None else np.asarray(im, dtype=np.float64)
    ok, ore, oim = [], [], []
    for t in range(re.size):
        a = sum(int(keys[w, t]) << (64 * w) for w in range(4))
        x = z = 0
        jpow = 0
        i = 0
        while a >> i:
            if (a >> i) & 1:
                j, r = divmod(i, 2)
                bx = 1 << j
                bz = (1 << (j + r)) - 1
                jpow += _popc(x & z) + _popc(bx & bz) + 2 * _popc(z & bx)
                x ^= bx
                z ^= bz
                jpow -= _popc(x & z)
            i += 1
        v = complex(re[t], im[t])
        p = _ipow(jpow)
        c = complex(v.real * p.real - v.imag * p.imag, v.real * p.imag + v.imag * p.real)
        c = complex(0.0 + c.real, 0.0 + c.imag)
        if c.real == 0.0 and c.imag == 0.0:
            continue
        m64 = (1 << 64) - 1
        ok.append([x & m64, x >> 64, z & m64, z >> 64])
        ore.append(c.real)
        oim.append(c.imag)
    k = np.array(ok, dtype=np.uint64).T.reshape(4, -1) if ok else np.zeros((4, 0), dtype=np.uint64)
    return k, np.array(ore), np.array(oim)


def pauli_sparse(keys, re, im, n):
    """CSC arrays (indptr, indices, data) of the 2^n x 2^n matrix of a Pauli
    polynomial (src/pauli/sparse.h:20-131): qubit q maps to bit n-1-q of the
    basis index (qubits >= n ignored); terms grouped by the flipped X mask in
    increasing order; column b gets, per group, the entry at row b ^ xf with
    value sum_t (-1)^|b & zf_t| i^{#Y_t} c_t when it is not zero.  Ties inside a
    group are summed in increasing flipped-Z order, then term order."""
    keys = np.asarray(keys, dtype=np.uint64).reshape(4, -1)

    def flip(v):
        r = 0
        for q in range(n):
            if (v >> q) & 1:
                r |= 1 << (n - 1 - q)
        return r
    mask = (1 << n) - 1
    terms = []
    for t in range(keys.shape[1]):
        x0, x1, z0, z1 = (int(keys[w, t]) for w in range(4))
        ny = _popc(x0 & z0) + _popc(x1 & z1)
        p = _ipow(ny)
        v = complex(re[t], im[t])
        c = complex(p.real * v.real - p.imag * v.imag, p.real * v.imag + p.imag * v.real)
        terms.append((flip(x0 & mask), flip(z0 & mask), c))
    terms.sort(key=lambda u: (u[0], u[1]))
    groups = []
    for xf, zf, c in terms:
        if groups and groups[-1][0] == xf:
            groups[-1][1].append((zf, c))
        else:
            groups.append((xf, [(zf, c)]))
    indptr = [0]
    indices, data = [], []
    for b in range(1 << n):
        for xf, members in groups:
            sr = si = 0.0
            for zf, c in members:
                sg = -1.0 if _popc(b & zf) & 1 else 1.0
                sr += sg * c.real
                si += sg * c.imag
            if sr != 0.0 or si != 0.0:
                indices.append(b ^ xf)
                data.append(complex(sr, si))
        indptr.append(len(indices))
    return np.array(indptr, dtype=np.int64), np.array(indices, dtype=np.int64), np.array(data, dtype=complex)
