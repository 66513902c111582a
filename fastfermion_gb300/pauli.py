"""Pauli strings, Pauli polynomials, Pauli gates and product states.

Same names, constructors and conventions as fastfermion's Python API for these
types (src/python_bind.cpp:590-700, src/pauli/algebra.h, src/pauli/gates.h,
src/qubitproductstate.h): two bits per qubit, I=(0,0) X=(1,0) Y=(1,1)
Z=(0,1) in (xory, yorz); at most 128 qubits; errors raise RuntimeError.

A PauliPolynomial returned by ``propagate`` keeps its terms on the GPU and
copies them to the host only when they are inspected; its expectation values
are computed on the device.
"""
import cmath
import math
import numbers

import numpy as np

MAX_QUBITS = 128
_MASK = (1 << MAX_QUBITS) - 1


def _popc(v):
    return bin(v).count("1")


def _ipow(m):
    return (1 + 0j, 1j, -1 + 0j, -1j)[m & 3]


def _check_loc(loc):
    if not (0 <= loc < MAX_QUBITS):
        raise RuntimeError(f"Invalid PauliString (qubit index {loc} invalid, should be between 0 "
                           f"and {MAX_QUBITS - 1})")


def _parse_indexed(s):
    """'X0 Z1 Y4' (spaces or '*' between factors) -> [(0,'X'), (1,'Z'), (4,'Y')]"""
    if s in ("I", "1"):
        return []
    out, i, n = [], 0, len(s)
    while i < n:
        if i > 0 and s[i] in " *":
            i += 1
            continue
        if s[i] in "XYZ":
            j = i + 1
            while j < n and s[j].isdigit():
                j += 1
            if j == i + 1:
                raise RuntimeError("Invalid Pauli string")
            out.append((int(s[i + 1:j]), s[i]))
            i = j
        else:
            raise RuntimeError("Invalid Pauli string")
    return out


class PauliString:
    """A Pauli string on up to 128 qubits."""
    __slots__ = ("x", "z")

    def __init__(self, arg=None):
        self.x = 0
        self.z = 0
        if arg is None:
            return
        if isinstance(arg, PauliString):
            self.x, self.z = arg.x, arg.z
            return
        if isinstance(arg, str):
            if all(c in "IXYZ" for c in arg):
                for i, c in enumerate(arg):
                    if i >= MAX_QUBITS and c != "I":
                        _check_loc(i)
                    if c in "XY":
                        self.x |= 1 << i
                    if c in "YZ":
                        self.z |= 1 << i
                return
            arg = _parse_indexed(arg)
        pairs = [(int(l), str(a)) for l, a in arg]
        for k, (loc, act) in enumerate(pairs):
            for m, (loc2, _) in enumerate(pairs):
                if m != k and loc2 == loc:
                    raise RuntimeError(f"Invalid PauliString (qubit index {loc} appears multiple times)")
            _check_loc(loc)
            if act not in ("I", "X", "Y", "Z"):
                raise RuntimeError(f"Invalid PauliString (symbol '{act}' not recognized)")
            if act in "XY":
                self.x |= 1 << loc
            if act in "YZ":
                self.z |= 1 << loc

    @classmethod
    def from_masks(cls, x, z):
        s = cls.__new__(cls)
        s.x = int(x)
        s.z = int(z)
        return s

    # ---- queries -------------------------------------------------------
    def indices(self):
        out = []
        sup = self.x | self.z
        pos = 0
        while sup:
            if sup & 1:
                p, q = (self.x >> pos) & 1, (self.z >> pos) & 1
                out.append((pos, "Y" if p and q else ("X" if p else "Z")))
            sup >>= 1
            pos += 1
        return out

    def degree(self, v=None):
        if v is None or v == "\0":
            return _popc(self.x | self.z)
        if v in ("X", "x"):
            return _popc(self.x & ~self.z)
        if v in ("Y", "y"):
            return _popc(self.x & self.z)
        if v in ("Z", "z"):
            return _popc(~self.x & self.z & _MASK)
        raise RuntimeError("Invalid argument: should be either 'X', 'Y', or 'Z' or empty char")

    def extent(self):
        return (self.x | self.z).bit_length()

    def support(self):
        return [p for p, _ in self.indices()]

    def commutes(self, other):
        if isinstance(other, PauliPolynomial):
            return all(self.commutes(s) for s in other.terms)
        return _popc(self.x & other.z) % 2 == _popc(self.z & other.x) % 2

    def _mul(self, other):
        """(string, phase) of self * other (pauli_string_multiply)."""
        j = _popc(self.x & self.z) + _popc(other.x & other.z) + 2 * _popc(self.z & other.x)
        x, z = self.x ^ other.x, self.z ^ other.z
        j -= _popc(x & z)
        return PauliString.from_masks(x, z), _ipow(j)

    def to_string(self, n=0):
        s = ["I"] * max(self.extent(), n)
        for p, a in self.indices():
            s[p] = a
        return "".join(s)

    def to_compact_string(self):
        if not (self.x | self.z):
            return "I"
        return " ".join(f"{a}{p}" for p, a in self.indices())

    __str__ = to_compact_string
    __repr__ = to_compact_string

    def __hash__(self):
        return hash((self.x, self.z))

    def __eq__(self, other):
        if isinstance(other, PauliString):
            return self.x == other.x and self.z == other.z
        if isinstance(other, numbers.Number):
            return False
        return NotImplemented

    # ---- arithmetic (returns polynomials) -----------------------------
    def __mul__(self, other):
        return PauliPolynomial(self) * other

    def __rmul__(self, other):
        return PauliPolynomial(self) * other

    def __add__(self, other):
        return PauliPolynomial(self) + other

    def __radd__(self, other):
        return PauliPolynomial(self) + other

    def __sub__(self, other):
        return PauliPolynomial(self) - other

    def __rsub__(self, other):
        return -PauliPolynomial(self) + other

    def __neg__(self):
        return -PauliPolynomial(self)


class PauliPolynomial:
    """Linear combination of Pauli strings with complex coefficients.

    ``terms`` is a dict PauliString -> complex.  Polynomials produced by
    ``propagate`` are backed by device memory (``_dev``) and by host arrays
    (``keys`` (4, n) uint64 planes, ``re``, ``im``) materialised on demand.
    """

    def __init__(self, arg=None, coeff=None):
        self._terms = {}
        self._arrays = None
        self._dev = None
        if arg is None:
            return
        if isinstance(arg, PauliPolynomial):
            self._terms = dict(arg.terms)
        elif isinstance(arg, PauliString):
            self._terms = {PauliString(arg): complex(1 if coeff is None else coeff)}
        elif isinstance(arg, numbers.Number):
            self._terms = {PauliString(): complex(arg)}
        elif isinstance(arg, dict):
            self._terms = {PauliString(k): complex(v) for k, v in arg.items()}
        else:
            # sequence of (loc, action), locations may repeat (phases tracked)
            u, ph = PauliString(), 1 + 0j
            for loc, act in arg:
                s, p = u._mul(PauliString([(int(loc), act)]))
                u, ph = s, ph * p
            self._terms = {u: ph * complex(1 if coeff is None else coeff)}

    # ---- construction from arrays / device results ----------------------
    @classmethod
    def from_arrays(cls, keys, re, im=None):
        p = cls()
        keys = np.asarray(keys, dtype=np.uint64).reshape(4, -1)
        re = np.asarray(re, dtype=np.float64)
        im = np.zeros_like(re) if im is None else np.asarray(im, dtype=np.float64)
        p._arrays = (keys, re, im)
        p._terms = None
        return p

    @classmethod
    def _from_result(cls, res):
        p = cls()
        p._dev = res
        p._terms = None
        return p

    def arrays(self):
        """(keys (4, n) uint64, re, im) of the terms."""
        if self._arrays is None:
            if self._dev is not None:
                self._arrays = self._dev.copy()
            else:
                n = len(self._terms)
                keys = np.zeros((4, n), dtype=np.uint64)
                re = np.zeros(n)
                im = np.zeros(n)
                m64 = (1 << 64) - 1
                for i, (s, c) in enumerate(self._terms.items()):
                    keys[0, i] = s.x & m64
                    keys[1, i] = s.x >> 64
                    keys[2, i] = s.z & m64
                    keys[3, i] = s.z >> 64
                    re[i] = c.real
                    im[i] = c.imag
                return keys, re, im
        return self._arrays

    @property
    def terms(self):
        if self._terms is None:
            keys, re, im = self.arrays()
            k = keys.astype(object)
            xs = (k[1] << 64) | k[0]
            zs = (k[3] << 64) | k[2]
            self._terms = {PauliString.from_masks(x, z): complex(a, b)
                           for x, z, a, b in zip(xs.tolist(), zs.tolist(), re.tolist(), im.tolist())}
        return self._terms

    def _mutate(self):
        t = self.terms
        self._arrays = None
        self._dev = None
        return t

    def __len__(self):
        if self._terms is not None:
            return len(self._terms)
        if self._dev is not None:
            return self._dev.n
        return self._arrays[1].size

    # ---- queries ----------------------------------------------------------
    def overlapwithzero(self):
        """<0...0|O|0...0> (src/pauli/algebra.h:549-557)."""
        if self._dev is not None:
            return self._dev.overlapwithzero()
        if self._arrays is not None and self._terms is None:
            k, re, im = self._arrays
            m = (k[0] == 0) & (k[1] == 0)
            return complex(float(np.sum(re[m])), float(np.sum(im[m])))
        r = 0j
        for s, c in self.terms.items():
            if s.x == 0:
                r += c
        return r

    def sparse(self, n=None, nup=None):
        """The 2^n x 2^n matrix as a scipy.sparse.csc_matrix, built on the GPU
        (src/pauli/sparse.h:20-131; n defaults to the extent).  The
        fixed-particle-number subspace (nup) is not provided."""
        if nup is not None:
            raise NotImplementedError("sparse(n, nup): the subspace variant is not provided")
        import scipy.sparse as sp

        n = self.extent() if n is None else int(n)
        if self._dev is not None:
            res = self._dev
        else:
            keys, re, im = self.arrays()
            from .propagation import propagate
            res = propagate([], PauliPolynomial.from_arrays(keys, re, im))._dev
        indptr, indices, data = res.sparse(n)
        return sp.csc_matrix((data, indices, indptr), shape=(1 << n, 1 << n))

    def coefficient(self, s):
        if not isinstance(s, PauliString):
            s = PauliString(s)
        return self.terms.get(s, 0j)

    def degree(self, v=None):
        d = 0
        for s, c in self.terms.items():
            if c != 0:
                d = max(d, s.degree(v))
        return d

    def extent(self):
        return max((s.extent() for s in self.terms), default=0)

    def support(self):
        m = 0
        for s in self.terms:
            m |= s.x | s.z
        return [i for i in range(m.bit_length()) if (m >> i) & 1]

    def compress(self, threshold=1e-8):
        return PauliPolynomial({s: c for s, c in self.terms.items() if abs(c) > threshold})

    def truncate(self, k):
        return PauliPolynomial({s: c for s, c in self.terms.items() if s.degree() <= k})

    def dagger(self):
        return PauliPolynomial({s: c.conjugate() for s, c in self.terms.items()})

    def is_hermitian(self):
        return all(c.imag == 0 for c in self.terms.values())

    def norm(self, v=1):
        vals = [abs(c) for c in self.terms.values()]
        if v == "inf":
            return max(vals, default=0.0)
        if v == 0:
            return float(sum(1 for a in vals if a != 0))
        if v == 1:
            return float(sum(vals))
        if v == 2:
            return math.sqrt(sum(a * a for a in vals))
        raise RuntimeError("Invalid argument")

    def commutes(self, other):
        if isinstance(other, PauliString):
            other = PauliPolynomial(other)
        return len((self * other - other * self).compress(0)) == 0

    # ---- arithmetic ---------------------------------------------------------
    def copy(self):
        return PauliPolynomial(self)

    @staticmethod
    def _as_poly(o):
        if isinstance(o, PauliPolynomial):
            return o
        if isinstance(o, PauliString):
            return PauliPolynomial(o)
        if isinstance(o, numbers.Number):
            return PauliPolynomial(complex(o)) if o != 0 else PauliPolynomial()
        return None

    def __add__(self, o):
        o = self._as_poly(o)
        if o is None:
            return NotImplemented
        t = dict(self.terms)
        for s, c in o.terms.items():
            t[s] = t.get(s, 0j) + c
        return PauliPolynomial(t)

    __radd__ = __add__

    def __neg__(self):
        return PauliPolynomial({s: -c for s, c in self.terms.items()})

    def __sub__(self, o):
        o = self._as_poly(o)
        if o is None:
            return NotImplemented
        return self + (-o)

    def __rsub__(self, o):
        return (-self) + o

    def __mul__(self, o):
        if isinstance(o, numbers.Number):
            return PauliPolynomial({s: c * o for s, c in self.terms.items()})
        o = self._as_poly(o)
        if o is None:
            return NotImplemented
        t = {}
        for a, ca in self.terms.items():
            for b, cb in o.terms.items():
                s, ph = a._mul(b)
                t[s] = t.get(s, 0j) + ph * ca * cb
        return PauliPolynomial(t)

    def __rmul__(self, o):
        if isinstance(o, numbers.Number):
            return self * o
        o = self._as_poly(o)
        return o * self

    def __truediv__(self, o):
        return self * (1.0 / o)

    def __iadd__(self, o):
        return self + o

    def __isub__(self, o):
        return self - o

    def __imul__(self, o):
        return self * o

    def __eq__(self, o):
        o = self._as_poly(o)
        if o is None:
            return NotImplemented
        return (self - o).norm("inf") == 0

    def to_compact_string(self):
        if not self.terms:
            return "0"
        return " + ".join(f"({c.real:g}{c.imag:+g}j) {s}" for s, c in self.terms.items())

    __str__ = to_compact_string
    __repr__ = to_compact_string


# --------------------------------------------------------------------------
# gates (src/pauli/gates.h)
# --------------------------------------------------------------------------

class _Clifford:
    __slots__ = ("i", "j")
    kind = 0
    nq = 1

    def __init__(self, i, j=None):
        self.i = int(i)
        if self.nq == 2:
            if j is None:
                raise TypeError(f"{type(self).__name__} takes two qubits")
            self.j = int(j)
        else:
            self.j = 0

    @property
    def qubits(self):
        return [self.i, self.j] if self.nq == 2 else [self.i]

    def _apply(self, s):
        """(new string, sign) for the Heisenberg map of one Pauli string."""
        x, z = s.x, s.z
        i, j = self.i, self.j
        bi = lambda v, k: (v >> k) & 1  # noqa: E731

        def setb(v, k, b):
            return (v & ~(1 << k)) | (b << k)

        flip = 0
        if self.kind == 1:    # H: X<->Z, Y -> -Y
            xi, zi = bi(x, i), bi(z, i)
            x, z = setb(x, i, zi), setb(z, i, xi)
            flip = xi & zi
        elif self.kind == 2:  # S: X -> -Y, Y -> X
            xi, zi = bi(x, i), bi(z, i)
            z = setb(z, i, xi ^ zi)
            flip = xi & (zi ^ 1)
        elif self.kind == 3:  # CNOT
            xi, xj, zi, zj = bi(x, i), bi(x, j), bi(z, i), bi(z, j)
            x, z = setb(x, j, xi ^ xj), setb(z, i, zi ^ zj)
            flip = xi & zj & ((zi ^ xj) ^ 1)
        elif self.kind == 4:  # SWAP
            xi, xj, zi, zj = bi(x, i), bi(x, j), bi(z, i), bi(z, j)
            x = setb(setb(x, i, xj), j, xi)
            z = setb(setb(z, i, zj), j, zi)
        elif self.kind == 5:  # CZ
            xi, xj, zi, zj = bi(x, i), bi(x, j), bi(z, i), bi(z, j)
            flip = xi & xj & (zi ^ zj)
            z ^= (xj << i) | (xi << j)
        return PauliString.from_masks(x, z), (-1 if flip else 1)

    def __call__(self, o):
        if isinstance(o, PauliString):
            s, sg = self._apply(o)
            return s, complex(sg)
        t = {}
        for s, c in o.terms.items():
            y, sg = self._apply(s)
            t[y] = t.get(y, 0j) + sg * c
        return PauliPolynomial(t)

    def __repr__(self):
        return f"{type(self).__name__}({','.join(str(q) for q in self.qubits)})"

    __str__ = __repr__


class H(_Clifford):
    """Hadamard: U = (X_p + Z_p)/sqrt(2)."""
    kind = 1

    def aspoly(self):
        r = 1 / math.sqrt(2)
        return PauliPolynomial({PauliString([(self.i, "X")]): r, PauliString([(self.i, "Z")]): r})


class S(_Clifford):
    """S gate: U = ((1+1j) + (1-1j) Z_p)/2."""
    kind = 2

    def aspoly(self):
        return PauliPolynomial({PauliString(): 0.5 + 0.5j, PauliString([(self.i, "Z")]): 0.5 - 0.5j})


class CNOT(_Clifford):
    """CNOT: U = (1 + Z_p + X_q - Z_p X_q)/2."""
    kind = 3
    nq = 2

    def aspoly(self):
        return PauliPolynomial({PauliString(): 0.5, PauliString([(self.i, "Z")]): 0.5,
                                PauliString([(self.j, "X")]): 0.5,
                                PauliString([(self.i, "Z"), (self.j, "X")]): -0.5})


class SWAP(_Clifford):
    """SWAP: U = (1 + X_p X_q + Y_p Y_q + Z_p Z_q)/2."""
    kind = 4
    nq = 2

    def aspoly(self):
        i, j = self.i, self.j
        return PauliPolynomial({PauliString(): 0.5, PauliString([(i, "X"), (j, "X")]): 0.5,
                                PauliString([(i, "Y"), (j, "Y")]): 0.5,
                                PauliString([(i, "Z"), (j, "Z")]): 0.5})


class CZ(_Clifford):
    """CZ: U = (1 + Z_p + Z_q - Z_p Z_q)/2."""
    kind = 5
    nq = 2

    def aspoly(self):
        i, j = self.i, self.j
        return PauliPolynomial({PauliString(): 0.5, PauliString([(i, "Z")]): 0.5,
                                PauliString([(j, "Z")]): 0.5,
                                PauliString([(i, "Z"), (j, "Z")]): -0.5})


class ROT:
    """Pauli rotation U = exp(-i theta/2 P).

    ROT("XX", [0, 1], 0.75), ROT(PauliString, theta) or ROT("XZ", theta)."""
    __slots__ = ("axis", "theta")

    def __init__(self, a, b, c=None):
        if c is None:
            self.axis = PauliString(a) if not isinstance(a, PauliString) else PauliString(a)
            self.theta = float(b)
        else:
            locs = list(b)
            if len(locs) != len(a):
                raise RuntimeError("Invalid arguments (both arguments should have the same size)")
            self.axis = PauliString(list(zip(locs, a)))
            self.theta = float(c)

    @property
    def qubits(self):
        return self.axis.support()

    def aspoly(self):
        return PauliPolynomial({PauliString(): math.cos(self.theta / 2)}) + \
            PauliPolynomial(self.axis, complex(0, -math.sin(self.theta / 2)))

    def __call__(self, o):
        """U^dagger o U for one gate (src/pauli/gates.h:234-252)."""
        if isinstance(o, PauliString):
            o = PauliPolynomial(o)
        t = dict(o.terms)
        new = []
        c, s = math.cos(self.theta), math.sin(self.theta)
        for q, v in list(t.items()):
            if not q.commutes(self.axis):
                k, ph = self.axis._mul(q)
                new.append((k, v * complex(0, s) * ph))
                t[q] = v * c
        for k, v in new:
            t[k] = t.get(k, 0j) + v
        return PauliPolynomial(t)

    def __repr__(self):
        return f"ROT({self.axis.to_compact_string()},{self.theta:f})"

    __str__ = __repr__


# --------------------------------------------------------------------------
# product state (src/qubitproductstate.h)
# --------------------------------------------------------------------------

class QubitProductState:
    """Computational-basis product state |b>; ``up`` lists the qubits in |1>."""

    def __init__(self, up=None):
        self.b = 0
        if isinstance(up, numbers.Integral):
            self.b = int(up)
        elif up is not None:
            for q in up:
                self.b |= 1 << int(q)

    def up(self):
        return [i for i in range(self.b.bit_length()) if (self.b >> i) & 1]

    def __call__(self, o):
        if isinstance(o, PauliString):
            return complex(-1 if _popc(o.z & self.b) % 2 else 1) if o.x == 0 else 0j
        if o._dev is not None:
            m = (1 << 64) - 1
            return o._dev.qubit_state(self.b & m, self.b >> 64)
        r = 0j
        for s, c in o.terms.items():
            if s.x == 0:
                r += c * (-1 if _popc(s.z & self.b) % 2 else 1)
        return r

    def vec(self, n, nocc=None):
        if nocc is None:
            v = [0.0] * (1 << n)
            v[int(format(self.b, f"0{n}b")[::-1], 2) if n else 0] = 1.0
            return v
        raise NotImplementedError("subspace vectors are not provided")


def paulis(n):
    """X, Y, Z lists of single-qubit Pauli polynomials on n qubits."""
    return ([PauliPolynomial(PauliString([(i, a)])) for i in range(n)] for a in "XYZ")


__all__ = ["PauliString", "PauliPolynomial", "H", "S", "CNOT", "SWAP", "CZ", "ROT",
           "QubitProductState", "paulis", "MAX_QUBITS"]
