"""Majorana strings, Majorana polynomials, Majorana rotations and Fock states.

Same names, constructors and conventions as fastfermion's Python API for these
types (src/majorana_algebra.h, src/majorana_gates.h, src/fockstate.h): a
string is the increasing product gamma_{i1} ... gamma_{ik} of at most 256
Majorana operators; errors raise RuntimeError.
"""
import math
import numbers

import numpy as np

MAX_MAJORANAS = 256


def _popc(v):
    return bin(v).count("1")


def _merge_parity(x, y):
    """parity of #{(i, j) : i in x, j in y, i < j} (src/bits_utils.h:14-38)"""
    tot = 0
    while y:
        b = y.bit_length() - 1
        tot += _popc(x & ((1 << b) - 1))
        y ^= 1 << b
    return tot & 1


def _parse_majorana(s):
    if s in ("I", "1"):
        return []
    out, i, n = [], 0, len(s)
    while i < n:
        if i > 0 and s[i] in " *":
            i += 1
            continue
        if s[i] == "m":
            j = i + 1
            while j < n and s[j].isdigit():
                j += 1
            if j == i + 1:
                raise RuntimeError("Invalid Majorana string")
            out.append(int(s[i + 1:j]))
            i = j
        else:
            raise RuntimeError("Invalid Majorana string")
    return out


class MajoranaString:
    __slots__ = ("alpha",)

    def __init__(self, supp=None):
        self.alpha = 0
        if supp is None:
            return
        if isinstance(supp, MajoranaString):
            self.alpha = supp.alpha
            return
        if isinstance(supp, str):
            supp = _parse_majorana(supp)
        supp = [int(v) for v in supp]
        for k, v in enumerate(supp):
            if k > 0 and v <= supp[k - 1]:
                raise RuntimeError("Invalid MajoranaString (not normal ordered)")
            if not (0 <= v < MAX_MAJORANAS):
                raise RuntimeError(f"Invalid MajoranaString (mode index {v} invalid, should be "
                                   f"between 0 and {MAX_MAJORANAS - 1})")
            self.alpha |= 1 << v

    @classmethod
    def from_mask(cls, alpha):
        s = cls.__new__(cls)
        s.alpha = int(alpha)
        return s

    def indices(self):
        a, out, p = self.alpha, [], 0
        while a:
            if a & 1:
                out.append(p)
            a >>= 1
            p += 1
        return out

    support_set = indices

    def degree(self):
        return _popc(self.alpha)

    def is_hermitian(self):
        return self.degree() % 4 in (0, 1)

    def extent(self):
        return self.alpha.bit_length()

    def commutes(self, other):
        if isinstance(other, MajoranaPolynomial):
            return all(self.commutes(s) for s in other.terms)
        na, nb, nab = self.degree(), other.degree(), _popc(self.alpha & other.alpha)
        return (na * nb - nab) % 2 == 0

    def _mul(self, other):
        """(string, sign) of self * other (src/majorana_algebra.h:441-444)."""
        return MajoranaString.from_mask(self.alpha ^ other.alpha), (-1 if _merge_parity(other.alpha, self.alpha) else 1)

    def to_compact_string(self):
        return " ".join(f"m{i}" for i in self.indices()) or "I"

    __str__ = to_compact_string
    __repr__ = to_compact_string

    def __hash__(self):
        return hash(("m", self.alpha))

    def __eq__(self, other):
        if isinstance(other, MajoranaString):
            return self.alpha == other.alpha
        if isinstance(other, numbers.Number):
            return False
        return NotImplemented

    def __mul__(self, o):
        return MajoranaPolynomial(self) * o

    def __rmul__(self, o):
        return MajoranaPolynomial(self) * o

    def __add__(self, o):
        return MajoranaPolynomial(self) + o

    __radd__ = __add__

    def __sub__(self, o):
        return MajoranaPolynomial(self) - o

    def __rsub__(self, o):
        return -MajoranaPolynomial(self) + o

    def __neg__(self):
        return -MajoranaPolynomial(self)


class MajoranaPolynomial:
    """Linear combination of Majorana strings; ``terms`` maps MajoranaString -> complex."""

    def __init__(self, arg=None, coeff=None):
        self._terms = {}
        self._arrays = None
        self._dev = None
        if arg is None:
            return
        if isinstance(arg, MajoranaPolynomial):
            self._terms = dict(arg.terms)
        elif isinstance(arg, MajoranaString):
            self._terms = {MajoranaString(arg): complex(1 if coeff is None else coeff)}
        elif isinstance(arg, numbers.Number):
            self._terms = {MajoranaString(): complex(arg)}
        elif isinstance(arg, dict):
            self._terms = {MajoranaString(k): complex(v) for k, v in arg.items()}
        else:
            # product gamma_{s0} gamma_{s1} ... of a possibly unsorted index list
            alpha, sgn = 0, 0
            for v in arg:
                v = int(v)
                if not (0 <= v < MAX_MAJORANAS):
                    raise RuntimeError(f"Invalid MajoranaString (mode index {v} invalid, should be "
                                       f"between 0 and {MAX_MAJORANAS - 1})")
                alpha ^= 1 << v
                sgn ^= _popc(alpha >> (v + 1)) & 1
            c = complex(1 if coeff is None else coeff)
            self._terms = {MajoranaString.from_mask(alpha): (-1 if sgn else 1) * c}

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
        if self._arrays is None:
            if self._dev is not None:
                self._arrays = self._dev.copy()
            else:
                n = len(self._terms)
                keys = np.zeros((4, n), dtype=np.uint64)
                re, im = np.zeros(n), np.zeros(n)
                m64 = (1 << 64) - 1
                for i, (s, c) in enumerate(self._terms.items()):
                    for w in range(4):
                        keys[w, i] = (s.alpha >> (64 * w)) & m64
                    re[i], im[i] = c.real, c.imag
                return keys, re, im
        return self._arrays

    @property
    def terms(self):
        if self._terms is None:
            keys, re, im = self.arrays()
            k = keys.astype(object)
            al = k[0] | (k[1] << 64) | (k[2] << 128) | (k[3] << 192)
            self._terms = {MajoranaString.from_mask(a): complex(x, y)
                           for a, x, y in zip(al.tolist(), re.tolist(), im.tolist())}
        return self._terms

    def __len__(self):
        if self._terms is not None:
            return len(self._terms)
        if self._dev is not None:
            return self._dev.n
        return self._arrays[1].size

    def degree(self):
        return max((s.degree() for s, c in self.terms.items() if c != 0), default=0)

    def coefficient(self, s):
        if not isinstance(s, MajoranaString):
            s = MajoranaString(s)
        return self.terms.get(s, 0j)

    def extent(self):
        return max((s.extent() for s in self.terms), default=0)

    def compress(self, threshold=1e-8):
        return MajoranaPolynomial({s: c for s, c in self.terms.items() if abs(c) > threshold})

    def truncate(self, k):
        return MajoranaPolynomial({s: c for s, c in self.terms.items() if s.degree() <= k})

    def is_hermitian(self):
        for s, c in self.terms.items():
            if s.is_hermitian() and c.imag != 0:
                return False
            if not s.is_hermitian() and c.real != 0:
                return False
        return True

    def dagger(self):
        t = {}
        for s, c in self.terms.items():
            d = s.degree()
            t[s] = (1 if (d * (d - 1) // 2) % 2 == 0 else -1) * c.conjugate()
        return MajoranaPolynomial(t)

    def norm(self, v=1):
        vals = [abs(c) for c in self.terms.values()]
        if v == "inf":
            return max(vals, default=0.0)
        if v == 1:
            return float(sum(vals))
        if v == 2:
            return math.sqrt(sum(a * a for a in vals))
        if v == 0:
            return float(sum(1 for a in vals if a != 0))
        raise RuntimeError("Invalid argument")

    @staticmethod
    def _as_poly(o):
        if isinstance(o, MajoranaPolynomial):
            return o
        if isinstance(o, MajoranaString):
            return MajoranaPolynomial(o)
        if isinstance(o, numbers.Number):
            return MajoranaPolynomial(complex(o)) if o != 0 else MajoranaPolynomial()
        return None

    def __add__(self, o):
        o = self._as_poly(o)
        if o is None:
            return NotImplemented
        t = dict(self.terms)
        for s, c in o.terms.items():
            t[s] = t.get(s, 0j) + c
        return MajoranaPolynomial(t)

    __radd__ = __add__

    def __neg__(self):
        return MajoranaPolynomial({s: -c for s, c in self.terms.items()})

    def __sub__(self, o):
        o = self._as_poly(o)
        if o is None:
            return NotImplemented
        return self + (-o)

    def __rsub__(self, o):
        return (-self) + o

    def __mul__(self, o):
        if isinstance(o, numbers.Number):
            return MajoranaPolynomial({s: c * o for s, c in self.terms.items()})
        o = self._as_poly(o)
        if o is None:
            return NotImplemented
        t = {}
        for a, ca in self.terms.items():
            for b, cb in o.terms.items():
                s, sg = a._mul(b)
                t[s] = t.get(s, 0j) + sg * ca * cb
        return MajoranaPolynomial(t)

    def __rmul__(self, o):
        if isinstance(o, numbers.Number):
            return self * o
        return self._as_poly(o) * self

    def __truediv__(self, o):
        return self * (1.0 / o)

    def __eq__(self, o):
        o = self._as_poly(o)
        if o is None:
            return NotImplemented
        return (self - o).norm("inf") == 0

    def __str__(self):
        if not self.terms:
            return "0"
        return " + ".join(f"({c.real:g}{c.imag:+g}j) {s}" for s, c in self.terms.items())

    __repr__ = __str__


class MROT:
    """Majorana rotation U = exp(-i theta/2 M), M = i^r gamma_S Hermitian.

    MROT(support_list, coeff, t), MROT(MajoranaString, theta) or
    MROT(MajoranaString, coeff, t); with a coefficient the monomial coeff*gamma_S
    must be Hermitian and theta = Im(coeff)*t (non-Hermitian string) or
    Re(coeff)*t (src/majorana_gates.h:27-48)."""
    __slots__ = ("axis", "theta", "_r")

    def __init__(self, a, b, c=None):
        ms = a if isinstance(a, MajoranaString) else MajoranaString(list(a))
        self.axis = MajoranaString(ms)
        if c is None:
            self.theta = float(b)
            self._r = not ms.is_hermitian()
            return
        coeff, t = complex(b), float(c)
        sh = ms.is_hermitian()
        if not ((sh and coeff.imag == 0) or (not sh and coeff.real == 0)):
            raise RuntimeError(f"Supplied Majorana monomial {coeff}*({ms}) is not Hermitian")
        self._r = not sh
        self.theta = coeff.imag * t if self._r else coeff.real * t

    @property
    def qubits(self):
        return self.axis.indices()

    def aspoly(self):
        s = math.sin(self.theta / 2)
        p = MajoranaPolynomial({MajoranaString(): math.cos(self.theta / 2)})
        return p + MajoranaPolynomial(self.axis, complex(s, 0) if self._r else complex(0, -s))

    def __call__(self, o):
        if isinstance(o, MajoranaString):
            o = MajoranaPolynomial(o)
        t = dict(o.terms)
        c, s = math.cos(self.theta), math.sin(self.theta)
        f = complex(-s, 0) if self._r else complex(0, s)
        new = []
        for x, v in list(t.items()):
            if not x.commutes(self.axis):
                k, sg = self.axis._mul(x)
                new.append((k, v * f * sg))
                t[x] = v * c
        for k, v in new:
            t[k] = t.get(k, 0j) + v
        return MajoranaPolynomial(t)

    def __repr__(self):
        return f"MROT({'1j ' if self._r else ''}{self.axis}, theta={self.theta:f})"

    __str__ = __repr__


class FockState:
    """Fock state with the modes in ``occ`` occupied."""

    def __init__(self, occ=None):
        self.b = 0
        if isinstance(occ, numbers.Integral):
            self.b = int(occ)
        elif occ is not None:
            for q in occ:
                self.b |= 1 << int(q)

    def occ(self):
        return [i for i in range(self.b.bit_length()) if (self.b >> i) & 1]

    @staticmethod
    def _pairs(alpha):
        ev, od = alpha & int("55" * 32, 16), (alpha >> 1) & int("55" * 32, 16)
        if ev != od:
            return None
        J, j = 0, 0
        while ev:
            if ev & 1:
                J |= 1 << j
            ev >>= 2
            j += 1
        return J

    def vec(self, m, nocc=None):
        """Dense basis vector of the state on m modes (mode 0 is the most
        significant bit of the index, as in the sparse export)."""
        if nocc is None:
            v = [0.0] * (1 << m)
            v[int(format(self.b, f"0{m}b")[::-1], 2) if m else 0] = 1.0
            return v
        raise NotImplementedError("subspace vectors are not provided")

    def __call__(self, o):
        if isinstance(o, MajoranaString):
            J = self._pairs(o.alpha)
            if J is None:
                return 0j
            return (1 + 0j, 1j, -1 + 0j, -1j)[(_popc(J) + 2 * _popc(J & self.b)) & 3]
        if o._dev is not None:
            m = (1 << 64) - 1
            return o._dev.fock_state(self.b & m, self.b >> 64)
        r = 0j
        for s, c in o.terms.items():
            r += c * self(s)
        return r


def majoranas(n):
    """[gamma_0, ..., gamma_{n-1}] as Majorana polynomials."""
    return [MajoranaPolynomial(MajoranaString([i])) for i in range(n)]


__all__ = ["MajoranaString", "MajoranaPolynomial", "MROT", "FockState", "majoranas",
           "MAX_MAJORANAS"]


def jw(x):
    """Jordan-Wigner map of a MajoranaString or MajoranaPolynomial to a
    PauliPolynomial, computed on the GPU (src/transforms.h:124-151; the
    reference binds it as ``jw``).  Index 2j maps to Z_0...Z_{j-1} X_j and 2j+1
    to Z_0...Z_{j-1} Y_j; terms whose coefficient maps to exactly zero are
    dropped."""
    from . import _native
    from .pauli import PauliPolynomial
    if isinstance(x, MajoranaString):
        x = MajoranaPolynomial(x)
    if not isinstance(x, MajoranaPolynomial):
        raise TypeError("jw(): expected a MajoranaString or MajoranaPolynomial")
    keys, re, im = x.arrays()
    return PauliPolynomial._from_result(_native.context().majorana_to_pauli(keys, re, im))
