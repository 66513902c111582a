"""``poly``: build a Pauli or Majorana polynomial from an expression string,
e.g. ``poly("-Z2 + 3*X0")``, ``poly("0.1 m0 m1 + 1j m0 - 4 m1")``.

Grammar (own recursive-descent parser): sums and differences of products;
factors are numbers (``2``, ``0.5``, ``1e-3``, ``2j``), Pauli atoms ``X<q>``,
``Y<q>``, ``Z<q>``, Majorana atoms ``m<i>`` and parenthesised expressions;
juxtaposition multiplies.
"""
import re

from .majorana import MajoranaPolynomial, MajoranaString
from .pauli import PauliPolynomial, PauliString

_TOKEN = re.compile(r"\s*(?:(?P<num>(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?j?)|(?P<atom>[XYZm]\d+)"
                    r"|(?P<op>[-+*/()]))")


def _tokens(s):
    pos, out = 0, []
    s = s.rstrip()
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise ValueError(f"Invalid expression near {s[pos:pos + 10]!r}")
        pos = m.end()
        if m.group("num"):
            out.append(("num", complex(m.group("num")) if m.group("num").endswith("j")
                        else float(m.group("num"))))
        elif m.group("atom"):
            a = m.group("atom")
            if a[0] == "m":
                out.append(("val", MajoranaPolynomial(MajoranaString([int(a[1:])]))))
            else:
                out.append(("val", PauliPolynomial(PauliString([(int(a[1:]), a[0])]))))
        else:
            out.append(("op", m.group("op")))
    return out


class _Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self):
        tok = self.peek()
        self.i += 1
        return tok

    def expr(self):
        v = self.term()
        while self.peek() in (("op", "+"), ("op", "-")):
            op = self.take()[1]
            r = self.term()
            v = v + r if op == "+" else v - r
        return v

    def term(self):
        v = self.unary()
        while True:
            k, x = self.peek()
            if (k, x) == ("op", "*"):
                self.take()
                v = v * self.unary()
            elif (k, x) == ("op", "/"):
                self.take()
                v = v / self.unary()
            elif k in ("num", "val") or (k, x) == ("op", "("):
                v = v * self.unary()
            else:
                return v

    def unary(self):
        k, x = self.peek()
        if (k, x) == ("op", "-"):
            self.take()
            return -self.unary()
        if (k, x) == ("op", "+"):
            self.take()
            return self.unary()
        return self.factor()

    def factor(self):
        k, x = self.take()
        if k in ("num", "val"):
            return x
        if (k, x) == ("op", "("):
            v = self.expr()
            if self.take() != ("op", ")"):
                raise ValueError("Invalid expression: missing ')'")
            return v
        raise ValueError("Invalid expression")


def poly(expr):
    """Parses a Pauli or Majorana polynomial expression."""
    p = _Parser(_tokens(expr))
    v = p.expr()
    if p.i != len(p.t):
        raise ValueError("Invalid expression")
    if isinstance(v, (int, float, complex)):
        return PauliPolynomial(complex(v))
    return v


__all__ = ["poly"]
