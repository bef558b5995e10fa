"""Lazy expression trees (the Python spelling of xtensor's xfunction) and
their lowering to the C ABI's postfix ``xtg_expr``.

    A = DeviceArray.from_numpy(a); b = DeviceArray.from_numpy(v)
    E = A * b + exp(-A * A)          # nothing is evaluated yet
    out = assign(DeviceArray.empty(A.shape, "float32"), E)

Python scalars follow C++ literal typing: ``2`` is an ``int``, ``2.0`` a
``double`` (so ``A * 2.0`` is a double-typed node, as ``A * 2.0`` is in
xtensor); numpy scalars keep their own dtype.
"""
from __future__ import annotations

import ctypes as C
from typing import Any, Callable

import numpy as np

from ._ffi import DTYPES, MAX_LEAVES, MAX_NODES, OP, Array, Expr, dtype_code


class E:
    """A node of a lazy expression tree."""

    __slots__ = ("op", "kids", "dtype", "arg", "aux", "imm", "src")
    __array_priority__ = 1000

    def __init__(self, op, kids=(), dtype=-1, arg=0, aux=0, imm=0, src=None):
        self.op = op
        self.kids = tuple(kids)
        self.dtype = dtype
        self.arg = arg
        self.aux = aux
        self.imm = imm
        self.src = src

    # arithmetic (xoperation.hpp operators)
    def __add__(self, o): return E(OP["ADD"], (self, as_expr(o)))
    def __radd__(self, o): return E(OP["ADD"], (as_expr(o), self))
    def __sub__(self, o): return E(OP["SUB"], (self, as_expr(o)))
    def __rsub__(self, o): return E(OP["SUB"], (as_expr(o), self))
    def __mul__(self, o): return E(OP["MUL"], (self, as_expr(o)))
    def __rmul__(self, o): return E(OP["MUL"], (as_expr(o), self))
    def __truediv__(self, o): return E(OP["DIV"], (self, as_expr(o)))
    def __rtruediv__(self, o): return E(OP["DIV"], (as_expr(o), self))
    def __mod__(self, o): return E(OP["MOD"], (self, as_expr(o)))
    def __neg__(self): return E(OP["NEG"], (self,))
    def __pos__(self): return E(OP["POS"], (self,))
    def __and__(self, o): return E(OP["BIT_AND"], (self, as_expr(o)))
    def __or__(self, o): return E(OP["BIT_OR"], (self, as_expr(o)))
    def __xor__(self, o): return E(OP["BIT_XOR"], (self, as_expr(o)))
    def __invert__(self): return E(OP["BIT_NOT"], (self,))
    def __lt__(self, o): return E(OP["LT"], (self, as_expr(o)))
    def __le__(self, o): return E(OP["LE"], (self, as_expr(o)))
    def __gt__(self, o): return E(OP["GT"], (self, as_expr(o)))
    def __ge__(self, o): return E(OP["GE"], (self, as_expr(o)))
    __hash__ = object.__hash__

    def eq(self, o): return E(OP["EQ"], (self, as_expr(o)))
    def ne(self, o): return E(OP["NE"], (self, as_expr(o)))


class ExprOps:
    """Operators for array types: `A * b` builds a lazy tree over leaf(A)."""

    __array_priority__ = 1000

    def _e(self):
        return leaf(self)

    def __add__(self, o): return self._e() + o
    def __radd__(self, o): return o + self._e() if isinstance(o, E) else as_expr(o) + self._e()
    def __sub__(self, o): return self._e() - o
    def __rsub__(self, o): return as_expr(o) - self._e()
    def __mul__(self, o): return self._e() * o
    def __rmul__(self, o): return as_expr(o) * self._e()
    def __truediv__(self, o): return self._e() / o
    def __rtruediv__(self, o): return as_expr(o) / self._e()
    def __mod__(self, o): return self._e() % o
    def __neg__(self): return -self._e()
    def __pos__(self): return +self._e()
    def __lt__(self, o): return self._e() < o
    def __le__(self, o): return self._e() <= o
    def __gt__(self, o): return self._e() > o
    def __ge__(self, o): return self._e() >= o
    def __and__(self, o): return self._e() & o
    def __or__(self, o): return self._e() | o
    def __xor__(self, o): return self._e() ^ o
    def __invert__(self): return ~self._e()
    __hash__ = object.__hash__


def leaf(a) -> E:
    """Wrap an array-like with an ``xtg_array()`` method as a tree leaf."""
    if not hasattr(a, "xtg_array"):
        raise TypeError(f"{type(a).__name__} is not an array leaf")
    return E(OP["LEAF"], src=a)


def scalar(v, dtype=None) -> E:
    """An xscalar leaf.  Without a dtype: Python int -> int32, float -> float64,
    bool -> bool, numpy scalars keep theirs."""
    if dtype is None:
        if isinstance(v, (bool, np.bool_)):
            dtype = "bool"
        elif isinstance(v, np.generic):
            dtype = np.dtype(type(v)).name
        elif isinstance(v, int):
            dtype = "int32" if -(2**31) <= v < 2**31 else "int64"
        elif isinstance(v, float):
            dtype = "float64"
        else:
            raise TypeError(f"unsupported scalar {v!r}")
    code = dtype_code(dtype)
    return E(OP["SCALAR"], dtype=code, imm=v)


def as_expr(x) -> E:
    if isinstance(x, E):
        return x
    if hasattr(x, "xtg_array"):
        return leaf(x)
    if isinstance(x, (int, float, bool, np.generic)):
        return scalar(x)
    raise TypeError(f"cannot use {type(x).__name__} in an expression")


def _u(name):
    def f(x):
        return E(OP[name], (as_expr(x),))
    f.__name__ = name.lower()
    return f


exp = _u("EXP")
log = _u("LOG")
sqrt = _u("SQRT")
abs_ = _u("ABS")
square = _u("SQUARE")
sin = _u("SIN")
cos = _u("COS")
tanh = _u("TANH")
negative = _u("NEG")
logical_not = _u("LOGICAL_NOT")


def _b(name):
    def f(x, y):
        return E(OP[name], (as_expr(x), as_expr(y)))
    f.__name__ = name.lower()
    return f


maximum = _b("MAXIMUM")
minimum = _b("MINIMUM")
pow_ = _b("POW")
logical_and = _b("LOGICAL_AND")
logical_or = _b("LOGICAL_OR")
equal = _b("EQ")
not_equal = _b("NE")
less = _b("LT")
greater = _b("GT")


def where(c, a, b) -> E:
    return E(OP["WHERE"], (as_expr(c), as_expr(a), as_expr(b)))


def cast(x, dtype) -> E:
    return E(OP["CAST"], (as_expr(x),), arg=dtype_code(dtype))


# keep-dims statistics over the trailing `naxes` axes, broadcast back
def rsum(x, naxes=1): return E(OP["RSUM"], (as_expr(x),), arg=naxes)
def rmean(x, naxes=1): return E(OP["RMEAN"], (as_expr(x),), arg=naxes)
def rvar(x, naxes=1, ddof=0): return E(OP["RVAR"], (as_expr(x),), arg=naxes, aux=ddof)
def rstd(x, naxes=1, ddof=0): return E(OP["RSTD"], (as_expr(x),), arg=naxes, aux=ddof)
def ramax(x, naxes=1): return E(OP["RMAX"], (as_expr(x),), arg=naxes)
def ramin(x, naxes=1): return E(OP["RMIN"], (as_expr(x),), arg=naxes)


def lower(root) -> tuple[Expr, list]:
    """Postfix lowering of a tree into an ``xtg_expr`` (leaves deduplicated by
    identity).  Returns the struct and the leaf objects (keep them alive)."""
    root = as_expr(root)
    ex = Expr()
    leaves: list = []
    ids: dict[int, int] = {}
    nodes: list[E] = []

    def walk(n: E):
        for k in n.kids:
            walk(k)
        nodes.append(n)

    walk(root)
    if len(nodes) > MAX_NODES:
        raise ValueError(f"expression has {len(nodes)} nodes (max {MAX_NODES})")
    for i, n in enumerate(nodes):
        nd = ex.nodes[i]
        nd.op = n.op
        nd.dtype = n.dtype
        nd.arg = n.arg
        nd.aux = n.aux
        if n.op == OP["LEAF"]:
            key = id(n.src)
            if key not in ids:
                if len(leaves) >= MAX_LEAVES:
                    raise ValueError(f"more than {MAX_LEAVES} distinct leaves")
                ids[key] = len(leaves)
                leaves.append(n.src)
                ex.leaves[ids[key]] = n.src.xtg_array()
            nd.arg = ids[key]
        elif n.op == OP["SCALAR"]:
            code = n.dtype
            if code in (DTYPES["float32"], DTYPES["float64"], DTYPES["bfloat16"]):
                nd.imm.f = float(n.imm)
            elif code == DTYPES["uint64"]:
                nd.imm.u = int(n.imm) & (2**64 - 1)
            else:
                nd.imm.i = int(n.imm)
    ex.n_nodes = len(nodes)
    ex.n_leaves = len(leaves)
    return ex, leaves
