"""Symbolic tracing of form callables.

The reference evaluates a form callable on numpy ``DiscreteField`` arrays
at every quadrature point (bilinear_form.py:150-151).  Here the callable is
run once on symbolic stand-ins: ``u``/``v`` carry symbols for their values
and derivatives and ``w.name`` yields a coefficient symbol.  Every symbol is
a ``Sym`` -- a polynomial that is at most linear in the trial quantities and
at most linear in the test quantities, whose coefficients are monomials in
the named coefficient fields.  Helpers written with numpy (einsum on object
arrays, as ``skfem.helpers`` does) trace unchanged.

The traced polynomial is then matched to the kernel's coefficient channels
(``FemBilinear`` / ``FemLinear`` in include/skfem_gb300.h); forms outside
those families raise NotImplementedError rather than falling back.
"""

import numbers

import numpy as np

__all__ = ["Sym", "SymField", "trace_bilinear", "trace_linear", "bilinear_channels",
           "linear_channels", "Poly"]

REL = 1e-13


class Poly(dict):
    """{fields tuple (sorted names, with multiplicity): float coefficient}."""

    def add(self, other, s=1.0):
        out = Poly(self)
        for k, v in other.items():
            out[k] = out.get(k, 0.0) + s * v
        return Poly({k: v for k, v in out.items() if v != 0.0})

    def scaled(self, s):
        return Poly({k: v * s for k, v in self.items() if v * s != 0.0})

    def close(self, other):
        keys = set(self) | set(other)
        scale = max([abs(v) for v in self.values()] + [abs(v) for v in other.values()] + [0.0])
        return all(abs(self.get(k, 0.0) - other.get(k, 0.0)) <= REL * scale for k in keys)

    def is_zero(self):
        return all(v == 0.0 for v in self.values())


class Sym:
    """Bilinear polynomial: {(uq, vq, fields): coef}; uq/vq are None, ('v', c)
    (value of component c) or ('d', c, k) (derivative k of component c)."""

    __slots__ = ("terms", "grad")
    __array_ufunc__ = None

    def __init__(self, terms=None):
        self.terms = {} if terms is None else {k: v for k, v in terms.items() if v != 0.0}
        self.grad = None

    @staticmethod
    def const(c):
        return Sym({(None, None, ()): float(c)})

    @staticmethod
    def lift(o):
        if isinstance(o, Sym):
            return o
        if isinstance(o, numbers.Number) or (isinstance(o, np.ndarray) and o.ndim == 0
                                             and o.dtype != object):
            return Sym.const(float(o))
        if isinstance(o, np.ndarray) and o.ndim == 0:
            return Sym.lift(o.item())
        raise TypeError("cannot combine %r with a traced form quantity" % type(o))

    # arithmetic --------------------------------------------------------
    def _bcast(self, o, op):
        return np.frompyfunc(lambda x: op(self, x), 1, 1)(o)

    def __add__(self, o):
        if isinstance(o, np.ndarray) and o.ndim > 0:
            return self._bcast(o, Sym.__add__)
        o = Sym.lift(o)
        t = dict(self.terms)
        for k, v in o.terms.items():
            t[k] = t.get(k, 0.0) + v
        return Sym(t)

    __radd__ = __add__

    def __neg__(self):
        return Sym({k: -v for k, v in self.terms.items()})

    def __pos__(self):
        return self

    def __sub__(self, o):
        if isinstance(o, np.ndarray) and o.ndim > 0:
            return self._bcast(o, Sym.__sub__)
        return self + (-Sym.lift(o))

    def __rsub__(self, o):
        if isinstance(o, np.ndarray) and o.ndim > 0:
            return self._bcast(o, Sym.__rsub__)
        return Sym.lift(o) + (-self)

    def __mul__(self, o):
        if isinstance(o, np.ndarray) and o.ndim > 0:
            return self._bcast(o, Sym.__mul__)
        o = Sym.lift(o)
        t = {}
        for (u1, v1, f1), c1 in self.terms.items():
            for (u2, v2, f2), c2 in o.terms.items():
                if u1 is not None and u2 is not None:
                    raise NotImplementedError("form is not linear in the trial function")
                if v1 is not None and v2 is not None:
                    raise NotImplementedError("form is not linear in the test function")
                k = (u1 if u1 is not None else u2, v1 if v1 is not None else v2,
                     tuple(sorted(f1 + f2)))
                t[k] = t.get(k, 0.0) + c1 * c2
        return Sym(t)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, numbers.Number):
            return self * (1.0 / o)
        o = Sym.lift(o)
        if set(o.terms) == {(None, None, ())}:
            return self * (1.0 / o.terms[(None, None, ())])
        raise NotImplementedError("division by a coefficient field is not supported")

    def __pow__(self, n):
        if not isinstance(n, numbers.Integral) or n < 0:
            raise NotImplementedError("only non-negative integer powers are supported")
        out = Sym.const(1.0)
        for _ in range(n):
            out = out * self
        return out

    def __repr__(self):
        return "Sym(%r)" % self.terms

    # numpy-compatible bits some helpers touch
    @property
    def shape(self):
        return ()


class SymField(np.ndarray):
    """Object array of Syms with a ``grad`` attribute (vector fields)."""

    def __new__(cls, value, grad=None):
        obj = np.asarray(value, dtype=object).view(cls)
        obj.grad = grad
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        self.grad = getattr(obj, "grad", None)


def _field(which, elem, dim):
    """Symbolic trial (which='u') or test (which='v') function."""
    def q(*key):
        if which == "u":
            return Sym({(key, None, ()): 1.0})
        return Sym({(None, key, ()): 1.0})

    if not elem.vector:
        s = q("v", 0)
        s.grad = np.array([q("d", 0, k) for k in range(dim)], dtype=object)
        return s
    val = np.array([q("v", c) for c in range(dim)], dtype=object)
    grad = np.array([[q("d", c, k) for k in range(dim)] for c in range(dim)], dtype=object)
    return SymField(val, grad)


class SymParams(dict):
    """The ``w`` argument: coefficient fields become symbols, numbers pass."""

    def __init__(self, fields, numbers_):
        super().__init__()
        for k in fields:
            self[k] = Sym({(None, None, (k,)): 1.0})
        for k, v in numbers_.items():
            self[k] = v

    def __getattr__(self, name):
        if name in self:
            return self[name]
        self._missing(name)

    def __getitem__(self, name):
        if name in self.keys():
            return dict.__getitem__(self, name)
        self._missing(name)

    @staticmethod
    def _missing(name):
        if name in ("x", "h"):
            raise NotImplementedError(
                "w.%s (quadrature-point %s) is not supported by the GPU kernels; pass "
                "per-element coefficient arrays instead" % (name, "coordinates" if name == "x"
                                                            else "mesh parameter"))
        raise AttributeError("Attribute '{}' not found in 'w'.".format(name))


def _scalarize(r):
    if isinstance(r, np.ndarray):
        if r.ndim != 0:
            raise ValueError("form must return a scalar field (got shape %s)" % (r.shape,))
        r = r.item()
    return Sym.lift(r)


def trace_bilinear(form, elem, dim, fields, numbers_):
    u = _field("u", elem, dim)
    v = _field("v", elem, dim)
    return _scalarize(form(u, v, SymParams(fields, numbers_)))


def trace_linear(form, elem, dim, fields, numbers_):
    v = _field("v", elem, dim)
    return _scalarize(form(v, SymParams(fields, numbers_)))


def _poly_table(sym):
    tab = {}
    for (uq, vq, f), c in sym.terms.items():
        tab.setdefault((uq, vq), Poly())
        tab[(uq, vq)] = tab[(uq, vq)].add(Poly({f: c}))
    return tab


def bilinear_channels(sym, elem, dim):
    """Map a traced bilinear form onto {diff, mass} (scalar) or
    {lam, lap, tr, mass} (vector) coefficient polynomials."""
    tab = _poly_table(sym)
    for (uq, vq) in tab:
        if uq is None or vq is None:
            raise NotImplementedError("form has terms that are not bilinear in (u, v)")
    zero = Poly()
    get = lambda uq, vq: tab.get((uq, vq), zero)  # noqa: E731
    used = set()
    if not elem.vector:
        diff = get(("d", 0, 0), ("d", 0, 0))
        for k in range(dim):
            for l in range(dim):
                p = get(("d", 0, k), ("d", 0, l))
                used.add((("d", 0, k), ("d", 0, l)))
                ref = diff if k == l else zero
                if not p.close(ref):
                    raise NotImplementedError(
                        "only isotropic diffusion k*dot(grad u, grad v) is implemented")
        mass = get(("v", 0), ("v", 0))
        used.add((("v", 0), ("v", 0)))
        rest = set(tab) - used
        if any(not tab[k].is_zero() for k in rest):
            raise NotImplementedError("form has value-derivative (advection-type) terms")
        return {"diff": diff, "mass": mass}
    # vector: T[(b,k),(a,l)] for d_k u_b d_l v_a
    if dim < 2:
        raise NotImplementedError("vector forms need dim >= 2")
    lam = get(("d", 0, 0), ("d", 1, 1))
    lap = get(("d", 0, 1), ("d", 0, 1))
    tr = get(("d", 0, 1), ("d", 1, 0))
    for b in range(dim):
        for k in range(dim):
            for a in range(dim):
                for l in range(dim):
                    key = (("d", b, k), ("d", a, l))
                    used.add(key)
                    ref = zero
                    if b == k and a == l:
                        ref = ref.add(lam)
                    if a == b and k == l:
                        ref = ref.add(lap)
                    if b == l and k == a:
                        ref = ref.add(tr)
                    if not get(*key).close(ref):
                        raise NotImplementedError(
                            "vector form is not of the isotropic form lam*div(u)div(v) + "
                            "lap*ddot(grad u, grad v) + tr*ddot(grad u, grad v^T)")
    mass = get(("v", 0), ("v", 0))
    for a in range(dim):
        for b in range(dim):
            key = (("v", b), ("v", a))
            used.add(key)
            if not get(*key).close(mass if a == b else zero):
                raise NotImplementedError("vector mass term must be c * dot(u, v)")
    rest = set(tab) - used
    if any(not tab[k].is_zero() for k in rest):
        raise NotImplementedError("form has value-derivative (advection-type) terms")
    return {"lam": lam, "lap": lap, "tr": tr, "mass": mass}


def linear_channels(sym, elem, dim):
    tab = _poly_table(sym)
    for (uq, vq) in tab:
        if uq is not None or vq is None:
            raise NotImplementedError("linear form must be linear in v only")
    if elem.vector:
        raise NotImplementedError("linear forms on vector bases are not implemented")
    load = tab.get((None, ("v", 0)), Poly())
    rest = set(tab) - {(None, ("v", 0))}
    if any(not tab[k].is_zero() for k in rest):
        raise NotImplementedError("only f * v load forms are implemented")
    return {"load": load}


# ---------------------------------------------------------------------------
# Exact-order tape (the pattern build's eliminate_zeros mask)
# ---------------------------------------------------------------------------
# The reference evaluates a form with numpy ufuncs and einsum on float64
# arrays; on the reference's platform every einsum contraction is a plain
# sequential sum in row-major index order without fused multiply-add, which
# is also the order numpy's einsum uses on object arrays.  Running the form
# on TapeNode objects therefore records, per quadrature point, the exact
# sequence of separately rounded operations the reference performs.  The
# CUDA mask kernel replays it for the local entries whose value is
# rounding noise, so that the entries the reference computes as exactly
# 0.0 -- and drops in eliminate_zeros -- are the entries dropped here.
#
# The same program is what the generic kernels evaluate for forms outside
# the coefficient channels above (anisotropic and advection terms,
# coefficients that vary inside cells, interpolated DOF vectors, the
# default parameters w.x and w.h, numpy functions of fields).

(OP_CONST, OP_U, OP_V, OP_COEF, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG, OP_X, OP_H,
 OP_SQRT, OP_EXP, OP_LOG, OP_SIN, OP_COS, OP_TAN, OP_TANH, OP_ARCTAN, OP_ABS,
 OP_POW, OP_N) = range(22)

# ops that are correctly rounded on both sides (the rest use libm)
EXACT_OPS = {OP_CONST, OP_U, OP_V, OP_COEF, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG, OP_X, OP_H,
             OP_SQRT, OP_ABS, OP_N}


class Tape:
    def __init__(self):
        self.ins = []
        self.consts = {}
        self.loads = {}

    def emit(self, op, a=-1, b=-1, imm=0.0):
        self.ins.append((op, a, b, float(imm)))
        return len(self.ins) - 1

    def const(self, c):
        c = float(c)
        key = (c, np.signbit(c))
        if key not in self.consts:
            self.consts[key] = self.emit(OP_CONST, imm=c)
        return TapeNode(self, self.consts[key])

    def load(self, op, k):
        if (op, k) not in self.loads:
            self.loads[(op, k)] = self.emit(op, a=k)
        return TapeNode(self, self.loads[(op, k)])


def _unary(op):
    def f(x):
        if isinstance(x, TapeNode):
            return TapeNode(x.tape, x.tape.emit(op, x.idx))
        return _NUMPY_UNARY[op](x)
    return f


def _binary(fn):
    return lambda a, b: fn(a, b)


_NUMPY_UNARY = {OP_SQRT: np.sqrt, OP_EXP: np.exp, OP_LOG: np.log, OP_SIN: np.sin,
                OP_COS: np.cos, OP_TAN: np.tan, OP_TANH: np.tanh, OP_ARCTAN: np.arctan,
                OP_ABS: np.abs, OP_NEG: np.negative}

_UFUNCS = {
    np.sqrt: _unary(OP_SQRT), np.exp: _unary(OP_EXP), np.log: _unary(OP_LOG),
    np.sin: _unary(OP_SIN), np.cos: _unary(OP_COS), np.tan: _unary(OP_TAN),
    np.tanh: _unary(OP_TANH), np.arctan: _unary(OP_ARCTAN), np.absolute: _unary(OP_ABS),
    np.negative: _unary(OP_NEG), np.positive: lambda x: x,
    np.add: _binary(lambda a, b: a + b), np.subtract: _binary(lambda a, b: a - b),
    np.multiply: _binary(lambda a, b: a * b), np.true_divide: _binary(lambda a, b: a / b),
    np.power: _binary(lambda a, b: a ** b),
    np.square: lambda x: x * x,
}


class TapeNode:
    """One recorded value (a register of the form program)."""
    __slots__ = ("tape", "idx", "grad")

    def __init__(self, tape, idx):
        self.tape, self.idx, self.grad = tape, idx, None

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        fn = _UFUNCS.get(ufunc)
        if method != "__call__" or kwargs or fn is None:
            raise NotImplementedError("numpy.%s is not supported in forms assembled on the GPU"
                                      % getattr(ufunc, "__name__", ufunc))
        if any(isinstance(x, np.ndarray) and x.ndim > 0 for x in inputs):
            return np.frompyfunc(fn, len(inputs), 1)(*inputs)
        return fn(*inputs)

    def _lift(self, o):
        if isinstance(o, TapeNode):
            return o
        if isinstance(o, numbers.Number):
            return self.tape.const(o)
        if isinstance(o, np.ndarray) and o.ndim == 0:
            return self._lift(o.item())
        raise TypeError("cannot combine %r with a traced form quantity" % type(o))

    def _bin(self, op, o, rev=False):
        if isinstance(o, np.ndarray) and o.ndim > 0:
            return np.frompyfunc(lambda x: self._bin(op, x, rev), 1, 1)(o)
        o = self._lift(o)
        a, b = (o, self) if rev else (self, o)
        return TapeNode(self.tape, self.tape.emit(op, a.idx, b.idx))

    def __add__(self, o):
        return self._bin(OP_ADD, o)

    def __radd__(self, o):
        return self._bin(OP_ADD, o, rev=True)

    def __sub__(self, o):
        return self._bin(OP_SUB, o)

    def __rsub__(self, o):
        return self._bin(OP_SUB, o, rev=True)

    def __mul__(self, o):
        return self._bin(OP_MUL, o)

    def __rmul__(self, o):
        return self._bin(OP_MUL, o, rev=True)

    def __truediv__(self, o):
        return self._bin(OP_DIV, o)

    def __rtruediv__(self, o):
        return self._bin(OP_DIV, o, rev=True)

    def __neg__(self):
        return TapeNode(self.tape, self.tape.emit(OP_NEG, self.idx))

    def __pos__(self):
        return self

    def __abs__(self):
        return TapeNode(self.tape, self.tape.emit(OP_ABS, self.idx))

    def __pow__(self, n):
        # numpy's scalar-exponent fast paths: x**2 = x*x, x**0.5 = sqrt(x),
        # x**-1 = 1/x, x**1 = x, x**0 = 1; other exponents call pow
        if isinstance(n, np.ndarray) and n.ndim == 0:
            n = n.item()
        if isinstance(n, numbers.Number) and not isinstance(n, TapeNode):
            if n == 2:
                return self * self
            if n == 1:
                return self
            if n == 0.5:
                return TapeNode(self.tape, self.tape.emit(OP_SQRT, self.idx))
            if n == -1:
                return self.tape.const(1.0) / self
            if n == 0:
                return self.tape.const(1.0)
        return self._bin(OP_POW, n)

    def __rpow__(self, o):
        return self._bin(OP_POW, o, rev=True)

    @property
    def value(self):
        return self

    @property
    def shape(self):
        return ()


class FieldSpec:
    """How a form argument appears to the program: 'elem' (one value per
    cell) and 'qp' (one per quadrature point) are scalar slots; 'field' is
    a DiscreteField -- ncomp value components (0: a scalar field) and, with
    grad, the gradient components, each a per-point slot."""

    def __init__(self, kind, ncomp=0, grad=False):
        self.kind, self.ncomp, self.grad = kind, ncomp, grad

    def quantities(self, dim):
        n = max(self.ncomp, 1)
        return n + (n * dim if self.grad else 0)


class TapeParams(dict):
    def __init__(self, tape, fields, numbers_, dim=None, defaults=False):
        super().__init__()
        self.slots = {}
        self.tape = tape
        specs = fields if isinstance(fields, dict) else {k: FieldSpec("elem") for k in fields}
        for k, s in specs.items():
            if s.kind in ("elem", "qp"):
                self[k] = self._slot(k)
            else:
                self[k] = self._field(k, s, dim)
        for k, v in numbers_.items():
            self[k] = v
        if defaults:
            # CellBasis.default_parameters (cell_basis.py:124-141);
            # FacetBasis adds the unit outward normal (facet_basis.py:112-118)
            if "x" not in self:
                self["x"] = SymField(np.array([tape.load(OP_X, i) for i in range(dim)],
                                              dtype=object))
            if "h" not in self:
                self["h"] = tape.load(OP_H, 0)
            if defaults == "facet" and "n" not in self:
                self["n"] = SymField(np.array([tape.load(OP_N, i) for i in range(dim)],
                                              dtype=object))

    def _slot(self, key):
        if key not in self.slots:
            self.slots[key] = len(self.slots)
        return self.tape.load(OP_COEF, self.slots[key])

    def _field(self, name, s, dim):
        if s.ncomp == 0:
            node = self._slot((name, 0))
            if s.grad:
                node.grad = np.array([self._slot((name, 1 + k)) for k in range(dim)],
                                     dtype=object)
            return node
        n = s.ncomp
        val = np.array([self._slot((name, c)) for c in range(n)], dtype=object)
        grad = None
        if s.grad:
            grad = np.array([[self._slot((name, n + c * dim + k)) for k in range(dim)]
                             for c in range(n)], dtype=object)
        return SymField(val, grad)

    __getattr__ = SymParams.__getattr__
    __getitem__ = SymParams.__getitem__
    _missing = SymParams._missing


def _tape_field(tape, which, elem, dim):
    """Quantity k: value of component c -> c; derivative k of component c ->
    ncomp + c*dim + k (ncomp = dim for vector bases, 1 for scalar)."""
    op = OP_U if which == "u" else OP_V
    if not elem.vector:
        s = tape.load(op, 0)
        s.grad = np.array([tape.load(op, 1 + k) for k in range(dim)], dtype=object)
        return s
    val = np.array([tape.load(op, c) for c in range(dim)], dtype=object)
    grad = np.array([[tape.load(op, dim + c * dim + k) for k in range(dim)] for c in range(dim)],
                    dtype=object)
    return SymField(val, grad)


def _compact(ins, out, slots):
    """Drop coefficient slots the output does not depend on (their loads
    become constants) and renumber the rest densely."""
    live = set()
    stack = [out]
    while stack:
        k = stack.pop()
        if k in live:
            continue
        live.add(k)
        op, a, b, _ = ins[k]
        if op in (OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_POW):
            stack += [a, b]
        elif op in (OP_NEG, OP_SQRT, OP_EXP, OP_LOG, OP_SIN, OP_COS, OP_TAN, OP_TANH,
                    OP_ARCTAN, OP_ABS):
            stack.append(a)
    by_index = {v: k for k, v in slots.items()}
    names, remap = [], {}
    new = []
    for k, (op, a, b, imm) in enumerate(ins):
        if op == OP_COEF:
            if k not in live:
                new.append((OP_CONST, -1, -1, 0.0))
                continue
            if a not in remap:
                remap[a] = len(names)
                names.append(by_index[a])
            new.append((op, remap[a], b, imm))
        else:
            new.append((op, a, b, imm))
    return new, names


def trace_tape(form, elem, dim, fields, numbers_, kind="bilinear", defaults=False, uelem=None):
    """Record the exact-order program of a form; returns (instructions,
    output index, coefficient slot keys).  kind: 'bilinear' (form(u, v, w)),
    'linear' (form(v, w)) or 'functional' (form(w)).  defaults: True / 'cell'
    adds w.x and w.h, 'facet' also w.n.  fields: names of
    per-element coefficients, or {name: FieldSpec}; slot keys are the names
    ('elem'/'qp') or (name, quantity) pairs ('field').  uelem: the trial
    element when it differs from the test element ``elem``."""
    tape = Tape()
    w = TapeParams(tape, fields, numbers_, dim=dim, defaults=defaults)
    if kind == "bilinear":
        u = _tape_field(tape, "u", uelem if uelem is not None else elem, dim)
        v = _tape_field(tape, "v", elem, dim)
        r = form(u, v, w)
    elif kind == "linear":
        r = form(_tape_field(tape, "v", elem, dim), w)
    else:
        r = form(w)
    if isinstance(r, np.ndarray):
        if r.ndim != 0:
            raise ValueError("form must return a scalar field")
        r = r.item()
    if not isinstance(r, TapeNode):
        r = tape.const(r)
    ins, names = _compact(tape.ins, r.idx, w.slots)
    return ins, r.idx, names
