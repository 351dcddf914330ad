"""Python front end: expression trees over SoA arrays, serialised to aether-ir/1.

The names follow the reference's consumer surface (expr/Operations.h:25-71,
expr/nodes/Elementwise.h:499-851, expr/Expression.h:127-486, random/Generator.h:
56-195) so a test reads like the reference's own: `d = a + b*c +
cwiseSin(a)*cwiseExp((c*c)*(-1.0))`. Building an expression does no work;
`assign(dst, expr)` lowers it to one kernel through the C-ABI.
"""

import math as _math

MASK64 = (1 << 64) - 1


def _shape_text(shape):
    return "[" + ",".join(str(int(s)) for s in shape) + "]"


def _prod(shape):
    p = 1
    for s in shape:
        p *= s
    return p


class IrContext:
    """Slot assignment for one plan: operands by buffer identity, scalars and
    generator keys in order of first use."""

    def __init__(self):
        self.operands = []     # (ptr, pitch, dtype, comps, owner)
        self._op_index = {}
        self.scalars = []
        self.keys = []
        self._key_index = {}

    def operand(self, leaf):
        k = (leaf.ptr, leaf.pitch, leaf.dtype, leaf.comps)
        if k not in self._op_index:
            self._op_index[k] = len(self.operands)
            self.operands.append((leaf.ptr, leaf.pitch, leaf.dtype, leaf.comps, leaf.owner))
        return self._op_index[k]

    def scalar(self, v):
        self.scalars.append(float(v))
        return len(self.scalars) - 1

    def key(self, key):
        if key not in self._key_index:
            self._key_index[key] = len(self.keys)
            self.keys.append(key)
        return self._key_index[key]


class Expr:
    shape = ()
    is_bool = False

    # -- arithmetic (expr/Operations.h:25-71) -------------------------------
    def __add__(self, o):
        return Node("add", (self, _as_expr(o, self.shape)), self.shape)

    def __radd__(self, o):
        return Node("add", (_as_expr(o, self.shape), self), self.shape)

    def __sub__(self, o):
        return Node("sub", (self, _as_expr(o, self.shape)), self.shape)

    def __rsub__(self, o):
        return Node("sub", (_as_expr(o, self.shape), self), self.shape)

    def __mul__(self, o):
        if isinstance(o, (int, float)):
            return Node("scale", (self, Scalar(o)), self.shape)   # e * s (CWiseScale: factor * e)
        if isinstance(o, Expr) and o.shape == () and self.shape != ():
            return Node("scale", (self, o), self.shape)
        return Node("mul", (self, o), self.shape)

    def __rmul__(self, o):
        if isinstance(o, (int, float)):
            return Node("scale", (self, Scalar(o)), self.shape)   # s * e
        return Node("mul", (o, self), self.shape)

    def __truediv__(self, o):
        if isinstance(o, (int, float)):
            # e / s is e * (1/s), the reciprocal rounded once (Operations.h:67-71)
            return Node("scale", (self, Scalar(1.0 / float(o))), self.shape)
        return Node("div", (self, o), self.shape)

    def __neg__(self):
        return Node("neg", (self,), self.shape)

    def __gt__(self, o):
        return Node("gt", (self, _as_expr(o, self.shape)), self.shape, is_bool=True)

    def __lt__(self, o):
        return Node("lt", (self, _as_expr(o, self.shape)), self.shape, is_bool=True)

    def __ge__(self, o):
        return Node("ge", (self, _as_expr(o, self.shape)), self.shape, is_bool=True)

    def __le__(self, o):
        return Node("le", (self, _as_expr(o, self.shape)), self.shape, is_bool=True)

    # -- member surface of Expression<Derived,T> (expr/Expression.h) --------
    def dot(self, o):
        return Node("dot", (self, o), ())

    def squaredNorm(self):
        return Node("sqnorm", (self,), ())

    def norm(self):
        return Node("norm", (self,), ())

    def rNorm(self):
        return Node("rnorm", (self,), ())

    def sum(self):
        return Node("sum", (self,), ())

    def rSquaredNorm(self):
        """1 / |e|^2 (Expression.h:182)."""
        return Node("div", (Literal(1.0), self.squaredNorm()), ())

    def cubedNorm(self):
        """|e|^2 |e| (Expression.h:183)."""
        return Node("mul", (self.squaredNorm(), self.norm()), ())

    def rCubedNorm(self):
        """1 / (|e|^2 |e|) (Expression.h:184)."""
        return Node("div", (Literal(1.0), self.cubedNorm()), ())

    def matDot(self, o):
        """Sum over every component of e * o, matrices included (Expression.h:205-207)."""
        n = 1
        for d in self.shape:
            n *= d
        return self.reshape((n,)).dot(o.reshape((n,)))

    def maxNorm(self):
        return Node("maxnorm", (self,), ())

    def cross(self, o):
        return Node("cross", (self, o), (3,))

    def unitVector(self):
        return Node("unit", (self,), self.shape)

    def quatMul(self, o):
        return Node("qmul", (self, o), (4,))

    def quatConj(self):
        return Node("qconj", (self,), (4,))

    def quatRotate(self, v):
        return Node("qrot", (self, v), (3,))

    def asPureQuaternion(self):
        return Node("pureq", (self,), (4,))

    def quatReciprocal(self):
        """conj(q) / |q|^2 (Expression.h:220-222)."""
        return Node("scale", (self.quatConj(), self.rSquaredNorm()), (4,))

    def asBack3DVector(self):
        """The vector part (x, y, z) of a quaternion (Expression.h:228)."""
        return self.tail(3)

    def inverse(self):
        return Node("inv", (self,), self.shape)

    def det(self):
        return Node("det", (self,), ())

    def trace(self):
        return Node("trace", (self,), ())

    def transpose(self):
        return Node("transpose", (self,), (self.shape[1], self.shape[0]))

    def row(self, r):
        return Node("row", (self,), (self.shape[1],), ints=(r,))

    def col(self, c):
        return Node("col", (self,), (self.shape[0],), ints=(c,))

    def segment(self, off, length):
        return Node("seg", (self,), (length,), ints=(off, length))

    def head(self, n):
        return self.segment(0, n)

    def tail(self, n):
        return self.segment(self.shape[0] - n, n)

    def block(self, r0, c0, br, bc):
        return Node("block", (self,), (br, bc), ints=(r0, c0, br, bc))

    def component(self, k):
        return Node("comp", (self,), (), ints=(k,))

    def matvec(self, v):
        return Node("matvec", (self, v), (self.shape[0],))

    def matmul(self, o):
        return Node("matmul", (self, o), (self.shape[0], o.shape[1]))

    def outer(self, o):
        return Node("outer", (self, o), (self.shape[0], o.shape[0]))

    def reshape(self, shape):
        return Node("reshape", (self,), tuple(shape), tail_text=_shape_text(shape))

    def at_sample0(self):
        return Node("at0", (self,), self.shape, is_bool=self.is_bool)

    def __repr__(self):
        return "<aether expr %s>" % self.ir(IrContext())


class Node(Expr):
    def __init__(self, op, kids, shape, is_bool=False, ints=(), tail_text=None):
        self.op = op
        self.kids = tuple(kids)
        self.shape = tuple(shape)
        self.is_bool = is_bool
        self.ints = tuple(ints)
        self.tail_text = tail_text

    def ir(self, ctx):
        parts = [k.ir(ctx) for k in self.kids]
        parts += [str(i) for i in self.ints]
        if self.tail_text:
            parts.append(self.tail_text)
        return "(" + self.op + " " + " ".join(parts) + ")"


class Operand(Expr):
    """A SoA array read as an expression leaf (view/View.h:369-377)."""

    def __init__(self, ptr, pitch, dtype, shape, owner=None):
        self.ptr = int(ptr)
        self.pitch = int(pitch)
        self.dtype = dtype
        self.shape = tuple(shape)
        self.comps = _prod(self.shape)
        self.owner = owner
        self.is_bool = dtype == "u8"

    def ir(self, ctx):
        return "(in %d %s %s)" % (ctx.operand(self), self.dtype, _shape_text(self.shape))


class Scalar(Expr):
    """A runtime scalar (a CWiseScale factor, a bound, a parameter)."""

    shape = ()

    def __init__(self, v):
        self.v = float(v)

    def ir(self, ctx):
        # a non-negative value is marked so the plan can drop cancellation-safe sums
        return ("(sc %d +)" if self.v >= 0.0 else "(sc %d)") % ctx.scalar(self.v)


class Literal(Expr):
    """A compile-time scalar baked into the kernel."""

    shape = ()

    def __init__(self, v):
        self.v = float(v)

    def ir(self, ctx):
        return "(lit %s)" % float(self.v).hex()


class Bcast(Expr):
    def __init__(self, s, shape):
        self.s = s
        self.shape = tuple(shape)

    def ir(self, ctx):
        return "(bcast %s %s)" % (self.s.ir(ctx), _shape_text(self.shape))


def _as_expr(o, shape):
    if isinstance(o, Expr):
        if o.shape == () and shape != ():
            return Bcast(o, shape)
        return o
    s = Scalar(o)
    return Bcast(s, shape) if shape != () else s


# Constants the kernels bake in (a handful of values, so the plan cache stays
# small): their magnitude bounds let the generator drop range tests.
_LITERAL_CONSTANTS = (1.0, -1.0, 2.0, 0.5)


def constant(value, shape):
    """aether::constant<extents<...>>(v) (expr/nodes/Constant.h:98-150)."""
    v = float(value)
    s = Literal(v) if v in _LITERAL_CONSTANTS else Scalar(v)
    return Bcast(s, shape) if tuple(shape) != () else s


def literal(value):
    return Literal(value)


def stack(*items):
    return Node("stack", items, (len(items),))


def _unary(op):
    def f(e):
        return Node(op, (e,), e.shape)
    f.__name__ = op
    return f


cwiseSqrt = _unary("sqrt")
cwiseRsqrt = _unary("rsqrt")
cwiseExp = _unary("exp")
cwiseExpm1 = _unary("expm1")
cwiseLog = _unary("log")
cwiseLog1p = _unary("log1p")
cwiseSin = _unary("sin")
cwiseCos = _unary("cos")
cwiseTan = _unary("tan")
cwiseAsin = _unary("asin")
cwiseAcos = _unary("acos")
cwiseAtan = _unary("atan")
cwiseTanh = _unary("tanh")
cwiseAbs = _unary("abs")
cwiseSign = _unary("sign")
cwiseSquare = _unary("sq")
cwiseSinh = _unary("sinh")
cwiseCosh = _unary("cosh")
cwiseExp2 = _unary("exp2")
cwiseLog2 = _unary("log2")
cwiseLog10 = _unary("log10")
cwiseCbrt = _unary("cbrt")
cwiseErf = _unary("erf")
cwiseFloor = _unary("floor")
cwiseCeil = _unary("ceil")
cwiseTrunc = _unary("trunc")


def cwiseMul(l, r):
    """Hadamard product (expr/nodes/Elementwise.h cwiseMul): the same node as l * r."""
    return l * r


def cwiseMin(e, o):
    if isinstance(o, Expr) and o.shape == e.shape:
        return Node("min", (e, o), e.shape)
    return Node("mins", (e, o if isinstance(o, Expr) else Scalar(o)), e.shape)


def cwiseMax(e, o):
    if isinstance(o, Expr) and o.shape == e.shape:
        return Node("max", (e, o), e.shape)
    return Node("maxs", (e, o if isinstance(o, Expr) else Scalar(o)), e.shape)


def clamp(e, lo, hi):
    return Node("clamp", (e, Scalar(lo) if not isinstance(lo, Expr) else lo,
                          Scalar(hi) if not isinstance(hi, Expr) else hi), e.shape)


def cwiseDiv(l, r):
    return Node("div", (l, r), l.shape)


def cwisePow(e, p):
    if isinstance(p, Expr) and p.shape == e.shape:
        return Node("pow", (e, p), e.shape)
    return Node("pows", (e, p if isinstance(p, Expr) else Scalar(p)), e.shape)


def select(cond, a, b):
    return Node("select", (cond, a, b), a.shape)


# ---------------------------------------------------------------------------
# Random leaves (random/Generator.h:56-195, random/detail/DistributionLeaf.h).
# ---------------------------------------------------------------------------
def splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & MASK64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & MASK64
    return x ^ (x >> 31)


class Generator:
    """Seed-carrying handle: key = splitmix64(seed ^ splitmix64(stream_id))."""

    SALT = 0x2545F4914F6CDD1D

    def __init__(self, seed, stream_id=0, _key=None):
        self.key = _key if _key is not None else splitmix64((seed & MASK64) ^ splitmix64(stream_id & MASK64))

    def substream(self, k):
        return Generator(0, _key=splitmix64(self.key ^ splitmix64((k & MASK64) ^ self.SALT)))

    def _leaf(self, op, vd, params):
        return RandomLeaf(op, self.key, vd, params)

    def uniform(self, vd, lo, hi):
        return self._leaf("uniform", vd, (lo, hi))

    def normal(self, vd, mean, sd):
        return self._leaf("normal", vd, (mean, sd))

    def lognormal(self, vd, mu, sigma):
        return self._leaf("lognormal", vd, (mu, sigma))

    def exponential(self, vd, lam):
        return self._leaf("exponential", vd, (lam,))

    def bernoulli(self, vd, p):
        return self._leaf("bernoulli", vd, (p,))


class RandomLeaf(Expr):
    def __init__(self, op, key, vd, params):
        self.op = op
        self.key = key
        self.shape = (vd,)
        # N(0, 1) keeps its parameters as literals: the kernel then skips the
        # affine step 0 + 1 z, which is z bit for bit (a Box-Muller draw is never 0)
        standard = (op in ("normal", "lognormal") and not any(isinstance(p, Expr) for p in params)
                    and float(params[0]) == 0.0 and float(params[1]) == 1.0)
        self.params = tuple(p if isinstance(p, Expr) else (Literal(p) if standard else Scalar(p)) for p in params)

    def ir(self, ctx):
        ps = " ".join(p.ir(ctx) for p in self.params)
        return "(%s %d %s %d)" % (self.op, ctx.key(self.key), ps, self.shape[0])


def plan_text(dst_dtype, dst_shape, op, expr, ctx):
    return "(plan %s %s %s %s)" % (dst_dtype, _shape_text(dst_shape), op, expr.ir(ctx))
