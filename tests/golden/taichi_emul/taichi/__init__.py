"""Serial emulator of the subset of the Taichi 1.2 Python API that tiSPHi uses.

Test infrastructure only: tests/golden/make_golden.py puts this package first on
sys.path so that the reference's unmodified source (eng/*.py) imports and runs in plain
CPython, producing golden vectors for the f64 oracle.  It is never imported by the
product or by the GPU tests.

What is emulated, following Taichi's documented semantics:
* ``@ti.kernel`` / ``@ti.func``: the function source is re-parsed and rewritten so that
  ``ti.template()`` arguments are passed by reference (accumulators like ``ret += ...``),
  atomics act on field elements, and ``x.attr[k] = v`` stores reach struct fields.
  Outermost loops of a kernel run serially in index order unless an order hook is set
  (``set_loop_order``), which lets a caller pick one valid serialisation of a parallel loop.
* vectors / matrices (``ti.Vector``, ``ti.Matrix``, ``ti.types.vector/matrix``) with
  value semantics, elementwise ``*``, ``@`` as matrix product, and reductions (norm, dot,
  sum, trace) accumulated left to right;
* ``ti.field`` scalars and 1-D fields, vector fields, ``@ti.dataclass`` struct fields;
* ``ti.pow`` (binary exponentiation for integer exponents, libm pow otherwise),
  ``ti.sqrt``, ``ti.max``, ``ti.min``, ``ti.abs``, ``ti.sin``, ``ti.tan``, ``ti.ceil``,
  ``ti.grouped``, ``ti.ndrange``, ``ti.static``, ``PrefixSumExecutor`` (inclusive scan).
A read of a 1-D field outside its bounds returns 0 and is counted in ``oob_reads``: the
reference's neighbour loop indexes one cell past either end of the grid, which Taichi
does not check; returning 0 makes such a cell empty.
"""
import ast
import builtins
import inspect
import math as _m
import random as _random
import textwrap

import numpy as np

f64, f32, i32, i64, u8 = "f64", "f32", "i32", "i64", "u8"
gpu, cpu, cuda, vulkan = "gpu", "cpu", "cuda", "vulkan"

oob_reads = [0]
_loop_order = {}


def init(*args, **kwargs):
    return None


def loop_config(*args, **kwargs):
    return None


def static(x, *rest):
    return x


def data_oriented(cls):
    return cls


def set_loop_order(key, fn):
    """Order hook for a kernel's outermost loop: key = (qualname, loop index)."""
    if fn is None:
        _loop_order.pop(key, None)
    else:
        _loop_order[key] = fn


class _Template:
    pass


def template():
    return _Template()


class _Ndarray:
    pass


# ---------------------------------------------------------------- values
class Mat:
    """Taichi vector (n, 1) or matrix (n, m) value."""

    __slots__ = ("a",)

    def __init__(self, a):
        a = np.asarray(a)
        if a.ndim == 1:
            a = a.reshape(-1, 1)
        if a.dtype.kind not in "fiub":
            a = a.astype(np.float64)
        if a.dtype.kind == "b":
            a = a.astype(np.int64)
        self.a = a.copy()

    # -- shape helpers
    @property
    def n(self):
        return self.a.shape[0]

    @property
    def m(self):
        return self.a.shape[1]

    def _vec(self):
        return self.a.shape[1] == 1

    def copy(self):
        return Mat(self.a)

    # -- indexing
    def __getitem__(self, k):
        if isinstance(k, tuple):
            return self.a[k].item()
        if self._vec():
            return self.a[k, 0].item()
        if self.a.shape[0] == 1:
            return self.a[0, k].item()
        return Mat(self.a[k])

    def __setitem__(self, k, v):
        if isinstance(k, tuple):
            self.a[k] = v
        elif self._vec():
            self.a[k, 0] = v
        else:
            self.a[k] = v

    @property
    def x(self):
        return self[0]

    @x.setter
    def x(self, v):
        self[0] = v

    @property
    def y(self):
        return self[1]

    @y.setter
    def y(self, v):
        self[1] = v

    @property
    def z(self):
        return self[2]

    @z.setter
    def z(self, v):
        self[2] = v

    # -- arithmetic (elementwise; numpy applies one IEEE operation per element)
    @staticmethod
    def _v(o):
        return o.a if isinstance(o, Mat) else o

    def __add__(self, o): return Mat(self.a + Mat._v(o))
    def __radd__(self, o): return Mat(Mat._v(o) + self.a)
    def __sub__(self, o): return Mat(self.a - Mat._v(o))
    def __rsub__(self, o): return Mat(Mat._v(o) - self.a)
    def __mul__(self, o): return Mat(self.a * Mat._v(o))
    def __rmul__(self, o): return Mat(Mat._v(o) * self.a)
    def __truediv__(self, o): return Mat(self.a / Mat._v(o))
    def __rtruediv__(self, o): return Mat(Mat._v(o) / self.a)
    def __neg__(self): return Mat(-self.a)
    def __abs__(self): return Mat(np.abs(self.a))
    def __lt__(self, o): return Mat(self.a < Mat._v(o))
    def __gt__(self, o): return Mat(self.a > Mat._v(o))

    def __pow__(self, e):
        if isinstance(e, int):
            out = np.empty_like(self.a, dtype=np.float64)
            for idx in np.ndindex(self.a.shape):
                out[idx] = _pow_scalar(float(self.a[idx]), e)
            return Mat(out)
        return Mat(self.a ** e)

    def __matmul__(self, o):
        A, B = self.a, o.a
        assert A.shape[1] == B.shape[0], (A.shape, B.shape)
        out = np.zeros((A.shape[0], B.shape[1]), dtype=np.result_type(A, B, np.float64))
        for r in range(A.shape[0]):
            for c in range(B.shape[1]):
                s = A[r, 0] * B[0, c]
                for k in range(1, A.shape[1]):
                    s = s + A[r, k] * B[k, c]
                out[r, c] = s
        return Mat(out)

    def __bool__(self):
        # all(mat) in a Taichi kernel is the elementwise all; Python's all() iterates the
        # rows and takes each row's truth value: all of its elements
        return bool(np.all(self.a != 0))

    def __iter__(self):
        if self._vec():
            return iter([v.item() for v in self.a[:, 0]])
        return iter([Mat(r) for r in self.a])

    def __len__(self):
        return self.a.shape[0]

    # -- reductions, left to right
    def sum(self):
        flat = self.a.reshape(-1)
        s = flat[0]
        for v in flat[1:]:
            s = s + v
        return s.item() if hasattr(s, "item") else s

    def norm_sqr(self):
        return (self * self).sum()

    def norm(self):
        return _m.sqrt(self.norm_sqr())

    def dot(self, o):
        return (self * o).sum()

    def transpose(self):
        return Mat(self.a.T)

    def trace(self):
        s = self.a[0, 0]
        for k in range(1, builtins.min(self.a.shape)):
            s = s + self.a[k, k]
        return s.item()

    def cast(self, t):
        if t in (int, i32, i64):
            return Mat(np.trunc(self.a).astype(np.int64))
        return Mat(self.a.astype(np.float64))

    def determinant(self):
        return _determinant(self)

    def inverse(self):
        return _inverse(self)

    def outer_product(self, o):
        return self @ o.transpose()

    def to_numpy(self):
        return self.a.reshape(-1).copy() if self._vec() else self.a.copy()

    def __repr__(self):
        return f"Mat({self.a.tolist()})"


def _determinant(M):
    a = M.a
    if a.shape == (2, 2):
        return (a[0, 0] * a[1, 1] - a[0, 1] * a[1, 0]).item()
    if a.shape == (3, 3):
        return (a[0, 0] * (a[1, 1] * a[2, 2] - a[2, 1] * a[1, 2]) - a[1, 0] * (a[0, 1] * a[2, 2] - a[2, 1] * a[0, 2])
                + a[2, 0] * (a[0, 1] * a[1, 2] - a[1, 1] * a[0, 2])).item()
    return float(np.linalg.det(a))


def _inverse(M):
    a = M.a.astype(np.float64)
    if a.shape == (2, 2):
        inv = 1.0 / _determinant(M)
        return Mat(np.array([[inv * a[1, 1], inv * (-a[0, 1])], [inv * (-a[1, 0]), inv * a[0, 0]]]))
    if a.shape == (3, 3):
        inv = 1.0 / _determinant(M)
        out = np.zeros((3, 3))
        for i in range(3):
            for j in range(3):
                out[j, i] = inv * (a[(i + 1) % 3, (j + 1) % 3] * a[(i + 2) % 3, (j + 2) % 3]
                                   - a[(i + 2) % 3, (j + 1) % 3] * a[(i + 1) % 3, (j + 2) % 3])
        return Mat(out)
    return Mat(np.linalg.inv(a))


def _pow_scalar(x, e):
    if isinstance(e, (int, np.integer)) and not isinstance(e, bool):
        n = int(e)
        neg = n < 0
        n = abs(n)
        r = 1.0 if not isinstance(x, (int, np.integer)) else 1
        first = True
        base = x
        while n > 0:
            if n & 1:
                r = base if first else r * base
                first = False
            n >>= 1
            if n:
                base = base * base
        return 1.0 / r if neg else r
    return _m.pow(x, e)


def _as_mat_args(args):
    if len(args) == 1:
        v = args[0]
        if isinstance(v, Mat):
            return v.a
        if isinstance(v, (list, tuple)):
            if v and isinstance(v[0], (list, tuple, np.ndarray)):
                return np.array([[float(q) if not isinstance(q, (int, np.integer)) else q for q in row] for row in v])
            return np.array(v)
        return np.asarray(v)
    if all(isinstance(v, (list, tuple)) for v in args):
        return np.array(args)
    return np.array(args)


class _VectorFactory:
    def __call__(self, *args, **kwargs):
        if len(args) >= 2 and isinstance(args[1], str) and isinstance(args[0], (list, tuple)):
            args = args[:1]
        a = _as_mat_args(args)
        return Mat(a.reshape(-1, 1))

    @staticmethod
    def zero(dtype, n):
        return Mat(np.zeros((n, 1), dtype=np.int64 if dtype in (int, i32) else np.float64))


class _MatrixFactory:
    def __call__(self, *args, **kwargs):
        a = _as_mat_args(args)
        if a.ndim == 1:
            a = a.reshape(-1, 1)
        return Mat(a)

    @staticmethod
    def identity(dtype, n):
        return Mat(np.eye(n))


Vector = _VectorFactory()
Matrix = _MatrixFactory()


class _VecType:
    def __init__(self, n, dtype):
        self.n, self.dtype = n, dtype

    def __call__(self, *args):
        if len(args) == 1 and isinstance(args[0], (int, float)) and not isinstance(args[0], bool):
            return Mat(np.full((self.n, 1), float(args[0])))
        a = _as_mat_args(args).astype(np.float64)
        return Mat(a.reshape(self.n, 1))

    def field(self, shape=(), **kw):
        return _StructField({"_v": ("vec", (self.n, 1))}, shape, value_member="_v")


class _MatType:
    def __init__(self, n, m, dtype):
        self.n, self.m, self.dtype = n, m, dtype

    def __call__(self, *args):
        if len(args) == 1 and isinstance(args[0], (int, float)) and not isinstance(args[0], bool):
            return Mat(np.full((self.n, self.m), float(args[0])))
        if len(args) == self.n and all(isinstance(r, (list, tuple)) for r in args):
            return Mat(np.array(args, dtype=np.float64))
        a = _as_mat_args(args).astype(np.float64)
        return Mat(a.reshape(self.n, self.m))

    def field(self, shape=(), **kw):
        return _StructField({"_v": ("mat", (self.n, self.m))}, shape, value_member="_v")


class types:
    @staticmethod
    def vector(n, dtype):
        return _VecType(n, dtype)

    @staticmethod
    def matrix(n, m, dtype):
        return _MatType(n, m, dtype)

    @staticmethod
    def ndarray(*args, **kwargs):
        return _Ndarray()


# ``ti.math`` namespace (shadowing the stdlib name only as an attribute of this module)
class _TiMath:
    pi = _m.pi

    @staticmethod
    def eye(n):
        return Mat(np.eye(n))

    @staticmethod
    def determinant(M):
        return _determinant(M)

    @staticmethod
    def inverse(M):
        return _inverse(M)


# ---------------------------------------------------------------- scalar functions
def _scalar_or_elem(f, x):
    if isinstance(x, Mat):
        out = np.empty(x.a.shape, dtype=np.float64)
        for idx in np.ndindex(x.a.shape):
            out[idx] = f(float(x.a[idx]))
        return Mat(out)
    return f(x)


def _sqrt(v):
    return _m.sqrt(v) if v >= 0 else float("nan")


def sqrt(x): return _scalar_or_elem(_sqrt, x)
def sin(x): return _scalar_or_elem(_m.sin, x)
def cos(x): return _scalar_or_elem(_m.cos, x)
def tan(x): return _scalar_or_elem(_m.tan, x)
def exp(x): return _scalar_or_elem(_m.exp, x)
def log(x): return _scalar_or_elem(_m.log, x)
def ceil(x): return _m.ceil(x) if not isinstance(x, Mat) else Mat(np.ceil(x.a))
def floor(x): return _m.floor(x) if not isinstance(x, Mat) else Mat(np.floor(x.a))


def abs(x):  # noqa: A001
    return Mat(np.abs(x.a)) if isinstance(x, Mat) else (x if x >= 0 else -x)


def max(a, b):  # noqa: A001
    if isinstance(a, Mat) or isinstance(b, Mat):
        return Mat(np.maximum(Mat._v(a), Mat._v(b)))
    return a if a >= b else b


def min(a, b):  # noqa: A001
    if isinstance(a, Mat) or isinstance(b, Mat):
        return Mat(np.minimum(Mat._v(a), Mat._v(b)))
    return a if a <= b else b


def pow(x, e):  # noqa: A001
    if isinstance(x, Mat):
        return x ** e
    if isinstance(e, float):
        return _m.pow(x, e)
    return _pow_scalar(x, e)


def cast(x, t):
    if isinstance(x, Mat):
        return x.cast(t)
    return int(x) if t in (int, i32, i64) else float(x)


def random(dtype=float):
    return _random.random()


def polar_decompose(A):
    """(R, S) with R the orthogonal polar factor of the 3x3 matrix A and S = R^T A.

    Taichi's own routine is not available here; the emulator uses the algorithm the oracle
    and the CUDA forms restate, in the same operation order (Python floats are IEEE f64):
    Higham's scaled Newton iteration X <- (g X + X^-T / g) / 2, g = (|X^-1|_F / |X|_F)^(1/2),
    X^-T from the cofactors, until an update changes X by at most 1e-14 (Frobenius) or after
    60 steps; a zero third row and column (2D body) gets A[2][2] = 1 first; a singular
    matrix gives the identity."""
    a = A.a.astype(np.float64)
    x = [[float(a[r, c]) for c in range(3)] for r in range(3)]
    if x[0][2] == 0.0 and x[1][2] == 0.0 and x[2][0] == 0.0 and x[2][1] == 0.0 and x[2][2] == 0.0:
        x[2][2] = 1.0
    eye = [[1.0 if r == c else 0.0 for c in range(3)] for r in range(3)]
    R = None
    for _ in range(60):
        c = [[0.0] * 3 for _ in range(3)]
        c[0][0] = x[1][1] * x[2][2] - x[1][2] * x[2][1]
        c[0][1] = x[1][2] * x[2][0] - x[1][0] * x[2][2]
        c[0][2] = x[1][0] * x[2][1] - x[1][1] * x[2][0]
        c[1][0] = x[0][2] * x[2][1] - x[0][1] * x[2][2]
        c[1][1] = x[0][0] * x[2][2] - x[0][2] * x[2][0]
        c[1][2] = x[0][1] * x[2][0] - x[0][0] * x[2][1]
        c[2][0] = x[0][1] * x[1][2] - x[0][2] * x[1][1]
        c[2][1] = x[0][2] * x[1][0] - x[0][0] * x[1][2]
        c[2][2] = x[0][0] * x[1][1] - x[0][1] * x[1][0]
        det = (x[0][0] * c[0][0] + x[0][1] * c[0][1]) + x[0][2] * c[0][2]
        if det == 0.0 or not _m.isfinite(det):
            R = eye
            break
        fx = 0.0
        fy = 0.0
        y = [[0.0] * 3 for _ in range(3)]
        for r in range(3):
            for k in range(3):
                y[r][k] = c[r][k] / det
                fx += x[r][k] * x[r][k]
                fy += y[r][k] * y[r][k]
        gm = _m.sqrt(_m.sqrt(fy) / _m.sqrt(fx))
        ch = 0.0
        xn = [[0.0] * 3 for _ in range(3)]
        for r in range(3):
            for k in range(3):
                xn[r][k] = 0.5 * (gm * x[r][k] + y[r][k] / gm)
                d = xn[r][k] - x[r][k]
                ch += d * d
        x = xn
        if ch <= 1e-28:
            break
    if R is None:
        R = x
    Rm = Mat(np.array(R, dtype=np.float64))
    return Rm, Rm.transpose() @ A


# ---------------------------------------------------------------- fields
class _ScalarField:
    def __init__(self, dtype):
        self.dtype = dtype
        self.v = 0 if dtype in (int, i32, i64) else 0.0

    def __getitem__(self, k):
        return self.v

    def __setitem__(self, k, v):
        self.v = int(v) if self.dtype in (int, i32, i64) else float(v)


class _Field1D:
    def __init__(self, dtype, n):
        self.dtype = dtype
        self.data = np.zeros(n, dtype=np.int64 if dtype in (int, i32, i64) else np.float64)
        self.shape = (n,)

    def _idx(self, k):
        if isinstance(k, tuple):
            k = k[0]
        return int(k)

    def __getitem__(self, k):
        i = self._idx(k)
        if i < 0 or i >= self.data.shape[0]:
            oob_reads[0] += 1
            return 0
        return self.data[i].item()

    def __setitem__(self, k, v):
        i = self._idx(k)
        if i < 0 or i >= self.data.shape[0]:
            raise IndexError(f"write outside field bounds: {i}")
        self.data[i] = v

    def fill(self, v):
        self.data[:] = v

    def to_numpy(self):
        return self.data.copy()

    def from_numpy(self, a):
        self.data[:] = a


def field(dtype, shape=(), **kwargs):
    if shape == () or shape is None:
        return _ScalarField(dtype)
    n = shape if isinstance(shape, int) else int(np.prod(shape))
    return _Field1D(dtype, n)


class _StructRef:
    __slots__ = ("_f", "_i")

    def __init__(self, f, i):
        object.__setattr__(self, "_f", f)
        object.__setattr__(self, "_i", i)

    def __getattr__(self, name):
        f = self._f
        if name in f.members:
            kind, _ = f.members[name]
            v = f.store[name][self._i]
            if kind == "sca":
                return v.item()
            return Mat(v)
        meth = f.methods.get(name)
        if meth is not None:
            return meth.__get__(self, type(self))
        raise AttributeError(name)

    def __setattr__(self, name, value):
        f = self._f
        kind, _ = f.members[name]
        if kind == "sca":
            f.store[name][self._i] = value
        else:
            f.store[name][self._i][...] = Mat._v(value) if isinstance(value, Mat) else np.asarray(value).reshape(
                f.store[name][self._i].shape)


class _StructField:
    def __init__(self, members, shape, methods=None, value_member=None):
        self.members = members
        self.methods = methods or {}
        self.value_member = value_member
        n = 1 if shape == () else (shape if isinstance(shape, int) else int(np.prod(shape)))
        self.n = n
        self.shape = (n,)
        self.store = {}
        for name, (kind, shp) in members.items():
            dt = np.int64 if shp == "int" else np.float64
            if kind == "sca":
                self.store[name] = np.zeros(n, dtype=dt)
            else:
                self.store[name] = np.zeros((n,) + shp, dtype=np.float64)

    def _idx(self, k):
        if k is None:
            return 0
        if isinstance(k, tuple):
            k = k[0]
        return int(k)

    def __getitem__(self, k):
        i = self._idx(k)
        if i < 0 or i >= self.n:
            raise IndexError(i)
        if self.value_member:
            return Mat(self.store[self.value_member][i])
        return _StructRef(self, i)

    def __setitem__(self, k, v):
        i = self._idx(k)
        if self.value_member:
            self.store[self.value_member][i][...] = Mat._v(v)
            return
        src = v
        for name in self.members:
            if isinstance(src, _StructRef):
                val = src._f.store[name][src._i]
            else:
                raise TypeError("struct assignment needs a struct value")
            self.store[name][i] = val

    def __getattr__(self, name):
        members = object.__getattribute__(self, "members")
        if name in members:
            return _MemberView(self, name)
        raise AttributeError(name)


class _MemberView:
    """``field.member`` handle (e.g. ``ps.pt.id0``) indexable like a field."""

    def __init__(self, f, name):
        self.f, self.name = f, name
        self.shape = f.shape

    def __getitem__(self, k):
        i = self.f._idx(k)
        kind, _ = self.f.members[self.name]
        v = self.f.store[self.name][i]
        return v.item() if kind == "sca" else Mat(v)

    def to_numpy(self):
        return self.f.store[self.name].copy()


class _StructType:
    def __init__(self, cls):
        self.cls = cls
        self.members = {}
        for name, ann in cls.__dict__.get("__annotations__", {}).items():
            if isinstance(ann, _VecType):
                self.members[name] = ("vec", (ann.n, 1))
            elif isinstance(ann, _MatType):
                self.members[name] = ("mat", (ann.n, ann.m))
            elif ann in (int, i32, i64):
                self.members[name] = ("sca", "int")
            else:
                self.members[name] = ("sca", "float")
        self.methods = {k: v for k, v in cls.__dict__.items() if isinstance(v, _TiFunc)}

    def field(self, shape=(), **kw):
        return _StructField(self.members, shape, methods=self.methods)


def dataclass(cls):
    return _StructType(cls)


struct_class = dataclass


# ---------------------------------------------------------------- loops
def ndrange(*ranges):
    spans = []
    for r in ranges:
        if isinstance(r, (tuple, list)):
            spans.append(range(int(r[0]), int(r[1])))
        else:
            spans.append(range(int(r)))
    import itertools
    for t in itertools.product(*spans):
        yield t


def grouped(x):
    if isinstance(x, (_Field1D, _StructField)):
        for i in range(x.shape[0]):
            yield (i,)
        return
    for t in x:
        yield Mat(np.array(t, dtype=np.int64))


class algorithms:
    class PrefixSumExecutor:
        def __init__(self, n):
            self.n = n

        def run(self, f):
            f.data[:] = np.cumsum(f.data)


# ---------------------------------------------------------------- kernels / funcs
class _Box:
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = v


def _is_value(a):
    return isinstance(a, (int, float, np.integer, np.floating, Mat)) and not isinstance(a, bool)


def __ti_deref(x):
    return x.v if isinstance(x, _Box) else x


def __ti_aug(target, op, value):
    if isinstance(target, _Box):
        target.v = _apply(op, target.v, value)
        return target
    return _apply(op, target, value)


def _apply(op, a, b):
    if op == "add":
        return a + b
    if op == "sub":
        return a - b
    if op == "mul":
        return a * b
    if op == "div":
        return a / b
    raise NotImplementedError(op)


def __ti_call(f, *args):
    mask = getattr(f, "_ti_mask", None)
    if mask is None:
        f(*args)
        return list(args)
    call_args = []
    boxed = []
    for k, a in enumerate(args):
        is_t = mask[k] if k < len(mask) else False
        if is_t and _is_value(a) and not isinstance(a, _Box):
            call_args.append(_Box(a.copy() if isinstance(a, Mat) else a))
            boxed.append(True)
        else:
            call_args.append(a)
            boxed.append(False)
    f(*call_args)
    return [c.v if b else c for c, b in zip(call_args, boxed)]


def __ti_atomic(op, container, index, value):
    old = container[index]
    if op == "add":
        new = old + value
    elif op == "sub":
        new = old - value
    elif op == "max":
        new = max(old, value)
    elif op == "min":
        new = min(old, value)
    else:
        raise NotImplementedError(op)
    container[index] = new
    return old


def __ti_atomic_local(op, old, value):
    if op == "add":
        return old + value
    if op == "sub":
        return old - value
    if op == "max":
        return max(old, value)
    if op == "min":
        return min(old, value)
    raise NotImplementedError(op)


def __ti_setsub(obj, attr, index, value):
    m = getattr(obj, attr)
    m[index] = value
    setattr(obj, attr, m)


def __ti_loop(key, it):
    fn = _loop_order.get(key)
    seq = list(it)
    if fn is None:
        return seq
    return fn(seq)


def call_with_refs(f, *args):
    """Call a ti.func from Python scope with template arguments passed by reference;
    returns the final values of all arguments (boxed values are unboxed)."""
    return __ti_call(f, *args)


_HELPERS = {"__ti_deref": __ti_deref, "__ti_aug": __ti_aug, "__ti_call": __ti_call, "__ti_atomic": __ti_atomic,
            "__ti_atomic_local": __ti_atomic_local, "__ti_setsub": __ti_setsub, "__ti_loop": __ti_loop}


def _is_ti_attr(node, names):
    return (isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name) and node.value.id == "ti"
            and node.attr in names)


class _Rewrite(ast.NodeTransformer):
    OPS = {ast.Add: "add", ast.Sub: "sub", ast.Mult: "mul", ast.Div: "div"}

    def __init__(self, template_params, kernel_key):
        self.tp = set(template_params)
        self.kernel_key = kernel_key
        self.depth = 0
        self.loop_counter = 0

    # keep function bodies, drop decorators
    def visit_FunctionDef(self, node):
        node.decorator_list = []
        node.body = self._stmts(node.body, top=True)
        return node

    def _stmts(self, body, top=False):
        out = []
        for st in body:
            if top and self.kernel_key is not None and isinstance(st, ast.For):
                key = ast.Tuple(elts=[ast.Constant(self.kernel_key), ast.Constant(self.loop_counter)], ctx=ast.Load())
                self.loop_counter += 1
                st.iter = ast.Call(func=ast.Name("__ti_loop", ast.Load()), args=[key, self.visit(st.iter)], keywords=[])
                st.body = self._stmts(st.body)
                st.orelse = self._stmts(st.orelse)
                out.append(st)
                continue
            r = self.visit(st)
            if isinstance(r, list):
                out.extend(r)
            elif r is not None:
                out.append(r)
        return out

    def visit_For(self, node):
        node.iter = self.visit(node.iter)
        node.body = self._stmts(node.body)
        node.orelse = self._stmts(node.orelse)
        return node

    def visit_While(self, node):
        node.test = self.visit(node.test)
        node.body = self._stmts(node.body)
        return node

    def visit_If(self, node):
        node.test = self.visit(node.test)
        node.body = self._stmts(node.body)
        node.orelse = self._stmts(node.orelse)
        return node

    def visit_Name(self, node):
        if isinstance(node.ctx, ast.Load) and node.id in self.tp:
            return ast.Call(func=ast.Name("__ti_deref", ast.Load()), args=[node], keywords=[])
        return node

    def visit_Expr(self, node):
        call = node.value
        if isinstance(call, ast.Call):
            # atomics on a local accumulator: NAME = op(NAME, v)
            if _is_ti_attr(call.func, {"atomic_add", "atomic_sub", "atomic_max", "atomic_min"}) and \
                    isinstance(call.args[0], ast.Name):
                op = call.func.attr.split("_")[1]
                name = call.args[0].id
                return ast.Assign(targets=[ast.Name(name, ast.Store())],
                                  value=ast.Call(func=ast.Name("__ti_atomic_local", ast.Load()),
                                                 args=[ast.Constant(op), ast.Name(name, ast.Load()),
                                                       self.visit(call.args[1])], keywords=[]))
            name_args = [k for k, a in enumerate(call.args) if isinstance(a, ast.Name)]
            if name_args and not _is_ti_attr(call.func, {"atomic_add", "atomic_sub", "atomic_max", "atomic_min"}):
                args = [a if isinstance(a, ast.Name) else self.visit(a) for a in call.args]
                tmp = f"__ti_r{id(node)}"
                stmts = [ast.Assign(targets=[ast.Name(tmp, ast.Store())],
                                    value=ast.Call(func=ast.Name("__ti_call", ast.Load()),
                                                   args=[self.visit(call.func)] + args, keywords=[]))]
                for k in name_args:
                    nm = call.args[k].id
                    stmts.append(ast.Assign(targets=[ast.Name(nm, ast.Store())],
                                            value=ast.Subscript(value=ast.Name(tmp, ast.Load()),
                                                                slice=ast.Constant(k), ctx=ast.Load())))
                return stmts
        node.value = self.visit(call)
        return node

    def visit_Call(self, node):
        if _is_ti_attr(node.func, {"atomic_add", "atomic_sub", "atomic_max", "atomic_min"}) and \
                isinstance(node.args[0], ast.Subscript):
            op = node.func.attr.split("_")[1]
            sub = node.args[0]
            return ast.Call(func=ast.Name("__ti_atomic", ast.Load()),
                            args=[ast.Constant(op), self.visit(sub.value), self.visit(sub.slice),
                                  self.visit(node.args[1])], keywords=[])
        self.generic_visit(node)
        return node

    def visit_AugAssign(self, node):
        op = self.OPS.get(type(node.op))
        if isinstance(node.target, ast.Name) and node.target.id in self.tp and op:
            nm = node.target.id
            return ast.Assign(targets=[ast.Name(nm, ast.Store())],
                              value=ast.Call(func=ast.Name("__ti_aug", ast.Load()),
                                             args=[ast.Name(nm, ast.Load()), ast.Constant(op), self.visit(node.value)],
                                             keywords=[]))
        if isinstance(node.target, ast.Subscript) and isinstance(node.target.value, ast.Attribute) and op:
            # X.attr[k] op= v  ->  __ti_setsub(X, 'attr', k, X.attr[k] op v)
            tgt = node.target
            load = ast.Subscript(value=ast.Attribute(value=self.visit(tgt.value.value), attr=tgt.value.attr,
                                                     ctx=ast.Load()), slice=self.visit(tgt.slice), ctx=ast.Load())
            val = ast.BinOp(left=load, op=node.op, right=self.visit(node.value))
            return ast.Expr(ast.Call(func=ast.Name("__ti_setsub", ast.Load()),
                                     args=[self.visit(tgt.value.value), ast.Constant(tgt.value.attr),
                                           self.visit(tgt.slice), val], keywords=[]))
        node.value = self.visit(node.value)
        if isinstance(node.target, ast.Attribute):
            node.target.value = self.visit(node.target.value)
        elif isinstance(node.target, ast.Subscript):
            node.target.value = self.visit(node.target.value)
            node.target.slice = self.visit(node.target.slice)
        return node

    def visit_Assign(self, node):
        if len(node.targets) == 1 and isinstance(node.targets[0], ast.Subscript) and \
                isinstance(node.targets[0].value, ast.Attribute):
            tgt = node.targets[0]
            return ast.Expr(ast.Call(func=ast.Name("__ti_setsub", ast.Load()),
                                     args=[self.visit(tgt.value.value), ast.Constant(tgt.value.attr),
                                           self.visit(tgt.slice), self.visit(node.value)], keywords=[]))
        node.value = self.visit(node.value)
        for t in node.targets:
            if isinstance(t, ast.Attribute):
                t.value = self.visit(t.value)
            elif isinstance(t, ast.Subscript):
                t.value = self.visit(t.value)
                t.slice = self.visit(t.slice)
        return node


class _TiFunc:
    """Rewritten @ti.func / @ti.kernel (template arguments by reference)."""

    def __init__(self, fn, kernel):
        self.fn = fn
        self.kernel = kernel
        self._compiled = None
        sig = inspect.signature(fn)
        params = list(sig.parameters.values())
        self.params = params
        self.tp = [p.name for p in params if isinstance(p.annotation, _Template)]
        first_self = params and params[0].name == "self"
        self._mask_unbound = [isinstance(p.annotation, _Template) for p in params]
        self._mask_bound = self._mask_unbound[1:] if first_self else self._mask_unbound
        self._ti_mask = self._mask_unbound
        self.__name__ = fn.__name__
        self.__qualname__ = fn.__qualname__

    def _compile(self):
        if self._compiled is None:
            src = textwrap.dedent(inspect.getsource(self.fn))
            tree = ast.parse(src)
            key = self.fn.__qualname__ if self.kernel else None
            tree = _Rewrite(self.tp, key).visit(tree)
            ast.fix_missing_locations(tree)
            code = compile(tree, filename=inspect.getsourcefile(self.fn) or "<ti>", mode="exec")
            g = dict(self.fn.__globals__)
            g.update(_HELPERS)
            loc = {}
            exec(code, g, loc)
            self._compiled = loc[self.fn.__name__]
        return self._compiled

    def __call__(self, *args, **kwargs):
        args = [a.copy() if isinstance(a, Mat) else a for a in args]
        return self._compile()(*args, **kwargs)

    def __get__(self, obj, objtype=None):
        if obj is None:
            return self
        return _Bound(self, obj)


class _Bound:
    def __init__(self, f, obj):
        self.f = f
        self.obj = obj
        self._ti_mask = f._mask_bound

    def __call__(self, *args, **kwargs):
        args = [a.copy() if isinstance(a, Mat) else a for a in args]
        return self.f._compile()(self.obj, *args, **kwargs)


def func(fn):
    return _TiFunc(fn, kernel=False)


def kernel(fn):
    return _TiFunc(fn, kernel=True)


# attribute namespaces expected by the reference
math = _TiMath
ui = None
