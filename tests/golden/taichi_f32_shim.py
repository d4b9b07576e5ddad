"""Float32 stand-in for the subset of the Taichi API used by the reference's
atmosphere kernels.  TEST INFRASTRUCTURE ONLY: it exists so that the
reference's own kernel source (``src/planet_renderer/atmosphere/renderer.py``)
can execute unmodified, on the CPU, in this container where Taichi is not
installed, to produce golden input/output vectors.  Nothing in the product
imports it.

Semantics mirrored from Taichi with ``default_fp=f32``
(``src/planet_renderer/cli.py:65-69``):

* every kernel argument annotated ``ti.f32`` / ``ti.types.vector(3, ti.f32)``
  is rounded to float32 on entry;
* Python float constants meeting an f32 value are rounded to f32 at that
  operation (numpy >= 2 "weak scalar" promotion gives exactly this), while
  arithmetic between two Python constants stays in double, as Taichi's AST
  builder evaluates it at trace time;
* vectors have value semantics (``+=`` rebinds, never aliases);
* ``ti.cast(x, ti.i32)`` truncates; ``ti.math.clamp(x, a, b)`` is
  ``min(max(x, a), b)``.

Known differences from compiled Taichi: Taichi's LLVM backends may contract
``a*b+c`` into FMA and use their own libm; both change results at the level
of a few float32 ULPs, far below the 1e-3 parity tolerance.

Iteration over a field can be restricted to a subset of indices with
:func:`restrict_iteration`, so full-size LUTs can be sampled at a few texels.
"""

from __future__ import annotations

import builtins as _builtins
import itertools
import math as _pymath
import sys
import types

import numpy as np

f32 = np.float32
i32 = np.int32
f64 = np.float64
# integer and other types that only appear in annotations and field
# declarations of modules the golden scripts import but do not run
u8 = np.uint8
u16 = np.uint16
u32 = np.uint32
class _U64:
    """ti.u64: a field dtype, and as a call a Python integer (numpy uint64
    does not mix with Python integers in bit operations)."""

    def __call__(self, value):
        return int(value) & 0xFFFFFFFFFFFFFFFF


u64 = _U64()
i8 = np.int8
i16 = np.int16
i64 = np.int64
f16 = np.float16

_F = np.float32


_FLOAT = np.float32


def set_precision(name: str) -> None:
    """"f32" (default, Taichi default_fp=f32) or "f64": run the same kernel
    source in double, to separate algorithm differences from f32 rounding."""

    global _FLOAT
    _FLOAT = np.float32 if name == "f32" else np.float64


def _check_f32(value) -> None:
    """Reject float64 numpy values: they would silently raise precision."""

    dtype = getattr(value, "dtype", None)
    if _FLOAT is np.float32 and dtype is not None and dtype == np.float64:
        raise TypeError("float64 value reached an f32 kernel expression")


class Vec(np.ndarray):
    """Small float32 vector with Taichi's ``x/y/z``, ``dot``, ``norm``."""

    def __new__(cls, data, dtype=None):
        dtype = _FLOAT if dtype is None else dtype
        if isinstance(data, (list, tuple)):
            for item in data:
                _check_f32(item)
        else:
            _check_f32(data)
        return np.array(data, dtype=dtype).view(cls)

    def __array_finalize__(self, obj):  # noqa: D401 - numpy hook
        return None

    @property
    def x(self):
        return self[0]

    @property
    def y(self):
        return self[1]

    @property
    def z(self):
        return self[2]

    @property
    def w(self):
        return self[3]

    def __getitem__(self, item):
        value = np.ndarray.__getitem__(self, item)
        if isinstance(value, np.ndarray) and value.ndim == 0:
            return value[()]
        return value

    def dot(self, other):  # ((a0*b0 + a1*b1) + a2*b2) in float32
        acc = self[0] * other[0]
        for k in range(1, self.shape[0]):
            acc = acc + self[k] * other[k]
        return acc

    def cross(self, other):
        a, b = self, other
        return Vec([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]],
                   dtype=self.dtype)

    def norm_sqr(self):
        return self.dot(self)

    def norm(self):
        return np.sqrt(self.dot(self))

    def normalized(self, eps=0):
        # Taichi: invlen = 1 / (norm + eps); return invlen * self
        invlen = 1 / (self.norm() + eps)
        return invlen * self

    # value semantics for augmented assignment
    def __iadd__(self, other):
        return np.add(self, other).view(Vec)

    def __isub__(self, other):
        return np.subtract(self, other).view(Vec)

    def __imul__(self, other):
        return np.multiply(self, other).view(Vec)

    def __itruediv__(self, other):
        return np.true_divide(self, other).view(Vec)


class IndexVec(tuple):
    """Grouped loop index (``pixel.x``, ``pixel.y``) usable as a field key."""

    @property
    def x(self):
        return self[0]

    @property
    def y(self):
        return self[1]

    @property
    def z(self):
        return self[2]


_RESTRICT: dict[int, list[tuple[int, ...]]] = {}


def restrict_iteration(field, indices) -> None:
    """Make loops over ``field`` visit only ``indices`` (list of tuples)."""

    _RESTRICT[id(field)] = [tuple(int(v) for v in idx) for idx in indices]


def clear_restrictions() -> None:
    _RESTRICT.clear()


class IntRef(int):
    """An integer read from a scalar field element that remembers where it
    came from, so that ``ti.atomic_add(field[i], v)`` can update the field
    (Python passes the value, not the element)."""

    def __new__(cls, value, field, key):
        obj = int.__new__(cls, int(value))
        obj.field, obj.key = field, key
        return obj


class Field:
    """Dense field: vector elements (n>0) or scalars (n=0)."""

    def __init__(self, n, dtype, shape):
        self.n = int(n)
        if dtype in (f32, float):
            self.dtype = _FLOAT
        elif dtype is u64:
            self.dtype = np.uint64
        elif dtype in (u32, i64):
            self.dtype = np.dtype(dtype).type
        else:
            self.dtype = np.int32
        self.shape = tuple(int(s) for s in (shape if isinstance(shape, tuple) else (shape,)))
        full = self.shape + ((self.n,) if self.n else ())
        self.data = np.zeros(full, dtype=self.dtype)

    def _key(self, idx):
        if idx is None:
            return ()
        if isinstance(idx, (tuple, list, np.ndarray)):
            return tuple(int(v) for v in idx)
        return (int(idx),)

    def __getitem__(self, idx):
        key = self._key(idx)
        if self.n:
            return Vec(self.data[key], dtype=self.dtype)
        value = self.data[key]
        if np.issubdtype(self.dtype, np.integer):
            return IntRef(value, self, key)
        return value

    def __setitem__(self, idx, value):
        key = self._key(idx)
        _check_f32(value)
        if np.issubdtype(self.dtype, np.integer) and not self.n:
            self.data[key] = self.dtype(int(value))
        else:
            self.data[key] = np.asarray(value, dtype=self.dtype)

    def _indices(self):
        if id(self) in _RESTRICT:
            return iter(_RESTRICT[id(self)])
        return itertools.product(*(range(s) for s in self.shape))

    def __iter__(self):
        return self._indices()

    def to_numpy(self):
        return self.data.copy()

    def from_numpy(self, array):
        self.data[...] = np.asarray(array, dtype=self.dtype)

    def fill(self, value):
        self.data[...] = value


class _VectorNamespace:
    def __call__(self, values, dt=None):
        items = list(values) if isinstance(values, (list, tuple)) else None
        if items and all(isinstance(v, (int, np.integer)) and not isinstance(v, bool) for v in items):
            return Vec(items, dtype=np.int64)  # an integer vector (ti.i32)
        return Vec(values)

    @staticmethod
    def zero(dtype, n):
        if dtype is i32:
            return Vec(np.zeros(n, dtype=np.int64), dtype=np.int64)
        return Vec(np.zeros(n, dtype=_FLOAT))

    @staticmethod
    def field(n, dtype=f32, shape=()):
        return Field(n, dtype, shape)


Vector = _VectorNamespace()


class Mat(np.ndarray):
    """Small matrix with value semantics; ``m[k, :]`` is a row vector."""

    def __setitem__(self, item, value):
        # write through the base array (numpy routes a subclass's slice
        # assignment through its __getitem__, which returns copies here)
        np.ndarray.__setitem__(self.view(np.ndarray), item, np.asarray(value))

    def __getitem__(self, item):
        value = np.ndarray.__getitem__(self, item)
        if isinstance(value, np.ndarray):
            if value.ndim == 0:
                return value[()]
            if value.ndim == 1:
                return Vec(np.array(value), dtype=value.dtype)
        return value


class _MatrixNamespace:
    @staticmethod
    def rows(rows):
        return np.array([np.asarray(r) for r in rows]).view(Mat)

    @staticmethod
    def zero(dtype, r, c):
        return np.zeros((r, c), dtype=np.int64 if dtype is i32 else _FLOAT).view(Mat)


Matrix = _MatrixNamespace()


def atomic_add(ref, value):
    """Add to the field element ``ref`` was read from; returns the old value."""

    old = int(ref.field.data[ref.key])
    ref.field.data[ref.key] = ref.field.dtype(old + int(value))
    return old


def atomic_min(ref, value):
    old = int(ref.field.data[ref.key])
    ref.field.data[ref.key] = ref.field.dtype(_builtins.min(old, int(value)))
    return old


def bit_cast(value, dtype):
    if dtype is u32:
        return int(np.array(value, dtype=np.float32).view(np.uint32))
    if dtype is f32:
        return np.array(int(value), dtype=np.uint32).view(np.float32)[()]
    raise TypeError(f"bit_cast to {dtype} not supported")


def loop_config(**kwargs):
    return None


def field(dtype=f32, shape=()):
    return Field(0, dtype, shape)


def grouped(fld):
    for idx in fld._indices():
        yield IndexVec(idx)


def ndrange(*sizes):
    """Sizes are extents or (start, stop) pairs."""

    ranges = [range(int(s[0]), int(s[1])) if isinstance(s, (tuple, list)) else range(int(s)) for s in sizes]
    return itertools.product(*ranges)


def static(value):
    return value


def cast(value, dtype):
    if dtype in (u64, u32):
        return int(value)
    if dtype is i32:
        if isinstance(value, (np.ndarray, tuple, list)):  # vectors: element-wise, truncating
            return Vec(np.trunc(np.asarray(value, dtype=np.float64)).astype(np.int64), dtype=np.int64)
        return int(value)
    if isinstance(value, (tuple, list)):
        return Vec([_FLOAT(v) for v in value])
    return _FLOAT(value)


def select(cond, a, b):
    return a if cond else b


def _is_py(value) -> bool:
    """A Python scalar: Taichi evaluates ops on these at trace time."""

    return isinstance(value, (bool, int, float)) and not isinstance(
        value, (np.generic, np.ndarray)
    )


def _unary(np_op, py_op):
    def op(x):
        if _is_py(x):
            return py_op(x)
        return np_op(x)

    return op


exp = _unary(np.exp, _pymath.exp)
sqrt = _unary(np.sqrt, _pymath.sqrt)
acos = _unary(np.arccos, _pymath.acos)
cos = _unary(np.cos, _pymath.cos)
sin = _unary(np.sin, _pymath.sin)
abs = _unary(np.abs, _builtins.abs)  # noqa: A001 - mirrors ti.abs
floor = _unary(np.floor, _pymath.floor)
ceil = _unary(np.ceil, _pymath.ceil)
tan = _unary(np.tan, _pymath.tan)


def pow(x, a):  # noqa: A001 - mirrors ti.pow
    if _is_py(x) and _is_py(a):
        return x ** a
    return np.power(x, _FLOAT(a) if _is_py(a) else a)


def atan2(y, x):
    if _is_py(y) and _is_py(x):
        return _pymath.atan2(y, x)
    return np.arctan2(y, x)


def max(a, b, *more):  # noqa: A001 - mirrors ti.max
    if more:
        return max(max(a, b), *more)
    if _is_py(a) and _is_py(b):
        return _builtins.max(a, b)
    return np.maximum(a, b)


def min(a, b, *more):  # noqa: A001 - mirrors ti.min
    if more:
        return min(min(a, b), *more)
    if _is_py(a) and _is_py(b):
        return _builtins.min(a, b)
    return np.minimum(a, b)


class _Math:
    @staticmethod
    def clamp(x, lo, hi):
        return min(max(x, lo), hi)

    @staticmethod
    def fract(x):
        return x - floor(x)

    pi = _pymath.pi


math = _Math()


class _Template:
    pass


def template():
    return _Template()


class _VectorType:
    def __init__(self, n, dtype):
        self.n = n
        self.dtype = dtype


class _Annotation:
    """Placeholder for annotations of kernels the golden scripts never call."""

    def __init__(self, *args, **kwargs):
        self.args, self.kwargs = args, kwargs


class _Types:
    @staticmethod
    def vector(n, dtype):
        return _VectorType(n, dtype)

    ndarray = _Annotation
    matrix = _Annotation


types_ = _Types()


def _convert(annotation, value):
    if annotation is f32:
        return _FLOAT(value)
    if annotation is i32:
        return int(value)
    if isinstance(annotation, _VectorType):
        return Vec([_FLOAT(v) for v in value])
    return value


def kernel(fn):
    import inspect

    signature = inspect.signature(fn)

    def wrapper(*args, **kwargs):
        bound = signature.bind(*args, **kwargs)
        for name, value in list(bound.arguments.items()):
            annotation = signature.parameters[name].annotation
            if annotation is inspect.Parameter.empty:
                continue
            bound.arguments[name] = _convert(annotation, value)
        return fn(*bound.args, **bound.kwargs)

    wrapper.__wrapped__ = fn
    return wrapper


def func(fn):
    return fn


def data_oriented(cls):
    return cls


def init(*args, **kwargs):
    return None


def sync():
    return None


cpu = "cpu"
cuda = "cuda"
gpu = "gpu"
vulkan = "vulkan"


def install() -> types.ModuleType:
    """Register this module as ``taichi`` in ``sys.modules``."""

    module = sys.modules[__name__]
    module.types = types_  # ``ti.types.vector``
    sys.modules["taichi"] = module
    return module
