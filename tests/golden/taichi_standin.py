"""A minimal Python stand-in for the part of Taichi that the reference's plugin kernels use, so
that the golden-fixture generators beside this file can execute the reference's own kernel
source in this container, where Taichi is not installed.  It is test infrastructure only:
nothing outside tests/golden imports it.

Semantics: a `ti.kernel` or `ti.func` runs as the plain Python function it decorates, serially;
`ti.ndrange` is a nested range.  Fields are NumPy arrays of their dtype (f32 -> float32,
i32 -> int32), so scalar arithmetic on field values stays in float32 as it does in Taichi (NumPy's
promotion keeps float32 against Python scalars).  Vectors are float32 NumPy arrays with .x/.y/.z,
.norm() and .dot(); `ti.cast` of a vector is a vector of the new type.  `ti.random()` returns 0.5.  Parallel-for atomics, struct-for over fields,
SNodes and autodiff are not provided: a generator that reaches them fails loudly.
"""
import itertools
import sys

import numpy as np

f32, f64, i32, i64, u8, u32 = np.float32, np.float64, np.int32, np.int64, np.uint8, np.uint32


class Vector(np.ndarray):
    """ti.Vector: a float32 array with component attributes."""

    def __new__(cls, values, dt=None):
        a = np.asarray(values, dtype=dt or np.float32).view(cls)
        return a

    x = property(lambda s: s[0], lambda s, v: s.__setitem__(0, v))
    y = property(lambda s: s[1], lambda s, v: s.__setitem__(1, v))
    z = property(lambda s: s[2], lambda s, v: s.__setitem__(2, v))

    def norm(self, eps=0):
        return np.float32(np.sqrt(np.sum(np.asarray(self, np.float32) ** 2) + eps))

    def norm_sqr(self):
        return np.float32(np.sum(np.asarray(self, np.float32) ** 2))

    def dot(self, other):
        return np.float32(np.sum(np.asarray(self, np.float32) * np.asarray(other, np.float32)))

    def normalized(self):
        return self / self.norm()

    @staticmethod
    def field(n, dtype, shape):
        return Field(dtype, shape, n)

    @staticmethod
    def zero(dtype, n):
        return Vector(np.zeros(n), dtype)


class Matrix(np.ndarray):
    def __new__(cls, rows, dt=None):
        return np.asarray(rows, dtype=dt or np.float32).view(cls)


class Field:
    """ti.field / ti.Vector.field over a NumPy array; field[None] addresses a 0-d field."""

    def __init__(self, dtype, shape, n=None):
        shape = () if shape is None else (tuple(shape) if isinstance(shape, (tuple, list)) else (shape,))
        self.n = n
        self.dtype = np.dtype(dtype)
        self.a = np.zeros(shape + ((n,) if n else ()), self.dtype)
        self.shape = shape

    def _key(self, k):
        if k is None:
            return ()
        return k if isinstance(k, tuple) else (k,)

    def __getitem__(self, k):
        v = self.a[self._key(k)]
        if self.n:
            return Vector(v.copy(), self.dtype)
        return self.dtype.type(v)

    def __setitem__(self, k, v):
        self.a[self._key(k)] = v

    def to_numpy(self):
        return self.a.copy()

    def from_numpy(self, arr):
        self.a[...] = arr

    def fill(self, v):
        self.a[...] = v


def field(dtype, shape=None, **_):
    return Field(dtype, shape)


def ndrange(*dims):
    return itertools.product(*[range(d) if isinstance(d, int) else range(*d) for d in dims])


def _ident(f=None, **_):
    return f if f is not None else (lambda g: g)


kernel = func = data_oriented = pyfunc = _ident


def template():
    return None


def static(x, *_):
    return x


def _f(fn):
    return lambda *a: fn(*a)


sqrt = _f(np.sqrt)
exp = _f(np.exp)
cos = _f(np.cos)
sin = _f(np.sin)
log = _f(np.log)
tanh = _f(np.tanh)
abs = _f(np.abs)  # noqa: A001  (the Taichi name)
floor = _f(np.floor)


def max(*a):  # noqa: A001
    return np.maximum.reduce(a) if len(a) > 2 else np.maximum(a[0], a[1])


def min(*a):  # noqa: A001
    return np.minimum.reduce(a) if len(a) > 2 else np.minimum(a[0], a[1])


def cast(x, dtype):
    if isinstance(x, np.ndarray) and x.ndim:
        return Vector(x, dtype)
    return np.dtype(dtype).type(x)


def loop_config(**_):
    """Launch hints (block_dim ...) have no meaning for serial execution."""
    return None


def random(dtype=None):
    """ti.random() is 0.5 here: random perturbations of the form (random() - 0.5) * c vanish, so
    a fixture pins everything but them."""
    return np.float32(0.5)


def atomic_add(ref, v):
    raise NotImplementedError("atomics are outside the stand-in")


def init(*_, **__):
    return None


cpu = gpu = cuda = vulkan = metal = "stand-in"


def install():
    """Register this module as `taichi` for the reference's `import taichi as ti`.

    Float32 field arithmetic stays float32 only under NumPy 2's promotion rules (NEP 50: a Python
    float does not widen an np.float32); under NumPy 1 it would silently become float64."""
    if int(np.__version__.split(".")[0]) < 2:
        raise RuntimeError("the Taichi stand-in needs NumPy >= 2 (float32 scalar promotion, NEP 50)")
    sys.modules["taichi"] = sys.modules[__name__]
    return sys.modules[__name__]

