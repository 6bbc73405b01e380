"""Minimal stand-in for the ``taichi`` API, used ONLY to run the reference's own
Python sources on the CPU (sequentially, in float64) so that golden fixtures can be
generated from the reference itself in a container where Taichi is not installed.

This is test infrastructure for ``tests/golden/make_golden.py``; nothing in the
product imports it.

Semantics that matter for the reference kernels:
  * ``@ti.kernel`` / ``@ti.data_oriented`` are identity decorators: a kernel body
    runs as plain sequential Python.  The reference's outermost loops are
    data-parallel with per-iteration private state and no cross-iteration
    dependences other than atomic sums, so a sequential run gives the parallel
    result (up to summation order of atomic adds).
  * ``ti.ndrange(a, b, ...)`` iterates the Cartesian product in row-major order;
    one argument yields plain ints.
  * ``ti.field`` stores float data as float64 (the shim's arithmetic precision),
    integer data as int64.  ``to_numpy`` returns a float64 copy.
  * Values read from fields and returned by the math functions are numpy
    float64 scalars, so division by zero gives inf/nan as on the GPU.
  * Kernel arguments annotated ``ti.f32`` are NOT rounded to float32: the shim
    evaluates the reference's discrete operator in float64.
  * ``ti.randn`` draws from a seeded Python ``random.Random`` (see ``seed``).
"""
import itertools
import math as _m
import random as _random

import numpy as np

# dtypes / archs (opaque tokens)
f16 = "f16"
f32 = "f32"
f64 = "f64"
i8 = "i8"
i16 = "i16"
i32 = "i32"
i64 = "i64"
u8 = "u8"
u32 = "u32"
gpu = "gpu"
cpu = "cpu"
cuda = "cuda"
vulkan = "vulkan"

_FLOAT_DTYPES = {f16, f32, f64}
_rng = _random.Random(0)


def seed(s):
    """Re-seed the generator behind ``ti.randn``."""
    global _rng
    _rng = _random.Random(s)


def init(*args, **kwargs):
    return None


def reset():
    return None


def kernel(fn):
    return fn


def func(fn):
    return fn


def data_oriented(cls):
    return cls


def template():
    return None


class types:  # noqa: N801 - mirrors ti.types
    @staticmethod
    def ndarray(*args, **kwargs):
        return None


def static(x):
    return x


def ndrange(*dims):
    rngs = []
    for d in dims:
        if isinstance(d, (tuple, list)):
            rngs.append(range(int(d[0]), int(d[1])))
        else:
            rngs.append(range(int(d)))
    if len(rngs) == 1:
        return rngs[0]
    return itertools.product(*rngs)


class Field:
    def __init__(self, dtype=f32, shape=(), order=None, needs_dual=False, **kwargs):
        if isinstance(shape, (int, np.integer)):
            shape = (int(shape),)
        shape = tuple(int(s) for s in shape)
        npdt = np.float64 if dtype in _FLOAT_DTYPES else np.int64
        self.dtype = dtype
        self.shape = shape
        self.arr = np.zeros(shape, dtype=npdt)

    def __getitem__(self, idx):
        # numpy scalars give IEEE semantics (x/0 -> inf) like Taichi does
        if isinstance(idx, tuple):
            return self.arr[tuple(int(i) for i in idx)]
        return self.arr[int(idx)]

    def __setitem__(self, idx, val):
        if isinstance(idx, tuple):
            self.arr[tuple(int(i) for i in idx)] = val
        else:
            self.arr[int(idx)] = val

    def from_numpy(self, a):
        a = np.asarray(a)
        self.arr[...] = a.reshape(self.arr.shape)

    def to_numpy(self):
        return self.arr.copy()

    def fill(self, v):
        self.arr[...] = v


def field(dtype=f32, shape=(), order=None, needs_dual=False, **kwargs):
    return Field(dtype, shape, order, needs_dual, **kwargs)


# scalar math in float64 with IEEE semantics (numpy scalars, warnings off)
np.seterr(all="ignore")
_F = np.float64


def cos(x):
    return np.cos(_F(x))


def sin(x):
    return np.sin(_F(x))


def tan(x):
    return np.tan(_F(x))


def atan2(y, x):
    return np.arctan2(_F(y), _F(x))


def floor(x):
    return np.floor(_F(x))


def ceil(x):
    return np.ceil(_F(x))


def sqrt(x):
    return np.sqrt(_F(x))


def exp(x):
    return np.exp(_F(x))


def log(x):
    return np.log(_F(x))


def abs(x):  # noqa: A001 - mirrors ti.abs
    return x if x >= 0 else -x


def randn(dtype=None):
    return _rng.gauss(0.0, 1.0)


def random(dtype=None):
    return _rng.random()


class math:  # noqa: N801 - mirrors ti.math
    cos = staticmethod(cos)
    sin = staticmethod(sin)
    tan = staticmethod(tan)
    atan2 = staticmethod(atan2)
    floor = staticmethod(floor)
    sqrt = staticmethod(sqrt)
    exp = staticmethod(exp)
    log = staticmethod(log)
    pi = _m.pi
