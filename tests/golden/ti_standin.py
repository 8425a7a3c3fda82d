"""A NumPy stand-in for the part of the Taichi 0.9 Python API that the
reference's SIMPLE path uses, so that the reference's own source files
(simple.py, bicgsolver.py, cgsolver.py, karman_taichi.py, debug/linalg.py)
run unmodified on the CPU and produce golden vectors.

Test infrastructure only: ``make_golden.py`` installs it as the ``taichi``
module while it imports the reference; nothing in the package, the tests'
GPU paths or bench.py imports it.

Semantics emulated (Taichi 0.9, ``ti.init(arch=ti.cpu, default_fp=ti.f64)``):

* fields are float64 (or int64 for integer dtypes) arrays, zero-initialised;
  ``ti.root.dense/pointer(...).place(...)`` allocates each placed field with
  the product of the levels' extents per axis; pointer levels are stored
  sparsely (a dict), which is what lets the reference's n x n matrices exist;
* reads outside a field's shape, and reads of never-written sparse entries,
  return 0 (debug/ti_sparse_test.py:38-39: out-of-range reads of a pointer
  field return 0.0); an out-of-range write is kept under its own index and
  read back only from that index (Taichi pads extents to powers of two, so
  such writes land in padding that no in-range read sees);
* kernels run their statements in program order, and every loop -- also the
  outermost, which Taichi parallelises -- serially in index order, so atomic
  reductions become left-to-right sums;
* arithmetic is IEEE binary64 in the source's evaluation order: values read
  from fields are numpy float64 scalars, so a division by zero gives inf/nan
  (as compiled Taichi does) instead of raising; LLVM fast-math contraction,
  which the real Taichi may apply, is not emulated;
* ``@ti.kernel`` converts scalar arguments to their annotated types and the
  return value to the annotated type; ``ti.template()`` arguments pass
  through; ``@ti.func`` and ``@ti.data_oriented`` are plain Python.

Anything else (GUI, sparse solvers, vectors and matrices) is absent.
"""
from __future__ import annotations

import builtins
import functools
import inspect
import itertools
import math

import numpy as np

np.seterr(all="ignore")

# ---- types, architectures, axes -------------------------------------------------------------
f64 = "f64"
f32 = "f32"
i32 = "i32"
i64 = "i64"
u8 = "u8"
cpu, gpu, cuda, x64 = "cpu", "gpu", "cuda", "x64"
i, j, k = ("i",), ("j",), ("k",)
ij, ijk = ("i", "j"), ("i", "j", "k")

_INT_TYPES = {i32, i64, u8, int}
_FLOAT_TYPES = {f64, f32, float}

_cfg = {"default_fp": f64}


def init(*args, **kwargs):
    _cfg.update(kwargs)


def reset():
    pass


class _Template:
    pass


def template():
    return _Template()


def static(x, *more):
    return x if not more else (x,) + more


def sqrt(x):
    return np.sqrt(np.float64(x))


def abs(x):  # noqa: A001 -- the Taichi name
    return np.abs(x)


def max(*a):  # noqa: A001
    return builtins.max(*a)


def min(*a):  # noqa: A001
    return builtins.min(*a)


def exp(x):
    return np.exp(np.float64(x))


# ---- iteration helpers --------------------------------------------------------------------
class ndrange:
    def __init__(self, *dims):
        self.ranges = []
        for d in dims:
            if isinstance(d, (tuple, list)):
                self.ranges.append(range(int(d[0]), int(d[1])))
            else:
                self.ranges.append(range(int(d)))

    def __iter__(self):
        if len(self.ranges) == 1:
            return iter(self.ranges[0])
        return itertools.product(*self.ranges)

    def grouped(self):
        return itertools.product(*self.ranges)


def grouped(x):
    if isinstance(x, ndrange):
        return x.grouped()
    if isinstance(x, Field):
        return (tuple(t) for t in np.ndindex(*x.shape))
    raise TypeError("ti.grouped: unsupported argument")


# ---- fields -------------------------------------------------------------------------------
class Field:
    def __init__(self, dtype=None, shape=None, name=""):
        self.dtype = dtype if dtype is not None else _cfg.get("default_fp", f64)
        self.shape = None
        self._a = None
        self._sp = None
        self._oob = {}
        if shape is not None:
            self._alloc(shape if isinstance(shape, (tuple, list)) else (shape,), sparse=False)

    @property
    def _is_int(self):
        return self.dtype in _INT_TYPES

    def _zero(self):
        return np.int64(0) if self._is_int else np.float64(0.0)

    def _alloc(self, shape, sparse):
        if self.shape is not None:
            raise RuntimeError("field placed twice")
        self.shape = tuple(int(s) for s in shape)
        if sparse:
            self._sp = {}
        else:
            self._a = np.zeros(self.shape, dtype=np.int64 if self._is_int else np.float64)

    def _key(self, I):
        if I is None:
            return ()
        if isinstance(I, tuple):
            return tuple(int(t) for t in I)
        return (int(I),)

    def _inside(self, key):
        if len(key) != len(self.shape):
            raise IndexError(f"field of shape {self.shape} indexed with {key}")
        for t, s in zip(key, self.shape):
            if t < 0 or t >= s:
                return False
        return True

    def __getitem__(self, I):
        key = self._key(I)
        if not self._inside(key):
            return self._oob.get(key, self._zero())
        if self._sp is not None:
            return self._sp.get(key, self._zero())
        return self._a[key]

    def __setitem__(self, I, value):
        key = self._key(I)
        if self._is_int:
            value = np.int64(value)
        else:
            value = np.float64(value)
        if not self._inside(key):
            self._oob[key] = value
            return
        if self._sp is not None:
            if value == 0 and key not in self._sp:
                return            # an unwritten entry reads 0 already
            self._sp[key] = value
            return
        self._a[key] = value

    def __iter__(self):
        # struct-for over a dense field: every index, row-major
        if len(self.shape) == 1:
            return iter(range(self.shape[0]))
        return (tuple(t) for t in np.ndindex(*self.shape))

    # Python-scope helpers
    def to_numpy(self):
        if self._sp is not None:
            raise RuntimeError("to_numpy of a pointer-sparse field is not supported (use entries())")
        return self._a.copy()

    def from_numpy(self, arr):
        arr = np.asarray(arr)
        if arr.shape != self.shape:
            raise ValueError(f"from_numpy: shape {arr.shape} != {self.shape}")
        if self._sp is not None:
            self._sp = {tuple(t): np.float64(arr[t]) for t in zip(*np.nonzero(arr))}
        else:
            self._a[...] = arr

    def fill(self, value):
        if self._sp is not None:
            self._sp = {}
            if value != 0:
                raise RuntimeError("fill of a sparse field with a nonzero value")
        else:
            self._a[...] = value

    def entries(self):
        """The written in-range entries of a sparse field as {index: value}."""
        return dict(self._sp) if self._sp is not None else None

    def copy_from(self, other):
        self.from_numpy(other.to_numpy())


def field(dtype=None, shape=None, name="", **kwargs):
    return Field(dtype, shape, name)


class _SNode:
    """One level chain of ti.root: extents per axis multiply down the chain."""

    def __init__(self, extents=None, sparse=False):
        self.extents = dict(extents or {})
        self.sparse = sparse

    def _child(self, axes, shape, sparse):
        if isinstance(shape, int):
            shape = (shape,) * len(axes)
        ext = dict(self.extents)
        for a, s in zip(axes, shape):
            ext[a] = ext.get(a, 1) * int(s)
        return _SNode(ext, self.sparse or sparse)

    def dense(self, axes, shape):
        return self._child(axes, shape, False)

    def pointer(self, axes, shape):
        return self._child(axes, shape, True)

    bitmasked = pointer

    def place(self, *fields, **kwargs):
        order = [a for a in ("i", "j", "k") if a in self.extents]
        shape = tuple(self.extents[a] for a in order)
        for f in fields:
            f._alloc(shape, self.sparse)
        return self


root = _SNode()


# ---- kernels ------------------------------------------------------------------------------
def _cast(value, ann):
    if ann in _INT_TYPES:
        return int(value)
    if ann in _FLOAT_TYPES:
        return np.float64(value)
    return value


def kernel(fn):
    sig = inspect.signature(fn)
    anns = dict(fn.__annotations__)
    ret = anns.pop("return", None)

    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        bound = sig.bind(*args, **kwargs)
        for name in list(bound.arguments):
            if name in anns:
                bound.arguments[name] = _cast(bound.arguments[name], anns[name])
        out = fn(*bound.args, **bound.kwargs)
        return _cast(out, ret) if ret is not None else out

    wrapper._ti_kernel = True
    return wrapper


def func(fn):
    return fn


def data_oriented(cls):
    return cls


class GUI:
    def __init__(self, *args, **kwargs):
        raise RuntimeError("the Taichi stand-in has no GUI (headless golden-vector runs only)")


Vector = None
Matrix = None
pi = math.pi
