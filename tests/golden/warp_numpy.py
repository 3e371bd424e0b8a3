"""A NumPy stand-in for the parts of NVIDIA Warp that the reference's element
code uses, so that the reference's own ``@wp.func`` and ``@wp.kernel`` bodies
(plain Python source) run unmodified on the CPU in FP64.

TEST INFRASTRUCTURE ONLY: used by ``make_elem_golden.py`` to generate golden
vectors; nothing in ``apple_gb300`` imports it.

Semantics restated from Warp's public documentation:

* ``wp.func`` / ``wp.kernel`` bodies are Python functions; ``wp.launch``
  calls a kernel once per thread index in ``dim`` (``wp.tid()`` returns it).
* Matrices and vectors are values: ``@`` is the matrix product, ``*`` with a
  scalar scales, ``+``/``-`` are elementwise; ``M[i]`` is row ``i`` (a
  vector), ``M[:, j]`` column ``j``, ``v[i]`` a scalar.  ``x.dtype`` is the
  scalar type, callable as a constructor (``F.dtype(2.0)``).
* ``wp.atomic_add(a, i, v)`` adds ``v`` into ``a[i]``; with one thread at a
  time here it is a plain read-modify-write.
* ``wp.svd3`` is compiled Warp code that is not part of the reference tree;
  the stand-in uses LAPACK with the rotation-variant sign convention
  (det U = det V = +1, the last singular value carries the sign of det F).
  For a non-inverted F with distinct singular values every quantity the
  reference builds from it (R = U V^T, the twist modes' squared projections,
  the lambdas) is independent of the column-sign convention, so golden
  inputs keep F non-inverted.
"""

from __future__ import annotations

import types
from typing import Any

import numpy as np

class Scalar(float):
    """A Warp scalar (FP64): arithmetic stays in this type so that ``x.dtype``
    (the scalar type, callable as a constructor) works on every result."""

    @property
    def dtype(self):
        return Scalar

    def _op(self, o, f):
        if isinstance(o, T):
            return NotImplemented
        return Scalar(f(float(self), float(o)))

    def __add__(self, o):
        return self._op(o, lambda a, b: a + b)

    def __radd__(self, o):
        return self._op(o, lambda a, b: b + a)

    def __sub__(self, o):
        return self._op(o, lambda a, b: a - b)

    def __rsub__(self, o):
        return self._op(o, lambda a, b: b - a)

    def __mul__(self, o):
        return self._op(o, lambda a, b: a * b)

    def __rmul__(self, o):
        return self._op(o, lambda a, b: b * a)

    def __truediv__(self, o):
        return self._op(o, lambda a, b: a / b)

    def __rtruediv__(self, o):
        return self._op(o, lambda a, b: b / a)

    def __pow__(self, o):
        return self._op(o, lambda a, b: a**b)

    def __neg__(self):
        return Scalar(-float(self))

    def __pos__(self):
        return self

    def __abs__(self):
        return Scalar(abs(float(self)))


class T:
    """A Warp vector or matrix value (FP64)."""

    __slots__ = ("a",)
    __array_ufunc__ = None  # numpy scalars defer to T's reflected operators

    def __init__(self, a):
        self.a = np.array(a, dtype=np.float64)

    # -- Warp value semantics --------------------------------------------------
    @property
    def dtype(self):
        return Scalar

    @property
    def shape(self):
        return self.a.shape

    def __getitem__(self, idx):
        r = self.a[idx]
        return Scalar(r) if np.ndim(r) == 0 else T(r)

    def __len__(self):
        return self.a.shape[0]

    @staticmethod
    def _v(x):
        return x.a if isinstance(x, T) else float(x)

    def __add__(self, o):
        return T(self.a + T._v(o))

    __radd__ = __add__

    def __sub__(self, o):
        return T(self.a - T._v(o))

    def __rsub__(self, o):
        return T(T._v(o) - self.a)

    def __neg__(self):
        return T(-self.a)

    def __mul__(self, o):
        if isinstance(o, T):  # Warp: matrix * matrix / matrix * vector is a product
            return T(self.a @ o.a)
        return T(self.a * float(o))

    def __rmul__(self, o):
        return T(float(o) * self.a)

    def __truediv__(self, o):
        return T(self.a / T._v(o))

    def __matmul__(self, o):
        return T(self.a @ T._v(o))

    def __rmatmul__(self, o):
        return T(T._v(o) @ self.a)

    def __repr__(self):
        return f"T({self.a!r})"


def _arr(x):
    return x.a if isinstance(x, T) else np.asarray(float(x) if isinstance(x, Scalar) else x, dtype=np.float64)


# -- builtins ---------------------------------------------------------------------
def transpose(m):
    return T(_arr(m).T)


def identity(n, dtype=None):
    return T(np.eye(n))


def matrix(*args, shape=None, dtype=None):
    if shape is not None and not args:
        return T(np.zeros(shape))
    return T(np.array([_arr(a) for a in args]).reshape(shape))


def matrix_from_rows(*rows):
    return T(np.stack([_arr(r) for r in rows]))


def matrix_from_cols(*cols):
    return T(np.stack([_arr(c) for c in cols], axis=1))


def vector(*xs, length=None, dtype=None):
    return T(np.array([float(x) for x in xs]))


def diag(v):
    return T(np.diag(_arr(v)))


def ddot(a, b):
    return Scalar(np.sum(_arr(a) * _arr(b)))


def dot(a, b):
    return Scalar(np.dot(_arr(a), _arr(b)))


def cross(a, b):
    return T(np.cross(_arr(a), _arr(b)))


def outer(a, b):
    return T(np.outer(_arr(a), _arr(b)))


def length_sq(v):
    return Scalar(np.dot(_arr(v), _arr(v)))


def cw_mul(a, b):
    return T(_arr(a) * _arr(b))


def trace(m):
    return Scalar(np.trace(_arr(m)))


def determinant(m):
    return Scalar(np.linalg.det(_arr(m)))


def sqrt(x):
    return Scalar(np.sqrt(float(x)))


def max(a, b):  # noqa: A001 - Warp's name
    if isinstance(a, T) or isinstance(b, T):
        return T(np.maximum(_arr(a), _arr(b)))
    return Scalar(a if float(a) >= float(b) else b)


def min(a, b):  # noqa: A001 - Warp's name
    if isinstance(a, T) or isinstance(b, T):
        return T(np.minimum(_arr(a), _arr(b)))
    return Scalar(a if float(a) <= float(b) else b)


def svd3(F):
    A = _arr(F)
    U, s, Vt = np.linalg.svd(A)
    V = Vt.T
    if np.linalg.det(U) < 0:
        U[:, 2] = -U[:, 2]
        s[2] = -s[2]
    if np.linalg.det(V) < 0:
        V[:, 2] = -V[:, 2]
        s[2] = -s[2]
    return T(U), T(s), T(V)


def static(x):
    return x


# -- kernels, launches, arrays ---------------------------------------------------------
_tid: tuple[int, ...] = ()


def tid():
    return _tid if len(_tid) > 1 else _tid[0]


class Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.__name__ = fn.__name__


def kernel(fn=None, **_kw):
    if fn is None:
        return lambda f: Kernel(f)
    return Kernel(fn)


def func(fn):
    return fn


def launch(kernel_, dim, inputs=(), outputs=(), **_kw):
    global _tid
    dim = (dim,) if isinstance(dim, int) else tuple(dim)
    try:
        for idx in np.ndindex(*dim):
            _tid = tuple(int(i) for i in idx)
            kernel_.fn(*inputs, *outputs)
    finally:
        _tid = ()


class Array:
    """A device array of scalars, vectors or matrices: ``a[i]`` / ``a[i, j]``
    returns a scalar or a value ``T``; stores go through ``atomic_add``."""

    def __init__(self, data, inner_ndim=0, dtype=np.float64):
        self.data = np.array(data, dtype=dtype)
        self.inner = inner_ndim

    def __getitem__(self, idx):
        r = self.data[idx]
        if np.ndim(r) == 0:
            return Scalar(r) if self.data.dtype.kind == "f" else int(r)
        return T(r) if self.data.dtype.kind == "f" else r

    def __setitem__(self, idx, v):
        self.data[idx] = _arr(v)

    @property
    def shape(self):
        return self.data.shape[: self.data.ndim - self.inner]


def atomic_add(a, idx, v):
    a[idx] = a[idx] + v


# -- names used only in annotations / class bodies -----------------------------------------
class _Subscriptable:
    def __class_getitem__(cls, item):
        return cls

    def __init__(self, *a, **k):
        pass


class array(_Subscriptable):  # noqa: N801 - Warp's name
    pass


class array1d(_Subscriptable):  # noqa: N801
    pass


class array2d(_Subscriptable):  # noqa: N801
    pass


class Function:
    pass


vec3 = vec4i = mat33 = Any
types = types.SimpleNamespace(matrix=lambda *a, **k: Any, vector=lambda *a, **k: Any)
