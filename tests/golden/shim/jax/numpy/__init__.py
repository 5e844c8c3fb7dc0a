"""Numpy-backed stand-in for ``jax.numpy`` (golden-vector generation only).

Arrays carry ``.at[idx].set(v)`` (functional update) and
``block_until_ready()``.  ``broadcast_to`` returns a float64 copy because the
reference accumulates into it with ``+=``.
"""
import numpy as _np


class _Updater:
    def __init__(self, arr, idx):
        self._arr, self._idx = arr, idx

    def set(self, value):
        out = self._arr.copy()
        out[self._idx] = value
        return out


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _Updater(self._arr, idx)


class ShimArray(_np.ndarray):
    @property
    def at(self):
        return _At(self)

    def block_until_ready(self):
        return self


def _wrap(x):
    return _np.asarray(x).view(ShimArray)


def asarray(x, *args, **kwargs):
    return _wrap(x)


array = asarray
nan = _np.nan


def broadcast_to(x, shape):
    arr = _np.asarray(x, dtype=_np.result_type(x, _np.float64))
    return _wrap(_np.broadcast_to(arr, shape).copy())


def zeros(shape, *args, **kwargs):
    return _wrap(_np.zeros(shape))


def einsum(*args, **kwargs):
    return _wrap(_np.einsum(*args, optimize=True))


def _lift(fn):
    return lambda *a, **k: _wrap(fn(*a, **k))


where = _lift(_np.where)
prod = _lift(_np.prod)
arange = _lift(_np.arange)
any = _lift(_np.any)
divide = _lift(_np.divide)
sum = _lift(_np.sum)
tile = _lift(_np.tile)
