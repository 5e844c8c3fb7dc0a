"""Numpy-backed stand-in for the small part of jax the reference uses.

Used only by ``tests/golden/make_golden.py`` to run the reference in a
container without jax.  ``vmap`` loops over the mapped axis; ``jit`` is the
identity; ``config.update`` is a no-op (numpy is float64 already).
"""
import numpy as _np

from . import numpy  # noqa: F401

Array = _np.ndarray


class _Config:
    def update(self, *args, **kwargs):
        pass


config = _Config()


def jit(fn, *args, **kwargs):
    return fn


def vmap(fn, in_axes):
    def mapped(*args):
        size = next(a.shape[0] for a, ax in zip(args, in_axes) if ax == 0)
        outs = [fn(*[a if ax is None else a[b] for a, ax in zip(args, in_axes)]) for b in range(size)]
        return numpy.asarray(_np.stack(outs))

    return mapped


class random:
    @staticmethod
    def PRNGKey(seed):
        return _np.random.default_rng(seed)

    @staticmethod
    def uniform(key, shape):
        return numpy.asarray(key.uniform(size=shape))
