"""Leja nodes (mirrors ``src/smolyax/nodes/leja.py``)."""
from __future__ import annotations

from functools import lru_cache

import numpy as np

from .base import Generator, Generator1D


class _LejaSequence:
    """Leja points on [-1, 1]: 0, 1, -1, 1/sqrt2, -1/sqrt2, then x_j = -x_{j-1}
    for even j and sqrt((x_{(j+1)/2} + 1) / 2) for odd j (``leja.py:17,48-57``)."""

    values = np.array([0.0, 1.0, -1.0, 1 / np.sqrt(2), -1 / np.sqrt(2)])

    @classmethod
    def upto(cls, n: int) -> np.ndarray:
        have = cls.values.shape[0]
        if n >= have:
            ext = np.empty(n + 1)
            ext[:have] = cls.values
            for j in range(have, n + 1):
                ext[j] = -ext[j - 1] if j % 2 == 0 else np.sqrt((ext[(j + 1) // 2] + 1) / 2)
            cls.values = ext
        return cls.values[: n + 1]


def _affine(x, src, dst):
    """Map x from interval src to interval dst in the reference's two-step form."""
    x = (x - src[0]) / (src[1] - src[0])
    return x * (dst[1] - dst[0]) + dst[0]


class Leja1D(Generator1D):
    """Nested Leja nodes on [-1, 1] or a custom interval."""

    def __init__(self, domain=None) -> None:
        super().__init__(is_nested=True)
        self._domain = None if domain is None else np.asarray(domain)
        self._ref = None if domain is None else (-1, 1)
        self._nodes = lru_cache(maxsize=None)(self._make_nodes)
        self._qw = lru_cache(maxsize=None)(self._make_qw)

    @property
    def domain(self):
        return self._domain

    def _make_nodes(self, n):
        return self.scale(_LejaSequence.upto(n).copy())

    def _make_qw(self, n):
        # Vandermonde solve against the moments of the uniform probability
        # measure on [-1, 1] (``leja.py:83-93``); not rescaled by the domain.
        pts = _LejaSequence.upto(n)
        vm = np.vstack([pts**i for i in range(n + 1)])
        rhs = np.array([(1 + (-1) ** i) / (2.0 * (i + 1)) for i in range(n + 1)])
        return np.linalg.solve(vm, rhs)

    def __call__(self, n: int) -> np.ndarray:
        return self._nodes(int(n))

    def get_quadrature_weights(self, n: int) -> np.ndarray:
        return self._qw(int(n))

    def scale(self, x, d1=None, d2=None):
        d1 = self._ref if d1 is None else d1
        d2 = self._domain if d2 is None else d2
        assert (d1 is None) == (d2 is None)
        if d1 is None:
            return x
        d1, d2 = np.squeeze(d1), np.squeeze(d2)
        assert d1.shape == d2.shape == (2,), f"shapes {d1.shape} and {d2.shape} do not match (2, )"
        assert d1[0] < d1[1]
        assert d2[0] < d2[1]
        shape = x.shape
        x = np.squeeze(x)
        assert x.ndim <= 1
        lo_ok = (x >= d1[0]) | np.isclose(x, d1[0])
        hi_ok = (x <= d1[1]) | np.isclose(x, d1[1])
        assert np.all(lo_ok), f"Assertion failed: Some values are below lower bounds\n{x[~lo_ok]}"
        assert np.all(hi_ok), f"Assertion failed: Some values are above upper bounds\n{x[~hi_ok]}"
        return _affine(x, d1, d2).reshape(shape)

    def scale_back(self, x):
        return self.scale(x, d1=self._domain, d2=self._ref)

    def get_random(self, n: int = 1):
        return self.scale(np.random.uniform(-1, 1, n))

    def spectral_map(self):
        if self._domain is None:
            return ("legendre", 1.0, 0.0)
        lo, hi = float(self._domain[0]), float(self._domain[1])
        a = 2.0 / (hi - lo)
        return ("legendre", a, -1.0 - a * lo)

    def __repr__(self) -> str:
        return f"Leja (domain = {self._domain})"


class Leja(Generator):
    """Leja nodes in every dimension, optionally on per-dimension intervals."""

    def __init__(self, *, domains=None, dim: int = None):
        self._domains = None
        self._refs = None
        if domains is not None:
            Generator.__init__(self, [Leja1D(dom) for dom in domains])
            self._domains = np.asarray(domains)
            self._refs = np.array([[-1, 1]] * len(domains))
        elif dim is not None:
            Generator.__init__(self, [Leja1D()] * dim)
        else:
            raise ValueError("Must specify one of 'domains' or 'dim'.")

    def scale(self, x, d1=None, d2=None):
        d1 = self._refs if d1 is None else d1
        d2 = self._domains if d2 is None else d2
        assert (d1 is None) == (d2 is None)
        if d1 is None:
            return x
        d1, d2 = np.asarray(d1), np.asarray(d2)
        assert d1.shape == d2.shape, f"shapes {d1.shape} and {d2.shape} do not match"
        if d1.ndim == 1:
            d1, d2 = d1.reshape(1, 2), d2.reshape(1, 2)
        d = d1.shape[0]
        for i in range(d):
            assert d1[i, 0] < d1[i, 1]
            assert d2[i, 0] < d2[i, 1]
        x = np.asarray(x)
        shape = x.shape
        if shape == ():
            x = np.array([[x]])
        elif x.ndim == 1:
            x = x.reshape((1, len(x))) if x.shape[0] == d else x.reshape((len(x), 1))
        lo_ok = (x >= d1[:, 0]) | np.isclose(x, d1[:, 0])
        hi_ok = (x <= d1[:, 1]) | np.isclose(x, d1[:, 1])
        assert np.all(lo_ok), f"Assertion failed: Some values are below lower bounds\n{x[~lo_ok]}"
        assert np.all(hi_ok), f"Assertion failed: Some values are above upper bounds\n{x[~hi_ok]}"
        assert x.ndim == 2 and x.shape[1] == d1.shape[0] == d2.shape[0]
        x = (x - d1[:, 0]) / (d1[:, 1] - d1[:, 0])
        x = x * (d2[:, 1] - d2[:, 0]) + d2[:, 0]
        return x.reshape(shape)

    def scale_back(self, x):
        return self.scale(x, d1=self._domains, d2=self._refs)

    def __repr__(self) -> str:
        if self._domains is not None:
            return f"Leja (d = {self.dim}, domains = {self._domains.tolist()})"
        return f"Leja (d = {self.dim})"
