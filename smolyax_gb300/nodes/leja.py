"""Leja nodes (the API of ``src/smolyax/nodes/leja.py``).

The nested Leja sequence on [-1, 1] starts 0, 1, -1, 1/sqrt(2), -1/sqrt(2);
after that, node j is the mirror -node[j-1] for even j and
sqrt((node[(j+1)/2] + 1) / 2) for odd j (``leja.py:17,48-57``).  The same
sequence gives the same interpolant, so these values are reproduced exactly.
Custom domains are reached by an affine map of each coordinate
(``nodes/_box.py``).
"""
from __future__ import annotations

import numpy as np

from ._box import UNIT_INTERVAL, as_box, map_points
from .base import Generator, Generator1D

_SEQUENCE = np.array([0.0, 1.0, -1.0, 1 / np.sqrt(2), -1 / np.sqrt(2)])


def leja_points(n: int) -> np.ndarray:
    """The first n+1 points of the Leja sequence on [-1, 1] (a copy)."""
    global _SEQUENCE
    have = _SEQUENCE.size
    if n >= have:
        grown = np.concatenate([_SEQUENCE, np.zeros(n + 1 - have)])
        for j in range(have, n + 1):
            grown[j] = np.sqrt((grown[(j + 1) // 2] + 1) / 2) if j & 1 else -grown[j - 1]
        _SEQUENCE = grown
    return _SEQUENCE[: n + 1].copy()


def _uniform_quadrature(n: int) -> np.ndarray:
    """Weights q with sum_j q_j p(x_j) = (1/2) int_{-1}^{1} p for every
    polynomial p of degree <= n, x = the first n+1 Leja points (``leja.py:83-93``):
    the moment equations sum_j q_j x_j^i = mean of x^i over [-1, 1], i = 0..n."""
    pts = leja_points(n)
    powers = np.arange(n + 1)
    moments = np.where(powers % 2 == 0, 1.0 / (powers + 1.0), 0.0)
    return np.linalg.solve(pts[None, :] ** powers[:, None], moments)


class Leja1D(Generator1D):
    """Nested Leja nodes on [-1, 1], or mapped to the interval `domain`."""

    def __init__(self, domain=None) -> None:
        super().__init__(is_nested=True)
        self._domain = None if domain is None else np.asarray(domain)
        self._nodes = {}
        self._weights = {}

    @property
    def domain(self):
        return self._domain

    def __call__(self, n: int) -> np.ndarray:
        n = int(n)
        if n not in self._nodes:
            self._nodes[n] = self.scale(leja_points(n))
        return self._nodes[n]

    def get_quadrature_weights(self, n: int) -> np.ndarray:
        """Weights of the uniform probability measure on the reference interval
        (they do not depend on the domain)."""
        n = int(n)
        if n not in self._weights:
            self._weights[n] = _uniform_quadrature(n)
        return self._weights[n]

    def scale(self, x, d1=None, d2=None):
        """Affine map from interval d1 (default [-1, 1]) to d2 (default: the domain).
        Without a domain and without explicit intervals, x is returned as is."""
        src = d1 if d1 is not None else (None if self._domain is None else UNIT_INTERVAL)
        dst = d2 if d2 is not None else self._domain
        if src is None and dst is None:
            return x
        if src is None or dst is None:
            raise AssertionError("Leja1D.scale: a source interval needs a target interval and vice versa")
        if as_box(src).shape[0] != 1 or as_box(dst).shape[0] != 1:
            raise AssertionError("Leja1D.scale: intervals must be single (lower, upper) pairs")
        return map_points(x, src, dst)

    def scale_back(self, x):
        """Domain -> [-1, 1]."""
        return self.scale(x, d1=self._domain, d2=None if self._domain is None else UNIT_INTERVAL)

    def get_random(self, n: int = 1):
        """n points uniform on the domain (numpy's global generator)."""
        return self.scale(np.random.uniform(-1.0, 1.0, n))

    def spectral_map(self):
        if self._domain is None:
            return ("legendre", 1.0, 0.0)
        lo, hi = (float(v) for v in np.ravel(self._domain)[:2])
        a = 2.0 / (hi - lo)
        return ("legendre", a, -1.0 - a * lo)

    def __repr__(self) -> str:
        where = "[-1, 1]" if self._domain is None else str(np.ravel(self._domain).tolist())
        return "Leja1D(domain=%s)" % where


class Leja(Generator):
    """Leja nodes in every dimension: give `dim` for [-1, 1]^dim, or `domains`
    (one (lower, upper) pair per dimension)."""

    def __init__(self, *, domains=None, dim: int = None):
        if domains is not None:
            boxes = as_box(domains, "Leja domains")
            super().__init__([Leja1D(row) for row in np.asarray(domains)])
            self._domains = boxes
        elif dim is not None:
            super().__init__([Leja1D() for _ in range(int(dim))])
            self._domains = None
        else:
            raise ValueError("Leja needs either `dim` or `domains`")

    def _resolve(self, d1, d2, forward):
        unit = None if self._domains is None else np.repeat(UNIT_INTERVAL, self.dim, axis=0)
        src = d1 if d1 is not None else (unit if forward else self._domains)
        dst = d2 if d2 is not None else (self._domains if forward else unit)
        return src, dst

    def _map(self, x, src, dst):
        if src is None and dst is None:
            return x
        if src is None or dst is None:
            raise AssertionError("Leja.scale: a source box needs a target box and vice versa")
        return map_points(x, src, dst)

    def scale(self, x, d1=None, d2=None):
        """Affine map of each coordinate from box d1 (default [-1, 1]^d) to box
        d2 (default: the domains); x has shape (d,) or (n, d)."""
        src, dst = self._resolve(d1, d2, forward=True)
        return self._map(x, src, dst)

    def scale_back(self, x):
        """Domains -> [-1, 1]^d."""
        src, dst = self._resolve(None, None, forward=False)
        return self._map(x, src, dst)

    def __repr__(self) -> str:
        if self._domains is None:
            return "Leja(dim=%d)" % self.dim
        return "Leja(dim=%d, domains=%s)" % (self.dim, self._domains.tolist())
