"""Node-generator interface (the API of ``src/smolyax/nodes/base.py``).

Node rules are FP64 set-up data computed on the host; the device only sees
the node and weight tables built from them.  A one-dimensional rule
(`Generator1D`) yields the first n+1 nodes of its sequence, maps points
between its reference domain and its custom domain, samples its measure and
gives quadrature weights; a `Generator` holds one rule per dimension.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Iterator, List

import numpy as np


class Generator1D(ABC):
    """One-dimensional node sequence (interface of ``base.py:8-128``)."""

    def __init__(self, is_nested: bool) -> None:
        self._is_nested = bool(is_nested)

    @property
    def is_nested(self) -> bool:
        return self._is_nested

    @abstractmethod
    def __call__(self, n: int) -> np.ndarray:
        """The first n+1 nodes on the custom domain."""

    @abstractmethod
    def scale(self, x):
        """Reference domain -> custom domain."""

    @abstractmethod
    def scale_back(self, x):
        """Custom domain -> reference domain."""

    @abstractmethod
    def get_random(self, n: int = 1):
        """n samples of the measure associated with the domain."""

    @abstractmethod
    def get_quadrature_weights(self, n: int) -> np.ndarray:
        """Quadrature weights of the first n+1 nodes."""

    def spectral_map(self):
        """(family, a, b): the orthogonal polynomial family of the mixed-precision
        path and the affine map z = a*x + b to its variable.  Rules that do not
        override it get Legendre polynomials on the hull of their first nodes."""
        pts = np.asarray(self(8), dtype=float)
        lo, hi = float(pts.min()), float(pts.max())
        if hi <= lo:
            return ("legendre", 1.0, 0.0)
        a = 2.0 / (hi - lo)
        return ("legendre", a, -1.0 - a * lo)


class Generator:
    """One rule per dimension (interface of ``base.py:131-262``).

    All rules must agree on nestedness (AssertionError otherwise), since the
    index set and the node-reuse cache depend on it."""

    def __init__(self, node_gens: List[Generator1D]):
        gens = list(node_gens)
        if not gens:
            raise AssertionError("a generator needs at least one one-dimensional rule")
        nested = {g.is_nested for g in gens}
        if len(nested) != 1:
            raise AssertionError("mixing nested and non-nested rules in one generator is not supported")
        self._gens = gens
        self._is_nested = nested.pop()

    @property
    def dim(self) -> int:
        return len(self._gens)

    @property
    def is_nested(self) -> bool:
        return self._is_nested

    def __getitem__(self, i: int) -> Generator1D:
        return self._gens[i]

    def __iter__(self) -> Iterator[Generator1D]:
        return iter(list(self._gens))

    def __len__(self) -> int:
        return len(self._gens)

    def get_random(self, n: int = 0):
        """Samples of the product measure: n = 0 gives one point of shape (d,),
        n >= 1 gives an array of shape (n, d)."""
        rows = max(int(n), 1)
        pts = np.empty((rows, self.dim))
        for j, g in enumerate(self._gens):
            pts[:, j] = np.reshape(g.get_random(rows), rows)
        if n:
            return pts
        return pts[0] if self.dim > 1 else pts[0, 0]

    def _per_column(self, x, method):
        x = np.asarray(x)
        if x.ndim == 0 or x.shape[-1] != self.dim:
            raise AssertionError("points of shape %s do not have %d coordinates" % (x.shape, self.dim))
        out = np.empty(x.shape)
        for j, g in enumerate(self._gens):
            out[..., j] = getattr(g, method)(x[..., j])
        return out

    def scale(self, x):
        """Reference domain -> custom domain, coordinate by coordinate."""
        return self._per_column(x, "scale")

    def scale_back(self, x):
        """Custom domain -> reference domain, coordinate by coordinate."""
        return self._per_column(x, "scale_back")
