"""Node-generator interface (mirrors ``src/smolyax/nodes/base.py``).

Node generation is FP64 set-up data computed on the host, exactly as in the
reference; the device only ever sees the resulting node tables.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Iterator, List

import numpy as np


class Generator1D(ABC):
    """One-dimensional node sequence (``base.py:8-128``)."""

    def __init__(self, is_nested: bool) -> None:
        self._is_nested = bool(is_nested)

    @property
    def is_nested(self) -> bool:
        return self._is_nested

    @abstractmethod
    def __call__(self, n: int) -> np.ndarray:
        """The first n+1 nodes."""

    @abstractmethod
    def scale(self, x):
        """Reference domain -> custom domain."""

    @abstractmethod
    def scale_back(self, x):
        """Custom domain -> reference domain."""

    @abstractmethod
    def get_random(self, n: int = 1):
        """Samples from the measure associated with the domain."""

    @abstractmethod
    def get_quadrature_weights(self, n: int) -> np.ndarray:
        """Quadrature weights of the first n+1 nodes."""

    def spectral_map(self):
        """(family, a, b): orthogonal family used by the mixed-precision path and the
        affine map z = a*x + b to its reference variable.  Generators that do not
        override it get Legendre polynomials on the hull of their first nodes."""
        pts = np.asarray(self(8), dtype=float)
        lo, hi = float(pts.min()), float(pts.max())
        if hi <= lo:
            return ("legendre", 1.0, 0.0)
        a = 2.0 / (hi - lo)
        return ("legendre", a, -1.0 - a * lo)


class Generator:
    """Container of per-dimension generators (``base.py:131-262``)."""

    def __init__(self, node_gens: List[Generator1D]):
        assert all(g.is_nested == node_gens[0].is_nested for g in node_gens)
        self._gens = list(node_gens)
        self._is_nested = node_gens[0].is_nested
        self._dim = len(node_gens)

    @property
    def dim(self) -> int:
        return self._dim

    @property
    def is_nested(self) -> bool:
        return self._is_nested

    def __getitem__(self, i: int) -> Generator1D:
        return self._gens[i]

    def __iter__(self) -> Iterator[Generator1D]:
        for i in range(self._dim):
            yield self._gens[i]

    def __len__(self) -> int:
        return self._dim

    def get_random(self, n: int = 0):
        """n = 0 returns one point of shape (d,), otherwise (n, d)."""
        if n == 0:
            return np.squeeze([g.get_random() for g in self._gens])
        return np.array([g.get_random(n) for g in self._gens]).T

    def scale(self, x):
        assert x.shape[-1] == self.dim
        if x.ndim == 1:
            return np.array([g.scale(v) for g, v in zip(self._gens, x)])
        return np.array([g.scale(col) for g, col in zip(self._gens, x.T)]).T

    def scale_back(self, x):
        assert x.shape[-1] == self.dim
        if x.ndim == 1:
            return np.array([g.scale_back(v) for g, v in zip(self._gens, x)])
        return np.array([g.scale_back(col) for g, col in zip(self._gens, x.T)]).T
