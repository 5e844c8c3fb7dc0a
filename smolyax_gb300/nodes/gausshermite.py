"""Gauss-Hermite nodes (the API of ``src/smolyax/nodes/gausshermite.py``).

The n+1 nodes of level n are the roots of the physicists' Hermite polynomial
H_{n+1} (numpy's ``hermgauss``), mapped to ``mean + scaling * z``; the rule
is not nested.  Quadrature weights are hermgauss's weights divided by
sqrt(pi), so that they sum to one.
"""
from __future__ import annotations

from functools import lru_cache

import numpy as np

from .base import Generator, Generator1D


@lru_cache(maxsize=None)
def _gauss_hermite(m: int):
    """(roots, weights) of the m-point Gauss-Hermite rule for the weight exp(-z^2)."""
    return np.polynomial.hermite.hermgauss(m)


class GaussHermite1D(Generator1D):
    """Gauss-Hermite nodes centred at `mean`, stretched by `scaling`."""

    def __init__(self, mean: float = 0.0, scaling: float = 1.0) -> None:
        super().__init__(is_nested=False)
        self._mean = mean
        self._scaling = scaling
        self._nodes = {}

    @property
    def mean(self) -> float:
        return self._mean

    @property
    def scaling(self) -> float:
        return self._scaling

    def __call__(self, n: int) -> np.ndarray:
        n = int(n)
        if n not in self._nodes:
            self._nodes[n] = self.scale(_gauss_hermite(n + 1)[0])
        return self._nodes[n]

    def get_quadrature_weights(self, n: int) -> np.ndarray:
        return _gauss_hermite(int(n) + 1)[1] / np.sqrt(np.pi)

    def scale(self, x):
        return self._mean + self._scaling * np.asarray(x)

    def scale_back(self, x):
        return (np.asarray(x) - self._mean) / self._scaling

    def get_random(self, n: int = 1):
        """n samples of the rule's measure: z ~ N(0, 1/2) (density ~ exp(-z^2)), mapped."""
        return self.scale(np.random.standard_normal(n) * np.sqrt(0.5))

    def spectral_map(self):
        a = 1.0 / float(self._scaling)
        return ("hermite", a, -float(self._mean) * a)

    def __repr__(self) -> str:
        return "GaussHermite1D(mean=%r, scaling=%r)" % (self._mean, self._scaling)


class GaussHermite(Generator):
    """Gauss-Hermite nodes in every dimension.  Give `dim` (mean 0, scaling 1),
    or per-dimension `mean` and/or `scaling` arrays (the other defaults to 0 or
    1); `dim`, when also given, must match their length."""

    def __init__(self, mean=None, scaling=None, dim: int = None):
        given = [np.atleast_1d(np.asarray(v, dtype=float)) for v in (mean, scaling) if v is not None]
        if dim is None and not given:
            raise ValueError("GaussHermite needs `dim`, `mean` or `scaling`")
        d = int(dim) if dim is not None else given[0].size
        self._mean = np.zeros(d) if mean is None else np.asarray(mean)
        self._scaling = np.ones(d) if scaling is None else np.asarray(scaling)
        super().__init__([GaussHermite1D(m, s) for m, s in zip(np.broadcast_to(self._mean, (d,)),
                                                               np.broadcast_to(self._scaling, (d,)))])

    @property
    def mean(self) -> np.ndarray:
        return self._mean

    @property
    def scaling(self) -> np.ndarray:
        return self._scaling

    def scale(self, x):
        return self._mean + self._scaling * np.asarray(x)

    def scale_back(self, x):
        return (np.asarray(x) - self._mean) / self._scaling

    def __repr__(self) -> str:
        return "GaussHermite(dim=%d, mean=%s, scaling=%s)" % (self.dim, np.ravel(self._mean).tolist(),
                                                              np.ravel(self._scaling).tolist())
