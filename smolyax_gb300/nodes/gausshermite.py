"""Gauss-Hermite nodes (mirrors ``src/smolyax/nodes/gausshermite.py``)."""
from __future__ import annotations

from functools import lru_cache

import numpy as np

from .base import Generator, Generator1D


@lru_cache(maxsize=None)
def _hermgauss(m: int):
    return np.polynomial.hermite.hermgauss(m)


class GaussHermite1D(Generator1D):
    """Non-nested Gauss-Hermite nodes ``mean + scaling * z`` (``gausshermite.py:10-164``)."""

    def __init__(self, mean: float = 0.0, scaling: float = 1.0) -> None:
        super().__init__(is_nested=False)
        self._mean = mean
        self._scaling = scaling
        self._nodes = lru_cache(maxsize=None)(lambda n: self.scale(_hermgauss(n + 1)[0]))

    @property
    def mean(self) -> float:
        return self._mean

    @property
    def scaling(self) -> float:
        return self._scaling

    def __call__(self, n: int) -> np.ndarray:
        return self._nodes(int(n))

    def get_quadrature_weights(self, n: int) -> np.ndarray:
        return _hermgauss(int(n) + 1)[1] / np.sqrt(np.pi)

    def scale(self, x):
        return self._mean + self._scaling * x

    def scale_back(self, x):
        return (x - self._mean) / self._scaling

    def get_random(self, n: int = 1):
        # N(mean, scaling/2)-style sampling of the reference: z ~ N(0, 1/2)
        return self.scale(np.random.randn(n) / np.sqrt(2))

    def spectral_map(self):
        a = 1.0 / float(self._scaling)
        return ("hermite", a, -float(self._mean) * a)

    def __repr__(self) -> str:
        return f"Gauss-Hermite (mean = {self._mean}, scaling = {self._scaling})"


class GaussHermite(Generator):
    """Gauss-Hermite nodes in every dimension (``gausshermite.py:167-249``)."""

    def __init__(self, mean=None, scaling=None, dim: int = None):
        if dim is None:
            if scaling is not None:
                dim = len(scaling)
            elif mean is not None:
                dim = len(mean)
            else:
                raise ValueError("Must specify at least one of 'dim', 'mean', or 'scaling'.")
        if mean is None and scaling is None:
            Generator.__init__(self, [GaussHermite1D()] * dim)
            self._mean = np.zeros(dim)
            self._scaling = np.ones(dim)
        else:
            self._mean = np.zeros(dim) if mean is None else np.asarray(mean)
            self._scaling = np.ones(dim) if scaling is None else np.asarray(scaling)
            Generator.__init__(self, [GaussHermite1D(m, s) for m, s in zip(self._mean, self._scaling)])

    def scale(self, x):
        return self._mean + self._scaling * x

    def scale_back(self, x):
        return (x - self._mean) / self._scaling

    def __repr__(self) -> str:
        return f"Gauss Hermite (d = {self.dim}, mean = {self._mean.tolist()}, scaling = {self._scaling.tolist()})"
