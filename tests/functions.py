"""Seeded target functions shared by the golden-vector generator and the tests.

They follow the workload descriptions of the benchmark configurations: the
rational function 1/(1 + w.x) with w_j ~ U(0,1)/(j+1)^2 rescaled to sum 0.5,
its vector-valued variant with one weight row per output, the exponential
family exp(-sum_j a_ij x_j / (j+1)^1.5) with a_ij ~ N(0, 0.3^2), and
tensor-product polynomials of a degree vector inside the index set (which
the interpolant reproduces exactly).
"""
import numpy as np
from numpy.polynomial import hermite, legendre


def rational(d, seed=0):
    rng = np.random.default_rng(seed)
    w = rng.uniform(0, 1, d) / (np.arange(d) + 1) ** 2
    w *= 0.5 / w.sum()

    def f(x):
        x = np.asarray(x, dtype=float)
        return np.atleast_1d(1.0 / (1.0 + x @ w)) if x.ndim == 1 else (1.0 / (1.0 + x @ w))[:, None]

    f.w = w
    return f


def rational_vec(d, d_out, seed=0):
    rng = np.random.default_rng(seed)
    W = rng.uniform(0, 1, (d_out, d)) / (np.arange(d) + 1) ** 2
    W *= 0.5 / W.sum(axis=1, keepdims=True)

    def f(x):
        x = np.asarray(x, dtype=float)
        return 1.0 / (1.0 + x @ W.T)

    f.W = W
    return f


def exponential(d, d_out, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.normal(0.0, 0.3, (d_out, d)) / (np.arange(d) + 1) ** 1.5

    def f(x):
        x = np.asarray(x, dtype=float)
        return np.exp(-(x @ A.T))

    f.A = A
    return f


class TensorPolynomial:
    """f_o(x) = prod_j p_{nu_oj}(s_j(x_j)): Legendre (Leja rules) or Hermite (GH rules).

    ``maps`` holds per-dimension affine maps (scale a, shift b) to the
    reference interval: s_j(x) = (x - b_j) / a_j.
    """

    def __init__(self, degrees, kind, shift, scale):
        self.degrees = [tuple(int(v) for v in nu) for nu in degrees]
        self.kind = kind
        self.shift = np.asarray(shift, dtype=float)
        self.scale = np.asarray(scale, dtype=float)

    def _p(self, deg, z):
        c = [0] * deg + [1]
        return legendre.legval(z, c) if self.kind == "leja" else hermite.hermval(z, c)

    def _dp(self, deg, z):
        c = [0] * deg + [1]
        if self.kind == "leja":
            return legendre.legval(z, legendre.legder(c))
        return hermite.hermval(z, hermite.hermder(c))

    def __call__(self, x):
        x = np.asarray(x, dtype=float)
        z = (x - self.shift) / self.scale
        cols = [np.prod([self._p(g, z[..., j]) for j, g in enumerate(nu)], axis=0) for nu in self.degrees]
        return np.stack(cols, axis=-1)

    def gradient(self, x):
        x = np.atleast_2d(np.asarray(x, dtype=float))
        z = (x - self.shift) / self.scale
        P, d = x.shape
        out = np.zeros((P, len(self.degrees), d))
        for o, nu in enumerate(self.degrees):
            vals = np.stack([self._p(g, z[:, j]) for j, g in enumerate(nu)])
            ders = np.stack([self._dp(g, z[:, j]) / self.scale[j] for j, g in enumerate(nu)])
            for j in range(d):
                others = np.prod(np.delete(vals, j, axis=0), axis=0) if d > 1 else 1.0
                out[:, o, j] = ders[j] * others
        return out

    def integral(self):
        # Legendre/Hermite of degree > 0 integrate to zero under the normalised measures.
        return np.array([1.0 if all(g == 0 for g in nu) else 0.0 for nu in self.degrees])
