"""Oracle restatement of the 1-D node rules (test infrastructure).

Follows ``src/smolyax/nodes/leja.py``, ``src/smolyax/nodes/gausshermite.py``
and ``src/smolyax/barycentric.py:13-31``.  A node rule is described by a plain
tuple so that the oracle does not depend on the product's classes:

* ``("leja", None)`` or ``("leja", (a, b))`` -- Leja nodes on [-1, 1] or
  affinely mapped to [a, b];
* ``("gh", (mean, scaling))`` -- Gauss-Hermite nodes ``mean + scaling * z``.
"""

from __future__ import annotations

import numpy as np

_LEJA_CACHE = [np.array([0.0, 1.0, -1.0, 1 / np.sqrt(2), -1 / np.sqrt(2)])]


def leja_reference_nodes(n):
    """First n+1 Leja nodes on [-1, 1] (``leja.py:17``, ``leja.py:48-57``).

    Seeds 0, 1, -1, 1/sqrt2, -1/sqrt2; then node j is ``-node[j-1]`` for even j
    and ``sqrt((node[(j+1)/2] + 1) / 2)`` for odd j.
    """
    seq = _LEJA_CACHE[0]
    if n >= seq.shape[0]:
        seq = list(seq)
        for j in range(len(seq), n + 1):
            if j % 2 == 0:
                seq.append(-seq[j - 1])
            else:
                seq.append(np.sqrt((seq[(j + 1) // 2] + 1) / 2))
        seq = np.array(seq, dtype=float)
        _LEJA_CACHE[0] = seq
    return seq[: n + 1].copy()


def _leja_scale(x, domain):
    """Affine map [-1, 1] -> domain (``leja.py:95-151``, two-step form)."""
    if domain is None:
        return x
    a, b = float(domain[0]), float(domain[1])
    y = (x - (-1.0)) / (1.0 - (-1.0))
    return y * (b - a) + a


def rule_nodes(rule, n):
    """The n+1 nodes of a rule (``leja.py:59-81``, ``gausshermite.py:57-79``)."""
    kind, par = rule
    if kind == "leja":
        return _leja_scale(leja_reference_nodes(n), par)
    mean, scaling = par
    return mean + scaling * np.polynomial.hermite.hermgauss(n + 1)[0]


def rule_quadrature_weights(rule, n):
    """Quadrature weights of the first n+1 nodes.

    Leja: Vandermonde solve against the moments of the uniform probability
    measure on [-1, 1] (``leja.py:83-93``), unscaled by the domain.  GH:
    ``hermgauss(n+1)[1] / sqrt(pi)`` (``gausshermite.py:81-87``).
    """
    kind, _ = rule
    if kind == "leja":
        pts = leja_reference_nodes(n)
        vm = np.vstack([pts**i for i in range(n + 1)])
        rhs = np.array([(1 + (-1) ** i) / (2.0 * (i + 1)) for i in range(n + 1)])
        return np.linalg.solve(vm, rhs)
    return np.polynomial.hermite.hermgauss(n + 1)[1] / np.sqrt(np.pi)


def barycentric_weights(nodes, dtype=np.float64):
    """w_b = prod_a 1/(xi_a - xi_b), zero differences replaced by 1 (``barycentric.py:13-31``)."""
    nodes = np.asarray(nodes, dtype=dtype)
    diffs = nodes[:, None] - nodes
    diffs = np.where(diffs == 0, dtype(1), diffs)
    return np.prod(dtype(1) / diffs, axis=0)
