"""Oracle restatement of the multi-index set algorithms (test infrastructure).

Follows ``src/smolyax/indices.py`` of the reference.  Floating-point
comparisons are performed in exactly the same order and form as the
reference (``j * k_i < rem`` with ``rem = rem - j * k_i``; additive
``used + j * k_i < t`` in the cardinality counter), because bit-exactness of
the index set depends on it.  All arithmetic is IEEE float64 (Python floats).

Sparse multi-indices are tuples ``((dim, degree), ...)`` in ascending ``dim``
order, as in the reference.
"""

from __future__ import annotations

from collections import defaultdict


def _as_floats(k):
    return [float(v) for v in k]


def indexset(k, t):
    """Lambda_{k,t} in the reference's DFS order.

    Follows ``src/smolyax/indices.py:20-69``: a LIFO stack of
    ``(dim, remaining budget, head)``; an entry is final when ``dim >= d`` or
    ``k[dim] >= remaining``; otherwise the ``nu_dim = 0`` continuation is
    pushed first and then ``nu_dim = 1, 2, ...`` while ``j * k[dim] <
    remaining`` (remaining budget updated subtractively).
    """
    k = _as_floats(k)
    t = float(t)
    d = len(k)
    out = []
    todo = [(0, t, ())]
    while todo:
        dim, rem, head = todo.pop()
        if dim >= d or k[dim] >= rem:
            out.append(head)
            continue
        todo.append((dim + 1, rem, head))
        j = 1
        while j * k[dim] < rem:
            todo.append((dim + 1, rem - j * k[dim], head + ((dim, j),)))
            j += 1
    return out


def indexset_cardinality(k, t):
    """|Lambda_{k,t}| by the additive DFS of ``src/smolyax/indices.py:72-118``."""
    k = _as_floats(k)
    t = float(t)
    d = len(k)
    count = 0
    todo = [(0, 0.0)]
    while todo:
        dim, used = todo.pop()
        if dim >= d:
            count += 1
            continue
        rem = t - used
        if dim + 1 < d and k[dim + 1] < rem:
            todo.append((dim + 1, used))
        else:
            count += 1
        j = 1
        while used + j * k[dim] < t:
            todo.append((dim + 1, used + j * k[dim]))
            j += 1
    return count


def smolyak_coefficient(k, d, rem_t, parity):
    """zeta = sum over admissible e in {0,1}^d of (-1)^|e| (``indices.py:121-168``).

    The DFS visits node ``(i, rt, p)``: the 'skip' child is pushed only if
    ``k[i+1] < rt`` (otherwise the branch terminates and contributes
    ``1 - 2p``); the 'include' child ``(i+1, rt - k[i], p ^ 1)`` is pushed if
    ``k[i] < rt``.
    """
    k = _as_floats(k)
    total = 0
    todo = [(0, float(rem_t), int(parity))]
    while todo:
        i, rt, p = todo.pop()
        if i >= d:
            total += 1 - (p << 1)
            continue
        if i + 1 < d and k[i + 1] < rt:
            todo.append((i + 1, rt, p))
        else:
            total += 1 - (p << 1)
        if k[i] < rt:
            todo.append((i + 1, rt - k[i], p ^ 1))
    return total


def _nodeset_cardinality_non_nested(k, t):
    """Sum of prod(nu_j + 1) over nu with zeta != 0 (``indices.py:175-211``)."""
    k = _as_floats(k)
    t = float(t)
    d = len(k)
    total = 0
    todo = [(0, t, 0, 1)]
    while todo:
        dim, rem, par, prod = todo.pop()
        if dim >= d or not (dim + 1 < d and k[dim + 1] < rem):
            if smolyak_coefficient(k, d, rem, par) != 0:
                total += prod
        if dim < d:
            if dim + 1 < d and k[dim + 1] < rem:
                todo.append((dim + 1, rem, par, prod))
            cost = k[dim]
            j = 1
            while cost * j < rem:
                todo.append((dim + 1, rem - cost * j, par ^ (j & 1), prod * (j + 1)))
                j += 1
    return total


def nodeset_cardinality(k, t, nested=False):
    """Number of interpolation nodes (``indices.py:262-289``)."""
    if nested:
        return indexset_cardinality(k, t)
    return _nodeset_cardinality_non_nested(k, t)


def non_zero_indices_and_zetas(k, t):
    """nu in Lambda_{k,t} with zeta != 0, binned by n = |supp nu| (``indices.py:214-259``).

    Emission happens when a node cannot take its 'skip' step
    (``not (i+1 < d and k[i+1] < rem)``); zeta is computed from the remaining
    budget alone with parity 0.  Returns ``(n2nus, n2zetas)`` as defaultdicts
    of lists, in the reference's DFS order.
    """
    k = _as_floats(k)
    t = float(t)
    d = len(k)
    n2nus, n2zetas = defaultdict(list), defaultdict(list)
    todo = [(0, t, ())]
    while todo:
        i, rem, nu = todo.pop()
        if i >= d or not (i + 1 < d and k[i + 1] < rem):
            z = smolyak_coefficient(k, d, rem, 0)
            if z != 0:
                n2nus[len(nu)].append(nu)
                n2zetas[len(nu)].append(z)
        if i < d:
            if i + 1 < d and k[i + 1] < rem:
                todo.append((i + 1, rem, nu))
            j = 1
            while j * k[i] < rem:
                todo.append((i + 1, rem - j * k[i], nu + ((i, j),)))
                j += 1
    return n2nus, n2zetas


def find_approximate_threshold(k, m, nested, max_iter=32, accuracy=0.001):
    """Bracket by factors of 1.2, then bisect (``indices.py:292-355``)."""
    assert m > 0
    if m == 1:
        return 1
    lo, hi = 1.0, 2.0
    while nodeset_cardinality(k, lo, nested) > m:
        lo, hi = lo / 1.2, lo
    while nodeset_cardinality(k, hi, nested) < m:
        lo, hi = hi, hi * 1.2
    t_c = lo + (hi - lo) / 2.0
    m_c = nodeset_cardinality(k, t_c, nested)
    for _ in range(max_iter):
        if m_c > m:
            hi = t_c
        else:
            lo = t_c
        t_c = lo + (hi - lo) / 2.0
        m_c = nodeset_cardinality(k, t_c, nested)
        if abs(m_c - m) / m < accuracy:
            break
    return t_c
