"""Affine maps between axis-aligned boxes, used by the node rules.

A box is held as an array of shape (d, 2) with one (lower, upper) row per
dimension.  Points are arrays whose last axis runs over the d dimensions; a
one-dimensional box maps arrays of any shape element by element.
"""
from __future__ import annotations

import numpy as np

# the interval on which the nested Leja sequence is defined
UNIT_INTERVAL = np.array([[-1.0, 1.0]])

# how far a coordinate may lie outside its source interval (relative to the
# larger of 1 and the bound's magnitude) and still count as inside: points
# that went through a map and back differ from the bounds by a few ulps
_SLACK = 1e-5


def as_box(bounds, what="box") -> np.ndarray:
    """(d, 2) float array of interval bounds; every upper bound must exceed its lower bound."""
    b = np.asarray(bounds, dtype=float)
    if b.ndim == 0 or b.shape[-1] != 2 or b.ndim > 2:
        raise AssertionError("%s: expected (lower, upper) pairs, got an array of shape %s" % (what, b.shape))
    b = b.reshape(-1, 2)
    if not np.all(b[:, 0] < b[:, 1]):
        raise AssertionError("%s: some lower bound is not below its upper bound: %s" % (what, b.tolist()))
    return b


def map_points(x, src, dst):
    """Maps x from box `src` to box `dst` (both (d, 2)): each coordinate goes
    through its position (x - lower) / width in the source interval, then to
    lower' + position * width' of the target.  Coordinates outside the source
    box raise AssertionError."""
    src = as_box(src, "source interval")
    dst = as_box(dst, "target interval")
    if src.shape != dst.shape:
        raise AssertionError("source and target boxes differ in dimension: %d vs %d" % (src.shape[0], dst.shape[0]))
    x = np.asarray(x, dtype=float)
    d = src.shape[0]
    if d > 1 and (x.ndim == 0 or x.shape[-1] != d):
        raise AssertionError("points of shape %s do not have %d coordinates on their last axis" % (x.shape, d))
    lo, hi = (src[:, 0], src[:, 1]) if d > 1 else (src[0, 0], src[0, 1])
    nlo, nhi = (dst[:, 0], dst[:, 1]) if d > 1 else (dst[0, 0], dst[0, 1])
    below = x < lo - _SLACK * np.maximum(1.0, np.abs(lo))
    above = x > hi + _SLACK * np.maximum(1.0, np.abs(hi))
    if np.any(below) or np.any(above):
        raise AssertionError("%d coordinate(s) below and %d above the source interval; first offenders: %s"
                             % (int(np.count_nonzero(below)), int(np.count_nonzero(above)),
                                np.asarray(x[below | above]).ravel()[:6].tolist()))
    pos = (x - lo) / (hi - lo)
    return pos * (nhi - nlo) + nlo
