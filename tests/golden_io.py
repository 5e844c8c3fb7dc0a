"""Readers for the golden vectors written by ``tests/golden/make_golden.py``."""
import os

import numpy as np

import functions as fns

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def unflatten(lens, dims, degs):
    out, pos = [], 0
    for n in lens:
        n = int(n)
        out.append(tuple((int(dims[pos + j]), int(degs[pos + j])) for j in range(n)))
        pos += n
    return out


def nonzero_list(z, prefix):
    nus = unflatten(z[prefix + "nz_lens"], z[prefix + "nz_dims"], z[prefix + "nz_degs"])
    return nus, [int(v) for v in z[prefix + "nz_zetas"]]


def small_case(z, name):
    """Node-rule description and target polynomial of one interpolation case."""
    g = lambda key: z[name + "/" + key]
    kind = str(g("kind"))
    k = g("k")
    d = len(k)
    if kind == "leja":
        dom = g("dom") if int(g("has_dom")) else None
        shift = np.zeros(d) if dom is None else dom.mean(axis=1)
        scale = np.ones(d) if dom is None else (dom[:, 1] - dom[:, 0]) / 2
        spec = dict(kind="leja", domains=dom)
    else:
        shift, scale = g("mean"), g("scaling")
        spec = dict(kind="gh", mean=shift, scaling=scale)
    f = fns.TensorPolynomial(g("poly_degrees"), kind, shift, scale)
    return spec, k, float(g("t")), int(g("d_out")), f
