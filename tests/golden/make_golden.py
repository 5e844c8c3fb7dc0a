"""Generate golden vectors by running the reference implementation itself.

Run from the repository root in a container that has the reference sources:

    python tests/golden/make_golden.py /root/reference/src

The reference (JoWestermann/smolyax) needs jax and numba, which are not
installed here; ``tests/golden/shim`` provides numpy-backed stand-ins for the
small surface the reference uses (``jax.numpy`` array ops, an identity
``jit``, a looping ``vmap``, an identity ``numba.njit``), so the reference's
own code runs unmodified.  The outputs are written to ``tests/golden/*.npz``
and are what the oracle and the GPU library are checked against.
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "shim"))
sys.path.insert(0, os.path.dirname(HERE))  # tests/ for functions.py


def _flatten_nus(nus, zetas=None):
    lens = np.array([len(nu) for nu in nus], dtype=np.int64)
    dims = np.array([d for nu in nus for d, _ in nu], dtype=np.int64)
    degs = np.array([g for nu in nus for _, g in nu], dtype=np.int64)
    out = dict(lens=lens, dims=dims, degs=degs)
    if zetas is not None:
        out["zetas"] = np.array(zetas, dtype=np.int64)
    return out


def _nonzero_flat(indices, k, t):
    n2nus, n2z = indices.non_zero_indices_and_zetas(k, t)
    keys = list(n2nus.keys())  # dict order of the reference (first emission order of n)
    nus, zs = [], []
    for n in keys:
        nus.extend(n2nus[n])
        zs.extend(n2z[n])
    flat = _flatten_nus(nus, zs)
    flat["n_keys"] = np.array(keys, dtype=np.int64)
    return flat


def gen_indices(indices, out):
    rng = np.random.default_rng(20240601)
    cases = []
    for i in range(12):
        d = int(rng.integers(1, 6))
        a = 1.1 + 2.9 * rng.random()
        b = 0.1 + 1.9 * rng.random()
        k = np.log([a + b * j for j in range(d)]) / np.log(a)
        n_t = int(rng.integers(1, 100))
        t = indices.find_approximate_threshold(k, n_t, nested=(i % 2) == 0)
        cases.append(("rand%d" % i, k, float(t), n_t, (i % 2) == 0))
    for i in range(3):  # unsorted weight vectors pin the DFS semantics for general k
        d = int(rng.integers(3, 6))
        k = rng.uniform(0.7, 3.0, d)
        cases.append(("unsorted%d" % i, k, float(rng.uniform(3.0, 7.0)), 0, True))
    data = {}
    for name, k, t, n_t, nested in cases:
        iset = indices.indexset(k, t)
        fl = _flatten_nus(iset)
        data[name + "/k"] = np.asarray(k, dtype=float)
        data[name + "/t"] = np.array(t)
        data[name + "/target"] = np.array([n_t, int(nested)])
        for key, v in fl.items():
            data[name + "/iset_" + key] = v
        data[name + "/card"] = np.array(
            [
                indices.indexset_cardinality(k, t),
                indices.nodeset_cardinality(k, t, nested=True),
                indices.nodeset_cardinality(k, t, nested=False),
            ]
        )
        # Smolyak coefficients with the remaining budget computed as the reference's test does.
        rems = np.array([t - sum(g * k[dd] for dd, g in nu) for nu in iset])
        data[name + "/coef_rem"] = rems
        data[name + "/coef"] = np.array([indices.smolyak_coefficient(k, len(k), r, 0) for r in rems])
        for key, v in _nonzero_flat(indices, k, t).items():
            data[name + "/nz_" + key] = v
    data["names"] = np.array([c[0] for c in cases])
    np.savez_compressed(os.path.join(out, "indices_small.npz"), **data)

    big = {}
    cfg = [
        ("cfg1", 10, 8.831421),
        ("cfg2", 1000, 8.224520),
        ("cfg3", 100, 9.464636),
        ("cfg3alt", 100, 7.723434),
        ("cfg4", 200, 7.853604),
    ]
    for name, d, t in cfg:
        k = np.log((2 + np.arange(d)) / np.log(2))
        t0 = time.time()
        for key, v in _nonzero_flat(indices, k, t).items():
            big[name + "/nz_" + key] = v
        big[name + "/card"] = np.array(
            [
                indices.indexset_cardinality(k, t),
                indices.nodeset_cardinality(k, t, nested=True),
                indices.nodeset_cardinality(k, t, nested=False),
            ]
        )
        big[name + "/d"] = np.array(d)
        big[name + "/t"] = np.array(t)
        print("  indices", name, "%.1fs" % (time.time() - t0))
    # cardinality pins of the reference's runtime tests: k_j = log2(2 + j), d = 10000
    k = np.log([2 + i for i in range(10000)]) / np.log(2)
    pins = []
    for t in (5.3, 7.78, 10.317):
        pins.append([t, len(indices.indexset(k, t)), indices.indexset_cardinality(k, t)])
    big["pins_d10000"] = np.array(pins)
    thr = []
    for d, m, nested in [(100, 1000, True), (100, 1000, False), (1000, 10000, True)]:
        kk = np.log([2 + i for i in range(d)]) / np.log(2)
        acc = 0.01 if nested else 0.1
        tt = indices.find_approximate_threshold(kk, m, nested=nested, accuracy=acc)
        thr.append([d, m, int(nested), acc, tt, indices.nodeset_cardinality(kk, tt, nested=nested)])
    big["thresholds"] = np.array(thr)
    np.savez_compressed(os.path.join(out, "indices_configs.npz"), **big)


def _node_gen(nodes, kind, d, rng, default):
    if kind == "leja":
        if default:
            return nodes.Leja(dim=d), ("leja", None, None)
        dom = np.sort(rng.random((d, 2)), axis=1)
        return nodes.Leja(domains=dom), ("leja", dom, None)
    if default:
        return nodes.GaussHermite(dim=d), ("gh", None, None)
    mean = rng.normal(size=d)
    scaling = rng.random(d) + 0.2
    return nodes.GaussHermite(mean, scaling), ("gh", mean, scaling)


def _points(spec, d, P, rng):
    kind, a, b = spec
    if kind == "leja":
        z = rng.uniform(-1, 1, (P, d))
        if a is None:
            return z
        return (z + 1) / 2 * (a[:, 1] - a[:, 0]) + a[:, 0]
    z = rng.normal(size=(P, d)) / np.sqrt(2)
    mean = np.zeros(d) if a is None else a
    scaling = np.ones(d) if b is None else b
    return mean + scaling * z


def gen_interp(interp_mod, nodes, indices, out):
    import functions as fns

    rng = np.random.default_rng(424242)
    data = {}
    names = []
    for case in range(16):
        kind = "leja" if case % 2 == 0 else "gh"
        default = (case // 2) % 2 == 0
        d = int(rng.integers(1, 5))
        gen, spec = _node_gen(nodes, kind, d, rng, default)
        k = np.sort(rng.uniform(1, 10, d))
        k = k / k[0]
        t = float(rng.uniform(1, 8))
        d_out = int(rng.integers(1, 4))
        iset = indices.indexset(k, t)
        degs = []
        for _ in range(d_out):
            nu = iset[int(rng.integers(len(iset)))]
            dense = [0] * d
            for dd, g in nu:
                dense[dd] = g
            degs.append(dense)
        if spec[0] == "leja":
            if spec[1] is None:
                shift, scale = np.zeros(d), np.ones(d)
            else:
                shift, scale = spec[1].mean(axis=1), (spec[1][:, 1] - spec[1][:, 0]) / 2
        else:
            shift = np.zeros(d) if spec[1] is None else spec[1]
            scale = np.ones(d) if spec[2] is None else spec[2]
        f = fns.TensorPolynomial(degs, kind, shift, scale)
        ip = interp_mod.SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=d_out, f=f)
        x = _points(spec, d, 7, rng)
        # one exact interpolation node (the zero point of every rule) exercises the one-hot rule
        zero = np.array([g(0)[0] for g in gen])
        xs = np.vstack([x, zero[None, :]])
        name = "case%d" % case
        names.append(name)
        data[name + "/kind"] = np.array(kind)
        data[name + "/k"] = k
        data[name + "/t"] = np.array(t)
        data[name + "/d_out"] = np.array(d_out)
        data[name + "/poly_degrees"] = np.array(degs)
        data[name + "/dom"] = np.zeros((d, 2)) if spec[1] is None or kind != "leja" else spec[1]
        data[name + "/has_dom"] = np.array(int(kind == "leja" and spec[1] is not None))
        data[name + "/mean"] = shift if kind == "gh" else np.zeros(d)
        data[name + "/scaling"] = scale if kind == "gh" else np.ones(d)
        data[name + "/x"] = xs
        data[name + "/y"] = np.asarray(ip(xs))
        data[name + "/grad"] = np.asarray(ip.gradient(x))
        data[name + "/integral"] = np.asarray(ip.integral())
        data[name + "/n_f_evals"] = np.array([ip.n_f_evals, ip.n_f_evals_new])
    data["names"] = np.array(names)
    np.savez_compressed(os.path.join(out, "interp_small.npz"), **data)


def gen_configs(interp_mod, nodes, out):
    import functions as fns

    data = {}
    # Plain FP64 Leja on [-1,1]^10, |Lambda| ~ 1000, 1e4 points (seed 1).
    d = 10
    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.rational(d, seed=0)
    t0 = time.time()
    ip = interp_mod.SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=d), k=k, t=8.831421, d_out=1, f=f)
    x = np.random.default_rng(1).uniform(-1, 1, (10000, d))
    data["cfg1/y"] = np.asarray(ip(x))
    data["cfg1/grad"] = np.asarray(ip.gradient(x[:64]))
    data["cfg1/integral"] = np.asarray(ip.integral())
    data["cfg1/n_f_evals"] = np.array([ip.n_f_evals, ip.n_f_evals_new])
    print("  cfg1 %.1fs" % (time.time() - t0))

    # d_in = 1000, |Lambda| ~ 1e4, scalar rational f; 256 points of the seed-1 stream.
    d = 1000
    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.rational(d, seed=0)
    t0 = time.time()
    ip = interp_mod.SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=d), k=k, t=8.224520, d_out=1, f=f)
    x = np.random.default_rng(1).uniform(-1, 1, (256, d))
    data["cfg2/x_checksum"] = np.array([x.sum(), (x * x).sum()])
    data["cfg2/y"] = np.asarray(ip(x))
    data["cfg2/grad"] = np.asarray(ip.gradient(x[:4]))
    data["cfg2/integral"] = np.asarray(ip.integral())
    data["cfg2/n_f_evals"] = np.array([ip.n_f_evals, ip.n_f_evals_new])
    print("  cfg2 %.1fs" % (time.time() - t0))

    # Differentiation workload: Leja d_in = 200, d_out = 64, |Lambda| ~ 5e3.
    d = 200
    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.rational_vec(d, 64, seed=0)
    t0 = time.time()
    ip = interp_mod.SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=d), k=k, t=7.853604, d_out=64, f=f)
    x = np.random.default_rng(1).uniform(-1, 1, (64, d))
    data["cfg4/y"] = np.asarray(ip(x))
    data["cfg4/grad"] = np.asarray(ip.gradient(x[:3]))
    data["cfg4/integral"] = np.asarray(ip.integral())
    print("  cfg4 %.1fs" % (time.time() - t0))

    # Gauss-Hermite d_in = 100 with the exponential family, reduced to 8 outputs.
    d = 100
    k = np.log((2 + np.arange(d)) / np.log(2))
    for tag, t in (("cfg3alt", 7.723434), ("cfg3", 9.464636)):
        f = fns.exponential(d, 8, seed=0)
        t0 = time.time()
        ip = interp_mod.SmolyakBarycentricInterpolator(node_gen=nodes.GaussHermite(dim=d), k=k, t=t, d_out=8, f=f)
        x = np.random.default_rng(1).normal(size=(32, d))
        data[tag + "/y"] = np.asarray(ip(x))
        data[tag + "/integral"] = np.asarray(ip.integral())
        data[tag + "/n_f_evals"] = np.array([ip.n_f_evals, ip.n_f_evals_new])
        if tag == "cfg3alt":
            data[tag + "/grad"] = np.asarray(ip.gradient(x[:2]))
        print("  %s %.1fs" % (tag, time.time() - t0))
    np.savez_compressed(os.path.join(out, "interp_configs.npz"), **data)


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference source dir (the folder holding smolyax/)> [indices|interp|configs ...]")
    ref_src = sys.argv[1]
    sys.path.insert(0, ref_src)
    from smolyax import indices, nodes
    from smolyax import interpolation as interp_mod

    out = HERE
    which = sys.argv[2:] or ["indices", "interp", "configs"]
    if "indices" in which:
        gen_indices(indices, out)
    if "interp" in which:
        gen_interp(interp_mod, nodes, indices, out)
    if "configs" in which:
        gen_configs(interp_mod, nodes, out)


if __name__ == "__main__":
    main()
