"""Extended-precision values of the benchmark workloads (oracle-based).

The combination sum of the Smolyak interpolant cancels strongly (its terms
are 3e3-2e4 times larger than the result for the workloads below), so any
FP64 evaluation -- the reference's included -- carries a relative rounding
error of 1e-12 .. 1e-10.  This script evaluates the same formula in numpy's
``longdouble`` (80-bit extended precision on x86-64) with the oracle
(``oracle.interp``), so that tests can pin the GPU FP64 path pointwise against
the exact value of the FP64 data, and compare its distance to the reference's
own outputs with the reference's distance to that exact value.

    python tests/golden/make_exact.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import functions as fns  # noqa: E402
from oracle import interp as ointerp  # noqa: E402

L = np.longdouble


def _case(d, t, kind, d_out, f, x, n_grad):
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = ointerp.OracleInterpolant(rules=ointerp.rules_from_spec(kind, d), k=k, t=t, d_out=d_out, f=f,
                                   nested=(kind == "leja"))
    out = {"y": ip(x, dtype=L, pchunk=500).astype(np.float64), "integral": ip.integral(dtype=L).astype(np.float64)}
    if n_grad:
        out["grad"] = ip.gradient(x[:n_grad], dtype=L).astype(np.float64)
    return out


def main():
    assert np.finfo(L).nmant >= 63, "needs extended precision long double"
    data = {}
    cases = {
        "cfg1": (10, 8.831421, "leja", 1, fns.rational(10, seed=0), np.random.default_rng(1).uniform(-1, 1, (10000, 10)), 64),
        "cfg2": (1000, 8.224520, "leja", 1, fns.rational(1000, seed=0),
                 np.random.default_rng(1).uniform(-1, 1, (256, 1000)), 4),
        "cfg4": (200, 7.853604, "leja", 64, fns.rational_vec(200, 64, seed=0),
                 np.random.default_rng(1).uniform(-1, 1, (64, 200)), 3),
        "cfg3alt": (100, 7.723434, "gh", 8, fns.exponential(100, 8, seed=0),
                    np.random.default_rng(1).normal(size=(32, 100)), 2),
        "cfg3": (100, 9.464636, "gh", 8, fns.exponential(100, 8, seed=0), np.random.default_rng(1).normal(size=(32, 100)),
                 0),
    }
    for tag, args in cases.items():
        for key, v in _case(*args).items():
            data[tag + "/" + key] = v
        print(tag, "done", flush=True)
    np.savez_compressed(os.path.join(HERE, "exact_configs.npz"), **data)


if __name__ == "__main__":
    main()
