"""Quadrature workloads (``smolyax_gb300.quadrature``): the integral of the
interpolant over a sweep of thresholds, pinned against the oracle's
``integral`` (the reference's ``interpolation.py:347-390``), and the
Monte-Carlo mean of the interpolant converging to it at the rate N^-1/2
(every estimate within 6 standard errors of the integral).

Bound against the oracle: 1e-12 relative for the Leja sweep; for the
Gauss-Hermite sweep, where the combination sum cancels more (|zeta| up to
553 at t = 7.723434), the same contract as the FP64 evaluation tests: within
the reference's own FP64 error of this configuration, 1.06e-11 against the
extended-precision value (``tests/golden/make_exact.py``), i.e. 2.2e-11
between two FP64 evaluations."""
import numpy as np
import pytest

import functions as fns

pytestmark = pytest.mark.gpu

SWEEPS = {
    # Leja d_in=10 rational f (the |Lambda| = 1000 configuration and coarser ones)
    "leja10": ("leja", 10, 1, fns.rational(10, seed=0), (5.0, 6.5, 8.0, 8.831421), 1e-12),
    # Gauss-Hermite d_in=100 exponential f, 2 outputs (up to the |nodes| ~ 2e4 threshold)
    "gh100": ("gh", 100, 2, fns.exponential(100, 2, seed=0), (4.0, 6.0, 7.723434), 2.2e-11),
}


@pytest.mark.parametrize("tag", list(SWEEPS))
def test_integral_sweep_matches_oracle(tag):
    from oracle import interp as ointerp
    from smolyax_gb300 import nodes
    from smolyax_gb300.quadrature import integral_sweep

    kind, d, d_out, f, ts, bound = SWEEPS[tag]
    k = np.log((2 + np.arange(d)) / np.log(2))
    gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
    res = integral_sweep(gen, k, f, ts, d_out=d_out)
    rule = ("leja", None) if kind == "leja" else ("gh", (0.0, 1.0))
    for r in res:
        ref = ointerp.OracleInterpolant(rules=[rule] * d, k=k, t=r["t"], d_out=d_out, f=f,
                                        nested=kind == "leja").integral()
        rel = float(np.max(np.abs(r["integral"] - ref) / np.abs(ref)))
        print("%s t=%.4f n_f_evals=%d: integral %s, rel diff vs oracle %.2e, |Q_t - Q_finest| %.2e"
              % (tag, r["t"], r["n_f_evals"], np.array2string(r["integral"], precision=12), rel, r["err"]))
        assert rel < bound
    assert [r["n_f_evals"] for r in res] == sorted(r["n_f_evals"] for r in res)
    assert res[-2]["err"] < res[0]["err"]


def test_monte_carlo_converges_to_the_integral():
    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes
    from smolyax_gb300.quadrature import monte_carlo

    for kind, d, t, f in (("leja", 10, 8.831421, fns.rational(10, seed=0)),
                          ("gh", 30, 6.0, fns.exponential(30, 1, seed=1))):
        k = np.log((2 + np.arange(d)) / np.log(2))
        gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
        ip = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=1, f=f)
        q = ip.integral().cpu().numpy()
        ses = []
        for n in (1 << 14, 1 << 18, 1 << 22):
            mean, se = monte_carlo(ip, n, seed=n)
            err = float(np.abs(mean - q)[0])
            print("%s MC N=%d: |mean - Q| %.3e, standard error %.3e" % (kind, n, err, se[0]))
            assert err <= 6 * se[0]
            ses.append(se[0])
        # the standard error falls as N^-1/2 (16x the samples: 4x smaller)
        assert 3.0 < ses[0] / ses[1] < 5.0 and 3.0 < ses[1] / ses[2] < 5.0
