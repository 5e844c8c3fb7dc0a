r"""Quadrature workloads on the interpolant (the reference's
``notebooks/smolyak_quadrature.ipynb`` study, on the GPU).

* :func:`integral_sweep` -- the Smolyak quadrature
  $Q^\Lambda[f] = \int I^\Lambda[f]\,d\mu$ (``integral()``,
  ``interpolation.py:347-390``) for a family of thresholds t, with the number
  of function evaluations of each and its distance to the finest one.
* :func:`monte_carlo` -- the Monte-Carlo estimate
  $\frac1N \sum_j I^\Lambda[f](x_j)$, $x_j \sim \mu$, of the same integral,
  with samples drawn on the device (uniform on a Leja rule's box, normal for
  Gauss-Hermite rules: the measure $e^{-z^2}/\sqrt\pi$ of the nodes, i.e.
  N(mean, scaling^2 / 2)) and evaluated in chunks; returns the mean and its
  standard error, so that convergence at the rate $N^{-1/2}$ can be checked.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import nodes as _nodes
from .interpolation import SmolyakBarycentricInterpolator


def integral_sweep(node_gen, k, f, thresholds, d_out=1, **kw):
    """Builds the interpolant of f for every threshold in `thresholds` and
    integrates it.  Returns one dict per threshold: t, n_f_evals, the integral
    (numpy, shape (d_out,)), the seconds the integral took, and ``err``: the
    distance max_o |Q_t - Q_last| to the last (finest) threshold's integral."""
    out = []
    f_evals = None
    for t in thresholds:
        ip = SmolyakBarycentricInterpolator(node_gen=node_gen, k=k, t=float(t), d_out=d_out, **kw)
        f_evals = ip.set_f(f=f, f_evals=f_evals)  # nodes shared between thresholds are evaluated once
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        q = ip.integral().cpu().numpy()
        out.append(dict(t=float(t), n_f_evals=int(ip.n_f_evals), integral=q, seconds=time.perf_counter() - t0))
    for r in out:
        r["err"] = float(np.max(np.abs(r["integral"] - out[-1]["integral"])))
    return out


def _device_sampler(node_gen, device):
    """Per-dimension (kind, a, b): x = a * u + b with u ~ U[-1, 1] (kind 0) or
    u ~ N(0, 1/2) (kind 1); None for rules whose measure is not one of these."""
    kind, a, b = [], [], []
    for g in node_gen:
        if isinstance(g, _nodes.Leja1D):
            dom = g.domain
            lo, hi = (-1.0, 1.0) if dom is None else (float(np.ravel(dom)[0]), float(np.ravel(dom)[1]))
            kind.append(0), a.append((hi - lo) / 2), b.append((hi + lo) / 2)
        elif isinstance(g, _nodes.GaussHermite1D):
            kind.append(1), a.append(float(g.scaling)), b.append(float(g.mean))
        else:
            return None
    T = lambda v, dt: torch.as_tensor(np.asarray(v), dtype=dt, device=device)
    return T(kind, torch.bool), T(a, torch.float64), T(b, torch.float64)


def monte_carlo(ip, n, seed=0, precision="fp32", chunk=1 << 20):
    """Monte-Carlo mean of the interpolant over n samples of its node rules'
    measure: (mean, standard error), numpy arrays of shape (d_out,).  Samples
    are drawn and evaluated on the device chunk by chunk; sums are kept in FP64."""
    dev = torch.device("cuda", torch.cuda.current_device())
    smp = _device_sampler(ip._node_gen, dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    s1 = torch.zeros(ip.d_out, dtype=torch.float64, device=dev)
    s2 = torch.zeros_like(s1)
    done = 0
    while done < n:
        m = min(chunk, n - done)
        if smp is None:
            x = torch.as_tensor(np.atleast_2d(ip._node_gen.get_random(m)).reshape(m, ip.d_in), device=dev)
        else:
            normal, a, b = smp
            u = torch.rand(m, ip.d_in, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
            z = torch.randn(m, ip.d_in, dtype=torch.float64, device=dev, generator=gen) * np.sqrt(0.5)
            x = torch.where(normal, z, u) * a + b
        y = ip(x, precision=precision).double()
        s1 += y.sum(0)
        s2 += (y * y).sum(0)
        done += m
    mean = (s1 / n).cpu().numpy()
    var = np.maximum((s2 / n).cpu().numpy() - mean**2, 0.0)
    return mean, np.sqrt(var / max(n - 1, 1))
