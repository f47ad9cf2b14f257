"""CPU restatement of the VEGAS map adaptation that the GPU table builder
runs (G. P. Lepage, J. Comput. Phys. 27 (1978) 192; the step vegas applies
to each dimension of an AdaptiveMap after a training pass, which PETITE's
map training relies on, all_processes.py:1160-1245).

TEST INFRASTRUCTURE: used by tests only.

Also find_maxes on one map row (``find_maxes_row``), pinned against the
reference's own do_find_max_work (tests/golden/findmax.npz).

Per dimension: the average (jac f)^2 of each increment, smoothed with
weights (1, 6, 1)/8 inside and (7, 1)/8 at the ends, normalised, compressed
as ((1 - r)/ln(1/r))^alpha, and new nodes placed so that every new increment
holds an equal share of the compressed weights, linearly inside the old
increments.  The vegas package is not installed here, so the restatement
is pinned by its own properties in the tests (a flat integrand leaves the
grid, the nodes move toward the weight, equal shares).
"""
from __future__ import annotations

import math

import numpy as np


def adapt(nodes, acc, cnt, alpha=0.5):
    """New nodes (len n+1) of one dimension from its accumulators (len n)."""
    g = np.asarray(nodes, np.float64)
    n = len(g) - 1
    avg = np.array([a / c if c else 0.0 for a, c in zip(acc[:n], cnt[:n])])
    if n < 2:
        return g.copy()
    sm = np.empty(n)
    for i in range(n):
        cur = avg[i]
        nxt = avg[i + 1] if i + 1 < n else cur
        prev = avg[i - 1] if i > 0 else cur
        if i == 0:
            sm[i] = (7.0 * cur + nxt) / 8.0
        elif i == n - 1:
            sm[i] = (prev + 7.0 * cur) / 8.0
        else:
            sm[i] = (prev + 6.0 * cur + nxt) / 8.0
    total = 0.0
    for v in sm:
        total += v
    if not total > 0.0 or not math.isfinite(total):
        return g.copy()
    d = np.zeros(n)
    s = 0.0
    for i in range(n):
        r = sm[i] / total
        if r > 0.0:
            d[i] = ((1.0 - r) / math.log(1.0 / r)) ** alpha if r < 1.0 - 1e-12 else 1.0
        s += d[i]
    if not s > 0.0:
        return g.copy()
    share = s / n
    out = g.copy()
    j, below = 0, 0.0
    for k in range(1, n):
        target = k * share
        while j < n - 1 and below + d[j] < target:
            below += d[j]
            j += 1
        f = (target - below) / d[j] if d[j] > 0.0 else 0.0
        f = min(max(f, 0.0), 1.0)
        out[k] = g[j] + f * (g[j + 1] - g[j])
    return out


def map_batch(grids, y):
    """AdaptiveMap's y -> x and jacobian for (n, d) uniforms: increment
    i = floor(y ninc) (at most ninc - 1), x = g[i] + (g[i+1] - g[i])(y ninc - i),
    jac = prod ninc (g[i+1] - g[i])."""
    y = np.atleast_2d(np.asarray(y, np.float64))
    x = np.empty_like(y)
    jac = np.ones(len(y))
    for d, g in enumerate(grids):
        g = np.asarray(g, np.float64)
        n = len(g) - 1
        t = y[:, d] * n
        i = np.minimum(np.floor(t).astype(np.int64), n - 1)
        w = g[i + 1] - g[i]
        x[:, d] = g[i] + w * (t - i)
        jac = jac * (n * w)
    return x, jac


def find_maxes_row(grids, f_by_target, neval, n_trials, uniform):
    """find_maxes on one map row (utilities/find_maxes.py:56-115): for each
    target in turn, n_trials batches of neval points with weight jac/neval
    from `uniform(neval * d)`; max_F = the largest weight * f, xsec = the
    sum of weight * f over the batches divided by n_trials.  f_by_target:
    target -> f(x) for one point.  Returns ({target: max_F}, {target: xsec})."""
    d = len(grids)
    mx, xs = {}, {}
    for t, f in f_by_target.items():
        mx[t], xs[t] = 0.0, 0.0
        for _ in range(n_trials):
            y = np.asarray(uniform(neval * d), np.float64).reshape(neval, d)
            x, jac = map_batch(grids, y)
            mm = (jac / neval) * np.array([f(x[k]) for k in range(neval)])
            if np.max(mm) > mx[t]:
                mx[t] = float(np.max(mm))
            xs[t] += np.sum(mm) / n_trials
    return mx, xs
