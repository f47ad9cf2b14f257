"""Minimal VEGAS map-sampling shim (see README.txt).

Only the surface PETITE's shower and find_maxes paths touch is provided:
``lbatchintegrand`` (identity decorator), ``AdaptiveMap(grid)`` and
``Integrator(map=..., neval=..., max_nhcube=..., nstrat=...)`` with
``set()``, ``random()`` and ``random_batch()``.  A single hypercube is used
(``max_nhcube=1``), so every point has weight ``jac / neval``.

``UNIFORM`` is the hook every draw goes through: ``UNIFORM(n)`` must return n
uniforms in [0, 1).  The golden-vector harness replaces it with the
per-particle Philox stream; by default it is numpy's global generator.
``random()`` draws each point's d uniforms lazily, just before yielding it, so
a proposal consumes d uniforms followed by the accept/reject uniform the
caller draws.
"""
import numpy as np

from ._vegas import AdaptiveMap

__all__ = ["AdaptiveMap", "Integrator", "lbatchintegrand", "UNIFORM"]


def _default_uniform(n):
    return np.random.random(n)


UNIFORM = _default_uniform


def lbatchintegrand(f):
    return f


class Integrator:
    def __init__(self, map=None, **kw):
        if map is None:
            raise NotImplementedError("shim supports Integrator(map=AdaptiveMap) only")
        if not isinstance(map, AdaptiveMap):
            map = AdaptiveMap(map)
        self.map = map
        self.neval = 1000
        self.set(**kw)

    def set(self, **kw):
        if "neval" in kw:
            self.neval = int(kw["neval"])
        return {}

    def random(self):
        """Yields (x, wgt) for one iteration of ``neval`` points."""
        d = self.map.dim
        for _ in range(self.neval):
            y = np.asarray(UNIFORM(d), dtype=float)
            x, jac = self.map.map_one(y)
            yield x, jac / self.neval

    def random_batch(self):
        d = self.map.dim
        y = np.asarray(UNIFORM(self.neval * d), dtype=float).reshape(self.neval, d)
        x, jac = self.map.map_batch(y)
        yield x, jac / self.neval
