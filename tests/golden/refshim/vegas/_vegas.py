"""AdaptiveMap stand-in; pickles as ``vegas._vegas.AdaptiveMap(grid)``."""
import numpy as np


class AdaptiveMap:
    def __init__(self, grid, ninc=None):
        self.grid = [np.asarray(g, dtype=float) for g in grid]
        self.dim = len(self.grid)

    def __reduce__(self):
        return (AdaptiveMap, ([list(map(float, g)) for g in self.grid],))

    def map_batch(self, y):
        """y: (n, d) uniforms -> x (n, d), jac (n,).

        Increment i = floor(y*ninc) (clamped to ninc-1), fraction
        dy = y*ninc - i, x = g[i] + (g[i+1]-g[i])*dy, jac = prod ninc*(g[i+1]-g[i]).
        """
        y = np.atleast_2d(y)
        x = np.empty_like(y)
        jac = np.ones(y.shape[0])
        for d, g in enumerate(self.grid):
            ninc = len(g) - 1
            t = y[:, d] * ninc
            i = np.minimum(np.floor(t).astype(np.int64), ninc - 1)
            dy = t - i
            inc = g[i + 1] - g[i]
            x[:, d] = g[i] + inc * dy
            jac = jac * (ninc * inc)
        return x, jac

    def map_one(self, y):
        x, jac = self.map_batch(np.asarray(y)[None, :])
        return x[0], float(jac[0])
