"""CPU restatement of PETITE's detector acceptance (oracle).

TEST INFRASTRUCTURE: used only by ``tests/`` and the CPU baseline of
``bench.py``; the product never imports it.

Follows ``src/PETITE/shower.py``:

* transverse_position   shower.py:815-823  (x, y) = r0 + (z - z0)/pz * p
* detector_cut           shower.py:825-865  open energy window, then per disk
                                            detector an open annulus
                                            inner < r_T < radius; methods
                                            "Sample", "SampleW", "Efficiency",
                                            "TotalWeight"

on arrays instead of a list of Particle objects: p0 (n, 4), r0 (n, 3) and
w (n,).  The arithmetic is numpy's, one rounding per operation, as the
reference evaluates it per particle.
"""
import numpy as np


def window(p0, energy_cut):
    """Rows kept by the energy window E_min < E < E_max (shower.py:829-832)."""
    if energy_cut is None:
        return np.ones(len(p0), bool)
    E = p0[:, 0]
    return (E < energy_cut[1]) & (E > energy_cut[0])


def passes(p0, r0, z, radius, inner=0.0):
    """(n_detectors, n) acceptance of every row, window not applied
    (shower.py:815-823 for the crossing point, 846-852 for the annulus)."""
    z = np.asarray(z, dtype=np.float64)
    T = (z[None, :] - r0[:, 2:3]) / p0[:, 3:4]
    x = r0[:, 0:1] + T * p0[:, 1:2]
    y = r0[:, 1:2] + T * p0[:, 2:3]
    rT = np.sqrt(x * x + y * y)
    return ((rT > inner) & (rT < radius)).T


def detector_cut(p0, r0, w, z, radius, method="Sample", energy_cut=None, inner=0.0):
    """The reference's four methods on arrays; "Sample" gives row indices
    (into the rows kept by the window), "SampleW" the mask over those rows."""
    keep = window(p0, energy_cut)
    p0, r0 = p0[keep], r0[keep]
    w = np.ones(len(p0)) if w is None else np.asarray(w, dtype=np.float64)[keep]
    nd = len(z)
    if len(p0) == 0:
        return [[] for _ in range(nd)] if method == "Sample" else [0.0] * nd
    m = passes(p0, r0, z, radius, inner)
    if method == "SampleW":
        return m
    if method == "Sample":
        return [np.nonzero(m[d])[0] for d in range(nd)]
    if method == "Efficiency":
        return [np.sum(w[m[d]]) / np.sum(w) for d in range(nd)]
    if method == "TotalWeight":
        return [np.sum(w[m[d]]) for d in range(nd)]
    return None
