"""The float32 form of the dark-vector production (pt_dark_params.precision
= 1: float32 uniforms, map transform and dark-brem screen, float64 cross
section wherever the float32 estimate cannot decide, float64 kinematics)
against the float64 form, on the same SM rows and random streams.

The yields are sums of GetBSMWeights over the vectors made, so they differ
only where a draw ends without a sample; the vectors' energies differ where
a float32 decision or sample differs from the float64 one.  The bound of the
spec target is 1e-5 relative on each process's yield.
"""
import math
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 0x5EED
MASSES = (0.01, 0.1, 0.3)
PROCESSES = ("DarkBrem", "DarkAnn", "DarkComp")


@pytest.fixture(scope="module")
def rows():
    """SM showers of 10 GeV electrons in graphite from the record engine."""
    from petite_gb300.dark import DarkShower
    sh = DarkShower(None, "graphite", 0.010, 0.1, seed=SEED, active_processes=list(PROCESSES))
    n = 400
    p = math.sqrt(100.0 - 0.000511 ** 2)
    opts = sh._opts(True, "fp64")
    opts.primary_offset = 0
    st, nr = sh._engine.run_sm(np.tile([10.0, 0, 0, p], (n, 1)), np.zeros((n, 3)), np.full(n, 11, np.int32),
                               np.full(n, 0.000511), np.ones(n), opts)
    return st, nr


@pytest.mark.parametrize("mV", MASSES)
def test_float32_dark_production_matches_float64(rows, mV):
    import torch
    from petite_gb300.dark import DarkShower
    st, nr = rows
    out, dt = {}, {}
    for prec in ("fp64", "mixed"):
        sh = DarkShower(None, "graphite", 0.010, mV, seed=SEED, active_processes=list(PROCESSES),
                        dark_precision=prec)
        sh._dark_engine.run_dark(sh._prm, st, nr, sh._opts())          # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out[prec] = sh._dark_engine.run_dark(sh._prm, st, nr, sh._opts())
        torch.cuda.synchronize()
        dt[prec] = time.perf_counter() - t0
    a, b = out["fp64"], out["mixed"]
    print(f"\nmV={mV}: {nr} rows, vectors {a['n']} (float64) {b['n']} (float32); "
          f"time {dt['fp64']:.4f} s / {dt['mixed']:.4f} s = {dt['fp64'] / dt['mixed']:.2f}x")
    for k, name in enumerate(PROCESSES):
        ya, yb = a["yield"][k], b["yield"][k]
        ea, eb = a["yield_E"][k], b["yield_E"][k]
        if ya == 0:
            assert yb == 0
            continue
        print(f"  {name:8s} yield {ya:.6e} rel {abs(yb - ya) / ya:.2e}   <E_V> rel {abs(eb / yb - ea / ya) / (ea / ya):.2e}")
        assert abs(yb - ya) <= 1e-5 * ya, name
        assert abs(eb / yb - ea / ya) <= 2e-3 * (ea / ya), name
    assert abs(b["n"] - a["n"]) <= 1e-4 * a["n"] + 2
    # vectors of the same (row, process) carry the same weight
    ka = np.lexsort((a["process"], a["parent"]))
    kb = np.lexsort((b["process"], b["parent"]))
    if a["n"] == b["n"]:
        assert np.array_equal(a["parent"][ka], b["parent"][kb])
        np.testing.assert_array_equal(a["weight"][ka], b["weight"][kb])
        # the energies: most vectors come from identical decisions
        same = np.isclose(a["p4"][ka, 0], b["p4"][kb, 0], rtol=1e-5)
        print(f"  vectors with the float64 energy (1e-5): {same.mean():.4f}")
        assert same.mean() > 0.95
    from scipy import stats
    assert stats.ks_2samp(a["p4"][:, 0], b["p4"][:, 0]).pvalue > 0.01
