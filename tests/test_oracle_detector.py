"""The CPU restatement of detector_cut (oracle/detector.py) against the
reference's own outputs (tests/golden/particles.npz, from PETITE's
shower.py:825-865 via tests/golden/make_golden.py)."""
import os

import numpy as np

from conftest import GOLDEN
from oracle import detector as od

P = np.load(os.path.join(GOLDEN, "particles.npz"))
ZS, R = [5.0, 50.0, 100.0], 1.0


def test_oracle_matches_reference_outputs():
    p0, r0, w = P["det/p0"], P["det/r0"], P["det/w"]
    np.testing.assert_array_equal(od.detector_cut(p0, r0, w, ZS, R, method="SampleW"), P["det/sampleW"])
    np.testing.assert_allclose(od.detector_cut(p0, r0, w, ZS, R, method="Efficiency", energy_cut=(1.0, 20.0),
                                               inner=0.05), P["det/eff"], rtol=1e-15)
    np.testing.assert_allclose(od.detector_cut(p0, r0, w, ZS, R, method="TotalWeight"), P["det/total"], rtol=1e-15)
    s = od.detector_cut(p0, r0, w, ZS, R, method="Sample")
    assert [len(x) for x in s] == list(P["det/sampleW"].sum(axis=1))


def test_oracle_empty_window():
    p0, r0, w = P["det/p0"], P["det/r0"], P["det/w"]
    assert od.detector_cut(p0, r0, w, ZS, R, method="Efficiency", energy_cut=(1e6, 2e6)) == [0.0] * 3
    assert od.detector_cut(p0, r0, w, ZS, R, method="Sample", energy_cut=(1e6, 2e6)) == [[], [], []]
