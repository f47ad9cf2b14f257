"""The CPU side of the independent-stream spectrum comparison
(tests/golden/spectra.npz) and the statistics it is compared with."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
import spectra


@pytest.fixture(scope="module")
def cpu():
    return np.load(os.path.join(GOLDEN, "spectra.npz"))


def test_fixture_matches_its_workloads(cpu):
    for name, cfg in spectra.CONFIGS.items():
        p0, pid, _ = spectra.primaries(cfg)
        assert np.array_equal(cpu[f"{name}/pid"], pid)
        np.testing.assert_array_equal(cpu[f"{name}/E0"], p0[:, 0])
        mult, edep, h = cpu[f"{name}/mult"], cpu[f"{name}/edep"], cpu[f"{name}/hist"].astype(np.int64)
        assert len(mult) == cfg["n"] and (mult >= 1).all()
        # every particle is binned once in each of the three histograms
        for k in range(3):
            assert np.array_equal(h[:, k].sum(axis=(1, 2)), mult)
        # the deposit is the primary's energy plus the rest energy of the
        # target electrons set in motion: never less than E0
        assert (edep >= p0[:, 0] * (1 - 1e-12)).all()


def _neighbour_split(cpu, name):
    """The CPU showers sorted by species and energy, split into even and odd
    positions: two samples whose primaries pair up nearly exactly."""
    h = cpu[f"{name}/hist"].astype(np.int64)
    pid, E0 = cpu[f"{name}/pid"], cpu[f"{name}/E0"]
    o = np.lexsort((E0, pid))
    n = len(o) // 2
    return h, pid, E0, o[0:2 * n:2], o[1:2 * n:2]


def test_hotelling_statistics_are_calibrated_and_have_power(cpu):
    """Two halves of the same CPU sample agree, and a 5 % excess of
    particles, or a histogram shifted by one bin, is rejected."""
    for name in spectra.CONFIGS:
        h, pid, E0, a, b = _neighbour_split(cpu, name)
        for k in range(3):
            A = h[a, k].reshape(len(a), -1)
            B = h[b, k].reshape(len(b), -1)
            _, dof, p = spectra.hotelling_paired(A.mean(axis=0), 1, B, pid[b], E0[b])
            assert dof > 0 and p > 0.01, (name, k, p)
            _, _, p_scaled = spectra.hotelling_paired(1.05 * A.mean(axis=0), 1, B, pid[b], E0[b])
            assert p_scaled < 1e-3, (name, k, p_scaled)
            _, _, p_shift = spectra.hotelling_paired(np.roll(A.mean(axis=0), 1), 1, B, pid[b], E0[b])
            assert p_shift < 1e-6, (name, k, p_shift)
    # the unpaired form on equal-energy primaries
    h = cpu["e1_graphite/hist"].astype(np.int64)
    n = len(h) // 2
    for k in range(3):
        _, dof, p = spectra.hotelling(h[:n, k].reshape(n, -1).mean(axis=0), n, h[n:2 * n, k].reshape(n, -1))
        assert dof > 0 and p > 0.01, (k, p)


def test_ks_rejects_a_scaled_sample(cpu):
    m = cpu["e1_graphite/mult"]
    assert spectra.ks(m[:500], m[500:])[1] > 0.01
    assert spectra.ks(m[:500], np.round(m[500:] * 1.05))[1] < 1e-3
