"""Detector acceptance on the GPU (pt_detector_cut, detector_cut_rows)
against the reference's own detector_cut outputs (tests/golden/particles.npz,
made by tests/golden/make_golden.py from PETITE's shower.py:825-865) and
against the host form on rows with edge cases."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from petite_gb300.particle import Particle
from petite_gb300.shower import detector_cut, detector_cut_rows

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

P = np.load(os.path.join(GOLDEN, "particles.npz"))
ZS, R = [5.0, 50.0, 100.0], 1.0


def test_matches_reference_outputs():
    p0, r0, w = P["det/p0"], P["det/r0"], P["det/w"]
    mask = detector_cut_rows(p0, r0, w, ZS, R, method="SampleW")
    np.testing.assert_array_equal(mask.cpu().numpy(), P["det/sampleW"])          # bit-exact acceptance
    eff = detector_cut_rows(p0, r0, w, ZS, R, method="Efficiency", energy_cut=(1.0, 20.0), detector_inner_radius=0.05)
    np.testing.assert_allclose(eff, P["det/eff"], rtol=1e-12)
    np.testing.assert_allclose(detector_cut_rows(p0, r0, w, ZS, R, method="TotalWeight"), P["det/total"], rtol=1e-12)
    s = detector_cut_rows(p0, r0, w, ZS, R, method="Sample")
    for d in range(len(ZS)):
        np.testing.assert_array_equal(s[d].cpu().numpy(), np.nonzero(P["det/sampleW"][d])[0])


def edge_rows(n, seed):
    rng = np.random.default_rng(seed)
    E = 10 ** rng.uniform(-1, 2, n)
    th = 10 ** rng.uniform(-4, 0.3, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    p0 = np.c_[E, E * np.sin(th) * np.cos(ph), E * np.sin(th) * np.sin(ph), E * np.cos(th)]
    r0 = np.c_[rng.normal(0, 0.3, n), rng.normal(0, 0.3, n), rng.uniform(-1, 2, n)]
    p0[:8, 3] = 0.0                       # parallel to the detectors: never crosses
    p0[8:12, 1:3] = 0.0                   # on the axis
    r0[8:12, :2] = 0.0
    p0[12:16, 3] *= -1.0                  # backwards
    r0[16:20, 2] = 5.0                    # starts on a detector plane
    w = rng.uniform(0.1, 2.0, n)
    return p0, r0, w


@pytest.mark.parametrize("n_det", [1, 3, 11])
def test_matches_host_form_with_edge_cases(n_det):
    p0, r0, w = edge_rows(5000, n_det)
    zs = list(np.linspace(0.5, 80.0, n_det))
    parts = [Particle(list(a), list(b), {"PID": 4900022, "weight": float(c), "mass": 0.01}) for a, b, c in zip(p0, r0, w)]
    for cut, inner in ((None, 0.0), ((1.0, 20.0), 0.05)):
        host = np.asarray(detector_cut(parts, zs, 2.0, method="SampleW", energy_cut=cut, detector_inner_radius=inner))
        dev = detector_cut_rows(p0, r0, w, zs, 2.0, method="SampleW", energy_cut=cut,
                                detector_inner_radius=inner).cpu().numpy()
        keep = np.ones(len(p0), bool) if cut is None else (p0[:, 0] < cut[1]) & (p0[:, 0] > cut[0])
        np.testing.assert_array_equal(dev[:, keep], host)
        assert not dev[:, ~keep].any()
        for method in ("Efficiency", "TotalWeight"):
            np.testing.assert_allclose(
                detector_cut_rows(p0, r0, w, zs, 2.0, method=method, energy_cut=cut, detector_inner_radius=inner),
                detector_cut(parts, zs, 2.0, method=method, energy_cut=cut, detector_inner_radius=inner), rtol=1e-12)


def test_reads_soa_store_in_place_and_handles_empty_windows():
    p0, r0, w = edge_rows(3000, 7)
    cap = 4096
    P4 = torch.zeros((4, cap), dtype=torch.float64, device="cuda")
    R3 = torch.zeros((3, cap), dtype=torch.float64, device="cuda")
    P4[:, :3000] = torch.as_tensor(p0.T, device="cuda")
    R3[:, :3000] = torch.as_tensor(r0.T, device="cuda")
    a = detector_cut_rows(P4[:, :3000].T, R3[:, :3000].T, w, ZS, R, method="SampleW")
    b = detector_cut_rows(p0, r0, w, ZS, R, method="SampleW")
    assert torch.equal(a, b)
    # no row in the window: efficiencies are 0 as in the list form
    assert detector_cut_rows(p0, r0, w, ZS, R, method="Efficiency", energy_cut=(1e6, 2e6)) == [0.0] * 3
    assert detector_cut_rows(np.zeros((0, 4)), np.zeros((0, 3)), None, ZS, R, method="TotalWeight") == [0.0] * 3
    assert [len(x) for x in detector_cut_rows(np.zeros((0, 4)), np.zeros((0, 3)), None, ZS, R)] == [0, 0, 0]


def test_rows_on_the_annulus_edges_take_the_exact_decision():
    """Rows whose crossing radius lies within 1e-3 .. 1e-16 of either edge:
    the float32 screen must hand the close ones to the float64 path."""
    R, inner, z = 1.0, 0.05, 50.0
    eps = np.array([0.0, 1e-16, 1e-15, 1e-13, 1e-11, 1e-9, 1e-7, 1e-6, 1e-5, 1e-4, 1e-3])
    eps = np.r_[eps, -eps[1:]]
    rows = []
    for edge in (R, inner):
        for e in eps:
            for phi in (0.0, 0.7, 2.1):
                rho = edge * (1 + e)
                rows.append(([10.0, rho / z * np.cos(phi), rho / z * np.sin(phi), 1.0], [0.0, 0.0, 0.0]))
                # the same radius reached from an offset start (cancellation in x0 + T px)
                rows.append(([10.0, (rho * np.cos(phi) + 3.0) / z, rho * np.sin(phi) / z, 1.0], [-3.0, 0.0, 0.0]))
    p0 = np.array([a for a, _ in rows])
    r0 = np.array([b for _, b in rows])
    parts = [Particle(list(a), list(b), {"PID": 4900022, "weight": 1.0, "mass": 0.01}) for a, b in zip(p0, r0)]
    host = np.asarray(detector_cut(parts, [z], R, method="SampleW", detector_inner_radius=inner))
    dev = detector_cut_rows(p0, r0, None, [z], R, method="SampleW", detector_inner_radius=inner).cpu().numpy()
    np.testing.assert_array_equal(dev, host)
    assert 0 < host.sum() < host.size


def test_million_rows_match_the_oracle():
    """10^6 rows drawn like the detector benchmark: the device mask equals
    the oracle's bit for bit, and the sums agree to 1e-12."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from oracle import detector as od
    w = bench.WORKLOADS["detector_cut_1e8"]
    p0, r0, wt = bench.detector_rows(w, 1_000_000, 123)
    zs = list(w["z"])
    m_dev = detector_cut_rows(p0, r0, wt, zs, w["radius"], method="SampleW", energy_cut=w["energy_cut"],
                              detector_inner_radius=w["inner"]).cpu().numpy()
    keep = od.window(p0, w["energy_cut"])
    m_ref = od.passes(p0, r0, zs, w["radius"], w["inner"]) & keep[None, :]
    np.testing.assert_array_equal(m_dev, m_ref)
    np.testing.assert_allclose(
        detector_cut_rows(p0, r0, wt, zs, w["radius"], method="Efficiency", energy_cut=w["energy_cut"],
                          detector_inner_radius=w["inner"]),
        od.detector_cut(p0, r0, wt, zs, w["radius"], method="Efficiency", energy_cut=w["energy_cut"],
                        inner=w["inner"]), rtol=1e-12)
