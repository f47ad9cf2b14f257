"""The bench's CPU arms on a tiny bounded sample (no GPU): the oracle's
transport loop and the oracle's dark production over spawned processes."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_cpu_dark_baseline_runs_bounded():
    import bench
    w = dict(bench.WORKLOADS["dark_e10_graphite_1e5"])
    w["masses"] = (0.1,)
    cb = bench.cpu_dark_baseline(w, n_proc=2, budget=0.5, per_proc=1)
    assert cb["unit"] == "row-masses/s" and cb["value"] > 0 and cb["cores"] == 2 and cb["kind"] == "port"


def test_dark_cpu_sample_is_bounded_for_400gev_muons():
    import bench
    assert bench.dark_cpu_sample(bench.WORKLOADS["batchdark_mu400_lead_1e3"])["per_proc"] == 1
    assert bench.dark_cpu_sample(bench.WORKLOADS["dark_e10_graphite_1e5"])["per_proc"] > 1


def test_detector_cpu_baseline_runs_bounded():
    import bench
    w = bench.WORKLOADS["detector_cut_1e8"]
    cb = bench.detector_cpu_baseline(w, 20_000, chunk=7_000)
    assert cb["unit"] == "row-detectors/s" and cb["value"] > 0 and cb["cores"] == 1 and cb["kind"] == "port"
