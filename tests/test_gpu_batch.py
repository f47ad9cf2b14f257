"""Batched (tally) engine: float64 form vs the record engine, ring-capacity
independence, and the mixed-precision form vs float64."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 1


def primaries(n, seed=7, emin=0.1, emax=10.0, species=(11, -11, 22)):
    rng = np.random.default_rng(seed)
    pid = np.asarray(species)[rng.integers(0, len(species), n)]
    E = 10 ** rng.uniform(math.log10(emin), math.log10(emax), n)
    m = np.where(np.abs(pid) == 11, 0.000511, np.where(np.abs(pid) == 13, 0.1056583755, 0.0))
    p0 = np.c_[E, np.zeros(n), np.zeros(n), np.sqrt(E * E - m * m)]
    return p0, pid.astype(np.int32), m


@pytest.fixture(scope="module")
def lead():
    from petite_gb300 import Shower
    return Shower(None, "lead", 0.010, seed=SEED)


def run_batch(sh, p0, pid, m, precision, cap=0, offset=0):
    eng = sh._engine
    opts = sh._opts(True, precision)
    opts.primary_offset = offset
    t = eng.new_tally(len(p0), z_max=0.3)
    eng.run_batch(p0, np.zeros((len(p0), 3)), pid, m, opts, t, queue_capacity=cap)
    return t


def test_fp64_batch_equals_record_engine(lead):
    p0, pid, m = primaries(300)
    b = lead.generate_showers(p0, pid=pid, mass=m, first_primary=0)
    rows_per_primary = np.bincount(b.primary, minlength=len(p0))
    t = run_batch(lead, p0, pid, m, "fp64")
    s = t.summary()
    assert np.array_equal(t.primary_count.cpu().numpy(), rows_per_primary)
    assert s["steps"] == b.n
    sp = [int((b.pid == q).sum()) for q in (22, 11, -11)]
    assert [s["photon_steps"], s["electron_steps"], s["positron_steps"]] == sp
    # continuous dE/dx loss summed over the records
    np.testing.assert_allclose(s["E_continuous"], float(np.sum(b.p0[:, 0] - b.pf[:, 0])), rtol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_capacity_does_not_change_results(lead, precision):
    p0, pid, m = primaries(400, seed=3)
    big = run_batch(lead, p0, pid, m, precision, cap=1 << 22)
    small = run_batch(lead, p0, pid, m, precision, cap=1 << 12)
    assert np.array_equal(big.primary_count.cpu().numpy(), small.primary_count.cpu().numpy())
    assert np.array_equal(big.hist.cpu().numpy(), small.hist.cpu().numpy())
    np.testing.assert_allclose(big.primary_edep.cpu().numpy(), small.primary_edep.cpu().numpy(), rtol=1e-9)


def mixed_vs_fp64_errors(f, x, z_max):
    """Per-observable error of the mixed form against the float64 form on the
    same random streams (the float64 form equals the record engine, which
    equals the oracle draw for draw)."""
    sf, sx = f.summary(), x.summary()
    cf, cx = f.primary_count.cpu().numpy(), x.primary_count.cpu().numpy()
    ef, ex = f.primary_edep.cpu().numpy(), x.primary_edep.cpu().numpy()
    hf, hx = f.hist.cpu().numpy().astype(np.int64), x.hist.cpu().numpy().astype(np.int64)
    out = {"identical showers": float(np.mean(cf == cx)),
           "multiplicity (total)": abs(sx["steps"] - sf["steps"]) / sf["steps"],
           "E_dep (total)": abs(sx["E_deposited"] - sf["E_deposited"]) / sf["E_deposited"],
           "E_dep (largest per shower)": float(np.max(np.abs(ex - ef) / ef))}
    lo_hi = ((-2.0, 2.0), (-6.0, 0.5), (0.0, z_max))
    for k, name in enumerate(("creation energy", "polar angle", "depth")):
        a, b = hf[k].sum(axis=0), hx[k].sum(axis=0)
        centres = lo_hi[k][0] + (np.arange(a.size) + 0.5) * (lo_hi[k][1] - lo_hi[k][0]) / a.size
        out[f"{name} (entries in another bin)"] = float(np.abs(hf[k] - hx[k]).sum() / (2 * hf[k].sum()))
        out[f"{name} (binned mean)"] = float(abs((centres * b).sum() / b.sum() - (centres * a).sum() / a.sum())
                                             / abs((centres * a).sum() / a.sum()))
    return out


def test_mixed_matches_fp64(lead):
    """Same random streams: the float32 sampler changes a decision only when a
    uniform falls within float32 rounding of the acceptance boundary, and the
    shower below that decision is then drawn again.  The benchmark spec's bound is
    total deposited energy within 1e-5 of float64."""
    p0, pid, m = primaries(3000, seed=11, emax=100.0)
    f = run_batch(lead, p0, pid, m, "fp64")
    x = run_batch(lead, p0, pid, m, "mixed")
    err = mixed_vs_fp64_errors(f, x, 0.3)
    print()
    for k, v in err.items():
        print(f"  {k:40s} {v:.3e}")
    assert err["identical showers"] > 0.98
    assert err["E_dep (total)"] < 1e-5
    assert err["multiplicity (total)"] < 1e-4
    for name in ("creation energy", "polar angle", "depth"):
        assert err[f"{name} (entries in another bin)"] < 2e-2, name
        assert err[f"{name} (binned mean)"] < 1e-3, name


def test_batch_no_sample_reports():
    from petite_gb300 import Shower
    sh = Shower(None, "graphite", 0.010, seed=1, max_n_integrators=1, maxF_fudge_global=1e300)
    p0, pid, m = primaries(4, species=(22,))
    with pytest.raises(Exception, match="No Sample Found"):
        run_batch(sh, p0, pid, m, "mixed")


def test_work_distribution_does_not_change_results(lead):
    """pt_set_batch_tuning changes only how warps share the work."""
    p0, pid, m = primaries(400, seed=5)
    eng = lead._engine
    a = run_batch(lead, p0, pid, m, "mixed")
    eng.set_tuning((1, 16), (32, 256))
    b = run_batch(lead, p0, pid, m, "mixed")
    eng.set_tuning((0, 0), (0, 0))
    assert np.array_equal(a.primary_count.cpu().numpy(), b.primary_count.cpu().numpy())
    assert np.array_equal(a.hist.cpu().numpy(), b.hist.cpu().numpy())
    with pytest.raises(Exception):
        eng.set_tuning((0, 0), (16, 0))          # a pool chunk below one warp


def test_autotune_picks_valid_settings(lead):
    from petite_gb300.autotune import GRID, autotune_batch
    best = autotune_batch(lead, n=2000, ring_capacity=1 << 18, use_cache=False)
    assert best["refill_min"][0] in (8,) + GRID["refill_min"]
    assert best["chunk"][0] in (128,) + GRID["chunk_propagate"]
    assert best["chunk"][1] in (64,) + GRID["chunk_sample"]
    assert best["loop"] in GRID["loop"]
    assert best["staging"] in GRID["staging"]
    assert best["threads"] in GRID["threads"]
    assert set(best["staging_seconds"]) == set(GRID["staging"])
    assert best["lanes"] in GRID["lanes"]
    assert best["lanes"] == 1 or best["loop"] == "host"
    assert best["seconds"] > 0
    lead._engine.set_tuning((0, 0), (0, 0))


def test_autotune_on_the_workloads_primaries(lead):
    """Calibration on muons of the workload: lanes are timed with the host loop."""
    from petite_gb300.autotune import GRID, autotune_batch
    n = 40
    p0 = np.tile([50.0, 0.0, 0.0, math.sqrt(2500.0 - 0.1056583755 ** 2)], (n, 1))
    best = autotune_batch(lead, n=0, ring_capacity=1 << 18, choose_loop=False,
                          primaries=(p0, np.full(n, 13, np.int32), np.full(n, 0.1056583755)))
    assert best["loop"] == "host" and best["lanes"] in GRID["lanes"]
    assert set(best["lanes_seconds"]) == set(GRID["lanes"])
    lead._engine.set_tuning((0, 0), (0, 0))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("loop", ["graph", "persistent"])
def test_device_planned_loops_give_identical_results(lead, precision, loop):
    """The waves planned on the GPU (a CUDA graph's conditional loop, or one
    persistent cooperative kernel) are the host loop's waves: the same
    particles, spectra and deposits; only the summation order of the float64
    deposits differs."""
    p0, pid, m = primaries(1500, seed=31, emax=50.0)
    eng = lead._engine
    a = run_batch(lead, p0, pid, m, precision, cap=1 << 16)
    eng.set_tuning((0, 0), (0, 0), loop)
    try:
        b = run_batch(lead, p0, pid, m, precision, cap=1 << 16)
    finally:
        eng.set_tuning((0, 0), (0, 0))
    assert np.array_equal(a.primary_count.cpu().numpy(), b.primary_count.cpu().numpy())
    assert np.array_equal(a.counts.cpu().numpy(), b.counts.cpu().numpy())
    ha, hb = a.hist.cpu().numpy().astype(np.int64), b.hist.cpu().numpy().astype(np.int64)
    if precision == "fp64":
        assert np.array_equal(ha, hb)
    else:
        # the persistent kernel inlines the float32 bodies into another kernel,
        # where the compiler may contract a product into a fused multiply-add
        # differently: a last-place difference can move a binned value across
        # a bin edge, never a particle or a decision
        for k in range(3):
            assert ha[k].sum() == hb[k].sum()
            assert np.abs(ha[k] - hb[k]).sum() <= 1e-5 * ha[k].sum(), k
    np.testing.assert_allclose(a.primary_edep.cpu().numpy(), b.primary_edep.cpu().numpy(), rtol=1e-9)
    np.testing.assert_allclose(a.energy.cpu().numpy(), b.energy.cpu().numpy(), rtol=1e-9)


@pytest.mark.parametrize("bethe", [False, True])
@pytest.mark.parametrize("loop", ["host", "graph"])
def test_shared_memory_staging_gives_identical_results(loop, bethe):
    """The propagation kernel that reads the n*sigma tables from shared
    memory (staged by TMA bulk copies) makes the same decisions as the one
    that reads them through the read-only cache."""
    from petite_gb300 import Shower
    sh = Shower(None, "lead", 0.010, seed=SEED, fast_MCS_mode=not bethe)
    p0, pid, m = primaries(800, seed=37, emax=50.0)
    eng = sh._engine
    eng.set_tuning((0, 0), (0, 0), "host", "cached")
    a = run_batch(sh, p0, pid, m, "mixed", cap=1 << 16)
    eng.set_tuning((0, 0), (0, 0), loop, "shared")
    try:
        b = run_batch(sh, p0, pid, m, "mixed", cap=1 << 16)
    finally:
        eng.set_tuning((0, 0), (0, 0))
    assert np.array_equal(a.primary_count.cpu().numpy(), b.primary_count.cpu().numpy())
    assert np.array_equal(a.counts.cpu().numpy(), b.counts.cpu().numpy())
    ha, hb = a.hist.cpu().numpy().astype(np.int64), b.hist.cpu().numpy().astype(np.int64)
    # another kernel instantiation: a contraction into a fused multiply-add
    # may differ and move a binned value across a bin edge, never a decision
    assert (np.abs(ha - hb).sum(axis=(1, 2)) <= 1e-5 * ha.sum(axis=(1, 2))).all()
    np.testing.assert_allclose(a.primary_edep.cpu().numpy(), b.primary_edep.cpu().numpy(), rtol=1e-9)
    with pytest.raises(Exception):
        eng.set_tuning((0, 0), (0, 0), "host", "tma")


@pytest.mark.parametrize("threads,loop", [(64, "host"), (256, "host"), (256, "graph")])
def test_block_size_gives_identical_results(lead, threads, loop):
    """The float32 kernels at 64 or 256 threads per block: the same
    particles, spectra and deposits as at 128."""
    p0, pid, m = primaries(800, seed=41, emax=50.0)
    eng = lead._engine
    a = run_batch(lead, p0, pid, m, "mixed", cap=1 << 16)
    eng.set_tuning((0, 0), (0, 0), loop, "default", threads)
    try:
        b = run_batch(lead, p0, pid, m, "mixed", cap=1 << 16)
    finally:
        eng.set_tuning((0, 0), (0, 0))
    assert np.array_equal(a.primary_count.cpu().numpy(), b.primary_count.cpu().numpy())
    assert np.array_equal(a.counts.cpu().numpy(), b.counts.cpu().numpy())
    ha, hb = a.hist.cpu().numpy().astype(np.int64), b.hist.cpu().numpy().astype(np.int64)
    assert (np.abs(ha - hb).sum(axis=(1, 2)) <= 1e-5 * ha.sum(axis=(1, 2))).all()
    np.testing.assert_allclose(a.primary_edep.cpu().numpy(), b.primary_edep.cpu().numpy(), rtol=1e-9)
    with pytest.raises(Exception):
        eng.set_tuning((0, 0), (0, 0), "host", "default", 96)


def test_device_planned_loop_in_bethe_mode():
    from petite_gb300 import Shower
    sh = Shower(None, "lead", 0.010, seed=SEED, fast_MCS_mode=False)
    p0, pid, m = primaries(500, seed=33)
    a = run_batch(sh, p0, pid, m, "mixed", cap=1 << 15)
    sh._engine.set_tuning((0, 0), (0, 0), "persistent")
    b = run_batch(sh, p0, pid, m, "mixed", cap=1 << 15)
    sh._engine.set_tuning((0, 0), (0, 0))
    assert np.array_equal(a.primary_count.cpu().numpy(), b.primary_count.cpu().numpy())
    ha, hb = a.hist.cpu().numpy().astype(np.int64), b.hist.cpu().numpy().astype(np.int64)
    assert (np.abs(ha - hb).sum(axis=(1, 2)) <= 1e-5 * ha.sum(axis=(1, 2))).all()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("lanes", [2, 3, 8])
def test_lanes_give_identical_results(lead, precision, lanes):
    """pt_batch_tuning.lanes: the primaries split over lanes with their own
    rings and streams whose waves interleave.  Every primary keeps its
    stream, so the particles, spectra and deposits are one lane's; only the
    summation order of the float64 deposits differs (and, through the
    float32 loss sums' order, nothing else: the histograms are equal)."""
    p0, pid, m = primaries(1500, seed=41, emax=50.0)
    eng = lead._engine
    a = run_batch(lead, p0, pid, m, precision, cap=1 << 16, offset=9)
    eng.set_tuning((0, 0), (0, 0), "host", lanes=lanes)
    try:
        b = run_batch(lead, p0, pid, m, precision, cap=1 << 16, offset=9)
        launches, waves = eng.last_run_stats()
    finally:
        eng.set_tuning((0, 0), (0, 0))
    assert waves > 0
    assert np.array_equal(a.primary_count.cpu().numpy(), b.primary_count.cpu().numpy())
    assert np.array_equal(a.counts.cpu().numpy(), b.counts.cpu().numpy())
    assert np.array_equal(a.hist.cpu().numpy(), b.hist.cpu().numpy())
    np.testing.assert_allclose(a.primary_edep.cpu().numpy(), b.primary_edep.cpu().numpy(), rtol=1e-12)
    np.testing.assert_allclose(a.energy.cpu().numpy(), b.energy.cpu().numpy(), rtol=1e-12)


def test_lanes_need_the_host_loop(lead):
    from petite_gb300 import _lib
    eng = lead._engine
    for loop in ("graph", "persistent"):
        with pytest.raises(_lib.PetiteGPUError):
            eng.set_tuning((0, 0), (0, 0), loop, lanes=2)
    with pytest.raises(_lib.PetiteGPUError):
        eng.set_tuning((0, 0), (0, 0), "host", lanes=9)
    eng.set_tuning((0, 0), (0, 0))
