"""Bounded device loops and waits: a bound that runs out returns PT_TIMEOUT
and the next call on the same handle gives the normal result; a particle
store that the showers outgrow (PT_OOM) is retried with twice the rows and
gives the same rows.

The bounds are the test settings of the ABI: ``pt_opts.loop_limit`` (the
record engine's substep iterations per particle, the batched engine's waves
per run) and ``pt_batch_tuning.barrier_ns`` (the persistent kernel's wait at
its grid barrier).  Nothing here makes a device copy or a kernel fail: a
bound that runs out only ends the loop it bounds.
"""
import ctypes as C

import numpy as np
import pytest

from petite_gb300 import _lib
from test_gpu_batch import primaries

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lead():
    from petite_gb300 import Shower
    return Shower(None, "lead", 0.010, seed=5)


def batch(sh, p0, pid, m, loop_limit=0, cap=1 << 16, precision="mixed"):
    eng = sh._engine
    o = sh._opts(True, precision)
    o.primary_offset = 0
    o.loop_limit = loop_limit
    t = eng.new_tally(len(p0), z_max=0.3)
    eng.run_batch(p0, np.zeros((len(p0), 3)), pid, m, o, t, queue_capacity=cap)
    return t


def same_rows(st_a, n_a, st_b, n_b, n_primaries):
    """Two particle stores hold the same showers (rows compared in the
    reference's list order; the kernels append rows in any order)."""
    from petite_gb300.shower import ShowerBatch
    assert n_a == n_b
    a, b = ShowerBatch(st_a.to_numpy(n_a), n_primaries), ShowerBatch(st_b.to_numpy(n_b), n_primaries)
    oa, ob = a.order, b.order
    assert np.array_equal(a.pid[oa], b.pid[ob]) and np.array_equal(a.proc[oa], b.proc[ob])
    np.testing.assert_array_equal(a.pf[oa], b.pf[ob])


def same(a, b):
    assert np.array_equal(a.counts.cpu().numpy(), b.counts.cpu().numpy())
    assert np.array_equal(a.primary_count.cpu().numpy(), b.primary_count.cpu().numpy())
    ha, hb = a.hist.cpu().numpy().astype(np.int64), b.hist.cpu().numpy().astype(np.int64)
    assert (np.abs(ha - hb).sum(axis=(1, 2)) <= 1e-5 * ha.sum(axis=(1, 2))).all()
    np.testing.assert_allclose(a.primary_edep.cpu().numpy(), b.primary_edep.cpu().numpy(), rtol=1e-9)


@pytest.mark.parametrize("loop", ["host", "graph", "persistent"])
def test_wave_bound_returns_timeout_and_the_handle_recovers(lead, loop):
    p0, pid, m = primaries(300, seed=21, emax=20.0)
    ref = batch(lead, p0, pid, m)
    lead._engine.set_tuning((0, 0), (0, 0), loop)
    try:
        with pytest.raises(_lib.PetiteGPUError) as e:
            batch(lead, p0, pid, m, loop_limit=2)
        assert e.value.status == _lib.PT_TIMEOUT
        assert lead._engine.unusable is None          # a loop bound, not a copy in flight
        again = batch(lead, p0, pid, m)
    finally:
        lead._engine.set_tuning((0, 0), (0, 0))
    same(ref, again)


def test_grid_barrier_bound_returns_timeout(lead):
    p0, pid, m = primaries(300, seed=22, emax=20.0)
    ref = batch(lead, p0, pid, m)
    # 1 ns: every block but the last to arrive gives up at the first barrier
    lead._engine.set_tuning((0, 0), (0, 0), "persistent", barrier_ns=1)
    try:
        with pytest.raises(_lib.PetiteGPUError) as e:
            batch(lead, p0, pid, m)
        assert e.value.status == _lib.PT_TIMEOUT
    finally:
        lead._engine.set_tuning((0, 0), (0, 0))
    lead._engine.set_tuning((0, 0), (0, 0), "persistent")
    try:
        again = batch(lead, p0, pid, m)
    finally:
        lead._engine.set_tuning((0, 0), (0, 0))
    same(ref, again)


def test_substep_bound_of_the_record_engine(lead):
    p0, pid, m = primaries(20, seed=23, species=(11,), emin=1.0, emax=1.0)
    eng = lead._engine
    o = lead._opts(True, "fp64")
    ref, n_ref = eng.run_sm(p0, np.zeros((20, 3)), pid, m, np.ones(20), o)
    o.loop_limit = 1                                   # every charged track needs more than one substep
    with pytest.raises(_lib.PetiteGPUError) as e:
        eng.run_sm(p0, np.zeros((20, 3)), pid, m, np.ones(20), o)
    assert e.value.status == _lib.PT_TIMEOUT
    proc, E, key = C.c_int32(), C.c_double(), C.c_int32()
    eng.lib.pt_last_error_info(eng.handle, C.byref(proc), C.byref(E), C.byref(key))
    assert proc.value == -1 and 0.0 < E.value <= 1.0
    o.loop_limit = 0
    again, n_again = eng.run_sm(p0, np.zeros((20, 3)), pid, m, np.ones(20), o)
    same_rows(ref, n_ref, again, n_again, 20)


def test_store_overflow_is_retried_with_a_larger_store(lead):
    """pt_run_sm returns PT_OOM when the particle store is too small; the
    engine retries with twice the rows until the showers fit, and the rows
    are those of a run that fit at once."""
    p0, pid, m = primaries(8, seed=24, species=(11,), emin=5.0, emax=5.0)
    eng = lead._engine
    o = lead._opts(True, "fp64")
    big, n_big = eng.run_sm(p0, np.zeros((8, 3)), pid, m, np.ones(8), o, capacity=1 << 20)
    assert eng.last_store_capacity == 1 << 20
    small, n_small = eng.run_sm(p0, np.zeros((8, 3)), pid, m, np.ones(8), o, capacity=64)
    assert n_big > 64 and eng.last_store_capacity >= n_big    # grown by doubling from 64
    same_rows(big, n_big, small, n_small, 8)


def test_batch_ring_size_does_not_change_the_tallies(lead):
    """The batched engine sizes each wave so that its daughters fit the
    ring: a ring of 2^10 entries gives the tallies of a ring of 2^22."""
    p0, pid, m = primaries(64, seed=24, emin=20.0, emax=100.0)
    same(batch(lead, p0, pid, m, cap=1 << 22), batch(lead, p0, pid, m, cap=1 << 10))


def test_wave_bound_with_lanes(lead):
    """The wave bound holds per lane, and the handle recovers."""
    p0, pid, m = primaries(300, seed=23, emax=20.0)
    ref = batch(lead, p0, pid, m)
    lead._engine.set_tuning((0, 0), (0, 0), "host", lanes=3)
    try:
        with pytest.raises(_lib.PetiteGPUError) as e:
            batch(lead, p0, pid, m, loop_limit=2)
        assert e.value.status == _lib.PT_TIMEOUT
        again = batch(lead, p0, pid, m)
    finally:
        lead._engine.set_tuning((0, 0), (0, 0))
    same(ref, again)
