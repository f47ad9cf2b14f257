"""pt_run_sm_noalloc (static device scratch, no allocation) against pt_run_sm.

Collected last on purpose: it must pass on its own and after every other
test has used the library on the same device."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 0x5EED
CAPACITY = 1 << 15


@pytest.fixture(scope="module")
def shower():
    from petite_gb300 import Shower
    return Shower(None, "graphite", 0.010, seed=SEED)


def primaries():
    rng = np.random.default_rng(5)
    n = 24
    pid = np.array([11, -11, 22])[rng.integers(0, 3, n)].astype(np.int32)
    E = 10 ** rng.uniform(-1, 0.5, n)
    m = np.where(np.abs(pid) == 11, 0.000511, 0.0)
    p0 = np.c_[E, np.zeros(n), np.zeros(n), np.sqrt(E * E - m * m)]
    return p0, pid, m


def filled_store(eng, p0, pid, m, capacity):
    import torch
    from petite_gb300.engine import ParticleStore
    n = len(p0)
    st = ParticleStore(capacity, eng.device)
    st.t["p0"][:, :n] = torch.as_tensor(p0.T, device=eng.device)
    st.t["pid"][:n] = torch.as_tensor(pid, device=eng.device)
    st.t["mass"][:n] = torch.as_tensor(m, device=eng.device)
    st.t["weight"][:n] = 1.0
    return st


def run(eng, entry, st, n, opts):
    abi = st.abi()
    rows = C.c_int64()
    s = getattr(eng.lib, entry)(eng.handle, C.byref(abi), n, C.byref(opts), C.byref(rows), eng._stream())
    return s, int(rows.value)


def test_noalloc_matches_pt_run_sm_twice(shower):
    eng = shower._engine
    opts = shower._opts(True, "fp64")
    p0, pid, m = primaries()
    n = len(p0)
    ref = filled_store(eng, p0, pid, m, CAPACITY)
    s, nref = run(eng, "pt_run_sm", ref, n, opts)
    assert s == 0 and nref > 10 * n
    want = ref.to_numpy(nref)
    for call in range(2):          # the second call must start from zeroed counters and status
        st = filled_store(eng, p0, pid, m, CAPACITY)
        s, rows = run(eng, "pt_run_sm_noalloc", st, n, opts)
        assert s == 0, call
        assert rows == nref, call
        got = st.to_numpy(rows)
        # rows are appended in a data-dependent order: compare in list order
        for k in ("pid", "gen", "proc", "bit", "primary", "draws", "pkey"):
            assert np.array_equal(np.sort(got[k]), np.sort(want[k])), (call, k)
        key_got, key_want = np.argsort(got["pkey"]), np.argsort(want["pkey"])
        for k in ("pid", "gen", "proc", "bit", "primary", "draws"):
            assert np.array_equal(got[k][key_got], want[k][key_want]), (call, k)
        for k in ("p0", "pf", "r0", "rf"):
            np.testing.assert_allclose(got[k][key_got], want[k][key_want], rtol=1e-12, atol=1e-300,
                                       err_msg=f"{call} {k}")


def test_noalloc_rejects_stores_above_its_limit(shower):
    from petite_gb300 import _lib
    eng = shower._engine
    opts = shower._opts(True, "fp64")
    p0, pid, m = primaries()
    st = filled_store(eng, p0[:1], pid[:1], m[:1], _lib.NOALLOC_MAX_ROWS + 1)
    s, _ = run(eng, "pt_run_sm_noalloc", st, 1, opts)
    assert s == _lib.PT_BAD_ARG
    # and the limit itself is accepted
    del st
    st = filled_store(eng, p0[:1], pid[:1], m[:1], _lib.NOALLOC_MAX_ROWS)
    s, rows = run(eng, "pt_run_sm_noalloc", st, 1, opts)
    assert s == 0 and rows >= 1
    assert math.isfinite(float(st.t["pf"][0, 0]))
