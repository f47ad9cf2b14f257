"""The GPU table builder (petite_gb300.train): the VEGAS adaptation against
its CPU restatement, trained maps against the cross sections PETITE ships,
and showers run on trained maps against showers on PETITE's maps."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_adapt_matches_oracle():
    import ctypes as C
    import torch
    from oracle.vegas_train import adapt
    from petite_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(3)
    ninc = [960, 1000]
    rows, D, mn = 3, 2, 1001
    g = np.zeros((rows, D, mn))
    acc = np.zeros((rows, D, 1000))
    cnt = np.zeros((rows, D, 1000), np.int32)
    for r in range(rows):
        for d in range(D):
            n = ninc[d]
            g[r, d, :n + 1] = np.sort(np.r_[0.0, rng.uniform(0, 3, n - 1), 3.0])
            acc[r, d, :n] = rng.gamma(0.3, 1.0, n) * (rng.uniform(size=n) < 0.8)
            cnt[r, d, :n] = rng.integers(0, 20, n)
    want = np.array([[adapt(g[r, d, :ninc[d] + 1], acc[r, d], cnt[r, d]) for d in range(D)] for r in range(rows)],
                    dtype=object)
    dev = "cuda"
    tg, ta, tc = (torch.as_tensor(a, device=dev) for a in (g, acc, cnt))
    tn = (C.c_int32 * D)(*ninc)                      # host array
    _lib.check(lib.pt_vegas_adapt(rows, D, tn, tg.data_ptr(), mn, ta.data_ptr(), tc.data_ptr(), 0.5,
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream)), "pt_vegas_adapt")
    got = tg.cpu().numpy()
    for r in range(rows):
        for d in range(D):
            np.testing.assert_allclose(got[r, d, :ninc[d] + 1], want[r, d], rtol=1e-12, atol=1e-14)


@pytest.fixture(scope="module")
def bundled():
    from petite_gb300 import tables as T
    return T.read_dict_dir(T.BUNDLED_DIR)


@pytest.mark.parametrize("process,tol", [("Comp", 0.01), ("Moller", 0.02), ("Brem", 0.03), ("PairProd", 0.03)])
def test_trained_maps_reproduce_shipped_cross_sections(bundled, process, tol):
    """Maps trained from flat grids at PETITE's energies: find_maxes' cross
    section on graphite against the shipped sm_xsec.pkl (PETITE's own
    find_maxes estimate with its own maps), row by row where it is not tiny."""
    from petite_gb300.train import MapSet, find_maxes, train
    rows = bundled.maps[process]
    sel = np.linspace(10, len(rows) - 1, 8).astype(int)
    E = np.array([rows[i].energy for i in sel])
    ms = train(MapSet.uniform(process, E), points_per_row=1 << 20)
    mf, xs = find_maxes(ms, targets=("graphite",), n_trials=400)
    ref_tab = bundled.xsec[process]["graphite"]
    ref = np.interp(E, ref_tab[:, 0], ref_tab[:, 1])
    ok = ref > 1e-3 * ref.max()
    rel = np.abs(xs[ok, 0] / ref[ok] - 1)
    print(process, "xsec ratio", np.round(xs[ok, 0] / ref[ok], 4), "max_F", mf[:, 0])
    assert ok.sum() >= 5 and rel.max() < tol, rel


@pytest.mark.parametrize("process", ["DarkBrem", "DarkMuonBrem"])
def test_trained_dark_maps_reproduce_400gev_cross_sections(process):
    """DarkBrem / DarkMuonBrem maps (mV = 0.1 GeV) trained from flat grids on
    hydrogen with mT = 200 GeV, as PETITE trains them, at energies up to 400
    GeV: find_maxes' cross sections on lead and graphite against PETITE's
    data_400GeV/dark_xsec.pkl rows (its find_maxes estimate with the maps it
    does not ship).  Each row carries both estimates' Monte Carlo error
    (a few per cent)."""
    import os
    from conftest import GOLDEN
    from petite_gb300.train import MapSet, find_maxes, train
    dx = np.load(os.path.join(GOLDEN, "dark_xsec_400GeV.npz"))
    E = dx[f"{process}/lead"][:, 0]
    ms = train(MapSet.uniform(process, E, mV=float(dx["mV"])), points_per_row=1 << 21)
    mf, xs = find_maxes(ms, targets=("lead", "graphite"), n_trials=400)
    assert (mf > 0).all()
    for j, t in enumerate(("lead", "graphite")):
        q = xs[:, j] / dx[f"{process}/{t}"][:, 1]
        print(process, t, np.round(q, 4))
        assert abs(np.median(q) - 1) < 0.03 and np.abs(q - 1).max() < 0.12, q


def test_showers_on_trained_maps_match_shipped(bundled):
    """Lead, 10 GeV electrons: the Brem and PairProd maps replaced by maps
    trained here (max_F from find_maxes); multiplicity, deposited energy
    and depth distributions against showers on PETITE's maps (KS)."""
    from scipy import stats
    from petite_gb300 import Shower
    from petite_gb300 import tables as T
    from petite_gb300.train import MapSet, find_maxes, train
    import copy
    raw = copy.deepcopy(bundled)
    targets = tuple(sorted(raw.maps["Brem"][0].max_F))
    for proc in ("Brem", "PairProd"):
        E = np.array([r.energy for r in raw.maps[proc]])
        ms = train(MapSet.uniform(proc, E), points_per_row=1 << 19)
        mf, _ = find_maxes(ms, targets=targets)
        for r, (row, g) in enumerate(zip(raw.maps[proc], ms.grids())):
            row.grid = g
            row.max_F = {t: float(mf[r, j]) for j, t in enumerate(targets)}
    ref = Shower(None, "lead", 0.010, seed=5)
    new = Shower(None, "lead", 0.010, seed=5)
    new.tables = T.SMTables(raw, "lead", 1)
    from petite_gb300.engine import SMEngine
    new._engine = SMEngine(new.tables, "cuda")
    n = 400
    p0 = np.tile([10.0, 0.0, 0.0, math.sqrt(100.0 - 0.000511 ** 2)], (n, 1))
    a = ref.generate_showers(p0, pid=11, mass=0.000511, first_primary=0)
    b = new.generate_showers(p0, pid=11, mass=0.000511, first_primary=1_000_000)
    def obs(bt):
        # per-shower observables (per-particle samples of ~1e5 would resolve
        # the small max_F clipping that both map sets have)
        mult = np.bincount(bt.primary, minlength=n)
        photons = np.bincount(bt.primary[bt.pid == 22], minlength=n)
        depth = np.bincount(bt.primary, weights=bt.rf[:, 2], minlength=n) / np.maximum(mult, 1)
        return mult, photons, depth
    (ma, ea, za), (mb, eb, zb) = obs(a), obs(b)
    for name, x, y in (("multiplicity", ma, mb), ("photons", ea, eb), ("mean depth", za, zb)):
        p = stats.ks_2samp(x, y).pvalue
        print(name, "KS p", p, len(x), len(y))
        assert p > 0.001, name
