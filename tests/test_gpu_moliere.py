"""Bethe-Moliere multiple scattering (Shower(..., fast_MCS_mode=False)) on the
GPU, through the C ABI: the inverse CDF against the oracle and the
reference, record-engine showers draw for draw against the oracle and the
reference's own showers, the batched engine against the record engine, the
float32 form against float64, and dark-vector production in that mode."""
import math
import os

import numpy as np
import pytest

from conftest import BUNDLED_DIR, BUNDLED_NPZ, GOLDEN
from test_gpu_batch import primaries, run_batch
from test_gpu_parity import _compare_showers

pytestmark = pytest.mark.gpu

SEED = 0x5EED
G = np.load(os.path.join(GOLDEN, "moliere.npz"))


@pytest.fixture(scope="module")
def bethe():
    from petite_gb300 import Shower
    return {t: Shower(None, t, 0.010, seed=SEED, fast_MCS_mode=False) for t in ("graphite", "lead")}


def device_inverse_cdf(u, B, precision):
    import ctypes as C
    import torch
    from petite_gb300 import _lib
    lib = _lib.load()
    ut = torch.as_tensor(np.asarray(u, np.float64), device="cuda")
    Bt = torch.as_tensor(np.asarray(B, np.float64), device="cuda")
    x = torch.empty_like(ut)
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.pt_moliere_inverse_cdf(ut.data_ptr(), Bt.data_ptr(), len(ut), precision, x.data_ptr(),
                                          C.c_void_p(st)), "pt_moliere_inverse_cdf")
    return x.cpu().numpy()


def cdf_cases(n_per_B=400, seed=9):
    rng = np.random.default_rng(seed)
    U, Bs = [], []
    for B in (3.15, 3.7, 5.0, 7.5, 10.0, 14.0, 19.0):
        f00 = 0.5 * (2.0 + 0.845568670196936 / B)
        u = np.concatenate([rng.uniform(0, 1, n_per_B), 1 - 10 ** rng.uniform(-7, -0.5, n_per_B // 4),
                            rng.uniform(0.0095, 0.0105 * f00, n_per_B // 4)])
        U.append(u)
        Bs.append(np.full(len(u), B))
    return np.concatenate(U), np.concatenate(Bs)


def test_inverse_cdf_fp64_matches_oracle_and_reference():
    from oracle import physics as P
    u, B = cdf_cases()
    got = device_inverse_cdf(u, B, 0)
    want = np.array([P.moliere_x(a, b) for a, b in zip(u, B)])
    # same equations and iterations; the device's exp/log differ from libm's
    # by an ulp or two, which the far tail's conditioning (~B x) magnifies
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)
    rows = G["icdf/rows"]
    got = device_inverse_cdf(rows[:, 1], rows[:, 0], 0)
    # the reference's Ridder search stops at |dx| <= 2e-12
    assert (np.abs(got - rows[:, 2]) <= 4e-12 + 2e-10 * rows[:, 2]).all()


def test_inverse_cdf_fp32_matches_oracle():
    """The float32 form: Newton to 1e-5 relative on a float32 tail whose
    truncations are ~2e-8 absolute; the explicit branches are exact up to the
    float32 rounding of u and B."""
    from oracle import physics as P
    u, B = cdf_cases(seed=10)
    u32 = u.astype(np.float32).astype(np.float64)
    B32 = B.astype(np.float32).astype(np.float64)
    got = device_inverse_cdf(u, B, 1)
    want = np.array([P.moliere_x(a, b) for a, b in zip(u32, B32)])
    rel = np.abs(got - want) / want
    print("float32 inverse CDF: median rel", np.median(rel), "max", rel.max())
    assert np.median(rel) < 2e-6
    assert rel.max() < 2e-3


CASES = [("graphite", 11, 1.0, 20, 0.000511, 1e-8), ("lead", -11, 3.0, 3, 0.000511, 1e-6),
         ("graphite", 13, 5.0, 3, 0.1056583755, 1e-8), ("lead", 11, 0.3, 30, 0.000511, 1e-8)]


@pytest.mark.parametrize("target,pid,E0,n,mass,vec_rtol", CASES)
def test_bethe_showers_match_oracle(bethe, target, pid, E0, n, mass, vec_rtol):
    from oracle.shower import OracleShower, OracleTables
    p = math.sqrt(E0 * E0 - mass * mass)
    batch = bethe[target].generate_showers(np.tile([E0, 0.0, 0.0, p], (n, 1)), pid=pid, mass=mass, first_primary=0)
    orc = OracleShower(OracleTables(BUNDLED_NPZ, target), 0.010, seed=SEED, fast_MCS_mode=False)
    rows = []
    for j in range(n):
        rows += orc.generate_shower((E0, 0.0, 0.0, p), pid=pid, mass=mass, primary_index=j)
    worst = _compare_showers(batch, rows, vec_rtol)
    print(target, pid, E0, "rows", batch.n, "worst", worst)


def test_bethe_golden_reference_showers(bethe):
    """The GPU against the reference's own fast_MCS_mode=False showers."""
    for name in ("e1gev_graphite", "pos3_lead", "mu5_graphite"):
        pre = f"shower/{name}"
        seed, pid, n = (int(v) for v in G[f"{pre}/meta"])
        E0, cut, mass = G[f"{pre}/params"]
        F, I = G[f"{pre}/f64"], G[f"{pre}/i64"]
        m = 0.0 if pid == 22 else mass
        p = math.sqrt(E0 * E0 - m * m)
        b = bethe[str(G[f"{pre}/target"])].generate_showers(np.tile([E0, 0, 0, p], (n, 1)), pid=pid,
                                                            mass=F[0, 15], first_primary=0)
        o = b.order
        assert len(o) == len(F), name
        parent_pid = np.where(b.parent[o] >= 0, b.pid[np.maximum(b.parent[o], 0)], 22)
        got = np.c_[b.pid[o], parent_pid, b.gen[o], b.proc[o], np.ones(len(o), int), b.primary[o]]
        assert np.array_equal(got, I), name
        assert np.array_equal(b.pkey[o], G[f"{pre}/pkey"]), name
        np.testing.assert_allclose(b.p0[o][:, 0], F[:, 0], rtol=1e-12, atol=0)
        np.testing.assert_allclose(b.pf[o][:, 0], F[:, 7], rtol=1e-12, atol=0)
        scale = np.abs(F[:, 7:11]).max(1)
        assert (np.abs(b.pf[o] - F[:, 7:11]).max(1) <= 1e-7 * scale).all(), name


def test_bethe_batch_fp64_equals_record_engine(bethe):
    sh = bethe["lead"]
    p0, pid, m = primaries(300, seed=21)
    b = sh.generate_showers(p0, pid=pid, mass=m, first_primary=0)
    t = run_batch(sh, p0, pid, m, "fp64")
    s = t.summary()
    assert np.array_equal(t.primary_count.cpu().numpy(), np.bincount(b.primary, minlength=len(p0)))
    assert s["steps"] == b.n
    np.testing.assert_allclose(s["E_continuous"], float(np.sum(b.p0[:, 0] - b.pf[:, 0])), rtol=1e-12)


def test_bethe_mixed_matches_fp64(bethe):
    """The float32 engine in Bethe-Moliere mode against float64 on the same
    streams: totals and the binned spectra of creation energy and depth."""
    sh = bethe["lead"]
    p0, pid, m = primaries(2000, seed=23, emax=100.0)
    f = run_batch(sh, p0, pid, m, "fp64")
    x = run_batch(sh, p0, pid, m, "mixed")
    sf, sx = f.summary(), x.summary()
    same = float(np.mean(f.primary_count.cpu().numpy() == x.primary_count.cpu().numpy()))
    print("Bethe mode: identical showers", same, "steps", sf["steps"], sx["steps"])
    assert same > 0.8
    assert abs(sx["steps"] - sf["steps"]) / sf["steps"] < 5e-3
    assert abs(sx["E_deposited"] - sf["E_deposited"]) / sf["E_deposited"] < 2e-3
    hf, hx = f.hist.cpu().numpy().astype(float), x.hist.cpu().numpy().astype(float)
    for kind in (0, 2):
        a, b = hf[kind].ravel(), hx[kind].ravel()
        mask = (a + b) > 20
        chi2 = np.sum((a[mask] - b[mask]) ** 2 / (a[mask] + b[mask]))
        assert chi2 / mask.sum() < 2.0, (kind, chi2 / mask.sum())


def test_bethe_dark_production_matches_oracle():
    """pt_run_dark in Bethe-Moliere mode (the parent's scattering to the
    interaction point, dark_shower.py:755-757) against the oracle."""
    from oracle import dark as D
    from oracle.shower import OracleTables
    from petite_gb300.dark import DarkShower
    procs = ("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")
    sh = DarkShower(None, "graphite", 0.010, 0.1, seed=SEED, active_processes=list(procs), fast_MCS_mode=False)
    n = 3
    p = math.sqrt(100.0 - 0.000511 ** 2)
    opts = sh._opts(True, "fp64")
    opts.primary_offset = 91
    st, nr = sh._engine.run_sm(np.tile([10.0, 0, 0, p], (n, 1)), np.zeros((n, 3)), np.full(n, 11, np.int32),
                               np.full(n, 0.000511), np.ones(n), opts)
    res = sh._dark_engine.run_dark(sh._prm, st, nr, sh._opts())
    rows = st.to_numpy(nr)

    class R:
        pass
    recs = []
    for k in range(nr):
        r = R()
        r.p0, r.pf, r.rf = tuple(rows["p0"][k]), tuple(rows["pf"][k]), tuple(rows["rf"][k])
        r.pid, r.mass, r.weight, r.pkey = int(rows["pid"][k]), float(rows["mass"][k]), 1.0, int(rows["pkey"][k])
        recs.append(r)
    dark_npz = os.path.join(BUNDLED_DIR, "dark_tables.npz")
    orc = D.DarkOracle(D.DarkTables(dark_npz, "graphite", 0.1), OracleTables(BUNDLED_NPZ, "graphite"), SEED,
                       fast_MCS_mode=False)
    out = orc.dark_shower(recs, processes=procs)
    want = np.array([[k, D.DARK_CODE[pp], w, *v] for k, pp, w, v, _ in out])
    want = want[np.lexsort((want[:, 1], want[:, 0]))]
    proc = res["process"] % 4
    o = np.lexsort((proc, res["parent"]))
    assert res["n"] == len(want) > 50
    assert np.array_equal(res["parent"][o], want[:, 0].astype(np.int64))
    assert np.array_equal(proc[o], want[:, 1].astype(np.int64))
    np.testing.assert_allclose(res["weight"][o], want[:, 2], rtol=1e-12, atol=0)
    np.testing.assert_allclose(res["p4"][o][:, 0], want[:, 3], rtol=1e-12, atol=0)
    scale = np.abs(want[:, 3:7]).max(1)
    assert (np.abs(res["p4"][o] - want[:, 3:7]).max(1) <= 1e-7 * scale).all()
