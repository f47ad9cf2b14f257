"""CUDA engine vs the CPU oracle (and the reference's golden showers).

All calls go through the C ABI (petite_gb300._lib -> libpetite_gpu.so).
Integer outputs (particle counts, PIDs, processes, parents, generations,
random-draw counts) must match exactly; energies to 1e-12 relative.
Directions and positions inherit the reference's conditioning (see
test_oracle_golden.py), so they are compared with the tolerances stated there.
"""
import math
import os

import numpy as np
import pytest

from conftest import BUNDLED_NPZ, GOLDEN

pytestmark = pytest.mark.gpu

SEED = 0x5EED


@pytest.fixture(scope="module")
def engines():
    from petite_gb300 import Shower
    out = {}
    for target in ("graphite", "lead"):
        out[target] = Shower(None, target, 0.010, seed=SEED)
    return out


def _oracle(target, cut=0.010):
    from oracle.shower import OracleShower, OracleTables
    return OracleShower(OracleTables(BUNDLED_NPZ, target), cut, seed=SEED)


@pytest.mark.parametrize("target", ["graphite", "lead"])
def test_dsigma_matches_oracle(engines, target):
    from oracle import physics as P
    from oracle.shower import map_point
    from petite_gb300.tables import PROCESSES
    sh = engines[target]
    orc = _oracle(target)
    rng = np.random.default_rng(7)
    for code, proc in enumerate(PROCESSES):
        rows = orc.t.maps[proc]
        X, E, want = [], [], []
        for r in rng.choice(len(rows), 20, replace=False):
            for _ in range(50):
                x, _ = map_point(rows[r]["grid"], rng.random(P.DIM[proc]))
                e = rows[r]["E"] * rng.uniform(0.9, 1.1)
                X.append(np.pad(x, (0, 4 - len(x))))
                E.append(e)
                m = P.m_muon if proc == "MuonBrem" else P.m_electron
                want.append(P.dsigma(proc, x, e, orc.t.Z, orc.t.Eg_min, orc.t.Ee_min, m))
        got = sh._engine.dsigma(code, np.array(X), np.array(E))
        want = np.array(want)
        assert (want != 0).sum() > 100
        # The engine's float64 hot loop fuses multiply-adds; the oracle rounds
        # every operation.  The reference formulas sum terms of opposite sign
        # (Brem/PairProd T4 < 0, all_processes.py:200,596-600; Compton
        # T1+T2+T3, :701-707; annihilation 1 - b^2 ct^2, :525), which magnifies
        # those last-place differences to at most ~1e-10 relative.  MuonBrem
        # evaluates the same Brem formula with the muon mass on maps trained
        # over physical ranges (all_processes.py:1120-1127), where T1+T2+T4
        # cancel to ~1e-9 of the individual terms: 1e-6 there.
        rtol = 1e-6 if proc == "MuonBrem" else 1e-10
        np.testing.assert_allclose(got, want, rtol=rtol, atol=0, err_msg=proc)


def test_draw_sample_matches_oracle(engines):
    from oracle.philox import Stream
    from oracle import physics as P
    from petite_gb300.tables import PROCESSES
    sh = engines["graphite"]
    orc = _oracle("graphite")
    for code, proc in enumerate(PROCESSES):
        if proc == "MuonBrem":
            # MuonBrem's maps sample where three terms of the Brem form cancel
            # to 1e-9 (all_processes.py:1120-1127): the GPU's fused
            # multiply-adds move the value by up to 1e-6, enough to flip an
            # accept/reject against the oracle; its showers are compared
            # statistically instead
            continue
        Es = np.geomspace(0.3 if proc == "MuonE" else 0.02, 90.0, 24)
        keys = np.array([1000 * code + i + 1 for i in range(len(Es))], np.uint64)
        opts = sh._opts()
        x, props, lu = sh._engine.sample_only(code, Es, keys, opts)
        for i, (E, k) in enumerate(zip(Es, keys)):
            cnt = []
            xo, key = orc.draw_sample(E, proc, Stream(SEED, int(k)), cnt)
            assert props[i] == cnt[0], (proc, E)
            assert lu[i] == key
            np.testing.assert_allclose(x[i, :P.DIM[proc]], xo, rtol=1e-14, atol=0)


def _compare_showers(batch, oracle_rows, vec_rtol):
    order = batch.order
    assert len(order) == len(oracle_rows)
    g = {k: getattr(batch, k)[order] for k in ("pid", "gen", "proc", "bit", "primary", "draws", "pkey")}
    oi = np.array([[r.pid, r.gen, r.proc, r.bit, r.primary] for r in oracle_rows])
    assert np.array_equal(np.c_[g["pid"], g["gen"], g["proc"], g["bit"], g["primary"]], oi)
    assert np.array_equal(g["pkey"], np.array([r.pkey for r in oracle_rows], np.uint64))
    # the reference stops the loop before the last particle's process choice
    # (shower.py:656-660), which only changes that particle's draw count
    od = np.array([r.draws for r in oracle_rows])
    diff = g["draws"] - od
    assert ((diff == 0) | (diff == 1)).all()
    # parent position in list order
    pos = np.empty(batch.n, np.int64)
    pos[order] = np.arange(batch.n)
    par = batch.parent[order]
    gpar = np.where(par >= 0, pos[np.maximum(par, 0)], -1)
    starts = {}
    for i, r in enumerate(oracle_rows):
        starts.setdefault(r.primary, i)
    opar = np.array([-1 if r.parent < 0 else starts[r.primary] + r.parent for r in oracle_rows])
    assert np.array_equal(gpar, opar)
    of = np.array([list(r.p0) + list(r.r0) + list(r.pf) + list(r.rf) for r in oracle_rows])
    gf = np.c_[batch.p0[order], batch.r0[order], batch.pf[order], batch.rf[order]]
    np.testing.assert_allclose(gf[:, [0, 7]], of[:, [0, 7]], rtol=1e-12, atol=0)
    worst = {}
    for name, sl in (("p0", slice(0, 4)), ("r0", slice(4, 7)), ("pf", slice(7, 11)), ("rf", slice(11, 14))):
        scale = np.maximum(np.abs(of[:, sl]).max(1), 1e-12)
        err = np.abs(gf[:, sl] - of[:, sl]).max(1) / scale
        worst[name] = float(err.max())
        assert err.max() <= vec_rtol, (name, err.max(), int(err.argmax()))
    return worst


CASES = [("graphite", 11, 1.0, 40, 0.000511, 1e-8), ("lead", 22, 10.0, 2, 0.0, 1e-6),
         ("lead", -11, 3.0, 4, 0.000511, 1e-6), ("graphite", 13, 5.0, 4, 0.1056583755, 1e-8),
         ("lead", 11, 0.3, 60, 0.000511, 1e-8)]


@pytest.mark.parametrize("target,pid,E0,n,mass,vec_rtol", CASES)
def test_showers_match_oracle(engines, target, pid, E0, n, mass, vec_rtol):
    sh = engines[target]
    p = math.sqrt(E0 * E0 - mass * mass)
    p0 = np.tile([E0, 0.0, 0.0, p], (n, 1))
    batch = sh.generate_showers(p0, pid=pid, mass=mass, first_primary=0)
    orc = _oracle(target)
    rows = []
    for j in range(n):
        rows += orc.generate_shower((E0, 0.0, 0.0, p), pid=pid, mass=mass, primary_index=j)
    worst = _compare_showers(batch, rows, vec_rtol)
    print(target, pid, E0, "rows", batch.n, "worst", worst)


def test_golden_reference_showers(engines):
    """The GPU against the reference's own showers (same streams)."""
    g = np.load(os.path.join(GOLDEN, "showers.npz"))
    for name in ("e1gev_graphite", "gamma10_lead", "pos3_lead", "mu5_graphite"):
        seed, pid, n = (int(v) for v in g[f"{name}/meta"])
        E0, cut, mass = g[f"{name}/params"]
        sh = engines[str(g[f"{name}/target"])]
        F, I = g[f"{name}/f64"], g[f"{name}/i64"]
        m = 0.0 if pid == 22 else mass
        p = math.sqrt(E0 * E0 - m * m)
        # the reference derived the primary's mass from its invariant (particle.py:125-131)
        b = sh.generate_showers(np.tile([E0, 0, 0, p], (n, 1)), pid=pid, mass=F[0, 15], first_primary=0)
        o = b.order
        assert len(o) == len(F), name
        parent_pid = np.where(b.parent[o] >= 0, b.pid[np.maximum(b.parent[o], 0)], 22)
        got = np.c_[b.pid[o], parent_pid, b.gen[o], b.proc[o], np.ones(len(o), int), b.primary[o]]
        assert np.array_equal(got, I), name
        assert np.array_equal(b.pkey[o], g[f"{name}/pkey"]), name
        np.testing.assert_allclose(b.p0[o][:, 0], F[:, 0], rtol=1e-12, atol=0)
        np.testing.assert_allclose(b.pf[o][:, 0], F[:, 7], rtol=1e-12, atol=0)


def test_dropin_generate_shower_ids(engines):
    from petite_gb300 import Particle
    sh = engines["graphite"]
    part = Particle([1.0, 0, 0, math.sqrt(1 - 0.000511 ** 2)], [0, 0, 0], {"PID": 11})
    out = sh.generate_shower(part)
    assert out[0].get_ids()["ID"] == 1 and out[0].get_ended()
    ids = {}
    for k, p in enumerate(out):
        d = p.get_ids()
        ids[d["ID"]] = p
        if k:
            parent = ids[d["parent_ID"]]
            assert d["ID"] // 2 == d["parent_ID"]
            assert d["generation_number"] == parent.get_ids()["generation_number"] + 1
            assert d["parent_PID"] == parent.get_ids()["PID"]
            assert d["generation_process"] in ("Brem", "Moller", "Ann", "Bhabha", "PairProd", "Comp")
            assert np.array_equal(p.get_r0(), parent.get_rf())
            assert p.get_p0()[0] > 0.010
    # below the cut: the primary comes back unchanged
    low = Particle([0.005, 0, 0, math.sqrt(0.005 ** 2 - 0.000511 ** 2)], [0, 0, 0], {"PID": 11})
    assert len(sh.generate_shower(low)) == 1


def test_no_sample_found_raises():
    """With max_F scaled far above every weight the sampler cannot accept;
    after max_n_integrators*neval proposals it must report PETITE's
    'No Sample Found' (shower.py:460-461) instead of looping on."""
    from petite_gb300 import Shower
    sh = Shower(None, "graphite", 0.010, seed=1, max_n_integrators=2, maxF_fudge_global=1e300)
    with pytest.raises(Exception, match="No Sample Found"):
        sh.draw_sample(1.0, process="Comp")
