"""Dark-vector production and the differentiable dark yield on the GPU, through
the C ABI, against the oracle and the reference's golden vectors."""
import math
import os

import numpy as np
import pytest

from conftest import BUNDLED_DIR, BUNDLED_NPZ, GOLDEN

pytestmark = pytest.mark.gpu

SEED = 0x5EED
G = np.load(os.path.join(GOLDEN, "dark.npz"))
DARK_NPZ = os.path.join(BUNDLED_DIR, "dark_tables.npz")


@pytest.fixture(scope="module")
def showers():
    from petite_gb300.dark import DarkShower
    out = {}
    for mV, t in ((0.1, "graphite"), (0.03, "graphite"), (0.01, "lead"), (0.3, "graphite"), (0.01, "graphite"),
                  (0.1, "lead"), (0.3, "lead")):
        out[(mV, t)] = DarkShower(None, t, 0.010, mV, seed=SEED,
                                  active_processes=["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"])
    return out


@pytest.mark.parametrize("mV", [0.01, 0.1, 0.3])
@pytest.mark.parametrize("target", ["graphite", "lead"])
def test_dark_dsigma_matches_oracle_and_reference(showers, mV, target):
    from oracle import dark as D
    from oracle import physics as P
    eng = showers[(mV, target)]._dark_engine
    ti = P.TARGETS[target]
    for code, proc in enumerate(D.DARK_PROCESSES):
        pre = f"dsigma/{mV}/{target}/{proc}"
        X, E, V = G[f"{pre}/x"], G[f"{pre}/E"], G[f"{pre}/value"]
        got = eng.dsigma(code, X, E, mV)
        want = np.array([D.dsigma_dark(proc, x, e, mV, ti["Z_T"], ti["A_T"]) for x, e in zip(X, E)])
        # fused multiply-adds and CUDA's pow/log against the oracle's rounded
        # operations.  The dark-brem form (all_processes.py:290-352) takes
        # W = |Y^2 - 4 q^2 p^2 k^2 (1-cos^2)(1-cos_q^2)/V^2| and A0 + Y A1 +
        # Am1/sqrt(W) + Y Am2/W^1.5, differences of nearly equal terms near
        # the edges of the allowed region, so last-place differences grow to
        # ~1e-7 there; the Compton form sums T1 + T2 + T3 of opposite signs
        # near threshold (mV = 0.3 GeV), ~1e-9; the radiative return ~1e-11.
        rtol = 1e-6 if proc in ("DarkBrem", "DarkMuonBrem") else 1e-8
        nz = want != 0
        if nz.any():
            print(proc, mV, target, "max rel", float(np.max(np.abs(got[nz] - want[nz]) / np.abs(want[nz]))))
        np.testing.assert_allclose(got, want, rtol=rtol, atol=0, err_msg=proc)
        np.testing.assert_allclose(got, V, rtol=rtol, atol=0, err_msg=proc)


def test_draw_dark_sample_matches_reference(showers):
    from oracle import dark as D
    sh = showers[(0.1, "graphite")]
    for row in G["draw/rows"]:
        case, pi, E = int(row[0]), int(row[1]), row[2]
        proc = D.DARK_PROCESSES[pi]
        x, props, _ = sh._dark_engine.sample_only(sh._prm, pi, [E], [np.uint64(60_000 + case)], sh._opts())
        assert props[0] == int(row[-1]), (proc, E)
        np.testing.assert_allclose(x[0, :D.DARK_DIM[proc]], row[3:3 + D.DARK_DIM[proc]], rtol=1e-12, atol=0)


def _store_from_golden(sh, name, g=None, pre=None):
    import torch
    from petite_gb300.engine import ParticleStore
    g = G if g is None else g
    pre = f"shower/{name}" if pre is None else pre
    F, I, K = g[f"{pre}/sm_f64"], g[f"{pre}/sm_i64"], g[f"{pre}/sm_pkey"]
    n = len(F)
    st = ParticleStore(n, sh._engine.device)
    dev = sh._engine.device
    st.t["p0"][:, :n] = torch.as_tensor(F[:, 0:4].T.copy(), device=dev)
    st.t["pf"][:, :n] = torch.as_tensor(F[:, 7:11].T.copy(), device=dev)
    st.t["rf"][:, :n] = torch.as_tensor(F[:, 11:14].T.copy(), device=dev)
    st.t["weight"][:n] = torch.as_tensor(F[:, 14].copy(), device=dev)
    st.t["mass"][:n] = torch.as_tensor(F[:, 15].copy(), device=dev)
    st.t["pid"][:n] = torch.as_tensor(I[:, 0].astype(np.int32), device=dev)
    st.t["pkey"][:n] = torch.as_tensor(K.astype(np.uint64).view(np.int64), device=dev)
    return st, n


@pytest.mark.parametrize("name", ["e10_graphite_m0.1", "e10_graphite_m0.03", "g5_lead_m0.01"])
def test_run_dark_matches_reference_showers(showers, name):
    mV = float(G[f"shower/{name}/params"][0])
    target = str(G[f"shower/{name}/target"])
    sh = showers[(mV, target)]
    st, n = _store_from_golden(sh, name)
    res = sh._dark_engine.run_dark(sh._prm, st, n, sh._opts())
    V = G[f"shower/{name}/V"]
    want = V[np.lexsort((V[:, 2], V[:, 0]))]
    proc = res["process"] % 4
    o = np.lexsort((proc, res["parent"]))
    assert res["n"] == len(want)
    assert np.array_equal(res["parent"][o], want[:, 0].astype(np.int64))
    assert np.array_equal(proc[o], want[:, 2].astype(np.int64))
    assert np.array_equal(res["process"][o] >= 4, np.isin(want[:, 2], (1, 2)))     # *_bound forms
    np.testing.assert_allclose(res["weight"][o], want[:, 3], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(res["r"][o], want[:, 8:11])
    np.testing.assert_allclose(res["p4"][o][:, 0], want[:, 4], rtol=1e-12, atol=0)
    scale = np.abs(want[:, 4:8]).max(1)
    err = np.abs(res["p4"][o] - want[:, 4:8]).max(1) / scale
    assert err.max() <= 1e-9, err.max()
    # summed yields
    np.testing.assert_allclose(res["yield"][:3], [want[want[:, 2] == p, 3].sum() for p in range(3)], rtol=1e-12)


def test_generate_dark_shower_dropin(showers):
    from petite_gb300 import Particle
    sh = showers[(0.1, "graphite")]
    part = Particle([10.0, 0, 0, math.sqrt(100 - 0.000511 ** 2)], [0, 0, 0], {"PID": 11})
    sm, vs = sh.generate_dark_shower(SParams=part)
    assert len(sm) > 50 and len(vs) > 10
    ids = {p.get_ids()["ID"]: p for p in sm}
    for v in vs:
        d = v.get_ids()
        assert d["PID"] == 4900022
        parent = ids[d["parent_ID"]]
        assert d["ID"] == 2 * d["parent_ID"]
        assert d["parent_PID"] == parent.get_ids()["PID"]
        assert d["generation_number"] == parent.get_ids()["generation_number"] + 1
        assert d["generation_process"] in ("DarkBrem", "DarkAnn_bound", "DarkComp_bound")
        assert np.array_equal(v.get_r0(), parent.get_rf())
        p4 = v.get_p0()
        assert p4[0] ** 2 - p4[1] ** 2 - p4[2] ** 2 - p4[3] ** 2 == pytest.approx(0.1 ** 2, rel=1e-6)
    w = sh.GetBSMWeights(sm[0], "DarkBrem")
    assert w > 0


def test_dark_yield_matches_oracle(showers):
    from oracle import dark as D
    from petite_gb300.dark import dark_yield
    sh = showers[(0.1, "graphite")]
    eng = sh._dark_engine
    tabs = D.DarkTables(DARK_NPZ, "graphite", 0.1)
    E = np.array([0.5, 2.0, 8.0, 30.0])
    mV = np.array([0.1, 0.12, 0.2, 0.25])
    for proc in ("DarkBrem", "DarkComp", "DarkAnn"):
        Y, M = dark_yield(eng, proc, E, mV, n_samples=1500, seed=SEED, mass_index=np.full(4, eng.mass_index(0.1)))
        Y, M = Y.cpu().numpy(), M.cpu().numpy()
        for i in range(len(E)):
            y, m = D.dark_yield(tabs, proc, E[i], mV[i], i, 1500, SEED)
            np.testing.assert_allclose([Y[i], M[i]], [y, m], rtol=1e-8, atol=0, err_msg=proc)


def test_dark_yield_gradient_matches_finite_differences(showers):
    """4096 (E, mV) pairs, E log-uniform on [0.05, 10] GeV, mV log-uniform on
    [0.001, 0.3] GeV, 10^4 map samples each: the adjoint d(yield)/d(mV) and
    d(moment)/d(mV) against central differences of the forward kernel
    (h = 1e-4 relative), within 1e-3 relative."""
    import torch
    from petite_gb300.dark import dark_yield, map_mass_index
    sh = showers[(0.1, "graphite")]
    eng = sh._dark_engine
    rng = np.random.default_rng(4)
    n = 4096
    E = 10 ** rng.uniform(math.log10(0.05), 1.0, n)
    mVh = 10 ** rng.uniform(-3, math.log10(0.3), n)
    h = 1e-4 * mVh
    results = {}
    for proc in ("DarkBrem", "DarkComp", "DarkAnn"):
        mi = map_mass_index(eng.data.masses, mVh, eng.has_maps(proc), proc)
        mV = torch.tensor(mVh, dtype=torch.float64, device=eng.device, requires_grad=True)
        Y, M = dark_yield(eng, proc, E, mV, n_samples=10_000, seed=SEED, mass_index=mi)
        (Y.sum()).backward()
        gY = mV.grad.cpu().numpy().copy()
        mV.grad = None
        Y, M = dark_yield(eng, proc, E, mV, n_samples=10_000, seed=SEED, mass_index=mi)
        (M.sum()).backward()
        gM = mV.grad.cpu().numpy().copy()
        with torch.no_grad():
            Yp, Mp = dark_yield(eng, proc, E, mVh + h, n_samples=10_000, seed=SEED, mass_index=mi, anchor=mVh)
            Ym, Mm = dark_yield(eng, proc, E, mVh - h, n_samples=10_000, seed=SEED, mass_index=mi, anchor=mVh)
        fdY = (Yp - Ym).cpu().numpy() / (2 * h)
        fdM = (Mp - Mm).cpu().numpy() / (2 * h)
        Yv = Y.detach().cpu().numpy()
        ok = np.isfinite(Yv) & (Yv > 0) & np.isfinite(fdY)
        assert ok.sum() > 100, proc
        # DarkBrem: the forward estimate at mV +/- h keeps each sample at its
        # fraction of the momentum-transfer range of mV (the anchor), so no
        # sample crosses a kinematic edge between the two evaluations
        relY = np.abs(gY[ok] - fdY[ok]) / np.maximum(np.abs(fdY[ok]), 1e-300)
        relM = np.abs(gM[ok] - fdM[ok]) / np.maximum(np.abs(fdM[ok]), 1e-300)
        print(proc, "pairs", ok.sum(), "median rel", np.median(relY), "frac>1e-3", np.mean(relY > 1e-3))
        results[proc] = (np.mean(relY <= 1e-3), np.mean(relM <= 1e-3), np.sort(relY)[-5:], np.sort(relM)[-5:])
        bad = np.where(ok)[0][~(relY <= 1e-3)][:5]
        for i in bad:
            print("  off", proc, "E", E[i], "mV", mVh[i], "Y", Yv[i], "g", gY[i], "fd", fdY[i])
    print(results)
    for proc, (fy, fm, wy, wm) in results.items():
        assert fy > 0.99 and fm > 0.99, (proc, fy, fm, wy, wm)


def test_dark_yield_gradient_matches_fp64_reference(showers):
    """The adjoint against the float64 oracle's forward-mode derivative of the
    same estimate (DarkBrem samples carried with mV, radiative return factored)."""
    import torch
    from oracle import dark as D
    from petite_gb300.dark import dark_yield
    sh = showers[(0.1, "graphite")]
    eng = sh._dark_engine
    tabs = D.DarkTables(DARK_NPZ, "graphite", 0.1)
    E = np.array([0.6, 2.0, 8.0, 30.0, 90.0])
    mVh = np.array([0.1, 0.12, 0.2, 0.15, 0.28])
    mi = np.full(len(E), eng.mass_index(0.1))
    ns = 400
    for proc in ("DarkBrem", "DarkComp", "DarkAnn"):
        mV = torch.tensor(mVh, dtype=torch.float64, device=eng.device, requires_grad=True)
        Y, M = dark_yield(eng, proc, E, mV, n_samples=ns, seed=SEED, mass_index=mi)
        (Y + 0.001 * M).sum().backward()
        g = mV.grad.cpu().numpy()
        for i in range(len(E)):
            gy, gm = D.dark_yield_gradient(tabs, proc, E[i], mVh[i], i, ns, SEED)
            ref = gy + 0.001 * gm
            if ref == 0.0:
                assert g[i] == 0.0
                continue
            assert abs(g[i] - ref) <= 1e-6 * abs(ref), (proc, E[i], mVh[i], g[i], ref)


@pytest.mark.parametrize("mV,target", [(0.1, "graphite"), (0.03, "iron"), (0.3, "molybdenum"), (0.05, "lead"),
                                       (0.001, "graphite")])
def test_dark_on_gpu_showers_matches_oracle(showers, mV, target):
    """SM showers from the GPU record engine, then pt_run_dark against the
    oracle's produce_bsm_particle on the same rows and streams (10 GeV e-).
    mV = 0.001 GeV: maps trained here, tables built natively, no DarkAnn."""
    from oracle import dark as D
    from oracle.shower import OracleTables
    from petite_gb300.dark import DarkShower, processes_at_mass
    procs = processes_at_mass(["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"], mV)
    sh = showers.get((mV, target)) or DarkShower(None, target, 0.010, mV, seed=SEED, active_processes=procs)
    n = 4
    p = math.sqrt(100.0 - 0.000511 ** 2)
    opts = sh._opts(True, "fp64")
    opts.primary_offset = 77
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
    orc = D.DarkOracle(D.DarkTables(DARK_NPZ, target, mV), OracleTables(BUNDLED_NPZ, target), SEED)
    out = orc.dark_shower(recs, processes=tuple(procs))
    want = np.array([[k, D.DARK_CODE[pp], w, *v] for k, pp, w, v, _ in out])
    want = want[np.lexsort((want[:, 1], want[:, 0]))]
    proc = res["process"] % 4
    o = np.lexsort((proc, res["parent"]))
    assert res["n"] == len(want) > 100
    assert np.array_equal(res["parent"][o], want[:, 0].astype(np.int64))
    assert np.array_equal(proc[o], want[:, 1].astype(np.int64))
    np.testing.assert_allclose(res["weight"][o], want[:, 2], rtol=1e-12, atol=0)
    np.testing.assert_allclose(res["p4"][o][:, 0], want[:, 3], rtol=1e-12, atol=0)
    for p_ in range(3):
        np.testing.assert_allclose(res["yield"][p_], want[want[:, 1] == p_, 2].sum(), rtol=1e-12)


MESONS = np.load(os.path.join(GOLDEN, "mesons.npz"))


@pytest.mark.parametrize("mV", [0.01, 0.1, 0.3])
def test_two_body_meson_decay_dropin(mV):
    """generate_dark_shower(ExDir=[Particle, ...]) with pi0s from the
    reference's beam file and photons in between, default active processes
    (TwoBody_BSMDecay included): the reference's vectors, in its order, with
    its IDs, weights, masses and momenta."""
    from petite_gb300 import Particle
    from petite_gb300.dark import DarkShower
    pre = f"m{mV}"
    F, I, K = MESONS[f"{pre}/parts_f64"], MESONS[f"{pre}/parts_i64"], MESONS[f"{pre}/parts_pkey"]
    parts = []
    for k in range(len(F)):
        ids = {"PID": int(I[k, 0]), "ID": int(I[k, 1]), "weight": float(F[k, 7])}
        p = Particle(list(F[k, 0:4]), list(F[k, 4:7]), ids)
        assert p.get_ids()["mass"] == F[k, 8]     # the invariant, rounded as the reference rounds it
        p._pkey = int(K[k])
        parts.append(p)
    ds = DarkShower(None, "graphite", 0.010, mV, seed=SEED)
    w = np.array([ds.GetBSMWeights(p, "TwoBody_BSMDecay") for p in parts])
    np.testing.assert_allclose(w, MESONS[f"{pre}/weights"], rtol=1e-15, atol=0)
    _, vs = ds.generate_dark_shower(ExDir=parts)
    V = MESONS[f"{pre}/V"]
    assert len(vs) == len(V)
    for v, row in zip(vs, V):
        d = v.get_ids()
        assert d["parent_ID"] == parts[int(row[0])].get_ids()["ID"]
        assert (d["generation_process"] == "TwoBody_BSMDecay") == (row[1] == 8)
        assert (d["ID"], d["parent_ID"]) == (int(row[10]), int(row[11]))
        assert d["weight"] == pytest.approx(row[2], rel=1e-14)
        np.testing.assert_allclose(v.get_p0(), row[3:7], rtol=0, atol=1e-12 * np.abs(row[3:7]).max())
        np.testing.assert_array_equal(v.get_r0(), row[7:10])
        if row[1] == 8:
            assert d["mass"] == row[12]


def test_eta_input_raises_like_the_reference():
    """The reference's GetBSMWeights has no threshold entry for eta and eta'
    (dark_shower.py:604) and raises KeyError."""
    from petite_gb300 import Particle
    from petite_gb300.dark import DarkShower
    assert int(MESONS["eta/raises"]) == 1
    ds = DarkShower(None, "graphite", 0.010, 0.03, seed=SEED)
    eta = Particle([5.0, 0.0, 0.0, math.sqrt(25.0 - 0.547862 ** 2)], [0, 0, 0], {"PID": 221})
    with pytest.raises(KeyError):
        ds.generate_dark_shower(ExDir=[eta])
    with pytest.raises(KeyError):
        ds.GetBSMWeights(eta, "DarkBrem")


FREE = np.load(os.path.join(GOLDEN, "dark_free.npz"))
FREE_CASES = ["e10_graphite_m0.01", "e5_lead_m0.03", "g5_lead_m0.01"]


@pytest.fixture(scope="module")
def free_showers():
    from petite_gb300.dark import DarkShower
    out = {}
    for name in FREE_CASES:
        mV, t = float(FREE[f"{name}/params"][0]), str(FREE[f"{name}/target"])
        out[name] = DarkShower(None, t, 0.010, mV, seed=SEED, bound_electron=False,
                               active_processes=["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"])
    return out


@pytest.mark.parametrize("name", FREE_CASES)
def test_free_electron_weights_match_reference(free_showers, name):
    """GetBSMWeights with bound_electron=False across the annihilation
    resonance (tabulated plus closed-form parts) and for DarkComp."""
    sh = free_showers[name]
    A, Cw = FREE[f"{name}/ann_weights"], FREE[f"{name}/comp_weights"]
    np.testing.assert_allclose([sh.GetBSMWeights([-11, e], "DarkAnn") for e in A[:, 0]], A[:, 1], rtol=1e-12, atol=0)
    np.testing.assert_allclose([sh.GetBSMWeights([22, e], "DarkComp") for e in Cw[:, 0]], Cw[:, 1], rtol=1e-12,
                               atol=0)


@pytest.mark.parametrize("name", FREE_CASES)
def test_free_electron_run_dark_matches_reference(free_showers, name):
    """pt_run_dark with free electrons on the reference's routed SM showers:
    its vectors exactly in integers, weights (the device's resonant DarkAnn
    weight included) and energies to 1e-12."""
    sh = free_showers[name]
    st, n = _store_from_golden(sh, name, FREE, name)
    res = sh._dark_engine.run_dark(sh._prm, st, n, sh._opts())
    V = FREE[f"{name}/V"]
    want = V[np.lexsort((V[:, 2], V[:, 0]))]
    proc = res["process"]
    o = np.lexsort((proc, res["parent"]))
    assert res["n"] == len(want) > 300
    assert (proc < 4).all()                          # no *_bound forms
    assert np.array_equal(res["parent"][o], want[:, 0].astype(np.int64))
    assert np.array_equal(proc[o], want[:, 2].astype(np.int64))
    assert (want[:, 2] == 1).sum() > 0               # free DarkAnn vectors present
    np.testing.assert_allclose(res["weight"][o], want[:, 3], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(res["r"][o], want[:, 8:11])
    np.testing.assert_allclose(res["p4"][o][:, 0], want[:, 4], rtol=1e-12, atol=0)
    scale = np.abs(want[:, 4:8]).max(1)
    assert (np.abs(res["p4"][o] - want[:, 4:8]).max(1) <= 1e-9 * scale).all()


def test_generate_dark_shower_reads_petite_shower_files():
    """generate_dark_shower(ExDir=path) on a shower file written by PETITE
    itself (pickled PETITE Particle objects), read without PETITE."""
    from petite_gb300.dark import DarkShower
    from petite_gb300.io import read_particle_file
    path = os.path.join(GOLDEN, "petite_shower_file.npy")
    ds = DarkShower(None, "graphite", 0.010, 0.03, seed=SEED)
    sm, vs = ds.generate_dark_shower(ExDir=path)
    assert len(sm) > 100 and len(vs) > 20
    parts = read_particle_file(path)
    for p, q in zip(parts, sm):
        p._pkey = q._pkey                     # the same streams as the first call
    _, vs2 = ds.generate_dark_shower(ExDir=parts)
    assert [v.get_ids()["parent_ID"] for v in vs] == [v.get_ids()["parent_ID"] for v in vs2]
    np.testing.assert_array_equal(np.array([v.get_p0() for v in vs]), np.array([v.get_p0() for v in vs2]))


def _record_dark(sh, p0, pid, m):
    """pt_run_sm rows of the primaries (stream offset 0), then pt_run_dark."""
    n = len(p0)
    opts = sh._opts(True, "fp64")
    opts.primary_offset = 0
    st, nr = sh._engine.run_sm(p0, np.zeros((n, 3)), np.full(n, pid, np.int32), np.full(n, m), np.ones(n), opts)
    return sh._dark_engine.run_dark(sh._prm, st, nr, sh._opts()), nr


@pytest.mark.parametrize("case", ["e10_graphite", "mu400_lead"])
def test_batched_dark_yields_match_record_rows(showers, case):
    """DarkShower.run_tallied (pt_run_batch_dark: the batched engine with dark
    vectors produced from every particle's row on each wave) against
    pt_run_sm + pt_run_dark on the same primaries and streams.  In float64
    the rows are the record engine's, so the vectors are the same ones: equal
    counts, yields equal up to the order of the atomic sums.  The mixed form
    agrees within its statistics."""
    from petite_gb300 import DarkShower
    if case == "e10_graphite":
        sh, pid, E0, m, n = showers[(0.1, "graphite")], 11, 10.0, 0.000511, 60
    else:
        sh = DarkShower(os.path.join(BUNDLED_DIR, "400GeV"), "lead", 0.010, 0.1, seed=SEED,
                        active_processes=["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"])
        pid, E0, m, n = 13, 400.0, 0.1056583755, 2
    p0 = np.tile([E0, 0.0, 0.0, math.sqrt(E0 * E0 - m * m)], (n, 1))
    rec, nr = _record_dark(sh, p0, pid, m)
    b = sh.run_tallied(p0, pid=pid, mass=m, precision="fp64", first_primary=0)
    assert b["steps"] == nr
    assert b["dark_vectors"] == rec["n"] > 100
    for k, p in enumerate(("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")):
        np.testing.assert_allclose(b["dark_yield"][p], rec["yield"][k], rtol=1e-9, atol=0)
        np.testing.assert_allclose(b["dark_yield_E"][p], rec["yield_E"][k], rtol=1e-9, atol=0)
    if case == "mu400_lead":
        assert b["dark_yield"]["DarkMuonBrem"] > 0
    # the vectors' energy histogram: the record vectors binned the same way
    edges = b["dark_energy_edges"]
    lo, hi, nb = math.log10(edges[0]), math.log10(edges[-1]), len(edges) - 1
    for k, p in enumerate(("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")):
        h = b["dark_energy_hist"][p]
        np.testing.assert_allclose(h.sum(), b["dark_yield"][p], rtol=1e-9, atol=0)
        sel = rec["process"] % 4 == k
        f = (np.log10(rec["p4"][sel, 0]) - lo) / (hi - lo)
        idx = np.clip(np.floor(np.where(f >= 0, f, 0.0) * nb).astype(int), 0, nb - 1)
        want = np.bincount(idx, weights=rec["weight"][sel], minlength=nb)
        np.testing.assert_allclose(h, want, rtol=1e-9, atol=1e-12 * max(want.sum(), 1e-300))
    mx = sh.run_tallied(p0, pid=pid, mass=m, precision="mixed", first_primary=0)
    tot_f, tot_m = sum(b["dark_yield"].values()), sum(mx["dark_yield"].values())
    print(case, "vectors", b["dark_vectors"], mx["dark_vectors"], "yield", tot_f, tot_m)
    assert abs(tot_m / tot_f - 1) < 0.05
    assert abs(mx["dark_vectors"] / b["dark_vectors"] - 1) < 0.05


def test_batched_dark_several_masses_on_one_run(showers):
    """Two dark masses on the same batched showers: each set's yields equal
    a run with that set alone."""
    a, c = showers[(0.1, "graphite")], showers[(0.3, "graphite")]
    n, m = 40, 0.000511
    p0 = np.tile([10.0, 0.0, 0.0, math.sqrt(100.0 - m * m)], (n, 1))
    import torch
    dev = a._engine.device
    ins = (torch.as_tensor(np.ascontiguousarray(p0.T), device=dev), torch.zeros((3, n), dtype=torch.float64, device=dev),
           torch.full((n,), 11, dtype=torch.int32, device=dev), torch.full((n,), m, dtype=torch.float64, device=dev))
    opts = a._opts(True, "fp64")
    both = a._dark_engine.run_batch([a._prm, c._prm], None, None, None, None, opts, a._engine.new_tally(n), 0, ins)
    one = a._dark_engine.run_batch(a._prm, None, None, None, None, opts, a._engine.new_tally(n), 0, ins)
    other = a._dark_engine.run_batch(c._prm, None, None, None, None, opts, a._engine.new_tally(n), 0, ins)
    np.testing.assert_allclose(both[1][0], one[1][0], rtol=1e-9)
    np.testing.assert_allclose(both[1][1], other[1][0], rtol=1e-9)
    assert both[3] == one[3] + other[3]
    assert not np.allclose(both[1][0], both[1][1])


@pytest.mark.parametrize("mV,target", [(0.01, "graphite"), (0.1, "lead"), (0.3, "graphite")])
def test_dark_brem_float32_screen_accuracy(showers, mV, target):
    """Where the float32 dark-brem screen returns a value, it is within
    1e-2 of the float64 cross section (the proposal loop rejects with it
    only when max_F u exceeds four times it), on map samples at every
    tabulated energy of DarkBrem and DarkMuonBrem; where it reports a point
    outside the allowed region, the float64 value is 0."""
    from petite_gb300.dark import DARK_CODE
    sh = showers[(mV, target)]
    z = sh._dark.z
    rng = np.random.default_rng(11)
    for name in ("DarkBrem", "DarkMuonBrem"):
        pre = f"m{mV}/{name}"
        E, grid, nn = z[f"{pre}/energy"], z[f"{pre}/grid"], z[f"{pre}/nnodes"]
        rows = np.repeat(np.arange(len(E)), 400)
        x = np.zeros((len(rows), 3))
        for d in range(3):
            y = rng.uniform(size=len(rows))
            ninc = nn[rows, d] - 1
            t = y * ninc
            i = np.minimum(t.astype(int), ninc - 1)
            g0, g1 = grid[rows, d, i], grid[rows, d, i + 1]
            x[:, d] = g0 + (g1 - g0) * (t - i)
        f64 = sh._dark_engine.dsigma(DARK_CODE[name], x, E[rows], mV)
        f32, code = sh._dark_engine.screen32(DARK_CODE[name], x, E[rows], mV)
        val = code == 1
        # muon samples sit mostly near cancellations the screen declines
        assert val.sum() > 100 and (name == "DarkMuonBrem" or val.mean() > 0.3), (name, val.mean())
        assert (f64[code == 2] == 0).all(), name
        rel = np.abs(f32[val] / f64[val] - 1)
        print(name, mV, target, "valued", round(val.mean(), 3), "max rel", rel.max(), "p99.9", np.quantile(rel, 0.999))
        assert rel.max() < 1e-2, (name, rel.max())


@pytest.mark.parametrize("mV", [0.01, 0.1, 0.3])
def test_radiative_return_float32_screen_accuracy(showers, mV):
    """Where the float32 radiative-return screen returns a value, it is within
    1e-3 of the float64 cross section (measured: 4e-4, the float64 form's
    own rounding; the float32 dark form decides with it only when the accept
    draw lies 0.2 % away), on map samples at every tabulated DarkAnn
    energy, u0 up to 1 - 1e-9."""
    from petite_gb300.dark import DARK_CODE
    sh = showers[(mV, "graphite")]
    z = sh._dark.z
    rng = np.random.default_rng(12)
    pre = f"m{mV}/DarkAnn"
    E, grid, nn = z[f"{pre}/energy"], z[f"{pre}/grid"], z[f"{pre}/nnodes"]
    rows = np.repeat(np.arange(len(E)), 500)
    y = np.concatenate([rng.uniform(size=len(rows) - 200), 1 - np.geomspace(1e-9, 1e-3, 200)])
    ninc = nn[rows, 0] - 1
    t = y * ninc
    i = np.minimum(t.astype(int), ninc - 1)
    g0, g1 = grid[rows, 0, i], grid[rows, 0, i + 1]
    x = (g0 + (g1 - g0) * (t - i))[:, None]
    f64 = sh._dark_engine.dsigma(DARK_CODE["DarkAnn"], x, E[rows], mV)
    f32, code = sh._dark_engine.screen32(DARK_CODE["DarkAnn"], x, E[rows], mV)
    val = (code == 1) & (f64 > 0)
    assert val.mean() > 0.9, val.mean()
    assert (code != 2).all()
    rel = np.abs(f32[val] / f64[val] - 1)
    print("DarkAnn", mV, "valued", round(val.mean(), 4), "max rel", rel.max(), "p99.9", np.quantile(rel, 0.999))
    assert rel.max() < 1e-3, rel.max()


def test_no_dark_annihilation_below_two_electron_masses():
    """mV = 0.001 GeV < 2 m_e: no DarkAnn map set, so an active DarkAnn is
    refused as PETITE refuses a process without maps (dark_shower.py:
    181-202), and the differentiable DarkAnn yield there is 0 with a 0
    gradient; DarkBrem and DarkComp run on the trained maps."""
    import torch
    from petite_gb300.dark import DarkShower, dark_yield
    with pytest.raises(Exception, match="Process String"):
        DarkShower(None, "graphite", 0.010, 0.001, seed=SEED, active_processes=["DarkBrem", "DarkAnn"])
    sh = DarkShower(None, "graphite", 0.010, 0.001, seed=SEED, active_processes=["DarkBrem", "DarkComp"])
    eng = sh._dark_engine
    E = np.array([0.5, 2.0, 8.0])
    mV = torch.tensor([0.001, 0.0012, 0.002], dtype=torch.float64, device=eng.device, requires_grad=True)
    Y, M = dark_yield(eng, "DarkAnn", E, mV, n_samples=500, seed=SEED)
    (Y.sum() + M.sum()).backward()
    assert Y.detach().cpu().numpy()[0] == 0.0 and M.detach().cpu().numpy()[0] == 0.0
    assert mV.grad.cpu().numpy()[0] == 0.0
    for proc in ("DarkBrem", "DarkComp"):
        Y, M = dark_yield(eng, proc, E, mV.detach(), n_samples=500, seed=SEED)
        assert (Y.cpu().numpy() > 0).all(), proc


def test_batched_dark_with_lanes(showers):
    """The batched dark run over three lanes (their own rings, streams and
    rows; the dark production per lane, ordered on the GPU): the vectors
    and yields of one lane."""
    sh = showers[(0.1, "graphite")]
    p0 = np.tile([10.0, 0.0, 0.0, math.sqrt(100.0 - 0.000511 ** 2)], (40, 1))
    a = sh.run_tallied(p0, pid=11, mass=0.000511, precision="fp64", first_primary=0)
    sh._engine.set_tuning((0, 0), (0, 0), "host", lanes=3)
    try:
        b = sh.run_tallied(p0, pid=11, mass=0.000511, precision="fp64", first_primary=0)
    finally:
        sh._engine.set_tuning((0, 0), (0, 0))
    assert a["steps"] == b["steps"] and a["dark_vectors"] == b["dark_vectors"] > 100
    for p in ("DarkBrem", "DarkAnn", "DarkComp"):
        np.testing.assert_allclose(b["dark_yield"][p], a["dark_yield"][p], rtol=1e-9, atol=0)
        np.testing.assert_allclose(b["dark_energy_hist"][p], a["dark_energy_hist"][p], rtol=1e-9, atol=1e-300)
