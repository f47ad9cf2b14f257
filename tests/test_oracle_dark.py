"""Pins the dark-vector oracle (oracle/dark.py) to golden vectors produced by
the unmodified reference (tests/golden/make_golden.py, ``dark`` mode): the
dark cross sections, the dark kinematics, draw_dark_sample on fixed streams
and generate_dark_shower on routed SM showers."""
import math
import os

import numpy as np
import pytest

from conftest import BUNDLED_DIR, BUNDLED_NPZ, GOLDEN
from oracle import dark as D
from oracle import physics as P
from oracle.philox import Stream
from oracle.shower import OracleTables

G = np.load(os.path.join(GOLDEN, "dark.npz"))
DARK_NPZ = os.path.join(BUNDLED_DIR, "dark_tables.npz")
SEED = 0x5EED


@pytest.mark.parametrize("mV", [0.01, 0.1, 0.3])
@pytest.mark.parametrize("target", ["graphite", "lead"])
@pytest.mark.parametrize("proc", D.DARK_PROCESSES)
def test_dark_dsigma_matches_reference(mV, target, proc):
    pre = f"dsigma/{mV}/{target}/{proc}"
    X, E, V = G[f"{pre}/x"], G[f"{pre}/E"], G[f"{pre}/value"]
    ti = P.TARGETS[target]
    got = np.array([D.dsigma_dark(proc, x, e, mV, ti["Z_T"], ti["A_T"]) for x, e in zip(X, E)])
    assert (V != 0).sum() >= 3
    # The reference calls numpy ufuncs (np.log, np.power) on scalars; on an
    # x86 host with AVX-512 numpy evaluates them with its SIMD routines, which
    # are a few ulp from the correctly rounded libm values the oracle uses.
    # The radiative-return form raises (1-x) to beta/2-1 ~ -0.99 and divides
    # by x, which magnifies those ulp to ~1e-11 relative.
    rtol = 2e-11 if proc == "DarkAnn" else 1e-12
    np.testing.assert_allclose(got, V, rtol=rtol, atol=0)


def test_dark_kinematics_match_reference():
    rows = G["kin/rows"]
    for case, row in enumerate(rows):
        kind, mV, E = int(row[0]), row[1], row[2]
        x, extra, b = row[3:6], row[6:8], row[12:16]
        s = Stream(SEED, 50_000 + case)
        if kind in (0, 1):
            m = P.m_electron if kind == 0 else P.m_muon
            v = D.l_to_lV(E, m, x, mV, 2.0 * math.pi * s.next())[1]
        elif kind == 2:
            v = P.compton(E, x[0], 2.0 * math.pi * s.next(), mV)[1]
        elif kind == 3:
            ph = 2.0 * math.pi * s.next()
            v = D.compton_bound(E, x[0], mV, extra[0], extra[1], ph, 2.0 * math.pi * s.next())
        else:
            v = D.radiative_return_V(E, x[0], mV)
        np.testing.assert_allclose(v, b, rtol=0, atol=1e-12 * max(abs(b[0]), 1.0), err_msg=str((case, kind)))


def test_draw_dark_sample_matches_reference():
    sm = OracleTables(BUNDLED_NPZ, "graphite")
    orc = D.DarkOracle(D.DarkTables(DARK_NPZ, "graphite", 0.1), sm, SEED)
    for row in G["draw/rows"]:
        case, pi, E = int(row[0]), int(row[1]), row[2]
        proc = D.DARK_PROCESSES[pi]
        cnt = []
        x, _ = orc.draw(E, proc, Stream(SEED, 60_000 + case), cnt)
        assert cnt[0] == int(row[-1]), (proc, E)
        d = D.DARK_DIM[proc]
        np.testing.assert_allclose(x, row[3:3 + d], rtol=1e-14, atol=0)


class _Rec:
    def __init__(self, f, i, key):
        self.p0, self.r0, self.pf, self.rf = tuple(f[0:4]), tuple(f[4:7]), tuple(f[7:11]), tuple(f[11:14])
        self.weight, self.mass = f[14], f[15]
        self.pid = int(i[0])
        self.pkey = int(key)


def sm_records(name):
    F, I, K = G[f"shower/{name}/sm_f64"], G[f"shower/{name}/sm_i64"], G[f"shower/{name}/sm_pkey"]
    return [_Rec(F[k], I[k], K[k]) for k in range(len(F))]


@pytest.mark.parametrize("name", ["e10_graphite_m0.1", "e10_graphite_m0.03", "g5_lead_m0.01"])
def test_dark_shower_matches_reference(name):
    mV = float(G[f"shower/{name}/params"][0])
    target = str(G[f"shower/{name}/target"])
    sm = OracleTables(BUNDLED_NPZ, target)
    orc = D.DarkOracle(D.DarkTables(DARK_NPZ, target, mV), sm, SEED)
    recs = sm_records(name)
    W = G[f"shower/{name}/weights"]
    got_w = np.array([[orc.weight(r.pid, r.p0[0], p) for p in D.DARK_PROCESSES] for r in recs])
    np.testing.assert_allclose(got_w, W, rtol=1e-12, atol=0)
    out = orc.dark_shower(recs)
    V = G[f"shower/{name}/V"]
    got = np.array([[k, D.DARK_CODE[p], w, *v, *r] for k, p, w, v, r in out])
    want = V[np.lexsort((V[:, 2], V[:, 0]))]
    got = got[np.lexsort((got[:, 1], got[:, 0]))]
    assert len(got) == len(want)
    assert np.array_equal(got[:, :2], want[:, [0, 2]])
    np.testing.assert_allclose(got[:, 2], want[:, 3], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(got[:, 7:10], want[:, 8:11])
    # V four-momenta: energies to 1e-12; directions carry the conditioning of
    # the rotation to the lab frame and of 1 - cos(theta) near the beam axis
    np.testing.assert_allclose(got[:, 3], want[:, 4], rtol=1e-12, atol=0)
    scale = np.abs(want[:, 4:8]).max(1)
    assert (np.abs(got[:, 3:7] - want[:, 4:8]).max(1) <= 1e-9 * scale).all()


@pytest.mark.parametrize("proc", ["DarkBrem", "DarkComp", "DarkAnn"])
def test_reference_gradient_matches_finite_differences(proc):
    """The float64 forward-mode reference of the dark-yield mass derivative
    against central differences of the same estimate (h = 1e-4 relative)."""
    tabs = D.DarkTables(DARK_NPZ, "graphite", 0.1)
    for E, mV in ((20.0, 0.12), (30.0, 0.15), (90.0, 0.29)):
        gy, gm = D.dark_yield_gradient(tabs, proc, E, mV, 1, 200, SEED)
        h = 1e-4 * mV
        yp, mp = D.dark_yield_anchored(tabs, proc, E, mV + h, mV, 1, 200, SEED)
        ym, mm = D.dark_yield_anchored(tabs, proc, E, mV - h, mV, 1, 200, SEED)
        assert gy != 0.0
        assert abs(gy - (yp - ym) / (2 * h)) <= 1e-5 * abs(gy)
        assert abs(gm - (mp - mm) / (2 * h)) <= 1e-5 * abs(gm)


MESONS = np.load(os.path.join(GOLDEN, "mesons.npz"))
REF_ORDER = ("DarkBrem", "DarkAnn", "DarkComp", "TwoBody_BSMDecay", "DarkMuonBrem")   # dark_shower.py:49


class _In:
    """An input Particle of generate_dark_shower(ExDir=list): pf = p0, rf = r0."""
    def __init__(self, f, i, key):
        self.p0 = self.pf = tuple(f[0:4])
        self.r0 = self.rf = tuple(f[4:7])
        self.weight, self.mass = f[7], f[8]
        self.pid = int(i[0])
        self.pkey = int(key)


@pytest.mark.parametrize("mV", [0.01, 0.03, 0.1, 0.3])
def test_two_body_meson_decay_matches_reference(mV):
    """pi0 inputs from the reference's beam file (with photons in between)
    through generate_dark_shower: TwoBody_BSMDecay weights and V momenta."""
    pre = f"m{mV}"
    F, I, K = MESONS[f"{pre}/parts_f64"], MESONS[f"{pre}/parts_i64"], MESONS[f"{pre}/parts_pkey"]
    recs = [_In(F[k], I[k], K[k]) for k in range(len(F))]
    orc = D.DarkOracle(D.DarkTables(DARK_NPZ, "graphite", mV), OracleTables(BUNDLED_NPZ, "graphite"), SEED)
    w = np.array([orc.weight(r.pid, r.p0[0], D.TWOBODY, r.mass) for r in recs])
    np.testing.assert_allclose(w, MESONS[f"{pre}/weights"], rtol=1e-15, atol=0)
    out = orc.dark_shower(recs, processes=REF_ORDER)
    V = MESONS[f"{pre}/V"]
    assert len(out) == len(V)
    code = {"TwoBody_BSMDecay": 8, "DarkComp": 2}
    got = np.array([[k, code[p], wt, *v, *r] for k, p, wt, v, r in out])
    np.testing.assert_array_equal(got[:, :2], V[:, :2])
    np.testing.assert_allclose(got[:, 2], V[:, 2], rtol=1e-14, atol=0)
    np.testing.assert_array_equal(got[:, 7:10], V[:, 7:10])
    scale = np.abs(V[:, 3:7]).max(1)
    assert (np.abs(got[:, 3:7] - V[:, 3:7]).max(1) <= 1e-13 * scale).all()
    if mV >= 0.135:
        assert not (V[:, 1] == 8).any()          # above the pi0 mass: no decay
    else:
        assert (V[:, 1] == 8).sum() == 40


FREE = np.load(os.path.join(GOLDEN, "dark_free.npz"))
FREE_CASES = ["e10_graphite_m0.01", "e5_lead_m0.03", "g5_lead_m0.01"]


def _free_oracle(name):
    mV = float(FREE[f"{name}/params"][0])
    target = str(FREE[f"{name}/target"])
    return D.DarkOracle(D.DarkTables(DARK_NPZ, target, mV, bound_electron=False), OracleTables(BUNDLED_NPZ, target),
                        SEED)


@pytest.mark.parametrize("name", FREE_CASES)
def test_free_electron_weights_match_reference(name):
    """GetBSMWeights with bound_electron=False: DarkAnn's tabulated plus
    closed-form resonant parts across the resonance, and DarkComp over the
    free cross section."""
    orc = _free_oracle(name)
    A = FREE[f"{name}/ann_weights"]
    got = np.array([orc.weight(-11, e, "DarkAnn") for e in A[:, 0]])
    assert (A[:, 1] > 0).sum() > 20
    np.testing.assert_allclose(got, A[:, 1], rtol=1e-12, atol=0)
    Cw = FREE[f"{name}/comp_weights"]
    got = np.array([orc.weight(22, e, "DarkComp") for e in Cw[:, 0]])
    np.testing.assert_allclose(got, Cw[:, 1], rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", FREE_CASES)
def test_free_electron_dark_shower_matches_reference(name):
    orc = _free_oracle(name)
    F, I, K = FREE[f"{name}/sm_f64"], FREE[f"{name}/sm_i64"], FREE[f"{name}/sm_pkey"]
    recs = [_Rec(F[k], I[k], K[k]) for k in range(len(F))]
    out = orc.dark_shower(recs)
    V = FREE[f"{name}/V"]
    got = np.array([[k, D.DARK_CODE[p], w, *v, *r] for k, p, w, v, r in out])
    want = V[np.lexsort((V[:, 2], V[:, 0]))]
    got = got[np.lexsort((got[:, 1], got[:, 0]))]
    assert len(got) == len(want)
    assert np.array_equal(got[:, :2], want[:, [0, 2]])
    np.testing.assert_allclose(got[:, 2], want[:, 3], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(got[:, 7:10], want[:, 8:11])
    np.testing.assert_allclose(got[:, 3], want[:, 4], rtol=1e-12, atol=0)
    scale = np.abs(want[:, 4:8]).max(1)
    assert (np.abs(got[:, 3:7] - want[:, 4:8]).max(1) <= 1e-9 * scale).all()
