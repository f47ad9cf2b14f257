"""Pins the CPU oracle to golden vectors produced by the unmodified reference.

The fixtures in tests/golden/ were written by tests/golden/make_golden.py,
which imports PETITE itself and routes its random-number call sites to the
same per-particle Philox streams the oracle and the engine use.
"""
import math
import os

import numpy as np
import pytest

from conftest import BUNDLED_NPZ, GOLDEN
from oracle import physics as P
from oracle.philox import Stream, philox4x32_10, uniforms
from oracle.shower import OracleShower, OracleTables, interp, map_point

SEED = 0x5EED
UNITS = np.load(os.path.join(GOLDEN, "units.npz"))
SHOWERS = np.load(os.path.join(GOLDEN, "showers.npz"))


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32_10
    cases = [([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
             ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
             ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
              [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1])]
    for c, k, want in cases:
        got = philox4x32_10(np.array([c], np.uint64), np.array([k], np.uint64))[0]
        assert [int(v) for v in got] == want


def test_stream_is_position_independent():
    s = Stream(7, 12345)
    seq = s.take(37)
    assert np.array_equal(seq, uniforms(7, 12345, 0, 37))
    assert np.array_equal(seq[11:30], uniforms(7, 12345, 11, 19))
    assert (seq >= 0).all() and (seq < 1).all()


def test_fma_is_correctly_rounded():
    from fractions import Fraction
    rng = np.random.default_rng(5)
    for a, b, c in rng.normal(size=(3000, 3)) * 10.0 ** rng.uniform(-6, 6, size=(3000, 3)):
        assert P.fma(a, b, c) == float(Fraction(a) * Fraction(b) + Fraction(c))


@pytest.mark.parametrize("target", ["graphite", "lead"])
@pytest.mark.parametrize("proc", ["Brem", "PairProd", "Comp", "Ann", "Moller", "Bhabha", "MuonE", "MuonBrem"])
def test_dsigma_matches_reference(target, proc):
    tab = OracleTables(BUNDLED_NPZ, target)
    X = UNITS[f"dsigma/{target}/{proc}/x"]
    E = UNITS[f"dsigma/{target}/{proc}/E"]
    V = np.nan_to_num(UNITS[f"dsigma/{target}/{proc}/value"])
    m_lep = P.m_muon if proc == "MuonBrem" else P.m_electron
    got = np.array([P.dsigma(proc, x[:P.DIM[proc]], e, tab.Z, tab.Eg_min, tab.Ee_min, m_lep) for x, e in zip(X, E)])
    assert (V != 0).sum() > 30
    np.testing.assert_allclose(got, V, rtol=1e-13, atol=0)


def test_kinematics_match_reference():
    for case, row in enumerate(UNITS["kin/rows"]):
        kind, E, x, a, b = int(row[0]), row[1], row[2:6], row[6:10], row[10:14]
        al = 2.0 * math.pi * Stream(SEED, 10_000 + case).next()
        f = {0: lambda: P.e_to_egamma(E, P.m_electron, x, al), 1: lambda: P.gamma_to_epem(E, x, al),
             2: lambda: P.compton(E, x[0], al), 3: lambda: P.annihilation(E, x[0], al),
             4: lambda: P.ee_to_ee(E, x[0], al), 5: lambda: P.mue_to_mue(E, x[0], al)}[kind]
        ra, rb = f()
        np.testing.assert_allclose(np.r_[ra, rb], np.r_[a, b], rtol=0, atol=1e-13 * E)


def test_multiple_scattering_matches_reference():
    for case, row in enumerate(UNITS["mcs/rows"]):
        E, t, A, Z, m = row[:5]
        p4, want = row[5:9], row[9:13]
        s = Stream(SEED, 20_000 + case)
        us = [s.next() for _ in range(4)]
        got = P.scattered_momentum_fast(tuple(p4), t, int(A), int(Z), 1, m, *us)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-14 * E)


def test_rotation_matrix_matches_reference():
    for row in UNITS["rot/rows"]:
        rm = np.array(P.rotation_matrix_from((10.0, *row[:3])))
        np.testing.assert_allclose(rm, row[3:].reshape(3, 3), rtol=0, atol=2e-15)


@pytest.mark.parametrize("target", ["graphite", "lead"])
def test_mfp_and_nsigma_match_reference(target):
    tab = OracleTables(BUNDLED_NPZ, target)
    sh = OracleShower(tab, 0.010)
    Es = UNITS[f"mfp/{target}/E"]
    got = np.array([[sh.mfp(pid, e) for e in Es] for pid in (11, -11, 22, 13)])
    np.testing.assert_allclose(got, UNITS[f"mfp/{target}/value"], rtol=1e-14)
    names = ("Brem", "PairProd", "Ann", "Comp", "Moller", "Bhabha", "MuonE", "MuonBrem")
    ns = np.array([[interp(e, tab.ns[n]) for e in Es] for n in names])
    np.testing.assert_allclose(ns, UNITS[f"nsigma/{target}/value"], rtol=1e-14, atol=0)


def test_interp_matches_numpy():
    rng = np.random.default_rng(3)
    xs = np.sort(rng.uniform(0, 10, 50))
    ys = rng.normal(size=50)
    q = np.r_[rng.uniform(-1, 11, 2000), xs]
    want = np.where((q < xs[0]) | (q > xs[-1]), 0.0, np.interp(q, xs, ys))
    got = np.array([interp(v, (xs.tolist(), ys.tolist())) for v in q])
    assert np.array_equal(got, want)


def test_draw_sample_matches_reference():
    tab = OracleTables(BUNDLED_NPZ, "graphite")
    sh = OracleShower(tab, 0.010)
    names = ("Brem", "PairProd", "Comp", "Ann", "Moller", "Bhabha", "MuonE")
    for row in UNITS["draw/rows"]:
        case, pi, E = int(row[0]), int(row[1]), row[2]
        count = []
        x, _ = sh.draw_sample(E, names[pi], Stream(SEED, 30_000 + case), count)
        d = P.DIM[names[pi]]
        np.testing.assert_allclose(x, row[3:3 + d], rtol=1e-15, atol=0)
        assert count[0] == int(row[7])


def test_map_weights_reproduce_shipped_cross_sections():
    """sum(wgt*f) over map samples must reproduce the shipped sm_xsec tables:
    pins the map transform and the jac/neval weight of the sampling layer.
    The shipped table rows scatter by ~1% around the current dsigma code (the
    reference's own find_maxes rebuild shows the same), so the check is on
    the mean ratio over many rows plus a loose per-row bound."""
    tab = OracleTables(BUNDLED_NPZ, "lead")
    z = np.load(BUNDLED_NPZ)
    rng = np.random.default_rng(11)
    for proc in ("Comp", "Moller", "Brem", "PairProd", "Ann"):
        xs = z[f"{proc}/xsec/lead"]
        ratios = []
        for r in range(25, 100, 6):
            if xs[r, 1] == 0:
                continue
            row = tab.maps[proc][r]
            vals = []
            for y in rng.random((3000, P.DIM[proc])):
                x, jac = map_point(row["grid"], y)
                vals.append(jac * P.dsigma(proc, x, row["E"], tab.Z, tab.Eg_min, tab.Ee_min, P.m_electron))
            ratios.append(np.mean(vals) / xs[r, 1])
        ratios = np.array(ratios)
        assert abs(ratios.mean() - 1) < 0.01, (proc, ratios)
        assert (abs(ratios - 1) < 0.06).all(), (proc, ratios)


def _oracle_showers(name):
    seed, pid, n = (int(v) for v in SHOWERS[f"{name}/meta"])
    E0, cut, mass = SHOWERS[f"{name}/params"]
    tab = OracleTables(BUNDLED_NPZ, str(SHOWERS[f"{name}/target"]))
    sh = OracleShower(tab, cut, seed=seed)
    rows = []
    for j in range(n):
        m = 0.0 if pid == 22 else mass
        rows += sh.generate_shower((E0, 0.0, 0.0, math.sqrt(E0 * E0 - m * m)), pid=pid, primary_index=j)
    return rows


# Directions and positions of charged tracks inherit the reference's own
# conditioning: the Lynch-Dahl width uses p = m*beta/sqrt(1-beta**2) with
# beta = |p|/E (moliere.py:206,218,360), which multiplies a last-place
# difference in beta by ~gamma**2, and numpy's scalar ``**`` is not correctly
# rounded.  Energies and every discrete decision do not depend on directions.
VECTOR_RTOL = {"e1gev_graphite": 2e-9, "gamma10_lead": 2e-7, "pos3_lead": 1e-7, "mu5_graphite": 1e-9}


@pytest.mark.parametrize("name", ["e1gev_graphite", "gamma10_lead", "pos3_lead", "mu5_graphite"])
def test_showers_match_reference(name):
    F, I = SHOWERS[f"{name}/f64"], SHOWERS[f"{name}/i64"]
    rows = _oracle_showers(name)
    assert len(rows) == len(F)
    oi = np.array([[r.pid, r.parent_pid, r.gen, r.proc, int(r.ended), r.primary] for r in rows])
    assert np.array_equal(oi, I)
    assert np.array_equal(np.array([r.pkey for r in rows], np.uint64), SHOWERS[f"{name}/pkey"])
    assert np.array_equal(np.array([r.draws for r in rows]), SHOWERS[f"{name}/draws"])
    of = np.array([list(r.p0) + list(r.r0) + list(r.pf) + list(r.rf) + [r.weight, r.mass] for r in rows])
    np.testing.assert_allclose(of[:, [0, 7]], F[:, [0, 7]], rtol=1e-13, atol=0)      # energies
    np.testing.assert_array_equal(of[:, 14:16], F[:, 14:16])                          # weight, mass
    for sl in (slice(0, 4), slice(7, 11)):
        scale = np.abs(F[:, sl]).max(1, keepdims=True)
        assert (np.abs(of[:, sl] - F[:, sl]) <= VECTOR_RTOL[name] * scale).all()
    for sl in (slice(4, 7), slice(11, 14)):
        scale = np.maximum(np.abs(F[:, sl]).max(1, keepdims=True), 1e-12)
        assert (np.abs(of[:, sl] - F[:, sl]) <= VECTOR_RTOL[name] * scale).all()
    # ID bookkeeping: ID = 2*parent_ID + bit (shower.py:486,494)
    ids = [tuple(int(v) for v in s.split(":")) for s in SHOWERS[f"{name}/id_str"]]
    start = 0
    for r_i, r in enumerate(rows):
        if r.parent < 0:
            start = r_i
            assert ids[r_i] == (1, -1)
        else:
            pid_ = ids[start + r.parent][0]
            assert ids[r_i] == (2 * pid_ + r.bit, pid_)
