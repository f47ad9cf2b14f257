"""Pins the Bethe-Moliere multiple scattering of the oracle (fast_MCS_mode=False,
oracle/physics.py) to golden vectors produced by the reference
(tests/golden/make_golden.py, ``moliere`` mode): Moliere's b and B, the
critical angle, the inverse CDF, get_scattered_momentum_Bethe on fixed
streams, and whole showers in that mode."""
import math
import os

import numpy as np
import pytest
from scipy import special

from conftest import BUNDLED_NPZ, GOLDEN
from oracle import physics as P
from oracle.philox import Stream
from oracle.shower import OracleShower, OracleTables

G = np.load(os.path.join(GOLDEN, "moliere.npz"))
SEED = 0x5EED


def test_h_matches_exponential_integral():
    """h(x) = x e^-x (Ei(x) - ln x) - 1 against scipy's Ei where scipy is
    accurate (its large-x branch is good to ~1e-12)."""
    for x in (1e-6, 1e-3, 0.01, 0.3, 1.0, 2.5, 7.0, 15.0, 30.0, 39.9):
        ref = x * math.exp(-x) * (special.expi(x) - math.log(x)) - 1.0
        assert abs(P.moliere_h(x) - ref) <= 5e-14 * abs(ref), x
    # asymptotic branch against the series, whose hundreds of rounded terms
    # and the subtraction of 1 leave a few 1e-15 absolute; h enters the tail
    # 1 - F additively, so the absolute size is what matters
    for x in (40.1, 55.0, 99.0, 180.0):
        assert abs(P.moliere_h(x) - P.moliere_h(x, series_below=1e9)) <= 5e-15, x


def test_closed_form_cdf_is_the_integral():
    """1 - Q(x, B) equals the quadrature of the reference's density."""
    from scipy import integrate
    for B in (3.2, 7.0, 18.0):
        for x in (0.02, 0.7, 4.0, 25.0, 90.0):
            f = lambda xp: P.moliere_density(max(xp, 1e-12), B)
            q = integrate.quad(f, 0.0, x, epsabs=1e-14, epsrel=1e-13, limit=200)[0]
            assert abs((1.0 - P.moliere_tail(x, B)) - q) <= 1e-12, (B, x)


def test_inverse_cdf_root_is_accurate():
    """The Newton root of the closed-form tail against a 30-digit root of the
    same equation (mpmath's Ei)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    rng = np.random.default_rng(3)

    def tail(x, B):
        x, B = mp.mpf(x), mp.mpf(B)
        return mp.e ** (-x) * (1 + 1 / B) + (x * mp.e ** (-x) * (mp.ei(x) - mp.log(x)) - 1) / B
    n = 0
    for k in range(80):
        B = rng.uniform(3.15, 20.0)
        u = rng.uniform(0.011, 0.999) if k % 3 else 1 - 10 ** rng.uniform(-3, -0.5)
        x = P.moliere_x(u, B)
        if not 0.01 < x < 100 or 1 - u < 1 / B / 100:
            continue
        root = mp.findroot(lambda t: tail(t, B) - (1 - mp.mpf(u)), x)
        assert abs(float(root) - x) <= 1e-13 * x, (u, B)
        n += 1
    assert n > 60


def test_b_B_and_chic2_match_reference():
    for Z, A, t, beta, b, B, chic2 in G["params/rows"]:
        assert P.moliere_b(t, beta, A, int(Z)) == pytest.approx(b, rel=0, abs=1e-13 * max(1.0, abs(b)))
        if not np.isnan(B):
            # the fixed-point stop (|B - b - ln B| <= 1e-3) is reached on the same step
            assert P.moliere_B(P.moliere_b(t, beta, A, int(Z))) == pytest.approx(B, rel=1e-13)
        assert P.chic2_bethe(t, beta, A, int(Z)) == pytest.approx(chic2, rel=1e-13)


def test_inverse_cdf_matches_reference():
    """The reference's Ridder search stops at |dx| <= 2e-12 (absolute).  Rows
    flagged 'band' have u inside the step of its piecewise CDF at x = 0.01,
    where two roots exist and the search's own path decides."""
    rows = G["icdf/rows"]
    assert (rows[:, 3] == 1).sum() >= 8
    for B, u, x, band in rows:
        got = P.moliere_x(u, B)
        assert abs(got - x) <= 4e-12 + 2e-10 * x, (B, u, got, x, band)


def test_scattered_momentum_bethe_matches_reference():
    rows = G["scatter/rows"]
    n_b_small = 0
    for case, row in enumerate(rows):
        E, t, A, Z, m = row[:5]
        p4, want, used = row[5:9], row[9:13], int(row[13])
        s = Stream(SEED, 70_000 + case)
        got = P.scattered_momentum_bethe(tuple(p4), t, A, int(Z), 1.0, s.next)
        assert s.n == used, case
        n_b_small += used == 4
        pn = math.sqrt(p4[1] ** 2 + p4[2] ** 2 + p4[3] ** 2)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-9 * pn, err_msg=str(case))
    assert 0 < n_b_small < len(rows)          # both branches of generate_moliere_angle


@pytest.mark.parametrize("name", ["e1gev_graphite", "pos3_lead", "mu5_graphite"])
def test_bethe_showers_match_reference(name):
    pre = f"shower/{name}"
    F, I = G[f"{pre}/f64"], G[f"{pre}/i64"]
    seed, pid, n = (int(v) for v in G[f"{pre}/meta"])
    E0, cut, mass = G[f"{pre}/params"]
    sh = OracleShower(OracleTables(BUNDLED_NPZ, str(G[f"{pre}/target"])), cut, seed=seed, fast_MCS_mode=False)
    rows = []
    for j in range(n):
        m = 0.0 if pid == 22 else mass
        rows += sh.generate_shower((E0, 0.0, 0.0, math.sqrt(E0 * E0 - m * m)), pid=pid, primary_index=j)
    assert len(rows) == len(F)
    oi = np.array([[r.pid, r.parent_pid, r.gen, r.proc, int(r.ended), r.primary] for r in rows])
    assert np.array_equal(oi, I)
    assert np.array_equal(np.array([r.pkey for r in rows], np.uint64), G[f"{pre}/pkey"])
    assert np.array_equal(np.array([r.draws for r in rows]), G[f"{pre}/draws"])
    of = np.array([list(r.p0) + list(r.r0) + list(r.pf) + list(r.rf) + [r.weight, r.mass] for r in rows])
    np.testing.assert_allclose(of[:, [0, 7]], F[:, [0, 7]], rtol=1e-13, atol=0)
    # directions carry the inverse CDF's root tolerance (~1e-10 relative in
    # x, half that in the angle) on top of the fast mode's conditioning
    for sl in (slice(0, 4), slice(7, 11), slice(4, 7), slice(11, 14)):
        scale = np.maximum(np.abs(F[:, sl]).max(1, keepdims=True), 1e-12)
        assert (np.abs(of[:, sl] - F[:, sl]) <= 1e-7 * scale).all(), name
