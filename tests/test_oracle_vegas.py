"""Properties of the VEGAS map adaptation restated in oracle/vegas_train.py
(the vegas package itself is not installed)."""
import numpy as np

from oracle.vegas_train import adapt


def test_flat_weight_keeps_a_uniform_grid():
    g = np.linspace(0.0, 2.0, 101)
    out = adapt(g, np.ones(100), np.full(100, 7))
    np.testing.assert_allclose(out, g, rtol=0, atol=1e-12)


def test_no_information_keeps_the_grid():
    g = np.linspace(-1.0, 1.0, 51)
    np.testing.assert_array_equal(adapt(g, np.zeros(50), np.zeros(50, int)), g)


def test_nodes_move_toward_the_weight():
    g = np.linspace(0.0, 1.0, 201)
    x = 0.5 * (g[1:] + g[:-1])
    w = np.exp(-((x - 0.3) / 0.02) ** 2) + 1e-6
    out = adapt(g, w, np.ones(200, int))
    width = np.diff(out)
    assert np.all(width > 0)
    assert out[0] == 0.0 and out[-1] == 1.0
    # finer increments near the peak than far from it (one damped step,
    # alpha = 0.5, moves the nodes part of the way)
    assert width[np.searchsorted(out, 0.3) - 1] < 0.5 * width[-1]


def test_compressed_weights_are_shared_equally():
    g = np.linspace(0.0, 1.0, 11)
    w = np.array([1, 1, 1, 1, 100, 100, 1, 1, 1, 1], float)
    out = adapt(g, w, np.ones(10, int), alpha=0.0)      # alpha = 0: every nonzero increment weighs 1
    np.testing.assert_allclose(out, g, atol=1e-12)


def test_find_maxes_restatement_matches_the_reference():
    """oracle.vegas_train.find_maxes_row against the reference's own
    do_find_max_work on shipped Comp and Brem map rows, both drawing from
    the same seeded generator (tests/golden/findmax.npz)."""
    import os
    from conftest import GOLDEN
    from oracle import physics as P
    from oracle.vegas_train import find_maxes_row
    z = np.load(os.path.join(GOLDEN, "findmax.npz"))
    seed = int(z["seed"])
    Z = {"graphite": 6, "lead": 82}
    me = 0.0005109989499999999
    n = 0
    for key in sorted({k.rsplit("/", 1)[0] for k in z.files if k.count("/") == 2}):
        proc, row = key.split("/")
        E, Eg, Ee = float(z[f"{key}/E"]), float(z[f"{key}/Eg_min"]), float(z[f"{key}/Ee_min"])
        grids = [z[f"{key}/grid{d}"] for d in range(4) if f"{key}/grid{d}" in z]
        fs = {t: (lambda x, zt=Z[t]: P.dsigma(proc, x, E, zt, Eg, Ee, me)) for t in ("graphite", "lead")}
        mx, xs = find_maxes_row(grids, fs, 300, 3, np.random.default_rng(seed + int(row)).random)
        np.testing.assert_allclose([mx["graphite"], mx["lead"]], z[f"{key}/max_F"], rtol=1e-10)
        np.testing.assert_allclose([xs["graphite"], xs["lead"]], z[f"{key}/xsec"], rtol=1e-10)
        n += 1
    assert n == 5


def test_integration_ranges_match_the_reference():
    """petite_gb300.train.integration_range against PETITE's own
    integration_range for every process the table builder trains
    (tests/golden/ranges.npz)."""
    import os
    from conftest import GOLDEN
    from petite_gb300.train import integration_range
    z = np.load(os.path.join(GOLDEN, "ranges.npz"))
    for p, E, mV, want in zip(z["process"], z["E"], z["mV"], z["ranges"]):
        got = np.asarray(integration_range(str(p), float(E), mV=float(mV)), float).ravel()
        w = want[~np.isnan(want)]
        np.testing.assert_allclose(got, w, rtol=1e-15, atol=0, err_msg=f"{p} {E} {mV}")
