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
