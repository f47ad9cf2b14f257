"""The native dark-table build (``petite_gb300.darktables``) against the
tables PETITE's own DarkShower constructor made (the bundled
``dark_tables.npz`` files, written by ``tests/golden/make_dark_tables.py``
from the constructed reference objects), and DarkShower's reading of a
PETITE dict_dir's dark pickles (CPU only: no engine is made)."""
import os
import platform

import numpy as np
import pytest

from conftest import BUNDLED_DIR
import darkpickles

B10 = os.path.join(BUNDLED_DIR, "dark_tables.npz")
B400 = os.path.join(BUNDLED_DIR, "400GeV", "dark_tables.npz")
SM10 = os.path.join(BUNDLED_DIR, "sm_tables.npz")
SM400 = os.path.join(BUNDLED_DIR, "400GeV", "sm_tables.npz")
# (0.03, graphite) and (0.03, molybdenum) came from PETITE's shipped
# dark_weights.pkl / dark_drate.pkl caches, which its constructor reads back
# instead of integrating; the others were integrated by the constructor.
CASES = [(B10, SM10, 0.003, "lead"), (B10, SM10, 0.01, "aluminum"), (B10, SM10, 0.1, "graphite"),
         (B10, SM10, 0.3, "molybdenum"), (B10, SM10, 0.05, "iron"), (B400, SM400, 0.1, "iron")]

CANCELLING = ("xsec/DarkAnn_bound", "xsec/DarkComp_bound", "weights/ann", "drate/ann/bins")


def _xsec_from_bundle(z, mV, t):
    pre = f"m{mV}/{t}"
    return {"DarkBrem": {t: z[f"{pre}/xsec/DarkBrem"]}, "DarkMuonBrem": {t: z[f"{pre}/xsec/DarkMuonBrem"]},
            "DarkAnn": {t: z[f"{pre}/free/xsec/DarkAnn"]}, "DarkComp": {t: z[f"{pre}/free/xsec/DarkComp"]}}


_sm = {}


def _sm_tables(path, target):
    from petite_gb300 import tables as T
    if path not in _sm:
        _sm[path] = T.load_npz(path)
    return T.SMTables(_sm[path], target)


@pytest.mark.parametrize("bundle,smz,mV,target", CASES)
def test_builder_reproduces_petite_constructor_tables(bundle, smz, mV, target):
    """Every array PETITE's constructor derives (bound-electron cross
    sections, thresholds, weights, dR/dE in both electron modes, interaction
    integrals) from the same dark_xsec rows and SM tables: equal to rounding.
    The integrals go through the same quad calls on the same integrands, so
    quad's truncation error (up to 1e-3 here) is PETITE's own."""
    from petite_gb300 import darktables as DT
    z = np.load(bundle)
    b = DT.DarkTableBuilder(_sm_tables(smz, target), _xsec_from_bundle(z, mV, target), target, mV)
    got = b.npz_entries(mV)
    assert set(got) == {k for k in z.files if k.startswith(f"m{mV}/{target}/") or k.startswith(f"{target}/ii/")}
    for k, v in got.items():
        ref = z[k]
        assert v.shape == ref.shape, k
        if ref.dtype.kind in "iu":
            assert np.array_equal(v, ref), k
        elif platform.machine() == "x86_64":
            # the machine family the bundled tables were made on
            np.testing.assert_allclose(v, ref, rtol=1e-12, atol=0, err_msg=k)
        elif k.endswith(CANCELLING):
            # PETITE's closed forms of the bound-electron cross sections
            # cancel strongly where they are small, so a last-digit change of
            # a libm function moves those entries; the others stay put
            big = np.abs(ref) > 1e-9 * np.abs(ref).max()
            np.testing.assert_allclose(v[big], ref[big], rtol=1e-6, atol=0, err_msg=k)
        else:
            np.testing.assert_allclose(v, ref, rtol=1e-9, atol=0, err_msg=k)


def test_interaction_integrals_carry_quads_error():
    """The SM interaction integrals are quad's values, not the exact
    integrals of the piecewise-linear n*sigma (which differ by up to ~1e-3)."""
    from petite_gb300 import darktables as DT
    z = np.load(B10)
    sm = _sm_tables(SM10, "graphite")
    s = DT.Survival(sm)
    for name in ("Brem", "Ann", "Bhabha"):
        ii = s.ii(name)
        np.testing.assert_array_equal(np.column_stack((ii.x, ii.y)), z[f"graphite/ii/{name}"])
    x, y = sm.nsigma[0]
    exact = np.concatenate([[0.0], np.cumsum(0.5 * np.diff(x) * (y[1:] + y[:-1]))])
    assert np.max(np.abs(exact - s.ii("Brem").y) / np.maximum(exact, 1e-300)) > 1e-6


def test_interpolants_match_scipy():
    from scipy.interpolate import interp1d
    from petite_gb300 import darktables as DT
    rng = np.random.default_rng(3)
    x = np.sort(rng.uniform(0.01, 10.0, 40))
    y = rng.uniform(0.0, 5.0, 40)
    f, g = DT.Linear(x, y), interp1d(x, y, fill_value=0.0, bounds_error=False)
    for E in np.concatenate([rng.uniform(0.0, 11.0, 500), x, [x[0], x[-1]]]):
        assert f(float(E)) == float(g(E))
    h = DT.LogLog(x, y * 1e-10)
    lg = interp1d(np.log10(x + 1e-20), np.log10(y * 1e-10 + 1e-20), fill_value=-20.0, bounds_error=False)
    for E in rng.uniform(0.005, 12.0, 500):
        assert h(float(E)) == pytest.approx(float(10 ** lg(np.log10(E))), rel=1e-15)


@pytest.fixture(scope="module")
def pickle_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("petite_dark")
    return darkpickles.write_dict_dir(B10, str(d), masses=[0.01, 0.1], targets=["graphite", "lead"], sm_npz=SM10)


def test_pickled_dict_dir_gives_the_bundled_tables(pickle_dir):
    """DarkData.from_pickles on a dict_dir holding only PETITE's
    dark_maps.pkl, dark_xsec.pkl (and the SM tables): its masses, maps and
    per-(mass, target) tables are the bundled ones."""
    from petite_gb300 import tables as T
    from petite_gb300.dark import DarkData
    raw = T.load_npz(SM10)
    dp = DarkData.from_pickles(pickle_dir, lambda t: T.SMTables(raw, t))
    db = DarkData(B10)
    assert dp.masses == [0.01, 0.1] and sorted(dp.targets) == ["graphite", "lead"]
    mp = dp.maps_for("lead", 1.0)
    mb = db.maps_for("lead", 1.0)
    sel = np.concatenate([np.arange(mb["base"][m, p], mb["base"][m, p] + mb["rows"][m, p])
                          for m in (db.masses.index(0.01), db.masses.index(0.1)) for p in range(4)])
    np.testing.assert_array_equal(mp["energy"], mb["energy"][sel])
    np.testing.assert_array_equal(mp["maxF"], mb["maxF"][sel])
    for mV in (0.01, 0.1):
        for bound in (True, False):
            a, b = dp.params_for(mV, "lead", bound), db.params_for(mV, "lead", bound)
            assert set(a) == set(b)
            for k in a:
                np.testing.assert_allclose(a[k], b[k], rtol=1e-12, atol=0, err_msg=f"{mV} {bound} {k}")


def test_caches_are_read_like_petite(tmp_path):
    """A dark_weights.pkl / dark_drate.pkl entry for the (mass, target) is
    used as PETITE uses it (dark_shower.py:401-593): the brem and muon-brem
    tables come from the cache, the bound-electron annihilation tables are
    recomputed."""
    from petite_gb300 import tables as T
    from petite_gb300.darktables import PickleTables
    z = np.load(B10)
    pre = "m0.1/graphite"
    w = {k: z[f"{pre}/{n}"] * np.array([1.0, 2.0]) for k, n in
         (("brem_elec_weights", "weights/brem_elec"), ("brem_positron_weights", "weights/brem_positron"),
          ("muon_brem_weights", "weights/muon_brem"), ("annihilation_weights", "free/weights/ann"))}
    dr = {}
    for key, n in (("brem_elec_drate", "brem_elec"), ("brem_positron_drate", "brem_positron"),
                   ("muon_brem_drate", "muon_brem")):
        Ei, bins, nb = (z[f"{pre}/drate/{n}/{s}"] for s in ("Ei", "bins", "nbins"))
        dr[key] = {np.float64(e): bins[i, :nb[i]] * np.array([1.0, 3.0]) for i, e in enumerate(Ei)}
    d = darkpickles.write_dict_dir(B10, str(tmp_path), masses=[0.1], targets=["graphite"],
                                   weights_cache={np.float64(0.1): {"graphite": w}},
                                   drate_cache={np.float64(0.1): {"graphite": dr}})
    raw = T.load_npz(SM10)
    pt = PickleTables(d, lambda t: T.SMTables(raw, t))
    np.testing.assert_array_equal(pt[f"{pre}/weights/brem_elec"][:, 1], 2.0 * z[f"{pre}/weights/brem_elec"][:, 1])
    np.testing.assert_array_equal(pt[f"{pre}/drate/muon_brem/bins"][..., 1], 3.0 * z[f"{pre}/drate/muon_brem/bins"][..., 1])
    np.testing.assert_allclose(pt[f"{pre}/weights/ann"], z[f"{pre}/weights/ann"], rtol=1e-12)
    np.testing.assert_allclose(pt[f"{pre}/drate/ann/bins"], z[f"{pre}/drate/ann/bins"], rtol=1e-12)
    np.testing.assert_array_equal(pt[f"{pre}/free/weights/ann"][:, 1], 2.0 * z[f"{pre}/free/weights/ann"][:, 1])


def test_missing_process_or_target_raises():
    from petite_gb300.darktables import DarkTableBuilder
    z = np.load(B10)
    sm = _sm_tables(SM10, "graphite")
    xs = _xsec_from_bundle(z, 0.1, "graphite")
    with pytest.raises(Exception, match="Target Material"):
        DarkTableBuilder(sm, {p: {"lead": v["graphite"]} for p, v in xs.items()}, "graphite", 0.1)
    del xs["DarkComp"]
    with pytest.raises(Exception, match="Process String"):
        DarkTableBuilder(sm, xs, "graphite", 0.1)


def test_approx_mode_thresholds_use_the_actual_mass(pickle_dir):
    """mode='approx' (dark_shower.py:167-176): the maps and dark_xsec rows of
    the closest lesser trained mass, the thresholds and bound-electron cross
    sections of the requested mass (dark_shower.py:232-233, 263, 283)."""
    from petite_gb300 import tables as T
    from petite_gb300.dark import DarkData
    raw = T.load_npz(SM10)
    dp = DarkData.from_pickles(pickle_dir, lambda t: T.SMTables(raw, t))
    dp.use_mass(0.02)
    d = dp.params_for(0.01, "graphite", True)
    me = T.M_ELECTRON
    assert d["E_res"] == (0.02 ** 2 - 2 * me ** 2) / (2 * me)
    assert d["E_compth"] == 0.02 ** 2 / (2 * me) + 0.02
    np.testing.assert_allclose(d["min_dark"][2:4], [d["E_res"] / 1000.0, d["E_compth"] / 1000.0], rtol=0)


def test_bundled_mass_below_two_electron_masses():
    """mV = 0.001 GeV (trained maps, natively built tables): DarkBrem,
    DarkComp and DarkMuonBrem maps on all five targets, no DarkAnn maps and
    no free-electron tables (no resonance below 2 m_e); the device map
    arrays give DarkAnn no rows there."""
    from petite_gb300.dark import DarkData
    d = DarkData(B10)
    assert d.masses[0] == 0.001
    z = d.z
    for p in ("DarkBrem", "DarkComp", "DarkMuonBrem"):
        assert len(z[f"m0.001/{p}/energy"]) == 100
        assert np.isfinite(z[f"m0.001/{p}/max_F"]).all()
    assert "m0.001/DarkAnn/energy" not in z
    for t in d.targets:
        assert f"m0.001/{t}/free/xsec/DarkAnn" not in z
        w = z[f"m0.001/{t}/weights/brem_elec"]
        assert (w[:, 1] >= 0).all() and w[-1, 1] > 0
    mp = d.maps_for("graphite", 1.0)
    assert mp["rows"][0, 1] == 0 and (mp["rows"][0, [0, 2, 3]] == 100).all()
    with pytest.raises(Exception, match="Process String"):
        d.params_for(0.001, "graphite", False)
    assert d.params_for(0.001, "graphite", True)["E_res"] < 0.000511
