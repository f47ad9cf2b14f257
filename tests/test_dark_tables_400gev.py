"""The bundled 400 GeV dark tables (data/400GeV/dark_tables.npz, written by
tests/golden/make_dark_tables_400GeV.py from maps built by
petite_gb300.train.build_dark_maps): layout, coverage and agreement of the
trained maps' find_maxes cross sections with PETITE's dark_xsec.pkl rows."""
import os

import numpy as np

from conftest import BUNDLED_DIR, GOLDEN
from petite_gb300.dark import DarkData

PATH = os.path.join(BUNDLED_DIR, "400GeV", "dark_tables.npz")


def test_layout_and_coverage():
    d = DarkData(PATH)
    assert d.masses == [0.1] and d.targets == ["graphite", "lead", "iron", "aluminum", "molybdenum"]
    m = d.maps_for("lead", 1.0)
    rows = m["rows"][0]
    assert list(rows[:4]) == [150, 150, 150, 150]
    E = m["energy"]
    for p in (0, 3):                                     # DarkBrem, DarkMuonBrem reach 400 GeV
        b = m["base"][0, p]
        assert abs(E[b + rows[p] - 1] - 400.0) < 1e-9
        assert (m["maxF"][b:b + rows[p]] > 0).all()
    ninc = m["ninc"].reshape(-1, 4)
    assert (ninc[m["base"][0, 3]:m["base"][0, 3] + 150, :3] == 1000).all()
    prm = d.params_for(0.1, "lead")
    for k in ("brem_elec", "brem_positron", "ann", "muon_brem"):
        assert prm[f"w/{k}"].shape[1] == 2 and len(prm[f"dr/{k}/Ei"]) > 10
    assert prm["w/muon_brem"][:, 0].max() > 300.0
    free = d.params_for(0.1, "lead", bound_electron=False)
    assert free["ann_E0"] > 0


def test_oracle_reads_the_tables():
    from oracle import dark as D
    t = D.DarkTables(PATH, "lead", 0.1)
    assert t.mV == 0.1 and len(t.maps["DarkMuonBrem"]) == 150


def test_trained_cross_sections_match_petite_rows():
    z = np.load(PATH)
    dx = np.load(os.path.join(GOLDEN, "dark_xsec_400GeV.npz"))
    targets = list(z["targets"])
    for p in ("DarkBrem", "DarkMuonBrem"):
        ref = dx[f"{p}/lead"]
        E = z[f"m0.1/{p}/energy"]
        idx = [int(np.argmin(np.abs(E - e))) for e in ref[:, 0]]
        assert np.allclose(E[idx], ref[:, 0], rtol=1e-12)
        # max_F only is bundled (the cross sections come from PETITE's table);
        # its scale follows the cross section: max_F * neval above the mean
        mf = z[f"m0.1/{p}/max_F"][idx, targets.index("lead")]
        assert (mf * 300 > ref[:, 1]).all()


def test_trained_mass_in_the_10gev_bundle():
    """mV = 0.05 GeV, which PETITE ships no maps for: maps trained at the
    energies of PETITE's generation script (petite_gb300.train.dark_energies,
    which reproduces the shipped masses' energies exactly), tables on every
    target."""
    from petite_gb300.train import dark_energies
    d = DarkData(os.path.join(BUNDLED_DIR, "dark_tables.npz"))
    assert 0.05 in d.masses and len(d.targets) == 5
    for p in ("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"):
        for mV in (0.03, 0.05):
            np.testing.assert_allclose(d.z[f"m{mV}/{p}/energy"], dark_energies(p, mV), rtol=1e-14)
        assert (d.z[f"m0.05/{p}/max_F"] > 0).all()
    for t in d.targets:
        prm = d.params_for(0.05, t)
        assert prm["w/brem_elec"][:, 1].max() > 0 and prm["E_res"] > 0
