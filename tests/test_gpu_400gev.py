"""The 400 GeV tables (PETITE's data_400GeV cross sections and maps, with the
Brem, PairProd and MuonBrem maps trained by petite_gb300.train): the engine
against the oracle on the same tables, draw for draw, for a 400 GeV muon and
a 30 GeV electron in lead (a 400 GeV muon leaves ~4e4 particles, ~50 s in the
oracle)."""
import math
import os

import numpy as np
import pytest

from conftest import BUNDLED_DIR
from test_gpu_parity import _compare_showers

pytestmark = pytest.mark.gpu

SEED = 3
TABLES = os.path.join(BUNDLED_DIR, "400GeV")


@pytest.mark.parametrize("pid,E0,mass,n", [(13, 400.0, 0.1056583755, 1), (11, 30.0, 0.000511, 1)])
def test_400gev_showers_match_oracle(pid, E0, mass, n):
    from oracle.shower import OracleShower, OracleTables
    from petite_gb300 import Shower
    sh = Shower(TABLES, "lead", 0.010, seed=SEED)
    p = math.sqrt(E0 * E0 - mass * mass)
    batch = sh.generate_showers(np.tile([E0, 0.0, 0.0, p], (n, 1)), pid=pid, mass=mass, first_primary=0)
    orc = OracleShower(OracleTables(os.path.join(TABLES, "sm_tables.npz"), "lead"), 0.010, seed=SEED)
    rows = []
    for j in range(n):
        rows += orc.generate_shower((E0, 0.0, 0.0, p), pid=pid, mass=mass, primary_index=j)
    worst = _compare_showers(batch, rows, 1e-6)
    print(pid, E0, "rows", batch.n, "worst", worst)
    assert batch.n > 200


def test_400gev_dark_muon_brem_matches_oracle():
    """Dark vectors (mV = 0.1 GeV) on a 400 GeV muon's shower in lead with the
    400 GeV dark tables (DarkBrem and DarkMuonBrem maps trained by
    petite_gb300.train): pt_run_dark against the oracle's
    produce_bsm_particle on the same rows and streams, for the muon's rows and
    every 50th other row."""
    from oracle import dark as D
    from oracle.shower import OracleTables
    from petite_gb300 import DarkShower
    sh = DarkShower(TABLES, "lead", 0.010, 0.1, seed=SEED)
    mmu = 0.1056583755
    p = math.sqrt(400.0 ** 2 - mmu ** 2)
    opts = sh._opts(True, "fp64")
    st, nr = sh._engine.run_sm(np.array([[400.0, 0, 0, p]]), np.zeros((1, 3)), np.array([13], np.int32),
                               np.array([mmu]), np.ones(1), opts)
    res = sh._dark_engine.run_dark(sh._prm, st, nr, sh._opts())
    rows = st.to_numpy(nr)
    keep = np.flatnonzero((np.abs(rows["pid"]) == 13) | (np.arange(nr) % 50 == 0))

    class R:
        pass
    recs = []
    for k in keep:
        r = R()
        r.p0, r.pf, r.rf = tuple(rows["p0"][k]), tuple(rows["pf"][k]), tuple(rows["rf"][k])
        r.pid, r.mass, r.weight, r.pkey = int(rows["pid"][k]), float(rows["mass"][k]), 1.0, int(rows["pkey"][k])
        recs.append(r)
    orc = D.DarkOracle(D.DarkTables(os.path.join(TABLES, "dark_tables.npz"), "lead", 0.1),
                       OracleTables(os.path.join(TABLES, "sm_tables.npz"), "lead"), SEED)
    out = orc.dark_shower(recs, processes=("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"))
    want = np.array([[keep[k], D.DARK_CODE[pp], w, *v] for k, pp, w, v, _ in out])
    want = want[np.lexsort((want[:, 1], want[:, 0]))]
    sel = np.isin(res["parent"], keep)
    proc = res["process"][sel] % 4
    par = res["parent"][sel]
    o = np.lexsort((proc, par))
    assert len(o) == len(want) > 50
    assert (want[:, 1] == D.DARK_CODE["DarkMuonBrem"]).sum() > 20
    assert np.array_equal(par[o], want[:, 0].astype(np.int64))
    assert np.array_equal(proc[o], want[:, 1].astype(np.int64))
    np.testing.assert_allclose(res["weight"][sel][o], want[:, 2], rtol=1e-12, atol=0)
    np.testing.assert_allclose(res["p4"][sel][o], want[:, 3:7], rtol=1e-9, atol=1e-12)
