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
