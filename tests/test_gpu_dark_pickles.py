"""DarkShower on a PETITE dict_dir that holds dark_maps.pkl and
dark_xsec.pkl (no dark_tables.npz): its tables are built natively
(``petite_gb300.darktables``) and its dark vectors are those of the
DarkShower on the bundled tables, which PETITE's constructor made."""
import math
import os

import numpy as np
import pytest

from conftest import BUNDLED_DIR
import darkpickles

pytestmark = pytest.mark.gpu

SEED = 0x5EED
PROCS = ["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"]


@pytest.fixture(scope="module")
def pickle_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("petite_dark")
    return darkpickles.write_dict_dir(os.path.join(BUNDLED_DIR, "dark_tables.npz"), str(d), masses=[0.01, 0.1],
                                      targets=["graphite", "lead"],
                                      sm_npz=os.path.join(BUNDLED_DIR, "sm_tables.npz"))


@pytest.mark.parametrize("mV,target,bound", [(0.1, "lead", True), (0.01, "graphite", True),
                                             (0.1, "graphite", False)])
def test_pickle_dict_dir_makes_the_bundled_vectors(pickle_dir, mV, target, bound):
    from petite_gb300.dark import DarkShower
    sh = {name: DarkShower(d, target, 0.010, mV, seed=SEED, active_processes=PROCS, bound_electron=bound)
          for name, d in (("pickles", pickle_dir), ("bundled", None))}
    assert sh["pickles"]._mV_list == [0.01, 0.1]
    # one set of SM rows (the record engine's row order is not fixed) for both
    n = 20
    p = math.sqrt(100.0 - 0.000511 ** 2)
    opts = sh["bundled"]._opts(True, "fp64")
    opts.primary_offset = 5
    st, nr = sh["bundled"]._engine.run_sm(np.tile([10.0, 0, 0, p], (n, 1)), np.zeros((n, 3)),
                                          np.full(n, 11, np.int32), np.full(n, 0.000511), np.ones(n), opts)
    out = {k: (s_._dark_engine.run_dark(s_._prm, st, nr, s_._opts()), nr) for k, s_ in sh.items()}
    (a, na), (b, nb) = out["pickles"], out["bundled"]
    assert na == nb and a["n"] == b["n"] > 50
    oa, ob = np.lexsort((a["process"], a["parent"])), np.lexsort((b["process"], b["parent"]))
    assert np.array_equal(a["parent"][oa], b["parent"][ob])
    assert np.array_equal(a["process"][oa], b["process"][ob])
    # The bundled tables may have been made on another machine family: where
    # PETITE's closed forms of the bound-electron cross sections cancel
    # (small values) a last-digit libm change moves the tables, by up to
    # ~1e-5 relative for DarkAnn weights 1e-7 of the largest, and wholly for
    # DarkComp weights 1e-10 of it; the weights that count, the yields and
    # the vectors agree.
    wa, wb = a["weight"][oa], b["weight"][ob]
    big = wb > 1e-6 * wb.max()
    np.testing.assert_allclose(wa[big], wb[big], rtol=1e-5, atol=0)
    np.testing.assert_allclose(a["yield"], b["yield"], rtol=1e-7, atol=0)
    same = np.all(np.isclose(a["p4"][oa], b["p4"][ob], rtol=1e-9, atol=1e-12), axis=1)
    assert same.mean() >= 0.999, same.mean()
