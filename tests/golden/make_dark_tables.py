"""Bundle PETITE's dark-shower tables as plain arrays (petite_gb300/data/dark_tables.npz).

Runs only in the development container: it imports the unmodified reference
(``refimport``) and constructs ``PETITE.dark_shower.DarkShower`` for each dark
mass and target, which is how PETITE itself produces its per-mass tables
(``dark_shower.py:69-130``): the track-length weight arrays
(``set_weight_arrays``, :401-452), the dR/dE interaction-energy tables
(``set_drate_dE``, :535-593), the bound-electron cross sections
(``set_DarkAnnXSec``/``set_DarkCompXSec``, :254-284) and the thresholds.
The arrays are read back from the constructed object.  The VEGAS maps and
max_F come from ``dark_maps.pkl`` rebuilt by ``rebuild_maps.py --dark``.

Usage: python tests/golden/make_dark_tables.py DARK_DICT_DIR SM_DICT_DIR [OUT.npz]
       python tests/golden/make_dark_tables.py --add-free DARK_DICT_DIR SM_DICT_DIR [OUT.npz]
(every target of PETITE's find_maxes: graphite, lead, iron, aluminum, molybdenum)
(SM_DICT_DIR: the output of rebuild_maps.py, which DarkShower's Shower base reads)
"""
import multiprocessing as mp
import os
import shutil
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import refimport  # noqa: E402

MASSES = [0.003, 0.01, 0.03, 0.1, 0.3]
TARGETS = ["graphite", "lead", "iron", "aluminum", "molybdenum"]
PROCS = ["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"]
DRATE = {"brem_elec": "_d_rate_dict_elec_brem", "brem_positron": "_d_rate_dict_positron_brem",
         "ann": "_d_rate_dict_positron_ann", "muon_brem": "_d_rate_dict_muon_brem"}
WEIGHTS = {"brem_elec": "_brem_elec_numerical_weight", "brem_positron": "_brem_positron_numerical_weight",
           "ann": "_annihilation_numerical_weight", "muon_brem": "_muon_brem_numerical_weight"}


def one(args):
    dict_dir, sm_dir, mV, target = args
    refimport.setup()
    from PETITE.dark_shower import DarkShower
    # private copy: the constructor writes its caches into dict_dir
    work = tempfile.mkdtemp(prefix="dark_")
    for f in os.listdir(dict_dir):
        src = os.path.join(dict_dir, f)
        if f.endswith(".pkl") and f != "dark_maps.pkl":
            shutil.copyfile(src, os.path.join(work, f))
        else:
            os.symlink(os.path.realpath(src), os.path.join(work, f))
    for f in os.listdir(sm_dir):
        if not os.path.exists(os.path.join(work, f)):
            os.symlink(os.path.realpath(os.path.join(sm_dir, f)), os.path.join(work, f))
    t0 = time.time()
    sh = DarkShower(work + "/", target, 0.010, mV, active_processes=list(PROCS))
    out = {"mV": np.array(sh._mV), "E_res": np.array(sh._resonant_annihilation_energy),
           "E_compth": np.array(sh._compton_threshold_energy)}
    out["xsec/DarkBrem"] = np.asarray(sh.get_DarkBremXSec(), float)
    out["xsec/DarkMuonBrem"] = np.asarray(sh.get_DarkMuonBremXSec(), float)
    out["xsec/DarkAnn_bound"] = np.asarray(sh.get_DarkAnnXSec(), float)
    out["xsec/DarkComp_bound"] = np.asarray(sh.get_DarkCompXSec(), float)
    for name, attr in WEIGHTS.items():
        f = getattr(sh, attr)
        out[f"weights/{name}"] = np.c_[np.asarray(f.x, float), np.asarray(f.y, float)]
    for name, attr in DRATE.items():
        d = getattr(sh, attr)
        Ei = np.array(sorted(d.keys()), float)
        bins = [np.asarray(d[e], float) for e in Ei]
        nb = max(len(b) for b in bins)
        arr = np.zeros((len(Ei), nb, 2))
        cnt = np.zeros(len(Ei), np.int32)
        for i, b in enumerate(bins):
            arr[i, :len(b)] = b
            cnt[i] = len(b)
        out[f"drate/{name}/Ei"] = Ei
        out[f"drate/{name}/bins"] = arr
        out[f"drate/{name}/nbins"] = cnt
    mc = sh._minimum_calculable_dark_energy
    out["min_dark"] = np.array([mc[11]["DarkBrem"], mc[-11]["DarkBrem"], mc[-11]["DarkAnn"], mc[22]["DarkComp"],
                                mc[13]["DarkMuonBrem"]])
    shutil.rmtree(work, ignore_errors=True)
    print(f"mV={mV} {target}: {time.time() - t0:.0f} s", flush=True)
    return mV, target, out


def one_free(args):
    """The free-electron tables (DarkShower(bound_electron=False)): the
    DarkAnn/DarkComp cross sections of dark_xsec.pkl, the annihilation weights
    and dR/dE with the resonant bin (dark_shower.py:382-400,495-517), the
    thresholds, and the positron interaction integrals (shower.py:296-314)
    behind the analytic resonant weight (dark_shower.py:621-629).  The private
    directory has no dark_weights.pkl or dark_drate.pkl: with a cached entry
    for the mass and target, set_drate_dE indexes a float with a string
    (dark_shower.py:550) and raises TypeError in this mode."""
    dict_dir, sm_dir, mV, target = args
    refimport.setup()
    from PETITE.dark_shower import DarkShower
    work = tempfile.mkdtemp(prefix="darkfree_")
    for d in (dict_dir, sm_dir):
        for f in os.listdir(d):
            if f in ("dark_weights.pkl", "dark_drate.pkl") or os.path.exists(os.path.join(work, f)):
                continue
            os.symlink(os.path.realpath(os.path.join(d, f)), os.path.join(work, f))
    t0 = time.time()
    sh = DarkShower(work + "/", target, 0.010, mV, active_processes=list(PROCS), bound_electron=False)
    out = {"free/xsec/DarkAnn": np.asarray(sh.get_DarkAnnXSec(), float),
           "free/xsec/DarkComp": np.asarray(sh.get_DarkCompXSec(), float)}
    f = sh._annihilation_numerical_weight
    out["free/weights/ann"] = np.c_[np.asarray(f.x, float), np.asarray(f.y, float)]
    d = sh._d_rate_dict_positron_ann
    Ei = np.array(sorted(d.keys()), float)
    bins = [np.asarray(d[e], float).reshape(-1, 2) for e in Ei]
    nb = max(len(b) for b in bins)
    arr = np.zeros((len(Ei), nb, 2))
    cnt = np.zeros(len(Ei), np.int32)
    for i, b in enumerate(bins):
        arr[i, :len(b)] = b
        cnt[i] = len(b)
    out["free/drate/ann/Ei"], out["free/drate/ann/bins"], out["free/drate/ann/nbins"] = Ei, arr, cnt
    mc = sh._minimum_calculable_dark_energy
    out["free/min_dark"] = np.array([mc[11]["DarkBrem"], mc[-11]["DarkBrem"], mc[-11]["DarkAnn"], mc[22]["DarkComp"],
                                     mc[13]["DarkMuonBrem"]])
    ii = {}
    for name in ("Brem", "Ann", "Bhabha"):
        g = getattr(sh, f"_interaction_integral_{name}")
        ii[f"ii/{name}"] = np.c_[np.asarray(g.x, float), np.asarray(g.y, float)]
    shutil.rmtree(work, ignore_errors=True)
    print(f"free mV={mV} {target}: {time.time() - t0:.0f} s", flush=True)
    return mV, target, out, ii


def add_free(dict_dir, sm_dir, path):
    """Adds the free-electron tables to an existing bundle."""
    res = dict(np.load(path))
    jobs = [(dict_dir, sm_dir, mV, t) for mV in MASSES for t in TARGETS]
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        for mV, t, out, ii in pool.imap_unordered(one_free, jobs):
            for k, v in out.items():
                res[f"m{mV}/{t}/{k}"] = v
            for k, v in ii.items():
                res[f"{t}/{k}"] = v
    np.savez_compressed(path, **res)
    print("wrote", path, os.path.getsize(path) // 1024, "KB")


def main():
    if sys.argv[1] == "--add-free":
        refimport.setup()
        add_free(os.path.abspath(sys.argv[2]), os.path.abspath(sys.argv[3]), sys.argv[4] if len(sys.argv) > 4 else
                 os.path.join(os.path.dirname(os.path.dirname(HERE)), "petite_gb300", "data", "dark_tables.npz"))
        return
    dict_dir = os.path.abspath(sys.argv[1])
    sm_dir = os.path.abspath(sys.argv[2])
    out_path = sys.argv[3] if len(sys.argv) > 3 else os.path.join(
        os.path.dirname(os.path.dirname(HERE)), "petite_gb300", "data", "dark_tables.npz")
    refimport.setup()
    from petite_gb300.tables import _MapsUnpickler
    with open(os.path.join(dict_dir, "dark_maps.pkl"), "rb") as f:
        maps = _MapsUnpickler(f).load()
    res = {"masses": np.array(MASSES), "targets": np.array(TARGETS)}
    for mV in MASSES:
        key = [k for k in maps if abs(float(k) - mV) < 1e-12][0]
        for p in PROCS:
            rows = maps[key][p]
            d = len(rows[0][1]["adaptive_map"].grid)
            nmax = max(len(g) for r in rows for g in r[1]["adaptive_map"].grid)
            grid = np.zeros((len(rows), d, nmax))
            nn = np.zeros((len(rows), d), np.int32)
            for i, (E, info) in enumerate(rows):
                for k, g in enumerate(info["adaptive_map"].grid):
                    grid[i, k, :len(g)] = g
                    nn[i, k] = len(g)
            pre = f"m{mV}/{p}"
            res[f"{pre}/energy"] = np.array([float(r[0]) for r in rows])
            res[f"{pre}/neval"] = np.array([int(r[1]["neval"]) for r in rows])
            res[f"{pre}/max_F"] = np.array([[float(r[1]["max_F"][t]) for t in TARGETS] for r in rows])
            res[f"{pre}/grid"] = grid
            res[f"{pre}/nnodes"] = nn
    jobs = [(dict_dir, sm_dir, mV, t) for mV in MASSES for t in TARGETS]
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        for mV, t, out in pool.imap_unordered(one, jobs):
            for k, v in out.items():
                res[f"m{mV}/{t}/{k}"] = v
    np.savez_compressed(out_path, **res)
    print("wrote", out_path, os.path.getsize(out_path) // 1024, "KB")
    add_free(dict_dir, sm_dir, out_path)


if __name__ == "__main__":
    main()
