"""Add a dark mass that PETITE ships no maps for to the bundled dark tables.

Input: MAPS.npz, ``petite_gb300.train.build_dark_maps`` output for that mass
(all four dark processes trained on the GPU at the energies PETITE's
generation script uses, max_F and the cross section of every row from
find_maxes, five targets).  As PETITE's own pipeline would, the script adds
the mass to a private copy of the dark dict_dir: its maps to
``dark_maps.pkl`` and the find_maxes cross sections to ``dark_xsec.pkl``.
It then constructs the unmodified ``PETITE.dark_shower.DarkShower`` for the
mass on every target of the bundle (``make_dark_tables.one`` /
``one_free``: weight arrays, dR/dE tables, bound-electron cross sections,
thresholds) and merges the maps and tables into the bundle.  Runs only in
the development container.

Usage: python tests/golden/add_trained_dark_mass.py MAPS.npz DARK_DICT_DIR SM_DICT_DIR [BUNDLE.npz]
(DARK_DICT_DIR: the output of rebuild_maps.py --dark; SM_DICT_DIR: of rebuild_maps.py)
"""
import multiprocessing as mp
import os
import pickle
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)
import refimport  # noqa: E402
import make_dark_tables as mdt  # noqa: E402

PROCS = ["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"]


def main():
    maps_npz, dark_dir, sm_dir = (os.path.abspath(a) for a in sys.argv[1:4])
    bundle = sys.argv[4] if len(sys.argv) > 4 else os.path.join(ROOT, "petite_gb300", "data", "dark_tables.npz")
    refimport.setup()
    from vegas import AdaptiveMap
    from petite_gb300.tables import _MapsUnpickler
    z = np.load(maps_npz)
    ztargets = [str(t) for t in z["targets"]]
    masses = sorted({float(k.split("/")[0][1:]) for k in z.files if k.startswith("m")})
    assert len(masses) == 1, masses
    mV = masses[0]
    work = tempfile.mkdtemp(prefix="darkmass_")
    for f in os.listdir(dark_dir):
        if f not in ("dark_maps.pkl", "dark_xsec.pkl"):
            os.symlink(os.path.realpath(os.path.join(dark_dir, f)), os.path.join(work, f))
    with open(os.path.join(dark_dir, "dark_maps.pkl"), "rb") as f:
        dmaps = _MapsUnpickler(f).load()
    with open(os.path.join(dark_dir, "dark_xsec.pkl"), "rb") as f:
        dxs = pickle.load(f)
    dmaps[mV], dxs[mV] = {}, {}
    for p in PROCS:
        pre = f"m{mV}/{p}"
        E = z[f"{pre}/energy"]
        rows = []
        for i in range(len(E)):
            grid = [z[f"{pre}/grid"][i, k, :z[f"{pre}/nnodes"][i, k]] for k in range(z[f"{pre}/grid"].shape[1])]
            rows.append([float(E[i]), {"neval": int(z[f"{pre}/neval"][i]),
                                       "max_F": {t: float(z[f"{pre}/max_F"][i, j]) for j, t in enumerate(ztargets)},
                                       "adaptive_map": AdaptiveMap(grid)}])
        dmaps[mV][p] = rows
        dxs[mV][p] = {t: [[float(E[i]), float(z[f"{pre}/xsec"][i, j])] for i in range(len(E))]
                      for j, t in enumerate(ztargets)}
    with open(os.path.join(work, "dark_maps.pkl"), "wb") as f:
        pickle.dump(dmaps, f)
    with open(os.path.join(work, "dark_xsec.pkl"), "wb") as f:
        pickle.dump(dxs, f)

    res = dict(np.load(bundle))
    targets = [str(t) for t in res["targets"]]
    cols = [ztargets.index(t) for t in targets]
    for p in PROCS:
        pre = f"m{mV}/{p}"
        for k in ("energy", "neval", "grid", "nnodes"):
            res[f"{pre}/{k}"] = z[f"{pre}/{k}"]
        res[f"{pre}/max_F"] = z[f"{pre}/max_F"][:, cols]
    jobs = [(work, sm_dir, mV, t) for t in targets]
    with mp.get_context("spawn").Pool(min(2 * len(jobs), os.cpu_count() or 1)) as pool:
        bound = pool.map_async(mdt.one, jobs)
        free = pool.map_async(mdt.one_free, jobs)
        for m, t, out in bound.get():
            for k, v in out.items():
                res[f"m{m}/{t}/{k}"] = v
        for m, t, out, ii in free.get():
            for k, v in out.items():
                res[f"m{m}/{t}/{k}"] = v
    res["masses"] = np.array(sorted(set(float(m) for m in res["masses"]) | {mV}))
    np.savez_compressed(bundle, **res)
    shutil.rmtree(work, ignore_errors=True)
    print("added mV =", mV, "to", bundle, os.path.getsize(bundle) // 1024, "KB; masses", list(res["masses"]))


if __name__ == "__main__":
    main()
