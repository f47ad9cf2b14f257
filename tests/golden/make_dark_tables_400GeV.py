"""Bundle the 400 GeV dark-shower tables (petite_gb300/data/400GeV/dark_tables.npz).

PETITE's ``data_400GeV`` ships ``dark_xsec.pkl`` and the DarkAnn/DarkComp maps
but not the DarkBrem/DarkMuonBrem maps, ``dark_maps.pkl`` or ``sm_maps.pkl``.
Inputs:

* MAPS.npz -- ``petite_gb300.train.build_dark_maps`` output for one mass
  (trained DarkBrem/DarkMuonBrem maps, shipped DarkAnn/DarkComp maps, max_F
  from find_maxes, all on the GPU);
* the bundled ``petite_gb300/data/400GeV/sm_tables.npz`` (SM maps, max_F and
  ``sm_xsec.pkl``).

The script writes both as PETITE pickles (``dark_maps.pkl``, ``sm_maps.pkl``)
into a private dict_dir next to the shipped ``sm_xsec.pkl`` and
``dark_xsec.pkl``, constructs the unmodified ``PETITE.dark_shower.DarkShower``
there for each target (``make_dark_tables.one`` / ``one_free``: the weight
arrays, dR/dE tables, bound-electron cross sections and thresholds, as PETITE
computes them), and bundles the maps with those tables in the layout of
``dark_tables.npz``.  Runs only in the development container.

Usage: python tests/golden/make_dark_tables_400GeV.py MAPS.npz [--targets graphite lead ...] [OUT.npz]
"""
import argparse
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

DATA_400 = os.path.join(refimport.REFERENCE, "data_400GeV")
PROCS = ["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"]


def write_dict_dir(maps_npz, work):
    refimport.setup()
    from vegas import AdaptiveMap
    from petite_gb300 import tables as T
    z = np.load(maps_npz)
    targets = [str(t) for t in z["targets"]]
    masses = sorted({float(k.split("/")[0][1:]) for k in z.files if k.startswith("m")})
    dark = {}
    for mV in masses:
        dark[mV] = {}
        for p in PROCS:
            pre = f"m{mV}/{p}"
            rows = []
            for i, E in enumerate(z[f"{pre}/energy"]):
                grid = [z[f"{pre}/grid"][i, k, :z[f"{pre}/nnodes"][i, k]] for k in range(z[f"{pre}/grid"].shape[1])]
                rows.append([float(E), {"neval": int(z[f"{pre}/neval"][i]),
                                        "max_F": {t: float(z[f"{pre}/max_F"][i, j]) for j, t in enumerate(targets)},
                                        "adaptive_map": AdaptiveMap(grid)}])
            dark[mV][p] = rows
    with open(os.path.join(work, "dark_maps.pkl"), "wb") as f:
        pickle.dump(dark, f)
    raw = T.load_npz(os.path.join(ROOT, "petite_gb300", "data", "400GeV", "sm_tables.npz"))
    sm = {}
    for p, rows in raw.maps.items():
        out = []
        for r in rows:
            info = {"neval": r.neval, "max_F": dict(r.max_F), "adaptive_map": AdaptiveMap(r.grid)}
            if r.Eg_min is not None:
                info["Eg_min"] = r.Eg_min
            if r.Ee_min is not None:
                info["Ee_min"] = r.Ee_min
            out.append([r.energy, info])
        sm[p] = out
    with open(os.path.join(work, "sm_maps.pkl"), "wb") as f:
        pickle.dump(sm, f)
    for name in ("sm_xsec.pkl", "dark_xsec.pkl"):
        shutil.copyfile(os.path.join(DATA_400, name), os.path.join(work, name))
    return masses, z


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("maps_npz")
    ap.add_argument("out", nargs="?", default=os.path.join(ROOT, "petite_gb300", "data", "400GeV", "dark_tables.npz"))
    ap.add_argument("--targets", nargs="+", default=["graphite", "lead", "iron", "aluminum", "molybdenum"])
    a = ap.parse_args()
    work = tempfile.mkdtemp(prefix="dark400_")
    masses, z = write_dict_dir(os.path.abspath(a.maps_npz), work)
    ztargets = [str(t) for t in z["targets"]]
    cols = [ztargets.index(t) for t in a.targets]
    res = {"masses": np.array(masses), "targets": np.array(a.targets)}
    for mV in masses:
        for p in PROCS:
            pre = f"m{mV}/{p}"
            for k in ("energy", "neval", "grid", "nnodes"):
                res[f"{pre}/{k}"] = z[f"{pre}/{k}"]
            res[f"{pre}/max_F"] = z[f"{pre}/max_F"][:, cols]
    # dark and SM parts of the dict_dir are the same private directory
    jobs = [(work, work, mV, t) for mV in masses for t in a.targets]
    with mp.get_context("spawn").Pool(min(2 * len(jobs), os.cpu_count() or 1)) as pool:
        bound = pool.map_async(mdt.one, jobs)
        free = pool.map_async(mdt.one_free, jobs)
        for mV, t, out in bound.get():
            for k, v in out.items():
                res[f"m{mV}/{t}/{k}"] = v
        for mV, t, out, ii in free.get():
            for k, v in out.items():
                res[f"m{mV}/{t}/{k}"] = v
            for k, v in ii.items():
                res[f"{t}/{k}"] = v
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    np.savez_compressed(a.out, **res)
    shutil.rmtree(work, ignore_errors=True)
    print("wrote", a.out, os.path.getsize(a.out) // 1024, "KB")


if __name__ == "__main__":
    main()
