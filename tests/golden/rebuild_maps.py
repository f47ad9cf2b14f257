"""Rebuild PETITE's missing ``sm_maps.pkl`` / ``dark_maps.pkl`` with PETITE's own find_maxes code.

PETITE ships the trained VEGAS maps (``data/<Process>/<Process>_AdaptiveMaps.npy``)
and ``sm_xsec.pkl`` but not ``sm_maps.pkl`` (listed as a missing large blob),
which ``Shower.__init__`` needs (``shower.py:153-162,210-215``).  This script
runs the reference's ``utilities/find_maxes.py:main`` (``find_maxes.py:121-209``)
unmodified, through the VEGAS shim in ``refshim/``, with the parameters the
reference's generation script uses (``neval=300``, ``n_trials=100``,
``generate_integrators.py:592-596``), on numpy's global generator seeded with
``--seed``.

Output directory layout (a complete PETITE ``dict_dir``):

* ``sm_maps.pkl``          -- rebuilt (new random max_F scan; the originals are lost)
* ``sm_xsec.pkl``          -- the shipped file, copied unchanged
* ``sm_xsec_rebuilt.pkl``  -- find_maxes' own sum(wgt*f) estimate, kept to pin the
                              shim's weight normalisation against the shipped table
* ``<Process>/``           -- symlinks to the shipped map directories

With ``--dark`` the same is done for the dark processes with
``find_maxes.py:main_dark`` (``find_maxes.py:212-305``) over the shipped dark
masses, writing ``dark_maps.pkl``; ``dark_xsec.pkl``, ``dark_weights.pkl`` and
``dark_drate.pkl`` are copied unchanged and find_maxes' own estimate is kept
as ``dark_xsec_rebuilt.pkl``.

Usage: python tests/golden/rebuild_maps.py OUT_DIR [--seed 20261203] [--dark]
"""
import argparse
import os
import shutil
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import refimport  # noqa: E402

SM_PROCESSES = ["PairProd", "Comp", "Ann", "Brem", "Moller", "Bhabha", "MuonE", "MuonBrem"]
DARK_PROCESSES = ["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"]
DARK_MASSES = [0.003, 0.01, 0.03, 0.1, 0.3, 1.0]      # data/<Process>/mV_<n>MeV
TARGETS = ["graphite", "lead", "iron", "aluminum", "molybdenum"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("out_dir")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--data", default="data", help="reference data directory name")
    ap.add_argument("--dark", action="store_true", help="rebuild dark_maps.pkl instead of sm_maps.pkl")
    args = ap.parse_args()
    refimport.setup()
    import find_maxes  # reference utilities/find_maxes.py, unmodified

    src = os.path.join(refimport.REFERENCE, args.data)
    out = os.path.abspath(args.out_dir)
    os.makedirs(out, exist_ok=True)
    if args.dark:
        return rebuild_dark(find_maxes, src, out, args.seed)
    for proc in SM_PROCESSES:
        link = os.path.join(out, proc)
        if not os.path.exists(link):
            os.symlink(os.path.join(src, proc), link)
    np.random.seed(args.seed)
    t0 = time.time()
    find_maxes.main({"process": list(SM_PROCESSES), "process_targets": list(TARGETS),
                     "neval": 300, "n_trials": 100, "save_location": out})
    os.replace(os.path.join(out, "sm_xsec.pkl"), os.path.join(out, "sm_xsec_rebuilt.pkl"))
    shutil.copyfile(os.path.join(src, "sm_xsec.pkl"), os.path.join(out, "sm_xsec.pkl"))
    print(f"rebuilt sm_maps.pkl in {time.time() - t0:.1f} s -> {out}")


def rebuild_dark(find_maxes, src, out, seed):
    for proc in DARK_PROCESSES:
        link = os.path.join(out, proc)
        if not os.path.exists(link):
            os.symlink(os.path.join(src, proc), link)
    np.random.seed(seed)
    t0 = time.time()
    find_maxes.main_dark({"process": list(DARK_PROCESSES), "process_targets": list(TARGETS),
                          "mV_list": list(DARK_MASSES), "mode": "MeV", "neval": 300, "n_trials": 100,
                          "save_location": out + "/"})
    os.replace(os.path.join(out, "dark_xsec.pkl"), os.path.join(out, "dark_xsec_rebuilt.pkl"))
    for f in ("dark_xsec.pkl", "dark_weights.pkl", "dark_drate.pkl"):
        shutil.copyfile(os.path.join(src, f), os.path.join(out, f))
    print(f"rebuilt dark_maps.pkl in {time.time() - t0:.1f} s -> {out}")


if __name__ == "__main__":
    main()
