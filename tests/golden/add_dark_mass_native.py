"""Add a dark mass to the bundled dark tables without the reference.

    python tests/golden/add_dark_mass_native.py train MASS MAPS.npz     (on a GPU)
    python tests/golden/add_dark_mass_native.py bundle MAPS.npz [BUNDLE.npz]

``train`` trains the mass's dark maps on the GPU (``petite_gb300.train.
build_dark_maps``: PETITE's generation-script energies, find_maxes for max_F
and the cross sections of every row, five targets; DarkAnn is left out
below mV = 2 m_e) into MAPS.npz.  ``bundle`` adds them to the bundle with
the weight, dR/dE and bound-electron tables that PETITE's DarkShower
constructor would derive from those maps and cross sections
(``petite_gb300.darktables.bundle_mass``, on the bundled SM tables).
mV = 0.001 GeV was added this way.
"""
import os
import pickle
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    cmd = sys.argv[1]
    if cmd == "train":
        from petite_gb300 import train
        mV, out = float(sys.argv[2]), sys.argv[3]
        d = tempfile.mkdtemp(prefix="darkmass_")
        with open(os.path.join(d, "dark_xsec.pkl"), "wb") as f:
            pickle.dump({}, f)                 # a mass PETITE has no rows for
        print(train.build_dark_maps(d, out, mV))
    elif cmd == "bundle":
        from petite_gb300 import darktables
        data = os.path.join(ROOT, "petite_gb300", "data")
        bundle = sys.argv[3] if len(sys.argv) > 3 else os.path.join(data, "dark_tables.npz")
        print(darktables.bundle_mass(sys.argv[2], bundle, os.path.join(data, "sm_tables.npz")))
    else:
        raise SystemExit(__doc__)


if __name__ == "__main__":
    main()
