"""Single-core speed of the unmodified reference's ``Shower.generate_shower``
against the oracle port (``oracle/shower.py``) on the same primaries.

Both transport the same primaries (species uniform over e-, e+ and photons,
E0 log-uniform on [0.1, EMAX] GeV, lead, cut 0.010 GeV) with their random
numbers drawn from the same Philox streams (the reference's generators are
routed there as in ``make_golden.py``), so both make the same particles; the
script prints the particle count and particle-steps/s of each.

Runs only in the development container.  Usage:
    PETITE_REFERENCE=<PETITE checkout> python tests/golden/time_port_vs_reference.py DICT_DIR [N] [EMAX]
with DICT_DIR from ``rebuild_maps.py``.
"""
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import make_golden as mg  # noqa: E402
from oracle.philox import primary_key  # noqa: E402
from oracle.shower import OracleShower, OracleTables  # noqa: E402


def main():
    dict_dir = sys.argv[1].rstrip("/") + "/"
    n = int(sys.argv[2]) if len(sys.argv) > 2 else 20
    emax = float(sys.argv[3]) if len(sys.argv) > 3 else 100.0
    rng = np.random.default_rng(5)
    pid = np.array([11, -11, 22])[rng.integers(0, 3, n)]
    E = 10 ** rng.uniform(-1, math.log10(emax), n)
    mass = np.where(pid == 22, 0.0, 0.000511)
    target = "lead"

    orc = OracleShower(OracleTables(os.path.join(ROOT, "petite_gb300/data/sm_tables.npz"), target), 0.010,
                       seed=mg.SEED)
    t0 = time.time()
    rows_o = 0
    for j in range(n):
        p = math.sqrt(E[j] ** 2 - mass[j] ** 2)
        rows_o += len(orc.generate_shower((E[j], 0, 0, p), pid=int(pid[j]), mass=float(mass[j]), primary_index=j))
    t_o = time.time() - t0

    mg.refimport.setup()
    from PETITE.particle import Particle
    from PETITE.shower import Shower
    router = mg.StreamRouter(mg.SEED)
    sh = Shower(dict_dir, target, 0.010)
    mg.wrap_shower(sh, router)
    saved = mg.install(router)
    t0 = time.time()
    rows_r = 0
    try:
        for j in range(n):
            p = math.sqrt(E[j] ** 2 - mass[j] ** 2)
            ids = {"PID": int(pid[j])} if pid[j] == 22 else {"PID": int(pid[j]), "mass": float(mass[j])}
            part = Particle([E[j], 0.0, 0.0, p], [0.0, 0.0, 0.0], ids)
            part._pkey = primary_key(j)
            rows_r += len(sh.generate_shower(part))
    finally:
        mg.uninstall(saved)
    t_r = time.time() - t0
    print(f"{n} primaries in {target}: port {rows_o} particles in {t_o:.1f} s ({rows_o / t_o:.0f}/s); "
          f"reference {rows_r} particles in {t_r:.1f} s ({rows_r / t_r:.0f}/s); "
          f"port/reference speed {(rows_o / t_o) / (rows_r / t_r):.2f}")


if __name__ == "__main__":
    main()
