"""Generate the CPU side of the independent-stream spectrum comparison.

Runs the oracle's ``generate_shower`` (oracle/shower.py, pinned draw for draw
to the unmodified PETITE reference by tests/test_oracle_golden.py) on the
primaries of each workload in ``tests/spectra.py:CONFIGS`` and stores, per
shower: the particle count, the deposited energy (continuous dE/dx loss, the
energy of daughters at or below the cut, and the energy of particles that
end without an interaction, as the batched engine's tally counts it), the
primary's energy and PID, and the coarse per-shower histograms of creation
energy, polar angle and interaction depth.

Usage: python tests/golden/make_spectra.py [--procs N] [--workloads a,b]   (writes tests/golden/spectra.npz)
"""
import argparse
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import spectra  # noqa: E402

_SH = {}


def _shower(target, seed):
    key = (target, seed)
    if key not in _SH:
        from oracle.shower import OracleShower, OracleTables
        t = OracleTables(os.path.join(ROOT, "petite_gb300", "data", "sm_tables.npz"), target)
        _SH[key] = OracleShower(t, spectra.MIN_ENERGY, seed=seed)
    return _SH[key]


def one(args):
    """One CPU shower: (count, edep, coarse histograms)."""
    target, seed, z_max, i, p0, pid, mass = args
    sh = _shower(target, seed)
    interacted = set()
    below = [0.0]
    orig = sh.sample_scattering

    def tracked(r, process, s, index):
        kids = orig(r, process, s, index)
        if kids is None:
            return None
        interacted.add(index)
        for k in kids:
            if not k.p0[0] > sh.min_energy:
                below[0] += k.p0[0]
        return kids

    sh.sample_scattering = tracked
    try:
        rows = sh.generate_shower(p0, pid=int(pid), mass=float(mass), primary_index=int(i))
    finally:
        sh.sample_scattering = orig
    edep = below[0]
    for k, r in enumerate(rows):
        edep += r.p0[0] - r.pf[0]
        if k not in interacted:            # no interaction: its energy stays here
            edep += r.pf[0]
    P0 = np.array([r.p0 for r in rows])
    z = np.array([r.rf[2] for r in rows])
    h = spectra.coarse_shower_hist(np.array([r.pid for r in rows]), P0[:, 0], P0[:, 1], P0[:, 2], P0[:, 3], z,
                                   z_max)
    return len(rows), edep, h


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--procs", type=int, default=os.cpu_count())
    ap.add_argument("--out", default=os.path.join(HERE, "spectra.npz"))
    ap.add_argument("--workloads", default=",".join(spectra.CONFIGS),
                    help="workloads to make; the others are kept from an existing output file")
    a = ap.parse_args()
    out = {}
    if os.path.exists(a.out):
        old = np.load(a.out)
        out = {k: old[k] for k in old.files}
    ctx = mp.get_context("spawn")
    with ctx.Pool(a.procs) as pool:
        for name, cfg in spectra.CONFIGS.items():
            if name not in a.workloads.split(","):
                continue
            t0 = time.time()
            p0, pid, m = spectra.primaries(cfg)
            # largest showers first, so the pool's tail is short
            order = np.argsort(-p0[:, 0], kind="stable")
            jobs = [(cfg["target"], cfg["cpu_seed"], cfg["z_max"], int(i), p0[i], pid[i], m[i]) for i in order]
            res = pool.map(one, jobs, chunksize=1)
            n = len(p0)
            mult = np.zeros(n, np.int32)
            edep = np.zeros(n)
            hist = np.zeros((n, 3, 3, spectra.NCOARSE), np.uint16)
            for i, (c, e, h) in zip(order, res):
                mult[i], edep[i] = c, e
                assert h.max() < 65536
                hist[i] = h
            out[f"{name}/mult"] = mult
            out[f"{name}/edep"] = edep
            out[f"{name}/E0"] = p0[:, 0]
            out[f"{name}/pid"] = pid
            out[f"{name}/hist"] = hist
            print(f"{name}: {n} showers, {mult.sum()} particles, {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(a.out, **out)


if __name__ == "__main__":
    main()
