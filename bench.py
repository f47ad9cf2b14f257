#!/usr/bin/env python
"""Throughput of the shower transport path on one GB300 (or N, one rank each).

A step transports one batch of primaries of the selected workload to the end
of their showers.  The metric is particle-steps/s: one particle-step is one
visit of a live particle in the transport loop (propagation with all its
substeps, process choice and the sampled interaction), i.e. one row of
PETITE's output list.  Every step uses fresh random streams (primary index
offset by the step number).

Prints one JSON line (rank 0).  ``--impl reference`` times the CPU oracle
(a restatement of PETITE's transport loop) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300: batched mixed-precision vs plain FP64 GPU, matched spectra"

WORKLOADS = {
    # 1,000 electrons at 1 GeV along +z in graphite, cut 0.010 GeV, float64 throughout
    "sm_e1gev_graphite_1k": dict(target="graphite", cut=0.010, n=1000, species=(11,), emin=1.0, emax=1.0,
                                 seed=0, precision="fp64"),
}

# algorithmic HBM bytes per particle-step of the float64 record engine:
# read the live row (p0 32, r0 24, pid 4, mass 8, pkey 8, weight 8, gen 4,
# primary 4, live index 8 = 100), write its final state (pf 32, rf 24,
# draws 4 = 60) and write the one row it creates on average (176).
BYTES_PER_STEP = 336


def make_primaries(w, n, offset):
    rng = np.random.default_rng(1_000_003 * (offset + 1) + w["seed"])
    species = np.asarray(w["species"])
    pid = species[rng.integers(0, len(species), n)] if len(species) > 1 else np.full(n, species[0])
    if w["emin"] == w["emax"]:
        E = np.full(n, w["emin"])
    else:
        E = 10 ** rng.uniform(math.log10(w["emin"]), math.log10(w["emax"]), n)
    m = np.where(np.abs(pid) == 11, 0.000511, np.where(np.abs(pid) == 13, 0.1056583755, 0.0))
    p0 = np.c_[E, np.zeros(n), np.zeros(n), np.sqrt(E * E - m * m)]
    return p0, pid.astype(np.int32), m


class ClockSampler:
    """nvidia-smi clocks/throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except Exception:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle_worker(args):
    """Runs the oracle on a slice of primaries (spawned process)."""
    sys.path.insert(0, ROOT)
    from oracle.shower import OracleShower, OracleTables
    target, cut, seed, p0, pid, mass, first = args
    npz = os.path.join(ROOT, "petite_gb300", "data", "sm_tables.npz")
    sh = OracleShower(OracleTables(npz, target), cut, seed=seed)
    rows = 0
    for i in range(len(p0)):
        rows += len(sh.generate_shower(tuple(p0[i]), pid=int(pid[i]), mass=float(mass[i]), primary_index=first + i))
    return rows


def cpu_baseline(w, n_sample, cores=None):
    import multiprocessing as mp
    cores = cores or os.cpu_count()
    p0, pid, m = make_primaries(w, n_sample, offset=10_000)
    chunks = np.array_split(np.arange(n_sample), cores * 4)
    jobs = [(w["target"], w["cut"], w["seed"], p0[c], pid[c], m[c], int(c[0]) if len(c) else 0) for c in chunks if len(c)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        rows = sum(pool.map(cpu_oracle_worker, jobs))
    dt = time.perf_counter() - t0
    return {"value": rows / dt, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": f"{n_sample} primaries of the workload ({rows} particle-steps) in {dt:.1f} s, "
                      f"oracle (CPU restatement of PETITE's loop) over {cores} spawned processes"}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        return dist, rank, ws
    return None, 0, 1


def run_reference(args, w, name):
    dist, rank, ws = dist_setup()
    if rank != 0:
        return
    n_sample = args.cpu_sample
    vals = []
    for _ in range(args.warmup if args.warmup < 1 else 1):
        pass
    for s in range(args.steps):
        cb = cpu_baseline(w, n_sample)
        vals.append(cb["value"])
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": name, "target": w["target"], "cut_GeV": w["cut"], "primaries_per_step": n_sample},
            "cpu_baseline": {**cb, "value": v},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sm_e1gev_graphite_1k", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-sample", type=int, default=400)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w, args.workload)

    import torch
    dist, rank, ws = dist_setup()
    from petite_gb300 import Shower
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    sh = Shower(None, w["target"], w["cut"], seed=w["seed"], precision=w["precision"], device=dev)
    eng = sh._engine
    opts = sh._opts(True, w["precision"])
    n = w["n"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # > 129 MB L2

    def one_step(step):
        p0, pid, m = make_primaries(w, n, offset=step * ws + rank)
        opts.primary_offset = (step * ws + rank) * n
        st, rows = eng.run_sm(p0, np.zeros((n, 3)), pid, m, np.ones(n), opts)
        return st, rows

    for s in range(args.warmup):
        one_step(1000 + s)
    # device-timed steps (inputs resident: the primaries are staged before the timer starts)
    times, rows_tot, launches = [], 0, 0
    with ClockSampler(dev.index or 0) as clk:
        for s in range(args.steps):
            flush.zero_()
            p0, pid, m = make_primaries(w, n, offset=s * ws + rank)
            opts.primary_offset = (s * ws + rank) * n
            from petite_gb300.engine import ParticleStore
            cap = int(np.sum(2.0 * p0[:, 0] / w["cut"]) + 16 * n)
            st = ParticleStore(cap, dev)
            st.t["p0"][:, :n] = torch.as_tensor(p0.T, device=dev)
            st.t["pid"][:n] = torch.as_tensor(pid, device=dev)
            st.t["mass"][:n] = torch.as_tensor(m, device=dev)
            st.t["weight"][:n] = 1.0
            abi = st.abi()
            import ctypes as C
            nrows = C.c_int64()
            if dist:
                dist.barrier()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            stream = torch.cuda.current_stream(dev)
            e0.record(stream)
            status = eng.lib.pt_run_sm(eng.handle, C.byref(abi), n, C.byref(opts), C.byref(nrows),
                                       C.c_void_p(stream.cuda_stream))
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if status != 0:
                raise RuntimeError(f"pt_run_sm status {status}")
            times.append(e0.elapsed_time(e1) / 1e3)
            rows_tot += nrows.value
            launches += eng.last_run_stats()[0]
    t_local = float(sum(times))
    rows_local = rows_tot
    if dist:
        t = torch.tensor([t_local], device=dev)
        r = torch.tensor([rows_local], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(r, op=dist.ReduceOp.SUM)
        t_max, rows_all = float(t.item()), float(r.item())
    else:
        t_max, rows_all = t_local, float(rows_local)
    value = rows_all / t_max

    # end-to-end through the public API: host primaries in, host records out
    e2e_rows, e2e_t, h2d, d2h = 0, 0.0, 0, 0
    for s in range(args.steps):
        p0, pid, m = make_primaries(w, n, offset=500 + s * ws + rank)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        b = sh.generate_showers(p0, pid=pid, mass=m, precision=w["precision"], first_primary=(500 + s * ws + rank) * n)
        torch.cuda.synchronize(dev)
        e2e_t += time.perf_counter() - t0
        e2e_rows += b.n
        h2d += p0.nbytes + pid.nbytes + m.nbytes + 8 * n + 24 * n
        d2h += b.n * (16 * 8 + 6 * 4 + 2 * 8)
    e2e = {"value": e2e_rows / e2e_t, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d // args.steps,
           "d2h_bytes_per_step": d2h // args.steps}

    if rank != 0:
        return
    achieved = rows_all * BYTES_PER_STEP / t_max / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    cb = None
    if not args.no_cpu_baseline:
        cb = cpu_baseline(w, args.cpu_sample)
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if w["precision"] == "fp64" else "f32+f64",
        "data": "synthetic",
        "config": {"workload": args.workload, "target": w["target"], "cut_GeV": w["cut"],
                   "primaries_per_step": n, "precision": w["precision"], "l2": "flushed (256 MB write) before each step",
                   "parallelism": f"replicas{ws}"},
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"},
        "cpu_baseline": cb,
        "clocks": clk.summary(),
        "particle_steps": rows_all,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
