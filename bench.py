#!/usr/bin/env python
"""Throughput of the shower transport path on one GB300 (or N, one rank each).

Headline workload (default): batched SM showers -- 10^6 primaries, species
uniform over {e-, e+, gamma}, E0 log-uniform on [0.1, 100] GeV along +z, lead,
energy cut 0.010 GeV, seed 1 -- transported by the mixed-precision engine
(float32 sampling and scattering, float64 energies).  A step transports one
such batch to the end of every shower; each step uses fresh random streams
(primary indices offset by the step number).

Metric: particle-steps/s.  One particle-step is one visit of a live particle
in the transport loop (propagation with its substeps, process choice and the
sampled interaction), i.e. one row of PETITE's output list.

The same line carries the plain float64 engine on a same-stream subsample
(and the matched-spectra statistics between the two), the roofline figures,
the end-to-end figure through Shower.run_tallied (pinned host inputs in, host
tallies out) and the CPU oracle baseline.  ``--impl reference`` times the CPU
oracle (a restatement of PETITE's transport loop) alone on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from petite_gb300.replicas import block_index, first_primary, reduce_job  # noqa: E402

METRIC = "particle-steps/s on 1 GB300: batched mixed-precision vs plain FP64 GPU, matched spectra"

WORKLOADS = {
    "sm_batched_lead_1M": dict(target="lead", cut=0.010, n=1_000_000, species=(11, -11, 22), emin=0.1, emax=100.0,
                               seed=1, precision="mixed", fp64_sample=20_000, cpu_sample=160, mode="batch"),
    "sm_e1gev_graphite_1k": dict(target="graphite", cut=0.010, n=1000, species=(11,), emin=1.0, emax=1.0,
                                 seed=0, precision="fp64", fp64_sample=1000, cpu_sample=400, mode="records"),
    # dark vectors on SM showers: 10^5 e- at 10 GeV in graphite, cut 0.010 GeV,
    # dark masses {0.001, 0.01, 0.05, 0.1, 0.3} GeV (0.001 and 0.05: maps
    # trained by petite_gb300.train; PETITE ships the others; no DarkAnn at
    # 0.001, below 2 m_e)
    "dark_e10_graphite_1e5": dict(target="graphite", cut=0.010, n=100_000, species=(11,), emin=10.0, emax=10.0,
                                  seed=0, masses=(0.001, 0.01, 0.05, 0.1, 0.3), chunk=10_000, mode="dark",
                                  dark_precision="mixed"),
    # 10^5 mu- at 400 GeV in lead, cut 0.010 GeV, seed 3 (the SM transport of
    # the 400 GeV muon configuration): tables with PETITE's data_400GeV cross
    # sections, its shipped maps and Brem/PairProd/MuonBrem maps trained by
    # petite_gb300.train (PETITE ships none above 100 GeV)
    "sm_mu400_lead_1e5": dict(target="lead", cut=0.010, n=100_000, species=(13,), emin=400.0, emax=400.0,
                              seed=3, precision="mixed", fp64_sample=1000, cpu_sample=1, mode="batch",
                              tables="400GeV"),
    # the dark part of the 400 GeV muon configuration: mu- at 400 GeV in lead,
    # cut 0.010 GeV, seed 3, mV = 0.1 GeV, DarkMuonBrem on the muon and
    # DarkBrem/DarkAnn/DarkComp on its cascade, on the 400 GeV dark tables
    # (DarkBrem/DarkMuonBrem maps trained by petite_gb300.train); 10^3 of the
    # configuration's 10^5 primaries per step (4.4e7 SM rows), in one chunk:
    # the record engine runs a generation per launch, and a muon's line is
    # hundreds of generations deep
    "dark_mu400_lead_1e3": dict(target="lead", cut=0.010, n=1000, species=(13,), emin=400.0, emax=400.0,
                                seed=3, masses=(0.1,), chunk=1000, mode="dark", tables="400GeV",
                                dark_processes=("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")),
    # the same two dark configurations on the batched engine
    # (pt_run_batch_dark): the showers are not stored, every wave's particles
    # go through the dark production, all masses on one run (mixed precision)
    "batchdark_e10_graphite_2e4": dict(target="graphite", cut=0.010, n=20_000, species=(11,), emin=10.0, emax=10.0,
                                       seed=0, masses=(0.001, 0.01, 0.05, 0.1, 0.3), mode="batchdark",
                                       precision="mixed",
                                       dark_processes=("DarkBrem", "DarkAnn", "DarkComp"), dark_precision="mixed"),
    "batchdark_mu400_lead_1e3": dict(target="lead", cut=0.010, n=1000, species=(13,), emin=400.0, emax=400.0,
                                     seed=3, masses=(0.1,), mode="batchdark", precision="mixed", tables="400GeV",
                                     dark_processes=("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"),
                                     dark_precision="mixed"),
    # detector acceptance (detector_cut, shower.py:825-865) of 10^8 dark-vector
    # rows: E log-uniform on [0.1, 30] GeV, polar angle log-uniform on
    # [1e-4, 0.3] rad, production points spread 1 cm transversely over 1 m
    # of target, weights uniform on [0.1, 2]; disks at z = 5, 50, 100 m,
    # radius 1 m around a 5 cm hole, energy window (1, 20) GeV
    # (a step is 100 passes over the rows, so the timed region is long enough
    # for the clock samples)
    "detector_cut_1e8": dict(n=100_000_000, seed=0, z=(5.0, 50.0, 100.0), radius=1.0, inner=0.05,
                             energy_cut=(1.0, 20.0), cpu_sample=20_000_000, passes=100, mode="detector"),
    # differentiable dark yield: 4096 (E, mV) pairs, E log-uniform on [0.05, 10] GeV,
    # mV log-uniform on [0.001, 0.3] GeV, 10^4 map samples each, graphite
    "dark_yield_4096": dict(target="graphite", n=4096, samples=10_000, seed=0, mode="yield"),
}

# Algorithmic HBM bytes of the batched engine's two kernels, per unit of work.
# The ring is a structure of arrays (E and key 8 B; momentum, position and
# mass 8 B in the float64 form and 4 B in the mixed form, where E also has a
# 4 B float copy; pid, primary and generation 4 B each).  A particle that
# interacts is parked as one task record (64 B mixed, 96 B float64) in a
# chunk of 32 records of its process, plus a 4-byte chunk-list entry per
# chunk.  Tables (maps, n*sigma) are L2-resident and not counted.
#   propagation, per particle-step: read E, p, r, mass, key, pid, primary
#     (and the float copy of E); per sampled particle: write its task record
#     (reading the generation it carries).
#   sampler, per sampled particle: read its task record; per pushed
#     daughter: write E, p, r, mass, key, pid, primary, generation.
def ring_bytes(precision):
    f = 8 if precision == "fp64" else 4
    rec = 96 if precision == "fp64" else 64
    e32 = 0 if precision == "fp64" else 4
    return {"prop_per_step": 8 + e32 + 7 * f + 8 + 8,
            "prop_per_sampled": rec + 4 + 4 / 32,
            "sample_per_sampled": rec + 4 / 32,
            "sample_per_pushed": 8 + e32 + 7 * f + 8 + 12}
# Record engine: read the live row (100 B), write its final state (60 B) and
# the one row it creates on average (176 B).
BYTES_PER_STEP_RECORDS = 336


# DRAM traffic per particle-step of each batched kernel in a large wave, from
# one ncu capture of every launch of the two kernels in a 2e4-primary step
# (dram__bytes_read.sum + dram__bytes_write.sum over the step's
# particle-steps, scaled to a large wave by the 20 longest launches' bytes
# per executed thread-instruction); the capture and its command are
# summarised in the named profile.  The bench scales it to its own launches
# by the particle-steps they process.
NCU_TRAFFIC = {
    "propagate": {"bytes_per_step": 98.0, "profile": "profiles/batched_kernels_lead_20k.md"},
    "sample": {"bytes_per_step": 141.0, "profile": "profiles/batched_kernels_lead_20k.md"},
}


# DRAM bytes per row of k_detector_cut with three detectors, from one ncu
# capture of a 4e6-row launch (profiles/k_detector_cut_4e6_rows.md):
# (256.04 + 11.57) MB / 4e6 rows; the traffic of a launch scales with its rows.
NCU_DETECTOR_BYTES_PER_ROW = 66.9


def measured_peak_hbm():
    """The HBM copy bandwidth of MEASURED_PEAKS.json (GB/s), else the
    fallback figure, with its source."""
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return {"value": float(peaks["hbm_gbs"]), "source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    except Exception:
        return {"value": 6800.0, "source": "fallback 6.8 TB/s"}


# Arithmetic and issue rates of the two mixed-form kernels while they run,
# from one ncu capture of a mid-run launch of each (the profile named):
# float32 flop/s = (fadd + fmul + 2 ffma thread instructions) / duration,
# float64 likewise, the issue-active fraction of the schedulers and the lanes
# active per executed instruction.  The bench divides the flop rates by the
# FMA peaks it measures in the same run (pt_alu_peaks).
NCU_ALU = {
    "propagate": {"fp32_tflops": 2.74, "fp64_tflops": 0.0069, "issue_active": 0.580, "fp64_pipe": 0.039,
                  "threads_per_inst": 19.7, "profile": "profiles/alu_batched_lead_20k.md"},
    "sample": {"fp32_tflops": 3.21, "fp64_tflops": 0.0113, "issue_active": 0.486, "fp64_pipe": 0.092,
               "threads_per_inst": 21.9, "profile": "profiles/alu_batched_lead_20k.md"},
}


def alu_roofline():
    """The issue-bound kernels' arithmetic roofline: measured FMA peaks of
    this GPU and each kernel's fraction of them (rates from NCU_ALU)."""
    from petite_gb300 import _lib
    a, b = C.c_double(), C.c_double()
    if _lib.load().pt_alu_peaks(C.byref(a), C.byref(b), None) != 0:
        return None
    p32, p64 = a.value / 1e12, b.value / 1e12
    ks = {k: {"fp32_tflops": v["fp32_tflops"], "fp32_frac": v["fp32_tflops"] / p32,
              "fp64_tflops": v["fp64_tflops"], "fp64_frac": v["fp64_tflops"] / p64,
              "fp64_pipe_busy": v["fp64_pipe"], "issue_active": v["issue_active"],
              "threads_per_inst": v["threads_per_inst"], "profile": v["profile"]} for k, v in NCU_ALU.items()}
    return {"bound": "issue", "fp32_peak_tflops": p32, "fp64_peak_tflops": p64,
            "peak_source": "pt_alu_peaks: FMA chains on every SM, CUDA events, this run (of measured)",
            "kernels": ks}


def measured_traffic(kernel, kd, kt):
    t = NCU_TRAFFIC.get(kernel)
    if not t or kd["launches"] == 0:
        return None
    return t["bytes_per_step"] * kt["steps"] / kd["launches"]


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
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
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
        for l in self.lines:
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


def tables_dir(w):
    """The workload's table directory: the bundled tables, or a bundled
    variant (``tables``: a subdirectory of petite_gb300/data)."""
    base = os.path.join(ROOT, "petite_gb300", "data")
    return os.path.join(base, w["tables"]) if w.get("tables") else base


def cpu_oracle_worker(args):
    """Runs the CPU oracle on a slice of primaries (spawned process)."""
    sys.path.insert(0, ROOT)
    from oracle.shower import OracleShower, OracleTables
    target, cut, seed, p0, pid, mass, first, tdir = args
    npz = os.path.join(tdir, "sm_tables.npz")
    sh = OracleShower(OracleTables(npz, target), cut, seed=seed)
    rows = 0
    for i in range(len(p0)):
        rows += len(sh.generate_shower(tuple(p0[i]), pid=int(pid[i]), mass=float(mass[i]), primary_index=first + i))
    return rows


def cpu_baseline(w, n_sample, cores=None):
    import multiprocessing as mp
    cores = cores or os.cpu_count()
    p0, pid, m = make_primaries(w, n_sample, offset=10_000)
    order = np.argsort(-p0[:, 0])                      # large showers first for balance
    chunks = [order[k::cores * 2] for k in range(cores * 2)]
    jobs = [(w["target"], w["cut"], w["seed"], p0[c], pid[c], m[c], 0, tables_dir(w)) for c in chunks if len(c)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        rows = sum(pool.map(cpu_oracle_worker, jobs))
    dt = time.perf_counter() - t0
    return {"value": rows / dt, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": f"{n_sample} primaries drawn like the workload ({rows} particle-steps) in {dt:.1f} s: "
                      f"oracle (CPU restatement of PETITE's transport loop) over {cores} spawned processes"}


def cpu_dark_worker(args):
    """The CPU oracle on the primaries of one spawned process: each one's SM
    shower (untimed), then its produce_bsm_particle on every row and mass
    (timed), until the dark part has taken `budget` seconds: rows, vectors,
    dark seconds."""
    sys.path.insert(0, ROOT)
    from oracle.shower import OracleShower, OracleTables
    from oracle import dark as D
    target, cut, seed, p0, pid, mass, first, masses, procs, tdir, budget = args
    sm_t = OracleTables(os.path.join(tdir, "sm_tables.npz"), target)
    sh = OracleShower(sm_t, cut, seed=seed)
    orcs = [D.DarkOracle(D.DarkTables(os.path.join(tdir, "dark_tables.npz"), target, mV), sm_t, seed)
            for mV in masses]
    rows = vecs = 0
    t_dark = 0.0
    for i in range(len(p0)):
        recs = sh.generate_shower(tuple(p0[i]), pid=int(pid[i]), mass=float(mass[i]), primary_index=first + i)
        t0 = time.perf_counter()
        for orc, mV in zip(orcs, masses):
            # no DarkAnn below mV = 2 m_e (no resonance, no map set)
            ps = tuple(p for p in procs if p != "DarkAnn" or mV >= 2 * D.P.m_electron)
            vecs += len(orc.dark_shower(recs, processes=ps))
        t_dark += time.perf_counter() - t0
        rows += len(recs)
        if t_dark > budget:
            break
    return rows, vecs, t_dark


def dark_cpu_sample(w):
    """A bounded CPU sample: a 400 GeV muon shower takes the oracle about a
    minute, so those workloads take one primary per process."""
    return {"budget": 10.0, "per_proc": 1} if w["emin"] > 100.0 else {"budget": 15.0, "per_proc": 64}


def cpu_dark_baseline(w, n_proc=None, budget=15.0, per_proc=64):
    """The dark part on the host cores: row x mass per second of the oracle's
    dark production, summed over spawned processes that each take primaries
    drawn like the workload until their dark part has run about `budget`
    seconds (the SM showers are made first and not timed)."""
    import multiprocessing as mp
    n_proc = n_proc or os.cpu_count()
    p0, pid, m = make_primaries(w, n_proc * per_proc, offset=10_000)
    procs = list(w.get("dark_processes", ("DarkBrem", "DarkAnn", "DarkComp")))
    jobs = []
    for k in range(n_proc):
        sl = slice(k * per_proc, (k + 1) * per_proc)
        jobs.append((w["target"], w["cut"], w["seed"], p0[sl], pid[sl], m[sl], k * per_proc, list(w["masses"]),
                     procs, tables_dir(w), budget))
    with mp.get_context("spawn").Pool(n_proc) as pool:
        res = pool.map(cpu_dark_worker, jobs)
    rate = sum(r[0] * len(w["masses"]) / r[2] for r in res if r[2] > 0)   # the processes run side by side
    rows, vecs = sum(r[0] for r in res), sum(r[1] for r in res)
    return {"value": rate, "unit": "row-masses/s", "cores": n_proc, "kind": "port",
            "sample": f"primaries drawn like the workload over {n_proc} spawned processes: the oracle's "
                      f"produce_bsm_particle on {rows} SM rows x {len(w['masses'])} masses ({vecs} vectors), "
                      f"about {budget:.0f} s of dark work per process (the SM showers untimed)"}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        return dist, rank, ws
    return None, 0, 1


def run_reference(args, w, name):
    dist, rank, ws = dist_setup()
    if rank != 0:
        return
    if w["mode"] == "dark":
        # the same metric on the host cores: the oracle's dark production
        vals, cb = [], None
        for _ in range(args.steps):
            cb = cpu_dark_baseline(w, **dark_cpu_sample(w))
            vals.append(cb["value"])
        v = float(np.median(vals))
        print(json.dumps({"impl": "reference", "metric": "dark-vector production: SM rows x dark masses per second "
                          "(pt_run_dark)", "value": v, "unit": "row-masses/s", "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": name, "target": w["target"], "cut_GeV": w["cut"],
                                     "masses_GeV": list(w["masses"])},
                          "cpu_baseline": {**cb, "value": v},
                          "e2e": {"value": v, "unit": "row-masses/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    if w["mode"] == "detector":
        vals, cb = [], None
        for _ in range(args.steps):
            cb = detector_cpu_baseline(w, args.cpu_sample or w["cpu_sample"])
            vals.append(cb["value"])
        v = float(np.median(vals))
        print(json.dumps({"impl": "reference", "metric": "detector acceptance: rows x detectors per second "
                          "(pt_detector_cut)", "value": v, "unit": "row-detectors/s", "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": name, "rows": args.cpu_sample or w["cpu_sample"]},
                          "cpu_baseline": {**cb, "value": v},
                          "e2e": {"value": v, "unit": "row-detectors/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    if w["mode"] not in ("batch", "records"):
        print(json.dumps({"impl": "reference", "unavailable": f"no CPU arm for the {name} workload (its metric "
                          "counts the GPU's SM and dark work together); the dark_* workloads time the oracle's "
                          "dark production"}))
        return
    vals, cb = [], None
    for _ in range(args.steps):
        cb = cpu_baseline(w, args.cpu_sample or w["cpu_sample"])
        vals.append(cb["value"])
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": name, "target": w["target"], "cut_GeV": w["cut"],
                       "primaries_per_step": args.cpu_sample or w["cpu_sample"]},
            "cpu_baseline": {**cb, "value": v},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def matched_stats(a, b):
    """Same-stream comparison of two tally sets (float64 vs mixed)."""
    from scipy import stats
    ca, cb = a["primary_count"], b["primary_count"]
    ea, eb = a["primary_edep"], b["primary_edep"]
    out = {"identical_showers": float(np.mean(ca == cb)),
           "steps_rel_diff": (b["steps"] - a["steps"]) / a["steps"],
           "E_deposited_rel_diff": (b["E_deposited"] - a["E_deposited"]) / a["E_deposited"],
           "ks_p_multiplicity": float(stats.ks_2samp(ca, cb).pvalue),
           "ks_p_edep": float(stats.ks_2samp(ea, eb).pvalue)}
    ha, hb = a["hist"].astype(float), b["hist"].astype(float)
    for kind, nm in ((0, "energy"), (1, "angle"), (2, "depth")):
        x, y = ha[kind].ravel(), hb[kind].ravel()
        mk = (x + y) > 0
        chi2 = float(np.sum((x[mk] - y[mk]) ** 2 / (x[mk] + y[mk])))
        out[f"chi2_p_{nm}"] = float(stats.chi2.sf(chi2, max(int(mk.sum()) - 1, 1)))
    return out


def bench_batch(args, w, name, dist, rank, ws):
    import torch
    from petite_gb300 import Shower
    from petite_gb300.engine import ParticleStore  # noqa: F401  (ensures the package imports)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    sh = Shower(tables_dir(w), w["target"], w["cut"], seed=w["seed"], precision=w["precision"], device=dev)
    eng = sh._engine
    n = args.primaries or w["n"]
    cap = 1 << args.ring_log2
    zmax = 30.0 * 0.0056 if w["target"] == "lead" else 1.0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # > 129 MB L2

    def stage(step):
        p0, pid, m = make_primaries(w, n, offset=block_index(step, rank, ws))
        return (torch.as_tensor(np.ascontiguousarray(p0.T), device=dev), torch.zeros((3, n), dtype=torch.float64, device=dev),
                torch.as_tensor(pid, device=dev), torch.as_tensor(m, device=dev))

    def device_step(step, precision, tally, inputs):
        opts = sh._opts(True, precision)
        opts.primary_offset = first_primary(step, rank, ws, n)
        P0, R0, PID, M = inputs
        stream = torch.cuda.current_stream(dev)
        flush.zero_()
        tally.zero_()
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s = eng.lib.pt_run_batch(eng.handle, C.c_void_p(P0.data_ptr()), C.c_void_p(R0.data_ptr()),
                                 C.c_void_p(PID.data_ptr()), C.c_void_p(M.data_ptr()), P0.shape[1], C.byref(opts),
                                 C.byref(tally.abi()), cap, C.c_void_p(stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize(dev)
        if s != 0:
            raise RuntimeError(f"pt_run_batch status {s}")
        return e0.elapsed_time(e1) / 1e3

    tuning = None
    if not args.no_autotune:
        # work-distribution settings picked on a 1e5-primary calibration run
        # of the same species and energies (outside the timed region)
        from petite_gb300.autotune import autotune_batch
        # (the loops are timed too: host waves, graph loop, persistent kernel;
        # the timed steps keep the host loop, whose per-kernel times the
        # roofline uses)
        # calibration primaries drawn like the workload's (a deep muon line
        # picks lanes, the broad mix one lane)
        ncal = 500 if w["emin"] > 100.0 else 100_000
        cal = make_primaries(w, ncal, offset=20_000_000)
        # lanes only where the calibration is the whole batch: 500 muons
        # run as small waves that lanes overlap, 10^5 fill the GPU
        tuning = autotune_batch(sh, precision=w["precision"], n=ncal, ring_capacity=1 << 24, use_cache=False,
                                choose_loop=False, primaries=cal, tune_lanes=ncal >= n)
    tally = eng.new_tally(n, zmax)
    alu = alu_roofline() if rank == 0 and not args.quick else None
    for s in range(args.warmup):
        device_step(1000 + s, w["precision"], tally, stage(1000 + s))
    if args.quick:
        ts = [device_step(s, w["precision"], tally, stage(s)) for s in range(args.steps)]
        if rank == 0:
            summ = tally.summary()
            print(json.dumps({"workload": name, "primaries": n, "particle_steps": summ["steps"],
                              "sampled": summ["sampled"], "pushed": summ["pushed"], "seconds": ts,
                              "launches_waves": eng.last_run_stats(), "kernel_seconds": eng.last_kernel_times()}))
        return
    times, steps_done, launches = [], 0, 0
    kt = {"prop_s": 0.0, "sample_s": 0.0, "steps": 0, "sampled": 0, "pushed": 0, "waves": 0}
    with ClockSampler(dev.index or 0) as clk:
        for s in range(args.steps):
            inputs = stage(s)
            times.append(device_step(s, w["precision"], tally, inputs))
            summ = tally.summary()
            steps_done += summ["steps"]
            nl, nw = eng.last_run_stats()
            launches += nl
            tp, ts_ = eng.last_kernel_times()
            kt["prop_s"] += tp
            kt["sample_s"] += ts_
            kt["waves"] += nw
            for key in ("steps", "sampled", "pushed"):
                kt[key] += summ[key]
    t_local = float(sum(times))
    t_max, steps_all = reduce_job(t_local, steps_done, dist, dev)
    value = steps_all / t_max

    # plain float64 engine vs mixed on the same first primaries and streams
    nf = min(w["fp64_sample"], n)
    sub = tuple(x[..., :nf].contiguous() for x in stage(0))
    res = {}
    for prec in ("fp64", "mixed"):
        tl = eng.new_tally(nf, zmax)
        dt = device_step(0, prec, tl, sub)
        r_ = tl.summary()
        r_.update(hist=tl.hist.cpu().numpy(), primary_count=tl.primary_count.cpu().numpy(),
                  primary_edep=tl.primary_edep.cpu().numpy(), seconds=dt)
        res[prec] = r_
    fp64_rate = res["fp64"]["steps"] / res["fp64"]["seconds"]
    mixed_sub_rate = res["mixed"]["steps"] / res["mixed"]["seconds"]
    matched = matched_stats(res["fp64"], res["mixed"])

    # end to end through the public API: pinned host inputs, host tallies back
    e2e_steps, e2e_t, h2d, d2h = 0, 0.0, 0, 0
    for s in range(min(args.steps, 2)):
        p0, pid, m = make_primaries(w, n, offset=500 + block_index(s, rank, ws))
        p0h = torch.as_tensor(p0).pin_memory()
        pidh = torch.as_tensor(pid).pin_memory()
        mh = torch.as_tensor(m).pin_memory()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        out = sh.run_tallied(p0h, pidh, mh, precision=w["precision"], first_primary=(500 + block_index(s, rank, ws)) * n,
                             z_max=zmax, queue_capacity=cap)
        torch.cuda.synchronize(dev)
        e2e_t += time.perf_counter() - t0
        e2e_steps += out["steps"]
        h2d += p0.nbytes + pid.nbytes + m.nbytes
        d2h += out["hist"].nbytes + out["primary_count"].nbytes + out["primary_edep"].nbytes + 16 * 8 + 8 * 8
    ne2e = min(args.steps, 2)
    e2e = {"value": e2e_steps / e2e_t, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d // ne2e,
           "d2h_bytes_per_step": d2h // ne2e}
    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    rb = ring_bytes(w["precision"])
    kernels = {
        "propagate": {"seconds": kt["prop_s"], "launches": kt["waves"],
                      "bytes": kt["steps"] * rb["prop_per_step"] + kt["sampled"] * rb["prop_per_sampled"]},
        "sample": {"seconds": kt["sample_s"], "launches": kt["waves"],
                   "bytes": kt["sampled"] * rb["sample_per_sampled"] + kt["pushed"] * rb["sample_per_pushed"]},
    }
    for kd in kernels.values():
        kd["GB_per_s"] = kd["bytes"] / kd["seconds"] / 1e9 if kd["seconds"] > 0 else 0.0
        kd["share_of_step"] = kd["seconds"] / t_local if t_local > 0 else 0.0
    top = max(kernels, key=lambda k_: kernels[k_]["seconds"])
    achieved = kernels[top]["GB_per_s"]
    traffic = measured_traffic(top, kernels[top], kt)
    cb = None if args.no_cpu_baseline else cpu_baseline(w, args.cpu_sample or w["cpu_sample"])
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": name, "primaries_per_step": n, "species": list(w["species"]),
                   "E0_GeV": [w["emin"], w["emax"]], "target": w["target"], "cut_GeV": w["cut"],
                   "precision": w["precision"], "seed": w["seed"], "l2": "flushed (256 MB write) before each step",
                   "parallelism": f"replicas{ws}", "ring_capacity": cap, "tuning": tuning},
        "fp64_engine": {"value": fp64_rate, "unit": "particle-steps/s", "sample_primaries": nf,
                        "mixed_on_same_sample": mixed_sub_rate, "mixed_over_fp64": mixed_sub_rate / fp64_rate},
        "matched_spectra": matched,
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": top,
                     "algorithmic_bytes_per_launch": kernels[top]["bytes"] / max(kernels[top]["launches"], 1),
                     "avg_launch_ms": 1e3 * kernels[top]["seconds"] / max(kernels[top]["launches"], 1),
                     "kernels": kernels,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6.8 TB/s",
                     "note": "issue-bound kernels (Philox, transcendental and table work per byte); "
                             "HBM fraction of the algorithmic ring traffic",
                     "alu": alu},
        "cpu_baseline": cb,
        "clocks": clk.summary(),
        "particle_steps": steps_all,
    }
    print(json.dumps(line))


def bench_records(args, w, name, dist, rank, ws):
    import torch
    from petite_gb300 import Shower
    from petite_gb300.engine import ParticleStore
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    sh = Shower(None, w["target"], w["cut"], seed=w["seed"], precision="fp64", device=dev)
    eng = sh._engine
    opts = sh._opts(True, "fp64")
    n = args.primaries or w["n"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step(s):
        p0, pid, m = make_primaries(w, n, offset=block_index(s, rank, ws))
        opts.primary_offset = first_primary(s, rank, ws, n)
        cap = int(np.sum(2.0 * p0[:, 0] / w["cut"]) + 16 * n)
        st = ParticleStore(cap, dev)
        st.t["p0"][:, :n] = torch.as_tensor(p0.T, device=dev)
        st.t["pid"][:n] = torch.as_tensor(pid, device=dev)
        st.t["mass"][:n] = torch.as_tensor(m, device=dev)
        st.t["weight"][:n] = 1.0
        abi = st.abi()
        nrows = C.c_int64()
        flush.zero_()
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        stream = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        status = eng.lib.pt_run_sm(eng.handle, C.byref(abi), n, C.byref(opts), C.byref(nrows),
                                   C.c_void_p(stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize(dev)
        if status != 0:
            raise RuntimeError(f"pt_run_sm status {status}")
        return e0.elapsed_time(e1) / 1e3, nrows.value

    for s in range(args.warmup):
        step(1000 + s)
    times, rows, launches = [], 0, 0
    with ClockSampler(dev.index or 0) as clk:
        for s in range(args.steps):
            dt, r = step(s)
            times.append(dt)
            rows += r
            launches += eng.last_run_stats()[0]
    t_max, rows_all = reduce_job(float(sum(times)), float(rows), dist, dev)
    value = rows_all / t_max
    e2e_rows, e2e_t, h2d, d2h = 0, 0.0, 0, 0
    for s in range(args.steps):
        p0, pid, m = make_primaries(w, n, offset=500 + block_index(s, rank, ws))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        b = sh.generate_showers(p0, pid=pid, mass=m, first_primary=(500 + block_index(s, rank, ws)) * n)
        torch.cuda.synchronize(dev)
        e2e_t += time.perf_counter() - t0
        e2e_rows += b.n
        h2d += p0.nbytes + pid.nbytes + m.nbytes + 32 * n
        d2h += b.n * (16 * 8 + 6 * 4 + 2 * 8)
    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = value * BYTES_PER_STEP_RECORDS / 1e9
    cb = None if args.no_cpu_baseline else cpu_baseline(w, args.cpu_sample or w["cpu_sample"])
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": name, "primaries_per_step": n, "target": w["target"], "cut_GeV": w["cut"],
                   "precision": "fp64", "l2": "flushed (256 MB write) before each step",
                   "parallelism": f"replicas{ws}"},
        "e2e": {"value": e2e_rows / e2e_t, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d // args.steps,
                "d2h_bytes_per_step": d2h // args.steps},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "bytes_per_step": BYTES_PER_STEP_RECORDS},
        "cpu_baseline": cb, "clocks": clk.summary(), "particle_steps": rows_all}))


def bench_dark(args, w, name, dist, rank, ws):
    """SM showers (float64 record engine) then dark-vector production for every
    mass on the same rows; a step is the whole batch of primaries."""
    import torch
    from petite_gb300.dark import DarkShower, processes_at_mass
    n = args.primaries or w["n"]
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    procs = list(w.get("dark_processes", ("DarkBrem", "DarkAnn", "DarkComp")))
    dprec = w.get("dark_precision", "fp64")
    showers = [DarkShower(tables_dir(w), w["target"], w["cut"], m, seed=w["seed"], device=dev,
                          active_processes=processes_at_mass(procs, m), dark_precision=dprec)
               for m in w["masses"]]
    sm = showers[0]
    chunk = min(w["chunk"], n)

    def step(s):
        rows = vecs = 0
        ysum = np.zeros((len(showers), 4))
        t_sm = t_dark = 0.0
        for c0 in range(0, n, chunk):
            m = min(chunk, n - c0)
            p0, pid, mass = make_primaries(w, m, offset=block_index(s, rank, ws))
            opts = sm._opts(True, "fp64")
            opts.primary_offset = first_primary(s, rank, ws, n) + c0
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            st, nr = sm._engine.run_sm(p0, np.zeros((m, 3)), pid, mass, np.ones(m), opts)
            torch.cuda.synchronize(dev)
            t1 = time.perf_counter()
            for k, d in enumerate(showers):
                out = d._dark_engine.run_dark(d._prm, st, nr, d._opts(), keep_records=False)
                ysum[k] += out["yield"][:4]
                vecs += out["n"]
            torch.cuda.synchronize(dev)
            t2 = time.perf_counter()
            rows += nr
            t_sm += t1 - t0
            t_dark += t2 - t1
            del st
        return rows, vecs, ysum, t_sm, t_dark

    for s in range(args.warmup):
        step(1000 + s)
    tot = [0, 0, np.zeros((len(showers), 4)), 0.0, 0.0]
    with ClockSampler(dev.index or 0) as clk:
        for s in range(args.steps):
            r = step(s)
            for i in range(5):
                tot[i] = tot[i] + r[i]
    rows, vecs, ysum, t_sm, t_dark = tot
    if rank != 0:
        return
    per_mass = {f"{d.get_mV()}": {"yield_per_primary": (ysum[k] / (n * args.steps)).tolist()}
                for k, d in enumerate(showers)}
    # the float64 form of the dark production on the same rows and streams
    # (one chunk), against the form timed above
    cmp64 = None
    if dprec != "fp64":
        p0, pid, mass = make_primaries(w, chunk, offset=block_index(0, rank, ws))
        opts = sm._opts(True, "fp64")
        opts.primary_offset = first_primary(0, rank, ws, n)
        st, nr = sm._engine.run_sm(p0, np.zeros((chunk, 3)), pid, mass, np.ones(chunk), opts)
        t64 = tx = 0.0
        rel = []
        for m_ in w["masses"]:
            d64 = DarkShower(tables_dir(w), w["target"], w["cut"], m_, seed=w["seed"], device=dev,
                             active_processes=processes_at_mass(procs, m_), dark_precision="fp64")
            dx = [d for d in showers if d.get_mV() == d64.get_mV()][0]
            res = {}
            for tag, d in (("fp64", d64), ("x", dx)):
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                res[tag] = d._dark_engine.run_dark(d._prm, st, nr, d._opts(), keep_records=False)
                torch.cuda.synchronize(dev)
                if tag == "fp64":
                    t64 += time.perf_counter() - t0
                else:
                    tx += time.perf_counter() - t0
            y64, yx = res["fp64"]["yield"][:4], res["x"]["yield"][:4]
            rel += [abs(a - b) / a for a, b in zip(y64, yx) if a > 0]
        cmp64 = {"value": nr * len(w["masses"]) / t64, "unit": "row-masses/s", "sample_primaries": chunk,
                 "dark_over_fp64": t64 / tx, "yield_max_rel_diff": max(rel) if rel else 0.0}
    cb = None if args.no_cpu_baseline else cpu_dark_baseline(w, **dark_cpu_sample(w))
    print(json.dumps({
        "metric": "dark-vector production: SM rows x dark masses per second (pt_run_dark)",
        "value": rows * len(showers) / t_dark, "unit": "row-masses/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * (t_sm + t_dark) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if dprec == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": name, "primaries_per_step": n, "E0_GeV": w["emin"], "target": w["target"],
                   "cut_GeV": w["cut"], "masses_GeV": [d.get_mV() for d in showers], "chunk": chunk,
                   "dark_precision": dprec,
                   "processes": [p + "_bound" if p in ("DarkAnn", "DarkComp") else p for p in procs],
                   "tables": w.get("tables", "bundled")},
        "sm_rows": rows, "sm_rows_per_s": rows / t_sm, "vectors": vecs, "vectors_per_s": vecs / t_dark,
        "yields": per_mass, "fp64_dark": cmp64, "cpu_baseline": cb, "clocks": clk.summary()}))


def bench_yield(args, w, name, dist, rank, ws):
    """Dark-vector yield and its mass derivative at fixed uniforms for 4096
    (E, mV) pairs and the three electron/positron/photon dark processes."""
    import torch
    from petite_gb300.dark import DarkShower, dark_yield, map_mass_index
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    sh = DarkShower(None, w["target"], 0.010, 0.1, seed=w["seed"], device=dev)
    eng = sh._dark_engine
    rng = np.random.default_rng(w["seed"] + 17 * rank)
    n = args.primaries or w["n"]
    E = 10 ** rng.uniform(math.log10(0.05), 1.0, n)
    mVh = 10 ** rng.uniform(-3, math.log10(0.3), n)
    Et = torch.as_tensor(E, device=dev)
    procs = ("DarkBrem", "DarkComp", "DarkAnn")
    mi = {p: map_mass_index(eng.data.masses, mVh, eng.has_maps(p), p) for p in procs}

    def step():
        mV = torch.tensor(mVh, dtype=torch.float64, device=dev, requires_grad=True)
        loss = 0
        for p in procs:
            Y, M = dark_yield(eng, p, Et, mV, n_samples=w["samples"], seed=w["seed"], mass_index=mi[p])
            loss = loss + Y.sum() + 1e-3 * M.sum()
        loss.backward()
        return mV.grad

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index or 0) as clk:
        e0.record()
        for _ in range(args.steps):
            g = step()
        e1.record()
        torch.cuda.synchronize(dev)
    t = e0.elapsed_time(e1) / 1e3
    evals = args.steps * n * w["samples"] * len(procs) * 2          # forward and adjoint
    if rank != 0:
        return
    print(json.dumps({
        "metric": "dark yield + adjoint: map-sample evaluations/s (forward and d/dmV)",
        "value": evals / t, "unit": "sample-evaluations/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": name, "pairs": n, "samples_per_pair": w["samples"], "processes": list(procs),
                   "target": w["target"]},
        "grad_finite_fraction": float(torch.isfinite(g).float().mean().item()), "clocks": clk.summary()}))


def detector_rows(w, n, seed):
    """Synthetic dark-vector rows of the detector workload: p0 (n, 4), r0
    (n, 3), w (n,)."""
    rng = np.random.default_rng(seed)
    E = 10 ** rng.uniform(-1.0, math.log10(30.0), n)
    th = 10 ** rng.uniform(-4.0, math.log10(0.3), n)
    ph = rng.uniform(0.0, 2.0 * math.pi, n)
    p = np.sqrt(E * E - 0.01 ** 2)
    p0 = np.empty((n, 4))
    p0[:, 0] = E
    p0[:, 1] = p * np.sin(th) * np.cos(ph)
    p0[:, 2] = p * np.sin(th) * np.sin(ph)
    p0[:, 3] = p * np.cos(th)
    r0 = np.c_[rng.normal(0.0, 0.01, n), rng.normal(0.0, 0.01, n), rng.uniform(0.0, 1.0, n)]
    return p0, r0, rng.uniform(0.1, 2.0, n)


def detector_cpu_baseline(w, n_sample, chunk=5_000_000):
    """The oracle's detector_cut (numpy, one thread) on a bounded sample,
    in chunks of at most ``chunk`` rows (memory-bounded); the rows are drawn
    outside the timed region."""
    from oracle import detector as od
    t, done, k = 0.0, 0, 0
    while done < n_sample:
        m = min(chunk, n_sample - done)
        p0, r0, wt = detector_rows(w, m, w["seed"] + 99 + k)
        t0 = time.perf_counter()
        od.detector_cut(p0, r0, wt, list(w["z"]), w["radius"], method="TotalWeight", energy_cut=w["energy_cut"],
                        inner=w["inner"])
        t += time.perf_counter() - t0
        done += m
        k += 1
    return {"value": n_sample * len(w["z"]) / t, "unit": "row-detectors/s", "cores": 1, "kind": "port",
            "sample": f"{n_sample} rows x {len(w['z'])} detectors in {t:.1f} s: oracle/detector.py (numpy "
                      "restatement of detector_cut), one thread"}


def bench_detector(args, w, name, dist, rank, ws):
    """detector_cut over 10^8 device rows (pt_detector_cut): pass mask and
    weight sums for three disks; e2e through detector_cut_rows from pinned
    host arrays with the efficiencies read back."""
    import torch
    from petite_gb300 import _lib
    from petite_gb300.shower import detector_cut_rows
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    n = args.primaries or w["n"]
    nd = len(w["z"])
    p0, r0, wt = detector_rows(w, n, w["seed"] + 1000 * rank)
    P4 = torch.as_tensor(np.ascontiguousarray(p0.T), device=dev)
    R3 = torch.as_tensor(np.ascontiguousarray(r0.T), device=dev)
    W = torch.as_tensor(wt, device=dev)
    Z = torch.as_tensor(np.asarray(w["z"], np.float64), device=dev)
    mask = torch.empty((nd, n), dtype=torch.uint8, device=dev)
    sums = torch.empty(nd + 1, dtype=torch.float64, device=dev)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    lo, hi = w["energy_cut"]

    def launch():
        s = lib.pt_detector_cut(C.c_void_p(P4.data_ptr()), n, C.c_void_p(R3.data_ptr()), n, C.c_void_p(W.data_ptr()),
                                n, C.c_void_p(Z.data_ptr()), nd, w["inner"], w["radius"], 1, lo, hi,
                                C.c_void_p(mask.data_ptr()), C.c_void_p(sums.data_ptr()), C.c_void_p(stream.cuda_stream))
        if s != 0:
            raise RuntimeError(f"pt_detector_cut status {s}")

    for _ in range(max(args.warmup, 3)):
        launch()
    torch.cuda.synchronize(dev)
    times = []
    with ClockSampler(dev.index or 0) as clk:
        for _ in range(args.steps):
            if dist:
                dist.barrier()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(w["passes"]):
                launch()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            times.append(e0.elapsed_time(e1) / 1e3)
    t = float(sum(times))
    if dist:
        tt = torch.tensor([t], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    # e2e: pinned host rows in, efficiencies out, through the public function
    p0h = torch.as_tensor(p0).pin_memory()
    r0h = torch.as_tensor(r0).pin_memory()
    wh = torch.as_tensor(wt).pin_memory()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    eff = detector_cut_rows(p0h, r0h, wh, list(w["z"]), w["radius"], method="Efficiency",
                            energy_cut=w["energy_cut"], detector_inner_radius=w["inner"], device=dev)
    torch.cuda.synchronize(dev)
    te = time.perf_counter() - t0
    if rank != 0:
        return
    per_launch = n * (64 + nd)          # rows read (8 doubles), mask bytes written
    peak = measured_peak_hbm()
    ach = per_launch / (float(np.mean(times)) / w["passes"]) / 1e9
    cb = None if args.no_cpu_baseline else detector_cpu_baseline(w, args.cpu_sample or w["cpu_sample"])
    print(json.dumps({
        "metric": "detector acceptance: rows x detectors per second (pt_detector_cut)",
        "value": args.steps * w["passes"] * n * nd * ws / t, "unit": "row-detectors/s", "n_gpus": ws,
        "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": name, "rows": n, "passes_per_step": w["passes"], "detectors_z_m": list(w["z"]),
                   "radius_m": w["radius"],
                   "inner_radius_m": w["inner"], "energy_cut_GeV": list(w["energy_cut"]),
                   "l2": "inputs (6.4 GB) larger than L2"},
        "efficiency": [float(x) for x in eff],
        "e2e": {"value": n * nd / te, "unit": "row-detectors/s", "h2d_bytes_per_step": n * 64,
                "d2h_bytes_per_step": 8 * (nd + 1)},
        "gpu_launches": args.steps * w["passes"],
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peak["value"], "unit": "GB/s",
                     "frac": ach / peak["value"], "traffic": NCU_DETECTOR_BYTES_PER_ROW * n, "kernel": "k_detector_cut",
                     "algorithmic_bytes_per_launch": per_launch,
                     "avg_launch_ms": 1e3 * float(np.mean(times)) / w["passes"],
                     "peak_source": peak["source"]},
        "cpu_baseline": cb, "clocks": clk.summary()}))


def bench_batchdark(args, w, name, dist, rank, ws):
    """The batched engine with dark vectors on every wave for all masses at
    once (DarkShower.run_tallied, pt_run_batch_dark); a step is the batch of
    primaries, host inputs copied in and the yields read back inside it."""
    import torch
    from petite_gb300.dark import DarkShower, processes_at_mass
    n = args.primaries or w["n"]
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    procs = list(w["dark_processes"])
    dprec = w.get("dark_precision", "fp64")
    showers = [DarkShower(tables_dir(w), w["target"], w["cut"], m, seed=w["seed"], device=dev,
                          active_processes=processes_at_mass(procs, m), dark_precision=dprec)
               for m in w["masses"]]
    sh = showers[0]
    prms = [d._prm for d in showers]
    tuning = None
    if not args.no_autotune:
        # the SM engine's work distribution and lanes, calibrated on primaries
        # drawn like the workload's (outside the timed region)
        from petite_gb300.autotune import autotune_batch
        ncal = min(n, 500 if w["emin"] > 100.0 else 20_000)
        tuning = autotune_batch(sh, precision=w["precision"], n=ncal, ring_capacity=1 << 24, use_cache=False,
                                choose_loop=False, primaries=make_primaries(w, ncal, offset=20_000_000),
                                tune_lanes=ncal >= n)

    def step(s):
        p0, pid, mass = make_primaries(w, n, offset=block_index(s, rank, ws))
        ins = (torch.as_tensor(np.ascontiguousarray(p0.T)).pin_memory(), torch.as_tensor(pid).pin_memory(),
               torch.as_tensor(mass).pin_memory())
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        dins = (ins[0].to(dev, non_blocking=True), torch.zeros((3, n), dtype=torch.float64, device=dev),
                ins[1].to(dev, non_blocking=True), ins[2].to(dev, non_blocking=True))
        opts = sh._opts(True, w["precision"])
        opts.primary_offset = first_primary(s, rank, ws, n)
        tally = sh._engine.new_tally(n, 1.0)
        _, y, yE, nv = sh._dark_engine.run_batch(prms, None, None, None, None, opts, tally, 1 << 24, dins)
        steps = tally.summary()["steps"]
        torch.cuda.synchronize(dev)
        return steps, nv, y, time.perf_counter() - t0

    for s in range(args.warmup):
        step(1000 + s)
    steps = vecs = 0
    ysum = np.zeros((len(showers), 5))
    t = 0.0
    with ClockSampler(dev.index or 0) as clk:
        for s in range(args.steps):
            a, v, y, dt = step(s)
            steps += a
            vecs += v
            ysum += y
            t += dt
    if rank != 0:
        return
    per_mass = {f"{d.get_mV()}": {"yield_per_primary": (ysum[k][:4] / (n * args.steps)).tolist()}
                for k, d in enumerate(showers)}
    # the host cores' rate of the dark part alone (row x mass per second), for
    # the row_masses_per_s figure of this line
    cb = None if args.no_cpu_baseline else cpu_dark_baseline(w, **dark_cpu_sample(w))
    print(json.dumps({
        "metric": "SM showers with dark-vector production on the batched engine: particle-steps/s",
        "value": steps / t, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if w["precision"] == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": name, "primaries_per_step": n, "E0_GeV": w["emin"], "target": w["target"],
                   "cut_GeV": w["cut"], "masses_GeV": [d.get_mV() for d in showers], "precision": w["precision"],
                   "dark_precision": dprec,
                   "processes": [p + "_bound" if p in ("DarkAnn", "DarkComp") else p for p in procs],
                   "tables": w.get("tables", "bundled"), "timed": "host inputs in, yields out",
                   "tuning": tuning},
        "row_masses_per_s": steps * len(showers) / t, "vectors": vecs, "vectors_per_s": vecs / t,
        "yields": per_mass, "cpu_baseline": cb, "clocks": clk.summary()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sm_batched_lead_1M", choices=sorted(WORKLOADS))
    ap.add_argument("--primaries", type=int, default=0, help="override primaries per step")
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ring-log2", type=int, default=27,
                    help="batched engine: log2 of the ring capacity (2^27: waves of ~1.2e7 entries; larger "
                         "rings saturate on the 1e6-primary workload)")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default=None,
                    help="batched engine: override the workload's precision (profiling the float64 form)")
    ap.add_argument("--no-autotune", action="store_true", help="batched engine: library default work distribution")
    ap.add_argument("--quick", action="store_true",
                    help="device steps only (no float64 comparison, e2e or CPU baseline): for profiling")
    args = ap.parse_args()
    w = dict(WORKLOADS[args.workload])
    if args.precision:
        w["precision"] = args.precision
    if args.impl == "reference":
        return run_reference(args, w, args.workload)
    dist, rank, ws = dist_setup()
    if w["mode"] == "batch":
        bench_batch(args, w, args.workload, dist, rank, ws)
    elif w["mode"] == "dark":
        bench_dark(args, w, args.workload, dist, rank, ws)
    elif w["mode"] == "batchdark":
        bench_batchdark(args, w, args.workload, dist, rank, ws)
    elif w["mode"] == "yield":
        bench_yield(args, w, args.workload, dist, rank, ws)
    elif w["mode"] == "detector":
        bench_detector(args, w, args.workload, dist, rank, ws)
    else:
        bench_records(args, w, args.workload, dist, rank, ws)


if __name__ == "__main__":
    main()
