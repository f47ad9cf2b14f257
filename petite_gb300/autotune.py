"""Autotuner for the batched engine's work distribution.

Picks, for one GPU, target and precision, the settings of
``pt_set_batch_tuning`` -- idle lanes gathered before a refill and pool
entries claimed per atomic, for the propagation and the sampler kernel,
the threads per block of the mixed kernels, where the mixed propagation
kernel reads its cross-section tables (the
read-only data cache, or shared memory staged by TMA bulk copies), and who
runs the waves (the host, a CUDA graph's conditional loop, or one
persistent kernel), and with the host loop the lanes (groups of primaries
with their own rings and streams whose waves interleave) -- by timing short
calibration transports (CUDA events around the whole run on its stream)
over a small grid, one coordinate at a time.  The calibration primaries
are a mix of e-, e+ and photons at 0.1-100 GeV unless the caller passes
primaries drawn like its workload (a deep muon line wants lanes, a broad
mix does not).
Results are cached in ``$XDG_CACHE_HOME/petite_gb300/tuning.json`` (or
``~/.cache/...``) keyed by device name, target and precision.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

GRID = {"refill_min": (4, 8, 12, 16), "chunk_propagate": (64, 128, 256), "chunk_sample": (32, 64, 128),
        "threads": (64, 128, 256), "staging": ("cached", "shared"), "loop": ("host", "graph", "persistent"),
        "lanes": (1, 2, 4, 8)}
DEFAULT = {"refill_min": (8, 8), "chunk": (128, 64), "loop": "host", "staging": "shared", "threads": 128, "lanes": 1}
CACHE_VERSION = 5


def _cache_path():
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "petite_gb300", "tuning.json")


def _calibration_primaries(n, seed):
    rng = np.random.default_rng(seed)
    pid = np.array([11, -11, 22])[rng.integers(0, 3, n)].astype(np.int32)
    E = 10 ** rng.uniform(-1.0, 2.0, n)
    m = np.where(np.abs(pid) == 11, 0.000511, 0.0)
    return np.c_[E, np.zeros(n), np.zeros(n), np.sqrt(E * E - m * m)], pid, m


def autotune_batch(shower, precision="mixed", n=20_000, ring_capacity=1 << 22, seed=0, use_cache=True,
                   verbose=False, choose_loop=True, primaries=None, tune_lanes=True):
    """Tunes ``shower``'s engine and returns the chosen settings
    ``{"refill_min": [p, s], "chunk": [p, s], "threads": b, "staging": g, "loop": l, "lanes": k,
    "seconds": t, "threads_seconds": {...}, "staging_seconds": {...}, "loop_seconds": {...},
    "lanes_seconds": {...}}`` (``*_seconds``: the calibration run under each option, the earlier
    coordinates already chosen).  ``choose_loop=False`` times the loops but keeps the host
    loop, whose per-kernel event times a roofline needs.  ``primaries`` =
    (p0 (n,4), pid, mass): calibrate on these instead of the mix (not cached).
    ``tune_lanes=False`` keeps one lane: lanes pay off for a batch that the
    GPU runs as a few small waves, so a calibration smaller than the real
    batch would pick them where the real batch fills the GPU."""
    import torch
    eng = shower._engine
    key = f"{torch.cuda.get_device_name(eng.device)}|{shower.get_target_material()}|{precision}|v{CACHE_VERSION}"
    if primaries is not None:
        use_cache = False
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        best = cache[key]
        eng.set_tuning(best["refill_min"], best["chunk"], best.get("loop", "host"), best.get("staging", "default"),
                       best.get("threads", 0), lanes=best.get("lanes", 1))
        return best

    p0, pid, m = _calibration_primaries(n, seed) if primaries is None else primaries
    n = len(p0)
    dev = eng.device
    P0 = torch.as_tensor(np.ascontiguousarray(p0.T), device=dev)
    R0 = torch.zeros((3, n), dtype=torch.float64, device=dev)
    PID = torch.as_tensor(pid, device=dev)
    M = torch.as_tensor(m, device=dev)
    tally = eng.new_tally(n, 1.0)

    stream = torch.cuda.current_stream(dev)

    def run(cfg):
        eng.set_tuning(cfg["refill_min"], cfg["chunk"], cfg["loop"], cfg["staging"],
                       cfg["threads"] if precision == "mixed" else 0, lanes=cfg["lanes"])
        opts = shower._opts(True, precision)
        tally.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.run_batch(None, None, None, None, opts, tally, queue_capacity=ring_capacity,
                      device_inputs=(P0, R0, PID, M))
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / 1e3

    cfg = {"refill_min": list(DEFAULT["refill_min"]), "chunk": list(DEFAULT["chunk"]), "loop": DEFAULT["loop"],
           "staging": DEFAULT["staging"], "threads": DEFAULT["threads"], "lanes": DEFAULT["lanes"]}
    run(cfg)                                            # warm-up (scratch, caches)
    best_t = run(cfg)
    seconds = {"threads": {}, "staging": {}, "loop": {}, "lanes": {}}
    for name, values in GRID.items():
        if name in ("threads", "staging") and precision != "mixed":
            continue                                    # float32 kernels only
        if name == "lanes" and (cfg["loop"] != "host" or not tune_lanes):
            continue                                    # lanes are a form of the host loop
        for v in values:
            trial = {"refill_min": list(cfg["refill_min"]), "chunk": list(cfg["chunk"]), "loop": cfg["loop"],
                     "staging": cfg["staging"], "threads": cfg["threads"], "lanes": cfg["lanes"]}
            if name == "refill_min":
                trial["refill_min"] = [v, v]
            elif name == "chunk_propagate":
                trial["chunk"][0] = v
            elif name == "chunk_sample":
                trial["chunk"][1] = v
            else:
                trial[name] = v
            if trial == cfg:
                if name in seconds:
                    seconds[name][v] = best_t
                continue
            if name == "lanes":
                run(trial)                              # a new lane's scratch is allocated on its first run
            t = run(trial)
            if name in seconds:
                seconds[name][v] = t
                if name == "loop" and not choose_loop:
                    continue
            if verbose:
                print("autotune", trial, round(t, 4))
            if t < best_t * 0.97:                       # a change must beat run-to-run noise (~1-2 %)
                best_t, cfg = t, trial
    best = {"refill_min": cfg["refill_min"], "chunk": cfg["chunk"], "threads": cfg["threads"],
            "staging": cfg["staging"], "loop": cfg["loop"], "lanes": cfg["lanes"], "seconds": best_t,
            "threads_seconds": seconds["threads"], "staging_seconds": seconds["staging"],
            "loop_seconds": seconds["loop"], "lanes_seconds": seconds["lanes"]}
    eng.set_tuning(best["refill_min"], best["chunk"], best["loop"], best["staging"],
                   best["threads"] if precision == "mixed" else 0, lanes=best["lanes"])
    if use_cache:
        cache[key] = best
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return best
