"""Device side of the SM shower: tables in HBM and the calls into the C ABI.

Torch owns every device buffer; the library only reads and writes them.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .tables import M_ELECTRON, SMTables

U64 = (1 << 64) - 1


def mix64(z: int) -> int:
    """SplitMix64 finaliser; same as the device's (pt_common.cuh)."""
    z &= U64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & U64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & U64
    return z ^ (z >> 31)


def primary_key(i: int) -> int:
    """Random-stream key of primary number i."""
    return mix64(i + 1)


def daughter_key(parent: int, bit: int) -> int:
    """Random-stream key of daughter `bit` (0 or 1) of a particle."""
    return mix64(parent + 0x9E3779B97F4A7C15 * (1 + bit))

PRECISIONS = {"fp64": 0, "mixed": 1}


def _torch():
    import torch
    return torch


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class ParticleStore:
    """SoA particle rows on the device (layout of ``pt_particles``)."""

    FIELDS_F64 = {"p0": 4, "r0": 3, "pf": 4, "rf": 3, "weight": 1, "mass": 1}
    FIELDS_I32 = ("pid", "gen", "proc", "bit", "primary", "draws")

    def __init__(self, capacity: int, device):
        torch = _torch()
        self.capacity = int(capacity)
        self.t = {}
        for k, n in self.FIELDS_F64.items():
            self.t[k] = torch.zeros((n, self.capacity) if n > 1 else (self.capacity,), dtype=torch.float64, device=device)
        for k in self.FIELDS_I32:
            self.t[k] = torch.zeros(self.capacity, dtype=torch.int32, device=device)
        self.t["parent"] = torch.zeros(self.capacity, dtype=torch.int64, device=device)
        self.t["pkey"] = torch.zeros(self.capacity, dtype=torch.int64, device=device)   # uint64 bits

    def abi(self) -> _lib.PtParticles:
        s = _lib.PtParticles()
        for k in ("p0", "r0", "pf", "rf", "weight", "mass", "pid", "gen", "proc", "bit", "primary", "draws",
                  "parent", "pkey"):
            setattr(s, k, self.t[k].data_ptr())
        s.capacity = self.capacity
        return s

    def to_numpy(self, n: int) -> dict:
        out = {}
        for k, v in self.t.items():
            a = v[..., :n].cpu().numpy()
            out[k] = a.T.copy() if a.ndim == 2 else a
        out["pkey"] = out["pkey"].view(np.uint64)
        return out


class Tally:
    """Device tallies of pt_run_batch (layout of ``pt_tally``)."""

    COUNT_NAMES = {0: "steps", 1: "proposals", 2: "substeps", 3: "ended", 4: "pushed", 5: "below_cut",
                   7: "sampled", 8: "photon_steps", 9: "electron_steps", 10: "positron_steps", 11: "muon_steps"}

    def __init__(self, n_primaries: int, device, z_max: float = 1.0):
        torch = _torch()
        self.counts = torch.zeros(_lib.N_COUNTS, dtype=torch.int64, device=device)
        self.energy = torch.zeros(_lib.N_ESUM, dtype=torch.float64, device=device)
        self.hist = torch.zeros((3, 4, _lib.HIST_BINS), dtype=torch.int32, device=device)
        self.primary_count = torch.zeros(max(n_primaries, 1), dtype=torch.int32, device=device)
        self.primary_edep = torch.zeros(max(n_primaries, 1), dtype=torch.float64, device=device)
        self.z_max = float(z_max)

    def zero_(self):
        for t in (self.counts, self.energy, self.hist, self.primary_count, self.primary_edep):
            t.zero_()

    def abi(self) -> _lib.PtTally:
        t = _lib.PtTally()
        t.counts = self.counts.data_ptr()
        t.energy = self.energy.data_ptr()
        t.hist = self.hist.data_ptr()
        t.primary_count = self.primary_count.data_ptr()
        t.primary_edep = self.primary_edep.data_ptr()
        t.z_max = self.z_max
        self._abi = t
        return t

    def summary(self) -> dict:
        c = self.counts.cpu().numpy()
        e = self.energy.cpu().numpy()
        out = {name: int(c[k]) for k, name in self.COUNT_NAMES.items()}
        out.update(E_continuous=float(e[0]), E_below_cut=float(e[1]), E_ended=float(e[2]), E_primaries=float(e[3]))
        out["E_deposited"] = float(e[0] + e[1] + e[2])
        return out


class SMEngine:
    """Uploads one target's tables and exposes the C-ABI entry points."""

    MAX_ROWS = 2 ** 31 - 1          # largest particle store run_sm grows to
    MAX_RING = 1 << 28              # largest live-particle ring run_batch grows to

    def __init__(self, tables: SMTables, device="cuda"):
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("petite_gb300 needs a CUDA device (GB300); there is no CPU fallback")
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.tables = tables
        self.unusable = None            # set when a device copy may still be in flight
        self.last_store_capacity = 0    # particle store of the last run_sm (after PT_OOM retries)
        dev = self.device
        f64 = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float64), device=dev)
        self._keep = {
            "map_energy": f64(tables.map_energy),
            "map_maxF": f64(tables.map_maxF),
            "map_neval": f64(tables.map_neval),
            "grid_offset": torch.as_tensor(np.ascontiguousarray(tables.grid_offset.reshape(-1), np.int64), device=dev),
            "grid_ninc": torch.as_tensor(np.ascontiguousarray(tables.grid_ninc.reshape(-1), np.int32), device=dev),
            "grid_nodes": f64(tables.grid_nodes),
            "grid_f32x4": torch.as_tensor(tables.grid_f32x4(), device=dev),
        }
        ns_x = np.concatenate([x for x, _ in tables.nsigma])
        ns_y = np.concatenate([y for _, y in tables.nsigma])
        self._keep["ns_x"] = f64(ns_x)
        self._keep["ns_y"] = f64(ns_y)
        self._keep["ns_x32"] = torch.as_tensor(ns_x.astype(np.float32), device=dev)
        self._keep["ns_y32"] = torch.as_tensor(ns_y.astype(np.float32), device=dev)
        slopes = []
        for x, y in tables.nsigma:
            sl = np.zeros_like(x)
            sl[:-1] = (y[1:] - y[:-1]) / (x[1:] - x[:-1])
            slopes.append(sl)
        self._keep["ns_s32"] = torch.as_tensor(np.concatenate(slopes).astype(np.float32), device=dev)
        self._keep["map_energy32"] = torch.as_tensor(tables.map_energy.astype(np.float32), device=dev)
        self._keep["map_cnorm32"] = torch.as_tensor(self._cnorm(tables).astype(np.float32), device=dev)
        pt = _lib.PtTables()
        for p in range(_lib.N_PROC):
            pt.map_base[p] = int(tables.map_base[p])
            pt.map_rows[p] = int(tables.map_rows[p])
        pt.n_rows = int(len(tables.map_energy))
        for k in ("map_energy", "map_maxF", "map_neval", "grid_offset", "grid_ninc", "grid_nodes", "grid_f32x4"):
            setattr(pt, k, self._keep[k].data_ptr())
        pt.n_nodes = int(len(tables.grid_nodes))
        base = 0
        for s, (x, _) in enumerate(tables.nsigma):
            pt.ns_base[s] = base
            pt.ns_len[s] = len(x)
            base += len(x)
        pt.ns_x = self._keep["ns_x"].data_ptr()
        pt.ns_y = self._keep["ns_y"].data_ptr()
        pt.ns_x32 = self._keep["ns_x32"].data_ptr()
        pt.ns_y32 = self._keep["ns_y32"].data_ptr()
        pt.ns_s32 = self._keep["ns_s32"].data_ptr()
        pt.map_energy32 = self._keep["map_energy32"].data_ptr()
        pt.map_cnorm32 = self._keep["map_cnorm32"].data_ptr()
        for sl, (x, _) in enumerate(tables.nsigma):
            pt.ns_lnx0[sl] = float(np.log(x[0]))
            pt.ns_invdlog[sl] = float((len(x) - 1) / np.log(x[-1] / x[0]))
        for p in range(_lib.N_PROC):
            e = tables.map_energy[tables.map_base[p]:tables.map_base[p] + tables.map_rows[p]]
            pt.map_lnE0[p] = float(np.log(e[0]))
            pt.map_invdlog[p] = float((len(e) - 1) / np.log(e[-1] / e[0])) if len(e) > 1 else 0.0
        pt.Z, pt.A, pt.rho = tables.Z, tables.A, tables.rho
        pt.dEdx_GeV_per_m = tables.dEdx * 0.1
        pt.Eg_min, pt.Ee_min = tables.Eg_min, tables.Ee_min
        mc = tables.min_calc
        pt.min_calc_electron, pt.min_calc_positron = mc[11], mc[-11]
        pt.min_calc_muon, pt.min_calc_photon = mc[13], mc[22]
        # all_processes.py:92-103 and moliere.py:219, same expressions as the reference
        Z = tables.Z_int
        a0 = 184.15 * (2.718) ** -0.5 * Z ** (-1.0 / 3.0) / M_ELECTRON
        pt.a0sq = a0 ** 2
        pt.Z2a04 = Z ** 2 * a0 ** 4
        pt.Z23 = Z ** (2. / 3.)
        pt.Z13 = Z ** (1. / 3.)
        self._pt = pt
        h = C.c_void_p()
        _lib.check(self.lib.pt_create(C.byref(pt), C.byref(h)), "pt_create")
        self.handle = h

    @staticmethod
    def _cnorm(tables) -> np.ndarray:
        """Per map row: the energy-independent prefactor of the float32
        acceptance ratio divided by max_F * neval (see pt_physics32.cuh)."""
        from .tables import ALPHA_EM, PROCESSES
        a0 = 184.15 * (2.718) ** -0.5 * tables.Z_int ** (-1.0 / 3.0) / M_ELECTRON
        brem = 8.0 * ALPHA_EM ** 3 * tables.Z_int ** 2 * a0 ** 4
        K = {"Brem": brem, "MuonBrem": brem, "PairProd": brem, "Comp": math.pi * ALPHA_EM ** 2,
             "MuonE": math.pi * ALPHA_EM ** 2, "Ann": 2 * math.pi * ALPHA_EM ** 2,
             "Moller": 2 * math.pi * ALPHA_EM ** 2, "Bhabha": math.pi * ALPHA_EM ** 2 / 2}
        out = np.zeros(len(tables.map_energy))
        for p, name in enumerate(PROCESSES):
            b, n = tables.map_base[p], tables.map_rows[p]
            # rows with max_F = 0 give an infinite ratio: the first proposal with
            # f > 0 is accepted, as max_F*U < wgt*f does in the reference
            with np.errstate(divide="ignore"):
                out[b:b + n] = K[name] / (tables.map_maxF[b:b + n] * tables.map_neval[b:b + n])
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _stream(self):
        return C.c_void_p(_torch().cuda.current_stream(self.device).cuda_stream)

    def _raise(self, status, what):
        if status == _lib.PT_NO_SAMPLE:
            proc, E, key = C.c_int32(), C.c_double(), C.c_int32()
            self.lib.pt_last_error_info(self.handle, C.byref(proc), C.byref(E), C.byref(key))
            from .tables import PROCESSES
            raise Exception("No Sample Found", PROCESSES[proc.value], E.value, key.value)
        if status == _lib.PT_TIMEOUT:
            proc, E, key = C.c_int32(), C.c_double(), C.c_int32()
            self.lib.pt_last_error_info(self.handle, C.byref(proc), C.byref(E), C.byref(key))
            if proc.value == -2:
                # a table-staging copy into shared memory did not land in time
                # and may still be in flight: nothing this handle computes on
                # the device afterwards can be trusted
                self.unusable = f"{what}: a table-staging copy timed out; make a new Shower"
        _lib.check(status, what)

    def _usable(self):
        if self.unusable:
            raise _lib.PetiteGPUError(_lib.PT_TIMEOUT, self.unusable)

    @staticmethod
    def opts(min_energy, max_n_integrators=10000, rescale_MCS=1.0, ms=True, precision="fp64", seed=0,
             primary_offset=0, fast_MCS_mode=True):
        o = _lib.PtOpts()
        o.min_energy = float(min_energy)
        o.max_n_integrators = int(max_n_integrators)
        o.rescale_MCS = float(rescale_MCS)
        o.multiple_scattering = 1 if ms else 0
        o.precision = PRECISIONS[precision]
        o.seed = int(seed) & ((1 << 64) - 1)
        o.primary_offset = int(primary_offset)
        o.mcs_mode = 0 if fast_MCS_mode else 1
        return o

    def run_sm(self, p0, r0, pid, mass, weight, opts: _lib.PtOpts, capacity: int | None = None):
        """Transports primaries (host arrays); returns (store, n_rows)."""
        self._usable()
        torch = _torch()
        p0 = np.asarray(p0, np.float64).reshape(-1, 4)
        n = len(p0)
        r0 = np.asarray(r0, np.float64).reshape(n, 3)
        if capacity is None:
            est = np.sum(2.0 * p0[:, 0] / max(opts.min_energy, 1e-3)) + 16 * n
            capacity = int(min(max(est, 1024), self.MAX_ROWS))
        while True:
            st = ParticleStore(capacity, self.device)
            st.t["p0"][:, :n] = torch.as_tensor(p0.T, device=self.device)
            st.t["r0"][:, :n] = torch.as_tensor(r0.T, device=self.device)
            st.t["pid"][:n] = torch.as_tensor(np.asarray(pid, np.int32), device=self.device)
            st.t["mass"][:n] = torch.as_tensor(np.asarray(mass, np.float64), device=self.device)
            st.t["weight"][:n] = torch.as_tensor(np.asarray(weight, np.float64), device=self.device)
            abi = st.abi()
            nrows = C.c_int64()
            s = self.lib.pt_run_sm(self.handle, C.byref(abi), n, C.byref(opts), C.byref(nrows), self._stream())
            self.last_store_capacity = capacity
            if s == _lib.PT_OOM and capacity < self.MAX_ROWS:
                # the showers outgrew the store: start over with twice the rows
                capacity = min(2 * capacity, self.MAX_ROWS)
                del st
                continue
            self._raise(s, "pt_run_sm")
            return st, int(nrows.value)

    def last_run_stats(self):
        l, w = C.c_int64(), C.c_int64()
        _lib.check(self.lib.pt_last_run_stats(self.handle, C.byref(l), C.byref(w)), "pt_last_run_stats")
        return int(l.value), int(w.value)

    LOOPS = {"host": 0, "graph": 1, "persistent": 2}
    STAGING = {"default": 0, "cached": 1, "shared": 2}

    def set_tuning(self, refill_min=(0, 0), chunk=(0, 0), loop="host", staging="default", threads=0, barrier_ns=0,
                   lanes=0):
        """Work distribution of the batched engine (0 = library default), who
        runs its waves -- "host" (two launches per wave, counters read back),
        "graph" (a CUDA graph's conditional loop, planned on the GPU) or
        "persistent" (one cooperative kernel) -- and where the mixed
        propagation kernel reads the n*sigma tables: "shared" (each block's
        shared memory, filled by TMA bulk copies; "default"), or "cached"
        (the read-only data cache) -- and the mixed kernels' threads per block
        (64, 128 or 256; 0 = 128) -- and the persistent kernel's bound on a
        grid-barrier wait in ns (0 = the library's 20 s) -- and, with the host
        loop, the lanes: groups of primaries with their own rings and streams
        whose waves interleave (0 or 1 = one; up to 8)."""
        t = _lib.PtBatchTuning()
        t.refill_min[0], t.refill_min[1] = int(refill_min[0]), int(refill_min[1])
        t.chunk[0], t.chunk[1] = int(chunk[0]), int(chunk[1])
        t.loop = self.LOOPS[loop]
        t.staging = self.STAGING[staging]
        t.threads = int(threads)
        t.barrier_ns = int(barrier_ns)
        t.lanes = int(lanes)
        _lib.check(self.lib.pt_set_batch_tuning(self.handle, C.byref(t)), "pt_set_batch_tuning")
        self.tuning = {"refill_min": list(refill_min), "chunk": list(chunk), "loop": loop, "staging": staging,
                       "threads": int(threads), "lanes": int(lanes)}

    def last_kernel_times(self):
        """Device seconds of the last batched run: (propagation, sampler)."""
        a, b = C.c_double(), C.c_double()
        _lib.check(self.lib.pt_last_kernel_times(self.handle, C.byref(a), C.byref(b)), "pt_last_kernel_times")
        return a.value / 1e3, b.value / 1e3

    def new_tally(self, n_primaries: int, z_max: float = 1.0) -> "Tally":
        return Tally(n_primaries, self.device, z_max)

    def run_batch(self, p0, r0, pid, mass, opts: _lib.PtOpts, tally: "Tally", queue_capacity: int = 0,
                  device_inputs=None, dark=None):
        """Transports primaries without storing particle lists; accumulates into `tally`.

        p0 (n,4), r0 (n,3), pid (n,), mass (n,) host arrays, or device tensors in
        `device_inputs` = (p0 [4,n], r0 [3,n], pid [n], mass [n]) already resident.
        ``dark`` = (dark handle, pt_dark_params array, yield, yield_E, hist, counts)
        runs pt_run_batch_dark instead: dark vectors on every wave for each
        parameter set, yields accumulated into the two device tensors
        ([sets, N_DARK + 1]) and, with ``hist`` a PtDarkHist over the device
        tensor ``counts`` (or both None), their energy histogram; returns
        (tally, vectors)."""
        self._usable()
        torch = _torch()
        if device_inputs is None:
            p0 = np.asarray(p0, np.float64).reshape(-1, 4)
            n = len(p0)
            dev = self.device
            P0 = torch.as_tensor(np.ascontiguousarray(p0.T), device=dev)
            R0 = torch.as_tensor(np.ascontiguousarray(np.asarray(r0, np.float64).reshape(n, 3).T), device=dev)
            PID = torch.as_tensor(np.asarray(pid, np.int32), device=dev)
            M = torch.as_tensor(np.asarray(mass, np.float64), device=dev)
        else:
            P0, R0, PID, M = device_inputs
            n = P0.shape[1]
        # the kernels read n entries of every input: a short one is refused here
        shapes = [tuple(P0.shape), tuple(R0.shape), tuple(PID.shape), tuple(M.shape)]
        if shapes != [(4, n), (3, n), (n,), (n,)] or not all(t.is_contiguous() for t in (P0, R0, PID, M)):
            raise ValueError(f"run_batch: inputs p0 [4,n], r0 [3,n], pid [n], mass [n] (contiguous) expected, "
                             f"got {shapes}")
        if PID.dtype != torch.int32 or not all(t.dtype == torch.float64 for t in (P0, R0, M)):
            raise ValueError("run_batch: pid int32 and float64 p0, r0, mass expected")
        cap = int(queue_capacity) if queue_capacity else (1 << 24)
        while True:
            if dark is None:
                s = self.lib.pt_run_batch(self.handle, _ptr(P0), _ptr(R0), _ptr(PID), _ptr(M), n, C.byref(opts),
                                          C.byref(tally.abi()), cap, self._stream())
            else:
                dh, prm, yld, yldE, hist = dark[:5]
                nv = C.c_int64()
                s = self.lib.pt_run_batch_dark(self.handle, dh, prm, len(prm), _ptr(P0), _ptr(R0), _ptr(PID),
                                               _ptr(M), n, C.byref(opts), C.byref(tally.abi()), cap, _ptr(yld),
                                               _ptr(yldE), C.byref(hist) if hist is not None else None,
                                               C.byref(nv), self._stream())
            if s == _lib.PT_OOM and cap < self.MAX_RING:
                # the live population outgrew the ring: start over with twice the room
                tally.zero_()
                if dark is not None:
                    dark[2].zero_()
                    dark[3].zero_()
                    if dark[5] is not None:
                        dark[5].zero_()
                cap *= 2
                continue
            self._raise(s, "pt_run_batch" if dark is None else "pt_run_batch_dark")
            return tally if dark is None else (tally, int(nv.value))

    def sample_only(self, process: int, energy, pkey, opts: _lib.PtOpts):
        torch = _torch()
        E = torch.as_tensor(np.asarray(energy, np.float64), device=self.device)
        K = torch.as_tensor(np.asarray(pkey, np.uint64).view(np.int64), device=self.device)
        n = E.numel()
        x = torch.zeros(n * 4, dtype=torch.float64, device=self.device)
        props = torch.zeros(n, dtype=torch.int64, device=self.device)
        lu = torch.zeros(n, dtype=torch.int32, device=self.device)
        s = self.lib.pt_sample_only(self.handle, int(process), _ptr(E), _ptr(K), n, C.byref(opts), _ptr(x),
                                    _ptr(props), _ptr(lu), self._stream())
        self._raise(s, "pt_sample_only")
        return x.view(n, 4).cpu().numpy(), props.cpu().numpy(), lu.cpu().numpy()

    def dsigma(self, process: int, x, energy, precision="fp64"):
        torch = _torch()
        x = np.asarray(x, np.float64).reshape(-1, 4)
        X = torch.as_tensor(x, device=self.device).contiguous()
        E = torch.as_tensor(np.asarray(energy, np.float64), device=self.device)
        out = torch.zeros(len(x), dtype=torch.float64, device=self.device)
        s = self.lib.pt_dsigma(self.handle, int(process), _ptr(X), _ptr(E), len(x), PRECISIONS[precision],
                               _ptr(out), self._stream())
        _lib.check(s, "pt_dsigma")
        return out.cpu().numpy()
