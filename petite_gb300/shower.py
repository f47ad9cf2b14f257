"""Drop-in ``Shower`` for PETITE's SM shower path (shower.py:98-708).

Same constructor and ``generate_shower`` signature as PETITE; the transport
runs in the CUDA engine.  ``generate_showers`` is the batched form (many
primaries per launch, structure-of-arrays output).

Random numbers: PETITE draws from process-global generators in list order.
Here each particle has its own Philox stream, keyed by ``seed`` and by its
lineage (primary index, then the daughter bit at every generation), so a
shower does not depend on how the engine schedules particles.
"""
from __future__ import annotations

import copy
import os

import numpy as np

from . import tables as T
from ._lib import PetiteGPUError
from .engine import SMEngine
from .particle import MASS, Particle

SUPPORTED_PIDS = (11, -11, 22, 13, -13)


class ShowerBatch:
    """Output of :meth:`Shower.generate_showers`: one row per particle.

    Arrays (numpy): p0 (n,4), r0 (n,3), pf (n,4), rf (n,3), weight, mass,
    pid, gen, proc (-1 = "Input"), bit, primary, parent (row, -1 for
    primaries), pkey, draws.  ``order`` lists rows in PETITE's list order
    (primary by primary, breadth first).
    """

    def __init__(self, arrays: dict, n_primaries: int):
        self.__dict__.update(arrays)
        self.n_primaries = n_primaries
        self.n = len(self.pid)
        self._order = None

    @property
    def order(self):
        if self._order is None:
            self._order = list_order(self.primary, self.gen, self.parent, self.bit)
        return self._order


def list_order(primary, gen, parent, bit):
    """Row order of PETITE's ``all_particles`` list (shower.py:634-706):
    per primary, generation by generation, children in the order of their
    parents' positions, first daughter before second."""
    n = len(primary)
    pos = np.full(n, -1, np.int64)
    roots = np.where(parent < 0)[0]
    roots = roots[np.argsort(primary[roots], kind="stable")]
    pos[roots] = np.arange(len(roots))          # provisional, per-generation
    order_by_gen = [roots]
    g = 1
    while True:
        rows = np.where(gen == g)[0]
        if len(rows) == 0:
            break
        keys = np.lexsort((bit[rows], pos[parent[rows]]))
        rows = rows[keys]
        pos[rows] = np.arange(len(rows))
        order_by_gen.append(rows)
        g += 1
    allrows = np.concatenate(order_by_gen)
    # stable sort by primary keeps the breadth-first order inside each shower
    return allrows[np.argsort(primary[allrows], kind="stable")]


class Shower:
    """Representation of a shower (shower.py:98-142)."""

    def __init__(self, dict_dir, target_material, min_energy, maxF_fudge_global=1,
                 max_n_integrators=int(1e4), fast_MCS_mode=True, seed=None, rescale_MCS=1,
                 precision="fp64", device="cuda"):
        if dict_dir is None:
            dict_dir = T.BUNDLED_DIR
        self._dict_dir = dict_dir
        self._target_material = target_material
        self.min_energy = min_energy
        self._raw = T.read_dict_dir(dict_dir)
        self.tables = T.SMTables(self._raw, target_material, maxF_fudge_global)
        self._ZTarget, self._ATarget = T.TARGET_INFORMATION[target_material]["Z_T"], T.TARGET_INFORMATION[target_material]["A_T"]
        self._rhoTarget, self._dEdx = self.tables.rho, self.tables.dEdx
        self._maxF_fudge_global = maxF_fudge_global
        self._max_n_integrators = max_n_integrators
        self._MCS_rescale_factor = rescale_MCS
        self._fast_MCS_mode = bool(fast_MCS_mode)     # shower.py:147-151
        self._precision = precision
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        self._seed = int(seed)
        self._next_primary = 0          # successive showers use fresh streams
        self._engine = SMEngine(self.tables, device)

    # ------------------------------------------------------------- accessors
    def get_dict_dir(self):
        return self._dict_dir

    def get_target_material(self):
        return self._target_material

    def get_material_properties(self):
        return self._ZTarget, self._ATarget, self._rhoTarget, self._dEdx

    def get_n_targets(self):
        return self.tables.n_target, self.tables.n_elec

    def _opts(self, GlobalMS=True, precision=None):
        return SMEngine.opts(self.min_energy, self._max_n_integrators, self._MCS_rescale_factor,
                             ms=GlobalMS, precision=precision or self._precision, seed=self._seed,
                             fast_MCS_mode=self._fast_MCS_mode)

    # ------------------------------------------------------------- n*sigma
    def _ns(self, slot, E):
        x, y = self.tables.nsigma[slot]
        E = np.asarray(E, dtype=np.float64)
        return np.where((E < x[0]) | (E > x[-1]), 0.0, np.interp(E, x, y))

    def get_mfp(self, particle):
        """Mean free path in metres (shower.py:370-389)."""
        if isinstance(particle, (list, tuple, np.ndarray)):
            PID, E = particle
        else:
            PID, E = particle.get_ids()["PID"], particle.get_pf()[0]
        slots = {22: (T.NS_PP, T.NS_COMP), 11: (T.NS_BREM, T.NS_MOLLER),
                 -11: (T.NS_BREM, T.NS_BHABHA, T.NS_ANN)}.get(PID, (T.NS_MUONBREM, T.NS_MUONE))
        ns = sum(self._ns(s, E) for s in slots)
        if ns <= 0.0:
            return 1.0e12
        return T.CMTOM / ns

    # ------------------------------------------------------------- sampling
    def draw_sample(self, Einc, LU_Key=-1, process="PairProd", VB=False, pkey=None):
        """Draws final-state variables from the trained map (shower.py:401-465).

        ``pkey`` selects the random stream (default: a fresh one per call)."""
        if process not in T.PROCESS_CODE:
            raise Exception("Your process is not in the list")
        if pkey is None:
            pkey = np.uint64(_stream_key(self._next_primary))
            self._next_primary += 1
        x, props, _ = self._engine.sample_only(T.PROCESS_CODE[process], [Einc], [pkey], self._opts())
        x = x[0, :T.DIMENSIONS[process]]
        if VB:
            return np.concatenate([x, [props[0]]])
        return x

    # ------------------------------------------------------------- showers
    def generate_showers(self, p0, r0=None, pid=11, mass=None, weight=1.0, GlobalMS=True,
                         precision=None, first_primary=None) -> ShowerBatch:
        """Batched generate_shower: p0 (n,4) four-momenta, r0 (n,3) positions,
        pid (n,) or scalar.  Returns every particle of every shower."""
        p0 = np.atleast_2d(np.asarray(p0, np.float64))
        n = len(p0)
        r0 = np.zeros((n, 3)) if r0 is None else np.asarray(r0, np.float64).reshape(n, 3)
        pid = np.broadcast_to(np.asarray(pid, np.int32), (n,)).copy()
        for q in np.unique(pid):
            if int(q) not in SUPPORTED_PIDS:
                raise ValueError(f"PID {int(q)} is not transported by the shower path")
        if mass is None:
            mass = np.array([MASS[int(q)] for q in pid])
        mass = np.broadcast_to(np.asarray(mass, np.float64), (n,)).copy()
        weight = np.broadcast_to(np.asarray(weight, np.float64), (n,)).copy()
        if first_primary is None:
            first_primary = self._next_primary
            self._next_primary += n
        opts = self._opts(GlobalMS, precision)
        opts.primary_offset = int(first_primary)      # primary i uses stream first_primary + i
        st, rows = self._engine.run_sm(p0, r0, pid, mass, weight, opts)
        return ShowerBatch(st.to_numpy(rows), n)

    def run_tallied(self, p0, pid=11, mass=None, r0=None, GlobalMS=True, precision=None, first_primary=None,
                    z_max=None, queue_capacity=0) -> dict:
        """Transports many primaries without keeping particle lists and returns
        host tallies: counts, energy sums, histograms and per-primary arrays.

        p0 (n,4) and pid/mass (n,) may be numpy arrays or (pinned) CPU torch
        tensors; they are copied to the device inside this call."""
        import torch
        dev = self._engine.device
        p0t = torch.as_tensor(p0, dtype=torch.float64)
        n = p0t.shape[0]
        pidt = torch.as_tensor(np.broadcast_to(np.asarray(pid, np.int32), (n,)).copy()) if not torch.is_tensor(pid) \
            else pid.to(torch.int32)
        # one comparison pass per supported PID (no sort of the batch)
        known = torch.zeros(pidt.shape, dtype=torch.bool, device=pidt.device)
        for q in SUPPORTED_PIDS:
            known |= pidt == q
        if not bool(known.all()):
            raise ValueError(f"PID {int(pidt[~known].min())} is not transported by the shower path")
        if mass is None:
            mass = torch.zeros(pidt.shape, dtype=torch.float64, device=pidt.device)
            for q in SUPPORTED_PIDS:
                mass[pidt == q] = MASS[q]
        mt = torch.as_tensor(mass, dtype=torch.float64)
        if mt.dim() == 0:                               # one mass for every primary
            mt = mt.expand(n).contiguous()
        if mt.shape != (n,) or pidt.shape != (n,) or tuple(p0t.shape) != (n, 4):
            raise ValueError(f"run_tallied: p0 (n,4), pid and mass (n,) expected, got {tuple(p0t.shape)}, "
                             f"{tuple(pidt.shape)}, {tuple(mt.shape)}")
        P0 = p0t.to(dev, non_blocking=True).t().contiguous()
        R0 = (torch.zeros((3, n), dtype=torch.float64, device=dev) if r0 is None
              else torch.as_tensor(r0, dtype=torch.float64).to(dev, non_blocking=True).t().contiguous())
        PID = pidt.to(dev, non_blocking=True)
        M = mt.to(dev, non_blocking=True)
        if first_primary is None:
            first_primary = self._next_primary
            self._next_primary += n
        opts = self._opts(GlobalMS, precision)
        opts.primary_offset = int(first_primary)
        zmax = z_max if z_max is not None else 30.0 * radiation_length_m(self._target_material)
        t = self._engine.new_tally(n, zmax)
        extra = self._run_batch_tallied(opts, t, queue_capacity, (P0, R0, PID, M))
        out = t.summary()
        out.update(extra)
        out["hist"] = t.hist.cpu().numpy()
        out["primary_count"] = t.primary_count.cpu().numpy()
        out["primary_edep"] = t.primary_edep.cpu().numpy()
        out["z_max"] = zmax
        return out

    def _run_batch_tallied(self, opts, tally, queue_capacity, device_inputs) -> dict:
        self._engine.run_batch(None, None, None, None, opts, tally, queue_capacity, device_inputs=device_inputs)
        return {}

    def generate_shower(self, p0, VB=False, GlobalMS=True):
        """Generates a particle shower from an initial particle (shower.py:603-708)."""
        ids = p0.get_ids()
        if ids.get("stability", "stable") != "stable":
            raise NotImplementedError("decays of unstable primaries are outside the shower path")
        p0.set_ended(False)
        p0copy = copy.deepcopy(p0)
        if p0.get_p0()[0] < self.min_energy:
            p0.set_ended(True)
            return [p0copy]
        mass = ids["mass"]
        b = self.generate_showers(np.asarray(p0.get_p0(), np.float64)[None], np.asarray(p0.get_r0(), np.float64)[None],
                                  pid=ids["PID"], mass=mass, weight=ids["weight"], GlobalMS=GlobalMS)
        return batch_to_particles(b, [p0copy])[0]


def radiation_length_m(target):
    """Approximate radiation length (PDG, m) used only to size depth histograms."""
    return {"lead": 0.0056, "graphite": 0.19, "iron": 0.0176, "tungsten": 0.0035, "aluminum": 0.089,
            "molybdenum": 0.0096, "hydrogen": 7.5}.get(target, 0.1)


def _stream_key(i):
    from .engine import primary_key
    return primary_key(i)   # host copy of the device's key derivation


def batch_to_particles(b: ShowerBatch, primaries):
    """Builds PETITE Particle lists (one per primary) from a ShowerBatch."""
    order = b.order
    out = [[] for _ in range(b.n_primaries)]
    ids_of = {}
    for r in order:
        k = int(b.primary[r])
        if b.parent[r] < 0:
            part = primaries[k]
            part.set_pf(b.pf[r].copy())
            part.set_rf(b.rf[r].copy())
            part.set_ended(True)
            part._pkey = int(b.pkey[r])
            ids_of[r] = (part.get_ids()["ID"], part.get_ids()["generation_number"], part.get_ids()["PID"])
            out[k].append(part)
            continue
        pr = int(b.parent[r])
        pid_parent, gen_parent, pdg_parent = ids_of[pr]
        my_id = 2 * pid_parent + int(b.bit[r])
        d = {"PID": int(b.pid[r]), "parent_PID": pdg_parent, "ID": my_id, "parent_ID": pid_parent,
             "generation_number": gen_parent + 1, "generation_process": T.PROCESSES[int(b.proc[r])],
             "weight": float(b.weight[r]), "mass": float(b.mass[r])}
        part = Particle(b.p0[r].copy(), b.r0[r].copy(), d)
        part.set_pf(b.pf[r].copy())
        part.set_rf(b.rf[r].copy())
        part.set_ended(True)
        part._pkey = int(b.pkey[r])          # random-stream key (dark production draws from it)
        ids_of[r] = (my_id, gen_parent + 1, int(b.pid[r]))
        out[k].append(part)
    return out


# ------------------------------------------------------- detector acceptance
def transverse_position(particle, z):
    """shower.py:815-823: (x, y) where the particle's initial straight line
    (r0 along p0) reaches longitudinal position(s) z."""
    x0, y0, z0 = particle.get_r0()
    E, px, py, pz = particle.get_p0()
    T = (np.asarray(z) - z0) / pz
    return [x0 + T * px, y0 + T * py]


def detector_cut(particle_list, detector_positions, detector_radius, method="Sample", energy_cut=None,
                 detector_inner_radius=0.0):
    """shower.py:825-865: which particles cross disk detectors at the
    longitudinal positions ``detector_positions`` (an annulus between
    ``detector_inner_radius`` and ``detector_radius``, both exclusive), after
    an optional open energy window ``energy_cut`` = (min, max).  ``method``:
    "Sample" (the passing particles per detector), "SampleW" (the pass mask,
    detectors by particles), "Efficiency" (weighted fraction per detector) or
    "TotalWeight".  Evaluated on arrays of all particles at once."""
    parts = np.array(particle_list, dtype=object)
    if energy_cut is not None and len(parts):
        E = np.array([p.get_p0()[0] for p in parts])
        parts = parts[(E < energy_cut[1]) & (E > energy_cut[0])]
    nd = len(detector_positions)
    if len(parts) == 0:
        return [[] for _ in range(nd)] if method == "Sample" else [0.0 for _ in range(nd)]
    r0 = np.array([p.get_r0() for p in parts], dtype=np.float64)
    p0 = np.array([p.get_p0() for p in parts], dtype=np.float64)
    z = np.asarray(detector_positions, dtype=np.float64)
    T = (z[None, :] - r0[:, 2:3]) / p0[:, 3:4]
    xf, yf = r0[:, 0:1] + T * p0[:, 1:2], r0[:, 1:2] + T * p0[:, 2:3]
    rT = np.sqrt(xf * xf + yf * yf)                                   # (particles, detectors)
    passed = ((rT > detector_inner_radius) & (rT < detector_radius)).T
    if method == "SampleW":
        return passed
    cuts = [parts[passed[i]] for i in range(nd)]
    if method == "Sample":
        return cuts
    w = np.array([p.get_ids()["weight"] for p in parts], dtype=np.float64)
    if method == "Efficiency":
        return [np.sum(w[passed[i]]) / np.sum(w) for i in range(nd)]
    if method == "TotalWeight":
        return [np.sum(w[passed[i]]) for i in range(nd)]
    return None


def _soa_columns(t, ncomp, dev):
    """(n, ncomp) float64 rows on ``dev`` as (base tensor, column stride,
    first column): a column-major view (strides (1, S), e.g.
    ``store.t["p0"][:, :n].T``) is used in place, anything else is copied
    into SoA form."""
    import torch
    t = torch.as_tensor(t, dtype=torch.float64, device=dev)
    if t.dim() != 2 or t.shape[1] != ncomp:
        raise ValueError(f"expected an (n, {ncomp}) array, got shape {tuple(t.shape)}")
    if t.shape[0] > 0 and t.stride(0) == 1 and t.stride(1) >= t.shape[0]:
        return t, t.stride(1), t[:, 0]
    s = t.T.contiguous()
    return s, max(t.shape[0], 1), s[0]


def detector_cut_rows(p0, r0, weight, detector_positions, detector_radius, method="Sample", energy_cut=None,
                      detector_inner_radius=0.0, device=None, stream=None):
    """detector_cut (shower.py:825-865) on particle rows held as arrays, on
    the GPU (``pt_detector_cut``): p0 (n, 4) four-momenta, r0 (n, 3)
    positions, weight (n,) or None (weights 1), as numpy arrays or torch
    tensors; device tensors in SoA layout (``ParticleStore.t["p0"][:, :n].T``,
    the dark run's ``p4`` buffer) are read in place.

    Same arguments and acceptance as ``detector_cut``; the results index the
    rows instead of holding Particle objects:
      "SampleW": bool tensor (n_detectors, n) on the device, False for rows
                 outside ``energy_cut`` (the list form keeps only the rows
                 inside it);
      "Sample": per detector, the int64 indices of the rows that pass;
      "Efficiency": per detector, passing weight / weight in the window
                    (0.0 when no row is in the window);
      "TotalWeight": per detector, the passing weight."""
    import ctypes as C
    import torch
    from . import _lib
    dev = torch.device(device) if device is not None else (
        p0.device if torch.is_tensor(p0) and p0.is_cuda else torch.device("cuda"))
    P, ps, E = _soa_columns(p0, 4, dev)
    R, rs, _ = _soa_columns(r0, 3, dev)
    n = int(p0.shape[0])
    if int(r0.shape[0]) != n:
        raise ValueError("p0 and r0 must have the same number of rows")
    W = None
    if weight is not None:
        W = torch.as_tensor(weight, dtype=torch.float64, device=dev).contiguous()
        if W.shape != (n,):
            raise ValueError(f"weight must have shape ({n},), got {tuple(W.shape)}")
    zs = torch.as_tensor(np.asarray(detector_positions, dtype=np.float64).reshape(-1), device=dev)
    nd = int(zs.numel())
    want_mask = method in ("SampleW", "Sample")
    mask = torch.zeros((nd, n), dtype=torch.uint8, device=dev) if want_mask else None
    sums = torch.zeros(nd + 1, dtype=torch.float64, device=dev)
    win = energy_cut is not None
    lo, hi = (float(energy_cut[0]), float(energy_cut[1])) if win else (0.0, 0.0)
    st = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    lib = _lib.load()
    s = lib.pt_detector_cut(C.c_void_p(P.data_ptr()), ps, C.c_void_p(R.data_ptr()), rs,
                            C.c_void_p(W.data_ptr()) if W is not None else None, n,
                            C.c_void_p(zs.data_ptr()) if nd else None, nd, float(detector_inner_radius),
                            float(detector_radius), int(win), lo, hi,
                            C.c_void_p(mask.data_ptr()) if mask is not None else None, C.c_void_p(sums.data_ptr()),
                            C.c_void_p(st))
    _lib.check(s, "pt_detector_cut")
    if method == "SampleW":
        return mask.bool()
    if method == "Sample":
        return [torch.nonzero(mask[d], as_tuple=True)[0] for d in range(nd)]
    if method not in ("Efficiency", "TotalWeight"):
        return None
    tot = sums.cpu().numpy()
    if method == "TotalWeight":
        return [float(v) for v in tot[:nd]]
    in_window = bool(((E < hi) & (E > lo)).any()) if win else n > 0
    if not in_window:
        return [0.0] * nd
    return [float(v / tot[nd]) for v in tot[:nd]]
