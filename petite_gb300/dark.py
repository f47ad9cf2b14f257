"""Drop-in ``DarkShower`` (PETITE dark_shower.py) on the CUDA engine, and the
differentiable dark-vector yield.

``DarkShower`` keeps PETITE's constructor and methods (``GetBSMWeights``,
``draw_dark_sample``, ``produce_bsm_particle``, ``generate_dark_shower``);
the dark-vector production runs in ``pt_run_dark`` over the SM particle
rows.  Tables come from the dict_dir, as PETITE reads them: its
``dark_maps.pkl`` and ``dark_xsec.pkl`` (with the ``dark_weights.pkl`` and
``dark_drate.pkl`` caches), from which ``petite_gb300.darktables`` builds
the weight, dR/dE and bound-electron tables PETITE's constructor builds
(dark_shower.py:219-593); or a ``dark_tables.npz`` bundle of the same
content.  Bundled: ``data/dark_tables.npz`` (six masses, five targets), and
``data/400GeV/dark_tables.npz`` for the 400 GeV tables (mV = 0.1 GeV, five
targets): the dark VEGAS maps (PETITE's shipped ``<Process>/mV_*`` maps, or
maps trained by ``petite_gb300.train`` where PETITE ships none, with max_F
from find_maxes) and the constructor's tables.

``dark_yield`` is a ``torch.autograd.Function``: forward = the map estimate
of a dark cross section and its V-energy moment at fixed Philox uniforms
(``pt_dark_yield``), backward = the hand-written adjoint kernel
(``pt_dark_yield_adjoint``), d/dmV through the DarkBrem, DarkComp and DarkAnn
differential cross sections.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import warnings

import numpy as np

from . import _lib
from . import tables as T
from .particle import Particle
from .shower import Shower, _stream_key

DARK_PROCESSES = ("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")          # engine codes 0..3
DARK_CODE = {p: i for i, p in enumerate(DARK_PROCESSES)}
DARK_PROCESS_CODES = ["DarkBrem", "DarkAnn", "DarkComp", "TwoBody_BSMDecay", "DarkMuonBrem"]   # dark_shower.py:49
DIMENSIONALITIES_DARK = {"DarkComp": 1, "DarkBrem": 3, "DarkAnn": 1, "DarkMuonBrem": 3}     # dark_shower.py:67
V_PID = 4900022
TWOBODY = "TwoBody_BSMDecay"
MESON_TWOBODY_BR_PI0 = 0.98823                  # meson_twobody_branchingratios[111], particle.py:39-48
DARK_NPZ = os.path.join(T.BUNDLED_DIR, "dark_tables.npz")
_TABLES = ("brem_elec", "brem_positron", "ann", "muon_brem")
# DarkShower.run_tallied's vector-energy histogram: log bins over
# [1e-3, 1e3] GeV (under- and overflow in the end bins)
DARK_HIST_BINS = 60
DARK_HIST_E = (1e-3, 1e3)


def processes_at_mass(processes, mV: float):
    """``processes`` without DarkAnn below mV = 2 m_e, where e+ e- -> V has
    no resonance (its energy lies below the positron's rest mass) and no
    map set exists."""
    return [p for p in processes if p != "DarkAnn" or mV >= 2 * T.M_ELECTRON]


def closest_lesser_value(input_list, input_value):
    """dark_shower.py:158-165 for values at or above the smallest mass."""
    arr = np.asarray(input_list, dtype=float)
    index = int(np.abs(arr - input_value).argmin())
    if arr[index] <= input_value:
        return float(arr[index])
    if index == 0:
        raise ValueError(f"no dark map at or below mV = {input_value} GeV (smallest: {arr.min()} GeV)")
    return float(arr[index - 1])


class DarkData:
    """Content of ``dark_tables.npz`` (all masses and targets), or the same
    content built from a PETITE dict_dir's dark pickles (``from_pickles``)."""

    def __init__(self, path: str = DARK_NPZ, content=None):
        if content is None:
            if not os.path.exists(path):
                raise FileNotFoundError(path)
            content = np.load(path, allow_pickle=False)
        self.z = content
        self.masses = [float(m) for m in self.z["masses"]]
        self.targets = [str(t) for t in self.z["targets"]]

    @classmethod
    def from_pickles(cls, dict_dir: str, sm_for_target, Zeff: float = 29.508):
        """``dark_maps.pkl`` + ``dark_xsec.pkl`` (+ the ``dark_weights.pkl`` and
        ``dark_drate.pkl`` caches) of a PETITE dict_dir: maps up front, each
        (mass, target)'s tables built on first use (``petite_gb300.darktables``)."""
        from .darktables import PickleTables
        return cls(content=PickleTables(dict_dir, sm_for_target, Zeff))

    def use_mass(self, mV: float) -> None:
        """The vector mass of the thresholds and bound-electron cross sections
        of tables built from pickles (PETITE's ``_mV``, which differs from the
        map mass in mode='approx'); the bundled tables are at the map mass."""
        if hasattr(self.z, "mV_actual"):
            self.z.mV_actual = float(mV)

    def maps_for(self, target: str, fudge: float):
        """Dense map arrays of every mass for one target (pt_dark_maps layout)."""
        if target not in self.targets:
            raise Exception("Target Material is not in library")
        j = self.targets.index(target)
        energy, maxF, neval, offs, ninc, nodes = [], [], [], [], [], []
        base = np.zeros((_lib.DARK_MAX_MASSES, _lib.N_DARK), np.int32)
        rows = np.zeros_like(base)
        n_rows = n_nodes = 0
        for m, mv in enumerate(self.masses):
            for p, name in enumerate(DARK_PROCESSES):
                pre = f"m{mv}/{name}"
                if f"{pre}/energy" not in self.z:      # no maps (DarkAnn below mV = 2 m_e)
                    base[m, p], rows[m, p] = n_rows, 0
                    continue
                E = self.z[f"{pre}/energy"]
                grid, nn = self.z[f"{pre}/grid"], self.z[f"{pre}/nnodes"]
                base[m, p], rows[m, p] = n_rows, len(E)
                for i in range(len(E)):
                    o = np.zeros(4, np.int64)
                    c = np.zeros(4, np.int32)
                    for k in range(grid.shape[1]):
                        g = grid[i, k, :nn[i, k]]
                        o[k], c[k] = n_nodes, len(g) - 1
                        nodes.append(g)
                        n_nodes += len(g)
                    offs.append(o)
                    ninc.append(c)
                energy.append(E)
                maxF.append(self.z[f"{pre}/max_F"][:, j] * fudge)
                neval.append(self.z[f"{pre}/neval"].astype(np.float64))
                n_rows += len(E)
        return dict(energy=np.concatenate(energy), maxF=np.concatenate(maxF), neval=np.concatenate(neval),
                    offset=np.concatenate(offs), ninc=np.concatenate(ninc), nodes=np.concatenate(nodes),
                    base=base, rows=rows)

    def params_for(self, mV_est: float, target: str, bound_electron: bool = True) -> dict:
        """The tables of one (mass, target).  bound_electron=False swaps in the
        free-electron DarkAnn/DarkComp cross sections, annihilation weights and
        dR/dE, thresholds, and the positron interaction integrals."""
        pre = f"m{mV_est}/{target}"
        z = self.z
        out = {"E_res": float(z[f"{pre}/E_res"]), "E_compth": float(z[f"{pre}/E_compth"]),
               "min_dark": z[f"{pre}/min_dark"].astype(np.float64),
               "xsec_DarkComp": z[f"{pre}/xsec/DarkComp_bound"]}
        for k in _TABLES:
            out[f"w/{k}"] = z[f"{pre}/weights/{k}"]
            out[f"dr/{k}/Ei"] = z[f"{pre}/drate/{k}/Ei"]
            out[f"dr/{k}/bins"] = z[f"{pre}/drate/{k}/bins"]
            out[f"dr/{k}/nbins"] = z[f"{pre}/drate/{k}/nbins"].astype(np.int32)
        if not bound_electron:
            f = f"{pre}/free"
            if f"{f}/xsec/DarkAnn" not in z:
                raise Exception("Process String does not match library")     # dark_shower.py:210
            out["min_dark"] = z[f"{f}/min_dark"].astype(np.float64)
            out["xsec_DarkComp"] = z[f"{f}/xsec/DarkComp"]
            out["ann_E0"] = float(z[f"{f}/xsec/DarkAnn"][0, 0])
            out["w/ann"] = z[f"{f}/weights/ann"]
            out["dr/ann/Ei"] = z[f"{f}/drate/ann/Ei"]
            out["dr/ann/bins"] = z[f"{f}/drate/ann/bins"]
            out["dr/ann/nbins"] = z[f"{f}/drate/ann/nbins"].astype(np.int32)
            for k in ("Brem", "Ann", "Bhabha"):
                out[f"ii/{k}"] = z[f"{target}/ii/{k}"]
        return out


class DarkEngine:
    """Device copy of one target's dark maps bound to an SM engine handle."""

    def __init__(self, sm_engine, data: DarkData, target: str, fudge: float = 1.0):
        import torch
        self.sm = sm_engine
        self.lib = sm_engine.lib
        self.device = sm_engine.device
        self.data = data
        mp = data.maps_for(target, fudge)
        dev = self.device
        self._keep = {k: torch.as_tensor(np.ascontiguousarray(v), device=dev)
                      for k, v in (("energy", mp["energy"]), ("maxF", mp["maxF"]), ("neval", mp["neval"]),
                                   ("offset", mp["offset"].reshape(-1)), ("ninc", mp["ninc"].reshape(-1)),
                                   ("nodes", mp["nodes"]))}
        M = _lib.PtDarkMaps()
        M.n_masses = len(data.masses)
        for m, mv in enumerate(data.masses):
            M.mass[m] = mv
        for m in range(_lib.DARK_MAX_MASSES):
            for p in range(_lib.N_DARK):
                M.map_base[m * _lib.N_DARK + p] = int(mp["base"][m, p])
                M.map_rows[m * _lib.N_DARK + p] = int(mp["rows"][m, p])
        M.n_rows = len(mp["energy"])
        M.map_energy, M.map_maxF, M.map_neval = (self._keep[k].data_ptr() for k in ("energy", "maxF", "neval"))
        M.grid_offset, M.grid_ninc, M.grid_nodes = (self._keep[k].data_ptr() for k in ("offset", "ninc", "nodes"))
        M.n_nodes = len(mp["nodes"])
        # float32 (node, increment to the next node) for the float32 proposals
        nodes = np.asarray(mp["nodes"], np.float64)
        inc = np.zeros_like(nodes)
        for o, c in zip(mp["offset"].reshape(-1), mp["ninc"].reshape(-1)):
            if c > 0:
                inc[o:o + c] = nodes[o + 1:o + c + 1] - nodes[o:o + c]
        self._keep["f32x2"] = torch.as_tensor(np.ascontiguousarray(np.stack([nodes, inc], axis=1).astype(np.float32)),
                                              device=dev)
        M.grid_f32x2 = self._keep["f32x2"].data_ptr()
        ti = T.TARGET_INFORMATION[target]
        M.Z, M.A = float(ti["Z_T"]), float(ti["A_T"])
        self._M = M
        h = C.c_void_p()
        _lib.check(self.lib.pt_dark_create(sm_engine.handle, C.byref(M), C.byref(h)), "pt_dark_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pt_dark_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def has_maps(self, process: str):
        """Per mass, whether ``process`` has a map set there."""
        p = DARK_CODE[process]
        return [self._M.map_rows[m * _lib.N_DARK + p] >= 2 for m in range(len(self.data.masses))]

    def mass_index(self, mV_est: float) -> int:
        return [abs(m - mV_est) < 1e-12 for m in self.data.masses].index(True)

    # ------------------------------------------------------------ entry points
    def dsigma(self, process: int, x, energy, mV: float):
        import torch
        x = np.atleast_2d(np.asarray(x, np.float64))
        xp = np.zeros((len(x), 4))
        xp[:, :x.shape[1]] = x
        X = torch.as_tensor(xp, device=self.device)
        E = torch.as_tensor(np.asarray(energy, np.float64), device=self.device)
        out = torch.empty(len(xp), dtype=torch.float64, device=self.device)
        _lib.check(self.lib.pt_dark_dsigma(self.handle, process, X.data_ptr(), E.data_ptr(), len(xp), float(mV),
                                           out.data_ptr(), self.sm._stream()), "pt_dark_dsigma")
        return out.cpu().numpy()

    def screen32(self, process: int, x, energy, mV: float):
        """The float32 dark-brem screen (pt_dark_screen32): (value, code)."""
        import torch
        x = np.atleast_2d(np.asarray(x, np.float64))
        xp = np.zeros((len(x), 4))
        xp[:, :x.shape[1]] = x
        X = torch.as_tensor(xp, device=self.device)
        E = torch.as_tensor(np.asarray(energy, np.float64), device=self.device)
        val = torch.empty(len(xp), dtype=torch.float32, device=self.device)
        code = torch.empty(len(xp), dtype=torch.int32, device=self.device)
        _lib.check(self.lib.pt_dark_screen32(self.handle, process, X.data_ptr(), E.data_ptr(), len(xp), float(mV),
                                             val.data_ptr(), code.data_ptr(), self.sm._stream()), "pt_dark_screen32")
        return val.cpu().numpy(), code.cpu().numpy()

    def sample_only(self, prm, process: int, energy, keys, opts):
        import torch
        E = torch.as_tensor(np.asarray(energy, np.float64), device=self.device)
        K = torch.as_tensor(np.asarray(keys, np.uint64).view(np.int64), device=self.device)
        n = len(E)
        x = torch.empty((n, 4), dtype=torch.float64, device=self.device)
        props = torch.empty(n, dtype=torch.int64, device=self.device)
        lk = torch.empty(n, dtype=torch.int32, device=self.device)
        _lib.check(self.lib.pt_dark_sample_only(self.handle, C.byref(prm), process, E.data_ptr(), K.data_ptr(), n,
                                                C.byref(opts), x.data_ptr(), props.data_ptr(), lk.data_ptr(),
                                                self.sm._stream()), "pt_dark_sample_only")
        return x.cpu().numpy(), props.cpu().numpy(), lk.cpu().numpy()

    def run_dark(self, prm, store, n_rows: int, opts, capacity: int | None = None, keep_records=True):
        """Dark vectors of the first n_rows of a ParticleStore: dict of numpy
        arrays (p4, r, weight, parent, process, draws) and the yields."""
        import torch
        dev = self.device
        yld = torch.zeros(_lib.N_DARK + 1, dtype=torch.float64, device=dev)
        yldE = torch.zeros(_lib.N_DARK + 1, dtype=torch.float64, device=dev)
        if capacity is None:
            capacity = max(16, 4 * n_rows)
        while True:
            o = _lib.PtDarkOut()
            bufs = {}
            if keep_records:
                bufs = {"p4": torch.empty((4, capacity), dtype=torch.float64, device=dev),
                        "r": torch.empty((3, capacity), dtype=torch.float64, device=dev),
                        "weight": torch.empty(capacity, dtype=torch.float64, device=dev),
                        "parent": torch.empty(capacity, dtype=torch.int64, device=dev),
                        "process": torch.empty(capacity, dtype=torch.int32, device=dev),
                        "draws": torch.empty(capacity, dtype=torch.int32, device=dev)}
                for k, v in bufs.items():
                    setattr(o, k, v.data_ptr())
            o.capacity = capacity
            o.yield_ = yld.data_ptr()
            o.yield_E = yldE.data_ptr()
            abi = store.abi()
            n_out = C.c_int64()
            s = self.lib.pt_run_dark(self.handle, C.byref(prm), C.byref(abi), int(n_rows), C.byref(opts), C.byref(o),
                                     C.byref(n_out), self.sm._stream())
            if s == _lib.PT_OOM and keep_records:
                capacity *= 2
                yld.zero_()
                yldE.zero_()
                continue
            _lib.check(s, "pt_run_dark")
            break
        n = int(n_out.value)
        out = {k: (v[..., :n].cpu().numpy()) for k, v in bufs.items()}
        if not keep_records:
            out = {}
        if "p4" in out:
            out["p4"], out["r"] = out["p4"].T.copy(), out["r"].T.copy()
        out["yield"] = yld.cpu().numpy()
        out["yield_E"] = yldE.cpu().numpy()
        out["n"] = n
        return out

    def run_batch(self, prms, p0, r0, pid, mass, opts, tally, queue_capacity: int = 0, device_inputs=None,
                  hist=None):
        """The SM engine's batched transport with dark vectors produced on
        every wave (pt_run_batch_dark) for each parameter set in ``prms``
        (one pt_dark_params, or a list: several masses on the same showers):
        returns (tally, yield [sets, N_DARK+1], yield_E [sets, N_DARK+1],
        vectors), and with ``hist`` = (bins, log10 E_lo, log10 E_hi) the
        vectors' energy histogram [sets, N_DARK+1, bins] as a fifth item;
        the yields and histogram as numpy arrays."""
        import torch
        prms = [prms] if isinstance(prms, _lib.PtDarkParams) else list(prms)
        arr = (_lib.PtDarkParams * len(prms))(*prms)
        yld = torch.zeros((len(prms), _lib.N_DARK + 1), dtype=torch.float64, device=self.device)
        yldE = torch.zeros_like(yld)
        counts = h = None
        if hist is not None:
            bins, lo, hi = hist
            counts = torch.zeros((len(prms), _lib.N_DARK + 1, int(bins)), dtype=torch.float64, device=self.device)
            h = _lib.PtDarkHist()
            h.counts, h.bins, h.log10_lo, h.log10_hi = counts.data_ptr(), int(bins), float(lo), float(hi)
        tally, nv = self.sm.run_batch(p0, r0, pid, mass, opts, tally, queue_capacity, device_inputs,
                                      dark=(self.handle, arr, yld, yldE, h, counts))
        out = (tally, yld.cpu().numpy(), yldE.cpu().numpy(), nv)
        return out + (counts.cpu().numpy(),) if counts is not None else out

    def yield_forward(self, process: int, energy, mV, mass_index, n_samples: int, seed: int, anchor=None):
        import torch
        n = energy.shape[0]
        Y = torch.empty(n, dtype=torch.float64, device=self.device)
        M = torch.empty(n, dtype=torch.float64, device=self.device)
        aptr = None if anchor is None else anchor.data_ptr()
        _lib.check(self.lib.pt_dark_yield(self.handle, process, energy.data_ptr(), mV.data_ptr(), aptr,
                                          mass_index.data_ptr(), n, int(n_samples), int(seed) & (2 ** 64 - 1),
                                          Y.data_ptr(), M.data_ptr(), self.sm._stream()), "pt_dark_yield")
        return Y, M

    def yield_adjoint(self, process: int, energy, mV, mass_index, n_samples: int, seed: int, gY, gM):
        import torch
        n = energy.shape[0]
        g = torch.empty(n, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.pt_dark_yield_adjoint(self.handle, process, energy.data_ptr(), mV.data_ptr(),
                                                  mass_index.data_ptr(), n, int(n_samples),
                                                  int(seed) & (2 ** 64 - 1), gY.data_ptr(), gM.data_ptr(),
                                                  g.data_ptr(), self.sm._stream()), "pt_dark_yield_adjoint")
        return g


def _ann_K(sh) -> float:
    """(1/dEdxT_GeVpercm) (2 pi^2 alpha/m_e) n_e GeVsqcm2 in the order of
    dark_shower.py:627 (the free-electron resonant DarkAnn weight's prefactor)."""
    dEdxT_GeVpercm = sh.get_material_properties()[3] * (0.1) * T.CMTOM
    return (1 / dEdxT_GeVpercm) * (2 * np.pi ** 2 * T.ALPHA_EM / T.M_ELECTRON) * (sh.get_n_targets()[1]) * T.GEVSQCM2


def _active_bits(processes) -> int:
    """pt_dark_params.active: bit p for engine process p, bit TWOBODY for the meson decay."""
    bits = sum(1 << DARK_CODE[p] for p in processes if p in DARK_CODE)
    return bits | ((1 << _lib.TWOBODY) if TWOBODY in processes else 0)


def _dark_params(engine: DarkEngine, sh, mV_est: float, mV: float, bound: bool, active, coupling, Zeff,
                 precision: str = "fp64"):
    """pt_dark_params for one DarkShower (tables kept alive on the engine)."""
    import torch
    d = engine.data.params_for(mV_est, sh.get_target_material(), bound)
    dev = engine.device
    keep = {}
    prm = _lib.PtDarkParams()
    prm.precision = {"fp64": 0, "mixed": 1}[precision]
    prm.mass_index = engine.mass_index(mV_est)
    prm.bound_electron = 1 if bound else 0
    prm.active = _active_bits(active)
    prm.mV, prm.coupling, prm.Zeff = float(mV), float(coupling), float(Zeff)
    prm.kinetic_mixing = float(sh.kinetic_mixing)
    if not bound:
        prm.ann_E0 = d["ann_E0"]
        prm.ann_K = _ann_K(sh)
        for k, name in enumerate(("Brem", "Ann", "Bhabha")):
            t = d[f"ii/{name}"]
            keep[f"iix{k}"] = torch.as_tensor(np.ascontiguousarray(t[:, 0]), device=dev)
            keep[f"iiy{k}"] = torch.as_tensor(np.ascontiguousarray(t[:, 1]), device=dev)
            prm.ii_x[k], prm.ii_y[k], prm.ii_n[k] = keep[f"iix{k}"].data_ptr(), keep[f"iiy{k}"].data_ptr(), len(t)
    prm.E_res, prm.E_compth = d["E_res"], d["E_compth"]
    for i in range(5):
        prm.min_dark[i] = float(d["min_dark"][i])
    prm.min_calc_photon = float(sh.tables.min_calc[22])
    for k, name in enumerate(_TABLES):
        w = d[f"w/{name}"]
        keep[f"wx{k}"] = torch.as_tensor(np.ascontiguousarray(w[:, 0]), device=dev)
        keep[f"wy{k}"] = torch.as_tensor(np.ascontiguousarray(w[:, 1]), device=dev)
        prm.w_x[k], prm.w_y[k], prm.w_n[k] = keep[f"wx{k}"].data_ptr(), keep[f"wy{k}"].data_ptr(), len(w)
        keep[f"ei{k}"] = torch.as_tensor(np.ascontiguousarray(d[f"dr/{name}/Ei"]), device=dev)
        bins = d[f"dr/{name}/bins"]
        keep[f"bi{k}"] = torch.as_tensor(np.ascontiguousarray(bins), device=dev)
        keep[f"nb{k}"] = torch.as_tensor(np.ascontiguousarray(d[f"dr/{name}/nbins"]), device=dev)
        prm.dr_Ei[k], prm.dr_bins[k], prm.dr_nbins[k] = (keep[f"{a}{k}"].data_ptr() for a in ("ei", "bi", "nb"))
        prm.dr_n[k], prm.dr_nbmax[k] = bins.shape[0], bins.shape[1]
    # set_dark_NSigmas (dark_shower.py:286-297): DarkComp n*sigma, log-log with fill -20
    DCS = d["xsec_DarkComp"]
    nZ, ne = sh.get_n_targets()
    lx = np.log10(np.transpose(DCS)[0] + 1e-20)
    ly = np.log10(ne * T.GEVSQCM2 * np.transpose(DCS)[1] + 1e-20)
    keep["lx"] = torch.as_tensor(np.ascontiguousarray(lx), device=dev)
    keep["ly"] = torch.as_tensor(np.ascontiguousarray(ly), device=dev)
    prm.nsc_lx, prm.nsc_ly, prm.nsc_n = keep["lx"].data_ptr(), keep["ly"].data_ptr(), len(lx)
    return prm, keep


class DarkShower(Shower):
    """A class to reprocess an SM shower into dark-vector emissions
    (dark_shower.py:69-130)."""

    def __init__(self, dict_dir, target_material, min_energy, mV_in_GeV, mode="exact", maxF_fudge_global=1,
                 max_n_integrators=int(1e4), kinetic_mixing=1.0, Zeff=29.508, bound_electron=True, g_e=None,
                 active_processes=None, fast_MCS_mode=True, rescale_MCS=1, seed=None, device="cuda",
                 dark_tables=None, dark_precision="fp64"):
        super().__init__(dict_dir, target_material, min_energy, maxF_fudge_global=maxF_fudge_global,
                         max_n_integrators=max_n_integrators, fast_MCS_mode=fast_MCS_mode, seed=seed,
                         rescale_MCS=rescale_MCS, device=device)
        self.active_processes = list(DARK_PROCESS_CODES if active_processes is None else active_processes)
        self.kinetic_mixing = kinetic_mixing
        self.bound_electron = bound_electron
        self.Zeff = Zeff
        self.g_e = kinetic_mixing * np.sqrt(4 * np.pi * T.ALPHA_EM) if g_e is None else g_e
        # the dict_dir's dark files, as PETITE reads them (dark_shower.py:
        # 69-130): a dark_tables.npz bundle, else PETITE's dark_maps.pkl and
        # dark_xsec.pkl (tables built natively), else the bundled tables
        ddir = self.get_dict_dir()
        own = os.path.join(ddir, "dark_tables.npz")
        pkl = [os.path.exists(os.path.join(ddir, f)) for f in ("dark_maps.pkl", "dark_xsec.pkl")]
        if dark_tables:
            self._dark = DarkData(dark_tables)
        elif os.path.exists(own):
            self._dark = DarkData(own)
        elif all(pkl):
            raw = self._raw
            self._dark = DarkData.from_pickles(
                ddir, lambda t: self.tables if t == target_material else T.SMTables(raw, t), Zeff)
        else:
            if any(pkl) and os.path.realpath(ddir) != os.path.realpath(T.BUNDLED_DIR):
                have, miss = (", ".join(f for f, h in zip(("dark_maps.pkl", "dark_xsec.pkl"), pkl) if h is v)
                              for v in (True, False))
                warnings.warn(f"DarkShower: {ddir} has {have} but not {miss}; the bundled dark tables are used",
                              stacklevel=2)
            self._dark = DarkData(DARK_NPZ)
        self._mV_list = list(self._dark.masses)
        if mode == "exact":
            self._mV = closest_lesser_value(self._mV_list, mV_in_GeV)
            self._mV_estimator = self._mV
        elif mode == "approx":
            self._mV = float(mV_in_GeV)
            self._mV_estimator = closest_lesser_value(self._mV_list, mV_in_GeV)
        else:
            raise Exception("Mode not valid. Chose exact or approx.")
        self._dark.use_mass(self._mV)
        for p in self.active_processes:
            # set_dark_samples (dark_shower.py:181-202) loads a map set for
            # every active dark process
            if p in DARK_CODE and f"m{self._mV_estimator}/{p}/energy" not in self._dark.z:
                raise Exception("Process String does not match library")
        self._coupling = self.g_e ** 2 / (4 * np.pi * T.ALPHA_EM)
        self._dark_engine = DarkEngine(self._engine, self._dark, target_material, maxF_fudge_global)
        if dark_precision not in ("fp64", "mixed"):
            raise ValueError("dark_precision is 'fp64' or 'mixed'")
        self.dark_precision = dark_precision
        self._prm, self._prm_keep = _dark_params(self._dark_engine, self, self._mV_estimator, self._mV,
                                                 bound_electron, self.active_processes, self._coupling, Zeff,
                                                 dark_precision)
        pd = self._dark.params_for(self._mV_estimator, target_material)
        self._resonant_annihilation_energy = pd["E_res"]
        self._compton_threshold_energy = pd["E_compth"]

    def get_mV(self):
        return self._mV

    def _run_batch_tallied(self, opts, tally, queue_capacity, device_inputs) -> dict:
        """run_tallied of a DarkShower: the batched transport with the dark
        vectors of every particle (GetBSMWeights and produce_bsm_particle on
        each particle's row, as generate_dark_shower over the SM list) tallied:
        summed weights and weight * E_V per dark process, and the count."""
        lo, hi = math.log10(DARK_HIST_E[0]), math.log10(DARK_HIST_E[1])
        _, y, yE, nv, h = self._dark_engine.run_batch(self._prm, None, None, None, None, opts, tally, queue_capacity,
                                                      device_inputs, hist=(DARK_HIST_BINS, lo, hi))
        return {"dark_yield": {p: float(y[0, k]) for k, p in enumerate(DARK_PROCESSES)},
                "dark_yield_E": {p: float(yE[0, k]) for k, p in enumerate(DARK_PROCESSES)},
                "dark_energy_hist": {p: h[0, k] for k, p in enumerate(DARK_PROCESSES)},
                "dark_energy_edges": np.logspace(lo, hi, DARK_HIST_BINS + 1),
                "dark_vectors": int(nv)}

    # ------------------------------------------------------------- weights
    def GetBSMWeights(self, particle, process):
        """dark_shower.py:595-647, evaluated by the engine for one particle."""
        if isinstance(particle, (list, np.ndarray)):
            PID, E = particle
            part = Particle([E, 0, 0, 0], [0, 0, 0], {"PID": int(PID), "mass": 0.0})
        else:
            part = particle
        pid = part.get_ids()["PID"]
        if pid in (221, 331):
            # dark_shower.py:604: _minimum_calculable_dark_energy has no entry for eta, eta'
            raise KeyError(pid)
        if process == TWOBODY:
            return self._twobody_weight(pid, part.get_ids()["mass"])
        if process not in DARK_CODE:
            return 0.0
        return float(self._weights_of([part])[0, DARK_CODE[process]])

    def _twobody_weight(self, pid, mass):
        """dark_shower.py:633-638 for a pi0 (the pt_run_dark column PT_TWOBODY)."""
        if pid != 111:
            return 0.0
        mass_ratio = self._mV / mass
        if mass_ratio >= 1.0:
            return 0.0
        return 2 * self.kinetic_mixing ** 2 * (1.0 - mass_ratio ** 2) ** 3 * MESON_TWOBODY_BR_PI0

    def draw_dark_sample(self, Einc, LU_Key=-1, process="DarkBrem", VB=False, pkey=None):
        """dark_shower.py:649-704 (LU_Key chosen from Einc)."""
        if process not in DARK_CODE:
            raise Exception("Your process is not in the list")
        if pkey is None:
            pkey = np.uint64(_stream_key(self._next_primary))
            self._next_primary += 1
        x, props, _ = self._dark_engine.sample_only(self._prm, DARK_CODE[process], [Einc], [pkey], self._opts())
        if props[0] < 0:
            print("No Sample Found", process, Einc, LU_Key)
            return None
        x = x[0, :DIMENSIONALITIES_DARK[process]]
        return np.concatenate([x, [props[0]]]) if VB else x

    # --------------------------------------------------------- production
    def _run_particles(self, parts, processes=None, records=True):
        """Runs pt_run_dark on Particle objects (their stream keys are
        their ``_pkey`` attributes, else fresh ones)."""
        import torch
        from .engine import ParticleStore
        n = len(parts)
        st = ParticleStore(max(n, 1), self._engine.device)
        p0 = np.array([p.get_p0() for p in parts], np.float64).reshape(n, 4)
        pf = np.array([p.get_pf() for p in parts], np.float64).reshape(n, 4)
        rf = np.array([p.get_rf() for p in parts], np.float64).reshape(n, 3)
        keys = []
        for p in parts:
            k = getattr(p, "_pkey", None)
            if k is None:
                k = _stream_key(self._next_primary)
                self._next_primary += 1
                p._pkey = k
            keys.append(int(k))
        dev = self._engine.device
        st.t["p0"][:, :n] = torch.as_tensor(p0.T, device=dev)
        st.t["pf"][:, :n] = torch.as_tensor(pf.T, device=dev)
        st.t["rf"][:, :n] = torch.as_tensor(rf.T, device=dev)
        st.t["pid"][:n] = torch.as_tensor(np.array([p.get_ids()["PID"] for p in parts], np.int32), device=dev)
        st.t["mass"][:n] = torch.as_tensor(np.array([p.get_ids()["mass"] for p in parts], np.float64), device=dev)
        st.t["weight"][:n] = torch.as_tensor(np.array([p.get_ids()["weight"] for p in parts], np.float64),
                                             device=dev)
        st.t["pkey"][:n] = torch.as_tensor(np.array(keys, np.uint64).view(np.int64), device=dev)
        prm = self._prm
        if processes is not None:
            prm = _lib.PtDarkParams.from_buffer_copy(self._prm)
            prm.active = _active_bits(processes)
        return self._dark_engine.run_dark(prm, st, n, self._opts(), keep_records=records)

    def _weights_of(self, parts):
        """GetBSMWeights for a few particles on the host, with the tables and
        arithmetic of the device's weight (the single-particle API; the
        shower path evaluates the weights in pt_run_dark)."""
        W = np.zeros((len(parts), len(DARK_PROCESSES)))
        pd = self._dark.params_for(self._mV_estimator, self.get_target_material(), self.bound_electron)
        md = pd["min_dark"]
        slots = {(11, "DarkBrem"): 0, (-11, "DarkBrem"): 1, (-11, "DarkAnn"): 2, (22, "DarkComp"): 3,
                 (13, "DarkMuonBrem"): 4, (-13, "DarkMuonBrem"): 4}
        DCS = pd["xsec_DarkComp"]
        nZ, ne = self.get_n_targets()
        lx = np.log10(np.transpose(DCS)[0] + 1e-20)
        ly = np.log10(ne * T.GEVSQCM2 * np.transpose(DCS)[1] + 1e-20)
        for i, p in enumerate(parts):
            pid, E = p.get_ids()["PID"], p.get_p0()[0]
            for c, proc in enumerate(DARK_PROCESSES):
                if (pid, proc) not in slots:
                    continue
                k = slots[(pid, proc)]
                if E < md[k]:
                    continue
                if k == 3:
                    if E < self.tables.min_calc[22]:
                        continue
                    le = np.log10(E)
                    v = -20.0 if (le < lx[0] or le > lx[-1]) else np.interp(le, lx, ly)
                    W[i, c] = self._coupling * 10 ** v / (float(self._ns(T.NS_PP, E)) + float(self._ns(T.NS_COMP, E)))
                else:
                    w = pd[f"w/{_TABLES[3 if k == 4 else k]}"]
                    v = 0.0 if (E < w[0, 0] or E > w[-1, 0]) else np.interp(E, w[:, 0], w[:, 1])
                    if k == 2 and not self.bound_electron:
                        v = (v if E > pd["ann_E0"] else 0.0) + self._ann_resonant_weight(pd, E)
                    W[i, c] = self._coupling * v
        return W

    def _ann_resonant_weight(self, pd, E):
        """The closed-form resonant DarkAnn weight of free electrons
        (dark_shower.py:621-627), as pt_run_dark evaluates it."""
        me = T.M_ELECTRON
        sMAX = 2 * (me * min(pd["ann_E0"], E) + me ** 2)
        beta = (2. * T.ALPHA_EM / np.pi) * (np.log(sMAX / me ** 2) - 1.)
        Er = self._resonant_annihilation_energy

        def ii(name, x):
            t = pd[f"ii/{name}"]
            return 0.0 if (x < t[0, 0] or x > t[-1, 0]) else float(np.interp(x, t[:, 0], t[:, 1]))
        ds = (ii("Brem", E) - ii("Brem", Er)) + (ii("Ann", E) - ii("Ann", Er)) + (ii("Bhabha", E) - ii("Bhabha", Er))
        pef = 0.0 if (ds < 0.0 or Er > E) else np.exp(-ds / (self.get_material_properties()[3] * 0.1) / T.CMTOM)
        with np.errstate(invalid="ignore"):
            return _ann_K(self) * np.float64(sMAX - self._mV ** 2) ** beta * pef

    def produce_bsm_particle(self, p_original, process, weight=None, VB=False):
        """dark_shower.py:721-804 for one particle; returns a Particle or None."""
        res = self._run_particles([p_original], processes=[process])
        if res["n"] == 0:
            return None
        return self._v_particle(p_original, res, 0, weight)

    def _v_particle(self, parent, res, j, weight=None):
        ids = parent.get_ids()
        code = int(res["process"][j])
        w = float(res["weight"][j])
        if code == _lib.TWOBODY_CODE:
            # dark_shower.py:836-843: ID 2*ID+1, the vector mass given
            v = {"mass": self._mV, "PID": V_PID, "weight": w, "parent_PID": ids["PID"], "parent_ID": ids["ID"],
                 "ID": 2 * ids["ID"] + 1, "generation_number": ids["generation_number"] + 1,
                 "generation_process": TWOBODY}
            return Particle(list(res["p4"][j]), list(res["r"][j]), v)
        name = DARK_PROCESSES[code % _lib.DARK_BOUND]
        if code >= _lib.DARK_BOUND:
            name += "_bound"
        if weight is not None and w != 0.0:
            w = weight * ids["weight"]       # dark_shower.py:723-726,795: the given weight times the parent's
        # dark_shower.py:789-804: no mass given, so Particle takes the invariant's
        v = {"PID": V_PID, "parent_PID": ids["PID"], "ID": 2 * ids["ID"] + 0, "parent_ID": ids["ID"],
             "generation_number": ids["generation_number"] + 1, "generation_process": name, "weight": w}
        return Particle(list(res["p4"][j]), list(res["r"][j]), v)

    def generate_dark_shower(self, ExDir=None, SParams=None):
        """dark_shower.py:806-849: (SM shower, list of dark vectors)."""
        if ExDir is None and SParams is None:
            print("Need an existing SM shower-file directory or SM incident particle to run dark shower")
            return None
        if ExDir is not None and isinstance(ExDir, str):
            from .io import read_particle_file
            ShowerToSamp = read_particle_file(ExDir)      # PETITE's files too, without PETITE
        elif ExDir is not None and isinstance(ExDir, list):
            ShowerToSamp = ExDir
        elif isinstance(SParams, Particle):
            ShowerToSamp = self.generate_shower(SParams)
        else:
            raise ValueError("Provided SParams must be a `Particle' class object")
        active = [p for p in self.active_processes if p in DARK_CODE or p == TWOBODY]
        if active:
            for p in ShowerToSamp:
                if p.get_ids()["PID"] in (221, 331):
                    # GetBSMWeights, dark_shower.py:604: no threshold entry for eta, eta'
                    raise KeyError(p.get_ids()["PID"])
        parts = [p for p in ShowerToSamp if p.get_ids()["PID"] in (11, -11, 22, 13, -13, 111)]
        res = self._run_particles(parts, processes=active)
        # the reference's order: particle by particle, processes in active order
        rank = np.array([active.index(p) if p in active else 0 for p in (*DARK_PROCESSES, TWOBODY)])
        col = np.where(res["process"] == _lib.TWOBODY_CODE, _lib.TWOBODY, res["process"] % _lib.DARK_BOUND)
        order = np.lexsort((rank[col], res["parent"]))
        NewShower = [self._v_particle(parts[int(res["parent"][j])], res, j) for j in order]
        return ShowerToSamp, NewShower


# ------------------------------------------------------------- dark yield
class _DarkYieldFn:
    """Builds the autograd Function lazily (torch is imported on use)."""
    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            import torch

            class DarkYield(torch.autograd.Function):
                @staticmethod
                def forward(ctx, energy, mV, engine, process, mass_index, n_samples, seed):
                    Y, M = engine.yield_forward(process, energy, mV, mass_index, n_samples, seed)
                    ctx.save_for_backward(energy, mV, mass_index)
                    ctx.cfg = (engine, process, n_samples, seed)
                    return Y, M

                @staticmethod
                def backward(ctx, gY, gM):
                    energy, mV, mass_index = ctx.saved_tensors
                    engine, process, n_samples, seed = ctx.cfg
                    z = torch.zeros_like(mV)
                    gY = z if gY is None else gY.contiguous()
                    gM = z if gM is None else gM.contiguous()
                    g = engine.yield_adjoint(process, energy, mV, mass_index, n_samples, seed, gY, gM)
                    return None, g, None, None, None, None, None

            cls.fn = DarkYield
        return cls.fn


def map_mass_index(masses, mV, has_maps=None, process=None):
    """Map block per pair: the bundled mass at or below mV (the smallest one
    below the grid).  With ``has_maps`` (per mass, whether ``process`` has
    maps there) a mass without maps gives way to the nearest lower one with
    maps, else the smallest with maps; DarkAnn below mV = 2 m_e, where it
    makes no vectors, keeps a mass without DarkAnn maps if there is one, so
    that its yield is 0."""
    m = np.asarray(masses)
    mv = np.atleast_1d(np.asarray(mV, np.float64))
    idx = np.clip(np.searchsorted(m, mv, side="right") - 1, 0, len(m) - 1).astype(np.int32)
    if has_maps is None:
        return idx
    ok = np.asarray(has_maps, bool)
    if not ok.any():
        raise Exception("Process String does not match library")
    lower = np.array([max([j for j in range(i + 1) if ok[j]], default=int(np.argmax(ok))) for i in range(len(m))],
                     np.int32)
    out = lower[idx]
    if process == "DarkAnn" and not ok.all():
        below = mv < 2 * T.M_ELECTRON
        out[below] = int(np.argmin(ok))
    return out


def dark_yield(engine: DarkEngine, process: str, energy, mV, n_samples: int = 10_000, seed: int = 0,
               mass_index=None, anchor=None):
    """Differentiable dark-vector yield per (energy, mV) pair: returns
    (yield, moment) tensors; yield = mean(jac * dsigma) over the map of
    `process` at fixed uniforms, moment = mean(jac * dsigma * E_V).
    Gradients flow to mV through the hand-written adjoint kernel.
    ``anchor`` (masses): evaluate the DarkBrem estimate with its samples
    carried from the anchor masses' momentum-transfer ranges (pt_dark_yield)."""
    import torch
    dev = engine.device
    energy = torch.as_tensor(energy, dtype=torch.float64, device=dev).contiguous()
    mV = torch.as_tensor(mV, dtype=torch.float64, device=dev)
    if mass_index is None:
        mass_index = map_mass_index(engine.data.masses, mV.detach().cpu().numpy(), engine.has_maps(process), process)
    mi = torch.as_tensor(np.asarray(mass_index, np.int32), device=dev).contiguous()
    if anchor is not None:
        a = torch.as_tensor(anchor, dtype=torch.float64, device=dev).contiguous()
        with torch.no_grad():
            return engine.yield_forward(DARK_CODE[process], energy, mV.contiguous(), mi, n_samples, seed, anchor=a)
    return _DarkYieldFn.get().apply(energy, mV.contiguous(), engine, DARK_CODE[process], mi, int(n_samples),
                                    int(seed))
