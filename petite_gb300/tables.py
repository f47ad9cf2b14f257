"""Host-side tables: PETITE's pickles -> dense arrays for the CUDA engine.

``Shower(dict_dir, ...)`` reads the same files PETITE reads
(``sm_maps.pkl`` and ``sm_xsec.pkl``, ``shower.py:153-175``).  The VEGAS
``AdaptiveMap`` objects inside ``sm_maps.pkl`` are unpickled without the
``vegas`` package: a map pickles as ``vegas._vegas.AdaptiveMap(grid)``, so a
stand-in class that keeps ``grid`` is enough.

A dict_dir may instead hold ``sm_tables.npz`` (written by :func:`save_npz`),
the same content in plain arrays; the package ships one under ``data/``
built from PETITE's ``data/`` directory (maps shipped by PETITE, ``max_F``
rebuilt with PETITE's own ``find_maxes`` because ``sm_maps.pkl`` is not
shipped).

:class:`SMTables` turns the raw content for one target into the arrays the
kernels read: map rows, grids, ``max_F * fudge`` and the eight
``n*sigma(E)`` interpolation tables of ``Shower.set_NSigmas``
(``shower.py:273-295``).
"""
from __future__ import annotations

import math
import os
import pickle
from dataclasses import dataclass, field

import numpy as np

# shower.py:36 -- the engine's process codes follow the reference's.
PROCESSES = ("Brem", "Ann", "PairProd", "Comp", "Moller", "Bhabha", "MuonE", "MuonBrem")
PROCESS_CODE = {p: i for i, p in enumerate(PROCESSES)}
DIMENSIONS = {"PairProd": 4, "Comp": 1, "Brem": 4, "MuonBrem": 4, "Ann": 1,
              "Moller": 1, "Bhabha": 1, "MuonE": 1}          # shower.py:47-56

# physical_constants.py:11-38
ALPHA_EM = 1 / 137.035999
M_ELECTRON = 510.998950 * 1e-6           # 510.998950*keV
M_MUON = 105.6583755 * 1e-3             # 105.6583755*MeV
M_PROTON_GRAMS = 1.67262192369e-24
HBARC = 0.1973269804e-13
GEVSQCM2 = HBARC ** 2
CMTOM = 0.01

# physical_constants.py:49-58
TARGET_INFORMATION = {
    "graphite": dict(Z_T=6, A_T=12, mT=11.178, rho=2.210),
    "lead": dict(Z_T=82, A_T=207, mT=207.2, rho=11.35),
    "iron": dict(Z_T=26, A_T=56, mT=55.845, rho=8.00),
    "hydrogen": dict(Z_T=1, A_T=1, mT=1.0, rho=1.0),
    "aluminum": dict(Z_T=13, A_T=27, mT=26.9815385, rho=2.699),
    "tungsten": dict(Z_T=74, A_T=183.84, mT=183.84, rho=19.3),
    "molybdenum": dict(Z_T=42, A_T=95.95, mT=95.95, rho=10.2),
}
for _t in TARGET_INFORMATION.values():
    _t["dEdx"] = 2.0 * _t["rho"]          # MeV/cm

BUNDLED_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


class _MapStandIn:
    """Receives ``AdaptiveMap(grid)`` reductions from sm_maps.pkl."""

    def __init__(self, grid, *args, **kwargs):
        self.grid = [np.asarray(g, dtype=np.float64) for g in grid]


class _MapsUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if module.split(".")[0] == "vegas" and name == "AdaptiveMap":
            return _MapStandIn
        return super().find_class(module, name)


@dataclass
class MapRow:
    energy: float
    neval: int
    max_F: dict
    grid: list          # one float64 node array per dimension
    Eg_min: float | None = None
    Ee_min: float | None = None


@dataclass
class RawTables:
    """Content of sm_maps.pkl + sm_xsec.pkl, independent of target."""
    maps: dict = field(default_factory=dict)      # process -> [MapRow]
    xsec: dict = field(default_factory=dict)      # process -> target -> (N,2) array


def read_dict_dir(dict_dir: str) -> RawTables:
    """Loads a PETITE dict_dir (pickles) or a bundled ``sm_tables.npz``."""
    npz = os.path.join(dict_dir, "sm_tables.npz")
    maps_pkl = os.path.join(dict_dir, "sm_maps.pkl")
    if not os.path.exists(maps_pkl) and os.path.exists(npz):
        return load_npz(npz)
    raw = RawTables()
    with open(maps_pkl, "rb") as f:
        maps = _MapsUnpickler(f).load()
    with open(os.path.join(dict_dir, "sm_xsec.pkl"), "rb") as f:
        xsec = pickle.load(f)
    for proc in PROCESSES:
        if proc not in maps or proc not in xsec:
            raise Exception("Process String does not match library")   # shower.py:162,170
        rows = []
        for energy, info in maps[proc]:
            rows.append(MapRow(float(energy), int(info["neval"]),
                               {k: float(v) for k, v in info["max_F"].items()},
                               list(info["adaptive_map"].grid),
                               info.get("Eg_min"), info.get("Ee_min")))
        raw.maps[proc] = rows
        raw.xsec[proc] = {t: np.asarray(v, dtype=np.float64) for t, v in xsec[proc].items()}
    return raw


def save_npz(raw: RawTables, path: str) -> None:
    out = {}
    targets = sorted({t for p in raw.xsec for t in raw.xsec[p]})
    out["targets"] = np.array(targets)
    for proc, rows in raw.maps.items():
        d = len(rows[0].grid)
        maxn = max(len(g) for r in rows for g in r.grid)
        grid = np.full((len(rows), d, maxn), np.nan)
        nn = np.zeros((len(rows), d), np.int32)
        for i, r in enumerate(rows):
            for k, g in enumerate(r.grid):
                grid[i, k, :len(g)] = g
                nn[i, k] = len(g)
        out[f"{proc}/energy"] = np.array([r.energy for r in rows])
        out[f"{proc}/neval"] = np.array([r.neval for r in rows], np.int64)
        out[f"{proc}/max_F"] = np.array([[r.max_F.get(t, np.nan) for t in targets] for r in rows])
        out[f"{proc}/Eg_min"] = np.array([np.nan if r.Eg_min is None else r.Eg_min for r in rows])
        out[f"{proc}/Ee_min"] = np.array([np.nan if r.Ee_min is None else r.Ee_min for r in rows])
        out[f"{proc}/grid"] = grid
        out[f"{proc}/nnodes"] = nn
        for t, v in raw.xsec[proc].items():
            out[f"{proc}/xsec/{t}"] = v
    np.savez_compressed(path, **out)


def load_npz(path: str) -> RawTables:
    z = np.load(path, allow_pickle=False)
    targets = [str(t) for t in z["targets"]]
    raw = RawTables()
    for proc in PROCESSES:
        if f"{proc}/energy" not in z:
            raise Exception("Process String does not match library")
        E, nev, mf = z[f"{proc}/energy"], z[f"{proc}/neval"], z[f"{proc}/max_F"]
        egm, eem, grid, nn = z[f"{proc}/Eg_min"], z[f"{proc}/Ee_min"], z[f"{proc}/grid"], z[f"{proc}/nnodes"]
        rows = []
        for i in range(len(E)):
            rows.append(MapRow(float(E[i]), int(nev[i]),
                               {t: float(mf[i, j]) for j, t in enumerate(targets) if not np.isnan(mf[i, j])},
                               [grid[i, k, :nn[i, k]].copy() for k in range(grid.shape[1])],
                               None if np.isnan(egm[i]) else float(egm[i]),
                               None if np.isnan(eem[i]) else float(eem[i])))
        raw.maps[proc] = rows
        raw.xsec[proc] = {t: z[f"{proc}/xsec/{t}"] for t in targets if f"{proc}/xsec/{t}" in z}
    return raw


# --------------------------------------------------------------------------
# Analytic totals used for the Moller / Bhabha / MuonE n*sigma tables
# (shower.py:285-293).  Vectorised restatements of all_processes.py.
def _heaviside(x, h0):
    return np.heaviside(x, h0)


def sigma_moller(Ee, Ee_min):
    """Total Moller cross section (all_processes.py:907-944), GeV^-2."""
    me = M_ELECTRON
    Te = Ee_min - me
    thr = 3 * me + 4 * Te
    pref = 2 * math.pi * ALPHA_EM ** 2 / (me * (Ee ** 2 - me ** 2))
    a = Ee - 3 * me - 4 * Te + 2 * Ee ** 2 * (-2 / (Ee - 3 * me - 2 * Te) + 1 / Te
                                              + 1 / (-Ee + me + Te) + 2 / (Ee + me + 2 * Te))
    above = _heaviside(Ee - thr, 1)
    logarg = ((-Ee + me + Te) * (-Ee + 3 * me + 2 * Te) / (Te * (Ee + me + 2 * Te))) * above \
        + _heaviside(thr - Ee, 1)
    with np.errstate(invalid="ignore", divide="ignore"):
        b = 2 * me * (me - 2 * Ee) / (Ee - me) * np.log(logarg)
    return pref * (a + b) * above


def sigma_bhabha(Ee, Ee_min):
    """Total Bhabha cross section (all_processes.py:1010-1051), GeV^-2."""
    me = M_ELECTRON
    Te = Ee_min - me
    thr = 3 * me + 4 * Te
    pref = math.pi * ALPHA_EM ** 2 / (12 * (Ee - me) * me * (Ee + me) ** 3 * (Ee - 3 * me - 2 * Te) * Te)
    a = (Ee - 3 * me - 4 * Te) * (24 * Ee ** 2 * (Ee + me) ** 2
                                  + (Ee - 3 * me) * (31 * Ee ** 2 + 84 * Ee * me + 57 * me ** 2) * Te
                                  - 4 * (16 * Ee ** 2 + 39 * Ee * me + 33 * me ** 2) * Te ** 2
                                  + 8 * (Ee - 3 * me) * Te ** 3 - 8 * Te ** 4)
    above = _heaviside(Ee - thr, 1)
    with np.errstate(invalid="ignore", divide="ignore"):
        b = 24 * (Ee + me) * (2 * Ee ** 2 + 4 * Ee * me + me ** 2) * (Ee - 3 * me - 2 * Te) * Te \
            * np.log((2 * Te / (Ee - 3 * me - 2 * Te)) * above + _heaviside(thr - Ee, 1))
    return pref * (a + b) * above


def muone_threshold(Ee_min):
    me, mm = M_ELECTRON, M_MUON
    return 1.0 / (2.0 * me) * (me * (Ee_min - me) + np.sqrt(me * (Ee_min + me) * (me * (Ee_min - me) + 2 * mm ** 2)))


def sigma_muone(Emu, Ee_min):
    """Total mu e -> mu e cross section (all_processes.py:888-905), GeV^-2."""
    me, mm = M_ELECTRON, M_MUON
    s = me ** 2 + mm ** 2 + 2 * me * Emu
    t_max = 2.0 * me * (me - Ee_min)
    t_min = -4.0 * ((s + me ** 2 - mm ** 2) ** 2 / (4 * s) - me ** 2)
    pref = 16 * math.pi ** 2 * ALPHA_EM ** 2 / (8.0 * math.pi * ((s - mm ** 2) ** 2 + me ** 4 - 2 * (s + mm ** 2) * me ** 2))
    a = -2.0 * (s ** 2 + mm ** 4 + 5 * me ** 4 - 2 * me ** 2 * (2 * s + mm ** 2)) * (1.0 / t_max - 1.0 / t_min)
    b = 2.0 * (s + 2 * mm ** 2 - 2 * me ** 2) * np.log(t_max / t_min)
    c = t_max - t_min
    return pref * (a + b + c) * _heaviside(Emu - muone_threshold(Ee_min), 1)


# Interpolant slots (order used by the kernels)
NS_BREM, NS_PP, NS_ANN, NS_COMP, NS_MOLLER, NS_BHABHA, NS_MUONE, NS_MUONBREM = range(8)
NS_NAMES = ("Brem", "PairProd", "Ann", "Comp", "Moller", "Bhabha", "MuonE", "MuonBrem")


class SMTables:
    """Everything the SM transport kernels read, for one target material."""

    def __init__(self, raw: RawTables, target_material: str, maxF_fudge_global: float = 1.0):
        if target_material not in TARGET_INFORMATION:
            raise Exception("Target Material is not in library")
        for proc in PROCESSES:
            if target_material not in raw.xsec[proc]:
                raise Exception("Target Material is not in library")      # shower.py:175
        ti = TARGET_INFORMATION[target_material]
        self.target = target_material
        self.Z, self.A, self.rho, self.dEdx = float(ti["Z_T"]), float(ti["A_T"]), float(ti["rho"]), float(ti["dEdx"])
        self.Z_int = ti["Z_T"]
        self.n_target = self.rho / M_PROTON_GRAMS / self.A                # shower.py:202-208
        self.n_elec = self.n_target * self.Z
        xs = {p: raw.xsec[p][target_material] for p in PROCESSES}
        mue = xs["MuonE"]
        while mue[0][1] == 0.0:                                            # shower.py:238-239
            mue = mue[1:]
        xs["MuonE"] = mue
        self.xsec = xs
        # shower.py:242-246
        self.min_calc = {
            11: float(min(xs["Brem"][0][0], xs["Moller"][0][0])),
            -11: float(min(xs["Brem"][0][0], xs["Bhabha"][0][0], xs["Ann"][0][0])),
            13: float(max(min(xs["MuonBrem"][0][0], mue[0][0]), 0.120)),
            -13: float(max(min(xs["MuonBrem"][0][0], mue[0][0]), 0.120)),
            22: float(min(xs["PairProd"][0][0], xs["Comp"][0][0])),
        }
        self.Eg_min = float(raw.maps["Brem"][0].Eg_min)                    # shower.py:214-215
        self.Ee_min = float(raw.maps["Brem"][0].Ee_min)
        self._build_nsigma(xs)
        self._build_maps(raw, target_material, maxF_fudge_global)

    # ------------------------------------------------------------------
    def _build_nsigma(self, xs):
        """n*sigma(E) tables in 1/cm, as in shower.py:273-295."""
        nZ, ne = self.n_target, self.n_elec
        BS = xs["Brem"]
        tabs = [None] * 8
        tabs[NS_BREM] = (BS[:, 0], nZ * GEVSQCM2 * BS[:, 1])
        tabs[NS_PP] = (xs["PairProd"][:, 0], nZ * GEVSQCM2 * xs["PairProd"][:, 1])
        tabs[NS_ANN] = (xs["Ann"][:, 0], ne * GEVSQCM2 * xs["Ann"][:, 1])
        tabs[NS_COMP] = (xs["Comp"][:, 0], ne * GEVSQCM2 * xs["Comp"][:, 1])
        bm = np.geomspace(3.0 * M_ELECTRON + self.Ee_min, BS[:, 0][-1], len(BS))
        tabs[NS_MOLLER] = (bm, ne * GEVSQCM2 * sigma_moller(bm, self.Ee_min))
        tabs[NS_BHABHA] = (bm, ne * GEVSQCM2 * sigma_bhabha(bm, self.Ee_min))
        emin = float(muone_threshold(self.Ee_min))
        if emin < xs["MuonE"][0][0]:
            emin = float(xs["MuonE"][0][0])
        me_grid = np.geomspace(emin, bm[-1], len(BS))
        tabs[NS_MUONE] = (me_grid, ne * GEVSQCM2 * sigma_muone(me_grid, self.Ee_min))
        tabs[NS_MUONBREM] = (xs["MuonBrem"][:, 0], nZ * GEVSQCM2 * xs["MuonBrem"][:, 1])
        self.nsigma = [(np.ascontiguousarray(x, np.float64), np.ascontiguousarray(y, np.float64)) for x, y in tabs]

    def _build_maps(self, raw, target, fudge):
        rows_E, rows_maxF, rows_neval, offs, nincs = [], [], [], [], []
        self.map_rows = []
        self.map_base = []
        nodes = []
        pos = 0
        base = 0
        for proc in PROCESSES:
            rows = raw.maps[proc]
            self.map_base.append(base)
            self.map_rows.append(len(rows))
            base += len(rows)
            for r in rows:
                rows_E.append(r.energy)
                rows_maxF.append(r.max_F[target] * fudge)
                rows_neval.append(float(r.neval))
                o4, n4 = [0] * 4, [0] * 4
                for k, g in enumerate(r.grid):
                    o4[k] = pos
                    n4[k] = len(g) - 1
                    nodes.append(np.asarray(g, np.float64))
                    pos += len(g)
                offs.append(o4)
                nincs.append(n4)
        self.map_energy = np.array(rows_E)
        self.map_maxF = np.array(rows_maxF)
        self.map_neval = np.array(rows_neval)
        self.grid_offset = np.array(offs, np.int64)
        self.grid_ninc = np.array(nincs, np.int32)
        self.grid_nodes = np.concatenate(nodes)
        self.map_rows = np.array(self.map_rows, np.int32)
        self.map_base = np.array(self.map_base, np.int32)
        self._node_is_last = np.zeros(len(self.grid_nodes), bool)
        for o4, n4 in zip(offs, nincs):
            for o, n in zip(o4, n4):
                if n:
                    self._node_is_last[o + n] = True

    def grid_f32x4(self) -> np.ndarray:
        """Float32 node table for the mixed-precision sampler: per node
        (value, increment to the next node, 1 - value, 1 + value), each
        computed in float64 and rounded once."""
        g = self.grid_nodes
        inc = np.zeros_like(g)
        inc[:-1] = g[1:] - g[:-1]
        inc[self._node_is_last] = 0.0
        return np.ascontiguousarray(np.stack([g, inc, 1.0 - g, 1.0 + g], axis=1).astype(np.float32))
