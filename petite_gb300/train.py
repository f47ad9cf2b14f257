"""The table builder: VEGAS maps and max_F for PETITE's SM processes, on the GPU.

PETITE trains one VEGAS map per (process, incoming energy) with the vegas
package (all_processes.py:1160-1245, ``vegas_integration(..., mode="Pickle")``
called by utilities/generate_integrators.py:49-84 with the hydrogen target,
:118-123), then scans every map with utilities/find_maxes.py:56-115 for
``max_F`` per target and the cross section.  Here all energy rows of a
process train together through ``pt_vegas_accumulate``/``pt_vegas_adapt``
and are scanned through ``pt_find_maxes``; the settings follow the
reference's: the integration ranges of ``integration_range``
(all_processes.py:1102-1160), grids of about 1000 increments kept a multiple
of each dimension's strata (``vegas_integrator_options``, :1085-1096; the
shipped maps have 960 for 60 strata), 2 x nitn adaptations (the burn-in
call and the final one), damping alpha = 0.5, and find_maxes' neval = 300,
100 trials.

``build_raw_tables`` assembles ``RawTables`` (tables.py) from trained or
shipped maps and a ``sm_xsec.pkl``; ``save_npz`` of it is a dict_dir that
``Shower`` loads.  ``build_400GeV_tables`` does this for PETITE's
``data_400GeV`` directory, whose Brem, PairProd and MuonBrem maps are not
shipped.
"""
from __future__ import annotations

import math
import os
import pickle

import numpy as np

from . import _lib
from . import tables as T

# vegas_integrator_options, all_processes.py:1085-1096 (DarkAnn: 1000
# increments, vegas' default, for its neval-only options)
NSTRAT = {"PairProd": (60, 50, 40, 50), "Brem": (60, 50, 50, 50), "MuonBrem": (60, 50, 50, 50),
          "Comp": (1000,), "Moller": (1000,), "MuonE": (1000,), "Bhabha": (1000,), "Ann": (1000,),
          "DarkBrem": (100, 100, 40), "DarkMuonBrem": (100, 100, 40), "DarkComp": (1000,), "DarkAnn": (1000,)}
NITN = {"PairProd": 10, "Brem": 10, "MuonBrem": 10, "Comp": 20, "Moller": 20, "MuonE": 20, "Bhabha": 20, "Ann": 20,
        "DarkBrem": 20, "DarkMuonBrem": 20, "DarkComp": 20, "DarkAnn": 10}
TRAINING_TARGET = "hydrogen"               # generate_integrators.py:118-123
# the dark maps train on hydrogen with mT = 200 GeV
# (script_generateintegrators_400GeV.py:51-55, generate_integrators.py:103-113)
DARK_TRAINING_MT = 200.0
FIND_MAXES_TARGETS = ("graphite", "lead", "iron", "aluminum", "molybdenum")
DARK_PROCESSES = ("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")     # engine dark codes 0..3


def process_code(process: str) -> int:
    """The table builder's code of a process (SM codes; dark: TRAIN_DARK + dark code)."""
    if process in DARK_PROCESSES:
        return _lib.TRAIN_DARK + DARK_PROCESSES.index(process)
    return T.PROCESS_CODE[process]


def integration_range(process: str, E: float, Eg_min: float = 0.001, Ee_min: float = 0.005, mV: float = 0.0):
    """integration_range, all_processes.py:1102-1160."""
    me = T.M_ELECTRON
    if process in ("DarkBrem", "DarkMuonBrem"):         # x, log10(1 - cos theta), log10 t~
        return [[max(0., mV / E), 1. - me / E], [-12.0, np.log10(2.0)], [-20.0, 0.0]]
    if process == "DarkComp":
        return [[-1., 1.0]]
    if process == "DarkAnn":
        return [[0., 1.0]] if 2.0 * me * (E + me) > mV ** 2 else [[0., 0.]]
    if process in ("PairProd", "Brem"):
        return [[0, 1], [0, 2], [-2, 2], [0, 1]]
    if process == "MuonBrem":
        maxdel = np.sqrt(E / np.max([me, mV]))
        return [[np.max([Eg_min, mV]), E - me], [0., maxdel], [0., maxdel], [0., 2 * np.pi]]
    if process in ("Comp", "Ann", "MuonE"):
        return [[-1., 1.0]]
    d = 2.0 * Ee_min / (E - me)
    return [[-1.0 + d, 1.0 - d]]


def n_increments(process: str):
    """Increments per dimension: about 1000, a multiple of the strata."""
    return [(1000 // s) * s for s in NSTRAT[process]]


def target_constants(target: str, Eg_min: float = 0.001, Ee_min: float = 0.005, mV: float = 0.0,
                     mT: float | None = None) -> _lib.PtTrainTarget:
    """What the cross sections read of a target: the SM screening constants
    (the engine's expressions, all_processes.py:92-103) and, for the dark
    processes, mV and the target's mT, Z_T, A_T (find_maxes.py:85-100; ``mT``
    overrides the table's, as the dark training does)."""
    ti = T.TARGET_INFORMATION[target]
    Z = ti["Z_T"]
    a0 = 184.15 * (2.718) ** -0.5 * Z ** (-1.0 / 3.0) / T.M_ELECTRON
    t = _lib.PtTrainTarget()
    t.Eg_min, t.Ee_min, t.a0sq, t.Z2a04 = Eg_min, Ee_min, a0 ** 2, Z ** 2 * a0 ** 4
    t.mV = float(mV)
    t.MT = float(ti["mT"] if mT is None else mT)
    t.Z, t.A = float(Z), float(ti["A_T"])
    return t


def _torch():
    import torch
    return torch


class MapSet:
    """The maps of one process at its energies: nodes (rows, dims, max_nodes)
    on the device, increments per dimension."""

    def __init__(self, process: str, energies, nodes, ninc, mV: float = 0.0):
        self.process = process
        self.energies = np.asarray(energies, np.float64)
        self.nodes = nodes
        self.ninc = list(ninc)
        self.mV = float(mV)                 # dark processes: the vector's mass

    @classmethod
    def uniform(cls, process, energies, device="cuda", mV: float = 0.0):
        torch = _torch()
        ninc = n_increments(process)
        D, mn = len(ninc), max(ninc) + 1
        g = np.zeros((len(energies), D, mn))
        for r, E in enumerate(energies):
            for d, (lo, hi) in enumerate(integration_range(process, float(E), mV=mV)):
                g[r, d, :ninc[d] + 1] = np.linspace(lo, hi, ninc[d] + 1)
        return cls(process, energies, torch.as_tensor(g, device=device), ninc, mV)

    @classmethod
    def from_grids(cls, process, energies, grids, device="cuda", mV: float = 0.0):
        """Maps given as per-row lists of node arrays (e.g. PETITE's shipped maps)."""
        torch = _torch()
        D = len(grids[0])
        ninc = [len(grids[0][d]) - 1 for d in range(D)]
        mn = max(ninc) + 1
        g = np.zeros((len(grids), D, mn))
        for r, gr in enumerate(grids):
            for d in range(D):
                if len(gr[d]) != ninc[d] + 1:
                    raise ValueError("rows of one process must share the increments per dimension")
                g[r, d, :len(gr[d])] = gr[d]
        return cls(process, energies, torch.as_tensor(g, device=device), ninc, mV)

    def grids(self):
        g = self.nodes.cpu().numpy()
        return [[g[r, d, :self.ninc[d] + 1].copy() for d in range(len(self.ninc))] for r in range(len(g))]

    def _args(self):
        """Energies on the device; increments per dimension on the host."""
        import ctypes as C
        torch = _torch()
        E = torch.as_tensor(self.energies, device=self.nodes.device)
        ninc = (C.c_int32 * len(self.ninc))(*self.ninc)
        return E, ninc


def train(maps: MapSet, points_per_row: int = 1 << 21, iterations: int | None = None, alpha: float = 0.5,
          seed: int = 20261204, target: str = TRAINING_TARGET, history: list | None = None,
          mT: float | None = None) -> MapSet:
    """Adapts ``maps`` in place: ``iterations`` (default 2 x nitn) rounds of
    accumulate + adapt.  ``history`` receives each round's per-row integral
    estimates (mean of jac f).  The dark processes train on ``target`` with
    mT = ``mT`` (default 200 GeV, as PETITE's dark training)."""
    torch = _torch()
    lib = _lib.load()
    dev = maps.nodes.device
    E, ninc = maps._args()
    n, D = len(maps.energies), len(maps.ninc)
    code = process_code(maps.process)
    dark = maps.process in DARK_PROCESSES
    tgt = target_constants(target, mV=maps.mV, mT=(DARK_TRAINING_MT if mT is None else mT) if dark else None)
    acc = torch.zeros((n, D, 1000), dtype=torch.float64, device=dev)
    cnt = torch.zeros((n, D, 1000), dtype=torch.int32, device=dev)
    sums = torch.zeros((n, 2), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    iters = 2 * NITN[maps.process] if iterations is None else iterations
    if iters > 64:
        raise ValueError("at most 64 training iterations")
    import ctypes as C
    for it in range(iters):
        acc.zero_()
        cnt.zero_()
        sums.zero_()
        _lib.check(lib.pt_vegas_accumulate(code, C.byref(tgt), E.data_ptr(), n, D, ninc,
                                           maps.nodes.data_ptr(), maps.nodes.shape[2], int(points_per_row),
                                           int(seed) & (2 ** 64 - 1), it, acc.data_ptr(), cnt.data_ptr(),
                                           sums.data_ptr(), C.c_void_p(stream)), "pt_vegas_accumulate")
        if history is not None:
            history.append((sums[:, 0] / points_per_row).cpu().numpy())
        _lib.check(lib.pt_vegas_adapt(n, D, ninc, maps.nodes.data_ptr(), maps.nodes.shape[2],
                                      acc.data_ptr(), cnt.data_ptr(), float(alpha), C.c_void_p(stream)),
                   "pt_vegas_adapt")
    torch.cuda.synchronize(dev)
    return maps


def find_maxes(maps: MapSet, targets=FIND_MAXES_TARGETS, neval: int = 300, n_trials: int = 100,
               seed: int = 20261205):
    """find_maxes.py:56-115 on every row: (max_F, xsec), each (rows, targets)."""
    torch = _torch()
    lib = _lib.load()
    dev = maps.nodes.device
    E, ninc = maps._args()
    n, D = len(maps.energies), len(maps.ninc)
    arr = (_lib.PtTrainTarget * len(targets))(*[target_constants(t, mV=maps.mV) for t in targets])
    mf = torch.zeros((n, len(targets)), dtype=torch.float64, device=dev)
    xs = torch.zeros_like(mf)
    import ctypes as C
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(lib.pt_find_maxes(process_code(maps.process), arr, len(targets), E.data_ptr(), n, D,
                                 ninc, maps.nodes.data_ptr(), maps.nodes.shape[2], int(neval), int(n_trials),
                                 int(seed) & (2 ** 64 - 1), mf.data_ptr(), xs.data_ptr(), C.c_void_p(stream)),
               "pt_find_maxes")
    return mf.cpu().numpy(), xs.cpu().numpy()


def mass_dir(mV: float) -> str:
    """The per-mass map directory name (generate_integrators.py:114-117)."""
    return f"mV_{int(np.floor(mV * 1000.))}MeV"


def load_shipped_maps(dict_dir: str, process: str, mV: float | None = None):
    """PETITE's ``<Process>/<Process>_AdaptiveMaps.npy`` (dark processes:
    ``<Process>/mV_<n>MeV/...``; a list of [event_info, AdaptiveMap]) as
    (energies, grids), without the vegas package."""
    sub = (process,) if mV is None else (process, mass_dir(mV))
    path = os.path.join(dict_dir, *sub, f"{process}_AdaptiveMaps.npy")
    with open(path, "rb") as f:
        np.lib.format.read_magic(f)
        np.lib.format.read_array_header_1_0(f)
        arr = T._MapsUnpickler(f).load()
    E = [float(ev["E_inc"]) for ev, _ in arr]
    grids = [[np.asarray(g, np.float64) for g in m.grid] for _, m in arr]
    return np.array(E), grids


def build_raw_tables(xsec: dict, maps: dict, max_F: dict, neval: int = 300, targets=FIND_MAXES_TARGETS,
                     Eg_min: float = 0.001, Ee_min: float = 0.005) -> T.RawTables:
    """RawTables from cross sections (``sm_xsec.pkl`` content: process ->
    target -> (E, sigma) rows), maps (process -> MapSet) and max_F (process
    -> (rows, targets))."""
    raw = T.RawTables()
    for proc in T.PROCESSES:
        ms = maps[proc]
        mf = max_F[proc]
        rows = []
        for r, (E, g) in enumerate(zip(ms.energies, ms.grids())):
            rows.append(T.MapRow(float(E), int(neval), {t: float(mf[r, j]) for j, t in enumerate(targets)}, g,
                                 Eg_min, Ee_min))
        raw.maps[proc] = rows
        raw.xsec[proc] = {t: np.asarray(v, np.float64) for t, v in xsec[proc].items()}
    return raw


def build_400GeV_tables(dict_dir: str, out_path: str, points_per_row: int = 1 << 21, device="cuda",
                        log=print) -> dict:
    """Tables for PETITE's ``data_400GeV``: its shipped maps (MuonE, Comp,
    Ann, Moller, Bhabha) and trained maps for Brem, PairProd and MuonBrem at
    the energies of its sm_xsec.pkl; max_F of every row from find_maxes.
    Writes ``out_path`` (``save_npz``) and returns a summary."""
    with open(os.path.join(dict_dir, "sm_xsec.pkl"), "rb") as f:
        xsec = pickle.load(f)
    maps, max_F, summary = {}, {}, {}
    for proc in T.PROCESSES:
        ship = os.path.join(dict_dir, proc, f"{proc}_AdaptiveMaps.npy")
        E_x = np.asarray(xsec[proc]["graphite"], np.float64)[:, 0]
        if os.path.exists(ship):
            E, grids = load_shipped_maps(dict_dir, proc)
            ms = MapSet.from_grids(proc, E, grids, device)
            how = "shipped"
        else:
            ms = train(MapSet.uniform(proc, E_x, device), points_per_row=points_per_row)
            how = "trained"
        mf, xs = find_maxes(ms)
        maps[proc], max_F[proc] = ms, mf
        ref = np.array([np.interp(e, np.asarray(xsec[proc]["graphite"])[:, 0],
                                  np.asarray(xsec[proc]["graphite"])[:, 1]) for e in ms.energies])
        ok = ref > 0
        ratio = xs[ok, 0] / ref[ok]
        summary[proc] = {"maps": how, "rows": len(ms.energies), "E_max": float(ms.energies.max()),
                         "xsec_ratio_graphite_median": float(np.median(ratio)) if ok.any() else None}
        log(proc, summary[proc])
    raw = build_raw_tables(xsec, maps, max_F)
    T.save_npz(raw, out_path)
    return summary


def dark_energies(process: str, mV: float, E_min: float = 0.0016, E_max: float = 100.0, n: int = 100):
    """The incoming energies of a dark map set (utilities/
    script_generateintegrators.py:53-82): DarkBrem from 1.25 mV, DarkMuonBrem
    from 1.25 (mV + m_mu), DarkAnn and DarkComp from their thresholds up to
    max(E_max, 100 x threshold)."""
    me, mmu = T.M_ELECTRON, T.M_MUON
    if process == "DarkBrem":
        return np.geomspace(1.25 * mV, E_max, n)
    if process == "DarkMuonBrem":
        return np.geomspace(1.25 * (mV + mmu), E_max, n)
    if process == "DarkAnn":
        e0 = (mV ** 2 - 2 * me ** 2) / (2 * me)
    else:
        e0 = mV * (1 + mV / (2 * me))
    top = np.max([E_max, 100 * e0])
    return e0 * (1 + np.geomspace(1e-4, (top - e0) / e0, n))


def build_dark_maps(dict_dir: str, out_path: str, mV: float, points_per_row: int = 1 << 21, device="cuda",
                    targets=FIND_MAXES_TARGETS, log=print, E_max: float = 100.0, n_energies: int = 100,
                    train_all: bool = False, processes=None) -> dict:
    """The dark maps of one mass for a PETITE dict_dir whose DarkBrem and
    DarkMuonBrem maps are not shipped (``data_400GeV``): shipped maps where
    they exist (DarkAnn, DarkComp), trained maps elsewhere at the energies of
    the directory's ``dark_xsec.pkl`` (the rows find_maxes wrote for the lost
    maps), and max_F and the cross section of every row (find_maxes,
    find_maxes.py:211-305).  Writes ``out_path`` with the map entries of
    ``dark_tables.npz`` (``m<mV>/<Process>/energy, neval, max_F, grid,
    nnodes``, plus ``xsec`` from find_maxes) and returns, per process, the
    median ratio of that cross section to ``dark_xsec.pkl`` (lead).  A mass
    that ``dark_xsec.pkl`` lacks trains every process at the energies of
    ``dark_energies`` (up to E_max, n_energies rows), as PETITE's generation
    script would, and reports no ratio.  ``train_all`` trains shipped
    processes too (to check the trainer against PETITE's rows).
    ``processes`` defaults to all four, less DarkAnn below mV = 2 m_e: there
    e+ e- -> V has no resonance (its energy (mV^2 - 2 m_e^2) / (2 m_e) lies
    below the positron's rest mass) and PETITE's generation script has no
    map energies for it."""
    with open(os.path.join(dict_dir, "dark_xsec.pkl"), "rb") as f:
        dx = pickle.load(f)
    keys = [k for k in dx if abs(float(k) - mV) < 1e-12]
    out, summary = {"targets": np.array(targets)}, {}
    if processes is None:
        processes = [p for p in DARK_PROCESSES if p != "DarkAnn" or mV >= 2 * T.M_ELECTRON]
    for proc in processes:
        ref = np.asarray(dx[keys[0]][proc]["lead"], np.float64) if keys else None
        ship = os.path.join(dict_dir, proc, mass_dir(mV), f"{proc}_AdaptiveMaps.npy")
        if os.path.exists(ship) and not train_all:
            E, grids = load_shipped_maps(dict_dir, proc, mV)
            ms = MapSet.from_grids(proc, E, grids, device, mV=mV)
            how = "shipped"
        else:
            E = ref[:, 0] if ref is not None else dark_energies(proc, mV, E_max=E_max, n=n_energies)
            ms = train(MapSet.uniform(proc, E, device, mV=mV), points_per_row=points_per_row)
            how = "trained"
        mf, xs = find_maxes(ms, targets=targets)
        g = ms.nodes.cpu().numpy()
        nn = np.tile(np.array(ms.ninc, np.int32) + 1, (len(ms.energies), 1))
        pre = f"m{mV}/{proc}"
        out[f"{pre}/energy"] = ms.energies
        out[f"{pre}/neval"] = np.full(len(ms.energies), 300, np.int64)
        out[f"{pre}/max_F"] = mf
        out[f"{pre}/xsec"] = xs
        out[f"{pre}/grid"] = g
        out[f"{pre}/nnodes"] = nn
        summary[proc] = {"maps": how, "rows": len(ms.energies), "E_max": float(ms.energies.max()),
                         "xsec_ratio_lead_median": None}
        if ref is not None:
            j = list(targets).index("lead")
            r = np.interp(ms.energies, ref[:, 0], ref[:, 1])
            ok = r > 0
            if ok.any():
                summary[proc]["xsec_ratio_lead_median"] = float(np.median(xs[ok, j] / r[ok]))
        log(proc, summary[proc])
    np.savez_compressed(out_path, **out)
    return summary
