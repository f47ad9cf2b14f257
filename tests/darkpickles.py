"""Writes a PETITE-format dark dict_dir from the bundled dark tables, for the
tests of the native dark-table build.

PETITE's dark_maps.pkl (find_maxes.py output) holds, per mass and dark
process, rows ``[E, {"neval", "max_F": {target: value}, "adaptive_map"}]``
with ``vegas._vegas.AdaptiveMap`` objects; its dark_xsec.pkl holds
``{mass: {process: {target: [[E, sigma], ...]}}}``; dark_weights.pkl and
dark_drate.pkl are the constructor's caches (dark_shower.py:401-593).  The
maps here pickle as that class through a stand-in module, so the files
read back exactly as PETITE's do, without the vegas package.
"""
import os
import pickle
import sys
import types

import numpy as np

PROCS = ("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")


class AdaptiveMap:
    """Pickles as vegas._vegas.AdaptiveMap(grid)."""

    def __init__(self, grid):
        self.grid = grid

    def __reduce__(self):
        return (AdaptiveMap, (self.grid,))


def _with_vegas_module(fn):
    pkg = types.ModuleType("vegas")
    mod = types.ModuleType("vegas._vegas")
    saved = {k: sys.modules.get(k) for k in ("vegas", "vegas._vegas")}
    qual = AdaptiveMap.__qualname__, AdaptiveMap.__module__
    AdaptiveMap.__qualname__, AdaptiveMap.__module__ = "AdaptiveMap", "vegas._vegas"
    mod.AdaptiveMap = AdaptiveMap
    pkg._vegas = mod
    sys.modules["vegas"], sys.modules["vegas._vegas"] = pkg, mod
    try:
        return fn()
    finally:
        AdaptiveMap.__qualname__, AdaptiveMap.__module__ = qual
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


def write_dict_dir(bundle: str, out_dir: str, masses=None, targets=None, sm_npz=None,
                   weights_cache=None, drate_cache=None):
    """dark_maps.pkl and dark_xsec.pkl of ``masses`` x ``targets`` from a
    dark_tables.npz bundle (its maps; its DarkBrem and DarkMuonBrem cross
    sections and the free-electron DarkAnn and DarkComp ones, which are
    dark_xsec.pkl's), plus the SM tables (``sm_npz``) and, if given,
    dark_weights.pkl / dark_drate.pkl content."""
    z = np.load(bundle)
    masses = [float(m) for m in z["masses"]] if masses is None else list(masses)
    targets = [str(t) for t in z["targets"]] if targets is None else list(targets)
    all_t = [str(t) for t in z["targets"]]
    maps, xsec = {}, {}
    for mV in masses:
        maps[mV], xsec[mV] = {}, {}
        for p in PROCS:
            pre = f"m{mV}/{p}"
            E, nev, mf = z[f"{pre}/energy"], z[f"{pre}/neval"], z[f"{pre}/max_F"]
            grid, nn = z[f"{pre}/grid"], z[f"{pre}/nnodes"]
            rows = []
            for i in range(len(E)):
                g = [grid[i, k, :nn[i, k]].copy() for k in range(grid.shape[1])]
                rows.append([float(E[i]), {"neval": int(nev[i]),
                                           "max_F": {t: float(mf[i, all_t.index(t)]) for t in targets},
                                           "adaptive_map": AdaptiveMap(g)}])
            maps[mV][p] = rows
            src = {"DarkBrem": "xsec/DarkBrem", "DarkMuonBrem": "xsec/DarkMuonBrem",
                   "DarkAnn": "free/xsec/DarkAnn", "DarkComp": "free/xsec/DarkComp"}[p]
            xsec[mV][p] = {t: [list(r) for r in z[f"m{mV}/{t}/{src}"]] for t in targets}
    os.makedirs(out_dir, exist_ok=True)

    def dump():
        with open(os.path.join(out_dir, "dark_maps.pkl"), "wb") as f:
            pickle.dump(maps, f)
    _with_vegas_module(dump)
    with open(os.path.join(out_dir, "dark_xsec.pkl"), "wb") as f:
        pickle.dump(xsec, f)
    for name, content in (("dark_weights.pkl", weights_cache), ("dark_drate.pkl", drate_cache)):
        if content is not None:
            with open(os.path.join(out_dir, name), "wb") as f:
                pickle.dump(content, f)
    if sm_npz is not None:
        os.symlink(os.path.realpath(sm_npz), os.path.join(out_dir, "sm_tables.npz"))
    return out_dir
