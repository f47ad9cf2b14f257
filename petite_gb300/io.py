"""Input and output formats around the shower path.

* ``read_particle_file``: a shower saved by PETITE (``np.save`` of a list or
  array of ``PETITE.particle.Particle``, which ``generate_dark_shower(ExDir=
  path)`` reads, dark_shower.py:822-823) into this package's ``Particle``
  objects, without PETITE installed: the pickled class is mapped to
  ``petite_gb300.particle.Particle``, whose attributes have the same names.
* ``save_particle_file``: the same format, written from these objects.
* ``load_beam``: PETITE's beam files (``examples/beams/*.npy``: one
  four-momentum (E, px, py, pz) per row) as ``Particle`` inputs.
* ``particles_to_arrays`` / ``arrays_to_particles``: bulk conversion
  between ``Particle`` lists and structure-of-arrays numpy dictionaries,
  the layout the engines read and write.
"""
from __future__ import annotations

import io as _io
import pickle

import numpy as np

from .particle import Particle

_PARTICLE_MODULES = ("PETITE.particle", "particle", "petite_gb300.particle")


class _ShowerUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if name == "Particle" and module in _PARTICLE_MODULES:
            return Particle
        return super().find_class(module, name)


def read_particle_file(path) -> list:
    """Particles of a shower file saved with ``np.save`` (object array)."""
    with open(path, "rb") as f:
        version = np.lib.format.read_magic(f)
        if version == (1, 0):
            shape, fortran, dtype = np.lib.format.read_array_header_1_0(f)
        else:
            shape, fortran, dtype = np.lib.format.read_array_header_2_0(f)
        if dtype != np.dtype(object):
            raise ValueError(f"{path}: not a file of Particle objects (dtype {dtype})")
        arr = _ShowerUnpickler(_io.BytesIO(f.read())).load()
    out = list(np.asarray(arr, dtype=object).ravel(order="F" if fortran else "C"))
    for p in out:
        if not isinstance(p, Particle):
            raise ValueError(f"{path}: entry of type {type(p).__name__}, not Particle")
    return out


def save_particle_file(path, particles) -> None:
    """Writes ``particles`` as ``np.save`` of an object array (PETITE's shower files)."""
    arr = np.empty(len(particles), dtype=object)
    for k, p in enumerate(particles):
        arr[k] = p
    np.save(path, arr, allow_pickle=True)


def load_beam(path_or_array, pid: int, weight=None, r0=(0.0, 0.0, 0.0), mass=None, first_id: int = 1) -> list:
    """Input particles from a beam file of four-momenta (one (E, px, py, pz)
    row per particle).  ``weight``: per particle (default 1/N, the beam
    normalised to one primary); ``mass``: the ``Particle`` mass (default:
    from each four-momentum, rounded as ``Particle`` rounds it); IDs count
    up from ``first_id``."""
    p4 = np.load(path_or_array) if isinstance(path_or_array, (str, bytes)) or hasattr(path_or_array, "__fspath__") \
        else np.asarray(path_or_array)
    p4 = np.asarray(p4, dtype=np.float64)
    if p4.ndim != 2 or p4.shape[1] != 4:
        raise ValueError(f"beam must hold one four-momentum per row, got shape {p4.shape}")
    n = len(p4)
    w = np.full(n, 1.0 / max(n, 1)) if weight is None else np.broadcast_to(np.asarray(weight, np.float64), (n,))
    out = []
    for k in range(n):
        ids = {"PID": int(pid), "ID": first_id + k, "weight": float(w[k])}
        if mass is not None:
            ids["mass"] = float(mass)
        out.append(Particle(list(p4[k]), list(r0), ids))
    return out


_ID_KEYS = ("PID", "ID", "parent_PID", "parent_ID", "generation_number", "weight", "mass")


def particles_to_arrays(particles) -> dict:
    """Structure-of-arrays copy of a ``Particle`` list: p0, r0, pf, rf
    (n, 4|3), the numeric IDs, ``generation_process`` (strings) and
    ``ended``."""
    n = len(particles)
    out = {"p0": np.empty((n, 4)), "r0": np.empty((n, 3)), "pf": np.empty((n, 4)), "rf": np.empty((n, 3))}
    for k in ("PID", "ID", "parent_PID", "parent_ID", "generation_number"):
        out[k] = np.empty(n, np.int64)
    out["weight"] = np.empty(n)
    out["mass"] = np.empty(n)
    out["generation_process"] = np.empty(n, dtype=object)
    out["ended"] = np.empty(n, bool)
    for i, p in enumerate(particles):
        d = p.get_ids()
        out["p0"][i], out["r0"][i] = p.get_p0(), p.get_r0()
        out["pf"][i], out["rf"][i] = p.get_pf(), p.get_rf()
        for k in _ID_KEYS:
            out[k][i] = d[k] if d[k] is not None else np.nan
        out["generation_process"][i] = d["generation_process"]
        out["ended"][i] = bool(p.get_ended())
    return out


def arrays_to_particles(a: dict) -> list:
    """``Particle`` objects from ``particles_to_arrays`` output (or any dict
    with p0 and PID; the other fields take Particle's defaults)."""
    n = len(a["p0"])
    out = []
    for i in range(n):
        ids = {k: (a[k][i].item() if hasattr(a[k][i], "item") else a[k][i]) for k in _ID_KEYS if k in a}
        if "generation_process" in a:
            ids["generation_process"] = a["generation_process"][i]
        r0 = a["r0"][i] if "r0" in a else (0.0, 0.0, 0.0)
        p = Particle(list(a["p0"][i]), list(r0), ids)
        if "pf" in a:
            p.set_pf(np.asarray(a["pf"][i], np.float64))
        if "rf" in a:
            p.set_rf(np.asarray(a["rf"][i], np.float64))
        if "ended" in a:
            p.set_ended(bool(a["ended"][i]))
        out.append(p)
    return out
