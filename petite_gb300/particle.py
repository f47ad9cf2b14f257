"""Particle record with PETITE's interface (particle.py:50-207).

``Shower.generate_shower`` returns a list of these, with the same keys in
``get_ids()`` as PETITE (``particle.py:22-28``).  Only the stable-particle
part of PETITE's class is provided: meson decays are outside the shower
transport path.
"""
from __future__ import annotations

import copy as _copy

import numpy as np

from .tables import M_ELECTRON, M_MUON

# particle.py:4-13 (leptons and photon; the shower path)
MASS = {11: M_ELECTRON, -11: M_ELECTRON, 12: 0.0, -12: 0.0, 22: 0.0, 13: M_MUON, -13: M_MUON,
        14: 0.0, -14: 0.0}

DEFAULT_IDS = {"PID": 11, "ID": 1, "parent_PID": 22, "parent_ID": -1, "generation_number": 0,
               "generation_process": "Input", "weight": 1.0, "mass": None, "stability": "stable",
               "production_time": 0.0, "decay_time": 0.0, "interaction_time": 0.0}


class Particle:
    """Container for particle information as it is propagated through target."""

    def __init__(self, p0, r0=np.array([0, 0, 0]), id_dictionary=None):
        if id_dictionary is None:
            id_dictionary = {}
        self.set_ids(id_dictionary)
        self.set_mass(self.get_ids()["mass"])
        if type(p0) is list:
            p0 = np.array(p0)
        elif type(p0) is int or type(p0) is float:
            if self.get_ids()["mass"] is None:
                self._mass = MASS[self.get_ids()["PID"]]
            p0 = np.array([p0, 0, 0, np.sqrt(p0 ** 2 - self._mass ** 2)])
        self.set_p0(p0)
        if type(r0) is list:
            r0 = np.array(r0)
        self.set_r0(r0)
        self.set_ended(False)
        self.set_pf(p0)
        self.set_rf(r0)

    def set_ids(self, value):
        self._IDs = {k: value.get(k, DEFAULT_IDS[k]) for k in DEFAULT_IDS}

    def get_ids(self):
        return self._IDs

    def update_ids(self, key, value):
        self._IDs[key] = value

    def get_pid(self):
        return self._IDs["PID"]

    def get_parent_pid(self):
        return self._IDs["parent_PID"]

    def get_weight(self):
        return self._IDs["weight"]

    def set_mass(self, value):
        self._mass = value

    def set_p0(self, value):
        self._p0 = value
        if self._mass is None:
            # particle.py:125-131: mass from the invariant, rounded to 6 places
            m = round(np.sqrt(round(value[0] ** 2 - value[1] ** 2 - value[2] ** 2 - value[3] ** 2, 12)), 6)
            self._mass = m
            self._IDs["mass"] = m

    def get_p0(self):
        return self._p0

    def set_pf(self, value):
        self._pf = value

    def get_pf(self):
        return self._pf

    def set_r0(self, value):
        self._r0 = value

    def get_r0(self):
        return self._r0

    def set_rf(self, value):
        self._rf = value

    def get_rf(self):
        return self._rf

    def set_ended(self, value):
        if value is not True and value is not False:
            raise ValueError("Ended property must be a boolean.")
        self._Ended = value

    def get_ended(self):
        return self._Ended

    def copy(self):
        return Particle(self.get_p0(), self.get_r0(), self.get_ids())

    def get_angle_to_z_0(self):
        E0, px0, py0, pz0 = self.get_p0()
        return np.arccos(pz0 / np.sqrt(px0 ** 2 + py0 ** 2 + pz0 ** 2))

    def rotation_matrix(self):
        """particle.py:176-185"""
        E0, px0, py0, pz0 = self.get_pf()
        ThZ = np.arccos(pz0 / np.sqrt(px0 ** 2 + py0 ** 2 + pz0 ** 2))
        PhiZ = np.arctan2(py0, px0)
        return [[np.cos(ThZ) * np.cos(PhiZ), -np.sin(PhiZ), np.sin(ThZ) * np.cos(PhiZ)],
                [np.cos(ThZ) * np.sin(PhiZ), np.cos(PhiZ), np.sin(ThZ) * np.sin(PhiZ)],
                [-np.sin(ThZ), 0, np.cos(ThZ)]]

    def __deepcopy__(self, memo):
        new = Particle.__new__(Particle)
        for k, v in self.__dict__.items():
            setattr(new, k, _copy.deepcopy(v, memo))
        return new
