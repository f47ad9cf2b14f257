"""Particle record with PETITE's interface (particle.py:50-424).

``Shower.generate_shower`` returns a list of these, with the same keys in
``get_ids()`` as PETITE (``particle.py:22-28``).  Besides the record, the
class carries PETITE's per-particle utilities: energy loss, the rest-to-lab
boost, two- and three-body decays and the meson decay chain
(``particle.py:143-424``).  Those draw from numpy's global generator in the
reference's order, so a seeded numpy state gives PETITE's own results.
"""
from __future__ import annotations

import copy as _copy

import numpy as np

from .tables import M_ELECTRON, M_MUON

MEV = 1e-3
# particle.py:4-13 with physical_constants.py:29-38 (masses in GeV)
M_PI0, M_PI_PM, M_K_PM = 134.9768 * MEV, 139.57039 * MEV, 493.677 * MEV
M_ETA, M_ETA_PRIME, M_OMEGA, M_PROTON = 547.862 * MEV, 957.78 * MEV, 782.65 * MEV, 938.272088 * MEV
MASS = {11: M_ELECTRON, -11: M_ELECTRON, 12: 0.0, -12: 0.0, 22: 0.0, 13: M_MUON, -13: M_MUON,
        14: 0.0, -14: 0.0, 111: M_PI0, 211: M_PI_PM, -211: M_PI_PM, 321: M_K_PM, -321: M_K_PM,
        221: M_ETA, 331: M_ETA_PRIME, 2212: M_PROTON, 223: M_OMEGA}

# particle.py:15-48: interaction lengths (m), decay lengths c*tau (m), and
# decay modes as (branching ratio, daughter PIDs), first mode first
INT_LENGTH = {211: 1.796e-1, -211: 1.796e-1, 321: 2.2875e-1, -321: 2.2875e-1}
DECAY_LENGTH = {211: 7.8045, -211: 7.8045, 321: 3.711, -321: 3.711, 111: 25.3 * (1e-9)}
MESON_DECAYS = {111: [(0.98823, (22, 22))],
                221: [(0.3936, (22, 22)), (0.3257, (111, 111, 111))],
                331: [(0.02307, (22, 22)), (0.224, (111, 111, 221)), (0.00250, (111, 111, 111))],
                223: [(0.0828, (22, 111))],
                211: [(0.9998, (-13, 14))], -211: [(0.9998, (13, -14))],
                321: [(0.6356, (-13, 14))], -321: [(0.6356, (13, -14))]}
MESON_TWOBODY_BR = {pid: modes[0][0] for pid, modes in MESON_DECAYS.items()}

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

    # -------------------------------------------------------- utilities
    def lose_energy(self, value):
        """particle.py:143-153: lowers the final energy by ``value`` (not below
        the mass), keeping the direction."""
        E0, px0, py0, pz0 = self.get_pf()
        p30 = np.linalg.norm([px0, py0, pz0])
        E = E0 - value
        if E <= self._mass:
            E = self._mass
        p3f = np.sqrt(E ** 2 - self._mass ** 2)
        if p3f > 0.0:
            self.set_pf([E, px0 / p30 * p3f, py0 / p30 * p3f, pz0 / p30 * p3f])
        elif p3f == 0.0:
            self.set_pf([self.get_ids()["mass"], 0.0, 0.0, 0.0])

    def boost_matrix(self):
        """particle.py:187-207: the Lorentz boost from the particle's rest
        frame to the lab, from its final momentum and mass."""
        E0, px0, py0, pz0 = self.get_pf()
        gamma = E0 / self._mass
        beta = 1.0 if gamma == 1.0 else np.sqrt(1.0 - 1.0 / gamma ** 2)
        pmag = np.linalg.norm([px0, py0, pz0])
        if pmag == 0.0:
            return np.identity(4)
        b = beta * np.array([px0, py0, pz0]) / pmag
        L = np.empty((4, 4))
        L[0, 0] = gamma
        L[0, 1:] = L[1:, 0] = gamma * b
        for i in range(3):
            for j in range(3):
                L[i + 1, j + 1] = (1 if i == j else 0) + (gamma - 1) * b[i] * b[j] / beta ** 2
        return L.tolist()

    @staticmethod
    def _daughter_mass(d, which):
        if "mass" in d:
            return d["mass"]
        if "PID" not in d:
            raise ValueError(f"Masses must be included in `{which}' when calling the decay")
        if d["PID"] not in MASS:
            raise ValueError("PID provided for unspecified particle.")
        d["mass"] = MASS[d["PID"]]
        return d["mass"]

    def two_body_decay(self, p1_dict, p2_dict, angular_information="Isotropic"):
        """particle.py:209-256: decay into two particles, back to back in the
        rest frame along a direction (cos theta, phi) drawn isotropically (or
        from the inverse CDFs given), then boosted to the lab.  Particle 1
        goes along -n, particle 2 along +n, n = (sin t sin p, sin t cos p, cos t)."""
        M = self._mass
        m1, m2 = self._daughter_mass(p1_dict, "p1_dict"), self._daughter_mass(p2_dict, "p2_dict")
        E1 = (M ** 2 - m2 ** 2 + m1 ** 2) / (2 * M)
        E2 = (M ** 2 - m1 ** 2 + m2 ** 2) / (2 * M)
        k = np.sqrt(E1 ** 2 - m1 ** 2)
        if angular_information == "Isotropic":
            ct = np.random.uniform(-1.0, 1.0)
            ph = np.random.uniform(0.0, 2.0 * np.pi)
        elif len(angular_information) == 2:
            u_ct, u_ph = np.random.uniform(low=0.0, high=1.0, size=2)
            ct, ph = angular_information[0](u_ct), angular_information[1](u_ph)
        else:
            ct = angular_information(np.random.uniform(low=0.0, high=1.0, size=1))
            ph = np.random.uniform(0.0, 2.0 * np.pi)
        st = np.sqrt(1 - ct ** 2)
        n = [st * np.sin(ph), st * np.cos(ph), ct]
        L = self.boost_matrix()
        q1 = np.dot(L, [E1, -k * n[0], -k * n[1], -k * n[2]])
        q2 = np.dot(L, [E2, k * n[0], k * n[1], k * n[2]])
        return [Particle(q1, self.get_rf(), p1_dict), Particle(q2, self.get_rf(), p2_dict)]

    def dalitz_range(self, m12sq, m1, m2, m3, M):
        """particle.py:258-264: the allowed m23^2 interval at a given m12^2
        (the energies of 2 and 3 in the 12 rest frame)."""
        r = np.sqrt(m12sq)
        e2 = (m12sq - m1 ** 2 + m2 ** 2) / (2 * r)
        e3 = (M ** 2 - m12sq - m3 ** 2) / (2 * r)
        k2, k3 = np.sqrt(e2 ** 2 - m2 ** 2), np.sqrt(e3 ** 2 - m3 ** 2)
        return (e2 + e3) ** 2 - (k2 + k3) ** 2, (e2 + e3) ** 2 - (k2 - k3) ** 2

    def three_body_decay(self, p1_dict, p2_dict, p3_dict, dalitz_information="Flat",
                         angular_information="Isotropic"):
        """particle.py:266-357: (m12^2, m23^2) drawn flat over the Dalitz plot
        (or by accept-reject against (max, f) when given); the rest-frame
        momenta from them; the event plane oriented by (cos theta, phi) of
        particle 1 (along -n) and the angle gamma of particle 2 about it; boosted."""
        M = self._mass
        m1 = self._daughter_mass(p1_dict, "p1_dict")
        m2 = self._daughter_mass(p2_dict, "p2_dict")
        m3 = self._daughter_mass(p3_dict, "p3_dict")
        lo12, hi12 = (m1 + m2) ** 2, (M - m3) ** 2
        lo23, hi23 = (m2 + m3) ** 2, (M - m1) ** 2
        while True:
            m12sq, m23sq = np.random.uniform(lo12, hi12), np.random.uniform(lo23, hi23)
            a, b = self.dalitz_range(m12sq, m1, m2, m3, M)
            if m23sq < a or m23sq > b:
                continue
            if dalitz_information == "Flat":
                break
            try:
                fmax, f = dalitz_information
                if f(m12sq, m23sq, m1, m2, m3, M) > np.random.uniform(0, fmax):
                    break
            except Exception:
                raise ValueError("Dalitz information must be a tuple of (max value, function) for matrix-element-level sampling")
        E1 = (M ** 2 - m23sq + m1 ** 2) / (2 * M)
        E3 = (M ** 2 - m12sq + m3 ** 2) / (2 * M)
        E2 = M - E1 - E3
        k1, k2, k3 = np.sqrt(E1 ** 2 - m1 ** 2), np.sqrt(E2 ** 2 - m2 ** 2), np.sqrt(E3 ** 2 - m3 ** 2)
        c12 = (m1 ** 2 + m2 ** 2 + 2 * E1 * E2 - m12sq) / (2 * k1 * k2)     # opening angle of 1 and 2
        s12 = np.sqrt(1 - c12 ** 2)
        if angular_information == "Isotropic":
            ct = np.random.uniform(-1.0, 1.0)
            ph, ga = np.random.uniform(0.0, 2.0 * np.pi, size=2)
        elif len(angular_information) == 3:
            u = np.random.uniform(low=0.0, high=1.0, size=3)
            ct, ph, ga = (angular_information[i](u[i]) for i in range(3))
        else:
            ct = angular_information(np.random.uniform(low=0.0, high=1.0, size=1))
            ph, ga = np.random.uniform(0.0, 2.0 * np.pi, size=2)
        st = np.sqrt(1 - ct ** 2)
        sp, cp, sg, cg = np.sin(ph), np.cos(ph), np.sin(ga), np.cos(ga)
        q1 = [E1, -k1 * st * sp, -k1 * st * cp, -k1 * ct]
        # particle 2 at angle acos(c12) from particle 1, turned by gamma about it
        q2 = [E2, k2 * (s12 * cp * sg - s12 * cg * ct * sp - c12 * st * sp),
              k2 * (-cp * (s12 * cg * ct + c12 * st) - s12 * sg * sp),
              k2 * (s12 * cg * st - c12 * ct)]
        q3 = [E3, -q1[1] - q2[1], -q1[2] - q2[2], -q1[3] - q2[3]]
        L = self.boost_matrix()
        return [Particle(np.dot(L, q1), self.get_rf(), p1_dict), Particle(np.dot(L, q2), self.get_rf(), p2_dict),
                Particle(np.dot(L, q3), self.get_rf(), p3_dict)]

    def decay_int_prob(self, x, int_length, ctau0):
        """particle.py:359-366: total rate (decay plus interaction, per m) and
        its exponential density at distance x."""
        gamma = self.get_p0()[0] / self.get_ids()["mass"]
        beta = np.sqrt(1 - 1 / gamma ** 2)
        rate = 1.0 / (ctau0 * gamma * beta) + 1.0 / int_length
        return rate, rate * np.exp(-rate * x)

    def draw_x_sample(self, int_length, ctau0):
        """particle.py:368-377: distance to the first decay or interaction, by
        accept-reject on [0, 4/density(0))."""
        c = self.decay_int_prob(0, int_length, ctau0)[0]
        x_max = 4 / self.decay_int_prob(0, int_length, ctau0)[1]
        while True:
            x = np.random.uniform(0, x_max)
            u = np.random.uniform(0, 1)
            if u < self.decay_int_prob(x, int_length, ctau0)[1] / c:
                return x

    def prob_decay_b_int(self, int_length, ctau0):
        """particle.py:379-389: probability that a long-lived particle decays
        before it interacts, at a drawn distance."""
        x = self.draw_x_sample(int_length, ctau0)
        gamma = self.get_p0()[0] / self.get_ids()["mass"]
        beta = np.sqrt(1 - 1 / gamma ** 2)
        ctau = ctau0 * gamma * beta
        rate = 1.0 / ctau + 1.0 / int_length
        return (1 - np.exp(-rate * x)) / (1 + ctau / int_length)

    def decay_particle(self):
        """particle.py:391-424: picks a decay mode by branching ratio and runs
        a two-body decay; daughters carry weight * (sum of the ratios), IDs
        2*ID and 2*ID+1 and "SMDecay".  A long-lived meson is first moved to
        its decay point and its daughters also weighted by the chance to
        decay before interacting."""
        pid = self.get_ids()["PID"]
        if pid not in MESON_DECAYS:
            raise ValueError("Decay options for particle not specified. Edit dictionary in 'particle.py' to include it")
        modes = MESON_DECAYS[pid]
        if len(modes) == 1:
            br_sum, decay = modes[0]
        else:
            brs = [m[0] for m in modes]
            br_sum = np.sum(brs)
            decay = modes[np.random.choice(range(len(modes)), p=brs / br_sum)][1]
        if len(decay) > 2:
            raise ValueError("Three-body (and above) decays not yet implemented")
        ids = self.get_ids()
        stability = ids["stability"]
        if stability not in ("short-lived", "long-lived"):
            # the reference leaves its result unassigned for a stable particle
            raise UnboundLocalError(f"decay_particle: no decay for a particle with stability {stability!r}")
        extra = 1.0
        if stability == "long-lived":
            dz = self.draw_x_sample(INT_LENGTH[pid], DECAY_LENGTH[pid])
            px, py, pz = self.get_pf()[1:]
            p = np.linalg.norm([px, py, pz])
            if p > 0.0:
                x, y, z = self.get_rf()
                self.set_rf([x + px / p * dz, y + py / p * dz, z + pz / p * dz])
        dicts = []
        for bit in (0, 1):
            if stability == "long-lived":
                extra = self.prob_decay_b_int(INT_LENGTH[pid], DECAY_LENGTH[pid])
            dicts.append({"PID": decay[bit], "mass": MASS[decay[bit]], "weight": ids["weight"] * br_sum * extra,
                          "ID": 2 * ids["ID"] + bit, "generation_process": "SMDecay",
                          "generation_number": ids["generation_number"] + 1, "production_time": ids["decay_time"]})
        new = self.two_body_decay(p1_dict=dicts[0], p2_dict=dicts[1])
        self.set_ended(True)
        return new

    def __deepcopy__(self, memo):
        new = Particle.__new__(Particle)
        for k, v in self.__dict__.items():
            setattr(new, k, _copy.deepcopy(v, memo))
        return new
