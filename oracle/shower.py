"""CPU restatement of PETITE's SM shower transport loop (oracle).

TEST INFRASTRUCTURE: used only by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``.  The product never imports it.

Follows ``src/PETITE/shower.py``:

* ``get_mfp``             shower.py:357-389
* ``propagate``           shower.py:509-601
* process choice          shower.py:665-698 (numpy ``choice``: cumsum, normalise
                          by the last element, ``searchsorted(side='right')``)
* ``draw_sample``         shower.py:401-465 (LU_Key = argmin|E_i - E| + 1,
                          clipped; proposals in batches of ``neval``)
* ``sample_scattering``   shower.py:467-507
* ``generate_shower``     shower.py:603-708 (list order = processing order)

Random numbers come from :mod:`oracle.philox` streams keyed by particle, in
the order the reference consumes them for that particle.
"""
from __future__ import annotations

import math
from bisect import bisect_right

import numpy as np

from . import physics as P
from .philox import Stream, daughter_key, primary_key


# ----------------------------------------------------------------- tables
class OracleTables:
    """Reads the bundled ``sm_tables.npz`` (or arrays in the same layout)."""

    def __init__(self, npz_path: str, target: str, maxF_fudge: float = 1.0):
        z = np.load(npz_path, allow_pickle=False)
        targets = [str(t) for t in z["targets"]]
        if target not in targets or target not in P.TARGETS:
            raise Exception("Target Material is not in library")
        ti = P.TARGETS[target]
        self.target = target
        self.Z, self.A, self.rho, self.dEdx = ti["Z_T"], ti["A_T"], ti["rho"], ti["dEdx"]
        j = targets.index(target)
        self.maps = {}
        for proc in P.PROCESS_CODE:
            E = z[f"{proc}/energy"]
            grid, nn = z[f"{proc}/grid"], z[f"{proc}/nnodes"]
            rows = []
            for i in range(len(E)):
                rows.append(dict(E=float(E[i]), neval=int(z[f"{proc}/neval"][i]),
                                 maxF=float(z[f"{proc}/max_F"][i, j]) * maxF_fudge,
                                 grid=[grid[i, k, :nn[i, k]].tolist() for k in range(grid.shape[1])]))
            self.maps[proc] = rows
            if proc == "Brem":
                self.Eg_min = float(z[f"{proc}/Eg_min"][0])
                self.Ee_min = float(z[f"{proc}/Ee_min"][0])
        self.map_E = {p: np.array([r["E"] for r in rows]) for p, rows in self.maps.items()}
        xs = {p: np.array(z[f"{p}/xsec/{target}"]) for p in P.PROCESS_CODE}
        while xs["MuonE"][0][1] == 0.0:                     # shower.py:238-239
            xs["MuonE"] = xs["MuonE"][1:]
        # shower.py:242-246
        self.min_calc = {
            11: min(xs["Brem"][0][0], xs["Moller"][0][0]),
            -11: min(xs["Brem"][0][0], xs["Bhabha"][0][0], xs["Ann"][0][0]),
            13: max(min(xs["MuonBrem"][0][0], xs["MuonE"][0][0]), 0.120),
            -13: max(min(xs["MuonBrem"][0][0], xs["MuonE"][0][0]), 0.120),
            22: min(xs["PairProd"][0][0], xs["Comp"][0][0]),
        }
        # shower.py:202-208, 273-295
        nZ = self.rho / P.m_proton_grams / self.A
        ne = nZ * self.Z
        k = P.GeVsqcm2
        BS = xs["Brem"]
        self.ns = {
            "Brem": (BS[:, 0].tolist(), (nZ * k * BS[:, 1]).tolist()),
            "PairProd": (xs["PairProd"][:, 0].tolist(), (nZ * k * xs["PairProd"][:, 1]).tolist()),
            "Ann": (xs["Ann"][:, 0].tolist(), (ne * k * xs["Ann"][:, 1]).tolist()),
            "Comp": (xs["Comp"][:, 0].tolist(), (ne * k * xs["Comp"][:, 1]).tolist()),
            "MuonBrem": (xs["MuonBrem"][:, 0].tolist(), (nZ * k * xs["MuonBrem"][:, 1]).tolist()),
        }
        bm = np.geomspace(3.0 * P.m_electron + self.Ee_min, BS[:, 0][-1], len(BS))
        self.ns["Moller"] = (bm.tolist(), [ne * k * P.sigma_moller(e, self.Ee_min) for e in bm])
        self.ns["Bhabha"] = (bm.tolist(), [ne * k * P.sigma_bhabha(e, self.Ee_min) for e in bm])
        me, mm, Em = P.m_electron, P.m_muon, self.Ee_min
        emin = 1.0 / (2.0 * me) * (me * (Em - me) + math.sqrt(me * (Em + me) * (me * (Em - me) + 2 * mm ** 2)))
        if emin < xs["MuonE"][0][0]:
            emin = xs["MuonE"][0][0]
        mg = np.geomspace(emin, bm[-1], len(BS))
        self.ns["MuonE"] = (mg.tolist(), [ne * k * P.sigma_muone(e, self.Ee_min) for e in mg])


def interp(E, table):
    """scipy ``interp1d(kind='linear', bounds_error=False, fill_value=0.0)`` at a
    scalar: numpy's ``interp`` arithmetic inside [x0, xN], 0 outside."""
    xs, ys = table
    if E < xs[0] or E > xs[-1]:
        return 0.0
    j = bisect_right(xs, E) - 1
    if j >= len(xs) - 1:
        return ys[-1]
    if xs[j] == E:
        return ys[j]
    slope = (ys[j + 1] - ys[j]) / (xs[j + 1] - xs[j])
    r = slope * (E - xs[j]) + ys[j]
    if math.isnan(r):
        r = slope * (E - xs[j + 1]) + ys[j + 1]
        if math.isnan(r) and ys[j] == ys[j + 1]:
            r = ys[j]
    return r


def map_point(grid, y):
    """VEGAS map y -> (x, jac): increment i = floor(y*ninc) (<= ninc-1),
    x = g[i] + (g[i+1]-g[i]) * (y*ninc - i), jac = prod ninc*(g[i+1]-g[i])."""
    x = []
    jac = 1.0
    for g, yy in zip(grid, y):
        ninc = len(g) - 1
        t = yy * ninc
        i = min(int(math.floor(t)), ninc - 1)
        inc = g[i + 1] - g[i]
        x.append(g[i] + inc * (t - i))
        jac = jac * (ninc * inc)
    return x, jac


# ----------------------------------------------------------------- records
class Rec:
    """One row of the output list (the reference's Particle)."""
    __slots__ = ("p0", "r0", "pf", "rf", "pid", "mass", "weight", "gen", "proc",
                 "parent", "bit", "pkey", "ended", "primary", "parent_pid", "draws")

    def __init__(self, p0, r0, pid, mass, weight, gen, proc, parent, bit, pkey, primary, parent_pid):
        self.p0 = tuple(float(v) for v in p0)
        self.r0 = tuple(float(v) for v in r0)
        self.pf = self.p0
        self.rf = self.r0
        self.pid = pid
        self.mass = mass
        self.weight = weight
        self.gen = gen
        self.proc = proc          # -1 = "Input"
        self.parent = parent      # index in the shower list, -1 for the primary
        self.bit = bit
        self.pkey = pkey
        self.ended = False
        self.primary = primary
        self.parent_pid = parent_pid
        self.draws = 0


class NoSampleFound(Exception):
    pass


def invariant_mass(p):
    """particle.py:125-131 -- mass when none is given (rounded to 6 dp)."""
    return round(math.sqrt(round(p[0] ** 2 - p[1] ** 2 - p[2] ** 2 - p[3] ** 2, 12)), 6)


class OracleShower:
    def __init__(self, tables: OracleTables, min_energy: float, seed: int = 0,
                 max_n_integrators: int = 10000, rescale_MCS: float = 1.0, fast_MCS_mode: bool = True):
        self.t = tables
        self.fast_mcs = fast_MCS_mode              # shower.py:147-151
        self.min_energy = min_energy
        self.seed = seed
        self.max_n_integrators = max_n_integrators
        self.rescale = rescale_MCS
        self.losses = tables.dEdx * 0.1          # MeV/cm -> GeV/m (shower.py:649-653)

    # -- shower.py:357-389
    def nsigma_total(self, pid, E):
        ns = self.t.ns
        if pid == 22:
            return interp(E, ns["PairProd"]) + interp(E, ns["Comp"])
        if pid == 11:
            return interp(E, ns["Brem"]) + interp(E, ns["Moller"])
        if pid == -11:
            return interp(E, ns["Brem"]) + interp(E, ns["Bhabha"]) + interp(E, ns["Ann"])
        if abs(pid) == 13:
            return interp(E, ns["MuonBrem"]) + interp(E, ns["MuonE"])
        raise ValueError(pid)

    def mfp(self, pid, E):
        n = self.nsigma_total(pid, E)
        if n <= 0.0:
            return 1.0e12
        return P.cmtom / n

    def _mcs(self, pf, t, m_lepton, s):
        E, px, py, pz = pf
        if not P.norm3(px, py, pz) > 0:
            return pf
        if not self.fast_mcs:
            return P.scattered_momentum_bethe(pf, t, self.t.A, self.t.Z, self.rescale, s.next)
        u1, u2, u3, u4 = s.next(), s.next(), s.next(), s.next()
        return P.scattered_momentum_fast(pf, t, self.t.A, self.t.Z, self.rescale, m_lepton, u1, u2, u3, u4)

    # -- shower.py:509-601
    def propagate(self, r: Rec, s: Stream, ms: bool):
        pme = max(self.t.min_calc[r.pid], self.min_energy, r.mass)
        if r.p0[0] < pme:
            r.ended = True
            return
        if r.pid == 22:
            mfp = self.mfp(r.pid, r.pf[0])
            distC = s.next()
            dist = mfp * math.log(1.0 / (1.0 - distC))
            _, px, py, pz = r.p0
            n = P.norm3(px, py, pz)
            hx, hy, hz = px / n, py / n, pz / n
            x0, y0, z0 = r.r0
            r.rf = (x0 + hx * dist, y0 + hy * dist, z0 + hz * dist)
        else:
            losses = self.losses
            rho = self.t.rho
            m_tab = P.MASS[r.pid]
            hard = False
            dz = 0.0
            while not hard and r.pf[0] >= pme:
                mfp = self.mfp(r.pid, r.pf[0])
                u_hard = s.next()
                dz = mfp / (6 + (20 - 6) * s.next())
                if u_hard > math.exp(-dz / mfp):
                    hard = True
                else:
                    r.pf = P.lose_energy(r.pf, r.mass, losses * dz)
                    self._move(r, dz)
                    if ms:
                        r.pf = self._mcs(r.pf, rho * (dz / P.cmtom), m_tab, s)
            distC = s.next()
            if r.pf[0] < pme:
                last = distC * dz
            else:
                mfp = self.mfp(r.pid, r.pf[0])
                last = mfp * math.log(1.0 / (1.0 + (math.exp(-dz / mfp) - 1) * distC))
            r.pf = P.lose_energy(r.pf, r.mass, losses * last)
            self._move(r, last)
            if ms:
                # shower.py:596-598 passes no m_lepton: the default (electron) applies
                r.pf = self._mcs(r.pf, rho * (last / P.cmtom), P.m_electron, s)
        r.ended = True

    @staticmethod
    def _move(r, dist):
        _, px, py, pz = r.pf
        n = P.norm3(px, py, pz)
        if n > 0.0:
            x, y, z = r.rf
            r.rf = (x + px / n * dist, y + py / n * dist, z + pz / n * dist)

    # -- shower.py:665-698
    def choose(self, r: Rec, s: Stream):
        E = r.pf[0]
        ns = self.t.ns
        if r.pid == 11:
            names = ("Brem", "Moller")
        elif r.pid == -11:
            names = ("Brem", "Ann", "Bhabha")
        elif r.pid == 22:
            names = ("PairProd", "Comp")
        else:
            names = ("MuonE", "MuonBrem")
        c = [interp(E, ns[n]) for n in names]
        SC = sum(c)
        if SC == 0.0 or math.isnan(SC):
            return None
        p = [v / SC for v in c]
        if min(p) < 0 or abs(sum(p) - 1.0) > 1.5e-8:
            raise ValueError("probabilities do not sum to 1 / are not non-negative")
        cdf = list(np.cumsum(p))
        cdf = [v / cdf[-1] for v in cdf]
        u = s.next()
        idx = bisect_right(cdf, u)
        return names[idx]

    # -- shower.py:401-465
    def draw_sample(self, E, process, s: Stream, count=None):
        rows = self.t.maps[process]
        energies = self.t.map_E[process]
        key = int(np.argmin(np.abs(energies - E))) + 1
        if key >= len(rows):
            key = len(rows) - 1
        row = rows[key]
        maxF, neval, grid = row["maxF"], row["neval"], row["grid"]
        d = P.DIM[process]
        m_lep = P.m_muon if process == "MuonBrem" else P.m_electron
        n_used = 0
        proposals = 0
        while n_used < self.max_n_integrators:
            n_used += 1
            for _ in range(neval):
                y = [s.next() for _ in range(d)]
                x, jac = map_point(grid, y)
                wgt = jac / neval
                proposals += 1
                f = P.dsigma(process, x, E, self.t.Z, self.t.Eg_min, self.t.Ee_min, m_lep)
                if maxF * s.next() < wgt * f:
                    if count is not None:
                        count.append(proposals)
                    return x, key
        raise NoSampleFound("No Sample Found", process, E, key)

    # -- shower.py:467-507
    def sample_scattering(self, r: Rec, process, s: Stream, index):
        E0 = r.pf[0]
        if E0 <= max(self.t.min_calc[r.pid], self.min_energy, r.mass):
            return None
        RM = P.rotation_matrix_from(r.pf)
        x, _ = self.draw_sample(E0, process, s)
        ph = 2.0 * math.pi * s.next()
        if process in ("Brem", "MuonBrem"):
            a, b = P.e_to_egamma(E0, r.mass, x, ph)
        elif process == "PairProd":
            a, b = P.gamma_to_epem(E0, x, ph)
        elif process == "Comp":
            a, b = P.compton(E0, x[0], ph)
        elif process == "Ann":
            a, b = P.annihilation(E0, x[0], ph)
        elif process in ("Moller", "Bhabha"):
            a, b = P.ee_to_ee(E0, x[0], ph)
        else:
            a, b = P.mue_to_mue(E0, x[0], ph)
        pids = P.PROCESS_PIDS[process]
        out = []
        for bit, (v, pid) in enumerate(zip((a, b), pids)):
            if pid == 0:
                pid = r.pid
            lab = (v[0],
                   RM[0][0] * v[1] + RM[0][1] * v[2] + RM[0][2] * v[3],
                   RM[1][0] * v[1] + RM[1][1] * v[2] + RM[1][2] * v[3],
                   RM[2][0] * v[1] + RM[2][1] * v[2] + RM[2][2] * v[3])
            out.append(Rec(lab, r.rf, pid, P.MASS[pid], r.weight, r.gen + 1,
                           P.PROCESS_CODE[process], index, bit, daughter_key(r.pkey, bit),
                           r.primary, r.pid))
        return out

    # -- shower.py:603-708
    def generate_shower(self, p0, r0=(0.0, 0.0, 0.0), pid=11, mass=None, weight=1.0,
                        primary_index=0, ms=True, pkey=None):
        if pid not in (11, -11, 22, 13, -13):
            raise ValueError(f"unsupported PID {pid}")
        if mass is None:
            mass = invariant_mass(p0)
        key = primary_key(primary_index) if pkey is None else pkey
        prim = Rec(p0, r0, pid, mass, weight, 0, -1, -1, 0, key, primary_index, 22)
        out = [prim]
        if prim.p0[0] < self.min_energy:
            return out
        k = 0
        while k < len(out):
            r = out[k]
            s = Stream(self.seed, r.pkey)
            self.propagate(r, s, ms=(ms and r.pid != 22))
            # shower.py:656-660: the last particle of the list stops the loop
            # before the process choice when it ended below min_energy.
            if k == len(out) - 1 and r.pf[0] < self.min_energy:
                r.draws = s.n
                break
            proc = self.choose(r, s)
            if proc is not None:
                kids = self.sample_scattering(r, proc, s, k)
                if kids is not None:
                    for dp in kids:
                        if dp.p0[0] > self.min_energy:
                            out.append(dp)
            r.draws = s.n
            k += 1
        return out
