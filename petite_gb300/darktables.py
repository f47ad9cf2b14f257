"""Native build of the per-(mass, target) dark-shower tables from PETITE's
dark pickles.

PETITE's ``DarkShower`` constructor (dark_shower.py:69-130) reads
``dark_maps.pkl`` and ``dark_xsec.pkl`` from its dict_dir and derives the
rest:

* the bound-electron DarkAnn/DarkComp cross sections on 200 log-spaced
  energies (``set_DarkAnnXSec``/``set_DarkCompXSec``, :254-284) from
  ``sigma_atomic`` (atomic_annihilation.py:95-104) and ``sigma_atomic_comp``
  (atomic_compton.py:94-109);
* the track-length weight of each incoming energy (``set_weight_arrays``,
  :337-452): the integral of n*sigma_dark(E)/(dE/dx) times the probability
  of reaching E without an SM interaction, from the first tabulated energy
  up to Ei, split at Ei minus ten mean free paths of loss;
* the dR/dE tables (``set_drate_dE``, :454-593): the same integrand over ten
  equal bins from max(Ei - 10 mfp dE/dx, E_first) to Ei, with the
  free-electron annihilation's extra resonant bin in closed form (:495-517);
* the thresholds (:219-240) and the SM interaction integrals behind the
  survival probabilities (shower.py:296-351).

PETITE caches the weights and dR/dE in ``dark_weights.pkl`` and
``dark_drate.pkl`` and reads them back for a (mass, target) it has seen;
the builder does the same (the bound-electron annihilation tables are always
recomputed there, as in :447-451 and :554-555).

Integrals.  PETITE integrates with scipy's ``quad`` (QUADPACK's adaptive
21-point Gauss-Kronrod rule, tolerance 1.49e-8, at most 50 subintervals),
and with many kinks in the integrands the 50-subinterval limit is often
what stops it: its interaction integrals and weights carry quad's
truncation error, up to about 1e-3 relative.  The builder therefore calls
the same ``quad`` on the same integrands, evaluated in plain floating point
in numpy's order of operations (``np.interp``'s slope form, the same
divisions), so that its tables are PETITE's, not a more accurate set.
"""
from __future__ import annotations

import bisect
import math
import os
import pickle

import numpy as np
from scipy.integrate import quad

from . import tables as T

DARK_PROCESSES = ("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")
# ------------------------------------------------------------ interpolants
class Linear:
    """scipy's interp1d(x, y, fill_value=0.0, bounds_error=False) at one
    point, as np.interp computes it."""

    def __init__(self, x, y, fill: float = 0.0):
        self.x = [float(v) for v in np.asarray(x, np.float64)]
        self.y = [float(v) for v in np.asarray(y, np.float64)]
        self.fill = fill

    def __call__(self, E: float) -> float:
        x, y = self.x, self.y
        if not (x[0] <= E <= x[-1]):                    # below, above, or nan
            return self.fill if E == E else E
        if E == x[-1]:
            return y[-1]
        j = bisect.bisect_right(x, E) - 1
        slope = (y[j + 1] - y[j]) / (x[j + 1] - x[j])
        r = slope * (E - x[j]) + y[j]
        if r != r:
            r = slope * (E - x[j + 1]) + y[j + 1]
            if r != r and y[j] == y[j + 1]:
                r = y[j]
        return r


class LogLog:
    """PETITE's interpolate1d(x, y, xspace='log', yspace='log',
    fill_value=-20.0, bounds_error=False) (dark_shower.py:31-45) at one
    point: linear in (log10(x + 1e-20), log10(y + 1e-20)), 10^-20 outside
    the nodes.  ``shift`` is subtracted from the nodes and the argument (the
    free-electron annihilation's E - E_res, dark_shower.py:295)."""

    def __init__(self, x, y, shift: float = 0.0):
        self.shift = shift
        self.x = np.asarray(x, np.float64)
        with np.errstate(invalid="ignore", divide="ignore"):      # nodes below the shift give nan, as there
            self._f = Linear(np.log10(self.x - shift + 1e-20), np.log10(np.asarray(y, np.float64) + 1e-20), -20.0)

    def __call__(self, E: float) -> float:
        u = E - self.shift
        lx = math.log10(u) if u > 0.0 else (-math.inf if u == 0.0 else math.nan)
        return 10.0 ** self._f(lx)


def interaction_integral(f: Linear, x) -> np.ndarray:
    """[quad(f, x[0], x[i]) for each i] (shower.py:298-320)."""
    return np.array([quad(f, x[0], x[i], full_output=1)[0] for i in range(len(x))])


# ------------------------------------------------------ SM survival factors
class Survival:
    """The SM interaction integrals of one target (shower.py:296-320) and the
    probability that an e-, e+ or mu keeps from interacting while it slows
    from Ei to E (``_electron/_positron/_muon_exponential_factor``,
    shower.py:322-351): exp(-(sum_k II_k(Ei) - II_k(E)) / dEdx / cmtom), 0
    for a negative sum or E > Ei."""

    def __init__(self, sm: "T.SMTables"):
        ns = {name: Linear(*sm.nsigma[k]) for k, name in enumerate(T.NS_NAMES)}
        self.ns = ns
        xs = sm.xsec
        bm = sm.nsigma[T.NS_MOLLER][0]
        grids = {"Brem": ("Brem", xs["Brem"][:, 0]), "Ann": ("Ann", xs["Ann"][:, 0]),
                 "Moller": ("Moller", bm), "Bhabha": ("Bhabha", bm),
                 # shower.py:316-317 integrates the mu-e n*sigma on the muon-brem energies
                 "MuonBrem": ("MuonE", xs["MuonBrem"][:, 0]),
                 "MuonE": ("MuonE", xs["MuonE"][:, 0])}
        self._grids = grids
        self._ii = {}
        self.parts = {11: ("Brem", "Moller"), -11: ("Brem", "Ann", "Bhabha"), 13: ("MuonBrem", "MuonE")}
        self.mfp_parts = {11: ("Brem", "Moller"), -11: ("Brem", "Bhabha", "Ann"), 13: ("MuonBrem", "MuonE")}
        self.dEdx = sm.dEdx * (0.1)                        # GeV/m
        self.dEdx_cm = sm.dEdx * (0.1) * T.CMTOM           # GeV/cm

    def ii(self, name: str) -> Linear:
        if name not in self._ii:
            src, x = self._grids[name]
            self._ii[name] = Linear(x, interaction_integral(self.ns[src], x))
        return self._ii[name]

    def factor(self, pid: int, E: float, Ei: float) -> float:
        d = None
        for k in self.parts[pid]:
            f = self.ii(k)
            d = (f(Ei) - f(E)) if d is None else d + (f(Ei) - f(E))
        if d < 0.0 or E > Ei:
            return 0.0
        return math.exp(-d / self.dEdx / T.CMTOM)

    def mfp(self, pid: int, E: float) -> float:
        """get_mfp (shower.py:369-388), metres; 1e12 where n*sigma is zero."""
        ns = None
        for k in self.mfp_parts[pid]:
            v = self.ns[k](E)
            ns = v if ns is None else ns + v
        if ns <= 0.0:
            return 1.0e12
        return T.CMTOM / ns


# ------------------------------------------------- bound-electron sigmas
def _atomic_ab(k, mV, Zeff, alpha, me):
    lam = Zeff * alpha * me
    return me / lam, mV ** 2 / (2 * k * lam), lam


def _annihilation_integral(a, b):
    """The radiative-tail integral of atomic_annihilation.py:10-56 (its b < 1000
    closed form; the b -> infinity series above), written out term by term in
    the same grouping, because the closed form cancels strongly at large b.
    Its second and third polynomial factors are the same expression, as
    there."""
    a2 = a ** 2
    P1 = (1 + a2) * (a * (1 + a2) ** 3 * (5 + 3 * a2) - (1 + a2) ** 2 * (-1 + 15 * a2 + 12 * a ** 4) * b
                     + a * (1 + a2) * (-23 + 38 * a2 + 21 * a ** 4) * b ** 2
                     + 4 * (5 + a2 - 18 * a ** 4 - 6 * a ** 6) * b ** 3
                     + 3 * a * (3 + a2) * (-1 + 7 * a2) * b ** 4
                     + (7 - 29 * a2 - 12 * a ** 4) * b ** 5
                     + a * (7 + 3 * a2) * b ** 6)
    P2 = (3 * (1 + a2) ** 6
          - a * (1 + a2) ** 3 * (3 + 26 * a2 + 15 * a ** 4) * b
          + 3 * (1 + a2) ** 2 * (-7 + 21 * a2 + 23 * a ** 4 + 11 * a ** 6) * b ** 2
          - 3 * a * (1 + a2) * (7 + 69 * a2 + 45 * a ** 4 + 15 * a ** 6) * b ** 3
          + (-11 + 132 * a2 + 9 * a ** 4 * (38 + 5 * a2 * (4 + a2))) * b ** 4
          - 3 * a * (11 + 73 * a2 + 41 * a ** 4 + 11 * a ** 6) * b ** 5
          + 3 * (-1 + 27 * a2 + 17 * a ** 4 + 5 * a ** 6) * b ** 6
          - a * (15 + 10 * a2 + 3 * a ** 4) * b ** 7)
    P4 = ((1 + a2) ** 3 + 6 * a * (1 + a2) ** 2 * b
          - 3 * (1 + 6 * a2 + 5 * a ** 4) * b ** 2
          + 4 * a * (3 + 5 * a2) * b ** 3
          - 3 * (1 + 5 * a2) * b ** 4
          + 6 * a * b ** 5 - b ** 6)
    num = (P1 + P2 * np.arctan2(a, 1) + P2 * np.arctan2(1 + a2 - a * b, b)
           + 4 * b * (P4 * (np.log(1 + (a - b) ** 2) - 2 * np.log(b))))
    closed = num / (8 * (1 + a2) ** 3 * (1 + (a - b) ** 2) ** 3 * b)
    series = (3081 / 280 - (3081 * a2) / 40) / b ** 8 - (709 * a) / (35 * b ** 7) - 91 / (30 * b ** 6)
    return closed if b < 1000 else series


# atomic_annihilation.py:4-5 uses its own rounded constants
_ANN_ALPHA = 1 / 137
_ANN_ME = 0.511E-3


def sigma_atomic(k, mV, Zeff):
    """e+ e-(bound) -> V: tree level plus radiative tail
    (atomic_annihilation.py:58-104), GeV^-2."""
    me, alpha = _ANN_ME, _ANN_ALPHA
    a, b, lam = _atomic_ab(k, mV, Zeff, alpha, me)
    pref = (4.0 * np.pi * alpha) * ((mV ** 2 + 2 * me ** 2) * (2 / 3 / lam / me) * (1 / k ** 2))
    tree = pref * (1 / ((a - b) ** 2 + 1) ** 3)
    s = 2 * k * me + me ** 2
    beta = 2 * alpha / np.pi * (np.log(s / me ** 2) - 1.0)
    return tree + pref * (beta / 2) * _annihilation_integral(a, b)


def _compton_above(a, b):
    """atomic_compton.py:7-41 (a^2 + 1 < a b)."""
    delta = (a - b) ** 2 + 1
    L = np.log(delta) - 2 * np.log(b)
    inner = (-a * (a ** 2 + 1) ** 3 * (3 * a ** 2 + 5)
             + 6 * (a ** 4 + 4 * a ** 2 - 5) * b ** 5
             - 4 * a * (6 * a ** 4 + 23 * a ** 2 - 31) * b ** 4
             + (a - 1) * (a + 1) * (39 * a ** 4 + 190 * a ** 2 + 55) * b ** 3
             - a * (a ** 2 + 1) * (33 * a ** 4 + 98 * a ** 2 - 111) * b ** 2
             + (a ** 2 + 1) ** 2 * (15 * a ** 4 + 32 * a ** 2 - 23) * b)
    Q = (3 * (a ** 2 + 1) ** 4
         - 2 * a * (3 * a ** 4 + 10 * a ** 2 + 15) * (a ** 2 + 1) * b
         + 6 * (a ** 6 + 5 * a ** 4 + 15 * a ** 2 - 5) * b ** 2)
    num = (8 * b * (a ** 2 - 6 * a * b + 1) * L + (a ** 2 + 1) * inner / delta ** 2
           + Q * (np.arctan(b / (a ** 2 - a * b + 1)) + np.arctan(1 / a)))
    return -num / (8 * (a ** 2 + 1) ** 4 * b)


def _compton_below(a, b):
    """atomic_compton.py:43-80 (a^2 + 1 >= a b)."""
    delta = (a - b) ** 2 + 1
    inner = (a * (a ** 2 + 1) ** 3 * (3 * a ** 2 + 5)
             - 6 * (a ** 4 + 4 * a ** 2 - 5) * b ** 5
             + 4 * a * (6 * a ** 4 + 23 * a ** 2 - 31) * b ** 4
             - (a - 1) * (a + 1) * (39 * a ** 4 + 190 * a ** 2 + 55) * b ** 3
             + a * (a ** 2 + 1) * (33 * a ** 4 + 98 * a ** 2 - 111) * b ** 2
             - (a ** 2 + 1) ** 2 * (15 * a ** 4 + 32 * a ** 2 - 23) * b)
    Q = (3 * (a ** 2 + 1) ** 4
         - 2 * a * (3 * a ** 4 + 10 * a ** 2 + 15) * (a ** 2 + 1) * b
         + 6 * (a ** 6 + 5 * a ** 4 + 15 * a ** 2 - 5) * b ** 2)
    L = np.log(delta) - 2 * np.log(b)
    num = ((a ** 2 + 1) * inner + np.pi * Q * delta ** 2 - Q * delta ** 2 * np.arctan(1 / a)
           - delta ** 2 * (8 * b * (a ** 2 - 6 * a * b + 1) * L + Q * np.arctan(b / (a ** 2 - a * b + 1))))
    return num / (8 * (a ** 2 + 1) ** 4 * b * delta ** 2)


def _compton_shape(a, b):
    """atomic_compton.py:82-92: the a^2 + 1 < a b branch falls back to its
    large-b series where the closed form turns negative or b is far past the
    switch."""
    if a ** 2 + 1 < a * b:
        e1 = _compton_above(a, b)
        if e1 < 0.0 or (a ** 2 + 1 < 0.01 * a * b):
            e1 = (-145 + 1015 * a ** 2 + 330 * a * b + 64 * b ** 2) / (420 * b ** 8)
        return e1
    return _compton_below(a, b)


def sigma_atomic_comp(k, mV, Zeff):
    """gamma e-(bound) -> V e- (atomic_compton.py:94-109), GeV^-2."""
    me, alpha = T.M_ELECTRON, T.ALPHA_EM
    a, b, lam = _atomic_ab(k, mV, Zeff, alpha, me)
    s = 2 * k * me + me ** 2
    beta = 2 * alpha / np.pi * (np.log(s / me ** 2) - 1.0)
    if beta < 0.0:
        beta = 0.0
    return (4.0 * np.pi * alpha) * ((mV ** 2 + 2 * me ** 2) * (2 / 3 / lam / me) * (1 / k ** 2) * (beta / 4)
                                    * _compton_shape(a, b))


# ------------------------------------------------------------ the builder
def _strip_zero_rows(xs):
    xs = np.asarray(xs, np.float64)
    while xs[0][1] == 0.0:                           # dark_shower.py:224-225,229-230
        xs = xs[1:]
    return xs


def _pad_bins(d: dict):
    """{Ei: [[center, weight], ...]} -> (Ei sorted, bins (n, nb, 2), nbins)."""
    Ei = np.array(sorted(d.keys()), np.float64)
    rows = [np.asarray(d[e], np.float64).reshape(-1, 2) for e in Ei]
    nb = max(len(r) for r in rows)
    bins = np.zeros((len(Ei), nb, 2))
    cnt = np.zeros(len(Ei), np.int32)
    for i, r in enumerate(rows):
        bins[i, :len(r)] = r
        cnt[i] = len(r)
    return Ei, bins, cnt


class DarkTableBuilder:
    """The tables PETITE's DarkShower constructor makes for one (mass, target).

    ``xsec``: the mass's entry of ``dark_xsec.pkl`` (process -> target ->
    [[E, sigma]]); ``mV``: the vector mass of the thresholds and the
    bound-electron cross sections (PETITE's ``_mV``; the estimator mass keys
    the pickles); ``cached``: the (mass, target) entries of
    ``dark_weights.pkl`` and ``dark_drate.pkl`` if present."""

    def __init__(self, sm: "T.SMTables", xsec: dict, target: str, mV: float, Zeff: float = 29.508,
                 cached_weights: dict | None = None, cached_drate: dict | None = None):
        self.sm, self.target, self.mV, self.Zeff = sm, target, float(mV), float(Zeff)
        for p in DARK_PROCESSES:
            if p not in xsec:
                if p == "DarkAnn":
                    continue                 # no DarkAnn below mV = 2 m_e: the free-electron tables are left out
                raise Exception("Process String does not match library")     # dark_shower.py:210
            if target not in xsec[p]:
                raise Exception("Target Material is not in library")         # dark_shower.py:216
        self.DBS = _strip_zero_rows(xsec["DarkBrem"][target])
        self.DMBS = _strip_zero_rows(xsec["DarkMuonBrem"][target])
        self.DAnnS_free = np.asarray(xsec["DarkAnn"][target], np.float64) if "DarkAnn" in xsec else None
        self.DCS_free = np.asarray(xsec["DarkComp"][target], np.float64)
        me = T.M_ELECTRON
        self.E_res = (self.mV ** 2 - 2 * me ** 2) / (2 * me)                 # dark_shower.py:232-233
        self.E_compth = self.mV ** 2 / (2 * me) + self.mV
        self.cached_weights = cached_weights or {}
        self.cached_drate = cached_drate or {}
        self.surv = Survival(sm)
        self.nZ, self.ne = sm.n_target, sm.n_elec
        self.DAnnS_bound = self._bound_xsec(sigma_atomic, max(sm.min_calc[-11], 0.001 * self.E_res),
                                            self.DBS[-1][0])
        self.DCS_bound = self._bound_xsec(sigma_atomic_comp, max(sm.min_calc[22], 0.001 * self.E_compth),
                                          self.DCS_free[-1][0])
        g = T.GEVSQCM2
        self.ns_brem = LogLog(self.DBS[:, 0], self.nZ * g * self.DBS[:, 1])
        self.ns_mubrem = LogLog(self.DMBS[:, 0], self.nZ * g * self.DMBS[:, 1])
        self.ns_ann_bound = LogLog(self.DAnnS_bound[:, 0], self.ne * g * self.DAnnS_bound[:, 1])
        self.ns_ann_free = None if self.DAnnS_free is None else \
            LogLog(self.DAnnS_free[:, 0], self.ne * g * self.DAnnS_free[:, 1], shift=self.E_res)

    def _bound_xsec(self, sigma, E_min, E_max):
        E = np.logspace(np.log10(E_min), np.log10(E_max), 200)
        return np.column_stack((E, [sigma(e, self.mV, self.Zeff) for e in E]))

    # -------------------------------------------------------- integrands
    def _spec(self, name: str, bound: bool):
        """(pid, integrand f(E, Ei), first tabulated energy, incoming energies)
        of one table (dark_shower.py:311-335)."""
        s = self.surv
        dx = s.dEdx_cm
        if name in ("brem_elec", "brem_positron", "muon_brem"):
            pid = {"brem_elec": 11, "brem_positron": -11, "muon_brem": 13}[name]
            ns = self.ns_mubrem if name == "muon_brem" else self.ns_brem

            def f(E, Ei):
                v = ns(E)
                if v < 1.0e-18:
                    return 0.0
                return v / dx * s.factor(pid, E, Ei)
            xs = self.DMBS if name == "muon_brem" else self.DBS
            return pid, f, xs[0][0], xs[:, 0]
        ns = self.ns_ann_bound if bound else self.ns_ann_free

        def f(E, Ei):
            return ns(E) / dx * s.factor(-11, E, Ei)
        xs = self.DAnnS_bound if bound else self.DAnnS_free
        return -11, f, xs[0][0], xs[:, 0]

    def _loss10(self, pid, Ei):
        return 10 * self.surv.mfp(pid, float(Ei)) * self.surv.dEdx

    # --------------------------------------------------------- the arrays
    def weights(self, name: str, bound: bool = True):
        """construct_*_weight_array (dark_shower.py:337-399): [[Ei, weight]]."""
        key = {"brem_elec": "brem_elec_weights", "brem_positron": "brem_positron_weights",
               "muon_brem": "muon_brem_weights", "ann": "annihilation_weights"}[name]
        if key in self.cached_weights and not (name == "ann" and bound):
            return np.asarray(self.cached_weights[key], np.float64)
        pid, f, E0, Eis = self._spec(name, bound)
        w = np.empty(len(Eis))
        for i, Ei in enumerate(Eis):
            Ei = float(Ei)
            Eb = Ei - self._loss10(pid, Ei)
            if not Eb > E0:
                Eb = E0
            w[i] = quad(f, E0, Eb, args=(Ei,), full_output=1)[0] + quad(f, Eb, Ei, args=(Ei,), full_output=1)[0]
        return np.column_stack((Eis, w))

    def drate(self, name: str, bound: bool = True):
        """_d_rate_d_E_* (dark_shower.py:454-517): {Ei: [[center, weight], ...]}."""
        key = {"brem_elec": "brem_elec_drate", "brem_positron": "brem_positron_drate",
               "muon_brem": "muon_brem_drate", "ann": "annihilation_drate"}[name]
        if key in self.cached_drate and not (name == "ann" and bound):
            return {float(k): np.asarray(v, np.float64) for k, v in self.cached_drate[key].items()}
        pid, f, E0, Eis = self._spec(name, bound)
        free_ann = name == "ann" and not bound
        out = {}
        for Ei in Eis:
            Ei = float(Ei)
            if free_ann and Ei < self.E_res:
                out[Ei] = np.array([[0.0, 0.0]])
                continue
            e = np.linspace(np.max([Ei - self._loss10(pid, Ei), E0]), Ei, 11)
            rows = [[(e[k] + e[k + 1]) / 2., quad(f, e[k], e[k + 1], args=(Ei,), full_output=1)[0]]
                    for k in range(10)]
            if free_ann:
                rows = [self._resonant_bin(Ei)] + rows
            out[Ei] = np.array(rows, np.float64)
        return out

    def _resonant_bin(self, Ei):
        """The free-electron annihilation's resonant bin (dark_shower.py:505-515)."""
        me, alpha = T.M_ELECTRON, T.ALPHA_EM
        mse = self.DAnnS_free[0][0]
        center = 0.5 * (self.E_res + min(mse, Ei))
        sMAX = 2 * (me * min(mse, Ei) + me ** 2)
        beta = (2. * alpha / np.pi) * (np.log(sMAX / me ** 2) - 1.)
        with np.errstate(invalid="ignore"):      # sMAX < mV^2 (mode='approx' above the map mass): nan, as there
            w = ((1 / self.surv.dEdx_cm) * (2 * np.pi ** 2 * alpha / me) * self.ne * T.GEVSQCM2
                 * np.power(np.float64(sMAX - self.mV ** 2), beta) * self.surv.factor(-11, self.E_res, Ei))
        return [center, w]

    def min_dark(self, bound: bool = True):
        """_minimum_calculable_dark_energy (dark_shower.py:234-244): e- brem,
        e+ brem, e+ annihilation, photon Compton, mu brem."""
        if bound:
            return np.array([self.DBS[0][0], self.DBS[0][0], self.E_res / 1000.0, self.E_compth / 1000.0,
                             self.DMBS[0][0]])
        return np.array([self.DBS[0][0], self.DBS[0][0], self.E_res, self.DCS_free[0][0], self.DMBS[0][0]])

    def interaction_integrals(self):
        """[[E, II(E)]] of the positron's three processes (shower.py:298-314)."""
        return {k: np.column_stack((self.surv.ii(k).x, self.surv.ii(k).y)) for k in ("Brem", "Ann", "Bhabha")}

    def npz_entries(self, mV_key: float) -> dict:
        """The (mass, target) entries of a ``dark_tables.npz`` bundle."""
        pre = f"m{mV_key}/{self.target}"
        out = {f"{pre}/mV": np.array(self.mV), f"{pre}/E_res": np.array(self.E_res),
               f"{pre}/E_compth": np.array(self.E_compth),
               f"{pre}/xsec/DarkBrem": self.DBS, f"{pre}/xsec/DarkMuonBrem": self.DMBS,
               f"{pre}/xsec/DarkAnn_bound": self.DAnnS_bound, f"{pre}/xsec/DarkComp_bound": self.DCS_bound,
               f"{pre}/min_dark": self.min_dark(True)}
        for name in ("brem_elec", "brem_positron", "ann", "muon_brem"):
            out[f"{pre}/weights/{name}"] = self.weights(name, True)
            Ei, bins, cnt = _pad_bins(self.drate(name, True))
            out[f"{pre}/drate/{name}/Ei"], out[f"{pre}/drate/{name}/bins"], out[f"{pre}/drate/{name}/nbins"] = \
                Ei, bins, cnt
        for k, v in self.interaction_integrals().items():
            out[f"{self.target}/ii/{k}"] = v
        if self.DAnnS_free is None:
            return out
        f = f"{pre}/free"
        out[f"{f}/xsec/DarkAnn"], out[f"{f}/xsec/DarkComp"] = self.DAnnS_free, self.DCS_free
        out[f"{f}/weights/ann"] = self.weights("ann", False)
        Ei, bins, cnt = _pad_bins(self.drate("ann", False))
        out[f"{f}/drate/ann/Ei"], out[f"{f}/drate/ann/bins"], out[f"{f}/drate/ann/nbins"] = Ei, bins, cnt
        out[f"{f}/min_dark"] = self.min_dark(False)
        return out


# ------------------------------------------------------- PETITE's pickles
def read_dark_pickles(dict_dir: str) -> dict:
    """dark_maps.pkl (VEGAS maps through the stand-in AdaptiveMap) and
    dark_xsec.pkl, plus dark_weights.pkl and dark_drate.pkl where present."""
    out = {}
    with open(os.path.join(dict_dir, "dark_maps.pkl"), "rb") as f:
        out["maps"] = T._MapsUnpickler(f).load()
    with open(os.path.join(dict_dir, "dark_xsec.pkl"), "rb") as f:
        out["xsec"] = pickle.load(f)
    for name in ("weights", "drate"):
        p = os.path.join(dict_dir, f"dark_{name}.pkl")
        out[name] = {}
        if os.path.exists(p):
            with open(p, "rb") as f:
                out[name] = pickle.load(f)
    return out


def _mass_entry(d: dict, mV: float):
    for k in d:
        if abs(float(k) - mV) < 1e-12:
            return d[k]
    return None


def maps_entries(maps: dict, targets) -> dict:
    """The map entries of a ``dark_tables.npz`` bundle (``m<mV>/<Process>/
    energy, neval, max_F, grid, nnodes``) from dark_maps.pkl's content:
    mass -> process -> [[E, {neval, max_F: {target: value}, adaptive_map}]]."""
    out = {"masses": np.array(sorted(float(k) for k in maps)), "targets": np.array(list(targets))}
    for key in maps:
        mV = float(key)
        for p in DARK_PROCESSES:
            if p not in maps[key]:
                continue                     # a process without maps at this mass cannot be made active
            rows = maps[key][p]
            d = len(rows[0][1]["adaptive_map"].grid)
            nmax = max(len(g) for r in rows for g in r[1]["adaptive_map"].grid)
            grid = np.zeros((len(rows), d, nmax))
            nn = np.zeros((len(rows), d), np.int32)
            for i, (E, info) in enumerate(rows):
                for k, g in enumerate(info["adaptive_map"].grid):
                    grid[i, k, :len(g)] = g
                    nn[i, k] = len(g)
            pre = f"m{mV}/{p}"
            out[f"{pre}/energy"] = np.array([float(r[0]) for r in rows])
            out[f"{pre}/neval"] = np.array([int(r[1]["neval"]) for r in rows])
            out[f"{pre}/max_F"] = np.array([[float(r[1]["max_F"].get(t, np.nan)) for t in targets] for r in rows])
            out[f"{pre}/grid"] = grid
            out[f"{pre}/nnodes"] = nn
    return out


class PickleTables:
    """A read-only mapping with the keys of a ``dark_tables.npz`` bundle,
    built from a PETITE dict_dir's dark pickles: the maps up front, and each
    (mass, target)'s tables on first use (``DarkTableBuilder``)."""

    def __init__(self, dict_dir: str, sm_for_target, Zeff: float = 29.508):
        pk = read_dark_pickles(dict_dir)
        self._pk = pk
        self._sm_for_target = sm_for_target
        self._Zeff = Zeff
        self.mV_actual = None               # the thresholds' mass if not the map mass
        targets = sorted({t for m in pk["xsec"].values() for p in m.values() for t in p})
        mapped = [k for k in pk["maps"] if _mass_entry(pk["xsec"], float(k)) is not None]
        self._z = maps_entries({k: pk["maps"][k] for k in mapped}, targets)
        self._built = set()

    @property
    def files(self):
        return list(self._z.keys())

    def _build(self, mV_key: float, target: str):
        if (mV_key, target) in self._built:
            return
        self._built.add((mV_key, target))
        pk = self._pk
        xs = _mass_entry(pk["xsec"], mV_key)
        cw = (_mass_entry(pk["weights"], mV_key) or {}).get(target)
        cd = (_mass_entry(pk["drate"], mV_key) or {}).get(target)
        mV = self.mV_actual if self.mV_actual is not None else mV_key
        b = DarkTableBuilder(self._sm_for_target(target), xs, target, mV, self._Zeff, cw, cd)
        self._z.update(b.npz_entries(mV_key))

    def __contains__(self, key):
        return key in self._z

    def __getitem__(self, key):
        if key not in self._z:
            parts = key.split("/")
            if key.startswith("m") and len(parts) > 2:
                self._build(float(parts[0][1:]), parts[1])
            elif len(parts) > 1 and parts[1] == "ii":
                for m in self._z["masses"]:
                    self._build(float(m), parts[0])
                    break
        return self._z[key]


def bundle_mass(maps_npz: str, bundle: str, sm_npz: str, out: str | None = None) -> float:
    """Adds one dark mass to a ``dark_tables.npz`` bundle, as PETITE's own
    pipeline adds one once find_maxes has written its maps and cross
    sections: the maps, max_F and find_maxes cross sections of
    ``petite_gb300.train.build_dark_maps`` (``maps_npz``), and for every
    target of the bundle the tables PETITE's constructor derives from them
    (``DarkTableBuilder`` on the SM tables ``sm_npz``).  Returns the mass."""
    z = dict(np.load(bundle, allow_pickle=False))
    m = np.load(maps_npz, allow_pickle=False)
    mt = [str(t) for t in m["targets"]]
    bt = [str(t) for t in z["targets"]]
    masses = sorted({float(k.split("/")[0][1:]) for k in m.files if k.startswith("m")})
    if len(masses) != 1:
        raise ValueError(f"{maps_npz} holds masses {masses}; one is expected")
    mV = masses[0]
    cols = [mt.index(t) for t in bt]
    xsec = {}
    for p in DARK_PROCESSES:
        pre = f"m{mV}/{p}"
        if f"{pre}/energy" not in m.files:
            continue
        E = m[f"{pre}/energy"]
        xsec[p] = {t: np.column_stack((E, m[f"{pre}/xsec"][:, c])) for t, c in zip(bt, cols)}
        z[f"{pre}/energy"], z[f"{pre}/neval"] = E, m[f"{pre}/neval"]
        z[f"{pre}/max_F"] = m[f"{pre}/max_F"][:, cols]
        z[f"{pre}/grid"], z[f"{pre}/nnodes"] = m[f"{pre}/grid"], m[f"{pre}/nnodes"]
    raw = T.load_npz(sm_npz)
    for t in bt:
        z.update(DarkTableBuilder(T.SMTables(raw, t), xsec, t, mV).npz_entries(mV))
    z["masses"] = np.array(sorted({float(v) for v in z["masses"]} | {mV}))
    np.savez_compressed(out or bundle, **z)
    return mV
