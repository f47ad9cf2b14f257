"""CPU restatement of PETITE's per-interaction physics (scalar, float64).

TEST INFRASTRUCTURE: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline of ``bench.py`` use this package; the product never imports it.

Every function follows one reference function; the citation gives the file and
line range inside PETITE (``src/PETITE/...``).  Operation order follows the
reference's expressions so float64 results agree to a few ulp.
"""
from __future__ import annotations

import math

# ---------------------------------------------------------------- constants
# physical_constants.py:11-38
GeV = 1.0
MeV = 1e-3
keV = 1e-6
alpha_em = 1 / 137.035999
m_electron = 510.998950 * keV
m_muon = 105.6583755 * MeV
m_proton = 938.272088 * MeV
m_proton_grams = 1.67262192369e-24
hbarc = 0.1973269804e-13 * GeV
GeVsqcm2 = hbarc ** 2
cmtom = 0.01
PI = math.pi

# physical_constants.py:49-58 (dEdx = 2*rho MeV/cm)
TARGETS = {
    "graphite": dict(Z_T=6, A_T=12, mT=11.178, rho=2.210),
    "lead": dict(Z_T=82, A_T=207, mT=207.2, rho=11.35),
    "iron": dict(Z_T=26, A_T=56, mT=55.845, rho=8.00),
    "hydrogen": dict(Z_T=1, A_T=1, mT=1.0, rho=1.0),
    "aluminum": dict(Z_T=13, A_T=27, mT=26.9815385, rho=2.699),
    "tungsten": dict(Z_T=74, A_T=183.84, mT=183.84, rho=19.3),
    "molybdenum": dict(Z_T=42, A_T=95.95, mT=95.95, rho=10.2),
}
for _t in TARGETS.values():
    _t["dEdx"] = 2.0 * _t["rho"]

# particle.py:4-13 (leptons and photon only: the shower path)
MASS = {11: m_electron, -11: m_electron, 22: 0.0, 13: m_muon, -13: m_muon,
        12: 0.0, -12: 0.0, 14: 0.0, -14: 0.0}

# shower.py:36 process codes; shower.py:47-56 dimensions; shower.py:87-96 PIDs
PROCESS_CODE = {"Brem": 0, "Ann": 1, "PairProd": 2, "Comp": 3, "Moller": 4,
                "Bhabha": 5, "MuonE": 6, "MuonBrem": 7}
PROCESS_NAME = {v: k for k, v in PROCESS_CODE.items()}
DIM = {"PairProd": 4, "Comp": 1, "Brem": 4, "MuonBrem": 4, "Ann": 1,
       "Moller": 1, "Bhabha": 1, "MuonE": 1}
PROCESS_PIDS = {"PairProd": (-11, 11), "Brem": (0, 22), "MuonBrem": (0, 22),
                "Comp": (11, 22), "Ann": (22, 22), "Moller": (0, 11),
                "Bhabha": (0, 11), "MuonE": (0, 11)}


# ------------------------------------------------------------ form factors
def aa(Z, me):
    """all_processes.py:92-94"""
    return 184.15 * (2.718) ** -0.5 * Z ** (-1.0 / 3.0) / me


def g2_elastic(Z, t):
    """all_processes.py:99-103"""
    a0 = aa(Z, m_electron)
    return Z ** 2 * a0 ** 4 * t ** 2 / (1 + a0 ** 2 * t) ** 2


# ------------------------------------------------------- differential sigma
def dsigma_brem(x, ep, Eg_min, m_lep, Z):
    """dsigma_brem_dimensionless.__call__, all_processes.py:153-206 (scalar x[4])."""
    x1, x2, x3, x4 = x
    w = Eg_min + x1 * (ep - m_lep - Eg_min)
    d = ep / (2 * m_lep) * (x2 + x3)
    dp = ep / (2 * m_lep) * (x2 - x3)
    ph = (x4 - 1 / 2) * 2 * PI
    epp = ep - w
    allowed = (Eg_min < w) and (w < ep - m_lep) and (m_lep < epp) and (epp < ep) \
        and (d > 0.0) and (dp > 0.0)
    if not allowed:
        return 0.0
    cph = math.cos(ph)
    qsq = m_lep ** 2 * ((d ** 2 + dp ** 2 - 2 * d * dp * cph)
                        + m_lep ** 2 * ((1 + d ** 2) / (2 * ep) - (1 + dp ** 2) / (2 * epp)) ** 2)
    PF = 8.0 / PI * alpha_em * (alpha_em / m_lep) ** 2 * (epp * m_lep ** 4) / (w * ep * qsq ** 2) * d * dp
    jac = PI * ep ** 2 * (ep - m_lep - Eg_min) / m_lep ** 2
    FF = g2_elastic(Z, qsq)
    T1 = d ** 2 / (1 + d ** 2) ** 2
    T2 = dp ** 2 / (1 + dp ** 2) ** 2
    T3 = w ** 2 / (2 * ep * epp) * (d ** 2 + dp ** 2) / ((1 + d ** 2) * (1 + dp ** 2))
    T4 = -(epp / ep + ep / epp) * (d * dp * cph) / ((1 + d ** 2) * (1 + dp ** 2))
    return PF * (T1 + T2 + T3 + T4) * jac * FF


def dsigma_pairprod(x, w, Z):
    """dsigma_pairprod_dimensionless.__call__, all_processes.py:546-622."""
    x1, x2, x3, x4 = x
    me = m_electron
    epp = me + x1 * (w - 2 * me)
    dp = w / (2 * me) * (x2 + x3)
    dm = w / (2 * me) * (x2 - x3)
    ph = x4 * 2 * PI
    epm = w - epp
    allowed = (me < epm) and (epm < w) and (me < epp) and (epp < w) and (dm > 0.0) and (dp > 0.0)
    if not allowed:
        return 0.0
    cph = math.cos(ph)
    q = (dp ** 2 + dm ** 2 + 2.0 * dp * dm * cph) + me ** 2 * ((1.0 + dp ** 2) / (2.0 * epp) + (1.0 + dm ** 2) / (2.0 * epm)) ** 2
    PF = 8.0 / PI * alpha_em * (alpha_em / me) ** 2 * epp * epm / (w ** 3 * q ** 2) * dp * dm
    jac = PI * w ** 2 * (w - 2 * me) / me ** 2
    FF = g2_elastic(Z, me ** 2 * q)
    T1 = -1.0 * dp ** 2 / (1.0 + dp ** 2) ** 2
    T2 = -1.0 * dm ** 2 / (1.0 + dm ** 2) ** 2
    T3 = w ** 2 / (2.0 * epp * epm) * (dp ** 2 + dm ** 2) / ((1.0 + dp ** 2) * (1.0 + dm ** 2))
    T4 = (epp / epm + epm / epp) * (dp * dm * cph) / ((1.0 + dp ** 2) * (1.0 + dm ** 2))
    return PF * (T1 + T2 + T3 + T4) * jac * FF


def dsigma_compton(ct, Eg, mV=0.0):
    """dsigma_compton_dCT.__call__, all_processes.py:639-742 (SM mV=0 and dark mV>0)."""
    me = m_electron
    s = me ** 2 + 2 * Eg * me
    if s < (me + mV) ** 2:
        return 0.0
    root = math.sqrt(me ** 4 + (mV ** 2 - s) ** 2 - 2 * me ** 2 * (mV ** 2 + s))
    jac = (s - me ** 2) / (2 * s) * math.sqrt((s - mV ** 2) ** 2 - 2 * me ** 2 * (s + mV ** 2) + me ** 4)
    t = -1 / 2 * (me ** 4 + s * (-(mV ** 2) + s + ct * root) - me ** 2 * (mV ** 2 + 2 * s + ct * root)) / s
    PF = 2.0 * PI * alpha_em ** 2 / (s - me ** 2) ** 2
    if mV == 0.0:
        T1 = (6.0 * me ** 2 * s + 3.0 * me ** 4 - s ** 2) / ((me ** 2 - s) * (-(me ** 2) + s + t))
        T2 = 4 * me ** 4 / (s + t - me ** 2) ** 2
        T3 = (t * (s - me ** 2) + (s + me ** 2) ** 2) / (s - me ** 2) ** 2
    else:
        T1 = (2.0 * me ** 2 * (mV ** 2 - 3 * s) - 3 * me ** 4 - 2 * mV ** 2 * s + 2 * mV ** 4 + s ** 2) \
            / ((me ** 2 - s) * (me ** 2 + mV ** 2 - s - t))
        T2 = (2 * me ** 2 * (2 * me ** 2 + mV ** 2)) / (me ** 2 + mV ** 2 - s - t) ** 2
        T3 = ((me ** 2 + s) * (me ** 2 + mV ** 2 + s) + t * (s - me ** 2)) / (me ** 2 - s) ** 2
    return PF * jac * (T1 + T2 + T3)


def dsigma_annihilation(ct, Ee, Eg_min, mV=0.0):
    """dsigma_annihilation_dCT.__call__, all_processes.py:475-529."""
    me = m_electron
    s = 2.0 * me * (Ee + me)
    ctMax = math.sqrt((Ee + me) / (Ee - me)) * (2 * me * (Ee - 2 * Eg_min + me) - mV ** 2) / (2 * me * (Ee + me) - mV ** 2)
    if s < mV ** 2:
        return 0.0
    b = math.sqrt(1.0 - 4.0 * me ** 2 / s)
    if ct > ctMax:
        return 0.0
    return 4.0 * PI * alpha_em ** 2 / (s * (1 - b ** 2 * ct ** 2)) * ((s - mV ** 2) / (2 * s) * (1 + ct ** 2) + 2.0 * mV ** 2 / (s - mV ** 2))


def dsigma_moller(ct, Ee, Ee_min):
    """dsigma_moller_dCT.__call__, all_processes.py:799-840."""
    me = m_electron
    lim = 2.0 * Ee_min / (Ee - me)
    if not ((ct > -1 + lim) and (ct < 1.0 - lim)):
        return 0.0
    s = me ** 2 + 2 * Ee * me
    return 16 * PI ** 2 * alpha_em ** 2 * (s ** 2 * (3 + ct ** 2) ** 2 - 8 * me ** 2 * s * (7 + ct ** 4)
                                           + 16 * me ** 4 * (6 - 3 * ct ** 2 + ct ** 4)) \
        / (8 * PI * s * (s - 4 * me ** 2) ** 2 * (1 - ct) ** 2 * (1 + ct) ** 2)


def dsigma_bhabha(ct, Ee, Ee_min):
    """dsigma_bhabha_dCT.__call__, all_processes.py:960-1007."""
    me = m_electron
    lim = 2.0 * Ee_min / (Ee - me)
    if not ((ct > -1 + lim) and (ct < 1.0 - lim)):
        return 0.0
    s = me ** 2 + 2 * Ee * me
    num = (256 * (-1 + ct) ** 2 * ct ** 2 * me ** 8
           - 128 * (-1 + ct) * (1 + ct * (1 + ct) * (-3 + 2 * ct)) * me ** 6 * s
           + 16 * (7 + ct * (2 + ct * (-5 + 6 * (-1 + ct) * ct))) * me ** 4 * s ** 2
           - 8 * (7 + ct * (-3 + ct * (3 + ct * (-1 + 2 * ct)))) * me ** 2 * s ** 3
           + (3 + ct ** 2) ** 2 * s ** 4)
    return alpha_em ** 2 * PI * num / (2 * (-1 + ct) ** 2 * s ** 3 * (-4 * me ** 2 + s) ** 2)


def dsigma_muone(ct, Emu, Ee_min):
    """dsigma_muonelectron_dCT.__call__, all_processes.py:855-886."""
    me, mm = m_electron, m_muon
    s = me ** 2 + mm ** 2 + 2 * me * Emu
    t_limit = 2.0 * me * (me - Ee_min)
    t = -2.0 * (1 - ct) * ((s + me ** 2 - mm ** 2) ** 2 / (4.0 * s) - me ** 2)
    if not (t < t_limit):
        return 0.0
    return 16 * PI ** 2 * alpha_em ** 2 * (s ** 2 + 2 * (me ** 2 + mm ** 2) * (2 * t + mm ** 2 - 3 * me ** 2)
                                           + (s + t - 4 * me ** 2) ** 2) / (16 * PI * s * t ** 2)


def dsigma(process, x, E, Z, Eg_min, Ee_min, m_lep):
    """Dispatch used by draw_sample (shower.py:435-445)."""
    if process == "Brem" or process == "MuonBrem":
        return dsigma_brem(x, E, Eg_min, m_lep, Z)
    if process == "PairProd":
        return dsigma_pairprod(x, E, Z)
    if process == "Comp":
        return dsigma_compton(x[0], E, 0.0)
    if process == "Ann":
        return dsigma_annihilation(x[0], E, Eg_min, 0.0)
    if process == "Moller":
        return dsigma_moller(x[0], E, Ee_min)
    if process == "Bhabha":
        return dsigma_bhabha(x[0], E, Ee_min)
    if process == "MuonE":
        return dsigma_muone(x[0], E, Ee_min)
    raise ValueError(process)


# -------------------------------------------------------- total cross sections
def _heaviside(x, h0):
    return 0.0 if x < 0 else (h0 if x == 0 else 1.0)


def sigma_moller(Ee, Ee_min):
    """all_processes.py:907-944 (scalar)."""
    me = m_electron
    Te = Ee_min - me
    thr = 3 * me + 4 * Te
    PF = 2 * PI * alpha_em ** 2 / (me * (Ee ** 2 - me ** 2))
    T1 = Ee - 3 * me - 4 * Te + 2 * Ee ** 2 * (-2 / (Ee - 3 * me - 2 * Te) + 1 / Te
                                               + 1 / (-Ee + me + Te) + 2 / (Ee + me + 2 * Te))
    arg = ((-Ee + me + Te) * (-Ee + 3 * me + 2 * Te) / (Te * (Ee + me + 2 * Te))) * _heaviside(Ee - thr, 1) \
        + _heaviside(thr - Ee, 1)
    T2 = 2 * me * (me - 2 * Ee) / (Ee - me) * math.log(arg) if arg > 0 else float("nan")
    return PF * (T1 + T2) * _heaviside(Ee - thr, 1)


def sigma_bhabha(Ee, Ee_min):
    """all_processes.py:1010-1051 (scalar)."""
    me = m_electron
    Te = Ee_min - me
    thr = 3 * me + 4 * Te
    PF = PI * alpha_em ** 2 / (12 * (Ee - me) * me * (Ee + me) ** 3 * (Ee - 3 * me - 2 * Te) * Te)
    T1 = (Ee - 3 * me - 4 * Te) * (24 * Ee ** 2 * (Ee + me) ** 2
                                   + (Ee - 3 * me) * (31 * Ee ** 2 + 84 * Ee * me + 57 * me ** 2) * Te
                                   - 4 * (16 * Ee ** 2 + 39 * Ee * me + 33 * me ** 2) * Te ** 2
                                   + 8 * (Ee - 3 * me) * Te ** 3 - 8 * Te ** 4)
    arg = (2 * Te / (Ee - 3 * me - 2 * Te)) * _heaviside(Ee - thr, 1) + _heaviside(thr - Ee, 1)
    T2 = 24 * (Ee + me) * (2 * Ee ** 2 + 4 * Ee * me + me ** 2) * (Ee - 3 * me - 2 * Te) * Te * math.log(arg)
    return PF * (T1 + T2) * _heaviside(Ee - thr, 1)


def sigma_muone(Emu, Ee_min):
    """all_processes.py:888-905 (scalar)."""
    me, mm = m_electron, m_muon
    thr = 1.0 / (2.0 * me) * (me * (Ee_min - me) + math.sqrt(me * (Ee_min + me) * (me * (Ee_min - me) + 2 * mm ** 2)))
    s = me ** 2 + mm ** 2 + 2 * me * Emu
    t_max = 2.0 * me * (me - Ee_min)
    t_min = -4.0 * ((s + me ** 2 - mm ** 2) ** 2 / (4 * s) - me ** 2)
    PF = 16 * PI ** 2 * alpha_em ** 2 / (8.0 * PI * ((s - mm ** 2) ** 2 + me ** 4 - 2 * (s + mm ** 2) * me ** 2))
    T1 = -2.0 * (s ** 2 + mm ** 4 + 5 * me ** 4 - 2 * me ** 2 * (2 * s + mm ** 2)) * (1.0 / t_max - 1.0 / t_min)
    T2 = 2.0 * (s + 2 * mm ** 2 - 2 * me ** 2) * math.log(t_max / t_min)
    T3 = t_max - t_min
    return PF * (T1 + T2 + T3) * _heaviside(Emu - thr, 1)


# ------------------------------------------------------------- kinematics
# Each takes the parent's final energy (and mass where the reference reads it
# from the Particle) plus the sampled variables and the azimuth uniform
# already scaled to [0, 2pi) by the caller, and returns two 4-vectors in the
# frame where the parent moves along +z.
def e_to_egamma(ep, m_lepton, x, al):
    """kinematics.py:10-41 (Egamma_min = 0.001 at kinematics.py:9)."""
    Egamma_min = 0.001
    x1, x2, x3, x4 = x
    w = Egamma_min + x1 * (ep - m_lepton - Egamma_min)
    ct = math.cos((x2 + x3) / 2)
    ctp = math.cos((x2 - x3) * ep / (2 * (ep - w)))
    ph = (x4 - 1 / 2) * 2.0 * PI
    epp = ep - w
    pp = math.sqrt(epp ** 2 - m_lepton ** 2)
    cal, sal = math.cos(al), math.sin(al)
    st, stp = math.sqrt(1.0 - ct ** 2), math.sqrt(1.0 - ctp ** 2)
    sp, cp = math.sin(ph), math.cos(ph)
    g = (w, w * cal * st, w * sal * st, w * ct)
    e = (epp, pp * (sal * sp * stp + cal * (ctp * st - cp * ct * stp)),
         pp * (ctp * sal * st - (cp * ct * sal + cal * sp) * stp), pp * (ct * ctp + cp * st * stp))
    return e, g


def gamma_to_epem(w, x, al):
    """kinematics.py:70-102 -> (positron, electron)."""
    me = m_electron
    x1, x2, x3, x4 = x
    epp = me + x1 * (w - 2 * me)
    ctp = math.cos(w * (x2 + x3) / (2 * epp))
    ctm = math.cos(w * (x2 - x3) / (2 * (w - epp)))
    ph = x4 * 2 * PI
    epm = w - epp
    pm, pp = math.sqrt(epm ** 2 - me ** 2), math.sqrt(epp ** 2 - me ** 2)
    cal, sal = math.cos(al), math.sin(al)
    stp, stm = math.sqrt(1.0 - ctp ** 2), math.sqrt(1.0 - ctm ** 2)
    spal, cpal = math.sin(ph + al), math.cos(ph + al)
    return (epp, pp * stp * cal, pp * stp * sal, pp * ctp), (epm, pm * stm * cpal, pm * stm * spal, pm * ctm)


def compton(Eg, ct, ph, mV=0.0):
    """kinematics.py:104-132 -> (electron, photon/V)."""
    me = m_electron
    s = me ** 2 + 2 * Eg * me
    rs = math.sqrt(s)
    Ee0 = (s + me ** 2) / (2.0 * rs)
    Ee = (s - mV ** 2 + me ** 2) / (2 * rs)
    EV = (s + mV ** 2 - me ** 2) / (2 * rs)
    pF = math.sqrt(Ee ** 2 - me ** 2)
    g0 = Ee0 / me
    b0 = 1.0 / g0 * math.sqrt(g0 ** 2 - 1.0)
    st = math.sqrt(1 - ct ** 2)
    sph, cph = math.sin(ph), math.cos(ph)
    pe = (g0 * Ee + b0 * g0 * pF * ct, -pF * st * sph, -pF * st * cph, b0 * g0 * Ee + g0 * pF * ct)
    pv = (g0 * EV - b0 * g0 * pF * ct, pF * st * sph, pF * st * cph, b0 * g0 * EV - g0 * pF * ct)
    return pe, pv


def ee_to_ee(Einc, ct, ph):
    """kinematics.py:213-237 -> (scattered lepton, new electron)."""
    me = m_electron
    s = 2 * me ** 2 + 2 * Einc * me
    Ee0 = math.sqrt(s) / 2.0
    pF = math.sqrt(Ee0 ** 2 - me ** 2)
    g0 = Ee0 / me
    b0 = 1.0 / g0 * math.sqrt(g0 ** 2 - 1.0)
    st = math.sqrt(1 - ct ** 2)
    sph, cph = math.sin(ph), math.cos(ph)
    a = (g0 * Ee0 + b0 * g0 * pF * ct, -pF * st * sph, -pF * st * cph, b0 * g0 * Ee0 + g0 * pF * ct)
    b = (g0 * Ee0 - b0 * g0 * pF * ct, pF * st * sph, pF * st * cph, b0 * g0 * Ee0 - g0 * pF * ct)
    return a, b


def mue_to_mue(Einc, ct, ph):
    """kinematics.py:239-265 -> (muon, electron)."""
    me, mm = m_electron, m_muon
    s = me ** 2 + mm ** 2 + 2 * Einc * me
    rs = math.sqrt(s)
    Ee0 = (s + me ** 2 - mm ** 2) / (2.0 * rs)
    Em0 = (s + mm ** 2 - me ** 2) / (2.0 * rs)
    pe = math.sqrt(Ee0 ** 2 - me ** 2)
    pm = math.sqrt(Em0 ** 2 - mm ** 2)
    g0 = Ee0 / me
    b0 = 1.0 / g0 * math.sqrt(g0 ** 2 - 1.0)
    st = math.sqrt(1 - ct ** 2)
    sph, cph = math.sin(ph), math.cos(ph)
    mu = (g0 * Em0 + b0 * g0 * pm * ct, pm * st * sph, pm * st * cph, b0 * g0 * Em0 + g0 * pm * ct)
    el = (g0 * Ee0 - b0 * g0 * pe * ct, -pe * st * sph, -pe * st * cph, b0 * g0 * Ee0 - g0 * pe * ct)
    return mu, el


def annihilation(Ee, ct, ph, mV=0.0):
    """kinematics.py:301-334 -> (photon, photon/V)."""
    me = m_electron
    s = 2 * me * (Ee + me)
    rs = math.sqrt(s)
    EeCM = rs / 2.0
    Eg = (s - mV ** 2) / (2 * rs)
    EV = (s + mV ** 2) / (2 * rs)
    pF = Eg
    g0 = EeCM / me
    b0 = 1.0 / g0 * math.sqrt(g0 ** 2 - 1.0)
    st = math.sqrt(1 - ct ** 2)
    sph, cph = math.sin(ph), math.cos(ph)
    a = (g0 * Eg - b0 * g0 * pF * ct, -pF * st * sph, -pF * st * cph, b0 * g0 * Eg - g0 * pF * ct)
    b = (g0 * EV + b0 * g0 * pF * ct, pF * st * sph, pF * st * cph, b0 * g0 * EV + g0 * pF * ct)
    return a, b


# ------------------------------------------------------- exact arithmetic
def fma(a, b, c):
    """Correctly rounded a*b + c (Python 3.12 has no math.fma): exact integer
    arithmetic on the binary significands, one final rounding by int->float."""
    if a == 0.0 or b == 0.0:
        return a * b + c
    ma, ea = math.frexp(a)
    mb, eb = math.frexp(b)
    ia, ib = int(ma * 9007199254740992.0), int(mb * 9007199254740992.0)   # 2**53
    ep = ea + eb - 106
    if c == 0.0:
        return math.ldexp(float(ia * ib), ep)
    mc, ec = math.frexp(c)
    ic = int(mc * 9007199254740992.0)
    ec -= 53
    e = min(ep, ec)
    n = (ia * ib << (ep - e)) + (ic << (ec - e))
    # keep the integer small enough for float(): drop bits below the final ulp
    # only through float()'s own correct rounding (n fits easily here).
    return math.ldexp(float(n), e)


def norm3(x, y, z):
    """numpy.linalg.norm of a 3-vector as the reference computes it
    (sqrt of a sequential fused dot product: fma(z, z, fma(y, y, x*x)))."""
    return math.sqrt(fma(z, z, fma(y, y, x * x)))


# ------------------------------------------------ multiple Coulomb scattering
def chic2_alt(t, beta, A, Z, z, m_lepton):
    """moliere.py:196-207 (Lynch & Dahl 1991 eq. 1)."""
    p = m_lepton / MeV * beta / math.sqrt(1. - beta ** 2)
    return 0.157 * Z * (Z + 1) * (t / A) * (z / (p * beta)) ** 2.


def chia2_alt(beta, A, Z, z, m_lepton):
    """moliere.py:209-219 (Lynch & Dahl 1991 eq. 2)."""
    p = m_lepton / MeV * beta / math.sqrt(1. - beta ** 2)
    return 2.007e-5 * Z ** (2. / 3.) * (1. + 3.34 * (Z * z * alpha_em / beta) ** 2.) / p ** 2


def theta0_lynch_dahl(t, beta, A, Z, m_lepton):
    """Gaussian width of moliere.py:265-280 (F = 0.98, z = 1)."""
    F = 0.98
    chic2 = chic2_alt(t, beta, A, Z, 1., m_lepton)
    chia2 = chia2_alt(beta, A, Z, 1., m_lepton)
    omega = chic2 / chia2
    v = 0.5 * omega / (1. - F)
    return math.sqrt(chic2 * ((1. + v) * math.log(1. + v) / v - 1) / (1. + F ** 2))


def rotation_to_z(vx, vy, vz):
    """moliere.py:287-348: matrix R with R v = |v| z_hat (returned as 3x3 tuple rows).

    The reference's fourth branch repeats the first condition
    (moliere.py:331); that is kept.
    """
    if abs(vx) > 0. and abs(vy) > 0.:
        a = math.atan(abs(vy / vx))
        if vx > 0. and vy > 0.:
            a = -a
        if vx < 0. and vy > 0.:
            a = -(PI - a)
        if vx < 0. and vy < 0.:
            a = -(PI + a)
        if vx > 0. and vy < 0.:
            a = -(2. * PI - a)
        ca, sa = math.cos(a), math.sin(a)
    elif abs(vy) > 0.:
        ca, sa = 0., 1.
    else:
        ca, sa = 1., 0.
    vxp = vx * ca - vy * sa
    if abs(vz) > 0. and abs(vxp) > 0.:
        b = math.atan(abs(vxp / vz))
        if vz > 0. and vxp > 0.:
            b = -b
        if vz < 0. and vxp > 0.:
            b = -(PI - b)
        if vz < 0. and vxp < 0.:
            b = -(PI + b)
        if vz > 0. and vxp > 0.:
            b = -(2. * PI - b)
        cb, sb = math.cos(b), math.sin(b)
    elif vxp > 0.:
        cb, sb = 0., -1.
    elif vxp < 0.:
        cb, sb = 0., 1.
    else:
        cb, sb = 1., 0.
    # Rb @ Ra with Ra = [[ca,-sa,0],[sa,ca,0],[0,0,1]], Rb = [[cb,0,sb],[0,1,0],[-sb,0,cb]]
    return ((cb * ca, -cb * sa, sb),
            (sa, ca, 0.),
            (-sb * ca, sb * sa, cb))


def _scatter_to_lab(p4, pn, theta, phi):
    """The rotation of moliere.py:384-398 (and :427-445): the scattered
    direction (theta, phi) about z, taken to the lab by the transpose of
    get_rotation_matrix."""
    E, px, py, pz = p4
    cth, sth = math.cos(theta), math.sin(theta)
    cph, sph = math.cos(phi), math.sin(phi)
    # Rphi @ Rtheta @ z_hat: Rtheta z = (0,-sth,cth); Rphi (0,-sth,cth) = (sph*sth, -cph*sth, cth)
    n = (pn * (sph * sth), pn * (-cph * sth), pn * cth)
    R = rotation_to_z(px, py, pz)
    # lab = R^T n
    lx = R[0][0] * n[0] + R[1][0] * n[1] + R[2][0] * n[2]
    ly = R[0][1] * n[0] + R[1][1] * n[1] + R[2][1] * n[2]
    lz = R[0][2] * n[0] + R[1][2] * n[1] + R[2][2] * n[2]
    return (E, lx, ly, lz)


def _lynch_dahl_theta(t, beta, A, Z, m_lepton, u_sign, u_ang, u_rad):
    """generate_moliere_angle_simplified_alt, moliere.py:265-284, on its
    draws: sign (random.choice), the Gaussian pair (random.gauss twice;
    Box-Muller from an angle uniform and a radius uniform)."""
    th0 = theta0_lynch_dahl(t, beta, A, Z, m_lepton)
    sign = -1.0 if u_sign < 0.5 else 1.0
    r = math.sqrt(-2.0 * math.log(1.0 - u_rad))
    ang = 2.0 * PI * u_ang
    g1 = th0 * (r * math.cos(ang))
    g2 = th0 * (r * math.sin(ang))
    return sign * math.sqrt(g1 ** 2 + g2 ** 2)


def scattered_momentum_fast(p4, t, A, Z, rescale, m_lepton, u_sign, u_ang, u_rad, u_phi):
    """get_scattered_momentum_fast, moliere.py:350-400, with its four draws:
    sign, the Gaussian pair (angle, radius), and phi (random.uniform).
    """
    E, px, py, pz = p4
    pn = norm3(px, py, pz)
    if not pn > 0:
        return tuple(p4)
    beta = pn / E
    theta = _lynch_dahl_theta(t, beta, A, Z, m_lepton, u_sign, u_ang, u_rad) * rescale
    phi = 2. * PI * u_phi
    return _scatter_to_lab(p4, pn, theta, phi)


# ------------------------------------ Bethe-Moliere multiple scattering
# moliere.py:33-174,221-247,403-453 (fast_MCS_mode=False).  The reference's
# inverse CDF integrates the Moliere density with scipy.integrate.quad inside
# a Ridder root search; here the integral is in closed form:
#   F(x, B) = (1 - e^-x)(1 + 1/B) - x e^-x g(x) / B,  g(x) = Ei(x) - ln x,
# from f1 = -2 d/dx[x e^-x g(x)] + 2 e^-x (g' = (e^x - 1)/x), which also
# shows that f1 integrates to 0.  With h(x) = x e^-x g(x) - 1 the tail is
#   Q(x) = 1 - F(x, B) = e^-x (1 + 1/B) + h(x) / B.
EULER_GAMMA = 0.57721566490153286061


def moliere_h(x, series_below=40.0, eps=1e-17):
    """x e^-x (Ei(x) - ln x) - 1.  Below ``series_below``: the power series
    g(x) = gamma + sum_k x^k / (k k!) (all terms positive); above it the
    asymptotic series x e^-x Ei(x) ~ sum_k k! / x^k, stopped at its smallest
    term (k ~ x), whose size sqrt(2 pi x) e^-x is below 3e-15 of h there."""
    if x < series_below:
        term, s, k = 1.0, 0.0, 1
        while True:
            term *= x / k
            d = term / k
            s += d
            if d <= eps * s or k >= 400:
                break
            k += 1
        return x * math.exp(-x) * (EULER_GAMMA + s) - 1.0
    term, s, k = 1.0, 0.0, 1
    while True:
        nxt = term * (k / x)
        if nxt >= term:
            break
        term = nxt
        s += term
        if term <= eps * s:
            break
        k += 1
    return s - x * math.exp(-x) * math.log(x)


def moliere_tail(x, B):
    """1 - moliere_cdf(x, B) in closed form (moliere.py:62-81 without quad)."""
    return math.exp(-x) * (1.0 + 1.0 / B) + moliere_h(x) / B


def moliere_density(x, B):
    """moliere_f(x, B) = (f0 + f1/B)/2 (moliere.py:33-59) in terms of h:
    f1 = 2((x-1) h - 1)/x + 4 e^-x."""
    e = math.exp(-x)
    f1 = 2.0 * ((x - 1.0) * moliere_h(x) - 1.0) / x + 4.0 * e
    return e + 0.5 * f1 / B


def moliere_f1_at_zero():
    """moliere_f1(0): the reference evaluates x <= 1e-6 at x = 1e-6 (moliere.py:45-50)."""
    x = 1e-6
    g = (moliere_h(x) + 1.0) / (x * math.exp(-x))
    return 2. * math.exp(-x) * (x - 1.) * g - 2. * (1. - 2. * math.exp(-x))


def moliere_cdf_pieces(x, B, f00):
    """moliere_cdf, moliere.py:62-81: f(0,B) x below 0.01, the integral (here
    closed form) up to 100, a three-term asymptote above."""
    if x > 100:
        return 1.0 - (1.0 / B / x + 2.0 / B / x ** 2 + 6.0 / B / x ** 3)
    if x < 0.01:
        return f00 * x
    return 1.0 - moliere_tail(x, B)


def ridders_root(f, a, b, xtol=2e-12, rtol=4 * 2.220446049250313e-16, max_iter=100):
    """Ridders' method (C. Ridders, IEEE Trans. Circuits Syst. 26 (1979) 979):
    the bracket's midpoint m, then the root of the exponentially scaled line
    through the three points, x = m - sign(f(b) - f(a)) (b - a)/2 f(m) /
    sqrt(f(m)^2 - f(a) f(b)); the sub-bracket with a sign change is kept.  The
    stopping rule |b - a| < xtol + rtol x is scipy's default for
    root_scalar(method='ridder')."""
    fa, fb = f(a), f(b)
    if fa == 0:
        return a
    if fb == 0:
        return b
    x = a
    for _ in range(max_iter):
        dm = 0.5 * (b - a)
        m = a + dm
        fm = f(m)
        x = m - math.copysign(1.0, fb - fa) * dm * fm / math.sqrt(fm * fm - fa * fb)
        fx = f(x)
        if fx * fm < 0:
            a, fa, b, fb = x, fx, m, fm
        elif fx * fa < 0:
            b, fb = x, fx
        else:
            a, fa = x, fx
        if fx == 0 or abs(b - a) < xtol + rtol * x:
            break
    return x


def moliere_x(u, B, tol=1e-10, max_iter=60):
    """inverse_moliere_cdf, moliere.py:84-120.  The explicit branches are the
    reference's.  Otherwise the root of the reference's piecewise CDF
    (moliere_cdf_pieces): the integral piece is solved by Newton steps on the
    closed-form tail, kept inside a bracket (bisection when a step leaves
    it); a root below 0.01 or above 100 falls on the other pieces.  At x =
    0.01 the pieces step down by ~5e-5; for u inside that step there are two
    roots about 1 % apart, and the reference's choice is reproduced by its
    own search: the bracket expansion of moliere.py:102-115 from [0.5, 2],
    then Ridders' method."""
    if 1 - u < 1 / B / 100:
        return 1 / (1 - u) / B
    if u < 0.01:
        return u
    f00 = 0.5 * (2. * math.exp(-0.) + moliere_f1_at_zero() / B)
    if 1.0 - moliere_tail(0.01, B) < u < f00 * 0.01:
        f = lambda xx: moliere_cdf_pieces(xx, B, f00) - u
        a, b, it = 0.5, 2.0, 0
        while f(a) * f(b) > 0 and it <= 20:
            if f(b) < 0:
                b *= 2
            if f(a) > 0:
                a *= 0.5
            it += 1
        return ridders_root(f, a, b)
    q = 1.0 - u
    lo, hi = 0.0, 200.0
    x = max(math.log((1.0 + 1.0 / B) / q), 1.0 / (B * q))
    if not lo < x < hi:
        x = 0.5 * (lo + hi)
    for _ in range(max_iter):
        Q = moliere_tail(x, B)
        if Q == q:
            break
        if Q > q:
            lo = x
        else:
            hi = x
        xn = x + (Q - q) / moliere_density(x, B)
        if xn == x:                      # the step is below one ulp of x
            break
        if lo < xn < hi:                 # a Newton step: the next error is ~ its square
            done = abs(xn - x) <= tol * xn
        else:                            # bisection ends only on a closed bracket
            xn = 0.5 * (lo + hi)
            done = hi - lo <= 4.5e-16 * xn
        x = xn
        if done:
            break
    if x < 0.01:
        return u / f00
    if x > 100.0:
        # 1 - (1/B/x + 2/B/x**2 + 6/B/x**3) = u, in y = 1/x; below x = 100
        # the pieces step up past u and the reference's search ends at 100
        c = B * q
        y = c
        for _ in range(max_iter):
            yn = y - (y + 2.0 * y * y + 6.0 * y * y * y - c) / (1.0 + 4.0 * y + 18.0 * y * y)
            done = abs(yn - y) <= tol * yn
            y = yn
            if done:
                break
        return max(1.0 / y, 100.0)
    return x


def moliere_b(t, beta, A, Z, z=1.):
    """get_b, moliere.py:139-155 (Bethe 1953 eq. 22)."""
    alpha = z * Z * alpha_em / beta
    expb = 6700. * t * (Z + 1.) * Z ** (1. / 3.) * z ** 2. / (beta * beta * A * (1. + 3.34 * alpha ** 2))
    return math.log(expb)


def moliere_B(b):
    """get_capital_B, moliere.py:157-174: B = b + ln B by fixed-point steps
    from b + ln b, stopped at |B - (b + ln B)| <= 1e-3."""
    B = b + math.log(b)
    B = b + math.log(B)
    while abs(B - (b + math.log(B))) > 1e-3:
        B = b + math.log(B)
    return B


n_avogadro = 6.0221409e+23                      # physical_constants.py:24


def chic2_bethe(t, beta, A, Z, z=1.):
    """get_chic_squared, moliere.py:180-192 (Bethe 1953 eq. 10); its momentum
    uses the electron mass for every lepton."""
    me_in_inv_cm = m_electron / hbarc
    p = me_in_inv_cm * beta / math.sqrt(1. - beta * beta)
    return 4. * PI * n_avogadro * alpha_em ** 2 * t * Z * (Z + 1.) * z ** 2 / (A * (p * p) * (beta * beta))


def scattered_momentum_bethe(p4, t, A, Z, rescale, draw):
    """get_scattered_momentum_Bethe, moliere.py:403-453, with
    generate_moliere_angle (moliere.py:221-247).  ``draw()`` returns the next
    uniform.  b < 2: the Lynch-Dahl angle with its default (electron) mass,
    four draws with phi.  Otherwise three: the inverse-CDF uniform
    (random.random in generate_moliere_x), the sign (random.choice) and phi.
    The reference passes m_lepton on to get_chic_squared (moliere.py:244),
    which does not take it (a TypeError); the momentum there is the electron's
    as that function defines it."""
    E, px, py, pz = p4
    pn = norm3(px, py, pz)
    if not pn > 0:
        return tuple(p4)
    beta = pn / E
    b = moliere_b(t, beta, A, Z)
    if b < 2:
        u_sign, u_ang, u_rad = draw(), draw(), draw()
        theta = _lynch_dahl_theta(t, beta, A, Z, m_electron, u_sign, u_ang, u_rad)
    else:
        B = moliere_B(b)
        x = moliere_x(draw(), B)
        chic2 = chic2_bethe(t, beta, A, Z)
        sign = -1 if draw() < 0.5 else 1
        theta = sign * math.sqrt(x * chic2 * B)
    theta = theta * rescale
    phi = 2. * PI * draw()
    return _scatter_to_lab(p4, pn, theta, phi)


def rotation_matrix_from(pf):
    """Particle.rotation_matrix, particle.py:176-185 (z_hat -> direction of pf)."""
    E0, px0, py0, pz0 = pf
    ThZ = math.acos(pz0 / math.sqrt(px0 ** 2 + py0 ** 2 + pz0 ** 2))
    PhiZ = math.atan2(py0, px0)
    cT, sT, cP, sP = math.cos(ThZ), math.sin(ThZ), math.cos(PhiZ), math.sin(PhiZ)
    return ((cT * cP, -sP, sT * cP), (cT * sP, cP, sT * sP), (-sT, 0.0, cT))


def lose_energy(pf, mass, value):
    """Particle.lose_energy, particle.py:143-153."""
    E0, px0, py0, pz0 = pf
    p30 = norm3(px0, py0, pz0)
    Eu = E0 - value
    if Eu <= mass:
        Eu = mass
    p3f = math.sqrt(Eu ** 2 - mass ** 2)
    if p3f > 0.0:
        return (Eu, px0 / p30 * p3f, py0 / p30 * p3f, pz0 / p30 * p3f)
    if p3f == 0.0:
        return (mass, 0.0, 0.0, 0.0)
    return tuple(pf)
