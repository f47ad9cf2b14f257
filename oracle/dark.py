"""CPU restatement of PETITE's dark-vector production on an SM shower (oracle).

TEST INFRASTRUCTURE: used only by ``tests/`` and the CPU baseline of
``bench.py``; the product never imports it.

Follows ``src/PETITE/``:

* dark bremsstrahlung dsigma     all_processes.py:208-372 (``Log`` variables:
                                 x, log10(1-cos theta), log10 t~), with the
                                 form factor of all_processes.py:112-133
* radiative return dsigma/du     all_processes.py:400-466, radiative_return.py:26-80
* dark Compton dsigma/dcos       all_processes.py:624-742 (mV > 0 branch)
* kinematics                     kinematics.py:43-68 (l -> l V), 134-183 (bound
                                 electron Compton), 267-299 (radiative return),
                                 radiative_return.py:18-24 (boost)
* draw_dark_sample               dark_shower.py:649-704
* draw_pe_sample                 dark_shower.py:706-719
* GetBSMWeights                  dark_shower.py:595-647
* produce_bsm_particle           dark_shower.py:721-804

Expressions keep the reference's operation order so float64 results agree to
a few ulp.  Random numbers come from :mod:`oracle.philox` streams: the stream
of an SM particle ``k`` and dark process ``p`` is ``dark_key(pkey_k, p)``.
"""
from __future__ import annotations

import math
from bisect import bisect_right

import numpy as np

from . import physics as P
from .philox import Stream, mix64
from .shower import interp, map_point

class Dual:
    """Value and derivative with respect to one input (forward mode), for the
    float64 reference gradient of the dark yield.  Comparisons use the value."""
    __slots__ = ("v", "d")

    def __init__(self, v, d=0.0):
        self.v, self.d = float(v), float(d)

    @staticmethod
    def _c(x):
        return x if isinstance(x, Dual) else Dual(x)

    def __add__(a, b):
        b = Dual._c(b)
        return Dual(a.v + b.v, a.d + b.d)
    __radd__ = __add__

    def __sub__(a, b):
        b = Dual._c(b)
        return Dual(a.v - b.v, a.d - b.d)

    def __rsub__(a, b):
        return Dual._c(b) - a

    def __mul__(a, b):
        b = Dual._c(b)
        return Dual(a.v * b.v, a.d * b.v + a.v * b.d)
    __rmul__ = __mul__

    def __truediv__(a, b):
        b = Dual._c(b)
        q = a.v / b.v
        return Dual(q, (a.d - q * b.d) / b.v)

    def __rtruediv__(a, b):
        return Dual._c(b) / a

    def __neg__(a):
        return Dual(-a.v, -a.d)

    def __abs__(a):
        return -a if a.v < 0 else a

    def __pow__(a, e):
        p = a.v ** e
        return Dual(p, 0.0 if (a.d == 0.0 or a.v == 0.0) else e * a.v ** (e - 1) * a.d)

    def __rpow__(a, base):               # base ** a for a float base
        p = base ** a.v
        return Dual(p, p * math.log(base) * a.d)

    def __lt__(a, b): return a.v < _val(b)
    def __le__(a, b): return a.v <= _val(b)
    def __gt__(a, b): return a.v > _val(b)
    def __ge__(a, b): return a.v >= _val(b)
    def __float__(a): return a.v


def _val(x):
    return x.v if isinstance(x, Dual) else x


def _sqrt(x):
    if isinstance(x, Dual):
        s = math.sqrt(x.v)
        return Dual(s, 0.0 if x.d == 0.0 else x.d / (2.0 * s))
    return math.sqrt(x)


def _fabs(x):
    return abs(x) if isinstance(x, Dual) else math.fabs(x)


def _log10(x):
    return Dual(math.log10(x.v), x.d / (x.v * math.log(10.0))) if isinstance(x, Dual) else math.log10(x)


DARK_PROCESSES = ("DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem")
DARK_CODE = {p: i for i, p in enumerate(DARK_PROCESSES)}
DARK_DIM = {"DarkComp": 1, "DarkBrem": 3, "DarkAnn": 1, "DarkMuonBrem": 3}   # dark_shower.py:67
V_PID = 4900022
TWOBODY = "TwoBody_BSMDecay"
MESON_TWOBODY_BR = {111: 0.98823}       # meson_twobody_branchingratios, particle.py:39-48


def dark_key(pkey: int, process: str) -> int:
    """Stream key of dark process `process` produced by the particle `pkey`
    (daughters use multipliers 1 and 2; dark processes 3..6, the two-body
    meson decay 7)."""
    idx = 4 if process == TWOBODY else DARK_CODE[process]
    return mix64((int(pkey) + 0x9E3779B97F4A7C15 * (3 + idx)) & 0xFFFFFFFFFFFFFFFF)


def boost_matrix(pf, m0):
    """Particle.boost_matrix, particle.py:187-207: rest frame -> lab for a
    particle of final momentum pf and mass m0."""
    E0, px0, py0, pz0 = pf
    gamma = E0 / m0
    beta = 1.0 if gamma == 1.0 else math.sqrt(1.0 - 1.0 / gamma ** 2)
    pmag = P.norm3(px0, py0, pz0)
    if pmag == 0.0:
        return [[1.0 if i == j else 0.0 for j in range(4)] for i in range(4)]
    bx, by, bz = beta * px0 / pmag, beta * py0 / pmag, beta * pz0 / pmag
    return [[gamma, gamma * bx, gamma * by, gamma * bz],
            [gamma * bx, 1 + (gamma - 1) * bx ** 2 / beta ** 2, (gamma - 1) * bx * by / beta ** 2,
             (gamma - 1) * bx * bz / beta ** 2],
            [gamma * by, (gamma - 1) * by * bx / beta ** 2, 1 + (gamma - 1) * by ** 2 / beta ** 2,
             (gamma - 1) * by * bz / beta ** 2],
            [gamma * bz, (gamma - 1) * bz * bx / beta ** 2, (gamma - 1) * bz * by / beta ** 2,
             1 + (gamma - 1) * bz ** 2 / beta ** 2]]


def two_body_V(pf, mX, mV, u_ct, u_phi):
    """Particle.two_body_decay (particle.py:209-256) into (gamma, V) with its
    two draws (np.random.uniform(-1, 1) for cos theta, (0, 2 pi) for phi):
    the V four-momentum in the lab."""
    m1, m2 = 0.0, mV
    E1 = (mX ** 2 - m2 ** 2 + m1 ** 2) / (2 * mX)
    E2 = (mX ** 2 - m1 ** 2 + m2 ** 2) / (2 * mX)
    pF = math.sqrt(E1 ** 2 - m1 ** 2)
    cos_theta = -1.0 + (1.0 - -1.0) * u_ct
    phi = 0.0 + (2.0 * math.pi - 0.0) * u_phi
    sin_theta = math.sqrt(1 - cos_theta ** 2)
    q = (E2, pF * sin_theta * math.sin(phi), pF * sin_theta * math.cos(phi), pF * cos_theta)
    M = boost_matrix(pf, mX)
    return tuple(M[i][0] * q[0] + M[i][1] * q[1] + M[i][2] * q[2] + M[i][3] * q[3] for i in range(4))


# ------------------------------------------------------------ cross sections
def g_el_inel_over_t2(Z, A, t):
    """Gelastic_inelastic_over_tsquared, all_processes.py:112-133."""
    me = P.m_electron
    c1 = (111 * Z ** (-1 / 3) / me) ** 2
    c2 = 0.164 * P.GeV ** 2 * A ** (-2 / 3)
    Gel = (1.0 / (1.0 + c1 * t)) ** 2 * (1 + t / c2) ** (-2)
    ap2 = (773.0 * Z ** (-2.0 / 3) / me) ** 2
    Ginel = (Z / ((c1 ** 2 * Z ** 2)) * (ap2 / (1.0 + ap2 * t)) ** 2.0
             * ((1.0 + (2.79 ** 2 - 1.0) * t / (4.0 * P.m_proton ** 2)) / (1.0 + t / 0.71) ** 4))
    return Z ** 2 * c1 ** 2 * (Gel + Ginel)


def dsigma_dark_brem(xv, E, mV, MT, m_lep, Z, A):
    """dsig_dx_dcostheta_dark_brem_exact_tree_level.__call__ (all_processes.py:227-372),
    method "Log": xv = (x = E_V/E, log10(1 - cos theta), log10 t~)."""
    x, l1mct, lttilde = xv
    one_minus_ct = 10 ** l1mct
    ct = 1.0 - one_minus_ct
    ttilde = 10 ** lttilde
    jac = one_minus_ct * ttilde * math.log(10.0) ** 2
    k = _sqrt(_fabs((x * E) ** 2 - mV ** 2))
    p = _sqrt(E ** 2 - m_lep ** 2)
    V = _sqrt(p ** 2 + k ** 2 - 2 * p * k * ct)
    ut = -2 * (x * E ** 2 - k * p * ct) + mV ** 2
    Er = (1 - x) * E + MT
    discr = ut ** 2 + 4 * MT * ut * Er + 4 * MT ** 2 * V ** 2
    rd = _sqrt(_fabs(discr))
    den = 2 * Er ** 2 - 2 * V ** 2
    Qp = _fabs((V * (ut + 2 * MT * Er) + Er * rd) / den)
    Qm = _fabs((V * (ut + 2 * MT * Er) - Er * rd) / den)
    tp = 2 * MT * (_sqrt(MT ** 2 + Qp ** 2) - MT)
    tm = 2 * MT * (_sqrt(MT ** 2 + Qm ** 2) - MT)
    tconv = (2 * MT * (MT + E) * _sqrt(E ** 2 + m_lep ** 2) / (MT * (MT + 2 * E) + m_lep ** 2)) ** 2
    t = ttilde * tconv
    q0 = -t / (2 * MT)
    q = _sqrt(t ** 2 / (4 * MT ** 2) + t)
    cq = -(V ** 2 + q ** 2 + m_lep ** 2 - (E + q0 - x * E) ** 2) / (2 * V * q)
    mm = mV ** 2 + 2 * m_lep ** 2
    Am2 = -8 * MT * (4 * E ** 2 * MT - t * (2 * E + MT)) * mm
    A1 = 8 * MT ** 2 / ut
    Am1 = (8 / ut) * (MT ** 2 * (2 * t * ut + ut ** 2 + 4 * E ** 2 * (2 * (x - 1) * mm - t * ((x - 2) * x + 2))
                                 + 2 * t * (-(mV ** 2) + 2 * m_lep ** 2 + t))
                      - 2 * E * MT * t * ((1 - x) * ut + (x - 2) * (mm + t)) + t ** 2 * (ut - mV ** 2))
    A0 = (8 / ut ** 2) * (MT ** 2 * (2 * t * ut + (t - 4 * E ** 2 * (x - 1) ** 2) * mm)
                          + 2 * E * MT * t * (ut - (x - 1) * mm))
    Y = -t + 2 * q0 * E - 2 * q * p * (p - k * ct) * cq / V
    W = _fabs(Y ** 2 - 4 * q ** 2 * p ** 2 * k ** 2 * (1 - ct ** 2) * (1 - cq ** 2) / V ** 2)
    allowed = (x * E >= mV and discr >= 0 and tp > tm and t > tm and t < tp and _fabs(cq) <= 1.0 and W > 0)
    if not allowed:
        return 0.0
    phi_int = (A0 + Y * A1 + Am1 / _sqrt(W) + Y * Am2 / W ** 1.5) / (8 * MT ** 2)
    ff = g_el_inel_over_t2(Z, A, t)
    ans = ff * P.alpha_em ** 3 * k * E * phi_int / (p * _sqrt(k ** 2 + p ** 2 - 2 * p * k * ct))
    return ans * tconv * jac


def _kf_beta(s):
    return (2. * P.alpha_em / math.pi) * (math.log(s / P.m_electron ** 2) - 1.)


def fl_kf(x, s):
    """radiative_return.py:26-36 (Kuraev-Fadin structure function)."""
    beta = _kf_beta(s)
    if x >= 1.0:
        x = 1. - 1e-10
    return (beta / 16.) * ((8. + 3. * beta) * (1. - x) ** (beta / 2. - 1.) - 4. * (1. + x))


def fl_kf_scaled(x, s):
    """radiative_return.py:38-47."""
    beta = _kf_beta(s)
    return (beta / 16.) * ((8. + 3. * beta) - 4. * (1. + x) * (1. - x) ** (1. - beta / 2.))


def transformed_lumi(s, y, u):
    """transformed_lepton_luminosity_integrand, radiative_return.py:61-80."""
    beta = _kf_beta(s)
    x = 1. - u ** (2. / beta)
    return fl_kf(y / x, s) * fl_kf_scaled(x, s) * (1. / x) * (2. / beta)


def dsigma_radiative_return(u0, Ee, mV):
    """dsigma_radiative_return_du.__call__, all_processes.py:419-466."""
    me = P.m_electron
    s = 2.0 * me * (Ee + me)
    if s < mV ** 2:
        return 0.0
    beta = (2.0 * P.alpha_em / math.pi) * (math.log(s / me ** 2) - 1.0)
    umax = (1.0 - mV ** 2 / s) ** (beta / 2.0)
    betaf = math.sqrt(1.0 - 4.0 * (me ** 2) / (mV ** 2))
    prefac = (4.0 * math.pi ** 2) * P.alpha_em * betaf * (3.0 / 2.0 - betaf ** 2 / 2.0) / s * umax
    x1 = 1.0 - (u0 * umax) ** (2.0 / beta)
    x2 = mV ** 2 / (x1 * s)
    if not (x2 < 1.0 and x1 > 0.0 and u0 < 1.0):
        return 0.0
    return 2.0 * prefac * transformed_lumi(s, mV ** 2 / s, u0 * umax)


def dsigma_radiative_return_factored(u0, Ee, mV):
    """dsigma_radiative_return with 1 - x2 written as (s - mV^2)(1 - u0^(2/beta))/(x1 s)
    (the same quantity without cancellation near x2 -> 1); used for yields."""
    me = P.m_electron
    s = 2.0 * me * (Ee + me)
    if s < mV ** 2:
        return 0.0
    beta = (2.0 * P.alpha_em / math.pi) * (math.log(s / me ** 2) - 1.0)
    umax = (1.0 - mV ** 2 / s) ** (beta / 2.0)
    betaf = _sqrt(1.0 - 4.0 * (me ** 2) / (mV ** 2))
    prefac = (4.0 * math.pi ** 2) * P.alpha_em * betaf * (3.0 / 2.0 - betaf ** 2 / 2.0) / s * umax
    omx1 = (u0 * umax) ** (2.0 / beta)
    x1 = 1.0 - omx1
    x2 = mV ** 2 / (x1 * s)
    if not (x2 < 1.0 and x1 > 0.0 and u0 < 1.0):
        return 0.0
    omx2 = (s - mV ** 2) * (-math.expm1((2.0 / beta) * math.log(u0))) / (x1 * s)
    fy = (beta / 16.) * ((8. + 3. * beta) * omx2 ** (beta / 2. - 1.) - 4. * (1. + x2))
    base = omx1 if isinstance(x1, Dual) else 1. - x1      # 1 - x1 without cancellation for derivatives
    fs = (beta / 16.) * ((8. + 3. * beta) - 4. * (1. + x1) * base ** (1. - beta / 2.))
    return 2.0 * prefac * (fy * fs * (1. / x1) * (2. / beta))


def dsigma_compton_dark(ct, Eg, mV):
    """dsigma_compton_dCT with mV > 0 (all_processes.py:639-742) for a float or
    Dual mass (same expressions as physics.dsigma_compton)."""
    me = P.m_electron
    s = me ** 2 + 2 * Eg * me
    if s < (me + mV) ** 2:
        return 0.0
    root = _sqrt(me ** 4 + (mV ** 2 - s) ** 2 - 2 * me ** 2 * (mV ** 2 + s))
    jac = (s - me ** 2) / (2 * s) * _sqrt((s - mV ** 2) ** 2 - 2 * me ** 2 * (s + mV ** 2) + me ** 4)
    t = -1 / 2 * (me ** 4 + s * (-(mV ** 2) + s + ct * root) - me ** 2 * (mV ** 2 + 2 * s + ct * root)) / s
    PF = 2.0 * math.pi * P.alpha_em ** 2 / (s - me ** 2) ** 2
    T1 = (2.0 * me ** 2 * (mV ** 2 - 3 * s) - 3 * me ** 4 - 2 * mV ** 2 * s + 2 * mV ** 4 + s ** 2) \
        / ((me ** 2 - s) * (me ** 2 + mV ** 2 - s - t))
    T2 = (2 * me ** 2 * (2 * me ** 2 + mV ** 2)) / (me ** 2 + mV ** 2 - s - t) ** 2
    T3 = ((me ** 2 + s) * (me ** 2 + mV ** 2 + s) + t * (s - me ** 2)) / (me ** 2 - s) ** 2
    return PF * jac * (T1 + T2 + T3)


def _ev(process, x, E, mV):
    """Lab energy of V for the yield moments (kinematics.py:57,119-130,282-298)."""
    if process in ("DarkBrem", "DarkMuonBrem"):
        return x[0] * E
    me = P.m_electron
    if process == "DarkComp":
        s = me ** 2 + 2 * E * me
        rs = math.sqrt(s)
        Ee0 = (s + me ** 2) / (2.0 * rs)
        Ee = (s - mV ** 2 + me ** 2) / (2 * rs)
        EV = (s + mV ** 2 - me ** 2) / (2 * rs)
        pF = _sqrt(Ee ** 2 - me ** 2)
        g0 = Ee0 / me
        b0 = 1.0 / g0 * math.sqrt(g0 ** 2 - 1.0)
        return g0 * EV - b0 * g0 * pF * x[0]
    s = 2. * me * (me + E)
    rs = math.sqrt(s)
    beta = (2. * P.alpha_em / math.pi) * (math.log(s / me ** 2) - 1.)
    umax = (1. - mV ** 2 / s) ** (beta / 2.)
    x1 = 1. - (x[0] * umax) ** (2. / beta)
    x2 = mV ** 2 / (x1 * s)
    E1, E2 = x1 * rs / 2., x2 * rs / 2.
    p0, p3 = rs / 2., -math.sqrt(s / 4. - me ** 2)
    return (p0 * (E1 + E2) - p3 * (E1 - E2)) / math.sqrt(p0 * p0 - p3 * p3)


def dsigma_dark(process, xv, E, mV, Z, A):
    """The differential cross section draw_dark_sample evaluates
    (dark_shower.py:673-684): target mass = A_T, lepton mass by process."""
    if process == "DarkBrem":
        return dsigma_dark_brem(xv, E, mV, A, P.m_electron, Z, A)
    if process == "DarkMuonBrem":
        return dsigma_dark_brem(xv, E, mV, A, P.m_muon, Z, A)
    if process == "DarkComp":
        return P.dsigma_compton(xv[0], E, mV)
    if process == "DarkAnn":
        return dsigma_radiative_return(xv[0], E, mV)
    raise Exception("Your process is not in the list")


# --------------------------------------------------------------- kinematics
def l_to_lV(ep, m_lep, xv, mV, al):
    """l_to_lV_fourvecs, kinematics.py:43-68 (al = azimuth)."""
    w = xv[0] * ep
    ct = (1 - 10 ** xv[1])
    p, k = math.sqrt(ep ** 2 - m_lep ** 2), math.sqrt(w ** 2 - mV ** 2)
    cal, sal = math.cos(al), math.sin(al)
    st = math.sqrt(1.0 - ct ** 2)
    return (ep, 0, 0, p), (w, k * cal * st, k * sal * st, k * ct)


def boost(p, v):
    """radiative_return.py:18-24: v in the rest frame of p."""
    def lor(a, b):
        return a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3]
    rsq = math.sqrt(lor(p, p))
    v0 = lor(p, v) / rsq
    c1 = (v[0] + v0) / (rsq + p[0])
    return (v0, v[1] - c1 * p[1], v[2] - c1 * p[2], v[3] - c1 * p[3])


def radiative_return_V(Ee, u0, mV):
    """radiative_return_fourvecs, kinematics.py:267-299: the V four-vector."""
    me = P.m_electron
    s = 2. * me * (me + Ee)
    beta = (2. * P.alpha_em / math.pi) * (math.log(s / me ** 2) - 1.)
    umax = (1. - mV ** 2 / s) ** (beta / 2.)
    x1 = 1. - (u0 * umax) ** (2. / beta)
    x2 = mV ** 2 / (x1 * s)
    E1 = x1 * math.sqrt(s) / 2.
    E2 = x2 * math.sqrt(s) / 2.
    pV = (E1 + E2, 0. + 0., 0. + 0., E1 + -E2)
    return boost((math.sqrt(s) / 2., 0., 0., -math.sqrt(s / 4. - me ** 2)), pV)


def compton_bound(Eg, ct, mV, Pe, cte, ph, phie):
    """compton_fourvecs_boundelectron, kinematics.py:134-183: the V four-vector."""
    me = P.m_electron
    s = me ** 2 + 2 * Eg * (math.sqrt(me ** 2 + Pe ** 2) - cte * Pe)
    rs = math.sqrt(s)
    Ee = (s - mV ** 2 + me ** 2) / (2 * rs)
    EV = (s + mV ** 2 - me ** 2) / (2 * rs)
    pF = math.sqrt(Ee ** 2 - me ** 2)
    bnum = math.sqrt(Eg ** 2 + 2 * cte * Eg * Pe + Pe ** 2)
    bden = Eg + math.sqrt(me ** 2 + Pe ** 2)
    b0 = bnum / bden
    g0 = 1.0 / math.sqrt(1.0 - b0 ** 2)
    st = math.sqrt(1 - ct ** 2)
    EVLab = g0 * EV - b0 * g0 * pF * ct
    v = (pF * st * math.sin(ph), pF * st * math.cos(ph), b0 * g0 * EV - g0 * pF * ct)
    ctz = (Eg + cte * Pe) / math.sqrt(Eg ** 2 + 2 * cte * Eg * Pe + Pe ** 2)
    stz = math.sqrt(1.0 - ctz ** 2)
    cf, sf = math.cos(phie), math.sin(phie)
    R = ((ctz * cf, -sf, stz * cf), (ctz * sf, cf, stz * sf), (-stz, 0, ctz))
    return (EVLab, R[0][0] * v[0] + R[0][1] * v[1] + R[0][2] * v[2],
            R[1][0] * v[0] + R[1][1] * v[1] + R[1][2] * v[2],
            R[2][0] * v[0] + R[2][1] * v[1] + R[2][2] * v[2])


def electron_wave_function(pe, Zeff):
    """dark_shower.py:706-708."""
    lam = P.alpha_em * Zeff * P.m_electron
    return 32 / math.pi * lam ** 5 * pe ** 2 / (pe ** 2 + lam ** 2) ** 4


def draw_pe_sample(Zeff, s: Stream):
    """dark_shower.py:710-719: accept-reject on [0, 1 MeV]."""
    c = electron_wave_function(P.alpha_em * Zeff * P.m_electron / math.sqrt(3), Zeff)
    pe_max = 1e-3
    while True:
        x = 0 + (pe_max - 0) * s.next()
        u = 0 + (1 - 0) * s.next()
        if u < electron_wave_function(x, Zeff) / (c):
            return x


# ------------------------------------------------------------------ tables
def closest_lesser(masses, v):
    """DarkShower.closest_lesser_value (dark_shower.py:158-165) for masses at
    or above the smallest one (below it the reference wraps to the last)."""
    arr = np.asarray(masses, dtype=float)
    i = int(np.abs(arr - v).argmin())
    return float(arr[i]) if arr[i] <= v else float(arr[i - 1])


class DarkTables:
    """One DarkShower's tables for (target, mV) from the bundled
    ``dark_tables.npz`` (maps rebuilt with PETITE's find_maxes; weight, dR/dE
    and bound-electron tables as PETITE's DarkShower constructor builds them)."""

    def __init__(self, npz_path, target, mV, maxF_fudge=1.0, Zeff=29.508, kinetic_mixing=1.0, bound_electron=True):
        z = np.load(npz_path, allow_pickle=False)
        self.bound = bound_electron
        masses = [float(m) for m in z["masses"]]
        targets = [str(t) for t in z["targets"]]
        if target not in targets:
            raise Exception("Target Material is not in library")
        if mV < masses[0]:
            raise ValueError("no dark map at or below this mass")
        self.mV = closest_lesser(masses, mV)
        key = f"m{self.mV}"
        j = targets.index(target)
        ti = P.TARGETS[target]
        self.Z, self.A, self.rho, self.dEdx = ti["Z_T"], ti["A_T"], ti["rho"], ti["dEdx"]
        self.Zeff = Zeff
        g_e = kinetic_mixing * math.sqrt(4 * math.pi * P.alpha_em)
        self.coupling = g_e ** 2 / (4 * math.pi * P.alpha_em)
        self.maps = {}
        for p in DARK_PROCESSES:
            if f"{key}/{p}/energy" not in z:         # no maps (DarkAnn below mV = 2 m_e)
                continue
            E = z[f"{key}/{p}/energy"]
            grid, nn = z[f"{key}/{p}/grid"], z[f"{key}/{p}/nnodes"]
            self.maps[p] = [dict(E=float(E[i]), neval=int(z[f"{key}/{p}/neval"][i]),
                                 maxF=float(z[f"{key}/{p}/max_F"][i, j]) * maxF_fudge,
                                 grid=[grid[i, k, :nn[i, k]].tolist() for k in range(grid.shape[1])])
                            for i in range(len(E))]
        self.map_E = {p: np.array([r["E"] for r in rows]) for p, rows in self.maps.items()}
        pre = f"{key}/{target}"
        self.E_res = float(z[f"{pre}/E_res"])
        self.E_compth = float(z[f"{pre}/E_compth"])
        md = z[f"{pre}/min_dark"]
        self.min_dark = {(11, "DarkBrem"): md[0], (-11, "DarkBrem"): md[1], (-11, "DarkAnn"): md[2],
                         (22, "DarkComp"): md[3], (13, "DarkMuonBrem"): md[4], (-13, "DarkMuonBrem"): md[4]}
        self.weights = {k: (z[f"{pre}/weights/{k}"][:, 0].tolist(), z[f"{pre}/weights/{k}"][:, 1].tolist())
                        for k in ("brem_elec", "brem_positron", "ann", "muon_brem")}
        self.drate = {k: (z[f"{pre}/drate/{k}/Ei"], z[f"{pre}/drate/{k}/bins"], z[f"{pre}/drate/{k}/nbins"])
                      for k in ("brem_elec", "brem_positron", "ann", "muon_brem")}
        # set_dark_NSigmas (dark_shower.py:286-297): DarkComp, log-log, fill -20
        DCS = z[f"{pre}/xsec/DarkComp_bound"]
        nZ = self.rho / P.m_proton_grams / self.A
        ne = nZ * self.Z
        self.ne = ne
        if not bound_electron:
            # free electrons (bound_electron=False): dark_xsec.pkl's DarkAnn and
            # DarkComp, the annihilation weights and dR/dE with the resonant bin,
            # the thresholds (dark_shower.py:229-245,254-309,382-452,495-593)
            fpre = f"{pre}/free"
            DCS = z[f"{fpre}/xsec/DarkComp"]
            self.ann_E0 = float(z[f"{fpre}/xsec/DarkAnn"][0, 0])
            md = z[f"{fpre}/min_dark"]
            self.min_dark = {(11, "DarkBrem"): md[0], (-11, "DarkBrem"): md[1], (-11, "DarkAnn"): md[2],
                             (22, "DarkComp"): md[3], (13, "DarkMuonBrem"): md[4], (-13, "DarkMuonBrem"): md[4]}
            w = z[f"{fpre}/weights/ann"]
            self.weights["ann"] = (w[:, 0].tolist(), w[:, 1].tolist())
            self.drate["ann"] = (z[f"{fpre}/drate/ann/Ei"], z[f"{fpre}/drate/ann/bins"], z[f"{fpre}/drate/ann/nbins"])
            # the positron interaction integrals of Shower.set_NSigmas (shower.py:296-314)
            self.ii = {k: (z[f"{target}/ii/{k}"][:, 0].tolist(), z[f"{target}/ii/{k}"][:, 1].tolist())
                       for k in ("Brem", "Ann", "Bhabha")}
        self.nsc = (np.log10(DCS[:, 0] + 1e-20).tolist(), np.log10(ne * P.GeVsqcm2 * DCS[:, 1] + 1e-20).tolist())


def _interp_fill(v, table, fill):
    xs, ys = table
    if not (v >= xs[0]) or v > xs[-1]:
        return fill
    return interp(v, table)


def _np_sum(a):
    """numpy's pairwise sum of a short 1-D float64 array."""
    n = len(a)
    if n < 8:
        r = 0.0
        for x in a:
            r += x
        return r
    r = [float(x) for x in a[:8]]
    i = 8
    while i + 8 <= n:
        for j in range(8):
            r[j] += a[i + j]
        i += 8
    res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]))
    while i < n:
        res += a[i]
        i += 1
    return res


class DarkOracle:
    """GetBSMWeights, draw_dark_sample and produce_bsm_particle on one SM
    particle record (fields of :class:`oracle.shower.Rec`)."""

    def __init__(self, dark: DarkTables, sm_tables, seed, max_n_integrators=10000, rescale=1.0,
                 fast_MCS_mode=True, kinetic_mixing=1.0):
        self.d, self.sm, self.seed = dark, sm_tables, seed
        self.kinetic_mixing = kinetic_mixing
        self.max_n_integrators = max_n_integrators
        self.rescale = rescale
        self.fast_mcs = fast_MCS_mode              # dark_shower.py:134-138

    # dark_shower.py:595-647 (bound-electron form)
    def weight(self, pid, E, process, mass=None):
        d = self.d
        if process == TWOBODY:
            # dark_shower.py:633-638 (pi0; eta and eta' raise KeyError at :604)
            if pid != 111:
                return 0.0
            mass_ratio = d.mV / mass
            if mass_ratio >= 1.0:
                return 0.0
            return 2 * self.kinetic_mixing ** 2 * (1.0 - mass_ratio ** 2) ** 3 * MESON_TWOBODY_BR[111]
        key = (pid, process)
        if key not in d.min_dark:
            return 0.0
        if E < d.min_dark[key]:
            return 0.0
        if pid == 22:
            if E < self.sm.min_calc[22]:
                return 0.0
            nd = 10 ** _interp_fill(math.log10(E), d.nsc, -20.0)
            return d.coupling * nd / (interp(E, self.sm.ns["PairProd"]) + interp(E, self.sm.ns["Comp"]))
        name = {(11, "DarkBrem"): "brem_elec", (-11, "DarkBrem"): "brem_positron", (-11, "DarkAnn"): "ann",
                (13, "DarkMuonBrem"): "muon_brem", (-13, "DarkMuonBrem"): "muon_brem"}[key]
        if key == (-11, "DarkAnn") and not d.bound:
            # dark_shower.py:619-630: the tabulated part above the first saved
            # energy plus the resonant part in closed form
            me = P.m_electron
            E0s = d.ann_E0
            sMAX = 2 * (me * min(E0s, E) + me ** 2)
            beta = (2. * P.alpha_em / math.pi) * (math.log(sMAX / me ** 2) - 1.)
            dEdxT_GeVpercm = d.dEdx * (0.1) * P.cmtom
            base = np.float64(sMAX - d.mV ** 2)
            with np.errstate(invalid="ignore"):
                wa = (1 / dEdxT_GeVpercm) * (2 * math.pi ** 2 * P.alpha_em / me) * d.ne * P.GeVsqcm2 * float(base ** beta) \
                    * self.positron_exponential_factor(d.E_res, E)
            wn = interp(E, d.weights[name]) if E > E0s else 0.0
            return d.coupling * (wn + wa)
        return d.coupling * interp(E, d.weights[name])

    def positron_exponential_factor(self, E, Ei):
        """Shower._positron_exponential_factor, shower.py:322-334."""
        ii = self.d.ii
        n_sigma_diff = (interp(Ei, ii["Brem"]) - interp(E, ii["Brem"])) \
            + (interp(Ei, ii["Ann"]) - interp(E, ii["Ann"])) \
            + (interp(Ei, ii["Bhabha"]) - interp(E, ii["Bhabha"]))
        if n_sigma_diff < 0.0 or E > Ei:
            return 0.0
        dEdxT = self.d.dEdx * (0.1)
        return math.exp(-n_sigma_diff / dEdxT / P.cmtom)

    # dark_shower.py:649-704
    def draw(self, E, process, s: Stream, count=None):
        rows, energies = self.d.maps[process], self.d.map_E[process]
        key = int(np.argmin(np.abs(energies - E))) + 1
        if key >= len(rows):
            key = len(rows) - 1
        row = rows[key]
        dim = DARK_DIM[process]
        proposals = 0
        for _ in range(self.max_n_integrators):
            for _ in range(row["neval"]):
                y = [s.next() for _ in range(dim)]
                x, jac = map_point(row["grid"], y)
                wgt = jac / row["neval"]
                proposals += 1
                f = dsigma_dark(process, x, E, self.d.mV, self.d.Z, self.d.A)
                if row["maxF"] * s.next() < wgt * f:
                    if count is not None:
                        count.append(proposals)
                    return x, key
        if count is not None:
            count.append(-1)
        return None, key

    # dark_shower.py:721-804; returns (V four-vector, weight) or None
    def produce(self, r, process, wg, s: Stream):
        d, me, mV = self.d, P.m_electron, self.d.mV
        pf = tuple(r.pf)
        table = None
        if process == "DarkAnn" and r.pid == -11:
            table = "ann"
        elif process == "DarkBrem":
            table = "brem_elec" if r.pid == 11 else "brem_positron"
        elif process == "DarkMuonBrem":
            table = "muon_brem"
        if table is not None:
            Ei_all, bins_all, nb_all = d.drate[table]
            E0 = r.p0[0]
            if E0 < Ei_all.min():
                j = int(np.argmin(Ei_all))
            elif E0 > Ei_all.max():
                j = int(np.argmax(Ei_all))
            else:
                j = int(np.flatnonzero(Ei_all == max(e for e in Ei_all if e <= E0))[0])
            nb = int(nb_all[j])
            en, w = bins_all[j, :nb, 0], bins_all[j, :nb, 1]
            tot = _np_sum(w)
            if tot == 0.0:
                return None
            p = [x / tot for x in w]
            cdf, c = [], 0.0
            for x in p:
                c += x
                cdf.append(c)
            u = s.next()
            idx = bisect_right([c_ / cdf[-1] for c_ in cdf], u)
            E_int = en[idx] + (E0 - Ei_all[j])
            dist = (r.p0[0] - E_int) / (d.dEdx * 0.1)
            ps = tuple(r.p0)
            if P.norm3(ps[1], ps[2], ps[3]) > 0 and not self.fast_mcs:
                ps = P.scattered_momentum_bethe(ps, d.rho * (dist / P.cmtom), d.A, d.Z, self.rescale, s.next)
            elif P.norm3(ps[1], ps[2], ps[3]) > 0:
                u1, u2, u3, u4 = s.next(), s.next(), s.next(), s.next()
                ps = P.scattered_momentum_fast(ps, d.rho * (dist / P.cmtom), d.A, d.Z, self.rescale,
                                               P.m_electron, u1, u2, u3, u4)
            pf = P.lose_energy(ps, r.mass, E0 - E_int)
        E0 = pf[0]
        RM = P.rotation_matrix_from(pf)
        if process == "DarkAnn" and E0 <= d.E_res and d.bound:
            v = (math.sqrt(E0 ** 2 - me ** 2 + mV ** 2), 0, 0, math.sqrt(E0 ** 2 - me ** 2))
        elif process == "DarkComp" and E0 <= d.E_compth and d.bound:
            v = (math.sqrt(E0 ** 2 + mV ** 2), 0, 0, E0)
        elif process == "DarkAnn" and not d.bound and E0 <= d.ann_E0:
            # dark_shower.py:767-768
            v = (d.E_res, 0, 0, math.sqrt(d.E_res ** 2 - mV ** 2))
        else:
            x, _ = self.draw(E0, process, s)
            if x is None:
                return None
            if process == "DarkComp" and not d.bound:
                # compton_fourvecs with mV (kinematics.py:104-132)
                v = P.compton(E0, x[0], 0 + (2.0 * math.pi - 0) * s.next(), mV)[1]
            elif process == "DarkComp":
                pe = draw_pe_sample(d.Zeff, s)
                c0 = -1 + (1 - -1) * s.next()
                ss = me ** 2 + 2 * E0 * (math.sqrt(me ** 2 + pe ** 2) - c0 * pe)
                Ee = (ss - mV ** 2 + me ** 2) / (2 * math.sqrt(ss))
                if Ee < me:
                    v, wg = (mV, 0, 0, 0), 0.0
                else:
                    ph = 0 + (2.0 * math.pi - 0) * s.next()
                    phie_u = s.next()
                    v = compton_bound(E0, x[0], mV, pe, c0, ph, 0 + (2.0 * math.pi - 0) * phie_u)
            elif process in ("DarkBrem", "DarkMuonBrem"):
                al = 0 + (2.0 * math.pi - 0) * s.next()
                v = l_to_lV(E0, r.mass, x, mV, al)[1]
            elif process == "DarkAnn":
                v = radiative_return_V(E0, x[0], mV)
        lab = (v[0],
               RM[0][0] * v[1] + RM[0][1] * v[2] + RM[0][2] * v[3],
               RM[1][0] * v[1] + RM[1][1] * v[2] + RM[1][2] * v[3],
               RM[2][0] * v[1] + RM[2][1] * v[2] + RM[2][2] * v[3])
        return lab, wg

    # dark_shower.py:806-849 over SM records
    def dark_shower(self, records, processes=DARK_PROCESSES):
        out = []
        for k, r in enumerate(records):
            for p in processes:
                wg = self.weight(r.pid, r.p0[0], p, r.mass)
                if wg > 0.0 and p == TWOBODY:
                    s = Stream(self.seed, dark_key(r.pkey, p))
                    v = two_body_V(tuple(r.pf), r.mass, self.d.mV, s.next(), s.next())
                    out.append((k, p, wg * r.weight, v, tuple(r.rf)))
                elif wg > 0.0:
                    s = Stream(self.seed, dark_key(r.pkey, p))
                    res = self.produce(r, p, wg, s)
                    if res is not None:
                        v, w = res
                        out.append((k, p, w * r.weight, v, tuple(r.rf)))
        return out


# ------------------------------------------------------------- dark yield
def yield_uniforms(seed, pair, process, j):
    """Draws 4j..4j+3 of the stream (seed, mix64(4*pair + process + 1))."""
    from .philox import uniforms
    return uniforms(seed, mix64(4 * pair + DARK_CODE[process] + 1), 4 * j, 4)


def _yield_sum(dark, process, E, mV, pair, n_samples, seed, anchor=None):
    rows, energies = dark.maps[process], dark.map_E[process]
    key = int(np.argmin(np.abs(energies - E))) + 1
    if key >= len(rows):
        key = len(rows) - 1
    grid = rows[key]["grid"]
    dim = DARK_DIM[process]
    from .philox import uniforms
    u_all = uniforms(seed, mix64(4 * pair + DARK_CODE[process] + 1), 0, 4 * n_samples).reshape(n_samples, 4)
    m = P.m_muon if process == "DarkMuonBrem" else P.m_electron
    sy = sm = 0.0
    for j in range(n_samples):
        x, jac = map_point(grid, u_all[j, :dim])
        if process in ("DarkBrem", "DarkMuonBrem") and anchor is not None:
            f = dsigma_dark_brem_anchored(x, E, mV, anchor, dark.A, m, dark.Z, dark.A)
            xa, xm = anchor / E, mV / E
            ev = (xm + (x[0] - xa) / (1.0 - xa) * (1.0 - xm)) * E
        else:
            if process == "DarkAnn":
                f = dsigma_radiative_return_factored(x[0], E, mV)
            elif process == "DarkComp":
                f = dsigma_compton_dark(x[0], E, mV)
            else:
                f = dsigma_dark_brem(x, E, mV, dark.A, m, dark.Z, dark.A)
            ev = None
        if _val(f) == 0.0:
            continue
        if ev is None:
            ev = _ev(process, x, E, mV)
        sy = sy + jac * f
        sm = sm + jac * f * ev
    return sy / n_samples, sm / n_samples


def dark_yield(dark: DarkTables, process, E, mV, pair, n_samples, seed):
    """Mean of jac*dsigma and of jac*dsigma*E_V over the map row LU_Key(E),
    at the uniforms of :func:`yield_uniforms` (float64, sequential); the
    radiative return in its factored form (1 - x2 without cancellation)."""
    return _yield_sum(dark, process, E, mV, pair, n_samples, seed)


def dark_yield_gradient(dark: DarkTables, process, E, mV, pair, n_samples, seed):
    """Float64 reference of d(yield)/d(mV) and d(moment)/d(mV): forward-mode
    derivatives of the same sums, DarkBrem samples carried with mV."""
    y, m = _yield_sum(dark, process, E, Dual(mV, 1.0), pair, n_samples, seed,
                      anchor=mV if process in ("DarkBrem", "DarkMuonBrem") else None)
    return (y.d if isinstance(y, Dual) else 0.0), (m.d if isinstance(m, Dual) else 0.0)


# --------------------------------------------- anchored dark-brem estimate
def _brem_limits_stable(x, ct, E, mV, MT, m):
    """t- and t+ of all_processes.py:261-283 written without cancellation:
    Q- = -ut (ut + 4 MT Er) / (2 (A + B)), t = 2 MT Q^2 / (sqrt(MT^2 + Q^2) + MT)."""
    k = _sqrt(_fabs((x * E) ** 2 - mV ** 2))
    p = _sqrt(E ** 2 - m ** 2)
    V = _sqrt(p ** 2 + k ** 2 - 2 * p * k * ct)
    ut = -2 * (x * E ** 2 - k * p * ct) + mV ** 2
    Er = (1 - x) * E + MT
    discr = ut ** 2 + 4 * MT * ut * Er + 4 * MT ** 2 * V ** 2
    A_ = V * (ut + 2 * MT * Er)
    B_ = Er * _sqrt(_fabs(discr))
    den = 2 * Er ** 2 - 2 * V ** 2
    Qp = abs((A_ + B_) / den)
    Qm = abs(ut * (ut + 4 * MT * Er) / (2 * (A_ + B_)))
    tp = 2 * MT * Qp ** 2 / (_sqrt(MT ** 2 + Qp ** 2) + MT)
    tm = 2 * MT * Qm ** 2 / (_sqrt(MT ** 2 + Qm ** 2) + MT)
    return discr, tm, tp


def dsigma_dark_brem_anchored(xv, E, mV, a, MT, m_lep, Z, A):
    """The dark-brem integrand with the sample (drawn for mass a) carried to
    mass mV: x keeps its fraction of (mV/E, 1), log10 t~ its fraction of the
    t-range; times the Jacobian of the move.  Equals dsigma_dark_brem at mV = a
    up to rounding; smooth in mV."""
    x0, l1mct, l0 = xv
    omc = 10 ** l1mct
    ct = 1.0 - omc
    tconv = (2 * MT * (MT + E) * _sqrt(E ** 2 + m_lep ** 2) / (MT * (MT + 2 * E) + m_lep ** 2)) ** 2
    xa = a / E
    w = (x0 - xa) / (1.0 - xa)
    if not (0.0 < w < 1.0):
        return 0.0
    d, tm, tp = _brem_limits_stable(x0, ct, E, a, MT, m_lep)
    if not (d >= 0 and tp > tm and tm > 0):
        return 0.0
    lma, lpa = _log10(tm / tconv), _log10(tp / tconv)
    v = (l0 - lma) / (lpa - lma)
    if not (0.0 < v < 1.0):
        return 0.0
    xm = mV / E
    x = xm + w * (1.0 - xm)
    d, tm, tp = _brem_limits_stable(x, ct, E, mV, MT, m_lep)
    if not (d >= 0 and tp > tm and tm > 0):
        return 0.0
    lm, lp = _log10(tm / tconv), _log10(tp / tconv)
    l = lm + (lp - lm) * v
    f = dsigma_dark_brem((x, l1mct, l), E, mV, MT, m_lep, Z, A)
    return f * ((lp - lm) / (lpa - lma)) * ((1.0 - xm) / (1.0 - xa))


def dark_yield_anchored(dark: DarkTables, process, E, mV, anchor, pair, n_samples, seed):
    """dark_yield with DarkBrem samples carried from the anchor mass."""
    a = anchor if process in ("DarkBrem", "DarkMuonBrem") else None
    return _yield_sum(dark, process, E, mV, pair, n_samples, seed, anchor=a)
