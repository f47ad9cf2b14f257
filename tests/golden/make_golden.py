"""Generate golden vectors by running the unmodified PETITE reference.

Runs only in the development container (the reference is not present on the
GPU machine); the outputs are committed as ``tests/golden/*.npz``.

The reference draws from numpy's and Python's global generators.  Here every
call site on the SM shower path is redirected to the per-particle Philox
stream of the particle being processed (``oracle/philox.py``):

* ``PETITE.shower.draw_U``      (accept/reject uniform, shower.py:30,457)
* ``numpy.random.uniform``      (shower.py:540,561-562,583; kinematics.py azimuths)
* ``numpy.random.choice``       (process choice, shower.py:671-697): cumsum,
                                  normalise by the last entry, searchsorted right
* ``random.choice/gauss/uniform`` (moliere.py:284,382); gauss is Box-Muller with
                                  the second value cached exactly as CPython does
* ``vegas.UNIFORM``             (the map-sampling shim's y draws)

The particle being processed is tracked by wrapping the Shower instance's
``propagate_particle`` and ``sample_scattering``; daughters get the keys of
``oracle.philox.daughter_key``.

Usage: python tests/golden/make_golden.py DICT_DIR [units|showers|dark|darkfree|moliere|mesons|files|particles|all]
(DICT_DIR from rebuild_maps.py; for ``dark`` it must also hold the output of
``rebuild_maps.py --dark``)
"""
import copy
import math
import os
import random
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import refimport  # noqa: E402
from oracle.philox import Stream, daughter_key, primary_key  # noqa: E402

SEED = 0x5EED


class StreamRouter:
    def __init__(self, seed):
        self.seed = seed
        self.streams = {}
        self.cur = None
        self.gauss_next = None

    def stream(self, pkey):
        if pkey not in self.streams:
            self.streams[pkey] = Stream(self.seed, pkey)
        return self.streams[pkey]

    def set_current(self, pkey):
        if self.gauss_next is not None:
            raise RuntimeError("gauss cache not empty on particle switch")
        self.cur = self.stream(pkey)

    def u(self):
        return self.cur.next()


def install(router):
    import vegas
    import PETITE.shower as sh
    saved = dict(draw_U=sh.draw_U, uniform=np.random.uniform, choice=np.random.choice,
                 rgauss=random.gauss, rchoice=random.choice, runiform=random.uniform,
                 vu=vegas.UNIFORM)

    def draw_U():
        return router.u()

    def np_uniform(low=0.0, high=1.0, size=None):
        if size is not None:
            raise RuntimeError("sized uniform not on the shower path")
        return low + (high - low) * router.u()

    def np_choice(a, size=None, replace=True, p=None):
        p = np.asarray(p, dtype=float)
        cdf = p.cumsum()
        cdf /= cdf[-1]
        idx = int(cdf.searchsorted(router.u(), side="right"))
        return a[idx]

    def r_gauss(mu=0.0, sigma=1.0):
        z = router.gauss_next
        router.gauss_next = None
        if z is None:
            x2pi = router.u() * (2 * math.pi)
            g2rad = math.sqrt(-2.0 * math.log(1.0 - router.u()))
            z = math.cos(x2pi) * g2rad
            router.gauss_next = math.sin(x2pi) * g2rad
        return mu + z * sigma

    def r_choice(seq):
        return seq[int(router.u() * len(seq))]

    def r_uniform(a, b):
        return a + (b - a) * router.u()

    sh.draw_U = draw_U
    np.random.uniform = np_uniform
    np.random.choice = np_choice
    random.gauss = r_gauss
    random.choice = r_choice
    random.uniform = r_uniform
    vegas.UNIFORM = lambda n: np.array([router.u() for _ in range(n)])
    return saved


def install_dark(router):
    """The dark module imports numpy's random() under its own name."""
    import PETITE.dark_shower as ds
    saved = ds.draw_U
    ds.draw_U = lambda: router.u()
    return saved


def uninstall_dark(saved):
    import PETITE.dark_shower as ds
    ds.draw_U = saved


def uninstall(saved):
    import vegas
    import PETITE.shower as sh
    sh.draw_U = saved["draw_U"]
    np.random.uniform = saved["uniform"]
    np.random.choice = saved["choice"]
    random.gauss, random.choice, random.uniform = saved["rgauss"], saved["rchoice"], saved["runiform"]
    vegas.UNIFORM = saved["vu"]


def wrap_shower(shower, router):
    orig_prop = shower.propagate_particle
    orig_ss = shower.sample_scattering

    def prop(ap, *a, **k):
        router.set_current(ap._pkey)
        return orig_prop(ap, *a, **k)

    def ss(ap, process, VB=False):
        router.set_current(ap._pkey)
        out = orig_ss(ap, process, VB=VB)
        if out is not None:
            for bit, d in enumerate(out):
                d._pkey = daughter_key(ap._pkey, bit)
        return out

    shower.propagate_particle = prop
    shower.sample_scattering = ss


PROC_CODE = {"Input": -1, "Brem": 0, "Ann": 1, "PairProd": 2, "Comp": 3, "Moller": 4,
             "Bhabha": 5, "MuonE": 6, "MuonBrem": 7}


def shower_arrays(parts, router, primary):
    n = len(parts)
    f = np.zeros((n, 16))
    i = np.zeros((n, 6), np.int64)
    ids = []
    keys = np.zeros(n, np.uint64)
    draws = np.zeros(n, np.int64)
    for k, p in enumerate(parts):
        d = p.get_ids()
        f[k, 0:4] = p.get_p0()
        f[k, 4:7] = p.get_r0()
        f[k, 7:11] = p.get_pf()
        f[k, 11:14] = p.get_rf()
        f[k, 14] = d["weight"]
        f[k, 15] = d["mass"]
        i[k] = [d["PID"], d["parent_PID"], d["generation_number"], PROC_CODE[d["generation_process"]],
                int(p.get_ended()), primary]
        ids.append((d["ID"], d["parent_ID"]))
        keys[k] = p._pkey
        s = router.streams.get(p._pkey)
        draws[k] = s.n if s is not None else 0
    return f, i, ids, keys, draws


def gen_showers(dict_dir, out_path, cases):
    refimport.setup()
    from PETITE.shower import Shower
    from PETITE.particle import Particle
    result = {}
    for name, target, cut, pid, E0, n, mass in cases:
        t0 = time.time()
        router = StreamRouter(SEED)
        shower = Shower(dict_dir, target, cut)
        wrap_shower(shower, router)
        saved = install(router)
        F, I, IDS, K, D = [], [], [], [], []
        try:
            for j in range(n):
                m = 0.0 if pid == 22 else mass
                p = math.sqrt(E0 * E0 - m * m)
                ids = {"PID": pid}
                part = Particle([E0, 0.0, 0.0, p], [0.0, 0.0, 0.0], ids)
                part._pkey = primary_key(j)
                parts = shower.generate_shower(part)
                f, i, ids_, k, d = shower_arrays(parts, router, j)
                F.append(f); I.append(i); K.append(k); D.append(d)
                IDS.extend(ids_)
        finally:
            uninstall(saved)
        F, I, K, D = np.concatenate(F), np.concatenate(I), np.concatenate(K), np.concatenate(D)
        result[f"{name}/f64"] = F
        result[f"{name}/i64"] = I
        result[f"{name}/pkey"] = K
        result[f"{name}/draws"] = D
        result[f"{name}/id_str"] = np.array([f"{a}:{b}" for a, b in IDS])
        result[f"{name}/meta"] = np.array([SEED, pid, n], np.int64)
        result[f"{name}/params"] = np.array([E0, cut, mass])
        result[f"{name}/target"] = np.array(target)
        print(f"{name}: {n} primaries, {len(F)} particles, {time.time() - t0:.1f} s")
    np.savez_compressed(out_path, **result)


def gen_units(dict_dir, out_path):
    """Known-answer vectors for the per-interaction functions."""
    refimport.setup()
    import PETITE.all_processes as proc
    from PETITE import kinematics as kin
    from PETITE import moliere
    from PETITE.particle import Particle
    from PETITE.shower import Shower
    from PETITE.physical_constants import m_electron, m_muon, alpha_em
    rng = np.random.default_rng(12345)
    out = {}
    # ---- differential cross sections at mapped points of the shipped maps
    sh = {t: Shower(dict_dir, t, 0.010) for t in ("graphite", "lead")}
    for t, s in sh.items():
        for pname in ("Brem", "PairProd", "Comp", "Ann", "Moller", "Bhabha", "MuonE", "MuonBrem"):
            rows = s._loaded_samples[pname]
            X, E, V, ROW = [], [], [], []
            for r in rng.choice(len(rows), size=12, replace=False):
                Erow, info = rows[r]
                amap = info["adaptive_map"]
                d = len(amap.grid)
                for _ in range(8):
                    Einc = float(Erow) * float(rng.uniform(0.9, 1.1))
                    x, _ = amap.map_one(rng.random(d))
                    ev = {'E_inc': Einc, 'm_e': m_electron, 'Z_T': s._ZTarget, 'A_T': s._ATarget,
                          'mT': s._ATarget, 'alpha_FS': alpha_em, 'mV': 0, 'Eg_min': s._Egamma_min,
                          'Ee_min': s._Ee_min}
                    if pname == "Brem":
                        ev["m_lepton"] = m_electron
                    if pname == "MuonBrem":
                        ev["m_lepton"] = m_muon
                    f = proc.__dict__[{"Brem": "dsigma_brem_dimensionless", "MuonBrem": "dsigma_brem_dimensionless",
                                       "PairProd": "dsigma_pairprod_dimensionless", "Comp": "dsigma_compton_dCT",
                                       "Ann": "dsigma_annihilation_dCT", "Moller": "dsigma_moller_dCT",
                                       "Bhabha": "dsigma_bhabha_dCT", "MuonE": "dsigma_muonelectron_dCT"}[pname]](ev, d)
                    with np.errstate(all="ignore"):
                        v = float(f(np.asarray(x)))
                    X.append(np.pad(x, (0, 4 - d))); E.append(Einc); V.append(v); ROW.append(r)
            out[f"dsigma/{t}/{pname}/x"] = np.array(X)
            out[f"dsigma/{t}/{pname}/E"] = np.array(E)
            out[f"dsigma/{t}/{pname}/value"] = np.array(V)
        # ---- mean free paths and branching inputs on a log grid
        Es = np.geomspace(1e-3, 120.0, 400)
        mf = np.array([[s.get_mfp([pid, e]) for e in Es] for pid in (11, -11, 22, 13)])
        out[f"mfp/{t}/E"] = Es
        out[f"mfp/{t}/value"] = mf
        ns = np.array([[float(fn(e)) for e in Es] for fn in (s._NSigmaBrem, s._NSigmaPP, s._NSigmaAnn, s._NSigmaComp,
                                                               s._NSigmaMoller, s._NSigmaBhabha, s._NSigmaMuonE,
                                                               s._NSigmaMuonBrem)])
        out[f"nsigma/{t}/value"] = ns
    # ---- kinematics with a fixed azimuth uniform
    router = StreamRouter(SEED)
    saved = install(router)
    try:
        K = []
        for case in range(200):
            kind = case % 6
            E = float(10 ** rng.uniform(-1.5, 2))
            router.set_current(10_000 + case)
            if kind == 0:
                part = Particle([E, 0, 0, math.sqrt(E * E - m_electron ** 2)], [0, 0, 0], {"PID": 11, "mass": m_electron})
                x = [rng.uniform(0, 0.999), rng.uniform(0, 0.01), rng.uniform(-0.01, 0.01), rng.uniform(0, 1)]
                a, b = kin.e_to_egamma_fourvecs(part, x)
            elif kind == 1:
                part = Particle([E, 0, 0, E], [0, 0, 0], {"PID": 22, "mass": 0.0})
                x = [rng.uniform(0.001, 0.999), rng.uniform(0, 0.01), rng.uniform(-0.01, 0.01), rng.uniform(0, 1)]
                a, b = kin.gamma_to_epem_fourvecs(part, x)
            elif kind == 2:
                part = Particle([E, 0, 0, E], [0, 0, 0], {"PID": 22, "mass": 0.0})
                x = [rng.uniform(-1, 1), 0, 0, 0]
                a, b = kin.compton_fourvecs(part, x)
            elif kind == 3:
                part = Particle([E, 0, 0, math.sqrt(E * E - m_electron ** 2)], [0, 0, 0], {"PID": -11, "mass": m_electron})
                x = [rng.uniform(-1, 0.99), 0, 0, 0]
                a, b = kin.annihilation_fourvecs(part, x)
            elif kind == 4:
                part = Particle([E, 0, 0, math.sqrt(E * E - m_electron ** 2)], [0, 0, 0], {"PID": 11, "mass": m_electron})
                x = [rng.uniform(-0.99, 0.99), 0, 0, 0]
                a, b = kin.ee_to_ee_fourvecs(part, x)
            else:
                E = E + 0.2
                part = Particle([E, 0, 0, math.sqrt(E * E - m_muon ** 2)], [0, 0, 0], {"PID": 13, "mass": m_muon})
                x = [rng.uniform(-1, 0.999), 0, 0, 0]
                a, b = kin.mue_to_mue_fourvecs(part, x)
            K.append(np.concatenate([[kind, E], x, a, b]))
        out["kin/rows"] = np.array(K)
        # ---- multiple scattering (moliere.py:350-400) with routed draws
        M = []
        for case in range(300):
            E = float(10 ** rng.uniform(-2, 2))
            m = m_muon if case % 5 == 4 else m_electron
            E = max(E, 1.5 * m)
            th, ph = rng.uniform(0, 0.5), rng.uniform(-math.pi, math.pi)
            pn = math.sqrt(E * E - m * m)
            p4 = np.array([E, pn * math.sin(th) * math.cos(ph), pn * math.sin(th) * math.sin(ph), pn * math.cos(th)])
            if case % 7 == 3:
                p4[1] = 0.0
            tt = float(10 ** rng.uniform(-4, 0))
            A, Z = (12, 6) if case % 2 else (207, 82)
            router.set_current(20_000 + case)
            r = moliere.get_scattered_momentum_fast(p4, tt, A, Z, 1, m_lepton=m)
            M.append(np.concatenate([[E, tt, A, Z, m], p4, r]))
        out["mcs/rows"] = np.array(M)
        # ---- Particle.rotation_matrix
        R = []
        for case in range(100):
            v = rng.normal(size=3)
            part = Particle([10.0, *v], [0, 0, 0], {"PID": 22, "mass": 0.0})
            R.append(np.concatenate([v, np.array(part.rotation_matrix()).ravel()]))
        out["rot/rows"] = np.array(R)
        # ---- draw_sample: returned x and proposal counts for a fixed stream
        s = sh["graphite"]
        D = []
        for case, (pname, E) in enumerate([(p, e) for p in ("Brem", "PairProd", "Comp", "Ann", "Moller", "Bhabha", "MuonE")
                                           for e in (0.05, 0.3, 1.0, 7.0, 60.0)]):
            if pname == "MuonE" and E < 0.3:
                continue
            router.set_current(30_000 + case)
            x = s.draw_sample(E, process=pname, VB=True)
            D.append(np.concatenate([[case, list(("Brem", "PairProd", "Comp", "Ann", "Moller", "Bhabha", "MuonE")).index(pname), E],
                                     np.pad(x[:-1], (0, 4 - (len(x) - 1))), [x[-1]]]))
        out["draw/rows"] = np.array(D)
    finally:
        uninstall(saved)
    np.savez_compressed(out_path, **out)
    print("units written", out_path)


DARK_PROCS = ["DarkBrem", "DarkAnn", "DarkComp", "DarkMuonBrem"]
V_PROC_CODE = {"DarkBrem": 0, "DarkAnn": 1, "DarkComp": 2, "DarkMuonBrem": 3,
               "DarkAnn_bound": 1, "DarkComp_bound": 2}


def gen_dark(dict_dir, out_path):
    """Dark-vector production: cross sections, kinematics, draw_dark_sample and
    generate_dark_shower on routed SM showers (dark_shower.py:595-849)."""
    refimport.setup()
    import PETITE.all_processes as proc
    from PETITE import kinematics as kin
    from PETITE.dark_shower import DarkShower
    from PETITE.particle import Particle
    from PETITE.physical_constants import m_electron, m_muon, alpha_em
    from oracle.dark import dark_key
    rng = np.random.default_rng(777)
    out = {}
    fns = {"DarkBrem": proc.dsig_dx_dcostheta_dark_brem_exact_tree_level,
           "DarkMuonBrem": proc.dsig_dx_dcostheta_dark_brem_exact_tree_level,
           "DarkComp": proc.dsigma_compton_dCT, "DarkAnn": proc.dsigma_radiative_return_du}
    showers = {}
    for mV in (0.01, 0.1, 0.3):
        for t in ("graphite", "lead"):
            ds = DarkShower(dict_dir, t, 0.010, mV, active_processes=list(DARK_PROCS))
            showers[(mV, t)] = ds
            for pname in DARK_PROCS:
                rows = ds._loaded_dark_samples[pname]
                X, E, V = [], [], []
                for r in rng.choice(len(rows), size=10, replace=False):
                    Erow, info = rows[r]
                    amap = info["adaptive_map"]
                    d = len(amap.grid)
                    for _ in range(6):
                        Einc = float(Erow) * float(rng.uniform(0.9, 1.1))
                        x, _ = amap.map_one(rng.random(d))
                        ev = {'E_inc': Einc, 'm_e': m_electron, 'Z_T': ds._ZTarget, 'A_T': ds._ATarget,
                              'mT': ds._ATarget, 'alpha_FS': alpha_em, 'mV': ds._mV, 'Eg_min': ds._Egamma_min,
                              'Zeff': ds.Zeff,
                              'm_lepton': m_muon if pname == "DarkMuonBrem" else m_electron}
                        with np.errstate(all="ignore"):
                            v = float(fns[pname](event_info=ev, ndim=d)(np.asarray(x)))
                        X.append(np.pad(x, (0, 3 - d))); E.append(Einc); V.append(v)
                out[f"dsigma/{mV}/{t}/{pname}/x"] = np.array(X)
                out[f"dsigma/{mV}/{t}/{pname}/E"] = np.array(E)
                out[f"dsigma/{mV}/{t}/{pname}/value"] = np.array(V)
    router = StreamRouter(SEED)
    saved = install(router)
    saved_d = install_dark(router)
    try:
        # ---- dark kinematics with routed azimuths
        K = []
        for case in range(120):
            kind = case % 5
            mV = (0.01, 0.1, 0.3)[case % 3]
            router.set_current(50_000 + case)
            if kind in (0, 1):
                m = m_electron if kind == 0 else m_muon
                E = float(10 ** rng.uniform(0, 2))
                part = Particle([E, 0, 0, math.sqrt(E * E - m * m)], [0, 0, 0], {"PID": 11 if kind == 0 else 13, "mass": m})
                x = [rng.uniform(mV / E * 1.01, 0.999), rng.uniform(-6, -0.5), 0.0]
                a, b = kin.l_to_lV_fourvecs(part, x, mV=mV)
                extra = [0.0, 0.0]
            elif kind == 2:
                E = float(10 ** rng.uniform(0, 2)) + mV ** 2 / (2 * m_electron) + mV
                part = Particle([E, 0, 0, E], [0, 0, 0], {"PID": 22, "mass": 0.0})
                x = [rng.uniform(-1, 1), 0.0, 0.0]
                a, b = kin.compton_fourvecs(part, x, mV=mV)
                extra = [0.0, 0.0]
            elif kind == 3:
                E = float(10 ** rng.uniform(0, 2)) + mV ** 2 / (2 * m_electron) + mV
                part = Particle([E, 0, 0, E], [0, 0, 0], {"PID": 22, "mass": 0.0})
                x = [rng.uniform(-1, 1), 0.0, 0.0]
                pe, cte = float(rng.uniform(0, 1e-3)), float(rng.uniform(-1, 1))
                a, b = kin.compton_fourvecs_boundelectron(part, x, mV=mV, Pe=pe, cte=cte)
                extra = [pe, cte]
            else:
                E = (mV ** 2 - 2 * m_electron ** 2) / (2 * m_electron) * float(rng.uniform(1.05, 3.0))
                part = Particle([E, 0, 0, math.sqrt(E * E - m_electron ** 2)], [0, 0, 0], {"PID": -11, "mass": m_electron})
                x = [rng.uniform(0.0, 0.999), 0.0, 0.0]
                a, b = kin.radiative_return_fourvecs(part, x, mV=mV)
                extra = [0.0, 0.0]
            K.append(np.concatenate([[kind, mV, E], x, extra, a, b]))
        out["kin/rows"] = np.array(K)
        # ---- draw_dark_sample (VB: x and proposal count) on fixed streams
        D = []
        ds = showers[(0.1, "graphite")]
        for case, (pname, E) in enumerate([(p, e) for p in DARK_PROCS for e in (0.5, 3.0, 20.0, 90.0)]):
            if pname in ("DarkAnn", "DarkComp") and E < 10.0:
                E = E + 10.0          # above the 0.1 GeV maps' first rows
            router.set_current(60_000 + case)
            x = ds.draw_dark_sample(E, process=pname, VB=True)
            D.append(np.concatenate([[case, DARK_PROCS.index(pname), E], np.pad(x[:-1], (0, 3 - (len(x) - 1))), [x[-1]]]))
        out["draw/rows"] = np.array(D)
        # ---- dark showers on routed SM showers
        for name, mV, t, pid, E0, n in (("e10_graphite_m0.1", 0.1, "graphite", 11, 10.0, 2),
                                        ("e10_graphite_m0.03", 0.03, "graphite", 11, 10.0, 2),
                                        ("g5_lead_m0.01", 0.01, "lead", 22, 5.0, 2)):
            ds = showers.get((mV, t)) or DarkShower(dict_dir, t, 0.010, mV, active_processes=list(DARK_PROCS))
            # a fresh router per case: streams restart at draw 0 for every key
            router.streams.clear()
            wrap_shower(ds, router)
            orig_pb = ds.produce_bsm_particle
            where = {}

            def pb(p_original, process, weight=None, VB=False, _orig=orig_pb, _where=where):
                router.set_current(dark_key(p_original._pkey, process))
                v = _orig(p_original, process, weight=weight, VB=VB)
                if v is not None:
                    _where[id(v)] = (id(p_original), process)
                return v

            ds.produce_bsm_particle = pb
            SMF, SMI, SMK, VV, WW = [], [], [], [], []
            t0 = time.time()
            for j in range(n):
                m = 0.0 if pid == 22 else 0.000511
                part = Particle([E0, 0.0, 0.0, math.sqrt(E0 * E0 - m * m)], [0.0, 0.0, 0.0], {"PID": pid})
                part._pkey = primary_key(j)
                sm = ds.generate_shower(part)
                f, i, _, k, _ = shower_arrays(sm, router, j)
                base = sum(len(x) for x in SMF)
                index = {id(p): base + r for r, p in enumerate(sm)}
                W = np.zeros((len(sm), len(DARK_PROCS)))
                for r, p in enumerate(sm):
                    for c, pc in enumerate(DARK_PROCS):
                        W[r, c] = ds.GetBSMWeights(p, pc)
                _, vs = ds.generate_dark_shower(ExDir=list(sm))
                for v in vs:
                    src, pc = where[id(v)]
                    d = v.get_ids()
                    VV.append(np.concatenate([[index[src], V_PROC_CODE[d["generation_process"]],
                                               DARK_PROCS.index(pc), d["weight"]], v.get_p0(), v.get_r0()]))
                SMF.append(f); SMI.append(i); SMK.append(k); WW.append(W)
            out[f"shower/{name}/sm_f64"] = np.concatenate(SMF)
            out[f"shower/{name}/sm_i64"] = np.concatenate(SMI)
            out[f"shower/{name}/sm_pkey"] = np.concatenate(SMK)
            out[f"shower/{name}/weights"] = np.concatenate(WW)
            out[f"shower/{name}/V"] = np.array(VV)
            out[f"shower/{name}/params"] = np.array([mV, E0, pid, n])
            out[f"shower/{name}/target"] = np.array(t)
            print(f"dark {name}: {len(out[f'shower/{name}/sm_f64'])} SM rows, {len(VV)} V, {time.time() - t0:.1f} s")
    finally:
        uninstall_dark(saved_d)
        uninstall(saved)
    np.savez_compressed(out_path, **out)
    print("dark golden written", out_path)


def install_bethe(router):
    """fast_MCS_mode=False draws its inverse-CDF uniform with random.random
    (moliere.py:132).  The reference's generate_moliere_angle passes
    m_lepton to get_chic_squared (moliere.py:244), which has no such
    parameter, so every call with b >= 2 raises TypeError; the wrapper drops
    the keyword (the function's momentum is the electron's by definition).
    Nothing else is changed."""
    from PETITE import moliere
    saved = dict(rrandom=random.random, chic=moliere.get_chic_squared)
    orig = moliere.get_chic_squared

    def chic(t, beta, A, Z, z, m_lepton=None):
        return orig(t, beta, A, Z, z)

    random.random = router.u
    moliere.get_chic_squared = chic
    return saved


def uninstall_bethe(saved):
    from PETITE import moliere
    random.random = saved["rrandom"]
    moliere.get_chic_squared = saved["chic"]


def gen_moliere(dict_dir, out_path):
    """Bethe-Moliere multiple scattering (fast_MCS_mode=False): its pieces,
    the routed get_scattered_momentum_Bethe, and showers in that mode."""
    refimport.setup()
    from PETITE import moliere
    from PETITE.shower import Shower
    from PETITE.particle import Particle
    rng = np.random.default_rng(777)
    out = {}
    targets = {"graphite": (6, 12), "lead": (82, 207), "iron": (26, 56)}
    # b, B and chi_c^2 over thickness and velocity
    rows = []
    for tname, (Z, A) in targets.items():
        for t in np.logspace(-4, 1.5, 12):
            for beta in (0.3, 0.8, 0.99, 0.99999, 1 - 1e-9):
                b = moliere.get_b(t, beta, A, Z, 1.)
                B = moliere.get_capital_B(t, beta, A, Z, 1.) if b >= 2 else np.nan
                chic2 = moliere.get_chic_squared(t, beta, A, Z, 1.)
                rows.append([Z, A, t, beta, b, B, chic2])
    out["params/rows"] = np.array(rows)
    # inverse CDF: uniform u, the far tail, both explicit branches and the
    # step of the piecewise CDF at x = 0.01
    rows = []
    for B in (3.15, 3.6, 4.5, 6.0, 8.0, 11.0, 15.0, 20.0):
        f00 = moliere.moliere_f(0, B)
        band = (moliere.moliere_cdf(0.0100000000001, B), 0.01 * f00)
        us = np.concatenate([rng.uniform(0, 1, 40), 1 - 10 ** rng.uniform(-7, -1, 12),
                             rng.uniform(0.005, 0.0125, 8), np.linspace(band[0], band[1], 4)[1:-1],
                             [0.0, 0.5, 1 - 1 / B / 100 * 1.0001]])
        for u in us:
            rows.append([B, u, moliere.inverse_moliere_cdf(u, B), float(band[0] < u < band[1])])
    out["icdf/rows"] = np.array(rows)
    # get_scattered_momentum_Bethe on fixed streams
    router = StreamRouter(SEED)
    saved = install(router)
    saved_b = install_bethe(router)
    rows = []
    try:
        case = 0
        for tname, (Z, A) in targets.items():
            for t in (3e-4, 1e-3, 4e-3, 0.03, 0.3, 3.0):
                for E, m in ((0.02, 0.000511), (1.0, 0.000511), (30.0, 0.000511), (2.0, 0.1056583755)):
                    d = rng.normal(size=3)
                    d /= np.linalg.norm(d)
                    pn = math.sqrt(E * E - m * m)
                    p4 = np.array([E, *(pn * d)])
                    router.set_current(70_000 + case)
                    outp = moliere.get_scattered_momentum_Bethe(p4, t, A, Z, 1.0, m_lepton=m)
                    rows.append([E, t, A, Z, m, *p4, *outp, router.cur.n])
                    case += 1
    finally:
        uninstall_bethe(saved_b)
        uninstall(saved)
    out["scatter/rows"] = np.array(rows)
    # showers with fast_MCS_mode=False
    for name, target, cut, pid, E0, n, mass in BETHE_CASES:
        t0 = time.time()
        router = StreamRouter(SEED)
        shower = Shower(dict_dir, target, cut, fast_MCS_mode=False)
        wrap_shower(shower, router)
        saved = install(router)
        saved_b = install_bethe(router)
        F, I, K, D = [], [], [], []
        try:
            for j in range(n):
                m = 0.0 if pid == 22 else mass
                part = Particle([E0, 0.0, 0.0, math.sqrt(E0 * E0 - m * m)], [0.0, 0.0, 0.0], {"PID": pid})
                part._pkey = primary_key(j)
                f, i, _, k, d = shower_arrays(shower.generate_shower(part), router, j)
                F.append(f); I.append(i); K.append(k); D.append(d)
        finally:
            uninstall_bethe(saved_b)
            uninstall(saved)
        out[f"shower/{name}/f64"] = np.concatenate(F)
        out[f"shower/{name}/i64"] = np.concatenate(I)
        out[f"shower/{name}/pkey"] = np.concatenate(K)
        out[f"shower/{name}/draws"] = np.concatenate(D)
        out[f"shower/{name}/meta"] = np.array([SEED, pid, n], np.int64)
        out[f"shower/{name}/params"] = np.array([E0, cut, mass])
        out[f"shower/{name}/target"] = np.array(target)
        print(f"bethe {name}: {n} primaries, {sum(len(x) for x in F)} particles, {time.time() - t0:.1f} s")
    np.savez_compressed(out_path, **out)


def gen_mesons(dict_dir, out_path, beam_path):
    """TwoBody_BSMDecay (dark_shower.py:633-638,836-844; particle.py:209-256):
    generate_dark_shower on lists of pi0s from the reference's own beam file
    (examples/beams, four-momenta) mixed with SM particles, with the decay's
    np.random.uniform draws routed to the decaying particle's stream; and the
    KeyError the reference raises for an eta."""
    refimport.setup()
    from PETITE.dark_shower import DarkShower
    from PETITE.particle import Particle
    from oracle.dark import dark_key
    beam = np.load(beam_path)[:40]
    out = {"beam/p4": beam}
    router = StreamRouter(SEED)
    saved = install(router)
    saved_d = install_dark(router)
    orig_tbd = Particle.two_body_decay

    def tbd(self, p1_dict, p2_dict, angular_information="Isotropic"):
        router.set_current(dark_key(self._pkey, "TwoBody_BSMDecay"))
        return orig_tbd(self, p1_dict, p2_dict, angular_information)

    Particle.two_body_decay = tbd
    # set_dark_samples (dark_shower.py:196-201) loads a map entry for every
    # active process, TwoBody_BSMDecay included, which is never sampled; the
    # rebuilt dark_maps.pkl holds the four sampled processes only
    orig_lds = DarkShower.load_dark_sample

    def lds(self, dict_dir, process):
        return [] if process == "TwoBody_BSMDecay" else orig_lds(self, dict_dir, process)

    DarkShower.load_dark_sample = lds
    try:
        for mV in (0.01, 0.03, 0.1, 0.3):
            router.streams.clear()
            ds = DarkShower(dict_dir, "graphite", 0.010, mV)
            orig_pb = ds.produce_bsm_particle

            def pb(p_original, process, weight=None, VB=False, _orig=orig_pb):
                router.set_current(dark_key(p_original._pkey, process))
                return _orig(p_original, process, weight=weight, VB=VB)

            ds.produce_bsm_particle = pb
            parts = []
            for j, p4 in enumerate(beam):
                part = Particle(list(p4), [0.0, 0.0, 0.01 * j], {"PID": 111, "weight": 1.0 / len(beam), "ID": j + 1})
                part._pkey = primary_key(j)
                parts.append(part)
                if j % 13 == 5:          # SM particles in between
                    sm = Particle([3.0 + j, 0.0, 0.0, 3.0 + j], [0.0, 0.0, 0.0], {"PID": 22, "ID": 100 + j})
                    sm._pkey = primary_key(1000 + j)
                    parts.append(sm)
            _, vs = ds.generate_dark_shower(ExDir=list(parts))
            index = {id(p): k for k, p in enumerate(parts)}
            rows = []
            for v in vs:
                d = v.get_ids()
                src = next(k for k, p in enumerate(parts) if p.get_ids()["ID"] == d["parent_ID"]
                           and p.get_ids()["PID"] == d["parent_PID"])
                rows.append([src, V_PROC_CODE.get(d["generation_process"], 8), d["weight"], *v.get_p0(),
                             *v.get_r0(), d["ID"], d["parent_ID"], d["mass"] if d["mass"] is not None else -1.0])
            out[f"m{mV}/V"] = np.array(rows).reshape(-1, 13)
            out[f"m{mV}/parts_f64"] = np.array([[*p.get_p0(), *p.get_r0(), p.get_ids()["weight"],
                                                  p.get_ids()["mass"]] for p in parts])
            out[f"m{mV}/parts_i64"] = np.array([[p.get_ids()["PID"], p.get_ids()["ID"]] for p in parts])
            out[f"m{mV}/parts_pkey"] = np.array([p._pkey for p in parts], np.uint64)
            out[f"m{mV}/weights"] = np.array([ds.GetBSMWeights(p, "TwoBody_BSMDecay") for p in parts])
            print(f"mesons mV={mV}: {len(parts)} inputs, {len(vs)} V")
        eta = Particle([5.0, 0.0, 0.0, math.sqrt(25.0 - 0.547862 ** 2)], [0, 0, 0], {"PID": 221})
        eta._pkey = primary_key(7)
        try:
            ds.generate_dark_shower(ExDir=[eta])
            out["eta/raises"] = np.array(0)
        except KeyError:
            out["eta/raises"] = np.array(1)
    finally:
        Particle.two_body_decay = orig_tbd
        DarkShower.load_dark_sample = orig_lds
        uninstall_dark(saved_d)
        uninstall(saved)
    np.savez_compressed(out_path, **out)


def gen_dark_free(dict_dir, out_path):
    """DarkShower(bound_electron=False): GetBSMWeights of DarkAnn (with the
    closed-form resonant part, dark_shower.py:619-630) and DarkComp over
    energy, and generate_dark_shower on routed SM showers.  Each shower is
    built in a private directory without dark_weights.pkl and
    dark_drate.pkl: with a cached entry for its mass and target,
    set_drate_dE raises TypeError in this mode (dark_shower.py:550)."""
    import shutil
    import tempfile
    refimport.setup()
    from PETITE.dark_shower import DarkShower
    from PETITE.particle import Particle
    from oracle.dark import dark_key
    out = {}
    router = StreamRouter(SEED)
    saved = install(router)
    saved_d = install_dark(router)
    try:
        for name, mV, t, pid, E0, n in (("e10_graphite_m0.01", 0.01, "graphite", 11, 10.0, 2),
                                        ("e5_lead_m0.03", 0.03, "lead", 11, 5.0, 2),
                                        ("g5_lead_m0.01", 0.01, "lead", 22, 5.0, 2)):
            work = tempfile.mkdtemp(prefix="darkfree_")
            for f in os.listdir(dict_dir):
                if f not in ("dark_weights.pkl", "dark_drate.pkl"):
                    os.symlink(os.path.realpath(os.path.join(dict_dir, f)), os.path.join(work, f))
            ds = DarkShower(work + "/", t, 0.010, mV, active_processes=list(DARK_PROCS), bound_electron=False)
            shutil.rmtree(work, ignore_errors=True)
            E_res = ds._resonant_annihilation_energy
            Es = np.concatenate([E_res * np.array([0.999, 1.0, 1.0 + 1e-6, 1.0001, 1.001, 1.01]),
                                 np.geomspace(E_res * 1.02, 100.0, 30)])
            out[f"{name}/ann_weights"] = np.c_[Es, [ds.GetBSMWeights([-11, e], "DarkAnn") for e in Es]]
            Ec = np.geomspace(1e-3, 100.0, 40)
            out[f"{name}/comp_weights"] = np.c_[Ec, [ds.GetBSMWeights([22, e], "DarkComp") for e in Ec]]
            router.streams.clear()
            wrap_shower(ds, router)
            orig_pb = ds.produce_bsm_particle
            where = {}

            def pb(p_original, process, weight=None, VB=False, _orig=orig_pb, _where=where):
                router.set_current(dark_key(p_original._pkey, process))
                v = _orig(p_original, process, weight=weight, VB=VB)
                if v is not None:
                    _where[id(v)] = (id(p_original), process)
                return v

            ds.produce_bsm_particle = pb
            SMF, SMI, SMK, VV = [], [], [], []
            for j in range(n):
                m = 0.0 if pid == 22 else 0.000511
                part = Particle([E0, 0.0, 0.0, math.sqrt(E0 * E0 - m * m)], [0.0, 0.0, 0.0], {"PID": pid})
                part._pkey = primary_key(j)
                sm = ds.generate_shower(part)
                f, i, _, k, _ = shower_arrays(sm, router, j)
                base = sum(len(x) for x in SMF)
                index = {id(p): base + r for r, p in enumerate(sm)}
                _, vs = ds.generate_dark_shower(ExDir=list(sm))
                for v in vs:
                    src, pc = where[id(v)]
                    d = v.get_ids()
                    VV.append(np.concatenate([[index[src], V_PROC_CODE[d["generation_process"]],
                                               DARK_PROCS.index(pc), d["weight"]], v.get_p0(), v.get_r0()]))
                SMF.append(f); SMI.append(i); SMK.append(k)
            out[f"{name}/sm_f64"] = np.concatenate(SMF)
            out[f"{name}/sm_i64"] = np.concatenate(SMI)
            out[f"{name}/sm_pkey"] = np.concatenate(SMK)
            out[f"{name}/V"] = np.array(VV).reshape(-1, 11)
            out[f"{name}/params"] = np.array([mV, E0, pid, n])
            out[f"{name}/target"] = np.array(t)
            procs = np.array(VV).reshape(-1, 11)[:, 2] if VV else np.array([])
            print(f"dark free {name}: {len(out[f'{name}/sm_f64'])} SM rows, {len(VV)} V, "
                  f"per process {np.bincount(procs.astype(int), minlength=4) if len(procs) else []}")
    finally:
        uninstall_dark(saved_d)
        uninstall(saved)
    np.savez_compressed(out_path, **out)


def gen_files(dict_dir, out_dir):
    """A shower file as PETITE writes it (np.save of its Particle objects,
    which generate_dark_shower(ExDir=path) reads), with its content as plain
    arrays for the test."""
    refimport.setup()
    from PETITE.shower import Shower
    from PETITE.particle import Particle
    router = StreamRouter(SEED)
    saved = install(router)
    try:
        sh = Shower(dict_dir, "graphite", 0.010)
        wrap_shower(sh, router)
        part = Particle([2.0, 0.0, 0.0, math.sqrt(4.0 - 0.000511 ** 2)], [0.0, 0.0, 0.0], {"PID": 11})
        part._pkey = primary_key(0)
        parts = sh.generate_shower(part)
    finally:
        uninstall(saved)
    for p in parts:                                  # the routing key is not part of PETITE's objects
        del p._pkey
    np.save(os.path.join(out_dir, "petite_shower_file.npy"), np.array(parts, dtype=object), allow_pickle=True)
    keys = ("PID", "ID", "parent_PID", "parent_ID", "generation_number", "weight", "mass")
    np.savez_compressed(os.path.join(out_dir, "petite_shower_file_content.npz"),
                        p0=np.array([p.get_p0() for p in parts]), r0=np.array([p.get_r0() for p in parts]),
                        pf=np.array([p.get_pf() for p in parts]), rf=np.array([p.get_rf() for p in parts]),
                        ids=np.array([[p.get_ids()[k] for k in keys] for p in parts], dtype=np.float64),
                        process=np.array([p.get_ids()["generation_process"] for p in parts]),
                        ended=np.array([p.get_ended() for p in parts]))
    print("shower file:", len(parts), "particles")


def gen_particles(out_path):
    """PETITE's Particle utilities on a seeded numpy generator: boost,
    two- and three-body decays, the meson decay chain (short- and
    long-lived), decay/interaction sampling, energy loss, detector_cut."""
    refimport.setup()
    from PETITE.particle import Particle
    from PETITE import shower as shmod
    rng = np.random.default_rng(91)
    out = {}
    rows = []
    for case in range(40):
        pid = [111, 221, 331, 223, 211, -211, 321][case % 7]
        m = {111: 0.1349768, 221: 0.547862, 331: 0.95778, 223: 0.78265, 211: 0.13957039, -211: 0.13957039,
             321: 0.493677}[pid]
        E = m * float(1.0 + 10 ** rng.uniform(-2, 2))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        pm = math.sqrt(E * E - m * m)
        p4 = [E, *(pm * d)]
        seed = 1000 + case
        # two-body (gamma + V, V of mass 0.01..0.5 m) and the boost
        par = Particle(list(p4), [0.0, 0.0, 0.1 * case], {"PID": pid, "mass": m, "ID": 3 + case})
        np.random.seed(seed)
        mv = m * float(rng.uniform(0.01, 0.5))
        a, b = par.two_body_decay({"mass": 0, "PID": 22}, {"mass": mv, "PID": 4900022})
        L = np.array(par.boost_matrix())
        # three-body (pi0 pi0 + light) where allowed
        t3 = np.zeros(12)
        if m > 3 * 0.1349768:
            np.random.seed(seed + 1)
            x = par.three_body_decay({"PID": 22, "mass": 0.0}, {"PID": 22, "mass": 0.0}, {"PID": 111})
            t3 = np.concatenate([q.get_p0() for q in x])
        # decay chain
        ch = np.full(12, np.nan)
        st = "short-lived" if pid in (111, 221, 331, 223) else "long-lived"
        q = Particle(list(p4), [0.0, 0.0, 0.0], {"PID": pid, "mass": m, "ID": 5, "stability": st, "weight": 0.5})
        np.random.seed(seed + 2)
        try:
            dd = q.decay_particle()
            ch = np.concatenate([dd[0].get_p0(), dd[1].get_p0(), [dd[0].get_ids()["weight"], dd[1].get_ids()["weight"],
                                 dd[0].get_ids()["PID"], dd[1].get_ids()["PID"]]])
        except ValueError:
            pass
        rows.append(np.concatenate([[pid, m, seed, mv], p4, a.get_p0(), b.get_p0(), L.ravel(), t3, ch,
                                    q.get_rf()]))
    out["decays"] = np.array(rows)
    # lose_energy
    le = []
    for case in range(20):
        m = [0.000511, 0.1056583755, 0.1349768][case % 3]
        E = m + float(10 ** rng.uniform(-3, 1))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        par = Particle([E, *(math.sqrt(E * E - m * m) * d)], [0, 0, 0], {"PID": 11, "mass": m})
        dE = float(rng.uniform(0, 1.2)) * (E - m)
        par.lose_energy(dE)
        le.append(np.concatenate([[m, E, dE], d, par.get_pf()]))
    out["lose"] = np.array(le)
    # detector_cut on V-like particles
    parts = []
    for k in range(300):
        E = float(10 ** rng.uniform(-1, 1.5))
        th = float(10 ** rng.uniform(-4, -0.5))
        ph = float(rng.uniform(0, 2 * math.pi))
        p4 = [E, E * math.sin(th) * math.cos(ph), E * math.sin(th) * math.sin(ph), E * math.cos(th)]
        parts.append(Particle(p4, [float(rng.normal(0, 0.01)), float(rng.normal(0, 0.01)), float(rng.uniform(0, 1))],
                              {"PID": 4900022, "weight": float(rng.uniform(0.1, 2.0)), "mass": 0.01}))
    out["det/p0"] = np.array([p.get_p0() for p in parts])
    out["det/r0"] = np.array([p.get_r0() for p in parts])
    out["det/w"] = np.array([p.get_ids()["weight"] for p in parts])
    zs, R = [5.0, 50.0, 100.0], 1.0
    out["det/sampleW"] = np.asarray(shmod.detector_cut(parts, zs, R, method="SampleW"), bool)
    out["det/eff"] = np.array(shmod.detector_cut(parts, zs, R, method="Efficiency", energy_cut=(1.0, 20.0),
                                                 detector_inner_radius=0.05))
    out["det/total"] = np.array(shmod.detector_cut(parts, zs, R, method="TotalWeight"))
    np.savez_compressed(out_path, **out)
    print("particle utilities:", len(rows), "decay cases")


BETHE_CASES = [
    ("e1gev_graphite", "graphite", 0.010, 11, 1.0, 6, 0.000511),
    ("pos3_lead", "lead", 0.010, -11, 3.0, 2, 0.000511),
    ("mu5_graphite", "graphite", 0.010, 13, 5.0, 2, 0.1056583755),
]

def gen_ranges(path):
    """PETITE's integration_range (all_processes.py:1102-1160) for the
    processes the table builder trains, at several energies and masses."""
    refimport.setup()
    import PETITE.all_processes as proc
    rows = []
    for p in ("PairProd", "Brem", "MuonBrem", "Comp", "Ann", "Moller", "Bhabha", "MuonE",
              "DarkBrem", "DarkMuonBrem", "DarkComp", "DarkAnn"):
        for E in (0.01, 0.3, 7.0, 350.0):
            for mV in ((0.0,) if not p.startswith("Dark") else (0.003, 0.05, 0.3)):
                ev = {"E_inc": E, "mV": mV, "Eg_min": 0.001, "Ee_min": 0.005}
                r = np.asarray(proc.integration_range(ev, p), float).ravel()
                rows.append((p, E, mV, np.pad(r, (0, 8 - len(r)), constant_values=np.nan)))
    np.savez_compressed(path, process=np.array([r[0] for r in rows]), E=np.array([r[1] for r in rows]),
                        mV=np.array([r[2] for r in rows]), ranges=np.array([r[3] for r in rows]))


def gen_findmax(path, seed=20261206):
    """PETITE's do_find_max_work (utilities/find_maxes.py:56-115, unmodified)
    on a few shipped map rows, neval 300, 3 trials, graphite and lead, with
    the VEGAS shim drawing from numpy's default_rng(seed + row): max_F and
    the cross section per target, and the rows' grids.  Pins
    oracle.vegas_train.find_maxes_row."""
    refimport.setup()
    import vegas
    import find_maxes as fm
    out = {"seed": np.array(seed)}
    for proc, rows in (("Comp", (5, 40, 90)), ("Brem", (10, 60))):
        arr = np.load(os.path.join(refimport.REFERENCE, "data", proc, f"{proc}_AdaptiveMaps.npy"), allow_pickle=True)
        for r in rows:
            event_info, amap = arr[r]
            vegas.UNIFORM = np.random.default_rng(seed + r).random
            params = {"process_targets": ["graphite", "lead"], "neval": 300, "n_trials": 3,
                      "diff_xsec": fm.process_info[proc]["diff_xsection"]}
            samp, xsec, E = fm.do_find_max_work(params, [event_info, amap])
            pre = f"{proc}/{r}"
            out[f"{pre}/E"] = np.array(float(E))
            for d, g in enumerate(amap.grid):
                out[f"{pre}/grid{d}"] = np.asarray(g, float)
            out[f"{pre}/max_F"] = np.array([samp[1]["max_F"][t] for t in ("graphite", "lead")])
            out[f"{pre}/xsec"] = np.array([xsec[t] for t in ("graphite", "lead")])
            out[f"{pre}/Eg_min"] = np.array(event_info["Eg_min"])
            out[f"{pre}/Ee_min"] = np.array(event_info["Ee_min"])
    vegas.UNIFORM = np.random.random
    np.savez_compressed(path, **out)


def gen_dark_xsec_400(path, mV=0.1, every=15):
    """Rows of data_400GeV/dark_xsec.pkl (find_maxes' cross sections with
    PETITE's own DarkBrem/DarkMuonBrem maps, which it does not ship): the
    anchor for maps trained by petite_gb300.train."""
    import pickle
    with open(os.path.join(refimport.REFERENCE, "data_400GeV", "dark_xsec.pkl"), "rb") as f:
        dx = pickle.load(f)
    key = [k for k in dx if abs(float(k) - mV) < 1e-12][0]
    out = {"mV": np.array(mV)}
    for p in ("DarkBrem", "DarkMuonBrem"):
        for t in ("lead", "graphite"):
            out[f"{p}/{t}"] = np.asarray(dx[key][p][t], float)[::every]
    np.savez_compressed(path, **out)


CASES = [
    # name, target, cut, pid, E0, n primaries, primary mass for the momentum
    ("e1gev_graphite", "graphite", 0.010, 11, 1.0, 12, 0.000511),
    ("gamma10_lead", "lead", 0.010, 22, 10.0, 2, 0.0),
    ("pos3_lead", "lead", 0.010, -11, 3.0, 4, 0.000511),
    ("mu5_graphite", "graphite", 0.010, 13, 5.0, 4, 0.1056583755),
]

if __name__ == "__main__":
    d = sys.argv[1].rstrip("/") + "/"
    which = sys.argv[2] if len(sys.argv) > 2 else "all"
    if which in ("all", "units"):
        gen_units(d, os.path.join(HERE, "units.npz"))
    if which in ("all", "showers"):
        gen_showers(d, os.path.join(HERE, "showers.npz"), CASES)
    if which in ("all", "dark"):
        gen_dark(d, os.path.join(HERE, "dark.npz"))
    if which in ("all", "moliere"):
        gen_moliere(d, os.path.join(HERE, "moliere.npz"))
    if which in ("all", "darkfree"):
        gen_dark_free(d, os.path.join(HERE, "dark_free.npz"))
    if which in ("all", "ranges"):
        gen_ranges(os.path.join(HERE, "ranges.npz"))
    if which in ("all", "findmax"):
        gen_findmax(os.path.join(HERE, "findmax.npz"))
    if which in ("all", "darkxsec400"):
        gen_dark_xsec_400(os.path.join(HERE, "dark_xsec_400GeV.npz"))
    if which in ("all", "particles"):
        gen_particles(os.path.join(HERE, "particles.npz"))
    if which in ("all", "files"):
        gen_files(d, HERE)
    if which in ("all", "mesons"):
        gen_mesons(d, os.path.join(HERE, "mesons.npz"),
                   os.path.join(refimport.REFERENCE, "examples", "beams", "Pi0_8GeVProtons_1000POT.npy"))
