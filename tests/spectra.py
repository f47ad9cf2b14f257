"""Shower observables shared by the spectrum fixture generator
(``tests/golden/make_spectra.py``) and the independent-stream GPU test
(``tests/test_gpu_spectra.py``).

The batched engine tallies three per-particle histograms per species
(``pt_tally.hist``: log10 of the creation energy in [-2, 2], log10 of the
polar angle of p0 in [-6, 0.5], depth z of the interaction point in
[0, z_max]; 100 bins each) and, per shower, the particle count and the
deposited energy.  The CPU showers are binned here the same way (float32
arithmetic, as the kernels bin), then merged into coarse bins of
``COARSE`` fine bins for the comparisons.

Particles of one shower are correlated, so a per-particle histogram is not a
multinomial sample and a plain Pearson chi-square would overstate its
significance.  The comparison therefore treats the shower as the independent
unit: the statistic is Hotelling's T^2 of the difference of the per-shower
mean histograms, with the per-shower covariance estimated from the CPU
showers, whose histograms are stored one per shower.
"""
from __future__ import annotations

import math

import numpy as np

HIST_BINS = 100
COARSE = 5
NCOARSE = HIST_BINS // COARSE
RANGES = ((-2.0, 2.0), (-6.0, 0.5))          # kinds 0 and 1; kind 2 is [0, z_max]
SPECIES = (22, 11, -11)                       # species slots 0..2 of the tally (3 = muon, unused here)


def _bins(v, lo, hi):
    v = np.asarray(v, np.float32)
    b = ((v - np.float32(lo)) / np.float32(hi - lo) * np.float32(HIST_BINS))
    b = np.where(np.isfinite(b), b, -1.0).astype(np.int64)
    return np.clip(b, 0, HIST_BINS - 1)


def fine_bins(E0, px, py, pz, z, z_max):
    """Fine-bin indices of the three tallies for particles (arrays)."""
    E0 = np.asarray(E0, np.float32)
    px, py, pz = (np.asarray(a, np.float32) for a in (px, py, pz))
    b0 = _bins(np.log10(E0), *RANGES[0])
    pt = np.sqrt(px * px + py * py)
    th = np.arctan2(pt, pz).astype(np.float32)
    with np.errstate(divide="ignore"):
        lth = np.where(th > 0, np.log10(np.maximum(th, np.float32(1e-38))), np.float32(-6.0))
    b1 = _bins(lth, *RANGES[1])
    b2 = _bins(z, 0.0, z_max)
    return b0, b1, b2


def species_slot(pid):
    pid = np.asarray(pid)
    return np.where(pid == 22, 0, np.where(pid == 11, 1, np.where(pid == -11, 2, 3)))


def coarse_shower_hist(pid, E0, px, py, pz, z, z_max):
    """[3 kinds][3 species][NCOARSE] counts of one shower's particles."""
    h = np.zeros((3, 3, NCOARSE), np.int64)
    sp = species_slot(pid)
    keep = sp < 3
    for k, b in enumerate(fine_bins(E0, px, py, pz, z, z_max)):
        np.add.at(h[k], (sp[keep], b[keep] // COARSE), 1)
    return h


def coarse_tally_hist(hist):
    """The GPU tally's [3][4][100] histogram in the same coarse layout."""
    h = np.asarray(hist, np.int64)[:, :3, :]
    return h.reshape(3, 3, NCOARSE, COARSE).sum(axis=-1)


def hotelling(mean_a, n_a, hist_b, min_count=25.0, rel_eig=1e-3):
    """Two-sample test of the per-shower mean histogram, for independent
    samples drawn from one primary distribution.

    mean_a: [d] mean counts per shower of sample A (n_a showers, e.g. the GPU
    tally divided by its primaries); hist_b: [n_b, d] per-shower counts of
    sample B.  Under the null both samples share the per-shower covariance C,
    estimated from B; the difference of means has covariance
    C (1/n_a + 1/n_b).  Returns (T2, dof, p); see ``_t2``."""
    hist_b = np.asarray(hist_b, np.float64)
    n_b = hist_b.shape[0]
    keep = hist_b.sum(axis=0) >= min_count
    B = hist_b[:, keep]
    C = np.atleast_2d(np.cov(B, rowvar=False)) * (1.0 / n_a + 1.0 / n_b)
    return _t2(np.asarray(mean_a, np.float64)[keep] - B.mean(axis=0), C, n_b, rel_eig)


def hotelling_paired(mean_a, replicas, hist_b, pid, E0, min_count=25.0, rel_eig=1e-3):
    """Two-sample test of the per-shower mean histogram when sample A holds
    ``replicas`` showers (independent streams) of each primary of sample B.

    The spread of the primaries' energies then cancels from the difference:
    it has covariance (1 + 1/replicas) / N^2 * sum_s C_s, with C_s the
    covariance of shower s's histogram at its own energy and species.  That
    sum is estimated from B by successive differences: sorted by species and
    energy, neighbouring showers have nearly equal primaries, and
    E[(h_j+1 - h_j)(h_j+1 - h_j)^T] = C_j+1 + C_j (plus the square of the
    small change of the mean between neighbours, which only makes the test
    conservative).  Returns (T2, dof, p); see ``_t2``."""
    hist_b = np.asarray(hist_b, np.float64)
    n = hist_b.shape[0]
    keep = hist_b.sum(axis=0) >= min_count
    order = np.lexsort((np.asarray(E0), np.asarray(pid)))
    H = hist_b[order][:, keep]
    P = np.asarray(pid)[order]
    dH = (H[1:] - H[:-1])[P[1:] == P[:-1]]
    C_mean = dH.T @ dH / (2.0 * len(dH))                 # mean over showers of C_s
    C = np.atleast_2d(C_mean) * (1.0 + 1.0 / replicas) / n
    return _t2(np.asarray(mean_a, np.float64)[keep] - H.mean(axis=0), C, len(dH), rel_eig)


def _t2(d, C, n_est, rel_eig):
    """Hotelling's T^2 of the difference d with covariance C estimated from
    n_est vectors; p from the F form.  Directions of C whose variance is below
    ``rel_eig`` of the largest are dropped: they are estimated from the few
    showers that reach them, and with them the statistic overstates
    significance (on random half-splits of the CPU sample of the lead mix, a
    fifth of the splits gave p < 0.01 with 1e-9; with 1e-3 the p-values are
    uniform or conservative)."""
    from scipy import stats
    w, V = np.linalg.eigh(C)
    if w.max() <= 0:
        return 0.0, 0, 1.0
    good = w > rel_eig * w.max()
    proj = V[:, good].T @ d
    t2 = float(np.sum(proj ** 2 / w[good]))
    p_dim = int(good.sum())
    f = t2 * (n_est - p_dim) / (p_dim * (n_est - 1))
    return t2, p_dim, float(stats.f.sf(f, p_dim, n_est - p_dim))


def ks(a, b):
    from scipy import stats
    r = stats.ks_2samp(np.asarray(a, np.float64), np.asarray(b, np.float64))
    return float(r.statistic), float(r.pvalue)


def chi2_binned(a, b, nbins=20):
    """Two-sample binned chi^2 (homogeneity of the two histograms), bins at
    quantiles of the pooled sample: (statistic, dof, p)."""
    from scipy import stats
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    edges = np.unique(np.quantile(np.concatenate([a, b]), np.linspace(0, 1, nbins + 1)))
    edges[-1] = np.nextafter(edges[-1], np.inf)
    ha, _ = np.histogram(a, edges)
    hb, _ = np.histogram(b, edges)
    keep = (ha + hb) > 0
    stat, p, dof, _ = stats.chi2_contingency(np.vstack([ha[keep], hb[keep]]))
    return float(stat), int(dof), float(p)


def mean_and_error(x):
    x = np.asarray(x, np.float64)
    return float(x.mean()), float(x.std(ddof=1) / math.sqrt(len(x)))


# The two workloads of the independent-stream comparison: 1 GeV electrons in
# graphite (the plain SM shower), and the batched mix of e-, e+ and photons,
# log-uniform in [0.1, 100] GeV, in lead.  The GPU transports ``replicas``
# showers of each CPU primary, all on streams independent of the CPU's
# (another Philox seed, and other stream indices).
CONFIGS = {
    "e1_graphite": dict(target="graphite", species=(11,), E=(1.0, 1.0), z_max=3.0, n=4000, replicas=10,
                        prim_seed=101, cpu_seed=1000, gpu_seed=0),
    "mix_lead": dict(target="lead", species=(11, -11, 22), E=(0.1, 100.0), z_max=0.3, n=2000, replicas=10,
                     prim_seed=102, cpu_seed=1001, gpu_seed=1),
}
MIN_ENERGY = 0.010


def primaries(cfg):
    """(p0 [n,4], pid [n], mass [n]) of a workload's primaries."""
    n = cfg["n"]
    rng = np.random.default_rng(cfg["prim_seed"])
    sp = np.asarray(cfg["species"])
    pid = sp[rng.integers(0, len(sp), n)].astype(np.int32)
    lo, hi = cfg["E"]
    E = 10 ** rng.uniform(math.log10(lo), math.log10(hi), n) if hi > lo else np.full(n, lo)
    m = np.where(np.abs(pid) == 11, 0.000511, 0.0)
    p0 = np.c_[E, np.zeros(n), np.zeros(n), np.sqrt(E * E - m * m)]
    return p0, pid, m
