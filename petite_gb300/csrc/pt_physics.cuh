// pt_physics.cuh -- per-interaction physics of PETITE's SM shower, float64.
//
// Each function cites the PETITE function it follows (paths inside
// src/PETITE/).  Expressions keep the reference's operation order; the
// kinematics, multiple scattering and lab rotation use the non-fusing S type
// (pt_common.cuh) because their formulas are ill-conditioned.
#pragma once
#include "pt_common.cuh"
#include "pt_moliere.cuh"
#include "petite_gpu.h"

namespace pt {

// Device copy of the table description plus derived constants.
struct Tabs {
  pt_tables t;
  double Z2a04;    // Z**2 * aa(Z, m_e)**4  (g2_elastic, all_processes.py:99-103)
  double a0sq;     // aa(Z, m_e)**2
};

// ------------------------------------------------------------ interpolation
// scipy interp1d(kind='linear', bounds_error=False, fill_value=0.0) on a 1-D
// table: numpy interp arithmetic inside [x0, xN], 0 outside.
__device__ __forceinline__ double interp_tab(const double* xs, const double* ys, int n, double E) {
  if (!(E >= xs[0]) || E > xs[n - 1]) return (E != E) ? E : 0.0;
  int lo = 0, hi = n - 1;               // find j with xs[j] <= E < xs[j+1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xs[mid] <= E) lo = mid; else hi = mid;
  }
  int j = (E >= xs[n - 1]) ? n - 1 : lo;
  if (j == n - 1) return ys[n - 1];
  if (xs[j] == E) return ys[j];
  const S slope = (S(ys[j + 1]) - S(ys[j])) / (S(xs[j + 1]) - S(xs[j]));
  S r = slope * (S(E) - S(xs[j])) + S(ys[j]);
  if (r.v != r.v) {
    r = slope * (S(E) - S(xs[j + 1])) + S(ys[j + 1]);
    if (r.v != r.v && ys[j] == ys[j + 1]) r = S(ys[j]);
  }
  return r.v;
}

__device__ __forceinline__ double nsig(const Tabs& T, int slot, double E) {
  const int b = T.t.ns_base[slot];
  return interp_tab(T.t.ns_x + b, T.t.ns_y + b, T.t.ns_len[slot], E);
}

// shower.py:357-368
__device__ __forceinline__ double nsigma_total(const Tabs& T, int pid, double E) {
  if (pid == 22) return nsig(T, 1, E) + nsig(T, 3, E);
  if (pid == 11) return nsig(T, 0, E) + nsig(T, 4, E);
  if (pid == -11) return nsig(T, 0, E) + nsig(T, 5, E) + nsig(T, 2, E);
  return nsig(T, 7, E) + nsig(T, 6, E);   // |pid| == 13
}
// shower.py:370-389
__device__ __forceinline__ double mfp_of(const Tabs& T, int pid, double E) {
  const double ns = nsigma_total(T, pid, E);
  if (ns <= 0.0) return 1.0e12;
  return kCmToM / ns;
}

__device__ __forceinline__ double min_calc(const Tabs& T, int pid) {   // shower.py:242-246
  if (pid == 11) return T.t.min_calc_electron;
  if (pid == -11) return T.t.min_calc_positron;
  if (pid == 22) return T.t.min_calc_photon;
  return T.t.min_calc_muon;
}
__host__ __device__ __forceinline__ double table_mass(int pid) {     // particle.py:4-13
  return (pid == 11 || pid == -11) ? kMe : ((pid == 13 || pid == -13) ? kMmu : 0.0);
}
__host__ __device__ __forceinline__ int process_dim(int p) {         // shower.py:47-56
  return (p == PT_BREM || p == PT_PAIRPROD || p == PT_MUONBREM) ? 4 : 1;
}

// LU_Key of draw_sample (shower.py:416-426): argmin|E_i - E| + 1, clipped.
__device__ __forceinline__ int lu_key(const Tabs& T, int process, double E) {
  const double* Ei = T.t.map_energy + T.t.map_base[process];
  const int n = T.t.map_rows[process];
  int lo = 0, hi = n;                   // first index with Ei >= E
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (Ei[mid] < E) lo = mid + 1; else hi = mid;
  }
  int best;
  if (lo == 0) best = 0;
  else if (lo == n) best = n - 1;
  else best = (fabs(Ei[lo - 1] - E) <= fabs(Ei[lo] - E)) ? lo - 1 : lo;
  int key = best + 1;
  if (key >= n) key = n - 1;
  return key;
}

// VEGAS map: y -> x, jac (Lepage 1978): i = floor(y*ninc) (<= ninc-1),
// x = g[i] + (g[i+1]-g[i])*(y*ninc - i), jac = prod ninc*(g[i+1]-g[i]).
__device__ __forceinline__ double map_dim(const double* g, int ninc, double y, double& jac) {
  const S t = S(y) * S((double)ninc);
  int i = (int)floor(t.v);
  if (i > ninc - 1) i = ninc - 1;
  const S inc = S(g[i + 1]) - S(g[i]);
  jac = (S(jac) * (S((double)ninc) * inc)).v;
  return (S(g[i]) + inc * (t - S((double)i))).v;
}

// ------------------------------------------------- differential cross sections
// dsigma_brem_dimensionless.__call__ (all_processes.py:153-206); also MuonBrem.
static __device__ double dsig_brem(const Tabs& T, const double* x, double ep, double m) {
  const double Eg = T.t.Eg_min;
  const double w = Eg + x[0] * (ep - m - Eg);
  const double k = ep / (2 * m);
  const double d = k * (x[1] + x[2]);
  const double dp = k * (x[1] - x[2]);
  const double ph = (x[3] - 0.5) * 2 * kPi;
  const double epp = ep - w;
  if (!((Eg < w) && (w < ep - m) && (m < epp) && (epp < ep) && (d > 0.0) && (dp > 0.0))) return 0.0;
  const double cph = cos(ph);
  const double m2 = m * m;
  const double A = (1 + d * d) / (2 * ep) - (1 + dp * dp) / (2 * epp);
  const double qsq = m2 * ((d * d + dp * dp - 2 * d * dp * cph) + m2 * (A * A));
  const double am = kAlpha / m;
  const double PF = 8.0 / kPi * kAlpha * (am * am) * (epp * (m2 * m2)) / (w * ep * (qsq * qsq)) * d * dp;
  const double jac = kPi * (ep * ep) * (ep - m - Eg) / m2;
  const double u = 1 + T.a0sq * qsq;
  const double FF = T.Z2a04 * (qsq * qsq) / (u * u);
  const double dd = d * d, pp = dp * dp, od = 1 + dd, op = 1 + pp;
  const double T1 = dd / (od * od);
  const double T2 = pp / (op * op);
  const double T3 = (w * w) / (2 * ep * epp) * (dd + pp) / (od * op);
  const double T4 = -(epp / ep + ep / epp) * (d * dp * cph) / (od * op);
  return PF * (T1 + T2 + T3 + T4) * jac * FF;
}

// dsigma_pairprod_dimensionless.__call__ (all_processes.py:546-622)
static __device__ double dsig_pairprod(const Tabs& T, const double* x, double w) {
  const double me = kMe;
  const double epp = me + x[0] * (w - 2 * me);
  const double k = w / (2 * me);
  const double dp = k * (x[1] + x[2]);
  const double dm = k * (x[1] - x[2]);
  const double ph = x[3] * 2 * kPi;
  const double epm = w - epp;
  if (!((me < epm) && (epm < w) && (me < epp) && (epp < w) && (dm > 0.0) && (dp > 0.0))) return 0.0;
  const double cph = cos(ph);
  const double B = (1.0 + dp * dp) / (2.0 * epp) + (1.0 + dm * dm) / (2.0 * epm);
  const double q = (dp * dp + dm * dm + 2.0 * dp * dm * cph) + (me * me) * (B * B);
  const double am = kAlpha / me;
  const double PF = 8.0 / kPi * kAlpha * (am * am) * epp * epm / ((w * w * w) * (q * q)) * dp * dm;
  const double jac = kPi * (w * w) * (w - 2 * me) / (me * me);
  const double t = (me * me) * q;
  const double u = 1 + T.a0sq * t;
  const double FF = T.Z2a04 * (t * t) / (u * u);
  const double d2 = dp * dp, m2 = dm * dm, o1 = 1.0 + d2, o2 = 1.0 + m2;
  const double T1 = -1.0 * d2 / (o1 * o1);
  const double T2 = -1.0 * m2 / (o2 * o2);
  const double T3 = (w * w) / (2.0 * epp * epm) * (d2 + m2) / (o1 * o2);
  const double T4 = (epp / epm + epm / epp) * (dp * dm * cph) / (o1 * o2);
  return PF * (T1 + T2 + T3 + T4) * jac * FF;
}

// dsigma_compton_dCT.__call__ (all_processes.py:639-742), mV = 0
static __device__ double dsig_compton(double ct, double Eg) {
  const double me = kMe, me2 = me * me, me4 = me2 * me2;
  const double s = me2 + 2 * Eg * me;
  if (s < me2) return 0.0;
  const double root = sqrt(me4 + s * s - 2 * me2 * s);
  const double jac = (s - me2) / (2 * s) * root;
  const double t = -1.0 / 2 * (me4 + s * (s + ct * root) - me2 * (2 * s + ct * root)) / s;
  const double PF = 2.0 * kPi * (kAlpha * kAlpha) / ((s - me2) * (s - me2));
  const double T1 = (6.0 * me2 * s + 3.0 * me4 - s * s) / ((me2 - s) * (-me2 + s + t));
  const double v = s + t - me2;
  const double T2 = 4 * me4 / (v * v);
  const double T3 = (t * (s - me2) + (s + me2) * (s + me2)) / ((s - me2) * (s - me2));
  return PF * jac * (T1 + T2 + T3);
}

// dsigma_annihilation_dCT.__call__ (all_processes.py:475-529), mV = 0
static __device__ double dsig_annihilation(const Tabs& T, double ct, double Ee) {
  const double me = kMe;
  const double s = 2.0 * me * (Ee + me);
  const double ctMax = sqrt((Ee + me) / (Ee - me)) * (2 * me * (Ee - 2 * T.t.Eg_min + me)) / (2 * me * (Ee + me));
  const double b2 = 1.0 - 4.0 * (me * me) / s;
  if (ct > ctMax) return 0.0;
  return 4.0 * kPi * (kAlpha * kAlpha) / (s * (1 - b2 * (ct * ct))) * (s / (2 * s) * (1 + ct * ct));
}

// dsigma_moller_dCT.__call__ (all_processes.py:799-840)
static __device__ double dsig_moller(const Tabs& T, double ct, double Ee) {
  const double me = kMe;
  const double lim = 2.0 * T.t.Ee_min / (Ee - me);
  if (!((ct > -1 + lim) && (ct < 1.0 - lim))) return 0.0;
  const double s = me * me + 2 * Ee * me;
  const double c2 = ct * ct, a = 3 + c2, me2 = me * me, v = s - 4 * me2;
  return 16 * (kPi * kPi) * (kAlpha * kAlpha) *
         ((s * s) * (a * a) - 8 * me2 * s * (7 + c2 * c2) + 16 * (me2 * me2) * (6 - 3 * c2 + c2 * c2)) /
         (8 * kPi * s * (v * v) * ((1 - ct) * (1 - ct)) * ((1 + ct) * (1 + ct)));
}

// dsigma_bhabha_dCT.__call__ (all_processes.py:960-1007)
static __device__ double dsig_bhabha(const Tabs& T, double ct, double Ee) {
  const double me = kMe;
  const double lim = 2.0 * T.t.Ee_min / (Ee - me);
  if (!((ct > -1 + lim) && (ct < 1.0 - lim))) return 0.0;
  const double s = me * me + 2 * Ee * me;
  const double m2 = me * me, m4 = m2 * m2, m6 = m4 * m2, m8 = m4 * m4;
  const double cm1 = -1 + ct, a = 3 + ct * ct;
  const double num = 256 * (cm1 * cm1) * (ct * ct) * m8
                   - 128 * cm1 * (1 + ct * (1 + ct) * (-3 + 2 * ct)) * m6 * s
                   + 16 * (7 + ct * (2 + ct * (-5 + 6 * cm1 * ct))) * m4 * (s * s)
                   - 8 * (7 + ct * (-3 + ct * (3 + ct * (-1 + 2 * ct)))) * m2 * (s * s * s)
                   + (a * a) * (s * s * s * s);
  const double v = -4 * m2 + s;
  return (kAlpha * kAlpha) * kPi * num / (2 * (cm1 * cm1) * (s * s * s) * (v * v));
}

// dsigma_muonelectron_dCT.__call__ (all_processes.py:855-886)
static __device__ double dsig_muone(const Tabs& T, double ct, double Emu) {
  const double me = kMe, mm = kMmu, me2 = me * me, mm2 = mm * mm;
  const double s = me2 + mm2 + 2 * me * Emu;
  const double t_limit = 2.0 * me * (me - T.t.Ee_min);
  const double a = s + me2 - mm2;
  const double t = -2.0 * (1 - ct) * ((a * a) / (4.0 * s) - me2);
  if (!(t < t_limit)) return 0.0;
  const double b = s + t - 4 * me2;
  return 16 * (kPi * kPi) * (kAlpha * kAlpha) * ((s * s) + 2 * (me2 + mm2) * (2 * t + mm2 - 3 * me2) + b * b) /
         (16 * kPi * s * (t * t));
}

__device__ __forceinline__ double dsigma_any(const Tabs& T, int process, const double* x, double E) {
  switch (process) {
    case PT_BREM: return dsig_brem(T, x, E, kMe);
    case PT_MUONBREM: return dsig_brem(T, x, E, kMmu);
    case PT_PAIRPROD: return dsig_pairprod(T, x, E);
    case PT_COMP: return dsig_compton(x[0], E);
    case PT_ANN: return dsig_annihilation(T, x[0], E);
    case PT_MOLLER: return dsig_moller(T, x[0], E);
    case PT_BHABHA: return dsig_bhabha(T, x[0], E);
    default: return dsig_muone(T, x[0], E);
  }
}

// ------------------------------------------------------------- kinematics
// Two four-vectors in the frame where the parent moves along +z; `al` is the
// azimuth already scaled to [0, 2pi).  kinematics.py.
struct V4 { double e, x, y, z; };

// e_to_egamma_fourvecs, kinematics.py:10-41 (Egamma_min = 0.001, :9)
static __device__ void kin_brem(double ep_, double m_, const double* xs, double al_, V4& lep, V4& gam) {
  const S ep(ep_), m(m_), Egmin(0.001), x1(xs[0]), x2(xs[1]), x3(xs[2]), x4(xs[3]), al(al_);
  const S w = Egmin + x1 * (ep - m - Egmin);
  const S ct = S(cos(((x2 + x3) / S(2.0)).v));
  const S ctp = S(cos(((x2 - x3) * ep / (S(2.0) * (ep - w))).v));
  const S ph = (x4 - S(0.5)) * S(2.0) * S(kPi);
  const S epp = ep - w;
  const S pp = ssqrt(sq(epp) - sq(m));
  const S cal(cos(al.v)), sal(sin(al.v));
  const S st = ssqrt(S(1.0) - sq(ct)), stp = ssqrt(S(1.0) - sq(ctp));
  const S sp(sin(ph.v)), cp(cos(ph.v));
  gam = {w.v, (w * cal * st).v, (w * sal * st).v, (w * ct).v};
  lep = {epp.v, (pp * (sal * sp * stp + cal * (ctp * st - cp * ct * stp))).v,
         (pp * (ctp * sal * st - (cp * ct * sal + cal * sp) * stp)).v,
         (pp * (ct * ctp + cp * st * stp)).v};
}

// gamma_to_epem_fourvecs, kinematics.py:70-102 -> (positron, electron)
static __device__ void kin_pairprod(double w_, const double* xs, double al_, V4& pos, V4& ele) {
  const S w(w_), me(kMe), x1(xs[0]), x2(xs[1]), x3(xs[2]), x4(xs[3]), al(al_);
  const S epp = me + x1 * (w - S(2.0) * me);
  const S ctp = S(cos((w * (x2 + x3) / (S(2.0) * epp)).v));
  const S ctm = S(cos((w * (x2 - x3) / (S(2.0) * (w - epp))).v));
  const S ph = x4 * S(2.0) * S(kPi);
  const S epm = w - epp;
  const S pm = ssqrt(sq(epm) - sq(me)), pp = ssqrt(sq(epp) - sq(me));
  const S cal(cos(al.v)), sal(sin(al.v));
  const S stp = ssqrt(S(1.0) - sq(ctp)), stm = ssqrt(S(1.0) - sq(ctm));
  const S phal = ph + al;
  const S spal(sin(phal.v)), cpal(cos(phal.v));
  pos = {epp.v, (pp * stp * cal).v, (pp * stp * sal).v, (pp * ctp).v};
  ele = {epm.v, (pm * stm * cpal).v, (pm * stm * spal).v, (pm * ctm).v};
}

// Shared tail of the 2->2 two-body forms: (g0*E1 +/- b0*g0*pF*ct, ...) with
// the signs of kinematics.py:129-130 (compton), 234-235 (ee), 262-263 (mue),
// 331-332 (annihilation).
// compton_fourvecs, kinematics.py:104-132, mV = 0 -> (electron, photon)
static __device__ void kin_compton(double Eg_, double ct_, double ph_, V4& e, V4& g) {
  const S Eg(Eg_), ct(ct_), ph(ph_), me(kMe);
  const S s = sq(me) + S(2.0) * Eg * me;
  const S rs = ssqrt(s);
  const S Ee0 = (s + sq(me)) / (S(2.0) * rs);
  const S Ee = (s - S(0.0) + sq(me)) / (S(2.0) * rs);
  const S EV = (s + S(0.0) - sq(me)) / (S(2.0) * rs);
  const S pF = ssqrt(sq(Ee) - sq(me));
  const S g0 = Ee0 / me;
  const S b0 = S(1.0) / g0 * ssqrt(sq(g0) - S(1.0));
  const S st = ssqrt(S(1.0) - sq(ct));
  const S sph(sin(ph.v)), cph(cos(ph.v));
  e = {(g0 * Ee + b0 * g0 * pF * ct).v, (-pF * st * sph).v, (-pF * st * cph).v, (b0 * g0 * Ee + g0 * pF * ct).v};
  g = {(g0 * EV - b0 * g0 * pF * ct).v, (pF * st * sph).v, (pF * st * cph).v, (b0 * g0 * EV - g0 * pF * ct).v};
}

// ee_to_ee_fourvecs, kinematics.py:213-237 -> (scattered lepton, new electron)
static __device__ void kin_ee(double Einc_, double ct_, double ph_, V4& a, V4& b) {
  const S E(Einc_), ct(ct_), ph(ph_), me(kMe);
  const S s = S(2.0) * sq(me) + S(2.0) * E * me;
  const S Ee0 = ssqrt(s) / S(2.0);
  const S pF = ssqrt(sq(Ee0) - sq(me));
  const S g0 = Ee0 / me;
  const S b0 = S(1.0) / g0 * ssqrt(sq(g0) - S(1.0));
  const S st = ssqrt(S(1.0) - sq(ct));
  const S sph(sin(ph.v)), cph(cos(ph.v));
  a = {(g0 * Ee0 + b0 * g0 * pF * ct).v, (-pF * st * sph).v, (-pF * st * cph).v, (b0 * g0 * Ee0 + g0 * pF * ct).v};
  b = {(g0 * Ee0 - b0 * g0 * pF * ct).v, (pF * st * sph).v, (pF * st * cph).v, (b0 * g0 * Ee0 - g0 * pF * ct).v};
}

// mue_to_mue_fourvecs, kinematics.py:239-265 -> (muon, electron)
static __device__ void kin_mue(double Einc_, double ct_, double ph_, V4& mu, V4& el) {
  const S E(Einc_), ct(ct_), ph(ph_), me(kMe), mm(kMmu);
  const S s = sq(me) + sq(mm) + S(2.0) * E * me;
  const S rs = ssqrt(s);
  const S Ee0 = (s + sq(me) - sq(mm)) / (S(2.0) * rs);
  const S Em0 = (s + sq(mm) - sq(me)) / (S(2.0) * rs);
  const S pe = ssqrt(sq(Ee0) - sq(me));
  const S pm = ssqrt(sq(Em0) - sq(mm));
  const S g0 = Ee0 / me;
  const S b0 = S(1.0) / g0 * ssqrt(sq(g0) - S(1.0));
  const S st = ssqrt(S(1.0) - sq(ct));
  const S sph(sin(ph.v)), cph(cos(ph.v));
  mu = {(g0 * Em0 + b0 * g0 * pm * ct).v, (pm * st * sph).v, (pm * st * cph).v, (b0 * g0 * Em0 + g0 * pm * ct).v};
  el = {(g0 * Ee0 - b0 * g0 * pe * ct).v, (-pe * st * sph).v, (-pe * st * cph).v, (b0 * g0 * Ee0 - g0 * pe * ct).v};
}

// annihilation_fourvecs, kinematics.py:301-334, mV = 0 -> (photon, photon)
static __device__ void kin_ann(double Ee_, double ct_, double ph_, V4& a, V4& b) {
  const S E(Ee_), ct(ct_), ph(ph_), me(kMe);
  const S s = S(2.0) * me * (E + me);
  const S rs = ssqrt(s);
  const S EeCM = rs / S(2.0);
  const S Eg = (s - S(0.0)) / (S(2.0) * rs);
  const S EV = (s + S(0.0)) / (S(2.0) * rs);
  const S pF = Eg;
  const S g0 = EeCM / me;
  const S b0 = S(1.0) / g0 * ssqrt(sq(g0) - S(1.0));
  const S st = ssqrt(S(1.0) - sq(ct));
  const S sph(sin(ph.v)), cph(cos(ph.v));
  a = {(g0 * Eg - b0 * g0 * pF * ct).v, (-pF * st * sph).v, (-pF * st * cph).v, (b0 * g0 * Eg - g0 * pF * ct).v};
  b = {(g0 * EV + b0 * g0 * pF * ct).v, (pF * st * sph).v, (pF * st * cph).v, (b0 * g0 * EV + g0 * pF * ct).v};
}

// ------------------------------------------------------ lab-frame rotation
// Particle.rotation_matrix, particle.py:176-185 (z_hat -> direction of pf)
struct Rot { double m[3][3]; };
__device__ __forceinline__ Rot rotation_from(const double* pf) {
  const S px(pf[1]), py(pf[2]), pz(pf[3]);
  const S r = ssqrt(sq(px) + sq(py) + sq(pz));
  const double ThZ = acos((pz / r).v);
  const double PhiZ = atan2(pf[2], pf[1]);
  const double cT = cos(ThZ), sT = sin(ThZ), cP = cos(PhiZ), sP = sin(PhiZ);
  Rot R;
  R.m[0][0] = (S(cT) * S(cP)).v; R.m[0][1] = -sP; R.m[0][2] = (S(sT) * S(cP)).v;
  R.m[1][0] = (S(cT) * S(sP)).v; R.m[1][1] = cP;  R.m[1][2] = (S(sT) * S(sP)).v;
  R.m[2][0] = -sT;               R.m[2][1] = 0.0; R.m[2][2] = cT;
  return R;
}
__device__ __forceinline__ V4 to_lab(const Rot& R, const V4& v) {
  // np.dot(RM, [px, py, pz]): row-wise sums in index order
  V4 o;
  o.e = v.e;
  o.x = (S(R.m[0][0]) * S(v.x) + S(R.m[0][1]) * S(v.y) + S(R.m[0][2]) * S(v.z)).v;
  o.y = (S(R.m[1][0]) * S(v.x) + S(R.m[1][1]) * S(v.y) + S(R.m[1][2]) * S(v.z)).v;
  o.z = (S(R.m[2][0]) * S(v.x) + S(R.m[2][1]) * S(v.y) + S(R.m[2][2]) * S(v.z)).v;
  return o;
}

// ----------------------------------------------- multiple Coulomb scattering
// generate_moliere_angle_simplified_alt (moliere.py:265-284): the Lynch-Dahl
// width (moliere.py:196-219) and the space angle from a Gaussian pair.  Draw
// order: sign, the pair (angle, radius; one Box-Muller evaluation).
static __device__ S lynch_dahl_theta(S beta, double t_, double A_, double Z_, double Z23, double m_lep, Rng& rng) {
  const S Z(Z_), A(A_), t(t_);
  const S p = S(m_lep / kMeV) * beta / ssqrt(S(1.0) - sq(beta));       // moliere.py:206
  const S pb = p * beta;
  const S chic2 = S(0.157) * Z * (Z + S(1.0)) * (t / A) * sq(S(1.0) / pb);
  const S zab = Z * S(1.0) * S(kAlpha) / beta;
  const S chia2 = S(2.007e-5) * S(Z23) * (S(1.0) + S(3.34) * sq(zab)) / sq(p);
  const S omega = chic2 / chia2;
  const S v = S(0.5) * omega / (S(1.0) - S(0.98));
  const S onev = S(1.0) + v;
  const S th0 = ssqrt(chic2 * (onev * S(log(onev.v)) / v - S(1.0)) / (S(1.0) + sq(S(0.98))));
  const double u_sign = rng.u(), u_ang = rng.u(), u_rad = rng.u();
  const S sign = (u_sign < 0.5) ? S(-1.0) : S(1.0);
  const S x2pi = S(u_ang) * S(2.0 * kPi);
  const S g2rad = ssqrt(S(-2.0) * S(log((S(1.0) - S(u_rad)).v)));
  const S g1 = S(0.0) + (S(cos(x2pi.v)) * g2rad) * th0;
  const S g2 = S(0.0) + (S(sin(x2pi.v)) * g2rad) * th0;
  return sign * ssqrt(sq(g1) + sq(g2));
}

// The rotation of moliere.py:384-398 (and :427-445): the direction (theta,
// phi) about z taken to the lab with the transpose of get_rotation_matrix.
static __device__ void mcs_rotate(double* p4, double pn, S theta, S phi) {
  const S cth(cos(theta.v)), sth(sin(theta.v)), cph(cos(phi.v)), sph(sin(phi.v));
  const S n0 = S(pn) * (sph * sth), n1 = S(pn) * (-cph * sth), n2 = S(pn) * cth;
  // get_rotation_matrix, moliere.py:287-348 (the repeated branch at :331 kept)
  const double vx = p4[1], vy = p4[2], vz = p4[3];
  double ca, sa, cb, sb;
  if (fabs(vx) > 0. && fabs(vy) > 0.) {
    double a = atan(fabs(vy / vx));
    if (vx > 0. && vy > 0.) a = -a;
    if (vx < 0. && vy > 0.) a = -(kPi - a);
    if (vx < 0. && vy < 0.) a = -(kPi + a);
    if (vx > 0. && vy < 0.) a = -(2. * kPi - a);
    ca = cos(a); sa = sin(a);
  } else if (fabs(vy) > 0.) { ca = 0.; sa = 1.; }
  else { ca = 1.; sa = 0.; }
  const double vxp = (S(vx) * S(ca) - S(vy) * S(sa)).v;
  if (fabs(vz) > 0. && fabs(vxp) > 0.) {
    double b = atan(fabs(vxp / vz));
    if (vz > 0. && vxp > 0.) b = -b;
    if (vz < 0. && vxp > 0.) b = -(kPi - b);
    if (vz < 0. && vxp < 0.) b = -(kPi + b);
    if (vz > 0. && vxp > 0.) b = -(2. * kPi - b);
    cb = cos(b); sb = sin(b);
  } else if (vxp > 0.) { cb = 0.; sb = -1.; }
  else if (vxp < 0.) { cb = 0.; sb = 1.; }
  else { cb = 1.; sb = 0.; }
  // R = Rb @ Ra; lab = R^T n
  const S R00 = S(cb) * S(ca), R01 = -(S(cb) * S(sa)), R02(sb);
  const S R10(sa), R11(ca), R12(0.0);
  const S R20 = -(S(sb) * S(ca)), R21 = S(sb) * S(sa), R22(cb);
  p4[1] = (R00 * n0 + R10 * n1 + R20 * n2).v;
  p4[2] = (R01 * n0 + R11 * n1 + R21 * n2).v;
  p4[3] = (R02 * n0 + R12 * n1 + R22 * n2).v;
}

// get_scattered_momentum_fast (moliere.py:350-400): four draws with phi.
static __device__ void mcs_fast(double* p4, double t_, double A_, double Z_, double Z23, double rescale, double m_lep,
                                Rng& rng) {
  const double pn = norm3_np(p4[1], p4[2], p4[3]);
  if (!(pn > 0)) return;
  const S beta = S(pn) / S(p4[0]);
  const S theta = lynch_dahl_theta(beta, t_, A_, Z_, Z23, m_lep, rng) * S(rescale);
  const S phi = S(0.0) + S(2.0 * kPi) * S(rng.u());
  mcs_rotate(p4, pn, theta, phi);
}

// get_scattered_momentum_Bethe (moliere.py:403-453) with
// generate_moliere_angle (moliere.py:221-247).  b < 2: the Lynch-Dahl angle
// with its default (electron) mass, four draws with phi.  Otherwise three:
// the inverse-CDF uniform (generate_moliere_x, moliere.py:124-136), the sign,
// phi.  The reference passes m_lepton on to get_chic_squared (moliere.py:244),
// which takes none (a TypeError there); its momentum is the electron's.
static __device__ void mcs_bethe(double* p4, double t_, double A_, double Z_, double Z13, double Z23, double rescale,
                                 Rng& rng) {
  const double pn = norm3_np(p4[1], p4[2], p4[3]);
  if (!(pn > 0)) return;
  const S beta = S(pn) / S(p4[0]);
  const S Z(Z_), A(A_), t(t_);
  // get_b, moliere.py:139-155 (z = 1)
  const S alpha = Z * S(kAlpha) / beta;
  const S expb = S(6700.0) * t * (Z + S(1.0)) * S(Z13) * S(1.0) / (sq(beta) * A * (S(1.0) + S(3.34) * sq(alpha)));
  const double b = log(expb.v);
  S theta;
  if (b < 2.0) {
    theta = lynch_dahl_theta(beta, t_, A_, Z_, Z23, kMe, rng);
  } else {
    const double B = moliere_B(b);
    const double x = moliere_x(rng.u(), B);
    // get_chic_squared, moliere.py:180-192
    const S p = S(kMe) / S(kHbarc) * beta / ssqrt(S(1.0) - sq(beta));
    const S chic2 = S(4.0) * S(kPi) * S(kNAvogadro) * sq(S(kAlpha)) * t * Z * (Z + S(1.0)) * S(1.0) /
                    (A * sq(p) * sq(beta));
    const S sign = rng.u() < 0.5 ? S(-1.0) : S(1.0);
    theta = sign * ssqrt(S(x) * chic2 * S(B));
  }
  theta = theta * S(rescale);
  const S phi = S(0.0) + S(2.0 * kPi) * S(rng.u());
  mcs_rotate(p4, pn, theta, phi);
}

// Shower._get_MCS_p (shower.py:147-151): mode 0 = fast (Lynch-Dahl), 1 = Bethe-Moliere.
__device__ __forceinline__ void mcs_apply(int mode, double* p4, double t, const pt_tables& tb, double rescale,
                                          double m_lep, Rng& rng) {
  if (mode) mcs_bethe(p4, t, tb.A, tb.Z, tb.Z13, tb.Z23, rescale, rng);
  else mcs_fast(p4, t, tb.A, tb.Z, tb.Z23, rescale, m_lep, rng);
}

// Particle.lose_energy, particle.py:143-153
__device__ __forceinline__ void lose_energy(double* pf, double mass, double value) {
  const double p30 = norm3_np(pf[1], pf[2], pf[3]);
  double Eu = (S(pf[0]) - S(value)).v;
  if (Eu <= mass) Eu = mass;
  const double p3f = ssqrt(sq(S(Eu)) - sq(S(mass))).v;
  if (p3f > 0.0) {
    pf[1] = (S(pf[1]) / S(p30) * S(p3f)).v;
    pf[2] = (S(pf[2]) / S(p30) * S(p3f)).v;
    pf[3] = (S(pf[3]) / S(p30) * S(p3f)).v;
    pf[0] = Eu;
  } else if (p3f == 0.0) {
    pf[0] = mass; pf[1] = 0.0; pf[2] = 0.0; pf[3] = 0.0;
  }
}

__device__ __forceinline__ void move_along(const double* pf, double* rf, double dist) {
  const double n = norm3_np(pf[1], pf[2], pf[3]);
  if (n > 0.0) {
    rf[0] = (S(rf[0]) + S(pf[1]) / S(n) * S(dist)).v;
    rf[1] = (S(rf[1]) + S(pf[2]) / S(n) * S(dist)).v;
    rf[2] = (S(rf[2]) + S(pf[3]) / S(n) * S(dist)).v;
  }
}

}  // namespace pt
