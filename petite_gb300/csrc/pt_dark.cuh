// pt_dark.cuh -- dark-vector physics of PETITE (DarkShower), float64.
//
// The differential cross sections are templates over the scalar type of the
// dark-vector mass: `double` for sampling and yields, `Dual` (value and
// derivative with respect to mV) for the adjoint of the dark yield.  Every
// other input is a plain double.  Expressions keep the reference's
// operation order; each function cites the PETITE function it follows
// (paths inside src/PETITE/).
#pragma once
#include <type_traits>

#include "pt_common.cuh"

namespace pt {

// ------------------------------------------------------------ dual numbers
struct Dual {
  double v, d;
};
__device__ __forceinline__ Dual mkd(double v, double d = 0.0) { return Dual{v, d}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual operator/(Dual a, double b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ Dual operator/(double a, Dual b) {
  const double q = a / b.v;
  return {q, -q * b.d / b.v};
}

__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(Dual x) { return x.v; }
__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ Dual dsqrt(Dual x) {
  const double s = sqrt(x.v);
  return {s, x.d == 0.0 ? 0.0 : x.d / (2.0 * s)};
}
__device__ __forceinline__ double dabs(double x) { return fabs(x); }
__device__ __forceinline__ Dual dabs(Dual x) { return x.v < 0.0 ? -x : x; }
__device__ __forceinline__ double dpow(double x, double e) { return pow(x, e); }
// The derivative is taken as 0 at x = 0 (where x^e underflowed but its
// derivative's factor x^(e-1) may not have).
__device__ __forceinline__ Dual dpow(Dual x, double e) {
  const double p = pow(x.v, e);
  return {p, (x.d == 0.0 || x.v == 0.0) ? 0.0 : e * pow(x.v, e - 1.0) * x.d};
}
__device__ __forceinline__ double dlog(double x) { return log(x); }
__device__ __forceinline__ Dual dlog(Dual x) { return {log(x.v), x.d / x.v}; }
__device__ __forceinline__ double dexp10(double x) { return pow(10.0, x); }
__device__ __forceinline__ Dual dexp10(Dual x) {
  const double e = pow(10.0, x.v);
  return {e, e * 2.302585092994046 * x.d};
}
template <class T>
__device__ __forceinline__ T sqr(T x) { return x * x; }

constexpr double kMproton = 938.272088 * kMeV;
constexpr double kLn10 = 2.302585092994046;

// ------------------------------------------------------ dark bremsstrahlung
// Gelastic_inelastic_over_tsquared (all_processes.py:112-133)
template <class T>
__device__ __forceinline__ T g_el_inel_over_t2(double Z, double A, T t) {
  const double c1 = sqr(111 * pow(Z, -1.0 / 3) / kMe);
  const double c2 = 0.164 * pow(A, -2.0 / 3);
  const T Gel = sqr(1.0 / (1.0 + c1 * t)) * dpow(1 + t / c2, -2.0);
  const double ap2 = sqr(773.0 * pow(Z, -2.0 / 3) / kMe);
  const T Ginel = Z / (sqr(c1) * sqr(Z)) * sqr(ap2 / (1.0 + ap2 * t)) *
                  ((1.0 + (2.79 * 2.79 - 1.0) * t / (4.0 * sqr(kMproton))) / dpow(1.0 + t / 0.71, 4.0));
  return sqr(Z) * sqr(c1) * (Gel + Ginel);
}

// Limits of the momentum transfer for fixed (x, cos theta)
// (all_processes.py:261-283): t- and t+ and the discriminant.
template <class T>
struct BremLimits {
  T k, V, ut, discr, tp, tm;
};
template <class T, class X>
__device__ __forceinline__ BremLimits<T> dark_brem_limits(X x, double ct, double E, T mV, double MT, double m) {
  BremLimits<T> L;
  const T mV2 = mV * mV;
  L.k = dsqrt(dabs(sqr(x * E) - mV2));
  const double p = sqrt(E * E - m * m);
  L.V = dsqrt(p * p + L.k * L.k - 2 * p * L.k * ct);
  L.ut = -2 * (x * (E * E) - L.k * p * ct) + mV2;
  const X Er = (1 - x) * E + MT;
  L.discr = L.ut * L.ut + 4 * MT * L.ut * Er + 4 * (MT * MT) * (L.V * L.V);
  const T rd = dsqrt(dabs(L.discr));
  const T den = 2 * (Er * Er) - 2 * (L.V * L.V);
  const T Qp = dabs((L.V * (L.ut + 2 * MT * Er) + Er * rd) / den);
  const T Qm = dabs((L.V * (L.ut + 2 * MT * Er) - Er * rd) / den);
  L.tp = 2 * MT * (dsqrt(MT * MT + Qp * Qp) - MT);
  L.tm = 2 * MT * (dsqrt(MT * MT + Qm * Qm) - MT);
  return L;
}

// The same limits without cancellation, for the anchored form below:
// Q- = (A - B)/den = -ut (ut + 4 MT Er) / (2 (A + B)) with A = V (ut + 2 MT Er),
// B = Er sqrt(discr), and 2 MT (sqrt(MT^2 + Q^2) - MT) = 2 MT Q^2 / (sqrt(MT^2 + Q^2) + MT).
template <class T, class X>
__device__ __forceinline__ BremLimits<T> dark_brem_limits_stable(X x, double ct, double E, T mV, double MT,
                                                                 double m) {
  BremLimits<T> L;
  const T mV2 = mV * mV;
  L.k = dsqrt(dabs(sqr(x * E) - mV2));
  const double p = sqrt(E * E - m * m);
  L.V = dsqrt(p * p + L.k * L.k - 2 * p * L.k * ct);
  L.ut = -2 * (x * (E * E) - L.k * p * ct) + mV2;
  const X Er = (1 - x) * E + MT;
  L.discr = L.ut * L.ut + 4 * MT * L.ut * Er + 4 * (MT * MT) * (L.V * L.V);
  const T Aq = L.V * (L.ut + 2 * MT * Er);
  const T Bq = Er * dsqrt(dabs(L.discr));
  const T den = 2 * (Er * Er) - 2 * (L.V * L.V);
  const T Qp = dabs((Aq + Bq) / den);
  const T Qm = dabs(L.ut * (L.ut + 4 * MT * Er) / (2 * (Aq + Bq)));
  L.tp = 2 * MT * (Qp * Qp) / (dsqrt(MT * MT + Qp * Qp) + MT);
  L.tm = 2 * MT * (Qm * Qm) / (dsqrt(MT * MT + Qm * Qm) + MT);
  return L;
}

__device__ __forceinline__ double dark_brem_tconv(double E, double MT, double m) {
  return sqr(2 * MT * (MT + E) * sqrt(E * E + m * m) / (MT * (MT + 2 * E) + m * m));
}

// dsig_dx_dcostheta_dark_brem_exact_tree_level.__call__, method "Log"
// (all_processes.py:227-372) at (x, cos theta, t~): the vector mass and t~
// may carry derivatives.  omc = 1 - cos theta.
template <class T, class X>
__device__ T dark_brem_core(X x, double omc, T tt, double E, T mV, double MT, double m, double Z, double A,
                            const BremLimits<T>& L) {
  const double ct = 1.0 - omc;
  const T jac = omc * tt * (kLn10 * kLn10);
  const T mV2 = mV * mV;
  const double p = sqrt(E * E - m * m);
  const T &k = L.k, &V = L.V, &ut = L.ut;
  const double tconv = dark_brem_tconv(E, MT, m);
  const T t = tt * tconv;
  const T q0 = -t / (2 * MT);
  const T q = dsqrt(t * t / (4 * (MT * MT)) + t);
  const T cq = -(V * V + q * q + m * m - sqr(E + q0 - x * E)) / (2 * V * q);
  const T mm = mV2 + 2 * (m * m);
  const T Am2 = -8 * MT * (4 * (E * E) * MT - t * (2 * E + MT)) * mm;
  const T A1 = 8 * (MT * MT) / ut;
  const T Am1 = (8 / ut) * ((MT * MT) * (2 * t * ut + ut * ut +
                                         4 * (E * E) * (2 * (x - 1) * mm - t * ((x - 2) * x + 2)) +
                                         2 * t * (-mV2 + 2 * (m * m) + t)) -
                            2 * E * MT * t * ((1 - x) * ut + (x - 2) * (mm + t)) + (t * t) * (ut - mV2));
  const T A0 = (8 / (ut * ut)) * ((MT * MT) * (2 * t * ut + (t - 4 * (E * E) * sqr(x - 1)) * mm) +
                                  2 * E * MT * t * (ut - (x - 1) * mm));
  const T Y = -t + 2 * q0 * E - 2 * q * p * (p - k * ct) * cq / V;
  const T W = dabs(Y * Y - 4 * (q * q) * (p * p) * (k * k) * (1 - ct * ct) * (1 - cq * cq) / (V * V));
  const bool allowed = (val(x) * E >= val(mV)) && (val(L.discr) >= 0) && (val(L.tp) > val(L.tm)) &&
                       (val(t) > val(L.tm)) && (val(t) < val(L.tp)) && (fabs(val(cq)) <= 1.0) && (val(W) > 0);
  if (!allowed) return T(mV * 0.0);
  const T phi = (A0 + Y * A1 + Am1 / dsqrt(W) + Y * Am2 / dpow(W, 1.5)) / (8 * (MT * MT));
  const T ff = g_el_inel_over_t2(Z, A, t);
  const T ans = ff * (kAlpha * kAlpha * kAlpha) * k * E * phi / (p * dsqrt(k * k + p * p - 2 * p * k * ct));
  return ans * tconv * jac;
}

// The reference's form: x = (E_V/E, log10(1 - cos theta), log10 t~).
template <class T>
__device__ T dsig_dark_brem(const double* xv, double E, T mV, double MT, double m, double Z, double A) {
  const double omc = pow(10.0, xv[1]);
  const BremLimits<T> L = dark_brem_limits(xv[0], 1.0 - omc, E, mV, MT, m);
  return dark_brem_core<T>(xv[0], omc, T(mV * 0.0) + pow(10.0, xv[2]), E, mV, MT, m, Z, A, L);
}

// The same integrand with the samples carried along the kinematic ranges of
// mV: a sample drawn for the anchor mass a at x0 sits at the fraction
// w = (x0 - a/E) / (1 - a/E) of the range x > mV/E and, for its x, at the
// fraction v = (l0 - l-(a)) / (l+(a) - l-(a)) of the log10 t~ range; for mass
// mV it moves to x = mV/E + w (1 - mV/E) and l = l-(mV) + v (l+(mV) - l-(mV)),
// with the Jacobian of both moves.  At mV = a this is the reference's
// integrand; for other masses it integrates the same cross section (a change
// of variables), but the kinematic edges no longer move through the fixed
// samples, so the estimate is smooth in mV.
template <class T>
__device__ T dsig_dark_brem_anchored(const double* xv, double E, T mV, double a, double MT, double m, double Z,
                                     double A) {
  const double omc = pow(10.0, xv[1]);
  const double ct = 1.0 - omc;
  const double tconv = dark_brem_tconv(E, MT, m);
  const double xa = a / E;
  const double w = (xv[0] - xa) / (1.0 - xa);
  if (!(w > 0.0 && w < 1.0)) return T(mV * 0.0);
  const BremLimits<double> La = dark_brem_limits_stable(xv[0], ct, E, a, MT, m);
  if (!(La.discr >= 0) || !(La.tp > La.tm) || !(La.tm > 0)) return T(mV * 0.0);
  const double lma = log10(La.tm / tconv), lpa = log10(La.tp / tconv);
  const double v = (xv[2] - lma) / (lpa - lma);
  if (!(v > 0.0 && v < 1.0)) return T(mV * 0.0);
  const T xm = mV / E;
  const T x = xm + w * (1.0 - xm);
  const BremLimits<T> L = dark_brem_limits_stable(x, ct, E, mV, MT, m);
  if (!(val(L.discr) >= 0) || !(val(L.tp) > val(L.tm)) || !(val(L.tm) > 0)) return T(mV * 0.0);
  const T lm = dlog(L.tm / tconv) / kLn10, lp = dlog(L.tp / tconv) / kLn10;
  const T l = lm + (lp - lm) * v;
  const T tt = dexp10(l);
  const T jac = ((lp - lm) / (lpa - lma)) * ((1.0 - xm) / (1.0 - xa));
  return dark_brem_core<T>(x, omc, tt, E, mV, MT, m, Z, A, L) * jac;
}

// A float32 estimate of the dark-bremsstrahlung integrand, used only to
// screen accept/reject decisions: it returns false whenever the estimate
// cannot be trusted -- within 0.1-0.2 % of a kinematic edge (k = 0, t-/t+,
// |cos theta_q| = 1, discriminant 0) or where a sum of terms cancels to less
// than 1e-3 .. 1e-2 of their magnitudes.  Otherwise its relative error is far
// below the factor the screen allows.  The forms avoid the cancellations of
// the reference's expressions: p - k = (p^2 - k^2)/(p + k),
// x E^2 - k p = (E^2 (x^2 m^2 + mV^2) - m^2 mV^2)/(x E^2 + k p),
// V^2 - ((1-x)E)^2 = (p - k - (1-x)E)(p - k + (1-x)E) + 2 k p (1 - cos theta),
// and the limits of dark_brem_limits_stable.
enum { kScreenUnsure = 0, kScreenValue = 1, kScreenOutside = 2 };

// The screen's per-draw constants (incident energy, masses, target and the
// form-factor scales), formed once per draw_dark_sample call.
struct Screen32K { float E, mV, MT, m, Z, cs1, cc2, ap2, tconv; };
__device__ __forceinline__ Screen32K screen32_constants(double E_, double mV_, double MT_, double m_, double Z_,
                                                        double A_, float tconv) {
  Screen32K K;
  K.E = (float)E_; K.mV = (float)mV_; K.MT = (float)MT_; K.m = (float)m_;
  const float Z = (float)Z_, A = (float)A_;
  K.Z = Z;
  const float cc1 = 111.f * powf(Z, -1.f / 3.f) / (float)kMe;
  K.cs1 = cc1 * cc1;
  K.cc2 = 0.164f * powf(A, -2.f / 3.f);
  const float ap = 773.f * powf(Z, -2.f / 3.f) / (float)kMe;
  K.ap2 = ap * ap;
  K.tconv = tconv;
  return K;
}

// The screen at a float32 sample (x, log10(1 - cos theta), log10 t~).
__device__ __forceinline__ int dark_brem_screen32k(float x, float lomc, float ltt, const Screen32K& K, float& out) {
  const float E = K.E, mV = K.mV, MT = K.MT, m = K.m;
  const float omc = exp10f(lomc);
  const float tt = exp10f(ltt);
  const float xE = x * E;
  if (xE < mV * 0.999f) return kScreenOutside;                      // x E >= mV fails
  if (!(xE > mV * 1.001f) || !(x < 1.f)) return kScreenUnsure;
  const float k = sqrtf((xE - mV) * (xE + mV));
  const float p = sqrtf((E - m) * (E + m));
  const float kp = k * p;
  const float pmk = ((1.f - x) * (1.f + x) * E * E - m * m + mV * mV) / (p + k);
  const float V2 = pmk * pmk + 2.f * kp * omc;
  const float V = sqrtf(V2);
  const float D = (E * E * (x * x * m * m + mV * mV) - m * m * mV * mV) / (x * E * E + kp);
  const float ut = mV * mV - 2.f * D - 2.f * kp * omc;
  const float Er = (1.f - x) * E + MT;
  const float d1 = ut * ut, d2 = 4.f * MT * ut * Er, d3 = 4.f * MT * MT * V2;
  const float discr = d1 + d2 + d3;
  const float dscale = fabsf(d1) + fabsf(d2) + d3;
  if (discr < -1e-3f * dscale) return kScreenOutside;                // discriminant < 0
  if (!(discr > 1e-3f * dscale)) return kScreenUnsure;
  const float Aq = V * (ut + 2.f * MT * Er), Bq = Er * sqrtf(discr);
  if (!(Aq > 0.f)) return kScreenUnsure;
  const float den = 2.f * (Er * Er - V2);
  const float Qp = fabsf((Aq + Bq) / den);
  const float Qm = fabsf(ut * (ut + 4.f * MT * Er) / (2.f * (Aq + Bq)));
  const float tp = 2.f * MT * Qp * Qp / (sqrtf(MT * MT + Qp * Qp) + MT);
  const float tm = 2.f * MT * Qm * Qm / (sqrtf(MT * MT + Qm * Qm) + MT);
  const float t = tt * K.tconv;
  if (tp > tm * 1.01f && (t < tm * 0.998f || t > tp * 1.002f)) return kScreenOutside;   // outside (t-, t+)
  if (!(t > tm * 1.002f && t < tp * 0.998f)) return kScreenUnsure;
  const float q0 = -t / (2.f * MT);
  const float q = sqrtf(t * t / (4.f * MT * MT) + t);
  const float a = (1.f - x) * E;
  const float dk = -m * m / (p + E) + mV * mV / (k + xE);           // p - k - (1-x)E
  const float n1 = dk * (pmk + a), n2 = 2.f * kp * omc, n3 = t * (1.f + a / MT), n4 = m * m;
  const float num = n1 + n2 + n3 + n4;
  if (!(fabsf(num) > 1e-3f * (fabsf(n1) + n2 + n3 + n4))) return kScreenUnsure;
  const float cq = -num / (2.f * V * q);
  if (fabsf(cq) > 1.001f) return kScreenOutside;                    // |cos theta_q| <= 1 fails
  if (!(fabsf(cq) < 0.999f)) return kScreenUnsure;
  const float y1 = -t + 2.f * q0 * E;
  const float y2 = -2.f * q * p * (pmk + k * omc) * cq / V;
  const float Y = y1 + y2;
  if (!(fabsf(Y) > 1e-2f * (fabsf(y1) + fabsf(y2)))) return kScreenUnsure;
  const float w2 = 4.f * q * q * p * p * k * k * (omc * (2.f - omc)) * ((1.f - cq) * (1.f + cq)) / V2;
  const float Wr = Y * Y - w2;
  if (!(fabsf(Wr) > 1e-2f * Y * Y)) return kScreenUnsure;
  const float W = fabsf(Wr);
  const float mm = mV * mV + 2.f * m * m;
  const float Am2 = -8.f * MT * (4.f * E * E * MT - t * (2.f * E + MT)) * mm;
  const float A1 = 8.f * MT * MT / ut;
  const float i1 = 2.f * t * ut, i2 = ut * ut, i3 = 4.f * E * E * (2.f * (x - 1.f) * mm - t * ((x - 2.f) * x + 2.f)),
              i4 = 2.f * t * (-mV * mV + 2.f * m * m + t);
  const float inner = i1 + i2 + i3 + i4;
  if (!(fabsf(inner) > 1e-3f * (fabsf(i1) + fabsf(i2) + fabsf(i3) + fabsf(i4)))) return kScreenUnsure;
  const float b1 = MT * MT * inner, b2 = -2.f * E * MT * t * ((1.f - x) * ut + (x - 2.f) * (mm + t)),
              b3 = t * t * (ut - mV * mV);
  const float bs = b1 + b2 + b3;
  if (!(fabsf(bs) > 1e-3f * (fabsf(b1) + fabsf(b2) + fabsf(b3)))) return kScreenUnsure;
  const float Am1 = (8.f / ut) * bs;
  const float c1 = MT * MT * (2.f * t * ut + (t - 4.f * E * E * (x - 1.f) * (x - 1.f)) * mm),
              c2 = 2.f * E * MT * t * (ut - (x - 1.f) * mm);
  const float cs = c1 + c2;
  if (!(fabsf(cs) > 1e-3f * (fabsf(c1) + fabsf(c2)))) return kScreenUnsure;
  const float A0 = (8.f / (ut * ut)) * cs;
  const float sw = sqrtf(W);
  const float P0 = A0, P1 = Y * A1, P2 = Am1 / sw, P3 = Y * Am2 / (W * sw);
  const float ps = P0 + P1 + P2 + P3;
  if (!(fabsf(ps) > 1e-2f * (fabsf(P0) + fabsf(P1) + fabsf(P2) + fabsf(P3)))) return kScreenUnsure;
  const float phi = ps / (8.f * MT * MT);
  // Gelastic_inelastic_over_tsquared in float32 (all_processes.py:112-133)
  const float Z = K.Z, cs1 = K.cs1, cc2 = K.cc2, ap2 = K.ap2;
  const float g1 = 1.f / (1.f + cs1 * t), g2 = 1.f / (1.f + t / cc2);
  const float g3 = ap2 / (1.f + ap2 * t), g4 = 1.f + t / 0.71f;
  const float Ginel = Z / (cs1 * cs1 * Z * Z) * (g3 * g3) *
                      ((1.f + (2.79f * 2.79f - 1.f) * t / (4.f * (float)(kMproton * kMproton))) / (g4 * g4 * g4 * g4));
  const float ff = Z * Z * cs1 * cs1 * (g1 * g1 * g2 * g2 + Ginel);
  const float al = (float)kAlpha;
  const float ans = ff * (al * al * al) * k * E * phi / (p * V);
  out = ans * K.tconv * (omc * tt * (float)(kLn10 * kLn10));
  return (out > 0.f && out < 3.0e38f) ? kScreenValue : kScreenUnsure;
}

__device__ __forceinline__ int dark_brem_screen32(const double* xv, double E_, double mV_, double MT_, double m_,
                                                  double Z_, double A_, float tconv, float& out) {
  return dark_brem_screen32k((float)xv[0], (float)xv[1], (float)xv[2],
                             screen32_constants(E_, mV_, MT_, m_, Z_, A_, tconv), out);
}

// ----------------------------------------------------------- dark Compton
// dsigma_compton_dCT.__call__ with mV > 0 (all_processes.py:639-742)
template <class T>
__device__ T dsig_dark_compton(double ct, double Eg, T mV) {
  const double me = kMe, me2 = me * me, me4 = me2 * me2;
  const double s = me2 + 2 * Eg * me;
  if (s < val(sqr(me + mV))) return T(mV * 0.0);
  const T mV2 = mV * mV;
  const T root = dsqrt(me4 + sqr(mV2 - s) - 2 * me2 * (mV2 + s));
  const T jac = (s - me2) / (2 * s) * dsqrt(sqr(s - mV2) - 2 * me2 * (s + mV2) + me4);
  const T t = -1.0 / 2 * (me4 + s * (-mV2 + s + ct * root) - me2 * (mV2 + 2 * s + ct * root)) / s;
  const double PF = 2.0 * kPi * (kAlpha * kAlpha) / sqr(s - me2);
  const T T1 = (2.0 * me2 * (mV2 - 3 * s) - 3 * me4 - 2 * mV2 * s + 2 * (mV2 * mV2) + s * s) /
               ((me2 - s) * (me2 + mV2 - s - t));
  const T T2 = (2 * me2 * (2 * me2 + mV2)) / sqr(me2 + mV2 - s - t);
  const T T3 = ((me2 + s) * (me2 + mV2 + s) + t * (s - me2)) / sqr(me2 - s);
  return PF * jac * (T1 + T2 + T3);
}

// ------------------------------------------------ radiative return (DarkAnn)
// Kuraev-Fadin structure functions (radiative_return.py:26-47)
__device__ __forceinline__ double kf_beta(double s) {
  return (2. * kAlpha / kPi) * (log(s / (kMe * kMe)) - 1.);
}
template <class T>
__device__ __forceinline__ T fl_kf(T x, double beta) {
  if (val(x) >= 1.0) x = T(x * 0.0) + (1. - 1e-10);
  return (beta / 16.) * ((8. + 3. * beta) * dpow(1. - x, beta / 2. - 1.) - 4. * (1. + x));
}
// The same with 1 - x given separately (no cancellation as x -> 1).
template <class T>
__device__ __forceinline__ T fl_kf_omx(T x, T omx, double beta) {
  return (beta / 16.) * ((8. + 3. * beta) * dpow(omx, beta / 2. - 1.) - 4. * (1. + x));
}
// omx = 1 - x computed without cancellation (x = 1 - u^(2/beta) rounds to 1
// for u < ~0.3 at these energies); the float64 form keeps the reference's 1 - x.
template <class T>
__device__ __forceinline__ T fl_kf_scaled(T x, T omx, double beta) {
  T base;
  if constexpr (std::is_same<T, double>::value) base = 1. - x;
  else base = omx;
  return (beta / 16.) * ((8. + 3. * beta) - 4. * (1. + x) * dpow(base, 1. - beta / 2.));
}
// dsigma_radiative_return_du.__call__ (all_processes.py:419-466) with
// transformed_lepton_luminosity_integrand (radiative_return.py:61-80).
// FACTORED: evaluate 1 - x2 as (s - mV^2)(1 - u0^(2/beta)) / (x1 s), the same
// quantity without the cancellation of 1 - x2 near the x2 -> 1 end (u0 -> 1),
// where (1 - x2)^(beta/2 - 1) is nearly singular; the yield kernels use this
// form so that the estimate is smooth in mV at fixed uniforms.
template <class T, bool FACTORED = false>
__device__ T dsig_radiative_return(double u0, double Ee, T mV) {
  const double me = kMe;
  const double s = 2.0 * me * (Ee + me);
  const T mV2 = mV * mV;
  if (s < val(mV2)) return T(mV * 0.0);
  const double beta = kf_beta(s);
  const T umax = dpow(1.0 - mV2 / s, beta / 2.0);
  const T betaf = dsqrt(1.0 - 4.0 * (me * me) / mV2);
  const T prefac = (4.0 * (kPi * kPi)) * kAlpha * betaf * (3.0 / 2.0 - betaf * betaf / 2.0) / s * umax;
  const T u = u0 * umax;
  const T omx1 = dpow(u, 2.0 / beta);
  const T x1 = 1.0 - omx1;
  const T x2 = mV2 / (x1 * s);
  if (!(val(x2) < 1.0 && val(x1) > 0.0 && u0 < 1.0)) return T(mV * 0.0);
  // transformed luminosity at (s, y = mV^2/s, u): x = 1 - u^(2/beta) (= x1)
  const T y = mV2 / s;
  T fy;
  if constexpr (FACTORED) {
    const double omu = -expm1((2.0 / beta) * log(u0));        // 1 - u0^(2/beta)
    fy = fl_kf_omx(y / x1, (s - mV2) * omu / (x1 * s), beta);
  } else {
    fy = fl_kf(y / x1, beta);
  }
  const T lumi = fy * fl_kf_scaled(x1, omx1, beta) * (1. / x1) * (2. / beta);
  return 2.0 * prefac * lumi;
}

// The float32 screen of the radiative-return cross section (the float32
// dark form's DarkAnn proposals).  Per task, in float64 once: y = mV^2/s,
// beta, and the constant factor 2 prefac (beta/16)^2 (2/beta) of
// dsig_radiative_return.  Per proposal, in float32, with q = u0^(2/beta):
// x1 = y + (1 - y)(1 - q) (= 1 - (u0 umax)^(2/beta), without the
// cancellation), x2 = y/x1, 1 - x2 = (1 - y)(1 - q)/x1 (the factored form),
// and the two luminosity factors.  Both factors are positive and free of
// cancellation (fl_kf >= 4, fl_kf_scaled >= 4), and the powers' relative
// error is ~|log| x 1e-7, so the estimate is within ~1e-5 of the float64
// value: measured within 4e-4 of the float64 form (whose own rounding makes
// up that difference) on map samples at every tabulated energy.
struct Ann32K {
  float y, omy, beta, tob, c8, bh, bk, K;
  int valid;           // s >= mV^2 and a finite constant
};

__device__ __forceinline__ Ann32K ann32_constants(double Ee, double mV) {
  Ann32K k{};
  const double me = kMe, s = 2.0 * me * (Ee + me), mV2 = mV * mV;
  k.valid = 0;
  if (!(s >= mV2) || !(mV2 > 4.0 * me * me)) return k;
  const double beta = kf_beta(s);
  const double umax = pow(1.0 - mV2 / s, beta / 2.0);
  const double betaf = sqrt(1.0 - 4.0 * (me * me) / mV2);
  const double prefac = (4.0 * (kPi * kPi)) * kAlpha * betaf * (3.0 / 2.0 - betaf * betaf / 2.0) / s * umax;
  const double K = 2.0 * prefac * (beta / 16.) * (beta / 16.) * (2. / beta);
  k.y = (float)(mV2 / s);
  k.omy = (float)(1.0 - mV2 / s);
  k.beta = (float)beta;
  k.tob = (float)(2.0 / beta);
  k.c8 = (float)(8. + 3. * beta);
  k.bh = (float)(beta / 2. - 1.);
  k.bk = (float)(1. - beta / 2.);
  k.K = (float)K;
  k.valid = (beta > 0.0 && K > 0.0 && K < 1e30) ? 1 : 0;
  return k;
}

__device__ __forceinline__ int ann_screen32(double u0d, const Ann32K& k, float& out) {
  out = 0.f;
  const float u0 = (float)u0d, om = (float)(1.0 - u0d);     // 1 - u0 from float64: u0 sits near 1
  if (!k.valid || !(u0 > 0.f) || !(om > 0.f)) return kScreenUnsure;
  const float lq = k.tob * (u0 < 0.5f ? logf(u0) : log1pf(-om));
  const float q = expf(lq), omq = -expm1f(lq);
  const float d = k.omy * omq;                               // x1 - y
  // the float64 form's x1 = 1 - omx1 carries ~1e-16 of rounding, which
  // 1 - x2 = (x1 - y)/x1 magnifies by 1/(x1 - y): below 1e-11 float64 decides
  if (!(d > 1e-11f)) return kScreenUnsure;
  // omx1 may underflow to 0 (u0^(2/beta) below 1e-38): the float64 form's
  // 1 - x1 is then 0 as well, and the term it scales drops out of both
  const float omx1 = k.omy * q;
  const float x1 = d + k.y;
  const float x2 = k.y / x1;
  const float omx2 = d / x1;
  const float fy = k.c8 * powf(omx2, k.bh) - 4.f * (1.f + x2);
  const float fks = k.c8 - 4.f * (1.f + x1) * powf(omx1, k.bk);
  out = k.K * fy * fks / x1;
  return (out > 0.f && out < 3.0e38f) ? kScreenValue : kScreenUnsure;
}

// ------------------------------------------------ energies of the dark vector
// Lab energy of V for the yield moments: x*E (kinematics.py:57), the Compton
// form (kinematics.py:119-130) and the boosted radiative-return form
// (kinematics.py:282-298).
template <class T>
__device__ T dark_compton_EV(double ct, double Eg, T mV) {
  const double me = kMe;
  const double s = me * me + 2 * Eg * me, rs = sqrt(s);
  const T mV2 = mV * mV;
  const double Ee0 = (s + me * me) / (2.0 * rs);
  const T Ee = (s - mV2 + me * me) / (2 * rs);
  const T EV = (s + mV2 - me * me) / (2 * rs);
  const T pF = dsqrt(Ee * Ee - me * me);
  const double g0 = Ee0 / me;
  const double b0 = 1.0 / g0 * sqrt(g0 * g0 - 1.0);
  return g0 * EV - b0 * g0 * pF * ct;
}
template <class T>
__device__ T dark_ann_EV(double u0, double Ee, T mV) {
  const double me = kMe;
  const double s = 2. * me * (me + Ee), rs = sqrt(s);
  const double beta = kf_beta(s);
  const T mV2 = mV * mV;
  const T umax = dpow(1. - mV2 / s, beta / 2.);
  const T x1 = 1. - dpow(u0 * umax, 2. / beta);
  const T x2 = mV2 / (x1 * s);
  const T E1 = x1 * rs / 2., E2 = x2 * rs / 2.;
  const double p0 = rs / 2., p3 = -sqrt(s / 4. - me * me);
  const double rsq = sqrt(p0 * p0 - p3 * p3);
  return (p0 * (E1 + E2) - p3 * (E1 - E2)) / rsq;
}

}  // namespace pt
