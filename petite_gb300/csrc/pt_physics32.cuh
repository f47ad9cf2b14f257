// pt_physics32.cuh -- float32 forms used by the mixed-precision engine.
//
// Same physics as pt_physics.cuh (PETITE's all_processes.py / moliere.py /
// kinematics.py), rearranged so float32 keeps its accuracy:
//  * every sampled variable comes with its complements (1-x, 1+x) read from
//    a node table built in float64, so 1-cos(theta) never cancels;
//  * the Brem and pair-production angular factors T1+T2+T3+T4 are rewritten
//    as sums of non-negative terms (they cancel near the peak otherwise):
//      Brem:  T*D = ((a-b)(1-ab))^2/D + 4ab s2 + W((a-b)^2/2 + 2ab s2),
//             a=delta, b=delta', s2=sin^2(phi/2), D=(1+a^2)(1+b^2), W=w^2/(E E')
//      pair:  T*D = (a-b)^2 (1 + (a+b)^2/D + K) + 4ab c2 (1+K),
//             a=delta+, b=delta-, c2=cos^2(phi/2), K=(E+ - E-)^2/(2 E+ E-)
//  * the form factor and prefactors are grouped so no intermediate leaves
//    the float32 range, and the result is the acceptance ratio
//    wgt*f/max_F directly;
//  * divisions whose divisors stay far inside float32's normal range (below
//    2^126: the angular denominators D are at most ~1e27 for electrons
//    below 1 TeV) use the approximate __fdividef (2 ulp) instead of the
//    correctly rounded division.
// Energies, positions and the final daughter four-momenta stay float64.
#pragma once
#include "pt_physics.cuh"

namespace pt {

// One map node in float32: value, increment to the next node, 1-value, 1+value.
struct Node32 { float g, inc, cm, cp; };

struct MapPt32 { float x, omx, opx; };   // x, 1-x, 1+x

__device__ __forceinline__ MapPt32 map_dim32(const float4* nodes, int ninc, float y, float& jac) {
  const float t = y * (float)ninc;
  int i = (int)t;
  if (i > ninc - 1) i = ninc - 1;
  const float f = t - (float)i;
  const float4 n = __ldg(nodes + i);     // (g, inc, 1-g, 1+g)
  jac *= (float)ninc * n.y;
  MapPt32 r;
  r.x = fmaf(n.y, f, n.x);
  r.omx = fmaf(-n.y, f, n.z);
  r.opx = fmaf(n.y, f, n.w);
  return r;
}

// Per-task constants of the float32 sampler (computed once per particle).
struct Samp32 {
  float E, m, k, span, Eg, C;      // C folds prefactors and 1/(max_F*neval)
  float b;                         // form-factor scale (a0*m)^2
  float aux0, aux1, aux2;          // process-specific
};

// ---- Brem / MuonBrem: dsigma_brem_dimensionless (all_processes.py:153-206)
// C_row = 8 alpha^3 Z^2 a0^4 / (max_F neval) for this map row (host table).
__device__ __forceinline__ void brem32_setup(Samp32& S, float E, float m, float Eg, float a0sq, float C_row) {
  S.E = E; S.m = m; S.k = E / (2.f * m); S.span = E - m - Eg; S.Eg = Eg;
  S.b = a0sq * m * m;                         // (a0 m)^2
  S.C = C_row;
  S.aux0 = E * S.span;
}
__device__ __forceinline__ float brem32_ratio(const Samp32& S, const MapPt32* x, float jac) {
  const float w = fmaf(x[0].x, S.span, S.Eg);
  const float epp = fmaf(S.span, x[0].omx, S.m);
  const float d = S.k * (x[1].x + x[2].x);
  const float dp = S.k * (x[1].x - x[2].x);
  if (!((S.Eg < w) && (w < S.E - S.m) && (S.m < epp) && (epp < S.E) && (d > 0.f) && (dp > 0.f))) return 0.f;
  const float sp = sinpif(x[3].x - 0.5f);      // sin(phi/2), phi = (x4-1/2)*2pi
  const float s2 = sp * sp;
  const float amb = 2.f * S.k * x[2].x;        // d - dp
  const float ab = d * dp;
  const float d2 = d * d;
  const float Anum = 4.f * S.k * S.k * x[1].x * x[2].x * S.E - (1.f + d2) * w;
  const float mA = __fdividef(S.m * Anum, 2.f * S.E * epp);
  const float qh = amb * amb + 4.f * ab * s2 + mA * mA;     // qsq / m^2
  const float D = (1.f + d2) * (1.f + dp * dp);
  const float iD = __fdividef(1.f, D);
  const float t1 = amb * (1.f - ab) * iD;
  const float W = __fdividef(w, S.E) * __fdividef(w, epp);
  const float T = t1 * t1 + 4.f * ab * s2 * iD + W * (0.5f * amb * amb + 2.f * ab * s2) * iD;
  const float u = __fdividef(1.f, fmaf(S.b, qh, 1.f));
  const float Q = S.aux0 * __fdividef(epp, w);  // E' E (E - m - Eg) / w
  return ((S.C * jac) * Q) * ((ab * T) * (u * u));
}

// ---- PairProd: dsigma_pairprod_dimensionless (all_processes.py:546-622)
__device__ __forceinline__ void pair32_setup(Samp32& S, float w, float a0sq, float C_row) {
  const float me = (float)kMe;
  S.E = w; S.m = me; S.k = w / (2.f * me); S.span = w - 2.f * me;
  S.b = a0sq * me * me;
  S.C = C_row;
  S.aux0 = S.span / w;
}
__device__ __forceinline__ float pair32_ratio(const Samp32& S, const MapPt32* x, float jac) {
  const float epp = fmaf(x[0].x, S.span, S.m);
  const float epm = fmaf(x[0].omx, S.span, S.m);
  const float dp = S.k * (x[1].x + x[2].x);
  const float dm = S.k * (x[1].x - x[2].x);
  if (!((S.m < epm) && (epm < S.E) && (S.m < epp) && (epp < S.E) && (dm > 0.f) && (dp > 0.f))) return 0.f;
  const float cp = cospif(x[3].x);             // cos(phi/2), phi = 2 pi x4
  const float c2 = cp * cp;
  const float dd = 2.f * S.k * x[2].x;         // dp - dm
  const float ab = dp * dm;
  const float B = __fdividef(1.f + dp * dp, 2.f * epp) + __fdividef(1.f + dm * dm, 2.f * epm);
  const float q = dd * dd + 4.f * ab * c2 + (S.m * B) * (S.m * B);
  const float D = (1.f + dp * dp) * (1.f + dm * dm);
  const float iD = __fdividef(1.f, D);
  const float dE = S.span * (x[0].x - x[0].omx);          // E+ - E-
  const float K = 0.5f * __fdividef(dE, epp) * __fdividef(dE, epm);
  const float spm = dp + dm;
  const float T = (dd * dd * (1.f + spm * spm * iD + K) + 4.f * ab * c2 * (1.f + K)) * iD;
  const float u = __fdividef(1.f, fmaf(S.b, q, 1.f));
  const float Q = (epp * epm) * S.aux0;        // E+ E- (w - 2 me) / w
  return ((S.C * jac) * Q) * ((ab * T) * (u * u));
}

// ---- Compton (mV = 0): dsigma_compton_dCT (all_processes.py:639-742),
// with s - m^2 = D = 2 E m, t = -D^2 (1+c)/(2s), s + t - m^2 = D (2m^2 + D(1-c))/(2s).
__device__ __forceinline__ void comp32_setup(Samp32& S, float Eg, float C_row) {
  const float me = (float)kMe, me2 = me * me, D = 2.f * Eg * me, s = me2 + D;
  S.E = D; S.m = me2; S.span = s;
  S.C = C_row / s;                            // PF * jac = pi alpha^2 / s
}
__device__ __forceinline__ float comp32_ratio(const Samp32& S, const MapPt32& c, float jac) {
  const float D = S.E, m2 = S.m, s = S.span;
  const float t = -D * D * c.opx / (2.f * s);
  const float u = D * fmaf(D, c.omx, 2.f * m2) / (2.f * s);
  const float T1 = (6.f * m2 * s + 3.f * m2 * m2 - s * s) / (-D * u);
  const float T2 = 4.f * m2 * m2 / (u * u);
  const float sp = s + m2;
  const float T3 = (t * D + sp * sp) / (D * D);
  return (S.C * jac) * (T1 + T2 + T3);
}

// ---- Annihilation (mV = 0): dsigma_annihilation_dCT (all_processes.py:475-529)
__device__ __forceinline__ void ann32_setup(Samp32& S, float Ee, float Eg_min, float C_row) {
  const float me = (float)kMe, s = 2.f * me * (Ee + me);
  const float p = sqrtf((Ee - me) * (Ee + me));
  // 1 - ctMax with ctMax = (E + m - 2 Eg_min)/p, written without cancellation
  S.E = s;
  S.aux0 = 4.f * me * me / s;                 // 1 - b^2
  S.aux1 = (2.f * Eg_min - me - me * me / (p + Ee)) / p;
  S.C = C_row / s;                            // 4 pi alpha^2 / s * 1/2
}
__device__ __forceinline__ float ann32_ratio(const Samp32& S, const MapPt32& c, float jac) {
  if (c.omx < S.aux1) return 0.f;
  const float den = fmaf(S.aux0 * c.x, c.x, c.omx * c.opx);   // 1 - b^2 c^2
  return (S.C * jac) * fmaf(c.x, c.x, 1.f) / den;
}

// ---- Moller: dsigma_moller_dCT (all_processes.py:799-840)
__device__ __forceinline__ void moller32_setup(Samp32& S, float Ee, float Ee_min, float C_row) {
  const float me = (float)kMe, s = me * me + 2.f * Ee * me, v = s - 4.f * me * me;
  S.E = s; S.m = me * me;
  S.aux0 = 2.f * Ee_min / (Ee - me);          // delta_ct_limit
  S.C = C_row / (s * v * v);                  // 16 pi^2 alpha^2 / (8 pi s v^2)
}
__device__ __forceinline__ float moller32_ratio(const Samp32& S, const MapPt32& c, float jac) {
  if (!(c.opx > S.aux0 && c.omx > S.aux0)) return 0.f;
  const float s = S.E, m2 = S.m, c2 = c.x * c.x, a = 3.f + c2;
  const float num = s * s * a * a - 8.f * m2 * s * (7.f + c2 * c2) + 16.f * m2 * m2 * (6.f - 3.f * c2 + c2 * c2);
  const float den = (c.omx * c.opx) * (c.omx * c.opx);
  return (S.C * jac) * (num / den);
}

// ---- Bhabha: dsigma_bhabha_dCT (all_processes.py:960-1007)
__device__ __forceinline__ void bhabha32_setup(Samp32& S, float Ee, float Ee_min, float C_row) {
  const float me = (float)kMe, s = me * me + 2.f * Ee * me, v = s - 4.f * me * me;
  S.E = s; S.m = me * me;
  S.aux0 = 2.f * Ee_min / (Ee - me);
  S.C = C_row / ((s * s) * (s * v * v));      // alpha^2 pi / (2 s^3 v^2)
}
__device__ __forceinline__ float bhabha32_ratio(const Samp32& S, const MapPt32& c, float jac) {
  if (!(c.opx > S.aux0 && c.omx > S.aux0)) return 0.f;
  const float s = S.E, m2 = S.m, ct = c.x, cm1 = -c.omx;
  const float m4 = m2 * m2, m6 = m4 * m2, m8 = m4 * m4, a = 3.f + ct * ct;
  const float num = 256.f * (cm1 * cm1) * (ct * ct) * m8
                  - 128.f * cm1 * (1.f + ct * (1.f + ct) * (-3.f + 2.f * ct)) * m6 * s
                  + 16.f * (7.f + ct * (2.f + ct * (-5.f + 6.f * cm1 * ct))) * m4 * (s * s)
                  - 8.f * (7.f + ct * (-3.f + ct * (3.f + ct * (-1.f + 2.f * ct)))) * m2 * (s * s * s)
                  + (a * a) * ((s * s) * (s * s));
  return (S.C * jac) * (num / (cm1 * cm1));
}

// ---- mu e -> mu e: dsigma_muonelectron_dCT (all_processes.py:855-886),
// with p_cm^2 = m_e^2 (E^2 - m_mu^2)/s so t = -2(1-c) p_cm^2 does not cancel.
__device__ __forceinline__ void muone32_setup(Samp32& S, float Emu, float Ee_min, float C_row) {
  const float me = (float)kMe, mm = (float)kMmu, s = me * me + mm * mm + 2.f * me * Emu;
  const float pcm2 = me * me * (Emu - mm) * (Emu + mm) / s;
  S.E = s; S.m = me * me; S.span = pcm2;
  S.aux0 = me * (Ee_min - me) / pcm2;         // t < t_limit <=> 1-c > this
  S.aux1 = mm * mm;
  S.C = C_row / s;                            // 16 pi^2 alpha^2 / (16 pi s)
}
__device__ __forceinline__ float muone32_ratio(const Samp32& S, const MapPt32& c, float jac) {
  if (!(c.omx > S.aux0)) return 0.f;
  const float s = S.E, m2 = S.m, mm2 = S.aux1;
  const float t = -2.f * c.omx * S.span;
  const float v = s + t - 4.f * m2;
  const float num = s * s + 2.f * (m2 + mm2) * (2.f * t + mm2 - 3.f * m2) + v * v;
  return (S.C * jac) * (num / (t * t));
}

// -------------------------------------------- multiple scattering, float32
// Lynch-Dahl width (moliere.py:196-219,265-284).  The reference's momentum
// m_lepton*beta/sqrt(1-beta^2) with beta = |p|/E equals |p| m_lepton / m; the
// caller passes that product as pmag (well conditioned, unlike 1 - beta^2),
// same four draws as the float64 form, frame rotation of moliere.py:287-348
// written algebraically (its branches reduce to ca = vx/rho, sa = -vy/rho,
// cb = vz/r, sb = -rho/r).
__device__ __forceinline__ float lynch_dahl_g(float v) {
  // (1+v) ln(1+v)/v - 1 without cancellation at small v
  if (v < 1e-2f) return v * (0.5f + v * (-1.f / 6.f + v * (1.f / 12.f - v * 0.05f)));
  return (1.f + v) * log1pf(v) / v - 1.f;
}

// Lynch-Dahl space angle (sign and Gaussian radius draws given; the pair's
// angle draw cancels in the space angle).  p = m_lepton beta gamma (GeV).
__device__ __forceinline__ float lynch_dahl_theta32(float p_gev, float beta, float t, float A, float Z, float Z23,
                                                    float u_sign, float u_rad) {
  const float p = p_gev * 1000.f;                       // MeV
  const float pb = p * beta;
  const float chic2 = 0.157f * Z * (Z + 1.f) * (t / A) / (pb * pb);
  const float zab = Z * (float)kAlpha / beta;
  const float chia2 = 2.007e-5f * Z23 * (1.f + 3.34f * zab * zab) / (p * p);
  const float v = 0.5f * (chic2 / chia2) / (1.f - 0.98f);
  const float th0 = sqrtf(chic2 * lynch_dahl_g(v) / (1.f + 0.98f * 0.98f));
  const float theta = th0 * sqrtf(-2.f * __logf(1.f - u_rad));
  return u_sign < 0.5f ? -theta : theta;
}

// The direction turned by (theta, phi) about itself.
__device__ __forceinline__ void mcs32_rotate(float3& dir, float theta, float u_phi) {
  float sth, cth, sph, cph;
  sincosf(theta, &sth, &cth);
  sincospif(2.f * u_phi, &sph, &cph);
  const float n0 = sph * sth, n1 = -cph * sth, n2 = cth;
  const float vx = dir.x, vy = dir.y, vz = dir.z;
  const float rho = sqrtf(vx * vx + vy * vy);
  float ca = 1.f, sa = 0.f, cb = 1.f, sb = 0.f;
  if (rho > 0.f) { ca = vx / rho; sa = -vy / rho; }
  const float rr = sqrtf(rho * rho + vz * vz);
  if (rho > 0.f) { cb = vz / rr; sb = -rho / rr; }
  // lab = Ra^T Rb^T n
  const float w0 = cb * n0 - sb * n2, w1 = n1, w2 = sb * n0 + cb * n2;
  float3 o = make_float3(ca * w0 + sa * w1, -sa * w0 + ca * w1, w2);
  const float inv = rsqrtf(o.x * o.x + o.y * o.y + o.z * o.z);
  dir = make_float3(o.x * inv, o.y * inv, o.z * inv);
}

// get_scattered_momentum_fast with its used draws given (sign, radius, phi).
__device__ __forceinline__ void mcs32_u(float3& dir, float pmag, float E, float t, float A, float Z, float Z23,
                                        float rescale, float u_sign, float u_rad, float u_phi, float beta_p) {
  const float beta = beta_p >= 0.f ? beta_p : pmag / E;
  mcs32_rotate(dir, lynch_dahl_theta32(pmag, beta, t, A, Z, Z23, u_sign, u_rad) * rescale, u_phi);
}

// Material constants of the Lynch-Dahl width folded for mcs32_ld.  With p
// the lepton momentum in GeV (the reference's formula takes MeV), beta and
// t in g/cm^2:
//   chi_c^2 = kc t / (p beta)^2,         kc = 0.157e-6 Z (Z+1) / A
//   chi_c^2 / chi_a^2 = kc t / (ka (beta^2 + k3)),
//                                        ka = 2.007e-11 Z^(2/3), k3 = 3.34 (Z alpha)^2
// (p cancels in the ratio), so v = 0.5 (chi_c^2/chi_a^2) / (1 - F) = kv t /
// (beta^2 + k3) with kv = 25 kc / ka, and theta0^2 = kth t g(v) / (p beta)^2
// with kth = kc / (1 + F^2), F = 0.98.
struct Ld32 { float kth, kv, k3; };
__host__ __device__ inline Ld32 ld32_constants(double A, double Z, double Z23) {
  const double kc = 0.157e-6 * Z * (Z + 1.0) / A, ka = 2.007e-11 * Z23;
  const double za = Z * kAlpha;
  return {(float)(kc / (1.0 + 0.98 * 0.98)), (float)(25.0 * kc / ka), (float)(3.34 * za * za)};
}

// mcs32_rotate for a unit direction: with rho = |(vx, vy)| the rotation
// there reduces to
//   lab = n2 v + n0 (vx vz / rho, vy vz / rho, -rho) + n1 (-vy / rho, vx / rho, 0),
// one reciprocal square root instead of two square roots and four
// divisions.  A direction along z (rho = 0) keeps n, as the reference's
// get_rotation_matrix does there; within 2^-50 of the axis the frame's
// azimuth is dropped (phi is uniform) and n is flipped for a backward
// direction.
__device__ __forceinline__ void mcs32_rotate_unit(float3& dir, float theta, float u_phi) {
  float sth, cth, sph, cph;
  sincosf(theta, &sth, &cth);
  sincospif(2.f * u_phi, &sph, &cph);
  const float n0 = sph * sth, n1 = -cph * sth, n2 = cth;
  const float vx = dir.x, vy = dir.y, vz = dir.z;
  const float r2 = fmaf(vx, vx, vy * vy);
  float3 o;
  if (r2 > 0x1p-100f) {
    const float inv = rsqrtf(r2);
    const float a = fmaf(n0 * vz, inv, n2), b = n1 * inv;
    o = make_float3(fmaf(a, vx, -b * vy), fmaf(a, vy, b * vx), fmaf(n2, vz, -n0 * (r2 * inv)));
  } else {
    o = make_float3(n0, n1, (vz < 0.f && (vx != 0.f || vy != 0.f)) ? -n2 : n2);
  }
  const float s = rsqrtf(o.x * o.x + o.y * o.y + o.z * o.z);
  dir = make_float3(o.x * s, o.y * s, o.z * s);
}

// get_scattered_momentum_fast (moliere.py:350-400) for a particle of mass m
// and momentum pmag (GeV) at energy E, scattered with lepton mass mlep
// (p = pmag mlep / m, beta = pmag / E): the Lynch-Dahl space angle on its
// sign, radius and phi draws, from the folded constants K, then the
// rotation of the unit direction.  Three approximate reciprocals
// (__fdividef, 2 ulp) on operands far inside float32's range replace the
// eleven divisions and two square roots of the term-by-term form.
__device__ __forceinline__ void mcs32_ld(float3& dir, float pmag, float E, float m, float mlep, float t,
                                         const Ld32& K, float rescale, float u_sign, float u_rad, float u_phi) {
  const float p2 = pmag * pmag, E2 = E * E;
  const float v = __fdividef(K.kv * t * E2, fmaf(K.k3, E2, p2));    // beta^2 = p2 / E2
  float g;                                                            // (1+v) ln(1+v)/v - 1
  if (v < 1e-2f) {
    g = v * (0.5f + v * (-1.f / 6.f + v * (1.f / 12.f - v * 0.05f)));
  } else {
    const float lg = log1pf(v);
    g = fmaf(lg, __fdividef(1.f, v), lg - 1.f);
  }
  // 1 / (p beta) = E m / (pmag^2 mlep)
  float theta = sqrtf(K.kth * t * g * (-2.f * __logf(1.f - u_rad))) * __fdividef(E * m, p2 * mlep) * rescale;
  if (u_sign < 0.5f) theta = -theta;
  mcs32_rotate_unit(dir, theta, u_phi);
}

// get_scattered_momentum_Bethe (moliere.py:403-453) on the next four draws
// u[0..3]; returns how many it used.  b < 2: the Lynch-Dahl angle with the
// electron mass, draws sign, (pair angle), radius, phi.  Otherwise the
// inverse-CDF draw, the sign and phi.  pe = m_e beta gamma (GeV): the
// reference's momentum m_e beta / sqrt(1 - beta^2) in a well-conditioned form.
__device__ __forceinline__ int mcs32_bethe(float3& dir, float pe, float beta, float t, float A, float Z, float Z13,
                                           float Z23, float rescale, float u0, float u1, float u2, float u3) {
  const float alpha = Z * (float)kAlpha / beta;        // get_b, moliere.py:139-155
  const float expb = 6700.f * t * (Z + 1.f) * Z13 / (beta * beta * A * (1.f + 3.34f * alpha * alpha));
  const float b = __logf(expb);
  if (b < 2.f) {
    mcs32_rotate(dir, lynch_dahl_theta32(pe, beta, t, A, Z, Z23, u0, u2) * rescale, u3);
    return 4;
  }
  const float B = moliere_B(b);
  const float x = moliere_x(u0, B);
  const float pb = pe * (float)(1.0 / kHbarc) * beta;  // get_chic_squared, moliere.py:180-192 (1/cm)
  const float chic2 = (float)(4.0 * kPi * kNAvogadro * kAlpha * kAlpha) * t * Z * (Z + 1.f) / (A * pb * pb);
  float theta = sqrtf(x * chic2 * B);
  if (u1 < 0.5f) theta = -theta;
  mcs32_rotate(dir, theta * rescale, u2);
  return 3;
}

// Lab frame from the parent's momentum: Particle.rotation_matrix
// (particle.py:176-185) with cos/sin of ThZ, PhiZ taken from the direction,
// by reciprocal square roots for |p| and for the transverse length.  A
// momentum below 2^-50 GeV keeps the z axis, and a direction within 2^-50
// of it the azimuth 0 (as at rho = 0).
struct Rot32 { float cT, sT, cP, sP; };
__device__ __forceinline__ Rot32 rot32_from_momentum(float px, float py, float pz) {
  Rot32 R = {1.f, 0.f, 1.f, 0.f};
  const float p2 = px * px + py * py + pz * pz;
  if (!(p2 > 0x1p-100f)) return R;
  const float r = rsqrtf(p2);
  const float dx = px * r, dy = py * r;
  const float t2 = dx * dx + dy * dy;
  R.cT = pz * r;
  if (t2 > 0x1p-100f) {
    const float ir = rsqrtf(t2);
    R.sT = t2 * ir; R.cP = dx * ir; R.sP = dy * ir;
  } else {
    R.sT = sqrtf(t2);
  }
  return R;
}
__device__ __forceinline__ float3 rot32_apply(const Rot32& R, float3 v) {
  return make_float3(R.cT * R.cP * v.x - R.sP * v.y + R.sT * R.cP * v.z,
                     R.cT * R.sP * v.x + R.cP * v.y + R.sT * R.sP * v.z,
                     -R.sT * v.x + R.cT * v.z);
}

}  // namespace pt
