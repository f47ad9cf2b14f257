// pt_moliere.cuh -- Bethe-Moliere multiple scattering (Shower(...,
// fast_MCS_mode=False), moliere.py:33-174,221-247,403-453), float64 and
// float32.
//
// The reference samples x = theta^2 / (chi_c^2 B) by inverting the Moliere
// CDF with scipy quad inside a Ridder root search.  Here the CDF is in
// closed form.  With g(x) = Ei(x) - ln x (g' = (e^x - 1)/x) the second-order
// density satisfies f1 = -2 d/dx[x e^-x g] + 2 e^-x, so with
// h(x) = x e^-x g(x) - 1 the tail of the CDF is
//   Q(x, B) = 1 - F(x, B) = e^-x (1 + 1/B) + h(x) / B
// and the density (f0 + f1/B)/2 = e^-x + ((x-1) h - 1)/(B x) + 2 e^-x / B.
// The inverse solves Q = 1 - u by Newton steps inside a bracket.  The
// float64 forms also compile for the host (a CPU test checks them against
// the oracle with and without contraction into fused multiply-adds).
#pragma once
#include "pt_common.cuh"

namespace pt {

template <class T> struct MolTol;
template <> struct MolTol<double> {
  static constexpr double series_below = 40.0;   // asymptotic truncation sqrt(2 pi x) e^-x < 3e-15 of h above
  static constexpr double eps = 1e-17;
  static constexpr double newton = 1e-10;         // |dx| <= newton x: the next error is below 1e-19
  static constexpr double closed = 4.5e-16;       // a bisection bracket this narrow (relative) ends the search
  static constexpr double xtol = 2e-12;           // the reference's root search (scipy ridder defaults)
  static constexpr double rtol = 8.881784197001252e-16;
};
template <> struct MolTol<float> {
  static constexpr float series_below = 20.f;     // truncation ~2e-8 absolute
  static constexpr float eps = 1e-8f;
  static constexpr float newton = 1e-5f;
  static constexpr float closed = 2.4e-7f;
  static constexpr float xtol = 1e-7f;
  static constexpr float rtol = 4.8e-7f;
};

__host__ __device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ float mexp(float x) { return __expf(x); }
__host__ __device__ __forceinline__ double mlog(double x) { return log(x); }
__device__ __forceinline__ float mlog(float x) { return __logf(x); }

// x e^-x (Ei(x) - ln x) - 1.  Below series_below: g = gamma + sum x^k/(k k!)
// (positive terms); above: x e^-x Ei(x) ~ sum k!/x^k to its smallest term.
template <class T>
__host__ __device__ T moliere_h(T x) {
  T term = T(1), s = T(0);
  if (x < MolTol<T>::series_below) {
    for (int k = 1; k <= 400; ++k) {
      term *= x / T(k);
      const T d = term / T(k);
      s += d;
      if (d <= MolTol<T>::eps * s) break;
    }
    return x * mexp(-x) * (T(0.57721566490153286061) + s) - T(1);
  }
  for (int k = 1; k <= 400; ++k) {
    const T nxt = term * (T(k) / x);
    if (nxt >= term) break;
    term = nxt;
    s += term;
    if (term <= MolTol<T>::eps * s) break;
  }
  return s - x * mexp(-x) * mlog(x);
}

template <class T>
__host__ __device__ __forceinline__ T moliere_tail(T x, T B) {
  return mexp(-x) * (T(1) + T(1) / B) + moliere_h(x) / B;
}

template <class T>
__host__ __device__ __forceinline__ T moliere_density(T x, T B) {
  const T e = mexp(-x);
  const T f1 = T(2) * ((x - T(1)) * moliere_h(x) - T(1)) / x + T(4) * e;
  return e + T(0.5) * f1 / B;
}

// moliere_f1(0): the reference evaluates x <= 1e-6 at 1e-6 (moliere.py:45-50)
template <class T>
__host__ __device__ __forceinline__ T moliere_f1_zero() {
  const double x = 1e-6;
  const double g = (moliere_h(x) + 1.0) / (x * exp(-x));
  return T(2. * exp(-x) * (x - 1.) * g - 2. * (1. - 2. * exp(-x)));
}

// moliere_cdf (moliere.py:62-81): f(0,B) x below 0.01, the integral up to
// 100, a three-term asymptote above.
template <class T>
__host__ __device__ T moliere_cdf_pieces(T x, T B, T f00) {
  if (x > T(100)) return T(1) - (T(1) / B / x + T(2) / B / (x * x) + T(6) / B / (x * x * x));
  if (x < T(0.01)) return f00 * x;
  return T(1) - moliere_tail(x, B);
}

// Ridders' method (Ridders 1979): midpoint, then the root of the
// exponentially scaled line through the three points; the sub-bracket with a
// sign change is kept.  Bounded at 100 steps.
template <class T>
__host__ __device__ T moliere_ridders(T u, T B, T f00, T a, T b) {
  T fa = moliere_cdf_pieces(a, B, f00) - u, fb = moliere_cdf_pieces(b, B, f00) - u;
  if (fa == T(0)) return a;
  if (fb == T(0)) return b;
  T x = a;
  for (int it = 0; it < 100; ++it) {
    const T dm = T(0.5) * (b - a);
    const T m = a + dm;
    const T fm = moliere_cdf_pieces(m, B, f00) - u;
    const T den = sqrt(fm * fm - fa * fb);
    x = m - copysign(T(1), fb - fa) * dm * fm / den;
    const T fx = moliere_cdf_pieces(x, B, f00) - u;
    if (fx * fm < T(0)) { a = x; fa = fx; b = m; fb = fm; }
    else if (fx * fa < T(0)) { b = x; fb = fx; }
    else { a = x; fa = fx; }
    if (fx == T(0) || fabs(b - a) < MolTol<T>::xtol + MolTol<T>::rtol * x) break;
  }
  return x;
}

// inverse_moliere_cdf (moliere.py:84-120): the explicit branches are the
// reference's.  Otherwise the root of the piecewise CDF; the integral piece
// by bracketed Newton steps on the closed-form tail.  Inside the step of the
// pieces at x = 0.01 (two roots ~1 % apart) the reference's own search
// decides: its bracket expansion from [0.5, 2], then Ridders' method.
template <class T>
__host__ __device__ T moliere_x(T u, T B) {
  if (T(1) - u < T(1) / B / T(100)) return T(1) / (T(1) - u) / B;
  if (u < T(0.01)) return u;
  const T f00 = T(0.5) * (T(2) + moliere_f1_zero<T>() / B);
  if (u < f00 * T(0.01) && T(1) - moliere_tail(T(0.01), B) < u) {
    T a = T(0.5), b = T(2);
    for (int it = 0; it <= 20; ++it) {
      const T fa = moliere_cdf_pieces(a, B, f00) - u, fb = moliere_cdf_pieces(b, B, f00) - u;
      if (!(fa * fb > T(0))) break;
      if (fb < T(0)) b *= T(2);
      if (fa > T(0)) a *= T(0.5);
    }
    return moliere_ridders(u, B, f00, a, b);
  }
  const T q = T(1) - u;
  T lo = T(0), hi = T(200);
  T x = fmax(mlog((T(1) + T(1) / B) / q), T(1) / (B * q));
  if (!(x > lo && x < hi)) x = T(0.5) * (lo + hi);
  for (int it = 0; it < 60; ++it) {
    const T Q = moliere_tail(x, B);
    if (Q == q) break;
    if (Q > q) lo = x; else hi = x;
    T xn = x + (Q - q) / moliere_density(x, B);
    if (xn == x) break;                                 // the step is below one ulp of x
    bool done;
    if (xn > lo && xn < hi) {                           // Newton: the next error is ~ the step squared
      done = fabs(xn - x) <= MolTol<T>::newton * xn;
    } else {                                            // bisection ends only on a closed bracket
      xn = T(0.5) * (lo + hi);
      done = hi - lo <= MolTol<T>::closed * xn;
    }
    x = xn;
    if (done) break;
  }
  if (x < T(0.01)) return u / f00;
  if (x > T(100)) {
    // 1 - (1/B/x + 2/B/x^2 + 6/B/x^3) = u in y = 1/x; below 100 the pieces
    // step up past u and the reference's search ends at 100
    const T c = B * q;
    T y = c;
    for (int it = 0; it < 60; ++it) {
      const T yn = y - (y + T(2) * y * y + T(6) * y * y * y - c) / (T(1) + T(4) * y + T(18) * y * y);
      const bool done = fabs(yn - y) <= MolTol<T>::newton * yn;
      y = yn;
      if (done) break;
    }
    return fmax(T(1) / y, T(100));
  }
  return x;
}

// get_capital_B (moliere.py:157-174): B = b + ln B from b + ln b, stopped at
// |B - (b + ln B)| <= 1e-3 (contraction 1/B < 1/3 for b >= 2; bounded).
template <class T>
__host__ __device__ __forceinline__ T moliere_B(T b) {
  T B = b + mlog(b);
  B = b + mlog(B);
  for (int it = 0; it < 200 && fabs(B - (b + mlog(B))) > T(1e-3); ++it) B = b + mlog(B);
  return B;
}

}  // namespace pt
