// pt_dark.cu -- dark-vector production and the differentiable dark yield.
//
//  * pt_run_dark: DarkShower.generate_dark_shower (dark_shower.py:806-849)
//    over an SM particle store.  One thread per (SM row, active dark process)
//    runs GetBSMWeights (:595-647) and produce_bsm_particle (:721-804): the
//    interaction energy from the dR/dE table, multiple scattering and the
//    continuous loss up to it, draw_dark_sample's accept/reject loop on the
//    dark map (:649-704), the bound-electron momentum (:706-719) and the
//    vector's four-momentum (kinematics.py:43-68,104-183,267-299).
//  * pt_dark_yield / pt_dark_yield_adjoint: the map estimate of a dark cross
//    section at fixed uniforms and its derivative with respect to the vector
//    mass, one block per (pair), samples split over the block's threads and
//    summed in a fixed order.
#include <cmath>
#include <cstdio>
#include <new>

#include "pt_dark.cuh"
#include "pt_internal.cuh"
#include "pt_physics.cuh"
#include "pt_physics32.cuh"

using namespace pt;

struct pt_dark {
  Tabs T;                 // SM tables of the bound handle
  pt_dark_maps M;
  int* status = nullptr;
  double* err_info = nullptr;
  unsigned long long* counter = nullptr;   // [0] vectors, [1] tasks, [2] tasks taken
  int* h_status = nullptr;
  unsigned long long* h_counter = nullptr;
  void* tasks = nullptr;                   // (row, process, weight) of a launch
  int64_t tasks_cap = 0;
};

namespace {

#define PT_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      fprintf(stderr, "petite_gpu: %s failed: %s\n", #call, cudaGetErrorString(e_)); \
      return PT_CUDA_ERR;                                                             \
    }                                                                                 \
  } while (0)

__device__ void dark_raise(int* status, double* info, int code, int process, double E, int key) {
  if (atomicCAS(status, 0, code) == 0 && info) {
    info[0] = process; info[1] = E; info[2] = key;
  }
}

constexpr int kMaxPeTrials = 1 << 22;   // draw_pe_sample accepts ~1 in 3 trials
constexpr unsigned kFull = 0xffffffffu;

// interp1d(kind='linear', bounds_error=False, fill_value=fill) on 1-D tables
__device__ __forceinline__ double interp_fill(const double* xs, const double* ys, int n, double v, double fill) {
  if (!(v >= xs[0]) || v > xs[n - 1]) return (v != v) ? v : fill;
  return interp_tab(xs, ys, n, v);
}

// ------------------------------------------------------------- dark maps
__device__ __forceinline__ int dark_lu_key(const pt_dark_maps& M, int block, double E) {
  const double* Ei = M.map_energy + M.map_base[block];
  const int n = M.map_rows[block];
  int lo = 0, hi = n;
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

__device__ __forceinline__ int dark_dim(int p) { return (p == PT_DARKBREM || p == PT_DARKMUONBREM) ? 3 : 1; }

template <class T>
__device__ __forceinline__ T dark_dsigma(const pt_dark_maps& M, int p, const double* x, double E, T mV) {
  switch (p) {
    case PT_DARKBREM: return dsig_dark_brem(x, E, mV, M.A, kMe, M.Z, M.A);
    case PT_DARKMUONBREM: return dsig_dark_brem(x, E, mV, M.A, kMmu, M.Z, M.A);
    case PT_DARKCOMP: return dsig_dark_compton(x[0], E, mV);
    default: return dsig_radiative_return(x[0], E, mV);
  }
}

// draw_dark_sample (dark_shower.py:649-704) as a state and one proposal at a
// time: up to max_n_integrators * neval proposals from the map row nearest
// E (its LU key), each accepted when max_F * u < wgt * f(x).
struct DarkDraw {
  int r, d, neval, key;
  double maxF, E;
  int64_t made, limit;          // proposals made; max_n_integrators * neval
  float maxF32, inv_neval32;    // the float32 proposals' acceptance ratio
  Screen32K sk;                 // the float32 dark-brem screen's constants
  Ann32K ak;                    // the float32 radiative-return screen's constants
};

__device__ __forceinline__ void dark_draw_begin(const pt_dark_maps& M, int block, int p, double E, double mV,
                                                int64_t max_n_integrators, DarkDraw& D) {
  D.key = dark_lu_key(M, block, E);
  D.r = M.map_base[block] + D.key;
  D.maxF = M.map_maxF[D.r];
  D.neval = (int)M.map_neval[D.r];
  D.d = dark_dim(p);
  D.E = E;
  D.made = 0;
  D.limit = max_n_integrators * (int64_t)D.neval;
  D.maxF32 = (float)D.maxF;
  D.inv_neval32 = 1.f / (float)D.neval;
  const bool brem = (p == PT_DARKBREM || p == PT_DARKMUONBREM);
  if (brem) {
    const double m = p == PT_DARKMUONBREM ? kMmu : kMe;
    D.sk = screen32_constants(E, mV, M.A, m, M.Z, M.A, (float)dark_brem_tconv(E, M.A, m));
  }
  if (p == PT_DARKANN) D.ak = ann32_constants(E, mV);
}

// One proposal: 1 accepted (x holds it), 0 rejected, -1 the limit was
// reached before it (the reference returns None).
__device__ int dark_propose(const pt_dark_maps& M, int p, double mV, DarkDraw& D, Rng& rng, double* x) {
  if (D.made >= D.limit) return -1;
  double jac = 1.0;
  for (int k = 0; k < D.d; ++k) {
    const double y = rng.u();
    x[k] = map_dim(M.grid_nodes + M.grid_offset[D.r * 4 + k], M.grid_ninc[D.r * 4 + k], y, jac);
  }
  const double wgt = jac / D.neval;
  ++D.made;
  const double u = rng.u();
  // Screen: a sample clearly outside the allowed region is rejected; where
  // the float32 estimate is trusted (its guards keep it within about 6e-3 of
  // the float64 value) and the proposal is rejected even at four times that
  // estimate, the float64 value cannot be accepted either.  Otherwise
  // float64 decides.  (Letting the estimate also accept, with a 5 % margin,
  // changed nothing measurable: the accepted proposals are few.)
  if (p == PT_DARKBREM || p == PT_DARKMUONBREM) {
    float f32;
    const int sc = dark_brem_screen32k((float)x[0], (float)x[1], (float)x[2], D.sk, f32);
    if (sc == kScreenOutside) return 0;                          // integrand 0: rejected
    if (sc == kScreenValue && D.maxF * u > 4.0 * wgt * (double)f32) return 0;
  }
  const double f = dark_dsigma<double>(M, p, x, D.E, mV);
  return D.maxF * u < wgt * f ? 1 : 0;
}

// The same proposal in float32 (pt_dark_params.precision = 1): the draws'
// float forms (the same draws, their top 24 bits), the map transform on the
// float32 grid, and the dark-brem screen decide whenever its estimate is
// trusted and the accept draw lies more than 2 % from the acceptance ratio
// (the screen is within 1 % of the float64 cross section wherever it
// returns a value), so such a decision is the float64 one at this sample.
// Otherwise the float64 cross section decides at the float32 sample.  x
// receives the sample (as float64) when it is accepted.
__device__ int dark_propose32(const pt_dark_maps& M, int p, double mV, DarkDraw& D, Rng& rng, const PhiloxRK& rk,
                              double* x) {
  if (D.made >= D.limit) return -1;
  float u[4];
  if (D.d == 3) {
    rng.take(u, rk);                                 // three y draws and the accept draw
  } else {
    float u2[2];
    rng.take(u2, rk);
    u[0] = u2[0];
    u[1] = u[2] = 0.f;
    u[3] = u2[1];
  }
  const float2* g2 = reinterpret_cast<const float2*>(M.grid_f32x2);
  float xf[3] = {0.f, 0.f, 0.f};
  float jac = 1.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (k < D.d) {
      const int ninc = M.grid_ninc[D.r * 4 + k];
      const float t = u[k] * (float)ninc;
      int i = (int)t;
      if (i > ninc - 1) i = ninc - 1;
      const float2 g = __ldg(g2 + M.grid_offset[D.r * 4 + k] + i);   // (node, increment)
      xf[k] = fmaf(g.y, t - (float)i, g.x);
      jac *= (float)ninc * g.y;
    }
  }
  ++D.made;
  const float wgt = jac * D.inv_neval32;
  const float ua = u[3];
  if ((p == PT_DARKBREM || p == PT_DARKMUONBREM)) {
    float f32;
    const int sc = dark_brem_screen32k(xf[0], xf[1], xf[2], D.sk, f32);
    if (sc == kScreenOutside) return 0;                          // integrand 0: rejected
    if (sc == kScreenValue && D.maxF32 > 0.f) {
      const float r = wgt * f32 / D.maxF32;
      if (ua > 1.02f * r) return 0;
      if (ua < 0.98f * r) {
        x[0] = xf[0]; x[1] = xf[1]; x[2] = xf[2];
        return 1;
      }
    }
  }
  x[0] = xf[0]; x[1] = xf[1]; x[2] = xf[2];
  const double f = dark_dsigma<double>(M, p, x, D.E, mV);
  return D.maxF * (double)ua < (double)wgt * f ? 1 : 0;
}

// A DarkAnn proposal of the float32 dark form: the float64 draws and map
// transform (the sample x is the float64 form's; the radiative-return map
// crowds its nodes against u = 1 closer than float32 resolves), the
// acceptance decided by the float32 screen when the accept draw lies more
// than 0.2 % from its ratio, else by the float64 cross section: the float64
// form's decisions and samples.
__device__ int dark_propose_ann32(const pt_dark_maps& M, double mV, DarkDraw& D, Rng& rng, double* x) {
  if (D.made >= D.limit) return -1;
  double jac = 1.0;
  x[0] = map_dim(M.grid_nodes + M.grid_offset[D.r * 4], M.grid_ninc[D.r * 4], rng.u(), jac);
  const double wgt = jac / D.neval;
  ++D.made;
  const double u = rng.u();
  float f32;
  if (ann_screen32(x[0], D.ak, f32) == kScreenValue && D.maxF32 > 0.f) {
    const float r = (float)wgt * f32 / D.maxF32, uf = (float)u;
    if (uf > 1.002f * r) return 0;
    if (uf < 0.998f * r) return 1;
  }
  const double f = dark_dsigma<double>(M, PT_DARKANN, x, D.E, mV);
  return D.maxF * u < wgt * f ? 1 : 0;
}

// The whole loop; false when no sample was found.
__device__ bool draw_dark(const pt_dark_maps& M, int block, int p, double E, double mV, int64_t max_n_integrators,
                          Rng& rng, double* x, int& key, int64_t& proposals) {
  DarkDraw D;
  dark_draw_begin(M, block, p, E, mV, max_n_integrators, D);
  key = D.key;
  int res;
  while ((res = dark_propose(M, p, mV, D, rng, x)) == 0) {
  }
  proposals = D.made;
  return res == 1;
}

// ----------------------------------------------------------- GetBSMWeights
__device__ double bsm_weight(const Tabs& T, const pt_dark_params& P, int pid, double E, int p) {
  if (!((P.active >> p) & 1)) return 0.0;
  int k;                                     // weight table / min_dark slot
  if (p == PT_DARKBREM && pid == 11) k = 0;
  else if (p == PT_DARKBREM && pid == -11) k = 1;
  else if (p == PT_DARKANN && pid == -11) k = 2;
  else if (p == PT_DARKCOMP && pid == 22) k = 3;
  else if (p == PT_DARKMUONBREM && (pid == 13 || pid == -13)) k = 4;
  else return 0.0;
  if (E < P.min_dark[k]) return 0.0;
  if (k == 3) {
    if (E < P.min_calc_photon) return 0.0;
    const double nd = pow(10.0, interp_fill(P.nsc_lx, P.nsc_ly, P.nsc_n, log10(E), -20.0));
    return P.coupling * nd / (nsig(T, 1, E) + nsig(T, 3, E));
  }
  const int w = (k == 4) ? 3 : k;
  if (k == 2 && !P.bound_electron) {
    // free electrons (dark_shower.py:619-630): the tabulated weight above the
    // first saved energy plus the resonant weight in closed form,
    // K (sMAX - mV^2)^beta exp(-(dII)/dEdx/cmtom) (shower.py:322-334)
    const double me = kMe;
    const double E0s = P.ann_E0;
    const S sMAX = S(2.0) * (S(me) * S(E0s < E ? E0s : E) + S(me) * S(me));
    const S beta = S(2.0) * S(kAlpha) / S(kPi) * (S(log((sMAX / (S(me) * S(me))).v)) - S(1.0));
    double pef = 0.0;
    const double Er = P.E_res;
    const double ds = ((S(interp_tab(P.ii_x[0], P.ii_y[0], P.ii_n[0], E)) - S(interp_tab(P.ii_x[0], P.ii_y[0], P.ii_n[0], Er))) +
                       (S(interp_tab(P.ii_x[1], P.ii_y[1], P.ii_n[1], E)) - S(interp_tab(P.ii_x[1], P.ii_y[1], P.ii_n[1], Er))) +
                       (S(interp_tab(P.ii_x[2], P.ii_y[2], P.ii_n[2], E)) - S(interp_tab(P.ii_x[2], P.ii_y[2], P.ii_n[2], Er)))).v;
    if (!(ds < 0.0 || Er > E)) pef = exp((S(-ds) / S(T.t.dEdx_GeV_per_m) / S(kCmToM)).v);
    const double wa = (S(P.ann_K) * S(pow((sMAX - S(P.mV) * S(P.mV)).v, beta.v)) * S(pef)).v;
    const double wn = E > E0s ? interp_tab(P.w_x[w], P.w_y[w], P.w_n[w], E) : 0.0;
    return (S(P.coupling) * (S(wn) + S(wa))).v;
  }
  return P.coupling * interp_tab(P.w_x[w], P.w_y[w], P.w_n[w], E);
}

// np.sum of the bin weights as numpy computes it for a short 1-D array:
// sequential below 8 elements, else eight partial sums combined pairwise and
// the remainder added in order.
__device__ double np_sum_weights(const double* bins, int nb) {
  if (nb < 8) {
    double tot = 0.0;
    for (int i = 0; i < nb; ++i) tot = (S(tot) + S(bins[2 * i + 1])).v;
    return tot;
  }
  double r[8];
  for (int i = 0; i < 8; ++i) r[i] = bins[2 * i + 1];
  int i = 8;
  for (; i + 8 <= nb; i += 8)
    for (int j = 0; j < 8; ++j) r[j] = (S(r[j]) + S(bins[2 * (i + j) + 1])).v;
  double tot = (((S(r[0]) + S(r[1])) + (S(r[2]) + S(r[3]))) + ((S(r[4]) + S(r[5])) + (S(r[6]) + S(r[7])))).v;
  for (; i < nb; ++i) tot = (S(tot) + S(bins[2 * i + 1])).v;
  return tot;
}

// numpy.random.choice(energies, p=w/tot): cumsum of w/tot, normalised by its
// last entry, searchsorted(u, side='right').
__device__ int drate_choice(const double* bins, int nb, double tot, double u) {
  double last = 0.0;
  for (int i = 0; i < nb; ++i) last = (S(last) + S(bins[2 * i + 1]) / S(tot)).v;
  double cum = 0.0;
  for (int i = 0; i < nb; ++i) {
    cum = (S(cum) + S(bins[2 * i + 1]) / S(tot)).v;
    if ((S(cum) / S(last)).v > u) return i;
  }
  return nb - 1;
}

struct DarkRow {
  int pid;
  double p0[4], pf[4], rf[3], mass, weight;
  uint64_t key;
};

// GetBSMWeights for TwoBody_BSMDecay (dark_shower.py:633-638): pi0 rows,
// 2 kappa^2 (1 - (mV/m)^2)^3 Br(pi0 -> gamma gamma) (particle.py:39-48), zero
// once mV >= m.  (The reference raises KeyError for eta and eta' rows, whose
// PIDs its threshold table lacks; the host refuses them before the launch.)
__device__ double twobody_weight(const pt_dark_params& P, int pid, double mass) {
  if (pid != 111) return 0.0;
  const S ratio = S(P.mV) / S(mass);
  if (!(ratio.v < 1.0)) return 0.0;
  const S omr = S(1.0) - sq(ratio);
  return (S(2.0) * sq(S(P.kinetic_mixing)) * (omr * omr * omr) * S(0.98823)).v;
}

// Particle.two_body_decay (particle.py:209-256) into (gamma, V), V kept: the
// rest-frame momenta, its two draws (cos theta on [-1, 1), phi on [0, 2 pi))
// and boost_matrix (particle.py:187-207) from the parent's final momentum and
// its mass.
__device__ void two_body_V(const DarkRow& r, double mV, Rng& rng, double* V) {
  const S mX(r.mass), m1(0.0), m2(mV);
  const S E1 = (sq(mX) - sq(m2) + sq(m1)) / (S(2.0) * mX);
  const S E2 = (sq(mX) - sq(m1) + sq(m2)) / (S(2.0) * mX);
  const S pF = ssqrt(sq(E1) - sq(m1));
  const S ct = S(-1.0) + (S(1.0) - S(-1.0)) * S(rng.u());
  const S phi = S(0.0) + (S(2.0 * kPi) - S(0.0)) * S(rng.u());
  const S st = ssqrt(S(1.0) - sq(ct));
  const S q[4] = {E2, pF * st * S(sin(phi.v)), pF * st * S(cos(phi.v)), pF * ct};
  const double px = r.pf[1], py = r.pf[2], pz = r.pf[3];
  const double pmag = norm3_np(px, py, pz);
  if (pmag == 0.0) {                              // np.identity(4)
    for (int i = 0; i < 4; ++i) V[i] = q[i].v;
    return;
  }
  const S gamma = S(r.pf[0]) / mX;
  const S beta = gamma.v == 1.0 ? S(1.0) : ssqrt(S(1.0) - S(1.0) / sq(gamma));
  const S b[3] = {beta * S(px) / S(pmag), beta * S(py) / S(pmag), beta * S(pz) / S(pmag)};
  const S g1 = gamma - S(1.0), b2 = sq(beta);
  S M[4][4];
  M[0][0] = gamma;
  for (int i = 0; i < 3; ++i) { M[0][i + 1] = gamma * b[i]; M[i + 1][0] = gamma * b[i]; }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      M[i + 1][j + 1] = i == j ? S(1.0) + g1 * sq(b[i]) / b2 : g1 * b[i] * b[j] / b2;
  for (int i = 0; i < 4; ++i) V[i] = (M[i][0] * q[0] + M[i][1] * q[1] + M[i][2] * q[2] + M[i][3] * q[3]).v;
}

// produce_bsm_particle (dark_shower.py:721-804) in three stages, so that a
// lane can run the map's accept/reject loop one proposal at a time.
//
// Stage 1: the interaction energy from dR/dE, multiple scattering and the
// continuous loss up to it (pf becomes the parent's momentum there), and the
// thresholds' closed forms.  Returns 0 when the reference returns None, 1
// when the vector is known (v, in pf's frame), 2 when the map draw follows
// (D set up for dark_propose).
__device__ int bsm_begin(const Tabs& T, const pt_dark_maps& M, const pt_dark_params& P, const pt_opts& o,
                         const DarkRow& r, int p, Rng& rng, double* pf, V4& v, DarkDraw& D,
                         const PhiloxRK* rk = nullptr) {
  for (int c = 0; c < 4; ++c) pf[c] = r.pf[c];
  int table = -1;
  if (p == PT_DARKANN && r.pid == -11) table = 2;
  else if (p == PT_DARKBREM) table = (r.pid == 11) ? 0 : 1;
  else if (p == PT_DARKMUONBREM) table = 3;
  if (table >= 0) {
    const double* Ei = P.dr_Ei[table];
    const int n = P.dr_n[table];
    const double E0 = r.p0[0];
    int j;
    if (E0 < Ei[0]) j = 0;
    else if (E0 > Ei[n - 1]) j = n - 1;
    else {                                            // largest saved energy <= E0
      int lo = 0, hi = n - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (Ei[mid] <= E0) lo = mid; else hi = mid - 1;
      }
      j = lo;
    }
    const double* bins = P.dr_bins[table] + (size_t)j * P.dr_nbmax[table] * 2;
    const int nb = P.dr_nbins[table][j];
    const double tot = np_sum_weights(bins, nb);
    if (tot == 0.0) return 0;                     // dark_shower.py:742-743, before any draw
    const int idx = drate_choice(bins, nb, tot, rng.u());
    const double E_int = (S(bins[2 * idx]) + (S(E0) - S(Ei[j]))).v;
    const double dEdx = T.t.dEdx_GeV_per_m;
    const double dist = ((S(E0) - S(E_int)) / S(dEdx)).v;
    double ps[4] = {r.p0[0], r.p0[1], r.p0[2], r.p0[3]};
    const double tms = (S(T.t.rho) * (S(dist) / S(kCmToM))).v;
    if (rk && o.mcs_mode == 0) {
      // the float32 form (rk given): Lynch-Dahl scattering on the same four
      // draws in float32 (as the mixed SM engine scatters), the momentum's
      // magnitude kept in float64
      const float fx = (float)ps[1], fy = (float)ps[2], fz = (float)ps[3], fE = (float)ps[0];
      const float pn = sqrtf(fx * fx + fy * fy + fz * fz);
      if (pn > 0.f) {
        float u4[4];
        rng.take(u4, *rk);
        float3 dir = make_float3(fx / pn, fy / pn, fz / pn);
        mcs32_u(dir, pn * ((float)kMe / (float)r.mass), fE, (float)tms, (float)T.t.A, (float)T.t.Z,
                (float)T.t.Z23, (float)o.rescale_MCS, u4[0], u4[2], u4[3], pn / fE);
        const double pnd = norm3_np(ps[1], ps[2], ps[3]);
        ps[1] = pnd * (double)dir.x; ps[2] = pnd * (double)dir.y; ps[3] = pnd * (double)dir.z;
      }
    } else {
      mcs_apply(o.mcs_mode, ps, tms, T.t, o.rescale_MCS, kMe, rng);
    }
    pf[0] = ps[0]; pf[1] = ps[1]; pf[2] = ps[2]; pf[3] = ps[3];
    lose_energy(pf, r.mass, (S(E0) - S(E_int)).v);
  }
  const double E0 = pf[0];
  const double mV = P.mV, me = kMe;
  const bool bound = P.bound_electron != 0;
  if (p == PT_DARKANN && bound && E0 <= P.E_res) {
    const double pz = sqrt((S(E0) * S(E0) - S(me) * S(me)).v);
    v = {sqrt((S(E0) * S(E0) - S(me) * S(me) + S(mV) * S(mV)).v), 0.0, 0.0, pz};
    return 1;
  }
  if (p == PT_DARKCOMP && bound && E0 <= P.E_compth) {
    v = {sqrt((S(E0) * S(E0) + S(mV) * S(mV)).v), 0.0, 0.0, E0};
    return 1;
  }
  if (p == PT_DARKANN && !bound && E0 <= P.ann_E0) {
    // free electrons below the first saved energy (dark_shower.py:767-768)
    v = {P.E_res, 0.0, 0.0, sqrt((S(P.E_res) * S(P.E_res) - S(mV) * S(mV)).v)};
    return 1;
  }
  dark_draw_begin(M, P.mass_index * PT_N_DARK + p, p, E0, mV, o.max_n_integrators, D);
  return 2;
}

// Stage 3: the vector from the accepted sample x (kinematics.py:43-68,
// 104-183, 267-299 and draw_pe_sample, dark_shower.py:706-719), in the
// frame of the parent's momentum (energy E0).  false: the reference's None
// (draw_pe_sample's bounded loop ran out; PT_TIMEOUT is recorded).
// draw_pe_sample's acceptance test, uu < wave(pe) / wave(lam / sqrt 3), in
// float32: with t = pe / lam the ratio is (256/27) t^2 / (t^2 + 1)^4.  The
// float32 form decides when the accept draw lies more than 1e-3 (relative)
// from it -- far above its error, so the decision is the float64 one -- and
// returns -1 otherwise.
__device__ __forceinline__ int pe_accept32(uint64_t dx, uint64_t du, float inv_lam) {
  const float xx = __uint2float_rn((uint32_t)(dx >> 40)) * 0x1p-24f * 1e-3f;
  const float uu = __uint2float_rn((uint32_t)(du >> 40)) * 0x1p-24f;
  const float t = xx * inv_lam, t2 = t * t, q = t2 + 1.f, q2 = q * q;
  const float ratio = (256.f / 27.f) * t2 / (q2 * q2);
  if (uu < 0.999f * ratio) return 1;
  if (uu > 1.001f * ratio) return 0;
  return -1;
}

__device__ bool bsm_finish(const pt_dark_params& P, const DarkRow& r, int p, double E0, const double* x, Rng& rng,
                           double& wg, V4& v, int* status, double* info, bool f32 = false) {
  const double mV = P.mV, me = kMe;
  const bool bound = P.bound_electron != 0;
  if (p == PT_DARKCOMP && bound) {
    // draw_pe_sample (dark_shower.py:706-719)
    const S lam = S(kAlpha) * S(P.Zeff) * S(me);
    const S lam5(pow(lam.v, 5.0));
    auto wave = [&](S pe) {
      return S(32.0) / S(kPi) * lam5 * (pe * pe) / S(pow((pe * pe + lam * lam).v, 4.0));
    };
    const S c = wave(lam / S(sqrt(3.0)));
    double pe = -1.0;
    const float inv_lam = 1.f / (float)lam.v;
    for (int it = 0; it < kMaxPeTrials; ++it) {
      // the draws as rng.u() takes them; the float32 form tests them in
      // float32 first (pe_accept32) and in float64 only near the boundary
      const uint64_t dx = rng.next_u64(), du = rng.next_u64();
      const int a = f32 ? pe_accept32(dx, du, inv_lam) : -1;
      const S xx = S(0.0) + (S(1e-3) - S(0.0)) * S((double)(dx >> 11) * 0x1p-53);
      if (a == 1) { pe = xx.v; break; }
      if (a == 0) continue;
      const S uu = S(0.0) + (S(1.0) - S(0.0)) * S((double)(du >> 11) * 0x1p-53);
      if (uu.v < (wave(xx) / c).v) { pe = xx.v; break; }
    }
    if (pe < 0.0) { dark_raise(status, info, PT_TIMEOUT, p, E0, 0); return false; }
    const double c0 = (S(-1.0) + (S(1.0) - S(-1.0)) * S(rng.u())).v;
    const S s = S(me) * S(me) + S(2.0) * S(E0) * (ssqrt(S(me) * S(me) + S(pe) * S(pe)) - S(c0) * S(pe));
    const S Ee = (s - S(mV) * S(mV) + S(me) * S(me)) / (S(2.0) * ssqrt(s));
    if (Ee.v < me) {
      v = {mV, 0.0, 0.0, 0.0};
      wg = 0.0;
    } else {
      // compton_fourvecs_boundelectron (kinematics.py:134-183), the V row
      const S Eg(E0), ct(x[0]), Pe(pe), cte(c0), mv(mV), m(me);
      const S rs = ssqrt(s);
      const S EV = (s + mv * mv - m * m) / (S(2.0) * rs);
      const S pF = ssqrt(Ee * Ee - m * m);
      const S bnum = ssqrt(Eg * Eg + S(2.0) * cte * Eg * Pe + Pe * Pe);
      const S bden = Eg + ssqrt(m * m + Pe * Pe);
      const S b0 = bnum / bden;
      const S g0 = S(1.0) / ssqrt(S(1.0) - b0 * b0);
      const S ph = S(0.0) + (S(2.0 * kPi) - S(0.0)) * S(rng.u());
      const S st = ssqrt(S(1.0) - ct * ct);
      const S EVL = g0 * EV - b0 * g0 * pF * ct;
      const S a0 = pF * st * S(sin(ph.v)), a1 = pF * st * S(cos(ph.v)), a2 = b0 * g0 * EV - g0 * pF * ct;
      const S ctz = (Eg + cte * Pe) / ssqrt(Eg * Eg + S(2.0) * cte * Eg * Pe + Pe * Pe);
      const S stz = ssqrt(S(1.0) - ctz * ctz);
      const S phe = S(0.0) + (S(2.0 * kPi) - S(0.0)) * S(rng.u());
      const S cf(cos(phe.v)), sf(sin(phe.v));
      v = {EVL.v, (ctz * cf * a0 + (-sf) * a1 + stz * cf * a2).v, (ctz * sf * a0 + cf * a1 + stz * sf * a2).v,
           ((-stz) * a0 + S(0.0) * a1 + ctz * a2).v};
    }
  } else if (p == PT_DARKBREM || p == PT_DARKMUONBREM) {
    // l_to_lV_fourvecs (kinematics.py:43-68), the V row
    const S ep(E0), m(r.mass), mv(mV);
    const S w = S(x[0]) * ep;
    const S ct = S(1.0) - S(pow(10.0, x[1]));
    const S k = ssqrt(w * w - mv * mv);
    const S al = S(0.0) + (S(2.0 * kPi) - S(0.0)) * S(rng.u());
    const S cal(cos(al.v)), sal(sin(al.v));
    const S st = ssqrt(S(1.0) - ct * ct);
    (void)m;
    v = {w.v, (k * cal * st).v, (k * sal * st).v, (k * ct).v};
  } else if (p == PT_DARKANN) {
    // radiative_return_fourvecs (kinematics.py:267-299) with boost
    // (radiative_return.py:18-24)
    const S s = S(2.0) * S(me) * (S(me) + S(E0));
    const double beta = (S(2.0) * S(kAlpha) / S(kPi) * (S(log((s / (S(me) * S(me))).v)) - S(1.0))).v;
    const S umax = S(pow((S(1.0) - S(mV) * S(mV) / s).v, beta / 2.0));
    const S x1 = S(1.0) - S(pow((S(x[0]) * umax).v, 2.0 / beta));
    const S x2 = S(mV) * S(mV) / (x1 * s);
    const S rs = ssqrt(s);
    const S E1 = x1 * rs / S(2.0), E2 = x2 * rs / S(2.0);
    const S q0 = rs / S(2.0), q3 = -ssqrt(s / S(4.0) - S(me) * S(me));
    const S w0 = E1 + E2, w3 = E1 + (-E2);
    const S rsq = ssqrt(q0 * q0 - S(0.0) * S(0.0) - S(0.0) * S(0.0) - q3 * q3);
    const S v0 = (q0 * w0 - S(0.0) * S(0.0) - S(0.0) * S(0.0) - q3 * w3) / rsq;
    const S c1 = (w0 + v0) / (rsq + q0);
    v = {v0.v, (S(0.0) - c1 * S(0.0)).v, (S(0.0) - c1 * S(0.0)).v, (w3 - c1 * q3).v};
  } else {
    // compton_fourvecs with mV (kinematics.py:104-132), the V row
    const S Eg(E0), ct(x[0]), m(me), mv(mV);
    const S s = m * m + S(2.0) * Eg * m;
    const S rs = ssqrt(s);
    const S Ee0 = (s + m * m) / (S(2.0) * rs);
    const S Ee = (s - mv * mv + m * m) / (S(2.0) * rs);
    const S EV = (s + mv * mv - m * m) / (S(2.0) * rs);
    const S pF = ssqrt(Ee * Ee - m * m);
    const S g0 = Ee0 / m;
    const S b0 = S(1.0) / g0 * ssqrt(g0 * g0 - S(1.0));
    const S ph = S(0.0) + (S(2.0 * kPi) - S(0.0)) * S(rng.u());
    const S st = ssqrt(S(1.0) - ct * ct);
    v = {(g0 * EV - b0 * g0 * pF * ct).v, (pF * st * S(sin(ph.v))).v, (pF * st * S(cos(ph.v))).v,
         (b0 * g0 * EV - g0 * pF * ct).v};
  }
  return true;
}

// The three stages in one call.  Returns false when the reference returns
// None; on true, V and wg hold the vector (lab frame) and its weight.
__device__ bool produce_bsm(const Tabs& T, const pt_dark_maps& M, const pt_dark_params& P, const pt_opts& o,
                            const DarkRow& r, int p, double& wg, double* V, Rng& rng, int* status, double* info) {
  double pf[4];
  V4 v;
  DarkDraw D;
  const int s = bsm_begin(T, M, P, o, r, p, rng, pf, v, D);
  if (s == 0) return false;
  if (s == 2) {
    double x[4] = {0, 0, 0, 0};
    int res;
    while ((res = dark_propose(M, p, P.mV, D, rng, x)) == 0) {
    }
    if (res < 0) return false;
    if (!bsm_finish(P, r, p, pf[0], x, rng, wg, v, status, info)) return false;
  }
  const V4 lab = to_lab(rotation_from(pf), v);
  V[0] = lab.e; V[1] = lab.x; V[2] = lab.y; V[3] = lab.z;
  return true;
}

// A vector and its weight: the yields, and its record when out.p4 is set.
__device__ void dark_emit(const pt_dark_params& P, const pt_dark_out& out, unsigned long long* counter, int* status,
                          const DarkRow& r, int64_t row, int p, double wg, const double* V, uint64_t draws) {
  const double w = (S(wg) * S(r.weight)).v;
  if (out.yield) atomicAdd(out.yield + p, w);
  if (out.yield_E) atomicAdd(out.yield_E + p, w * V[0]);
  if (out.hist.counts) {
    const pt_dark_hist& H = out.hist;
    const double f = (log10(V[0]) - H.log10_lo) / (H.log10_hi - H.log10_lo);
    int b = f >= 0.0 ? (int)(f * H.bins) : 0;         // NaN and underflow: the first bin
    if (b > H.bins - 1) b = H.bins - 1;
    atomicAdd(H.counts + (size_t)p * H.bins + b, w);
  }
  const unsigned long long slot = atomicAdd(counter, 1ull);   // vectors produced (returned in *n_out)
  if (!out.p4) return;
  if ((int64_t)slot >= out.capacity) { dark_raise(status, nullptr, PT_OOM, p, r.p0[0], 0); return; }
  const int64_t oc = out.capacity;
  for (int c = 0; c < 4; ++c) out.p4[c * oc + slot] = V[c];
  for (int c = 0; c < 3; ++c) out.r[c * oc + slot] = r.rf[c];
  out.weight[slot] = w;
  out.parent[slot] = row;
  out.process[slot] = p == PT_TWOBODY ? PT_TWOBODY_CODE
                                      : p + ((P.bound_electron && (p == PT_DARKANN || p == PT_DARKCOMP)) ? PT_DARK_BOUND : 0);
  out.draws[slot] = (int32_t)draws;
}

__device__ __forceinline__ void load_row(const pt_particles& sm, int64_t row, DarkRow& r) {
  const int64_t cap = sm.capacity;
  r.pid = sm.pid[row];
  for (int c = 0; c < 4; ++c) { r.p0[c] = sm.p0[c * cap + row]; r.pf[c] = sm.pf[c * cap + row]; }
  for (int c = 0; c < 3; ++c) r.rf[c] = sm.rf[c * cap + row];
  r.mass = sm.mass[row];
  r.weight = sm.weight[row];
  r.key = sm.pkey[row];
}

// The (row, process) pairs of a dark run with a positive GetBSMWeights
// (dark_shower.py:595-647), compacted: most pairs weigh nothing (a photon
// has no DarkBrem), so the production below runs only on the others.
struct DarkTasks {
  int64_t* row;
  int32_t* proc;
  double* wg;
  int64_t cap;
};

__global__ void k_dark_weigh(Tabs T, pt_dark_params P, pt_particles sm, int64_t n_rows, int ncol, DarkTasks tk,
                             unsigned long long* counter, int* status) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double wg = 0.0;
  int p = 0;
  int64_t row = 0;
  if (t < n_rows * ncol) {
    // column PT_TWOBODY (launched when active) decays the pi0 rows
    p = (int)(t / n_rows);
    row = t - (int64_t)p * n_rows;
    const int pid = sm.pid[row];
    if (p == PT_TWOBODY) wg = twobody_weight(P, pid, sm.mass[row]);
    else wg = bsm_weight(T, P, pid, sm.p0[row], p);
  }
  const bool keep = wg > 0.0;
  const unsigned m = __ballot_sync(kFull, keep);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(counter + 1, (unsigned long long)__popc(m));
  base = __shfl_sync(kFull, base, leader);
  if (!keep) return;
  const unsigned long long slot = base + __popc(m & ((1u << lane) - 1u));
  if ((int64_t)slot >= tk.cap) { dark_raise(status, nullptr, PT_OOM, p, 0.0, 0); return; }
  tk.row[slot] = row;
  tk.proc[slot] = p;
  tk.wg[slot] = wg;
}

// produce_bsm_particle over the tasks with every lane busy: a lane takes a
// task, runs its first stage, then one map proposal per iteration; a lane
// whose task ends (vector made, or None) takes the next one while the other
// lanes keep proposing.  Each task draws from its own stream, in the
// reference's order, so the vectors are produce_bsm's whatever the schedule.
constexpr int kDarkThreads = 128;
template <int PREC>
__global__ void __launch_bounds__(kDarkThreads) k_dark_produce(Tabs T, pt_dark_maps M, pt_dark_params P, pt_opts o,
                                                               pt_particles sm, DarkTasks tk, pt_dark_out out,
                                                               unsigned long long* counter, int* status,
                                                               double* info, PhiloxRK rk) {
  const int lane = threadIdx.x & 31;
  const unsigned long long nt = __ldcg(counter + 1);
  const int64_t n = (int64_t)nt < tk.cap ? (int64_t)nt : tk.cap;
  bool have = false, drained = false;
  DarkRow r;
  int p = 0;
  int64_t row = 0;
  double wg = 0.0, pf[4], x[4] = {0, 0, 0, 0};
  Rng rng;
  DarkDraw D;
  for (;;) {
    const bool want = !have && !drained;
    const unsigned m = __ballot_sync(kFull, want);
    int64_t t = -1;
    if (m) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(counter + 2, (unsigned long long)__popc(m));
      base = __shfl_sync(kFull, base, leader);
      if (want) {
        t = (int64_t)(base + __popc(m & ((1u << lane) - 1u)));
        if (t >= n) {
          drained = true;
          t = -1;
        }
      }
    }
    if (__all_sync(kFull, !have && drained)) break;
    if (t >= 0) {
      row = tk.row[t];
      p = tk.proc[t];
      wg = tk.wg[t];
      load_row(sm, row, r);
      rng.init(o.seed, mix64(r.key + 0x9E3779B97F4A7C15ull * (uint64_t)(3 + p)));
      double V[4];
      if (p == PT_TWOBODY) {
        two_body_V(r, P.mV, rng, V);
        dark_emit(P, out, counter, status, r, row, p, wg, V, rng.n);
      } else {
        V4 v;
        const int s = bsm_begin(T, M, P, o, r, p, rng, pf, v, D, PREC == 1 ? &rk : nullptr);
        if (s == 1) {
          const V4 lab = to_lab(rotation_from(pf), v);
          V[0] = lab.e; V[1] = lab.x; V[2] = lab.y; V[3] = lab.z;
          dark_emit(P, out, counter, status, r, row, p, wg, V, rng.n);
        }
        have = s == 2;
      }
    }
    if (have) {
      // the float32 proposals serve the 3-D dark bremsstrahlung maps; the 1-D
      // maps keep float64 (the radiative-return map crowds its nodes against
      // u = 1, closer than float32 resolves)
      const bool f32 = PREC == 1 && (p == PT_DARKBREM || p == PT_DARKMUONBREM);
      const int res = f32 ? dark_propose32(M, p, P.mV, D, rng, rk, x)
                          : (PREC == 1 && p == PT_DARKANN) ? dark_propose_ann32(M, P.mV, D, rng, x)
                                                           : dark_propose(M, p, P.mV, D, rng, x);
      if (res != 0) {
        have = false;
        V4 v;
        if (res == 1 && bsm_finish(P, r, p, pf[0], x, rng, wg, v, status, info, PREC == 1)) {
          const V4 lab = to_lab(rotation_from(pf), v);
          const double V[4] = {lab.e, lab.x, lab.y, lab.z};
          dark_emit(P, out, counter, status, r, row, p, wg, V, rng.n);
        }
      }
    }
  }
}

__global__ void k_dark_sample_only(pt_dark_maps M, pt_dark_params P, int p, const double* E, const uint64_t* key,
                                   int64_t n, uint64_t seed, int64_t max_n_integrators, double* x, int64_t* props,
                                   int32_t* keys) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Rng rng;
  rng.init(seed, key[i]);
  double xx[4] = {0, 0, 0, 0};
  int lk;
  int64_t pr;
  const bool ok = draw_dark(M, P.mass_index * PT_N_DARK + p, p, E[i], P.mV, max_n_integrators, rng, xx, lk, pr);
  for (int k = 0; k < 4; ++k) x[i * 4 + k] = xx[k];
  props[i] = ok ? pr : -1;
  keys[i] = lk;
}

__global__ void k_dark_screen(pt_dark_maps M, int p, const double* x, const double* E, int64_t n, double mV,
                              float* value, int32_t* code) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xx[4];
  for (int k = 0; k < 4; ++k) xx[k] = x[i * 4 + k];
  float f = 0.f;
  if (p == PT_DARKANN) {
    code[i] = ann_screen32(xx[0], ann32_constants(E[i], mV), f);
  } else {
    const double mlep = p == PT_DARKMUONBREM ? kMmu : kMe;
    code[i] = dark_brem_screen32(xx, E[i], mV, M.A, mlep, M.Z, M.A, (float)dark_brem_tconv(E[i], M.A, mlep), f);
  }
  value[i] = f;
}

__global__ void k_dark_dsigma(pt_dark_maps M, int p, const double* x, const double* E, int64_t n, double mV,
                              double* out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xx[4];
  for (int k = 0; k < 4; ++k) xx[k] = x[i * 4 + k];
  out[i] = dark_dsigma<double>(M, p, xx, E[i], mV);
}

// ------------------------------------------------------------- dark yield
constexpr int kYieldThreads = 256;

template <class T>
__device__ __forceinline__ T dark_EV(int p, const double* x, double E, T mV) {
  if (p == PT_DARKCOMP) return dark_compton_EV(x[0], E, mV);
  if (p == PT_DARKANN) return dark_ann_EV(x[0], E, mV);
  return T(mV * 0.0) + x[0] * E;               // l_to_lV: E_V = x E
}
// E_V of the anchored dark-brem sample: x moves with mV as in
// dsig_dark_brem_anchored
template <class T>
__device__ __forceinline__ T dark_EV_anchored(const double* x, double E, T mV, double a) {
  const double xa = a / E;
  const double w = (x[0] - xa) / (1.0 - xa);
  const T xm = mV / E;
  return (xm + w * (1.0 - xm)) * E;
}

// One block per pair.  Sample j uses draws 4j..4j+3 of the pair's stream
// (Philox blocks 2j and 2j+1); the block's partial sums are combined in a
// fixed tree order, so results do not depend on timing.
template <class T, bool ADJ>
__global__ void __launch_bounds__(kYieldThreads) k_dark_yield(pt_dark_maps M, int p, const double* Ein,
                                                               const double* mVin, const double* anchor,
                                                               const int32_t* mass_index, int64_t n_samples,
                                                               uint64_t seed, double* yield, double* moment,
                                                               const double* gY, const double* gM, double* g_mV) {
  __shared__ double sh_y[kYieldThreads], sh_m[kYieldThreads];
  const int64_t i = blockIdx.x;
  const double E = Ein[i];
  T mV;
  if constexpr (ADJ) mV = T{mVin[i], 1.0};
  else mV = mVin[i];
  const int mi = mass_index[i];
  const int block = mi * PT_N_DARK + p;
  if (mi < 0 || mi >= M.n_masses || M.map_rows[block] < 2) {
    // no maps for this process at this mass (DarkAnn below mV = 2 m_e): it
    // makes no vectors, so its yield and moment are 0 (uniform per block)
    if (threadIdx.x == 0) {
      if constexpr (ADJ) g_mV[i] = 0.0;
      else { yield[i] = 0.0; moment[i] = 0.0; }
    }
    return;
  }
  const int key = dark_lu_key(M, block, E);
  const int r = M.map_base[block] + key;
  const int d = dark_dim(p);
  const uint32_t s0 = (uint32_t)seed, s1 = (uint32_t)(seed >> 32);
  const uint64_t skey = mix64((uint64_t)i * 4 + (uint64_t)p + 1);
  const uint32_t k0 = (uint32_t)skey, k1 = (uint32_t)(skey >> 32);
  double acc_y = 0.0, acc_m = 0.0;
  for (int64_t j = threadIdx.x; j < n_samples; j += kYieldThreads) {
    double u[4];
    const uint64_t b0 = 2 * (uint64_t)j;
    uint4 o = philox4x32_10(make_uint4((uint32_t)b0, (uint32_t)(b0 >> 32), k0, k1), s0, s1);
    u[0] = (double)(((uint64_t)o.x | ((uint64_t)o.y << 32)) >> 11) * 0x1p-53;
    u[1] = (double)(((uint64_t)o.z | ((uint64_t)o.w << 32)) >> 11) * 0x1p-53;
    if (d > 2) {
      const uint64_t b1 = b0 + 1;
      o = philox4x32_10(make_uint4((uint32_t)b1, (uint32_t)(b1 >> 32), k0, k1), s0, s1);
      u[2] = (double)(((uint64_t)o.x | ((uint64_t)o.y << 32)) >> 11) * 0x1p-53;
      u[3] = 0.0;
    }
    double x[4] = {0, 0, 0, 0};
    double jac = 1.0;
    for (int k = 0; k < d; ++k) x[k] = map_dim(M.grid_nodes + M.grid_offset[r * 4 + k], M.grid_ninc[r * 4 + k], u[k], jac);
    T f, ev;
    const bool brem = (p == PT_DARKBREM || p == PT_DARKMUONBREM);
    if (brem && (ADJ || anchor)) {
      // the kinematic ranges follow mV (d/dmV includes the moving edges)
      const double a = ADJ ? mVin[i] : anchor[i];
      f = dsig_dark_brem_anchored<T>(x, E, mV, a, M.A, p == PT_DARKBREM ? kMe : kMmu, M.Z, M.A);
      if (val(f) == 0.0) continue;               // outside the allowed region: no value, no derivative
      ev = dark_EV_anchored<T>(x, E, mV, a);
    } else {
      f = (p == PT_DARKANN) ? dsig_radiative_return<T, true>(x[0], E, mV) : dark_dsigma<T>(M, p, x, E, mV);
      if (val(f) == 0.0) continue;
      ev = dark_EV<T>(p, x, E, mV);
    }
    const T fe = f * ev;
    if constexpr (ADJ) {
      acc_y += jac * f.d;
      acc_m += jac * fe.d;
    } else {
      acc_y += jac * f;
      acc_m += jac * fe;
    }
  }
  sh_y[threadIdx.x] = acc_y;
  sh_m[threadIdx.x] = acc_m;
  __syncthreads();
  for (int w = kYieldThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh_y[threadIdx.x] += sh_y[threadIdx.x + w];
      sh_m[threadIdx.x] += sh_m[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double ny = sh_y[0] / (double)n_samples, nm = sh_m[0] / (double)n_samples;
    if constexpr (ADJ) g_mV[i] = gY[i] * ny + gM[i] * nm;
    else { yield[i] = ny; moment[i] = nm; }
  }
}

pt_status read_dark_status(pt_dark* d, cudaStream_t st) {
  PT_CUDA(cudaMemcpyAsync(d->h_status, d->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  PT_CUDA(cudaStreamSynchronize(st));
  return (pt_status)d->h_status[0];
}

}  // namespace

// The dark production over rows [0, n_rows) of sm for one parameter set, on
// the stream without a host wait: k_dark_weigh compacts the (row, process)
// pairs of positive weight into the handle's task buffer (grown to n_rows *
// ncol entries), then k_dark_produce runs them on a resident grid.
static pt_status dark_launch(pt_dark* d, const pt_dark_params& prm, const pt_opts& o, const pt_particles& sm,
                             int64_t n_rows, int ncol, const pt_dark_out& out, cudaStream_t st) {
  const int64_t work = n_rows * ncol;
  if (work <= 0) return PT_OK;
  if (d->tasks_cap < work) {
    PT_CUDA(cudaStreamSynchronize(st));             // no launch still reads the old buffer
    cudaFree(d->tasks);
    d->tasks = nullptr;
    d->tasks_cap = 0;
    const size_t bytes = (size_t)work * (sizeof(int64_t) + sizeof(int32_t) + sizeof(double)) + 512;
    if (cudaMalloc(&d->tasks, bytes) != cudaSuccess) {     // a device allocation: not PT_OOM (see pt_run_dark)
      cudaGetLastError();
      d->tasks = nullptr;
      fprintf(stderr, "petite_gpu: no device memory for %zu bytes of dark tasks\n", bytes);
      return PT_CUDA_ERR;
    }
    d->tasks_cap = work;
  }
  DarkTasks tk;
  tk.cap = d->tasks_cap;
  char* q = (char*)d->tasks;
  tk.row = (int64_t*)q;
  q += ((size_t)tk.cap * sizeof(int64_t) + 255) & ~size_t(255);
  tk.wg = (double*)q;
  q += ((size_t)tk.cap * sizeof(double) + 255) & ~size_t(255);
  tk.proc = (int32_t*)q;
  PT_CUDA(cudaMemsetAsync(d->counter + 1, 0, 2 * sizeof(unsigned long long), st));
  const int tb = 128;
  k_dark_weigh<<<(unsigned)((work + tb - 1) / tb), tb, 0, st>>>(d->T, prm, sm, n_rows, ncol, tk, d->counter,
                                                               d->status);
  int dev = 0, sms = 0, per = 0;
  PT_CUDA(cudaGetDevice(&dev));
  PT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const bool f32 = prm.precision == 1;
  const void* kern = f32 ? (const void*)k_dark_produce<1> : (const void*)k_dark_produce<0>;
  PT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kDarkThreads, 0));
  if (per < 1) per = 1;
  int64_t grid = (int64_t)sms * per;
  const int64_t need = (work + kDarkThreads - 1) / kDarkThreads;
  if (grid > need) grid = need;
  const PhiloxRK rk = philox_round_keys(o.seed);
  if (f32)
    k_dark_produce<1><<<(unsigned)grid, kDarkThreads, 0, st>>>(d->T, d->M, prm, o, sm, tk, out, d->counter,
                                                               d->status, d->err_info, rk);
  else
    k_dark_produce<0><<<(unsigned)grid, kDarkThreads, 0, st>>>(d->T, d->M, prm, o, sm, tk, out, d->counter,
                                                               d->status, d->err_info, rk);
  PT_CUDA(cudaGetLastError());
  return PT_OK;
}

extern "C" pt_status pt_dark_create(pt_handle* sm, const pt_dark_maps* m, pt_dark** out) {
  if (!sm || !m || !out) return PT_BAD_ARG;
  *out = nullptr;
  if (m->n_masses <= 0 || m->n_masses > PT_DARK_MAX_MASSES || m->n_rows <= 0 || !m->map_energy || !m->map_maxF ||
      !m->map_neval || !m->grid_offset || !m->grid_ninc || !m->grid_nodes)
    return PT_BAD_TABLE;
  for (int b = 0; b < m->n_masses * PT_N_DARK; ++b)
    if (m->map_rows[b] < 0 || m->map_base[b] < 0 || m->map_base[b] + m->map_rows[b] > m->n_rows) return PT_BAD_TABLE;
  pt_dark* d = new (std::nothrow) pt_dark();
  if (!d) return PT_OOM;
  d->T = *handle_parts(sm).T;
  d->M = *m;
  if (cudaMalloc(&d->status, sizeof(int)) != cudaSuccess || cudaMalloc(&d->err_info, 4 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d->counter, 3 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&d->h_status, sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&d->h_counter, sizeof(unsigned long long)) != cudaSuccess) {
    pt_dark_destroy(d);
    return PT_CUDA_ERR;
  }
  *out = d;
  return PT_OK;
}

extern "C" void pt_dark_destroy(pt_dark* d) {
  if (!d) return;
  cudaFree(d->status);
  cudaFree(d->err_info);
  cudaFree(d->counter);
  cudaFree(d->tasks);
  cudaFreeHost(d->h_status);
  cudaFreeHost(d->h_counter);
  delete d;
}

extern "C" pt_status pt_dark_dsigma(pt_dark* d, int32_t process, const double* x, const double* energy, int64_t n,
                                    double mV, double* value, void* stream) {
  if (!d || process < 0 || process >= PT_N_DARK || n < 0) return PT_BAD_ARG;
  if (n == 0) return PT_OK;
  if (!x || !energy || !value) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  k_dark_dsigma<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d->M, process, x, energy, n, mV, value);
  PT_CUDA(cudaGetLastError());
  PT_CUDA(cudaStreamSynchronize(st));
  return PT_OK;
}

extern "C" pt_status pt_dark_screen32(pt_dark* d, int32_t process, const double* x, const double* energy, int64_t n,
                                      double mV, float* value, int32_t* code, void* stream) {
  if (!d || (process != PT_DARKBREM && process != PT_DARKMUONBREM && process != PT_DARKANN) || n < 0)
    return PT_BAD_ARG;
  if (n == 0) return PT_OK;
  if (!x || !energy || !value || !code) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  k_dark_screen<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d->M, process, x, energy, n, mV, value, code);
  PT_CUDA(cudaGetLastError());
  PT_CUDA(cudaStreamSynchronize(st));
  return PT_OK;
}

static bool mass_block_ok(const pt_dark* d, const pt_dark_params* prm, int p) {
  if (prm->mass_index < 0 || prm->mass_index >= d->M.n_masses) return false;
  return d->M.map_rows[prm->mass_index * PT_N_DARK + p] >= 2;
}

extern "C" pt_status pt_dark_sample_only(pt_dark* d, const pt_dark_params* prm, int32_t process, const double* energy,
                                         const uint64_t* key, int64_t n, const pt_opts* o, double* x,
                                         int64_t* proposals, int32_t* lu_key, void* stream) {
  if (!d || !prm || !o || process < 0 || process >= PT_N_DARK || n < 0) return PT_BAD_ARG;
  if (!mass_block_ok(d, prm, process)) return PT_BAD_TABLE;
  if (n == 0) return PT_OK;
  if (!energy || !key || !x || !proposals || !lu_key) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  k_dark_sample_only<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(d->M, *prm, process, energy, key, n, o->seed,
                                                                  o->max_n_integrators, x, proposals, lu_key);
  PT_CUDA(cudaGetLastError());
  PT_CUDA(cudaStreamSynchronize(st));
  return PT_OK;
}

extern "C" pt_status pt_run_dark(pt_dark* d, const pt_dark_params* prm, const pt_particles* sm, int64_t n_rows,
                                 const pt_opts* o, pt_dark_out* out, int64_t* n_out, void* stream) {
  if (!d || !prm || !sm || !o || !out || !n_out || n_rows < 0 || n_rows > sm->capacity) return PT_BAD_ARG;
  if (prm->mass_index < 0 || prm->mass_index >= d->M.n_masses) return PT_BAD_TABLE;
  if (prm->precision != 0 && (prm->precision != 1 || !d->M.grid_f32x2)) return PT_BAD_ARG;
  for (int p = 0; p < PT_N_DARK; ++p)
    if (((prm->active >> p) & 1) && !mass_block_ok(d, prm, p)) return PT_BAD_TABLE;
  for (int k = 0; k < 4; ++k)
    if (!prm->w_x[k] || !prm->w_y[k] || prm->w_n[k] < 2 || !prm->dr_Ei[k] || !prm->dr_bins[k] || !prm->dr_nbins[k] ||
        prm->dr_n[k] < 1 || prm->dr_nbmax[k] < 1)
      return PT_BAD_TABLE;
  if (!prm->nsc_lx || !prm->nsc_ly || prm->nsc_n < 2) return PT_BAD_TABLE;
  if (out->p4 && (!out->r || !out->weight || !out->parent || !out->process || !out->draws || out->capacity < 0))
    return PT_BAD_ARG;
  *n_out = 0;
  if (n_rows == 0) return PT_OK;
  cudaStream_t st = (cudaStream_t)stream;
  PT_CUDA(cudaMemsetAsync(d->status, 0, sizeof(int), st));
  PT_CUDA(cudaMemsetAsync(d->counter, 0, sizeof(unsigned long long), st));
  const int ncol = PT_N_DARK + ((prm->active >> PT_TWOBODY) & 1);
  const pt_status ls = dark_launch(d, *prm, *o, *sm, n_rows, ncol, *out, st);
  if (ls != PT_OK) return ls;
  PT_CUDA(cudaMemcpyAsync(d->h_counter, d->counter, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  const pt_status s = read_dark_status(d, st);
  *n_out = (int64_t)d->h_counter[0];
  return s;
}

// Dark vectors on the batched engine's waves: the dark production over the
// rows (the record engine's rows of those particles), yields only.
namespace {
constexpr int kMaxBatchMasses = 16;
struct BatchDark {
  pt_dark* d;
  int n;                                   // parameter sets (masses)
  pt_dark_params prm[kMaxBatchMasses];
  pt_opts o;
  pt_dark_out out[kMaxBatchMasses];
};

// The dark production per parameter set over the collected rows.
pt_status batch_dark_wave(void* ctx, const pt_particles* rows, int64_t n_rows, cudaStream_t st) {
  BatchDark* b = static_cast<BatchDark*>(ctx);
  for (int m = 0; m < b->n; ++m) {
    const pt_status s = dark_launch(b->d, b->prm[m], b->o, *rows, n_rows, PT_N_DARK, b->out[m], st);
    if (s != PT_OK) return s;
  }
  return PT_OK;
}
}  // namespace

extern "C" pt_status pt_run_batch_dark(pt_handle* h, pt_dark* d, const pt_dark_params* prm, int32_t n_params,
                                       const double* p0, const double* r0, const int32_t* pid, const double* mass,
                                       int64_t n, const pt_opts* o, pt_tally* tally, int64_t queue_capacity,
                                       double* yield, double* yield_E, const pt_dark_hist* hist, int64_t* n_vectors,
                                       void* stream) {
  if (!h || !d || !prm || !o || !tally || !yield || !yield_E || !n_vectors || n < 0 || n_params < 1 ||
      n_params > kMaxBatchMasses)
    return PT_BAD_ARG;
  if (hist && hist->counts && (hist->bins < 1 || !(hist->log10_hi > hist->log10_lo))) return PT_BAD_ARG;
  for (int m = 0; m < n_params; ++m) {
    const pt_dark_params* q = prm + m;
    if (q->mass_index < 0 || q->mass_index >= d->M.n_masses) return PT_BAD_TABLE;
    if (q->precision != 0 && (q->precision != 1 || !d->M.grid_f32x2)) return PT_BAD_ARG;
    for (int p = 0; p < PT_N_DARK; ++p)
      if (((q->active >> p) & 1) && !mass_block_ok(d, q, p)) return PT_BAD_TABLE;
    for (int k = 0; k < 4; ++k)
      if (!q->w_x[k] || !q->w_y[k] || q->w_n[k] < 2 || !q->dr_Ei[k] || !q->dr_bins[k] || !q->dr_nbins[k] ||
          q->dr_n[k] < 1 || q->dr_nbmax[k] < 1)
        return PT_BAD_TABLE;
    if (!q->nsc_lx || !q->nsc_ly || q->nsc_n < 2) return PT_BAD_TABLE;
  }
  *n_vectors = 0;
  cudaStream_t st = (cudaStream_t)stream;
  PT_CUDA(cudaMemsetAsync(d->status, 0, sizeof(int), st));
  PT_CUDA(cudaMemsetAsync(d->counter, 0, sizeof(unsigned long long), st));
  BatchDark* b = new (std::nothrow) BatchDark();
  if (!b) return PT_OOM;
  b->d = d;
  b->n = n_params;
  b->o = *o;
  for (int m = 0; m < n_params; ++m) {
    b->prm[m] = prm[m];
    b->prm[m].active &= (1 << PT_N_DARK) - 1;        // SM showers hold no mesons
    b->out[m] = pt_dark_out{};
    b->out[m].yield = yield + (size_t)m * (PT_N_DARK + 1);
    b->out[m].yield_E = yield_E + (size_t)m * (PT_N_DARK + 1);
    if (hist && hist->counts) {
      b->out[m].hist = *hist;
      b->out[m].hist.counts = hist->counts + (size_t)m * (PT_N_DARK + 1) * hist->bins;
    }
  }
  const WaveRowsHook hook{batch_dark_wave, b};
  const pt_status s = run_batch_rows(h, p0, r0, pid, mass, n, o, tally, queue_capacity, &hook, st);
  delete b;
  if (s != PT_OK) return s;
  PT_CUDA(cudaMemcpyAsync(d->h_counter, d->counter, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  const pt_status ds = read_dark_status(d, st);
  *n_vectors = (int64_t)d->h_counter[0];
  return ds;
}

template <bool ADJ>
static pt_status dark_yield_launch(pt_dark* d, int32_t process, const double* energy, const double* mV,
                                   const double* anchor, const int32_t* mass_index, int64_t n_pairs,
                                   int64_t n_samples, uint64_t seed, double* yield, double* moment, const double* gY,
                                   const double* gM, double* g_mV, void* stream) {
  if (!d || process < 0 || process >= PT_N_DARK || n_pairs < 0 || n_samples <= 0 || n_pairs > 0x7fffffff)
    return PT_BAD_ARG;
  if (n_pairs == 0) return PT_OK;
  if (!energy || !mV || !mass_index) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if constexpr (ADJ) {
    if (!gY || !gM || !g_mV) return PT_BAD_ARG;
    k_dark_yield<Dual, true><<<(unsigned)n_pairs, kYieldThreads, 0, st>>>(
        d->M, process, energy, mV, nullptr, mass_index, n_samples, seed, nullptr, nullptr, gY, gM, g_mV);
  } else {
    if (!yield || !moment) return PT_BAD_ARG;
    k_dark_yield<double, false><<<(unsigned)n_pairs, kYieldThreads, 0, st>>>(
        d->M, process, energy, mV, anchor, mass_index, n_samples, seed, yield, moment, nullptr, nullptr, nullptr);
  }
  PT_CUDA(cudaGetLastError());
  return PT_OK;
}

extern "C" pt_status pt_dark_yield(pt_dark* d, int32_t process, const double* energy, const double* mV,
                                   const double* mV_anchor, const int32_t* mass_index, int64_t n_pairs,
                                   int64_t n_samples, uint64_t seed, double* yield, double* moment, void* stream) {
  return dark_yield_launch<false>(d, process, energy, mV, mV_anchor, mass_index, n_pairs, n_samples, seed, yield,
                                  moment, nullptr, nullptr, nullptr, stream);
}

extern "C" pt_status pt_dark_yield_adjoint(pt_dark* d, int32_t process, const double* energy, const double* mV,
                                           const int32_t* mass_index, int64_t n_pairs, int64_t n_samples,
                                           uint64_t seed, const double* g_yield, const double* g_moment,
                                           double* g_mV, void* stream) {
  return dark_yield_launch<true>(d, process, energy, mV, nullptr, mass_index, n_pairs, n_samples, seed, nullptr,
                                 nullptr, g_yield, g_moment, g_mV, stream);
}
