// pt_batch.cu -- batched shower transport with tallies (pt_run_batch).
//
// Live particles sit in a power-of-two ring buffer in HBM (structure of
// arrays).  Primaries stream in while there is room; each wave takes up to
// (capacity - live)/2 entries from the head, so the at most two daughters
// per entry always fit behind the tail.  A wave is two kernels:
//  1. k_propagate: propagate_particle (shower.py:509-601) and the process
//     choice (shower.py:665-698).  Lanes refill themselves from the wave and
//     advance one charged-particle substep per iteration, so a long track does
//     not hold its warp.  Interacting particles are parked in place and listed
//     by process; the others are tallied and retired.
//  2. k_sample: draw_sample's accept/reject loop (shower.py:401-465) over the
//     task list ordered by process, one proposal per lane per iteration with
//     refill, then the final-state kinematics and lab rotation
//     (shower.py:467-507); daughters above min_energy are appended at the tail.
// PREC = 0 is the float64 engine (same device functions and operation order
// as pt_run_sm, hence the same showers); PREC = 1 samples and scatters in
// float32 and keeps energies, positions and daughter energies in float64.
#include <cstdio>

#include "pt_internal.cuh"
#include "pt_physics32.cuh"

using namespace pt;

namespace {

constexpr int kThreads = 128;
constexpr int kHB = PT_HIST_BINS;
constexpr int kHist = 3 * 4 * kHB;

struct Ring {
  double *E, *px, *py, *pz, *x, *y, *z, *mass;
  uint64_t* key;
  int32_t *pid, *prim, *gen, *row;
  uint32_t* draw;
};

struct Tally {
  unsigned long long* counts;
  double* energy;
  unsigned int* hist;
  unsigned int* prim_count;
  double* prim_edep;
  float z_max;
};

struct WaveCtx {
  Tabs T;
  double min_energy, rescale;
  int64_t max_n_integrators;
  int ms;
  uint64_t seed;
  Ring q;
  uint64_t mask;                      // ring capacity - 1
  uint64_t head, tail;                // ring positions of this wave's first entry and of the append point
  int64_t n_in;                       // entries in this wave
  int64_t list_cap;                   // entries per process list
  int32_t* idx;                       // [8][list_cap] ring indices of sampling tasks by process
  unsigned long long* ctr;            // [0] head1, [1] head2, [2] appended, [8..15] per-process counts
  int* status;
  double* err_info;
  Tally tally;
};

__device__ void raise_status(int* status, double* info, int code, int process, double E, int key) {
  if (atomicCAS(status, 0, code) == 0 && info) {
    info[0] = process; info[1] = E; info[2] = key;
  }
}

// Warp-aggregated pop: each requesting lane gets one index of [0, n) or -1.
__device__ __forceinline__ int64_t warp_pop(unsigned long long* head, int64_t n, bool need) {
  const unsigned mask = __activemask();
  const unsigned b = __ballot_sync(mask, need);
  const int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if ((int)(threadIdx.x & 31) == leader && b) base = atomicAdd(head, (unsigned long long)__popc(b));
  base = __shfl_sync(mask, base, leader);
  if (!need) return -1;
  const unsigned long long mine = base + __popc(b & lanemask_lt());
  return (int64_t)mine < n ? (int64_t)mine : -1;
}

__device__ __forceinline__ int species_of(int pid) {
  return pid == 22 ? 0 : (pid == 11 ? 1 : (pid == -11 ? 2 : 3));
}

__device__ __forceinline__ int bin_of(float v, float lo, float hi) {
  int b = (int)((v - lo) / (hi - lo) * kHB);
  return b < 0 ? 0 : (b >= kHB ? kHB - 1 : b);
}

struct LocalTally {
  unsigned long long steps = 0, props = 0, substeps = 0, ended = 0, pushed = 0, below = 0, sampled = 0;
  unsigned long long species[4] = {0, 0, 0, 0};
  double e_cont = 0, e_below = 0, e_ended = 0;
};

__device__ void flush_tally(const Tally& T, LocalTally& L, const unsigned int* sh_hist) {
  auto red = [](unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
  };
  auto redd = [](double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
  };
  __syncwarp();
  const unsigned long long c[7] = {red(L.steps), red(L.props), red(L.substeps), red(L.ended), red(L.pushed),
                                   red(L.below), red(L.sampled)};
  const unsigned long long sp[4] = {red(L.species[0]), red(L.species[1]), red(L.species[2]), red(L.species[3])};
  const double e[3] = {redd(L.e_cont), redd(L.e_below), redd(L.e_ended)};
  if ((threadIdx.x & 31) == 0) {
    const int map[7] = {PT_C_STEPS, PT_C_PROPOSALS, PT_C_SUBSTEPS, PT_C_ENDED, PT_C_PUSHED, PT_C_BELOW_CUT,
                        PT_C_SAMPLED};
    for (int k = 0; k < 7; ++k) if (c[k]) atomicAdd(T.counts + map[k], c[k]);
    for (int k = 0; k < 4; ++k) if (sp[k]) atomicAdd(T.counts + PT_C_SPECIES + k, sp[k]);
    if (e[0] != 0) atomicAdd(T.energy + PT_E_CONTINUOUS, e[0]);
    if (e[1] != 0) atomicAdd(T.energy + PT_E_BELOW_CUT, e[1]);
    if (e[2] != 0) atomicAdd(T.energy + PT_E_ENDED, e[2]);
  }
  if (sh_hist) {
    __syncthreads();
    for (int k = threadIdx.x; k < kHist; k += blockDim.x)
      if (sh_hist[k]) atomicAdd(T.hist + k, sh_hist[k]);
  }
}

// Process choice (shower.py:665-698), float64 in both engines.
__device__ int choose_process_b(const Tabs& T, int pid, double E, Rng& rng) {
  int names[3];
  double c[3];
  int n;
  if (pid == 11) { names[0] = PT_BREM; names[1] = PT_MOLLER; c[0] = nsig(T, 0, E); c[1] = nsig(T, 4, E); n = 2; }
  else if (pid == -11) {
    names[0] = PT_BREM; names[1] = PT_ANN; names[2] = PT_BHABHA;
    c[0] = nsig(T, 0, E); c[1] = nsig(T, 2, E); c[2] = nsig(T, 5, E); n = 3;
  } else if (pid == 22) { names[0] = PT_PAIRPROD; names[1] = PT_COMP; c[0] = nsig(T, 1, E); c[1] = nsig(T, 3, E); n = 2; }
  else { names[0] = PT_MUONE; names[1] = PT_MUONBREM; c[0] = nsig(T, 6, E); c[1] = nsig(T, 7, E); n = 2; }
  S SC = S(c[0]) + S(c[1]);
  if (n == 3) SC = SC + S(c[2]);
  if (SC.v == 0.0 || SC.v != SC.v) return -1;
  double cdf[3];
  S acc(0.0);
  for (int i = 0; i < n; ++i) {
    const S p = S(c[i]) / SC;
    acc = (i == 0) ? p : acc + p;
    cdf[i] = acc.v;
  }
  const S last(cdf[n - 1]);
  const double u = rng.u();
  int idx = 0;
  for (int i = 0; i < n; ++i) if ((S(cdf[i]) / last).v <= u) idx = i + 1;
  if (idx >= n) idx = n - 1;
  return names[idx];
}

// ------------------------------------------------------------ phase 1
template <int PREC>
__global__ void __launch_bounds__(kThreads) k_propagate(WaveCtx c) {
  __shared__ unsigned int sh_hist[kHist];
  for (int k = threadIdx.x; k < kHist; k += blockDim.x) sh_hist[k] = 0;
  __syncthreads();
  const Tabs& T = c.T;
  LocalTally L;
  bool active = false;
  uint64_t i = 0;
  double E0 = 0, E = 0, px = 0, py = 0, pz = 0, x = 0, y = 0, z = 0, mass = 0, pme = 0, dz = 0;
  float3 dir = make_float3(0.f, 0.f, 1.f), disp = make_float3(0.f, 0.f, 0.f);
  float pmag = 0.f;
  int pid = 0, prim = 0;
  Rng rng;
  const double losses = T.t.dEdx_GeV_per_m;
  const float zmax = c.tally.z_max;

  for (;;) {
    const bool need = !active;
    const int64_t got = warp_pop(c.ctr + 0, c.n_in, need);
    bool finish = false;
    if (need) {
      if (got < 0) break;
      i = (c.head + (uint64_t)got) & c.mask;
      E0 = c.q.E[i]; px = c.q.px[i]; py = c.q.py[i]; pz = c.q.pz[i];
      x = c.q.x[i]; y = c.q.y[i]; z = c.q.z[i];
      mass = c.q.mass[i]; pid = c.q.pid[i]; prim = c.q.prim[i];
      rng.init(c.seed, c.q.key[i]);
      E = E0;
      pme = fmax(fmax(min_calc(T, pid), c.min_energy), mass);
      ++L.steps;
      const int sp = species_of(pid);
      ++L.species[sp];
      atomicAdd(&sh_hist[(0 * 4 + sp) * kHB + bin_of(log10f((float)E0), -2.f, 2.f)], 1u);
      const float th = atan2f((float)sqrt(px * px + py * py), (float)pz);
      atomicAdd(&sh_hist[(1 * 4 + sp) * kHB + bin_of(th > 0.f ? log10f(th) : -6.f, -6.f, 0.5f)], 1u);
      if (E0 < pme) {
        finish = true;
      } else if (pid == 22) {               // shower.py:538-553
        const double mfp = mfp_of(T, pid, E);
        const double distC = rng.u();
        const double dist = (S(mfp) * S(log((S(1.0) / (S(1.0) - S(distC))).v))).v;
        const double n = norm3_np(px, py, pz);
        x = (S(x) + S(px) / S(n) * S(dist)).v;
        y = (S(y) + S(py) / S(n) * S(dist)).v;
        z = (S(z) + S(pz) / S(n) * S(dist)).v;
        finish = true;
      } else {
        active = true;
        dz = 0.0;
        if (PREC == 1) {
          const double pn = sqrt(px * px + py * py + pz * pz);
          pmag = (float)pn;
          dir = pn > 0 ? make_float3((float)(px / pn), (float)(py / pn), (float)(pz / pn)) : make_float3(0.f, 0.f, 1.f);
          disp = make_float3(0.f, 0.f, 0.f);
        }
      }
    }
    if (active) {
      // one iteration of the substep loop (shower.py:559-581)
      bool stop = !(E >= pme);
      if (!stop) {
        ++L.substeps;
        const double mfp = mfp_of(T, pid, E);
        const double u_hard = rng.u();
        if (PREC == 0) {
          dz = (S(mfp) / (S(6.0) + S(14.0) * S(rng.u()))).v;
          if (u_hard > exp(-dz / mfp)) {
            stop = true;
          } else {
            double pf[4] = {E, px, py, pz}, rf[3] = {x, y, z};
            lose_energy(pf, mass, (S(losses) * S(dz)).v);
            move_along(pf, rf, dz);
            if (c.ms) mcs_fast(pf, (S(T.t.rho) * (S(dz) / S(kCmToM))).v, T.t.A, T.t.Z, T.t.Z23, c.rescale,
                               table_mass(pid), rng);
            E = pf[0]; px = pf[1]; py = pf[2]; pz = pf[3]; x = rf[0]; y = rf[1]; z = rf[2];
          }
        } else {
          const float q = fmaf(14.f, rng.uf(), 6.f);
          dz = mfp / (double)q;
          if ((float)u_hard > __expf(-1.f / q)) {
            stop = true;
          } else {
            // lose_energy (particle.py:143-153): E in float64, |p| from (E-m)(E+m)
            double En = E - losses * dz;
            if (En <= mass) En = mass;
            E = En;
            pmag = sqrtf((float)((En - mass) * (En + mass)));
            if (pmag > 0.f) {
              const float dzf = (float)dz;
              disp.x = fmaf(dir.x, dzf, disp.x); disp.y = fmaf(dir.y, dzf, disp.y); disp.z = fmaf(dir.z, dzf, disp.z);
            }
            if (c.ms)
              mcs32(dir, pmag, (float)E, (float)(T.t.rho * (dz / kCmToM)), (float)T.t.A, (float)T.t.Z,
                    (float)T.t.Z23, (float)c.rescale, rng);
          }
        }
      }
      if (stop) {
        // final partial increment (shower.py:583-598)
        const double distC = rng.u();
        double last;
        if (E < pme) last = (S(distC) * S(dz)).v;
        else {
          const double mfp = mfp_of(T, pid, E);
          const S e = S(exp(-dz / mfp));
          last = (S(mfp) * S(log((S(1.0) / (S(1.0) + (e - S(1.0)) * S(distC))).v))).v;
        }
        if (PREC == 0) {
          double pf[4] = {E, px, py, pz}, rf[3] = {x, y, z};
          lose_energy(pf, mass, (S(losses) * S(last)).v);
          move_along(pf, rf, last);
          if (c.ms) mcs_fast(pf, (S(T.t.rho) * (S(last) / S(kCmToM))).v, T.t.A, T.t.Z, T.t.Z23, c.rescale, kMe, rng);
          E = pf[0]; px = pf[1]; py = pf[2]; pz = pf[3]; x = rf[0]; y = rf[1]; z = rf[2];
        } else {
          double En = E - losses * last;
          if (En <= mass) En = mass;
          E = En;
          pmag = sqrtf((float)((En - mass) * (En + mass)));
          if (pmag > 0.f) {
            const float lf = (float)last;
            disp.x = fmaf(dir.x, lf, disp.x); disp.y = fmaf(dir.y, lf, disp.y); disp.z = fmaf(dir.z, lf, disp.z);
          }
          if (c.ms)   // shower.py:596-598 passes no m_lepton (electron default); |p| enters here directly
            mcs32(dir, pmag, (float)E, (float)(T.t.rho * (last / kCmToM)), (float)T.t.A, (float)T.t.Z,
                  (float)T.t.Z23, (float)c.rescale, rng);
          x += disp.x; y += disp.y; z += disp.z;
          if (pmag > 0.f) { px = (double)pmag * dir.x; py = (double)pmag * dir.y; pz = (double)pmag * dir.z; }
          else { px = py = pz = 0.0; }
        }
        active = false;
        finish = true;
      }
    }
    if (finish) {
      const int sp = species_of(pid);
      atomicAdd(&sh_hist[(2 * 4 + sp) * kHB + bin_of((float)z, 0.f, zmax)], 1u);
      const double eloss = E0 - E;
      L.e_cont += eloss;
      atomicAdd(c.tally.prim_count + prim, 1u);
      const int process = choose_process_b(T, pid, E, rng);
      if (process >= 0 && E > pme) {
        // park the post-propagation state in place and list a sampling task
        c.q.E[i] = E; c.q.px[i] = px; c.q.py[i] = py; c.q.pz[i] = pz;
        c.q.x[i] = x; c.q.y[i] = y; c.q.z[i] = z;
        c.q.draw[i] = (uint32_t)rng.n;
        c.q.row[i] = T.t.map_base[process] + lu_key(T, process, E);
        const unsigned mask = __activemask();
        const unsigned grp = __match_any_sync(mask, process);
        const int leader = __ffs(grp) - 1;
        unsigned long long base = 0;
        if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(c.ctr + 8 + process, (unsigned long long)__popc(grp));
        base = __shfl_sync(grp, base, leader);
        const unsigned long long slot = base + __popc(grp & lanemask_lt());
        c.idx[(int64_t)process * c.list_cap + (int64_t)slot] = (int32_t)i;
        if (eloss != 0.0) atomicAdd(c.tally.prim_edep + prim, eloss);
      } else {
        ++L.ended;
        L.e_ended += E;
        atomicAdd(c.tally.prim_edep + prim, eloss + E);
      }
    }
  }
  flush_tally(c.tally, L, sh_hist);
}

// ------------------------------------------------------------ phase 2
struct Daughter { double E, px, py, pz; int pid; };

// Mixed engine: daughters in the parent frame with float64 energies (forms
// without cancellation), float64 momentum magnitudes, float32 directions.
struct KinOut { double E[2], P[2]; float3 d[2]; int pid[2]; };

__device__ __forceinline__ void set_dir(KinOut& k, int j, double pxx, double pyy, double pzz) {
  const double p = sqrt(pxx * pxx + pyy * pyy + pzz * pzz);
  k.P[j] = p;
  k.d[j] = p > 0 ? make_float3((float)(pxx / p), (float)(pyy / p), (float)(pzz / p)) : make_float3(0.f, 0.f, 1.f);
}

__device__ void kin_mixed(int process, int pid, double E, double mass, const double* x, double omx, double opx,
                          float ph, KinOut& k) {
  float sph, cph;
  sincosf(ph, &sph, &cph);
  const double me = kMe;
  switch (process) {
    case PT_BREM: case PT_MUONBREM: {        // kinematics.py:10-41
      const double Eg = 0.001;
      const double w = Eg + x[0] * (E - mass - Eg);
      const double epp = E - w;
      float st, ct, stp, ctp, sp, cp;
      sincosf((float)((x[1] + x[2]) / 2), &st, &ct);
      sincosf((float)((x[1] - x[2]) * E / (2 * (E - w))), &stp, &ctp);
      st = fabsf(st); stp = fabsf(stp);        // the reference takes sqrt(1 - cos^2)
      sincospif((float)(2.0 * (x[3] - 0.5)), &sp, &cp);
      const float sal = sph, cal = cph;        // azimuth 'al' of kinematics.py:33
      k.E[1] = w; k.P[1] = w; k.pid[1] = 22;
      k.d[1] = make_float3(cal * st, sal * st, ct);
      k.E[0] = epp; k.pid[0] = pid;
      k.P[0] = sqrt((epp - mass) * (epp + mass));
      const float3 v = make_float3(sal * sp * stp + cal * (ctp * st - cp * ct * stp),
                                   ctp * sal * st - (cp * ct * sal + cal * sp) * stp, ct * ctp + cp * st * stp);
      const float inv = rsqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
      k.d[0] = make_float3(v.x * inv, v.y * inv, v.z * inv);
      break;
    }
    case PT_PAIRPROD: {                       // kinematics.py:70-102
      const double w = E;
      const double epp = me + x[0] * (w - 2 * me);
      const double epm = me + omx * (w - 2 * me);
      float stp, ctp, stm, ctm, s2, c2;
      sincosf((float)(w * (x[1] + x[2]) / (2 * epp)), &stp, &ctp);
      sincosf((float)(w * (x[1] - x[2]) / (2 * epm)), &stm, &ctm);
      stp = fabsf(stp); stm = fabsf(stm);
      sincosf((float)(x[3] * 2 * kPi) + ph, &s2, &c2);
      k.E[0] = epp; k.P[0] = sqrt((epp - me) * (epp + me)); k.pid[0] = -11;
      k.d[0] = make_float3(stp * cph, stp * sph, ctp);
      k.E[1] = epm; k.P[1] = sqrt((epm - me) * (epm + me)); k.pid[1] = 11;
      k.d[1] = make_float3(stm * c2, stm * s2, ctm);
      break;
    }
    case PT_COMP: {                           // kinematics.py:104-132, mV = 0
      const double s = me * me + 2 * E * me, rs = sqrt(s);
      const double Ee = (s + me * me) / (2 * rs), EV = (s - me * me) / (2 * rs), pF = EV;
      const double g0 = Ee / me, sq = sqrt((g0 - 1) * (g0 + 1)), b0 = sq / g0;
      const double omb = 1.0 / (g0 * (g0 + sq));                 // 1 - b0
      const double pT = pF * sqrt(omx * opx);
      k.E[0] = g0 * Ee + b0 * g0 * pF * x[0]; k.pid[0] = 11;
      set_dir(k, 0, -pT * sph, -pT * cph, b0 * g0 * Ee + g0 * pF * x[0]);
      k.E[1] = g0 * EV * (omb + b0 * omx); k.pid[1] = 22;      // g0 (EV - b0 pF c)
      set_dir(k, 1, pT * sph, pT * cph, g0 * EV * (omx - omb));  // g0 (b0 EV - pF c)
      break;
    }
    case PT_ANN: {                            // kinematics.py:301-334, mV = 0
      const double s = 2 * me * (E + me), Eg = sqrt(s) / 2;
      const double g0 = Eg / me, sq = sqrt((g0 - 1) * (g0 + 1)), b0 = sq / g0;
      const double omb = 1.0 / (g0 * (g0 + sq));
      const double pT = Eg * sqrt(omx * opx);
      k.E[0] = g0 * Eg * (omb + b0 * omx); k.pid[0] = 22;
      set_dir(k, 0, -pT * sph, -pT * cph, g0 * Eg * (omx - omb));
      k.E[1] = g0 * Eg * (1 + b0 * x[0]); k.pid[1] = 22;
      set_dir(k, 1, pT * sph, pT * cph, g0 * Eg * (b0 + x[0]));
      break;
    }
    case PT_MOLLER: case PT_BHABHA: {         // kinematics.py:213-237 (b0 = pF/Ee0)
      const double s = 2 * me * me + 2 * E * me, Ee0 = sqrt(s) / 2;
      const double pF = sqrt((Ee0 - me) * (Ee0 + me)), g0 = Ee0 / me, b0 = pF / Ee0;
      const double pT = pF * sqrt(omx * opx);
      k.E[0] = g0 * (Ee0 + b0 * pF * x[0]); k.pid[0] = pid;
      set_dir(k, 0, -pT * sph, -pT * cph, g0 * pF * opx);
      k.E[1] = g0 * (me * me + pF * pF * omx) / Ee0; k.pid[1] = 11;   // g0 (Ee0 - b0 pF c)
      set_dir(k, 1, pT * sph, pT * cph, g0 * pF * omx);
      break;
    }
    default: {                                // kinematics.py:239-265 (b0 = pe/Ee0)
      const double mm = kMmu, s = me * me + mm * mm + 2 * E * me, rs = sqrt(s);
      const double Ee0 = (s + me * me - mm * mm) / (2 * rs), Em0 = (s + mm * mm - me * me) / (2 * rs);
      const double pe = sqrt((Ee0 - me) * (Ee0 + me)), pm = sqrt((Em0 - mm) * (Em0 + mm));
      const double g0 = Ee0 / me, b0 = pe / Ee0;
      const double st = sqrt(omx * opx);
      k.E[0] = g0 * (Em0 + b0 * pm * x[0]); k.pid[0] = pid;
      set_dir(k, 0, pm * st * sph, pm * st * cph, b0 * g0 * Em0 + g0 * pm * x[0]);
      k.E[1] = g0 * (me * me + pe * pe * omx) / Ee0; k.pid[1] = 11;     // g0 (Ee0 - b0 pe c)
      set_dir(k, 1, -pe * st * sph, -pe * st * cph, g0 * pe * omx);
      break;
    }
  }
}

template <int PREC>
__global__ void __launch_bounds__(kThreads) k_sample(WaveCtx c) {
  __shared__ unsigned long long sh_off[9];
  if (threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (int p = 0; p < 8; ++p) { sh_off[p] = acc; acc += c.ctr[8 + p]; }
    sh_off[8] = acc;
  }
  __syncthreads();
  const int64_t total = (int64_t)sh_off[8];
  const Tabs& T = c.T;
  LocalTally L;
  bool active = false;
  int process = 0, d = 1, row = 0;
  uint64_t i = 0;
  int64_t props = 0, cap = 0;
  double E = 0, maxF = 0, neval = 1;
  Rng rng;
  Samp32 S32;
  const float4* g32[4] = {nullptr, nullptr, nullptr, nullptr};
  const double* g64[4] = {nullptr, nullptr, nullptr, nullptr};
  int ninc[4] = {1, 1, 1, 1};
  uint64_t yk[4] = {0, 0, 0, 0};

  for (;;) {
    const bool need = !active;
    const int64_t t = warp_pop(c.ctr + 1, total, need);
    if (need) {
      if (t < 0) break;
      process = 0;
      while (process < 7 && (unsigned long long)t >= sh_off[process + 1]) ++process;
      i = (uint64_t)c.idx[(int64_t)process * c.list_cap + (t - (int64_t)sh_off[process])];
      E = c.q.E[i];
      row = c.q.row[i];
      rng.init(c.seed, c.q.key[i]);
      rng.n = c.q.draw[i];
      if (rng.n & 1ull) {   // resume inside a Philox block: regenerate its second half
        const uint64_t blk = rng.n >> 1;
        const uint4 o = philox4x32_10(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), rng.k0, rng.k1), rng.s0, rng.s1);
        rng.spare = (uint64_t)o.z | ((uint64_t)o.w << 32);
      }
      maxF = T.t.map_maxF[row];
      neval = T.t.map_neval[row];
      d = process_dim(process);
      cap = c.max_n_integrators * (int64_t)neval;
      props = 0;
      for (int k = 0; k < d; ++k) {
        const int64_t off = T.t.grid_offset[(int64_t)row * 4 + k];
        ninc[k] = T.t.grid_ninc[(int64_t)row * 4 + k];
        g64[k] = T.t.grid_nodes + off;
        g32[k] = reinterpret_cast<const float4*>(T.t.grid_f32x4) + off;
      }
      if (PREC == 1) {
        const double inv_norm = 1.0 / (maxF * neval);
        const double Z2 = T.t.Z * T.t.Z;
        switch (process) {
          case PT_BREM: brem32_setup(S32, E, kMe, T.t.Eg_min, T.a0sq, Z2, inv_norm); break;
          case PT_MUONBREM: brem32_setup(S32, E, kMmu, T.t.Eg_min, T.a0sq, Z2, inv_norm); break;
          case PT_PAIRPROD: pair32_setup(S32, E, T.a0sq, Z2, inv_norm); break;
          case PT_COMP: comp32_setup(S32, E, inv_norm); break;
          case PT_ANN: ann32_setup(S32, E, T.t.Eg_min, inv_norm); break;
          case PT_MOLLER: moller32_setup(S32, E, T.t.Ee_min, inv_norm); break;
          case PT_BHABHA: bhabha32_setup(S32, E, T.t.Ee_min, inv_norm); break;
          default: muone32_setup(S32, E, T.t.Ee_min, inv_norm); break;
        }
      }
      active = true;
    }
    // ---- one proposal (d uniforms for y, then the accept uniform)
    bool accept;
    double xd[4] = {0, 0, 0, 0};
    if (PREC == 0) {
      double jac = 1.0;
      for (int k = 0; k < d; ++k) xd[k] = map_dim(g64[k], ninc[k], rng.u(), jac);
      const double f = dsigma_any(T, process, xd, E);
      accept = maxF * rng.u() < (jac / neval) * f;
    } else {
      MapPt32 xm[4];
      float jac = 1.f;
      for (int k = 0; k < d; ++k) {
        yk[k] = rng.next_u64();
        xm[k] = map_dim32(g32[k], ninc[k], (float)(yk[k] >> 40) * 0x1p-24f, jac);
      }
      float r;
      switch (process) {
        case PT_BREM: case PT_MUONBREM: r = brem32_ratio(S32, xm, jac); break;
        case PT_PAIRPROD: r = pair32_ratio(S32, xm, jac); break;
        case PT_COMP: r = comp32_ratio(S32, xm[0], jac); break;
        case PT_ANN: r = ann32_ratio(S32, xm[0], jac); break;
        case PT_MOLLER: r = moller32_ratio(S32, xm[0], jac); break;
        case PT_BHABHA: r = bhabha32_ratio(S32, xm[0], jac); break;
        default: r = muone32_ratio(S32, xm[0], jac); break;
      }
      accept = rng.uf() < r;
      if (accept) {   // the accepted point in float64 from the same draws
        double jd = 1.0;
        for (int k = 0; k < d; ++k) xd[k] = map_dim(g64[k], ninc[k], (double)(yk[k] >> 11) * 0x1p-53, jd);
      }
    }
    ++props;
    ++L.props;
    if (!accept) {
      if (props >= cap) {
        raise_status(c.status, c.err_info, PT_NO_SAMPLE, process, E, row - T.t.map_base[process]);
        active = false;
      }
      continue;
    }
    // ---- accepted: kinematics and daughters (sample_scattering, shower.py:467-507)
    active = false;
    ++L.sampled;
    const double mass = c.q.mass[i];
    const int pid = c.q.pid[i];
    const double pf[4] = {E, c.q.px[i], c.q.py[i], c.q.pz[i]};
    Daughter dg[2];
    const double ph = 2.0 * kPi * rng.u();
    if (PREC == 0) {
      const Rot R = rotation_from(pf);
      V4 a, b;
      int pa, pb;
      switch (process) {
        case PT_BREM: case PT_MUONBREM: kin_brem(E, mass, xd, ph, a, b); pa = pid; pb = 22; break;
        case PT_PAIRPROD: kin_pairprod(E, xd, ph, a, b); pa = -11; pb = 11; break;
        case PT_COMP: kin_compton(E, xd[0], ph, a, b); pa = 11; pb = 22; break;
        case PT_ANN: kin_ann(E, xd[0], ph, a, b); pa = 22; pb = 22; break;
        case PT_MOLLER: case PT_BHABHA: kin_ee(E, xd[0], ph, a, b); pa = pid; pb = 11; break;
        default: kin_mue(E, xd[0], ph, a, b); pa = pid; pb = 11; break;
      }
      const V4 la = to_lab(R, a), lb = to_lab(R, b);
      dg[0] = {la.e, la.x, la.y, la.z, pa};
      dg[1] = {lb.e, lb.x, lb.y, lb.z, pb};
    } else {
      KinOut k;
      kin_mixed(process, pid, E, mass, xd, 1.0 - xd[0], 1.0 + xd[0], (float)ph, k);
      const double pn = sqrt(pf[1] * pf[1] + pf[2] * pf[2] + pf[3] * pf[3]);
      const float3 pd = pn > 0 ? make_float3((float)(pf[1] / pn), (float)(pf[2] / pn), (float)(pf[3] / pn))
                               : make_float3(0.f, 0.f, 1.f);
      const Rot32 R = rot32_from(pd);
      for (int j = 0; j < 2; ++j) {
        const float3 v = rot32_apply(R, k.d[j]);
        dg[j] = {k.E[j], k.P[j] * v.x, k.P[j] * v.y, k.P[j] * v.z, k.pid[j]};
      }
    }
    const int want = (dg[0].E > c.min_energy) + (dg[1].E > c.min_energy);
    double below = 0.0;
    for (int j = 0; j < 2; ++j)
      if (!(dg[j].E > c.min_energy)) { ++L.below; L.e_below += dg[j].E; below += dg[j].E; }
    const int prim = c.q.prim[i];
    if (below != 0.0) atomicAdd(c.tally.prim_edep + prim, below);
    const unsigned long long base = warp_reserve(c.ctr + 2, want);
    int slot = 0;
    const uint64_t key = c.q.key[i];
    const int gen = c.q.gen[i];
    const double x0 = c.q.x[i], y0 = c.q.y[i], z0 = c.q.z[i];
    for (int j = 0; j < 2; ++j) {
      if (!(dg[j].E > c.min_energy)) continue;
      const uint64_t q = (c.tail + base + (unsigned long long)slot++) & c.mask;
      ++L.pushed;
      c.q.E[q] = dg[j].E; c.q.px[q] = dg[j].px; c.q.py[q] = dg[j].py; c.q.pz[q] = dg[j].pz;
      c.q.x[q] = x0; c.q.y[q] = y0; c.q.z[q] = z0;
      c.q.mass[q] = table_mass(dg[j].pid);
      c.q.key[q] = daughter_key(key, j);
      c.q.pid[q] = dg[j].pid;
      c.q.prim[q] = prim;
      c.q.gen[q] = gen + 1;
    }
  }
  flush_tally(c.tally, L, nullptr);
}

__global__ void k_feed(Ring q, uint64_t mask, uint64_t tail, const double* p0, const double* r0, const int32_t* pid,
                       const double* mass, int64_t n_total, int64_t first, int64_t n, int64_t offset) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t g = first + j;
  const uint64_t i = (tail + (uint64_t)j) & mask;
  q.E[i] = p0[0 * n_total + g]; q.px[i] = p0[1 * n_total + g]; q.py[i] = p0[2 * n_total + g];
  q.pz[i] = p0[3 * n_total + g];
  q.x[i] = r0[0 * n_total + g]; q.y[i] = r0[1 * n_total + g]; q.z[i] = r0[2 * n_total + g];
  q.mass[i] = mass[g]; q.pid[i] = pid[g]; q.prim[i] = (int32_t)g; q.gen[i] = 0;
  q.key[i] = primary_key((uint64_t)(offset + g));
}

}  // namespace

// ------------------------------------------------------------- host side
struct BatchScratch {
  int64_t cap = 0;          // ring capacity (power of two)
  int64_t list_cap = 0;     // entries per process list (= max wave size)
  void* mem = nullptr;
  Ring q;
  int32_t* idx = nullptr;
  unsigned long long* ctr = nullptr;
  unsigned long long* h_ctr = nullptr;
  int* h_status = nullptr;
};

#define PT_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      fprintf(stderr, "petite_gpu: %s failed: %s\n", #call, cudaGetErrorString(e_));  \
      return PT_CUDA_ERR;                                                             \
    }                                                                                 \
  } while (0)

static size_t ring_bytes(int64_t cap) { return (size_t)cap * (9 * 8 + 5 * 4) + 16 * 256; }

pt_status batch_scratch_alloc(BatchScratch** out, int64_t cap) {
  int64_t c2 = 1;
  while (c2 < cap) c2 <<= 1;
  BatchScratch* s = *out;
  if (s && s->cap >= c2) return PT_OK;
  batch_scratch_free(s);
  *out = nullptr;
  s = new BatchScratch();
  s->cap = c2;
  s->list_cap = c2 / 2;
  if (cudaMalloc(&s->mem, ring_bytes(c2)) != cudaSuccess ||
      cudaMalloc(&s->idx, (size_t)8 * s->list_cap * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&s->ctr, 16 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&s->h_ctr, 16 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&s->h_status, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    batch_scratch_free(s);
    return PT_OOM;
  }
  char* p = (char*)s->mem;
  auto take = [&](size_t b) { char* r = p; p += (b + 255) & ~size_t(255); return r; };
  Ring& q = s->q;
  q.E = (double*)take(c2 * 8); q.px = (double*)take(c2 * 8); q.py = (double*)take(c2 * 8);
  q.pz = (double*)take(c2 * 8); q.x = (double*)take(c2 * 8); q.y = (double*)take(c2 * 8);
  q.z = (double*)take(c2 * 8); q.mass = (double*)take(c2 * 8); q.key = (uint64_t*)take(c2 * 8);
  q.pid = (int32_t*)take(c2 * 4); q.prim = (int32_t*)take(c2 * 4); q.gen = (int32_t*)take(c2 * 4);
  q.row = (int32_t*)take(c2 * 4); q.draw = (uint32_t*)take(c2 * 4);
  *out = s;
  return PT_OK;
}

void batch_scratch_free(BatchScratch* s) {
  if (!s) return;
  cudaFree(s->mem);
  cudaFree(s->idx);
  cudaFree(s->ctr);
  cudaFreeHost(s->h_ctr);
  cudaFreeHost(s->h_status);
  delete s;
}

static int resident_blocks(const void* kernel) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kThreads, 0);
  if (per < 1) per = 1;
  return sms * per;
}

extern "C" pt_status pt_run_batch(pt_handle* h, const double* p0, const double* r0, const int32_t* pid,
                                  const double* mass, int64_t n, const pt_opts* o, pt_tally* tally,
                                  int64_t queue_capacity, void* stream) {
  if (!h || !o || !tally || n < 0) return PT_BAD_ARG;
  if (n == 0) return PT_OK;
  if (!p0 || !r0 || !pid || !mass || !tally->counts || !tally->energy || !tally->hist || !tally->primary_count ||
      !tally->primary_edep || (o->precision != 0 && o->precision != 1) || n > 0x7fffffff)
    return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  BatchScratch* S = nullptr;
  pt_status s = batch_scratch_get(h, &S, queue_capacity > 0 ? queue_capacity : ((int64_t)1 << 24));
  if (s != PT_OK) return s;
  HandleParts hp = handle_parts(h);
  WaveCtx c;
  c.T = *hp.T;
  c.min_energy = o->min_energy;
  c.rescale = o->rescale_MCS;
  c.max_n_integrators = o->max_n_integrators;
  c.ms = o->multiple_scattering;
  c.seed = o->seed;
  c.q = S->q;
  c.mask = (uint64_t)S->cap - 1;
  c.list_cap = S->list_cap;
  c.idx = S->idx;
  c.ctr = S->ctr;
  c.status = hp.status;
  c.err_info = hp.err_info;
  c.tally = {tally->counts, tally->energy, tally->hist, tally->primary_count, tally->primary_edep,
             (float)(tally->z_max > 0 ? tally->z_max : 1.0)};
  const void* kp = o->precision ? (const void*)k_propagate<1> : (const void*)k_propagate<0>;
  const void* ks = o->precision ? (const void*)k_sample<1> : (const void*)k_sample<0>;
  const int rb_p = resident_blocks(kp), rb_s = resident_blocks(ks);
  PT_CUDA(cudaMemsetAsync(hp.status, 0, sizeof(int), st));
  const int64_t cap = S->cap;
  const int64_t feed_max = cap / 16;          // primaries added per refill
  uint64_t head = 0, tail = 0;
  int64_t fed = 0, nl = 1, nw = 0;
  while (fed < n || tail > head) {
    int64_t live = (int64_t)(tail - head);
    if (fed < n && live < cap / 2) {
      int64_t m = n - fed;
      if (m > cap / 2 - live) m = cap / 2 - live;
      if (m > feed_max) m = feed_max;
      k_feed<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(S->q, c.mask, tail, p0, r0, pid, mass, n, fed, m,
                                                          o->primary_offset);
      ++nl;
      tail += (uint64_t)m;
      fed += m;
      live += m;
    }
    int64_t k = (cap - live) / 2;
    if (k > live) k = live;
    if (k > S->list_cap) k = S->list_cap;
    if (k <= 0) return PT_OOM;                // unreachable: live stays below the capacity
    PT_CUDA(cudaMemsetAsync(S->ctr, 0, 16 * sizeof(unsigned long long), st));
    c.head = head;
    c.tail = tail;
    c.n_in = k;
    const int64_t want_blocks = (k + kThreads - 1) / kThreads;
    const unsigned gp = (unsigned)(want_blocks < rb_p ? want_blocks : rb_p);
    const unsigned gs = (unsigned)(want_blocks < rb_s ? want_blocks : rb_s);
    if (o->precision) {
      k_propagate<1><<<gp, kThreads, 0, st>>>(c);
      k_sample<1><<<gs, kThreads, 0, st>>>(c);
    } else {
      k_propagate<0><<<gp, kThreads, 0, st>>>(c);
      k_sample<0><<<gs, kThreads, 0, st>>>(c);
    }
    PT_CUDA(cudaGetLastError());
    nl += 3;
    ++nw;
    PT_CUDA(cudaMemcpyAsync(S->h_ctr, S->ctr, 16 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaMemcpyAsync(S->h_status, hp.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    if (*S->h_status != PT_OK) {
      hp.launches[0] = nl; hp.launches[1] = nw;
      if (*S->h_status == PT_NO_SAMPLE || *S->h_status == PT_TIMEOUT)
        PT_CUDA(cudaMemcpy(hp.last_info, hp.err_info, 3 * sizeof(double), cudaMemcpyDeviceToHost));
      return (pt_status)*S->h_status;
    }
    head += (uint64_t)k;
    tail += S->h_ctr[2];
  }
  hp.launches[0] = nl;
  hp.launches[1] = nw;
  return PT_OK;
}
