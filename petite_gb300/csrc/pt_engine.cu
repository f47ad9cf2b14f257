// pt_engine.cu -- shower transport kernels and the C ABI (include/petite_gpu.h).
//
// Float64 wavefront engine: one thread per live particle runs one iteration
// of PETITE's generate_shower loop for it (shower.py:641-706): propagation,
// process choice, draw_sample's accept/reject loop, final-state kinematics,
// lab rotation and the push of daughters above min_energy.  Daughters of a
// wave form the next wave.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

#include "pt_internal.cuh"
#include "pt_physics.cuh"

using namespace pt;

namespace {

struct RunCtx {
  Tabs T;
  double min_energy, rescale;
  int64_t max_n_integrators;
  int ms, mcs_mode;
  uint64_t seed;
  pt_particles P;
  const int64_t* live_in;
  int64_t n_in;
  int64_t* live_out;
  int64_t live_cap;          // entries of live_out
  unsigned long long* n_out;
  unsigned long long* n_rows;
  int* status;
  double* err_info;   // [process, energy, lu_key]
  int loop_limit;     // substep iterations per particle
};

__device__ void raise_status(int* status, double* info, int code, int process, double E, int key) {
  if (atomicCAS(status, 0, code) == 0 && info) {
    info[0] = process; info[1] = E; info[2] = key;
  }
}

// draw_sample (shower.py:401-465): proposals in batches of neval until
// max_F*U < wgt*f; d uniforms for y, then the accept uniform.
__device__ bool draw_sample_fp64(const Tabs& T, int process, double E, int64_t max_n_integrators,
                                 Rng& rng, double* x, int& key, int64_t& proposals) {
  key = lu_key(T, process, E);
  const int row = T.t.map_base[process] + key;
  const double maxF = T.t.map_maxF[row];
  const double neval = T.t.map_neval[row];
  const int d = process_dim(process);
  const int64_t cap = max_n_integrators * (int64_t)neval;
  const double* g[PT_MAX_DIM];
  int ninc[PT_MAX_DIM];
  for (int k = 0; k < d; ++k) {
    g[k] = T.t.grid_nodes + T.t.grid_offset[row * 4 + k];
    ninc[k] = T.t.grid_ninc[row * 4 + k];
  }
  proposals = 0;
  while (proposals < cap) {
    double jac = 1.0;
    for (int k = 0; k < d; ++k) x[k] = map_dim(g[k], ninc[k], rng.u(), jac);
    ++proposals;
    const double wgt = jac / neval;
    const double f = dsigma_any(T, process, x, E);
    if (maxF * rng.u() < wgt * f) return true;
  }
  return false;
}

// Process choice (shower.py:665-698): numpy choice over n*sigma weights.
__device__ int choose_process(const Tabs& T, int pid, double E, Rng& rng) {
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
  if (idx >= n) idx = n - 1;   // u < 1 always; guard only
  return names[idx];
}

__global__ void k_init_primaries(pt_particles P, int64_t n, int64_t offset) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t c = P.capacity;
  for (int k = 0; k < 4; ++k) P.pf[k * c + i] = P.p0[k * c + i];
  for (int k = 0; k < 3; ++k) P.rf[k * c + i] = P.r0[k * c + i];
  P.gen[i] = 0; P.proc[i] = -1; P.bit[i] = 0; P.primary[i] = (int32_t)i; P.draws[i] = 0;
  P.parent[i] = -1; P.pkey[i] = primary_key((uint64_t)(offset + i));
}

__global__ void k_iota(int64_t* a, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] = i;
}

// BETHE: Shower(fast_MCS_mode=False), instantiated apart from the fast mode.
template <int BETHE>
__global__ void __launch_bounds__(128) k_transport_fp64(RunCtx c) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= c.n_in) return;
  const Tabs& T = c.T;
  pt_particles& P = c.P;
  const int64_t cap = P.capacity;
  const int64_t row = c.live_in[i];
  double p0[4], pf[4], rf[3];
  for (int k = 0; k < 4; ++k) p0[k] = P.p0[k * cap + row];
  for (int k = 0; k < 3; ++k) rf[k] = P.r0[k * cap + row];
  for (int k = 0; k < 4; ++k) pf[k] = p0[k];
  const int pid = P.pid[row];
  const double mass = P.mass[row];
  const uint64_t key = P.pkey[row];
  Rng rng;
  rng.init(c.seed, key);

  // ---- propagate_particle (shower.py:509-601)
  const double pme = fmax(fmax(min_calc(T, pid), c.min_energy), mass);
  if (!(p0[0] < pme)) {
    if (pid == 22) {
      const double mfp = mfp_of(T, pid, pf[0]);
      const double distC = rng.u();
      const double dist = (S(mfp) * S(log((S(1.0) / (S(1.0) - S(distC))).v))).v;
      const double n = norm3_np(p0[1], p0[2], p0[3]);
      rf[0] = (S(rf[0]) + S(p0[1]) / S(n) * S(dist)).v;
      rf[1] = (S(rf[1]) + S(p0[2]) / S(n) * S(dist)).v;
      rf[2] = (S(rf[2]) + S(p0[3]) / S(n) * S(dist)).v;
    } else {
      const double losses = T.t.dEdx_GeV_per_m;
      const double m_tab = table_mass(pid);
      bool hard = false;
      double dz = 0.0;
      int guard = 0;
      while (!hard && pf[0] >= pme) {
        if (++guard > c.loop_limit) { raise_status(c.status, c.err_info, PT_TIMEOUT, -1, pf[0], 0); break; }
        const double mfp = mfp_of(T, pid, pf[0]);
        const double u_hard = rng.u();
        dz = (S(mfp) / (S(6.0) + S(14.0) * S(rng.u()))).v;
        if (u_hard > exp(-dz / mfp)) {
          hard = true;
        } else {
          lose_energy(pf, mass, (S(losses) * S(dz)).v);
          move_along(pf, rf, dz);
          if (c.ms) mcs_apply(BETHE, pf, (S(T.t.rho) * (S(dz) / S(kCmToM))).v, T.t, c.rescale, m_tab, rng);
        }
      }
      const double distC = rng.u();
      double last;
      if (pf[0] < pme) {
        last = (S(distC) * S(dz)).v;
      } else {
        const double mfp = mfp_of(T, pid, pf[0]);
        const S e = S(exp(-dz / mfp));
        last = (S(mfp) * S(log((S(1.0) / (S(1.0) + (e - S(1.0)) * S(distC))).v))).v;
      }
      lose_energy(pf, mass, (S(losses) * S(last)).v);
      move_along(pf, rf, last);
      // shower.py:596-598 passes no m_lepton: the electron mass applies
      if (c.ms) mcs_apply(BETHE, pf, (S(T.t.rho) * (S(last) / S(kCmToM))).v, T.t, c.rescale, kMe, rng);
    }
  }

  // ---- process choice and sample_scattering (shower.py:467-507, 665-698)
  int want = 0;
  V4 da, db;
  int pa = 0, pb = 0, process = -1;
  const int proc_choice = choose_process(T, pid, pf[0], rng);
  if (proc_choice >= 0 && pf[0] > pme) {
    process = proc_choice;
    const Rot R = rotation_from(pf);
    double x[4];
    int key_lu;
    int64_t props;
    if (!draw_sample_fp64(T, process, pf[0], c.max_n_integrators, rng, x, key_lu, props)) {
      raise_status(c.status, c.err_info, PT_NO_SAMPLE, process, pf[0], key_lu);
    } else {
      const double ph = 2.0 * kPi * rng.u();
      V4 a, b;
      switch (process) {
        case PT_BREM: case PT_MUONBREM: kin_brem(pf[0], mass, x, ph, a, b); pa = pid; pb = 22; break;
        case PT_PAIRPROD: kin_pairprod(pf[0], x, ph, a, b); pa = -11; pb = 11; break;
        case PT_COMP: kin_compton(pf[0], x[0], ph, a, b); pa = 11; pb = 22; break;
        case PT_ANN: kin_ann(pf[0], x[0], ph, a, b); pa = 22; pb = 22; break;
        case PT_MOLLER: case PT_BHABHA: kin_ee(pf[0], x[0], ph, a, b); pa = pid; pb = 11; break;
        default: kin_mue(pf[0], x[0], ph, a, b); pa = pid; pb = 11; break;
      }
      da = to_lab(R, a);
      db = to_lab(R, b);
      want = (da.e > c.min_energy) + (db.e > c.min_energy);
    }
  }

  // ---- write this particle's final state
  for (int k = 0; k < 4; ++k) P.pf[k * cap + row] = pf[k];
  for (int k = 0; k < 3; ++k) P.rf[k * cap + row] = rf[k];
  P.draws[row] = (int32_t)rng.n;

  // ---- push daughters (one atomic per warp)
  const unsigned long long base = warp_reserve(c.n_rows, want);
  const unsigned long long qbase = warp_reserve(c.n_out, want);
  if (want) {
    int slot = 0;
    for (int bit = 0; bit < 2; ++bit) {
      const V4& v = bit ? db : da;
      if (!(v.e > c.min_energy)) continue;
      const unsigned long long r = base + slot;
      const unsigned long long q = qbase + slot;
      ++slot;
      if ((int64_t)r >= cap || (int64_t)q >= c.live_cap) { raise_status(c.status, nullptr, PT_OOM, -1, 0.0, 0); continue; }
      const int dpid = bit ? pb : pa;
      P.p0[0 * cap + r] = v.e; P.p0[1 * cap + r] = v.x; P.p0[2 * cap + r] = v.y; P.p0[3 * cap + r] = v.z;
      P.pf[0 * cap + r] = v.e; P.pf[1 * cap + r] = v.x; P.pf[2 * cap + r] = v.y; P.pf[3 * cap + r] = v.z;
      for (int k = 0; k < 3; ++k) { P.r0[k * cap + r] = rf[k]; P.rf[k * cap + r] = rf[k]; }
      P.weight[r] = P.weight[row];
      P.mass[r] = table_mass(dpid);
      P.pid[r] = dpid;
      P.gen[r] = P.gen[row] + 1;
      P.proc[r] = process;
      P.bit[r] = bit;
      P.primary[r] = P.primary[row];
      P.draws[r] = 0;
      P.parent[r] = row;
      P.pkey[r] = daughter_key(key, bit);
      c.live_out[q] = (int64_t)r;
    }
  }
}

__global__ void k_sample_only(Tabs T, int process, const double* E, const uint64_t* pkey, int64_t n,
                              uint64_t seed, int64_t max_n_integrators, double* x, int64_t* props,
                              int32_t* keys, int* status, double* info) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Rng rng;
  rng.init(seed, pkey[i]);
  double xx[4] = {0, 0, 0, 0};
  int key;
  int64_t p;
  const bool ok = draw_sample_fp64(T, process, E[i], max_n_integrators, rng, xx, key, p);
  if (!ok) raise_status(status, info, PT_NO_SAMPLE, process, E[i], key);
  for (int k = 0; k < 4; ++k) x[i * 4 + k] = xx[k];
  props[i] = ok ? p : -1;
  keys[i] = key;
}

__global__ void k_dsigma(Tabs T, int process, const double* x, const double* E, int64_t n, double* out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xx[4];
  for (int k = 0; k < 4; ++k) xx[k] = x[i * 4 + k];
  out[i] = dsigma_any(T, process, xx, E[i]);
}

}  // namespace

// ----------------------------------------------------------------- handle
struct pt_handle {
  Tabs T;
  int64_t scratch_cap = 0;
  int64_t* live[2] = {nullptr, nullptr};
  unsigned long long* counters = nullptr;   // [0] n_out, [1] n_rows
  int* status = nullptr;
  double* err_info = nullptr;
  unsigned long long* h_counters = nullptr; // pinned
  int* h_status = nullptr;
  double last_info[3] = {0, 0, 0};
  int64_t launches[2] = {0, 0};   // kernel launches, waves of the last run
  double kernel_ms[2] = {0, 0};   // batched run: propagation and sampler device time
  int32_t tuning[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};   // pt_set_batch_tuning (0 = library default)
  BatchScratch* batch = nullptr;
  BatchScratch* lane_batch[kMaxLanes] = {};   // lanes 1.. of a run with pt_batch_tuning.lanes > 1
};

pt_status batch_scratch_get(pt_handle* h, BatchScratch** out, int64_t ring_capacity) {
  pt_status s = batch_scratch_alloc(&h->batch, ring_capacity);
  *out = h->batch;
  return s;
}

pt_status batch_lane_scratch_get(pt_handle* h, int lane, BatchScratch** out, int64_t ring_capacity) {
  if (lane == 0) return batch_scratch_get(h, out, ring_capacity);
  if (lane < 0 || lane >= kMaxLanes) return PT_BAD_ARG;
  pt_status s = batch_scratch_alloc(&h->lane_batch[lane], ring_capacity);
  *out = h->lane_batch[lane];
  return s;
}

HandleParts handle_parts(pt_handle* h) {
  return HandleParts{&h->T, h->status, h->err_info, h->last_info, h->launches, h->kernel_ms, h->tuning};
}

static const char* kMessages[] = {
    "ok", "No Sample Found", "device loop limit reached", "inconsistent tables",
    "capacity exceeded", "CUDA error", "invalid argument"};

extern "C" const char* pt_strerror(int s) {
  if (s < 0 || s > 6) return "unknown status";
  return kMessages[s];
}

#define PT_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      fprintf(stderr, "petite_gpu: %s failed: %s\n", #call, cudaGetErrorString(e_)); \
      return PT_CUDA_ERR;                                                      \
    }                                                                          \
  } while (0)

extern "C" pt_status pt_create(const pt_tables* t, pt_handle** out) {
  if (!t || !out) return PT_BAD_ARG;
  *out = nullptr;
  if (!t->map_energy || !t->map_maxF || !t->map_neval || !t->grid_offset || !t->grid_ninc ||
      !t->grid_nodes || !t->ns_x || !t->ns_y || t->n_rows <= 0)
    return PT_BAD_TABLE;
  for (int p = 0; p < PT_N_PROCESSES; ++p)
    if (t->map_rows[p] <= 0 || t->map_base[p] < 0 || t->map_base[p] + t->map_rows[p] > t->n_rows) return PT_BAD_TABLE;
  for (int s = 0; s < PT_N_NSIGMA; ++s)
    if (t->ns_len[s] < 2 || t->ns_base[s] < 0) return PT_BAD_TABLE;
  pt_handle* h = new (std::nothrow) pt_handle();
  if (!h) return PT_OOM;
  h->T.t = *t;
  h->T.a0sq = t->a0sq;
  h->T.Z2a04 = t->Z2a04;
  if (cudaMalloc(&h->counters, 4 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&h->status, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&h->err_info, 4 * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&h->h_counters, 4 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&h->h_status, 4 * sizeof(int)) != cudaSuccess) {
    pt_destroy(h);
    return PT_CUDA_ERR;
  }
  *out = h;
  return PT_OK;
}

extern "C" void pt_destroy(pt_handle* h) {
  if (!h) return;
  batch_scratch_free(h->batch);
  for (BatchScratch* b : h->lane_batch) batch_scratch_free(b);
  cudaFree(h->live[0]);
  cudaFree(h->live[1]);
  cudaFree(h->counters);
  cudaFree(h->status);
  cudaFree(h->err_info);
  cudaFreeHost(h->h_counters);
  cudaFreeHost(h->h_status);
  delete h;
}

extern "C" pt_status pt_last_error_info(pt_handle* h, int32_t* process, double* energy, int32_t* lu_key) {
  if (!h) return PT_BAD_ARG;
  if (process) *process = (int32_t)h->last_info[0];
  if (energy) *energy = h->last_info[1];
  if (lu_key) *lu_key = (int32_t)h->last_info[2];
  return PT_OK;
}

static pt_status ensure_scratch(pt_handle* h, int64_t cap) {
  if (h->scratch_cap >= cap) return PT_OK;
  cudaFree(h->live[0]);
  cudaFree(h->live[1]);
  h->live[0] = h->live[1] = nullptr;
  h->scratch_cap = 0;
  PT_CUDA(cudaMalloc(&h->live[0], cap * sizeof(int64_t)));
  PT_CUDA(cudaMalloc(&h->live[1], cap * sizeof(int64_t)));
  h->scratch_cap = cap;
  return PT_OK;
}

static pt_status read_status(pt_handle* h, cudaStream_t st) {
  PT_CUDA(cudaMemcpyAsync(h->h_status, h->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  PT_CUDA(cudaStreamSynchronize(st));
  const int s = h->h_status[0];
  if (s != PT_OK) {
    PT_CUDA(cudaMemcpy(h->last_info, h->err_info, 3 * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return (pt_status)s;
}

extern "C" pt_status pt_run_sm(pt_handle* h, pt_particles* P, int64_t n_primaries, const pt_opts* o,
                               int64_t* n_rows, void* stream) {
  if (!h || !P || !o || !n_rows || n_primaries < 0 || n_primaries > P->capacity) return PT_BAD_ARG;
  if (o->precision != 0) return PT_BAD_ARG;
  *n_rows = n_primaries;
  if (n_primaries == 0) return PT_OK;
  cudaStream_t st = (cudaStream_t)stream;
  pt_status s = ensure_scratch(h, P->capacity);
  if (s != PT_OK) return s;
  PT_CUDA(cudaMemsetAsync(h->status, 0, sizeof(int), st));
  PT_CUDA(cudaMemsetAsync(h->counters, 0, 4 * sizeof(unsigned long long), st));
  const int tb = 256;
  k_init_primaries<<<(unsigned)((n_primaries + tb - 1) / tb), tb, 0, st>>>(*P, n_primaries, o->primary_offset);
  k_iota<<<(unsigned)((n_primaries + tb - 1) / tb), tb, 0, st>>>(h->live[0], n_primaries);
  unsigned long long rows0 = (unsigned long long)n_primaries;
  PT_CUDA(cudaMemcpyAsync(h->counters + 1, &rows0, sizeof(rows0), cudaMemcpyHostToDevice, st));
  RunCtx c;
  c.T = h->T;
  c.min_energy = o->min_energy;
  c.rescale = o->rescale_MCS;
  c.max_n_integrators = o->max_n_integrators;
  c.ms = o->multiple_scattering;
  c.mcs_mode = o->mcs_mode;
  c.seed = o->seed;
  c.P = *P;
  c.n_out = h->counters + 0;
  c.n_rows = h->counters + 1;
  c.status = h->status;
  c.err_info = h->err_info;
  c.loop_limit = o->loop_limit > 0 ? o->loop_limit : (1 << 22);
  int cur = 0;
  int64_t n_in = n_primaries;
  const int tbt = 128;
  h->launches[0] = 2;
  h->launches[1] = 0;
  while (n_in > 0) {
    ++h->launches[0];
    ++h->launches[1];
    PT_CUDA(cudaMemsetAsync(h->counters + 0, 0, sizeof(unsigned long long), st));
    c.live_in = h->live[cur];
    c.n_in = n_in;
    c.live_out = h->live[cur ^ 1];
    c.live_cap = h->scratch_cap;
    if (c.mcs_mode) k_transport_fp64<1><<<(unsigned)((n_in + tbt - 1) / tbt), tbt, 0, st>>>(c);
    else k_transport_fp64<0><<<(unsigned)((n_in + tbt - 1) / tbt), tbt, 0, st>>>(c);
    PT_CUDA(cudaGetLastError());
    PT_CUDA(cudaMemcpyAsync(h->h_counters, h->counters, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    s = read_status(h, st);
    if (s != PT_OK) {
      *n_rows = (int64_t)h->h_counters[1];
      return s;
    }
    n_in = (int64_t)h->h_counters[0];
    cur ^= 1;
  }
  *n_rows = (int64_t)h->h_counters[1];
  return PT_OK;
}

// ------------------------------------------------- pt_run_sm without allocation
// pt_run_sm grows two live lists with cudaMalloc/cudaFree as the particle
// store grows.  Some callers cannot allocate device memory during a run: a
// host that has handed the device's free memory to its own caching pool
// (PyTorch's allocator, or an application with a fixed device-memory
// budget), where a cudaMalloc may fail, and callers that cannot accept the
// device-wide synchronisation of cudaFree.  pt_run_sm_noalloc runs the same
// kernels with their scratch (both live lists, the wave counters, the status
// word and the error record) in one static device array, located once per
// device with cudaGetSymbolAddress.
namespace {
constexpr int64_t kNoAllocMaxRows = int64_t(1) << 19;       // live-list entries (= particle rows)
constexpr size_t kNoAllocListBytes = size_t(kNoAllocMaxRows) * sizeof(int64_t);
constexpr size_t kNoAllocCtrOff = 2 * kNoAllocListBytes;    // 4 x u64 counters: [0] n_out, [1] n_rows
constexpr size_t kNoAllocStatusOff = kNoAllocCtrOff + 256;  // int status
constexpr size_t kNoAllocInfoOff = kNoAllocStatusOff + 256; // 4 x f64 error record
constexpr size_t kNoAllocBytes = kNoAllocInfoOff + 256;     // 8 MB + 768 B
constexpr int kNoAllocMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

unsigned char* g_noalloc_ptr[kNoAllocMaxDevices];
std::mutex g_noalloc_mu;

// Device address of the static scratch on the current device, looked up on
// the first call per device.  Only a successful lookup is kept: a lookup that
// failed (no context yet, or a call made during a stream capture) is tried
// again on the next call.
pt_status noalloc_scratch(unsigned char** out) {
  int dev = 0;
  PT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return PT_BAD_ARG;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      fprintf(stderr, "petite_gpu: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return PT_CUDA_ERR;
    }
    g_noalloc_ptr[dev] = (unsigned char*)p;
  }
  *out = g_noalloc_ptr[dev];
  return PT_OK;
}
}  // namespace

extern "C" pt_status pt_run_sm_noalloc(pt_handle* h, pt_particles* P, int64_t n_primaries, const pt_opts* o,
                                       int64_t* n_rows, void* stream) {
  if (!h || !P || !o || !n_rows || n_primaries < 0 || n_primaries > P->capacity) return PT_BAD_ARG;
  if (o->precision != 0) return PT_BAD_ARG;
  if (P->capacity > kNoAllocMaxRows) {
    fprintf(stderr, "petite_gpu: pt_run_sm_noalloc: particle capacity %lld exceeds the static scratch limit of %lld rows\n",
            (long long)P->capacity, (long long)kNoAllocMaxRows);
    return PT_BAD_ARG;
  }
  *n_rows = n_primaries;
  if (n_primaries == 0) return PT_OK;
  unsigned char* base = nullptr;
  pt_status s = noalloc_scratch(&base);
  if (s != PT_OK) return s;
  int64_t* live[2] = {(int64_t*)base, (int64_t*)(base + kNoAllocListBytes)};
  unsigned long long* counters = (unsigned long long*)(base + kNoAllocCtrOff);
  int* status = (int*)(base + kNoAllocStatusOff);
  double* err_info = (double*)(base + kNoAllocInfoOff);
  cudaStream_t st = (cudaStream_t)stream;
  // zero on entry: the status word, the error record and both counters; the
  // live lists are written before they are read
  PT_CUDA(cudaMemsetAsync(base + kNoAllocCtrOff, 0, kNoAllocBytes - kNoAllocCtrOff, st));
  const int tb = 256;
  k_init_primaries<<<(unsigned)((n_primaries + tb - 1) / tb), tb, 0, st>>>(*P, n_primaries, o->primary_offset);
  k_iota<<<(unsigned)((n_primaries + tb - 1) / tb), tb, 0, st>>>(live[0], n_primaries);
  // the row count starts at n_primaries, copied from the handle's pinned
  // host word (made by pt_create; every earlier copy into it has completed)
  h->h_counters[1] = (unsigned long long)n_primaries;
  PT_CUDA(cudaMemcpyAsync(counters + 1, h->h_counters + 1, sizeof(unsigned long long), cudaMemcpyHostToDevice, st));
  RunCtx c;
  c.T = h->T;
  c.min_energy = o->min_energy;
  c.rescale = o->rescale_MCS;
  c.max_n_integrators = o->max_n_integrators;
  c.ms = o->multiple_scattering;
  c.mcs_mode = o->mcs_mode;
  c.seed = o->seed;
  c.P = *P;
  c.n_out = counters + 0;
  c.n_rows = counters + 1;
  c.status = status;
  c.err_info = err_info;
  c.loop_limit = o->loop_limit > 0 ? o->loop_limit : (1 << 22);
  int cur = 0;
  int64_t n_in = n_primaries;
  const int tbt = 128;
  h->launches[0] = 2;
  h->launches[1] = 0;
  while (n_in > 0) {
    ++h->launches[0];
    ++h->launches[1];
    PT_CUDA(cudaMemsetAsync(counters + 0, 0, sizeof(unsigned long long), st));
    c.live_in = live[cur];
    c.n_in = n_in;
    c.live_out = live[cur ^ 1];
    c.live_cap = kNoAllocMaxRows;
    if (c.mcs_mode) k_transport_fp64<1><<<(unsigned)((n_in + tbt - 1) / tbt), tbt, 0, st>>>(c);
    else k_transport_fp64<0><<<(unsigned)((n_in + tbt - 1) / tbt), tbt, 0, st>>>(c);
    PT_CUDA(cudaGetLastError());
    PT_CUDA(cudaMemcpyAsync(h->h_counters, counters, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaMemcpyAsync(h->h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    PT_CUDA(cudaStreamSynchronize(st));
    if (h->h_status[0] != PT_OK) {
      PT_CUDA(cudaMemcpy(h->last_info, err_info, 3 * sizeof(double), cudaMemcpyDeviceToHost));
      *n_rows = (int64_t)h->h_counters[1];
      return (pt_status)h->h_status[0];
    }
    n_in = (int64_t)h->h_counters[0];
    cur ^= 1;
  }
  *n_rows = (int64_t)h->h_counters[1];
  return PT_OK;
}

extern "C" pt_status pt_last_run_stats(pt_handle* h, int64_t* launches, int64_t* waves) {
  if (!h) return PT_BAD_ARG;
  if (launches) *launches = h->launches[0];
  if (waves) *waves = h->launches[1];
  return PT_OK;
}

extern "C" pt_status pt_set_batch_tuning(pt_handle* h, const pt_batch_tuning* t) {
  if (!h) return PT_BAD_ARG;
  if (!t) {
    for (int k = 0; k < 9; ++k) h->tuning[k] = 0;
    return PT_OK;
  }
  for (int k = 0; k < 2; ++k) {
    if (t->refill_min[k] < 0 || t->refill_min[k] > 32) return PT_BAD_ARG;
    if (t->chunk[k] != 0 && (t->chunk[k] < 32 || t->chunk[k] > 4096)) return PT_BAD_ARG;
  }
  if (t->loop < PT_LOOP_HOST || t->loop > PT_LOOP_PERSISTENT) return PT_BAD_ARG;
  if (t->staging < PT_STAGE_DEFAULT || t->staging > PT_STAGE_SHARED) return PT_BAD_ARG;
  if (t->threads != 0 && t->threads != 64 && t->threads != 128 && t->threads != 256) return PT_BAD_ARG;
  if (t->barrier_ns < 0) return PT_BAD_ARG;
  if (t->lanes < 0 || t->lanes > kMaxLanes || (t->lanes > 1 && t->loop != PT_LOOP_HOST)) return PT_BAD_ARG;
  h->tuning[0] = t->refill_min[0];
  h->tuning[1] = t->refill_min[1];
  h->tuning[2] = t->chunk[0];
  h->tuning[3] = t->chunk[1];
  h->tuning[4] = t->loop;
  h->tuning[5] = t->staging;
  h->tuning[6] = t->threads;
  h->tuning[7] = t->barrier_ns;
  h->tuning[8] = t->lanes;
  return PT_OK;
}

extern "C" pt_status pt_last_kernel_times(pt_handle* h, double* propagate_ms, double* sample_ms) {
  if (!h) return PT_BAD_ARG;
  if (propagate_ms) *propagate_ms = h->kernel_ms[0];
  if (sample_ms) *sample_ms = h->kernel_ms[1];
  return PT_OK;
}

// ------------------------------------------------- arithmetic peak of the GPU
// Eight independent fused multiply-add chains per thread (a = a*b + c, which
// converges to c/(1-b): no overflow, no subnormals) on a grid that fills
// every SM's threads.  2 flops per FMA.
namespace {
template <class T>
__global__ void __launch_bounds__(256) k_fma_chains(T* sink, int iters, T b, T c) {
  T a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = (T)(threadIdx.x + 8 * k) * (T)1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == (T)-1) sink[blockIdx.x] = s;     // never true: keeps the chains live
}

template <class T>
pt_status fma_rate(T* sink, cudaStream_t st, double* flops_per_s) {
  int dev = 0, sms = 0, per = 0;
  PT_CUDA(cudaGetDevice(&dev));
  PT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fma_chains<T>, 256, 0));
  const int grid = sms * (per > 0 ? per : 1);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  PT_CUDA(cudaEventCreate(&e0));
  PT_CUDA(cudaEventCreate(&e1));
  pt_status rs = PT_OK;
  int iters = 256;
  float ms = 0.f;
  for (int pass = 0; pass < 8; ++pass) {         // grow the run to about 5 ms, then time it
    k_fma_chains<T><<<grid, 256, 0, st>>>(sink, iters, (T)0.999, (T)1e-3);
    cudaEventRecord(e0, st);
    k_fma_chains<T><<<grid, 256, 0, st>>>(sink, iters, (T)0.999, (T)1e-3);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      rs = PT_CUDA_ERR;
      break;
    }
    if (ms >= 4.f || iters >= (1 << 26)) break;
    iters = ms > 0.05f ? (int)std::min<double>(iters * 5.0 / ms, double(1 << 26)) : iters * 16;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rs != PT_OK || ms <= 0.f) return PT_CUDA_ERR;
  *flops_per_s = 2.0 * 8.0 * (double)iters * grid * 256.0 / (ms * 1e-3);
  return PT_OK;
}
}  // namespace

extern "C" pt_status pt_alu_peaks(double* fp32_flops, double* fp64_flops, void* stream) {
  if (!fp32_flops || !fp64_flops) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  double* sink = nullptr;
  PT_CUDA(cudaMalloc(&sink, 65536 * sizeof(double)));
  pt_status s = fma_rate<float>(reinterpret_cast<float*>(sink), st, fp32_flops);
  if (s == PT_OK) s = fma_rate<double>(sink, st, fp64_flops);
  cudaFree(sink);
  return s;
}

extern "C" pt_status pt_sample_only(pt_handle* h, int32_t process, const double* energy, const uint64_t* pkey,
                                    int64_t n, const pt_opts* o, double* x, int64_t* proposals,
                                    int32_t* lu, void* stream) {
  if (!h || !o || process < 0 || process >= PT_N_PROCESSES || n < 0) return PT_BAD_ARG;
  if (n == 0) return PT_OK;
  if (!energy || !pkey || !x || !proposals || !lu) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  PT_CUDA(cudaMemsetAsync(h->status, 0, sizeof(int), st));
  const int tb = 128;
  k_sample_only<<<(unsigned)((n + tb - 1) / tb), tb, 0, st>>>(h->T, process, energy, pkey, n, o->seed,
                                                              o->max_n_integrators, x, proposals, lu,
                                                              h->status, h->err_info);
  PT_CUDA(cudaGetLastError());
  return read_status(h, st);
}

static __global__ void k_moliere_x(const double* u, const double* B, int64_t n, int prec, double* x) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = prec ? (double)moliere_x<float>((float)u[i], (float)B[i]) : moliere_x<double>(u[i], B[i]);
}

extern "C" pt_status pt_moliere_inverse_cdf(const double* u, const double* B, int64_t n, int32_t precision,
                                            double* x, void* stream) {
  if (n < 0 || precision < 0 || precision > 1) return PT_BAD_ARG;
  if (n == 0) return PT_OK;
  if (!u || !B || !x) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int tb = 128;
  k_moliere_x<<<(unsigned)((n + tb - 1) / tb), tb, 0, st>>>(u, B, n, precision, x);
  PT_CUDA(cudaGetLastError());
  PT_CUDA(cudaStreamSynchronize(st));
  return PT_OK;
}

extern "C" pt_status pt_dsigma(pt_handle* h, int32_t process, const double* x, const double* energy, int64_t n,
                               int32_t precision, double* value, void* stream) {
  if (!h || process < 0 || process >= PT_N_PROCESSES || n < 0 || precision != 0) return PT_BAD_ARG;
  if (n == 0) return PT_OK;
  if (!x || !energy || !value) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int tb = 256;
  k_dsigma<<<(unsigned)((n + tb - 1) / tb), tb, 0, st>>>(h->T, process, x, energy, n, value);
  PT_CUDA(cudaGetLastError());
  PT_CUDA(cudaStreamSynchronize(st));
  return PT_OK;
}
