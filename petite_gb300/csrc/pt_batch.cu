// pt_batch.cu -- batched shower transport with tallies (pt_run_batch).
//
// Live particles sit in a power-of-two ring buffer in HBM (structure of
// arrays).  Primaries stream in while there is room; each wave takes up to
// (capacity - live)/2 entries from the head, so the at most two daughters per
// entry always fit behind the tail.  A wave is two kernels:
//  1. k_propagate: propagate_particle (shower.py:509-601) and the process
//     choice (shower.py:665-698).  Lanes refill themselves and advance one
//     charged-particle substep per iteration, so a long track does not hold
//     its warp.  Interacting particles are parked in place and listed by
//     process; the others are tallied and retired.
//  2. k_sample: draw_sample's accept/reject loop (shower.py:401-465) over the
//     task list ordered by process, one proposal per lane per iteration with
//     refill, then the final-state kinematics and lab rotation
//     (shower.py:467-507); daughters above min_energy are appended at the tail.
// Both kernels run warp-convergent loops: refills come from a warp-private
// pool of work indices fetched CHUNK at a time (one atomic per chunk), and
// sampling tasks are gathered per warp and process and published 32 at a
// time, so no counter is hit once per particle.
// PREC = 0 is the float64 engine (same device functions and operation order
// as pt_run_sm, hence the same showers); PREC = 1 samples, scatters and
// builds directions in float32 and keeps energies in float64.
#include <algorithm>
#include <chrono>
#include <thread>
#include <cstdio>
#include <type_traits>

#include "pt_internal.cuh"
#include "pt_physics32.cuh"
#include "pt_tma.cuh"

using namespace pt;

namespace {

constexpr int kThreads = 128;
// Defaults of the runtime tuning (pt_set_batch_tuning): idle lanes a warp
// gathers before refilling them (1 = refill at once), and work entries a
// warp claims from the wave's pool per atomic.
constexpr int kRefillMinPropagate = 8;
constexpr int kRefillMinSample = 8;
constexpr int kChunkPropagate = 128;
constexpr int kChunkSample = 64;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kHB = PT_HIST_BINS;
constexpr int kHist = 3 * 4 * kHB;

// Ring entry fields.  Energies are float64 in both engines; the mixed engine
// keeps momenta, positions and masses in float32.
template <int PREC> struct RingT {
  using R = typename std::conditional<PREC == 0, double, float>::type;
  double* E;
  float* E32;                           // (float)E, written with E in the mixed form: the propagation
                                        // kernel's refill then needs no float64 conversion
  R *px, *py, *pz, *x, *y, *z, *mass;
  uint64_t* key;
  int32_t *pid, *prim, *gen;
};

// A sampling task: the state of a particle that interacts, after its
// propagation (energy, momentum, position), its stream position, its map
// row and what its daughters inherit.  One record per task, so the sampler
// reads two 32-byte sectors per task in the mixed form instead of gathering
// a sector for each ring field.  The first 32 bytes hold what the sampler
// reads when it takes the task; the rest is read by the kinematics.
template <int PREC> struct Park;
template <> struct alignas(64) Park<1> {
  double E;
  uint64_t key;
  int32_t row;
  uint32_t draw;
  int32_t pid, gen;
  float px, py, pz, x, y, z, mass;
  int32_t prim;
};
template <> struct alignas(32) Park<0> {
  double E;
  uint64_t key;
  int32_t row;
  uint32_t draw;
  int32_t pid, gen;
  double px, py, pz, x, y, z, mass;
  int32_t prim, pad;
};
static_assert(sizeof(Park<1>) == 64 && sizeof(Park<0>) == 96, "task record layout");
// Tasks are parked in chunks of 32 records of one process.  A chunk-list
// entry is (chunk id << 5) | (tasks in the chunk - 1).
constexpr int kChunkTasks = 32;

struct Tally {
  unsigned long long* counts;
  double* energy;
  unsigned int* hist;
  unsigned int* prim_count;
  double* prim_edep;
  float z_max;
};

// The loop state when the GPU plans the waves itself (the graph-captured loop
// and the persistent kernel): written by plan_step between waves.
struct WavePlan {
  unsigned long long head, tail;      // ring positions of the wave's first entry and of the append point
  unsigned long long feed_at;         // ring position of this wave's fed primaries
  long long fed;                      // primaries fed so far
  long long n_in;                     // entries in this wave
  long long feed_m;                   // primaries this wave feeds
  long long waves;                    // waves run
  int out_chunk;                      // as WaveCtx::out_chunk
  int done;                           // 1: the run has ended (all primaries finished, or an error)
};

// Float32 forms of the table and option constants, rounded once on the
// host: the float32 kernels read them as parameters, with no float64
// conversion (a float64-pipe instruction) left for the compiler to repeat
// inside their loops.
struct Consts32 {
  float mc[4];                        // min_calc energy: photon, electron, positron, muon
  float min_energy, dedx, rho_cm, A, Z, Z23, Z13, rescale, Eg_min, Ee_min, a0sq;
  Ld32 ld;
};

template <int PREC> struct WaveCtx {
  Tabs T;
  Consts32 k32;
  double min_energy, rescale;
  int64_t max_n_integrators;
  int ms, mcs_mode;
  uint64_t seed;
  RingT<PREC> q;
  uint64_t mask;                      // ring capacity - 1
  uint64_t head, tail;                // ring positions of this wave's first entry and of the append point
  int64_t n_in;                       // entries in this wave
  int64_t list_cap;                   // largest wave
  int out_chunk;                      // output slots reserved per warp at a time (0 = exact)
  Park<PREC>* park;                   // [chunk_cap * 32] task records, in chunks of one process
  int32_t* chunks;                    // [8][chunk_cap] published chunks of each process
  int64_t chunk_cap;                  // chunks a wave may claim
  unsigned long long* ctr;            // [0] head1, [1] head2, [2] appended, [3] chunks claimed,
                                      // [8..15] chunks published per process
  int* status;
  double* err_info;
  Tally tally;
  int refill_min[2];                  // idle lanes a warp gathers before refilling: [0] propagation, [1] sampler
  int chunk[2];                       // pool entries a warp claims per atomic: [0] propagation, [1] sampler
  PhiloxRK rk;                        // round keys of `seed` (float32 kernels)
  int64_t max_waves;                  // waves a run may take (PT_TIMEOUT beyond)
  unsigned long long barrier_ns;      // the persistent kernel's bound on one grid-barrier wait
  // device-planned waves (null: the host plans each wave and passes it here)
  WavePlan* plan;
  pt_particles rows;                  // per-wave rows for a WaveRowsHook (capacity 0: none)
  const double* in_p0;                // the run's primaries, for the planned feed
  const double* in_r0;
  const int32_t* in_pid;
  const double* in_mass;
  int64_t n_prim, prim_offset, cap, feed_max, slack;
};

// This wave's parameters: from the plan when the GPU plans, else from the launch.
template <int PREC> __device__ __forceinline__ uint64_t w_head(const WaveCtx<PREC>& c) {
  return c.plan ? (uint64_t)__ldcg(&c.plan->head) : c.head;
}
template <int PREC> __device__ __forceinline__ uint64_t w_tail(const WaveCtx<PREC>& c) {
  return c.plan ? (uint64_t)__ldcg(&c.plan->tail) : c.tail;
}
template <int PREC> __device__ __forceinline__ int64_t w_n(const WaveCtx<PREC>& c) {
  return c.plan ? (int64_t)__ldcg(&c.plan->n_in) : c.n_in;
}
template <int PREC> __device__ __forceinline__ int w_out_chunk(const WaveCtx<PREC>& c) {
  return c.plan ? __ldcg(&c.plan->out_chunk) : c.out_chunk;
}

__device__ void raise_status(int* status, double* info, int code, int process, double E, int key) {
  if (atomicCAS(status, 0, code) == 0 && info) {
    info[0] = process; info[1] = E; info[2] = key;
  }
}

// ------------------------------------------------------- warp work pools
// Warp-uniform range [next, end) of work indices, refilled `chunk` at a time.
struct WarpPool {
  int64_t next = 0, end = 0;
  bool exhausted = false;
};

// Called by all 32 lanes.  Returns the lane's new index in [0, n) or -1.
__device__ __forceinline__ int64_t pool_take(WarpPool& P, unsigned long long* head, int64_t n, bool need,
                                             int chunk) {
  const unsigned b = __ballot_sync(kFull, need);
  if (!b) return -1;
  const int cnt = __popc(b);
  const int rank = __popc(b & lanemask_lt());
  const int64_t avail = P.end - P.next;
  int64_t got;
  if (avail >= cnt) {
    got = P.next + rank;
    P.next += cnt;
  } else {
    int64_t base = n;
    if (!P.exhausted) {
      unsigned long long bb = 0;
      if ((threadIdx.x & 31) == 0) bb = atomicAdd(head, (unsigned long long)chunk);
      base = (int64_t)__shfl_sync(kFull, bb, 0);
      if (base >= n) { P.exhausted = true; base = n; }
    }
    got = rank < avail ? P.next + rank : base + (rank - avail);
    P.next = base + (cnt - avail);
    P.end = P.exhausted ? base : base + chunk;
    if (P.next > P.end) P.next = P.end;
  }
  if (!need) return -1;
  return got < n ? got : -1;
}

// Pool entries claimed per atomic.  The sampler's: the tuned chunk, cut so
// that every warp of the grid can claim two (a deep shower's waves hold a
// few thousand tasks; 64-task claims left most warps idle), a multiple of
// 32, at least 32.  The propagation kernel's: 32 when the wave is no larger
// than the grid (one entry per thread), else the tuned chunk (cutting it for
// mid-sized waves on a full grid cost 1.5 % at 10^6 primaries).  The
// assignment of entries to warps changes no result: every particle and
// task draws from its own stream.
__device__ __forceinline__ int wave_chunk(int tuned, int64_t n) {
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t fair = (n / (2 * warps)) & ~(int64_t)31;
  return (int)(fair >= tuned ? tuned : (fair > 32 ? fair : 32));
}
__device__ __forceinline__ int wave_chunk_propagate(int tuned, int64_t n) {
  return n <= (int64_t)gridDim.x * blockDim.x ? 32 : tuned;
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
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
  };
  auto redd = [](double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
  };
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

// Per-primary tallies: one count atomic per distinct primary among the
// finishing lanes of the warp; energy deposits per lane.
__device__ __forceinline__ void primary_tally(const Tally& T, bool on, int prim, double edep) {
  if (!__any_sync(kFull, on)) return;
  const unsigned grp = __match_any_sync(kFull, on ? prim : -1 - (int)(threadIdx.x & 31));
  if (on && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(T.prim_count + prim, (unsigned)__popc(grp));
  if (on && edep != 0.0) atomicAdd(T.prim_edep + prim, edep);
}

// Output slots at the ring tail, reserved 64 at a time per warp.  Slots of a
// chunk left over when the kernel ends are written as dead entries (pid 0).
struct OutPool {
  uint64_t next = 0, end = 0;   // offsets from the wave's tail
};
constexpr int kOutChunk = 64;

// All lanes call.  Writes this lane's slot offsets (want of them) to slot[].
// chunk == 0 reserves exactly what is asked (small waves: no dead slots).
__device__ __forceinline__ void out_take(OutPool& P, unsigned long long* ctr, int want, uint64_t* slot, int chunk) {
  const unsigned b1 = __ballot_sync(kFull, want >= 1), b2 = __ballot_sync(kFull, want >= 2);
  const unsigned total = __popc(b1) + __popc(b2);
  if (!total) return;
  const unsigned lt = lanemask_lt();
  const uint64_t prefix = __popc(b1 & lt) + __popc(b2 & lt);
  if (chunk == 0) {
    unsigned long long bb = 0;
    if ((threadIdx.x & 31) == 0) bb = atomicAdd(ctr, (unsigned long long)total);
    bb = __shfl_sync(kFull, bb, 0);
    for (int j = 0; j < want; ++j) slot[j] = bb + prefix + j;
    return;
  }
  const uint64_t avail = P.end - P.next;
  uint64_t base = 0;
  if (avail < total) {
    unsigned long long bb = 0;
    if ((threadIdx.x & 31) == 0) bb = atomicAdd(ctr, (unsigned long long)kOutChunk);
    base = __shfl_sync(kFull, bb, 0);
  }
  for (int j = 0; j < want; ++j) {
    const uint64_t r = prefix + j;
    slot[j] = r < avail ? P.next + r : base + (r - avail);
  }
  if (avail < total) { P.next = base + (total - avail); P.end = base + kOutChunk; }
  else P.next += total;
}

// ---------------------------------------------- float32 table lookups
// The float32 n*sigma tables (nodes, values, slopes) read either through the
// read-only data path (SH = false) or from a block's shared-memory copy
// (SH = true; staged by TMA bulk copies, stage_ns_tables).  Each slot's
// first entry, length and index-guess constants sit in a small header in the
// block's shared memory, so lanes of different species look up different
// slots with the same instructions (one copy of the lookup code instead of
// one per species, which also keeps the kernel's code small).
struct NsHdr { int base, len; float lnx0, idl; };
template <bool SH> struct Ns32 { const float* x; const float* y; const float* s; const NsHdr* h; };
template <bool SH> __device__ __forceinline__ float ld32(const float* p) {
  if constexpr (SH) return *p;
  else return __ldg(p);
}
__device__ __forceinline__ Ns32<false> ns_global(const Tabs& T) {
  return {T.t.ns_x32, T.t.ns_y32, T.t.ns_s32, nullptr};
}

// One thread fills the block's slot headers (call before a block barrier).
__device__ __forceinline__ void fill_ns_hdr(const Tabs& T, NsHdr* h) {
  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < PT_N_NSIGMA; ++s) h[s] = {T.t.ns_base[s], T.t.ns_len[s], T.t.ns_lnx0[s], T.t.ns_invdlog[s]};
  }
}

template <bool SH>
__device__ __forceinline__ int geo_index(const float* x, int n, float lnx0, float idl, float lnE, float E) {
  int j = (int)((lnE - lnx0) * idl);
  j = j < 0 ? 0 : (j > n - 2 ? n - 2 : j);
  while (j > 0 && ld32<SH>(x + j) > E) --j;
  while (j < n - 2 && ld32<SH>(x + j + 1) <= E) ++j;
  return j;
}

// interp1d(kind='linear', fill_value=0) in float32 (shower.py:280-295);
// lnE = __logf(E), for the index guess on the geometric grid.
template <bool SH>
__device__ __forceinline__ float nsig32(const Ns32<SH>& v, int slot, float E, float lnE) {
  const NsHdr h = v.h[slot];
  const float* x = v.x + h.base;
  const int n = h.len;
  if (!(E >= ld32<SH>(x)) || E > ld32<SH>(x + n - 1)) return 0.f;
  const int j = geo_index<SH>(x, n, h.lnx0, h.idl, lnE, E);
  return fmaf(E - ld32<SH>(x + j), ld32<SH>(v.s + h.base + j), ld32<SH>(v.y + h.base + j));
}

// Mean free path (shower.py:357-389): the slots summed in the reference's
// order -- photon PairProd + Comp, electron Brem + Moller, positron Brem +
// Bhabha + Ann, muon MuonBrem + MuonE -- chosen by selects on the PID.
template <bool SH>
__device__ __forceinline__ float mfp32(const Ns32<SH>& v, int pid, float E) {
  const int a = pid == 22 ? 1 : (pid == 11 || pid == -11 ? 0 : 7);
  const int b = pid == 22 ? 3 : (pid == 11 ? 4 : (pid == -11 ? 5 : 6));
  const float lnE = __logf(E);
  float ns = nsig32(v, a, E, lnE) + nsig32(v, b, E, lnE);
  if (pid == -11) ns += nsig32(v, 2, E, lnE);
  return ns > 0.f ? __fdividef((float)kCmToM, ns) : 1.0e12f;   // ns far inside float32's range
}

// Process choice in float32 (shower.py:665-698): electron {Brem, Moller},
// positron {Brem, Ann, Bhabha}, photon {PairProd, Comp}, muon {MuonE,
// MuonBrem}, with slots and process codes chosen by selects on the PID.
template <bool SH>
__device__ __forceinline__ int choose32(const Ns32<SH>& v, int pid, float E, float u) {
  const bool g = pid == 22, em = pid == 11, ep = pid == -11;
  const int s0 = g ? 1 : (em || ep ? 0 : 6);
  const int s1 = g ? 3 : (em ? 4 : (ep ? 2 : 7));
  const int n0 = g ? PT_PAIRPROD : (em || ep ? PT_BREM : PT_MUONE);
  const int n1 = g ? PT_COMP : (em ? PT_MOLLER : (ep ? PT_ANN : PT_MUONBREM));
  const float lnE = __logf(E);
  const float c0 = nsig32(v, s0, E, lnE), c1 = nsig32(v, s1, E, lnE);
  const float c2 = ep ? nsig32(v, 5, E, lnE) : 0.f;
  const float sum = c0 + c1 + c2;
  if (!(sum > 0.f)) return -1;
  const float t = u * sum;
  if (c0 > t) return n0;
  if (c0 + c1 > t || !ep) return n1;
  return PT_BHABHA;
}

// LU_Key (shower.py:416-426) in float32: argmin |E_i - E| + 1, clipped.
__device__ __forceinline__ int lu_key32(const Tabs& T, int process, float E) {
  const float* Ei = T.t.map_energy32 + T.t.map_base[process];
  const int n = T.t.map_rows[process];
  int best;
  if (!(E > __ldg(Ei))) best = 0;
  else if (E >= __ldg(Ei + n - 1)) best = n - 1;
  else {
    const int j = geo_index<false>(Ei, n, T.t.map_lnE0[process], T.t.map_invdlog[process], __logf(E), E);  // Ei[j] <= E < Ei[j+1]
    best = (E - __ldg(Ei + j) <= __ldg(Ei + j + 1) - E) ? j : j + 1;
  }
  const int key = best + 1;
  return key >= n ? n - 1 : key;
}

// Process choice (shower.py:665-698), float64 (the float64 engine).
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

// Places this iteration's sampling tasks: returns, for each lane with
// `emit`, the record slot of its task of `process` in the warp's open chunk
// of that process (-1 for the other lanes); the caller writes the record.
// A warp holds one open chunk per process (`open[p]`: chunk id, or -1, and
// its fill; shared, written by lane 0 only), claims a new chunk from the
// wave's counter when the open one cannot take the group, and publishes a
// chunk to its process's list once it is full.  A claim beyond chunk_cap
// (the wave's bound, which the host's sizing keeps) records PT_OOM and those
// tasks get no slot.  All 32 lanes call it.
template <class Ctx>
__device__ __forceinline__ long long park_slot(const Ctx& c, volatile int (*open)[2], bool emit, int process) {
  unsigned left = __ballot_sync(kFull, emit);
  const int lane = threadIdx.x & 31;
  long long slot = -1;
  while (left) {
    const int leader = __ffs(left) - 1;
    const int p = __shfl_sync(kFull, process, leader);
    const unsigned m = __ballot_sync(kFull, emit && process == p);
    const int cnt = __popc(m);
    const int id = open[p][0], f = open[p][1];
    const int avail = id < 0 ? 0 : kChunkTasks - f;
    long long id2 = -1;
    if (cnt > avail) {
      unsigned long long b = 0;
      if (lane == 0) b = atomicAdd(c.ctr + 3, 1ull);
      id2 = (long long)__shfl_sync(kFull, b, 0);
      if (id2 >= c.chunk_cap) {
        if (lane == 0) atomicCAS(c.status, 0, PT_OOM);
        id2 = -1;
      }
    }
    if (emit && process == p) {
      const int r = __popc(m & lanemask_lt());
      if (r < avail) slot = (long long)id * kChunkTasks + f + r;
      else if (id2 >= 0) slot = id2 * kChunkTasks + (r - avail);
    }
    // the chunks this group filled go to the process's list
    int nid = id, nf = f + cnt;
    if (cnt >= avail) {
      if (lane == 0 && avail > 0) {
        const unsigned long long q = atomicAdd(c.ctr + 8 + p, 1ull);
        c.chunks[(int64_t)p * c.chunk_cap + (int64_t)q] = (int32_t)(((unsigned)id << 5) | (kChunkTasks - 1));
      }
      nid = (int)id2;
      nf = cnt - avail;
      if (nid >= 0 && nf == kChunkTasks) {
        if (lane == 0) {
          const unsigned long long q = atomicAdd(c.ctr + 8 + p, 1ull);
          c.chunks[(int64_t)p * c.chunk_cap + (int64_t)q] = (int32_t)(((unsigned)nid << 5) | (kChunkTasks - 1));
        }
        nid = -1;
      }
      if (nid < 0) nf = 0;
    }
    left &= ~m;
    __syncwarp();
    if (lane == 0) { open[p][0] = nid; open[p][1] = nf; }
    __syncwarp();
  }
  return slot;
}

// Publishes the warp's partly filled chunks and closes them.  All lanes call.
template <class Ctx>
__device__ __forceinline__ void park_rest(const Ctx& c, volatile int (*open)[2]) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    for (int p = 0; p < 8; ++p) {
      const int id = open[p][0], f = open[p][1];
      if (id >= 0 && f > 0) {
        const unsigned long long q = atomicAdd(c.ctr + 8 + p, 1ull);
        c.chunks[(int64_t)p * c.chunk_cap + (int64_t)q] = (int32_t)(((unsigned)id << 5) | (unsigned)(f - 1));
      }
      open[p][0] = -1;
      open[p][1] = 0;
    }
  }
  __syncwarp();
}

// ------------------------------------------------------ per-wave rows
// A particle's row for a WaveRowsHook (layout of pt_particles): written at
// the start of its propagation and completed at its end.
__device__ __forceinline__ void row_start(const pt_particles& r, int64_t s, int pid, double E, double px, double py,
                                          double pz, double mass, uint64_t key) {
  const int64_t cap = r.capacity;
  r.pid[s] = pid;
  if (pid == 0) return;
  r.p0[s] = E; r.p0[cap + s] = px; r.p0[2 * cap + s] = py; r.p0[3 * cap + s] = pz;
  r.mass[s] = mass;
  r.weight[s] = 1.0;
  r.pkey[s] = key;
}
__device__ __forceinline__ void row_end(const pt_particles& r, int64_t s, double E, double px, double py, double pz,
                                        double x, double y, double z) {
  const int64_t cap = r.capacity;
  r.pf[s] = E; r.pf[cap + s] = px; r.pf[2 * cap + s] = py; r.pf[3 * cap + s] = pz;
  r.rf[s] = x; r.rf[cap + s] = y; r.rf[2 * cap + s] = z;
}

// ------------------------------------------------------------ phase 1, float64
// Same device functions and operation order as the record engine (pt_run_sm).
struct PropShared64 {
  unsigned int hist[kHist];
  int open[kWarps][8][2];         // each warp's open task chunk per process: id, fill
};

template <int BETHE>
__device__ __forceinline__ void propagate_fp64_body(const WaveCtx<0>& c, PropShared64& sm) {
  unsigned int* sh_hist = sm.hist;
  const int64_t wave_n = w_n(c);
  const int chunk_p = wave_chunk_propagate(c.chunk[0], wave_n);
  const uint64_t wave_head = w_head(c);
  for (int k = threadIdx.x; k < kHist; k += blockDim.x) sh_hist[k] = 0;
  if (threadIdx.x < kWarps * 8) {
    sm.open[threadIdx.x / 8][threadIdx.x % 8][0] = -1;
    sm.open[threadIdx.x / 8][threadIdx.x % 8][1] = 0;
  }
  __syncthreads();
  volatile int (*open)[2] = sm.open[threadIdx.x / 32];
  const Tabs& T = c.T;
  LocalTally L;
  WarpPool pool;
  bool active = false;
  uint64_t i = 0;
  double E0 = 0, E = 0, px = 0, py = 0, pz = 0, x = 0, y = 0, z = 0, mass = 0, pme = 0, dz = 0;
  int pid = 0, prim = 0;
  Rng rng;
  const double losses = T.t.dEdx_GeV_per_m;
  const float zmax = c.tally.z_max;

  for (;;) {
    __syncwarp();
    const bool need = !active;
    const int64_t got = pool_take(pool, c.ctr + 0, wave_n, need, chunk_p);
    const bool fresh = need && got >= 0;
    if (__all_sync(kFull, !active && !fresh)) break;
    bool finish = false;
    if (fresh) {
      i = (wave_head + (uint64_t)got) & c.mask;
      E0 = c.q.E[i]; px = c.q.px[i]; py = c.q.py[i]; pz = c.q.pz[i];
      x = c.q.x[i]; y = c.q.y[i]; z = c.q.z[i];
      mass = c.q.mass[i]; pid = c.q.pid[i]; prim = c.q.prim[i];
      if (c.rows.capacity) row_start(c.rows, got, pid, E0, px, py, pz, mass, c.q.key[i]);
    }
    // a dead entry (pid 0, left by the sampler's slot pool) is consumed without work
    if (fresh && pid != 0) {
      rng.init(c.seed, c.q.key[i]);
      E = E0;
      pme = fmax(fmax(min_calc(T, pid), c.min_energy), mass);
      ++L.steps;
      const int sp = species_of(pid);
      ++L.species[sp];
      atomicAdd(&sh_hist[(0 * 4 + sp) * kHB + bin_of(log10f((float)E0), -2.f, 2.f)], 1u);
      const float th = atan2f(sqrtf((float)px * (float)px + (float)py * (float)py), (float)pz);
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
      }
    }
    if (active) {
      // one iteration of the substep loop (shower.py:559-581)
      bool stop;
      {
        stop = !(E >= pme);
        if (!stop) {
          ++L.substeps;
          const double mfp = mfp_of(T, pid, E);
          const double u_hard = rng.u();
          dz = (S(mfp) / (S(6.0) + S(14.0) * S(rng.u()))).v;
          if (u_hard > exp(-dz / mfp)) {
            stop = true;
          } else {
            double pf[4] = {E, px, py, pz}, rf[3] = {x, y, z};
            lose_energy(pf, mass, (S(losses) * S(dz)).v);
            move_along(pf, rf, dz);
            if (c.ms) mcs_apply(BETHE, pf, (S(T.t.rho) * (S(dz) / S(kCmToM))).v, T.t, c.rescale,
                                table_mass(pid), rng);
            E = pf[0]; px = pf[1]; py = pf[2]; pz = pf[3]; x = rf[0]; y = rf[1]; z = rf[2];
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
          double pf[4] = {E, px, py, pz}, rf[3] = {x, y, z};
          lose_energy(pf, mass, (S(losses) * S(last)).v);
          move_along(pf, rf, last);
          if (c.ms) mcs_apply(BETHE, pf, (S(T.t.rho) * (S(last) / S(kCmToM))).v, T.t, c.rescale, kMe, rng);
          E = pf[0]; px = pf[1]; py = pf[2]; pz = pf[3]; x = rf[0]; y = rf[1]; z = rf[2];
          active = false;
          finish = true;
        }
      }
    }
    // ---- end of propagation: tallies, process choice, task or retirement
    int process = -1;
    bool emit = false;
    double edep = 0.0;
    int row = 0;
    if (finish) {
      const int sp = species_of(pid);
      if (c.rows.capacity) row_end(c.rows, (int64_t)((i - wave_head) & c.mask), E, px, py, pz, x, y, z);
      atomicAdd(&sh_hist[(2 * 4 + sp) * kHB + bin_of((float)z, 0.f, zmax)], 1u);
      const double eloss = E0 - E;
      L.e_cont += eloss;
      process = choose_process_b(T, pid, E, rng);
      emit = process >= 0 && E > pme;
      if (emit) {
        row = T.t.map_base[process] + lu_key(T, process, E);
        edep = eloss;
      } else {
        ++L.ended;
        L.e_ended += E;
        edep = eloss + E;
      }
    }
    if (__any_sync(kFull, finish)) {
      primary_tally(c.tally, finish, prim, edep);
      const long long slot = park_slot(c, open, emit, process);
      if (slot >= 0) {                 // the post-propagation state, parked for the sampler
        Park<0>& r = c.park[slot];
        r.E = E; r.key = c.q.key[i]; r.row = row; r.draw = (uint32_t)rng.n; r.pid = pid; r.gen = c.q.gen[i];
        r.px = px; r.py = py; r.pz = pz; r.x = x; r.y = y; r.z = z; r.mass = mass; r.prim = prim; r.pad = 0;
      }
    }
  }
  park_rest(c, open);
  flush_tally(c.tally, L, sh_hist);
}

template <int BETHE>
__global__ void __launch_bounds__(kThreads) k_propagate_fp64(WaveCtx<0> c) {
  __shared__ PropShared64 sm;
  propagate_fp64_body<BETHE>(c, sm);
}

// ------------------------------------------------ phase 1, mixed precision
// A particle whose propagation ended, waiting for the process choice and its
// sampling task.  Finished particles are queued per warp and handled 32 at a
// time so this per-particle work runs with every lane busy.
// The float64 energy after propagation, E0 - loss clamped at the mass, is
// formed in run_finish, where every lane of the warp takes part: a float64
// instruction costs the narrow float64 pipe the same cycles whether one lane
// or thirty-two execute it.
struct FinEntry {
  uint32_t i, draw;
  int32_t pid, prim;
  double E0;
  uint64_t key;
  float loss;                               // continuous loss along the track (float32 sum)
  float px, py, pz, x, y, z, u, pme, th0;   // th0: polar angle of p0 (creation histogram)
  float mass;
  int32_t gen;
};

template <bool SH>
__device__ void run_finish(const WaveCtx<1>& c, const Ns32<SH>& ns, FinEntry* fq, int count, volatile int (*open)[2],
                           LocalTally& L, unsigned int* sh_hist) {
  const int lane = threadIdx.x & 31;
  const bool on = lane < count;
  int process = -1, prim = 0;
  bool emit = false;
  double edep = 0.0, Eout = 0.0;
  uint32_t i = 0;
  int row = 0;
  if (on) {
    const FinEntry& e = fq[lane];
    i = e.i;
    prim = e.prim;
    const bool moved = e.loss != 0.f;
    double E = moved ? e.E0 - (double)e.loss : e.E0;    // float64 energy bookkeeping
    if (moved && E <= (double)e.mass) E = (double)e.mass;
    const int sp = species_of(e.pid);
    atomicAdd(&sh_hist[(0 * 4 + sp) * kHB + bin_of(log10f((float)e.E0), -2.f, 2.f)], 1u);
    atomicAdd(&sh_hist[(1 * 4 + sp) * kHB + bin_of(e.th0 > 0.f ? log10f(e.th0) : -6.f, -6.f, 0.5f)], 1u);
    atomicAdd(&sh_hist[(2 * 4 + sp) * kHB + bin_of(e.z, 0.f, c.tally.z_max)], 1u);
    const double eloss = e.E0 - E;
    L.e_cont += eloss;
    if (c.rows.capacity)
      row_end(c.rows, (int64_t)((i - w_head(c)) & c.mask), E, e.px, e.py, e.pz, e.x, e.y, e.z);
    const float Ef = (float)E;
    process = choose32(ns, e.pid, Ef, e.u);             // shower.py:665-698
    emit = process >= 0 && Ef > e.pme;
    if (emit) {
      row = c.T.t.map_base[process] + lu_key32(c.T, process, Ef);
      edep = eloss;
    } else {
      ++L.ended;
      L.e_ended += E;
      edep = eloss + E;
    }
    Eout = E;
  }
  primary_tally(c.tally, on, prim, edep);
  const long long slot = park_slot(c, open, emit, process);
  if (slot >= 0) {                                       // the state parked for the sampler
    const FinEntry& e = fq[lane];
    Park<1>& r = c.park[slot];
    r.E = Eout; r.key = e.key; r.row = row; r.draw = e.draw; r.pid = e.pid; r.gen = e.gen;
    r.px = e.px; r.py = e.py; r.pz = e.pz; r.x = e.x; r.y = e.y; r.z = e.z; r.mass = e.mass; r.prim = e.prim;
  }
}

// BETHE: Shower(fast_MCS_mode=False); a separate instantiation keeps the
// Bethe-Moliere inverse CDF out of the fast mode's registers.
// NW: warps per block (the block size is a tuning choice of the float32 kernels).
template <int NW> struct PropSharedMixedT {
  unsigned int hist[kHist];
  int open[NW][8][2];             // each warp's open task chunk per process: id, fill
  FinEntry fin[NW][64];
  NsHdr hdr[PT_N_NSIGMA];
};
using PropSharedMixed = PropSharedMixedT<kWarps>;

template <int BETHE, bool SH, int NW>
__device__ __forceinline__ void propagate_mixed_body(const WaveCtx<1>& c, PropSharedMixedT<NW>& sm, Ns32<SH> ns) {
  unsigned int* sh_hist = sm.hist;
  FinEntry (*sh_fin)[64] = sm.fin;
  const int64_t wave_n = w_n(c);
  const int chunk_p = wave_chunk_propagate(c.chunk[0], wave_n);
  const uint64_t wave_head = w_head(c);
  const Tabs& T = c.T;
  for (int k = threadIdx.x; k < kHist; k += blockDim.x) sh_hist[k] = 0;
  if (threadIdx.x < NW * 8) {
    sm.open[threadIdx.x / 8][threadIdx.x % 8][0] = -1;
    sm.open[threadIdx.x / 8][threadIdx.x % 8][1] = 0;
  }
  fill_ns_hdr(T, sm.hdr);
  __syncthreads();
  ns.h = sm.hdr;
  const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
  FinEntry* fq = sh_fin[w];
  volatile int (*open)[2] = sm.open[w];
  int fcount = 0;                                        // warp-uniform
  const float mc0 = c.k32.mc[0], mc1 = c.k32.mc[1], mc2 = c.k32.mc[2], mc3 = c.k32.mc[3];
  const float minE = c.k32.min_energy;
  const float lossesf = c.k32.dedx;
  const float rho_cm = c.k32.rho_cm, A = c.k32.A, Z = c.k32.Z, Z23 = c.k32.Z23;
  const float Z13 = c.k32.Z13;
  const Ld32 ld = c.k32.ld;
  const float rescale = c.k32.rescale;
  const float me = (float)kMe;
  LocalTally L;
  WarpPool pool;
  bool active = false;
  uint32_t i = 0;
  double E0 = 0.0;
  float E0f = 0.f;                // (float)E0, converted once per particle
  float Ef = 0.f, mf = 0.f, pmef = 0.f, lossf = 0.f, dzf = 0.f, pmag = 0.f, th0 = 0.f, mtab = 0.f;
  float3 dir = make_float3(0.f, 0.f, 1.f), pos = make_float3(0.f, 0.f, 0.f), disp = make_float3(0.f, 0.f, 0.f);
  int pid = 0, prim = 0;
  Rng rng;
  float uc = 0.f;                 // the process-choice draw, already taken with the last step
  bool have_uc = false;

  for (;;) {
    __syncwarp();
    // a lane that is done waits until enough lanes are idle, so the refill's
    // loads and set-up run for several lanes at once
    const unsigned idle = __ballot_sync(kFull, !active);
    const bool need = !active && (__popc(idle) >= c.refill_min[0] || idle == kFull);
    const int64_t got = pool_take(pool, c.ctr + 0, wave_n, need, chunk_p);
    const bool fresh = need && got >= 0;
    if (__all_sync(kFull, !active && !fresh)) break;
    bool fin = false;
    if (fresh) {
      i = (uint32_t)((wave_head + (uint64_t)got) & c.mask);
      pid = c.q.pid[i];
      if (c.rows.capacity)
        row_start(c.rows, got, pid, c.q.E[i], c.q.px[i], c.q.py[i], c.q.pz[i], c.q.mass[i], c.q.key[i]);
    }
    // a dead entry (pid 0, left by the sampler's slot pool) is consumed without work
    if (fresh && pid != 0) {
      E0 = c.q.E[i];
      const float px = c.q.px[i], py = c.q.py[i], pz = c.q.pz[i];
      pos = make_float3(c.q.x[i], c.q.y[i], c.q.z[i]);
      mf = c.q.mass[i];
      prim = c.q.prim[i];
      rng.init(c.seed, c.q.key[i]);
      E0f = c.q.E32[i];
      Ef = E0f;
      const int sp = species_of(pid);
      const float mcs = sp == 0 ? mc0 : (sp == 1 ? mc1 : (sp == 2 ? mc2 : mc3));
      pmef = fmaxf(fmaxf(mcs, minE), mf);                // shower.py:532-533
      mtab = sp == 0 ? 0.f : (sp == 3 ? (float)kMmu : me);   // mass_dict[PID] (particle.py:4-13)
      ++L.steps;
      ++L.species[sp];
      // rounded explicitly: the angle tally must not depend on how the
      // compiler contracts this in each kernel that inlines the body
      const float pt = sqrtf(__fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py)));
      pmag = sqrtf(__fadd_rn(__fmul_rn(pt, pt), __fmul_rn(pz, pz)));
      th0 = atan2f(pt, pz);
      const float ip = __fdividef(1.f, pmag);           // |p| below 2^126; unused at rest
      dir = pmag > 0.f ? make_float3(px * ip, py * ip, pz * ip) : make_float3(0.f, 0.f, 1.f);
      disp = make_float3(0.f, 0.f, 0.f);
      lossf = 0.f;
      dzf = 0.f;
      if (Ef < pmef) fin = true;                         // ends without moving (shower.py:534-536)
      else active = true;
    }
    if (active) {
      // One step of propagate_particle (shower.py:538-598), the same body for
      // every lane: a photon's flight, a charged substep, or the charged
      // particle's final partial increment; only the step length differs.
      float step, mlep = mtab;
      bool last = true;
      const bool charged = pid != 22;
      // Every draw this step can take, in stream order, from four Philox
      // blocks for all lanes: a photon's flight and its process choice; a
      // substep's two draws, then the final increment's draw when the hard
      // scatter ends it, the four of multiple scattering and the choice.
      Rng::Drawn<8> dr;
      rng.peek(dr, c.rk);
      int base = 1;                                       // first multiple-scattering draw
      // One mean free path and one logarithm per lane, however the warp's
      // lanes branch: a photon's flight is mfp log(1/(1-u)) and a hard
      // scatter's final increment -mfp log(1 + (e^(-1/q) - 1) u).
      const float mfp = mfp32(ns, pid, Ef);
      float lx = -dr.u[0];
      bool flight = !charged;
      if (charged && !(Ef >= pmef)) {
        step = dr.u[0] * dzf;                             // shower.py:584-585
        mlep = me;                                        // shower.py:596-598: electron mass
      } else if (charged) {
        ++L.substeps;
        const float u_hard = dr.u[0];
        const float q = fmaf(14.f, dr.u[1], 6.f);         // delta_z = mfp / U(6, 20)
        const float iq = __fdividef(-1.f, q);            // q in [6, 20]
        dzf = -mfp * iq;
        if (u_hard > __expf(iq)) {                       // hard scatter: final increment
          lx = expm1f(iq) * dr.u[2];
          flight = true;
          mlep = me;
          base = 3;
        } else {
          step = dzf;
          last = false;
          base = 2;
        }
      }
      if (flight) step = -mfp * log1pf(lx);
      if (charged) {                                      // lose_energy (particle.py:143-153)
        lossf = fmaf(lossesf, step, lossf);
        Ef = E0f - lossf;
        if (Ef <= mf) Ef = mf;
        pmag = sqrtf((Ef - mf) * (Ef + mf));
      }
      if (pmag > 0.f) {
        disp.x = fmaf(dir.x, step, disp.x); disp.y = fmaf(dir.y, step, disp.y); disp.z = fmaf(dir.z, step, disp.z);
      }
      // Lynch-Dahl momentum p = m_lepton * beta * gamma = |p| m_lepton / m;
      // a particle at rest draws nothing (moliere.py:359-363)
      const bool scat = charged && c.ms && pmag > 0.f;
      int used = 0;
      if (scat) {
        if constexpr (BETHE) {
          // the electron's momentum throughout (moliere.py:237,244)
          used = mcs32_bethe(dir, pmag * (me / mf), pmag / Ef, rho_cm * step, A, Z, Z13, Z23, rescale,
                             pick_in<1, 3>(dr.u, base), pick_in<2, 4>(dr.u, base + 1), pick_in<3, 5>(dr.u, base + 2),
                             pick_in<4, 6>(dr.u, base + 3));
        } else {
          mcs32_ld(dir, pmag, Ef, mf, mlep, rho_cm * step, ld, rescale, pick_in<1, 3>(dr.u, base),
                   pick_in<3, 5>(dr.u, base + 2), pick_in<4, 6>(dr.u, base + 3));
          used = 4;
        }
      }
      const int after = base + used;
      if (last) uc = pick_in<1, 7>(dr.u, after);         // the process-choice draw
      rng.advance(dr, after + (last ? 1 : 0));
      have_uc = last;
      if (last) {
        active = false;
        fin = true;
      }
    }
    const unsigned fm = __ballot_sync(kFull, fin);
    if (fm) {
      if (fin) {
        FinEntry e;
        e.i = i;
        e.pid = pid;
        e.prim = prim;
        e.gen = c.q.gen[i];
        e.key = (uint64_t)rng.k0 | ((uint64_t)rng.k1 << 32);
        e.mass = mf;
        e.loss = lossf;
        e.E0 = E0;
        e.px = pmag * dir.x; e.py = pmag * dir.y; e.pz = pmag * dir.z;
        e.x = pos.x + disp.x; e.y = pos.y + disp.y; e.z = pos.z + disp.z;
        e.u = have_uc ? uc : rng.uf(c.rk);               // the process-choice draw
        have_uc = false;
        e.draw = (uint32_t)rng.n;
        e.pme = pmef;
        e.th0 = th0;
        fq[fcount + __popc(fm & lanemask_lt())] = e;
      }
      fcount += __popc(fm);
      __syncwarp();
      if (fcount >= 32) {
        run_finish(c, ns, fq, 32, open, L, sh_hist);
        __syncwarp();
        const int rest = fcount - 32;
        FinEntry carry;
        if (lane < rest) carry = fq[32 + lane];
        __syncwarp();
        if (lane < rest) fq[lane] = carry;
        fcount = rest;
        __syncwarp();
      }
    }
  }
  if (fcount > 0) run_finish(c, ns, fq, fcount, open, L, sh_hist);
  park_rest(c, open);
  flush_tally(c.tally, L, sh_hist);
}

// Entries of the float32 n*sigma tables (all slots, one after another).
__device__ __forceinline__ int ns_total(const Tabs& T) {
  int n = 0;
#pragma unroll
  for (int s = 0; s < PT_N_NSIGMA; ++s) n = max(n, T.t.ns_base[s] + T.t.ns_len[s]);
  return n;
}

// PT_STAGE_SHARED: the block copies the float32 n*sigma tables (nodes,
// values, slopes; each array padded to 16 bytes in shared memory) into its
// shared memory with three TMA bulk copies (cp.async.bulk) that complete on
// one mbarrier; the last total % 4 entries of each array, under 16 bytes,
// are plain loads.  The host selects this only when the sources are 16-byte
// aligned.  Bounded: copies that have not landed after kStageNs record
// PT_TIMEOUT, the block waits once more with the same bound for its copies
// in flight and returns false.
constexpr unsigned long long kStageNs = 1000ull * 1000ull * 1000ull;

__device__ bool stage_ns_tables(const WaveCtx<1>& c, float* sh, int total, int pad) {
  __shared__ __align__(8) unsigned long long bar;
  const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
  const float* src[3] = {c.T.t.ns_x32, c.T.t.ns_y32, c.T.t.ns_s32};
  const int bulk = total & ~3;
  const uint32_t bytes = (uint32_t)bulk * 4u;
  if (threadIdx.x == 0) {
    mbar_init(b);
    mbar_arrive_expect(b, 3u * bytes);
    if (bytes)
      for (int a = 0; a < 3; ++a) bulk_g2s(sh + a * pad, src[a], bytes, b);
  }
  const int rest = total - bulk;
  if (threadIdx.x < 3 * rest) {
    const int a = threadIdx.x / rest, k = bulk + threadIdx.x % rest;
    sh[a * pad + k] = __ldg(src[a] + k);
  }
  __syncthreads();                                       // the barrier is initialised before any wait
  const bool landed = __syncthreads_and(mbar_wait(b, 0, kStageNs));
  if (!landed) {
    // process -2: a copy may still be in flight into this block's shared
    // memory, so the host treats the handle's later results as suspect
    if (threadIdx.x == 0) {
      raise_status(c.status, c.err_info, PT_TIMEOUT, -2, 0.0, 0);
      mbar_wait(b, 0, kStageNs);
    }
    __syncthreads();
  }
  return landed;
}

// 96 registers at 2 and 4 warps per block (20 warps per SM), 128 at 8.
template <int NW> constexpr int min_blocks32() { return 20 / NW; }

template <int BETHE, bool STAGE, int NW>
__global__ void __launch_bounds__(NW * 32, min_blocks32<NW>()) k_propagate_mixed(WaveCtx<1> c) {
  __shared__ PropSharedMixedT<NW> sm;
  if constexpr (STAGE) {
    extern __shared__ __align__(16) float ns_sh[];
    const int total = ns_total(c.T), pad = (total + 3) & ~3;
    if (!stage_ns_tables(c, ns_sh, total, pad)) return;
    propagate_mixed_body<BETHE, true>(c, sm, Ns32<true>{ns_sh, ns_sh + pad, ns_sh + 2 * pad, nullptr});
  } else {
    propagate_mixed_body<BETHE, false>(c, sm, ns_global(c.T));
  }
}

// ------------------------------------------------------------ phase 2
template <class R> struct DaughterT { double E; R px, py, pz; int pid; };

// Mixed engine: daughters in the parent frame with float32 angles, float32
// momentum magnitudes and the energy split closed in float64
// (E_a + E_b = E_in + target mass for the two-body processes).
struct KinOut { double E[2]; float P[2]; float3 d[2]; int pid[2]; };

// One reciprocal square root for |p| and the unit direction; a momentum
// below 2^-50 GeV keeps the z axis.
__device__ __forceinline__ void set_dir32(KinOut& k, int j, float pxx, float pyy, float pzz) {
  const float p2 = pxx * pxx + pyy * pyy + pzz * pzz;
  if (p2 > 0x1p-100f) {
    const float r = rsqrtf(p2);
    k.P[j] = p2 * r;
    k.d[j] = make_float3(pxx * r, pyy * r, pzz * r);
  } else {
    k.P[j] = sqrtf(p2);
    k.d[j] = make_float3(0.f, 0.f, 1.f);
  }
}

__device__ void kin_mixed(int process, int pid, double E, double mass, const MapPt32* x, float ph, KinOut& k) {
  float sph, cph;
  sincosf(ph, &sph, &cph);
  const float me = (float)kMe;
  switch (process) {
    case PT_BREM: case PT_MUONBREM: {        // kinematics.py:10-41
      const float Ef = (float)E, mf = (float)mass;
      const float w = fmaf(x[0].x, (float)(E - mass - 0.001), 0.001f);
      const double epp = E - (double)w;        // energy closes in float64
      const float eppf = (float)epp;
      float st, ct, stp, ctp, sp, cp;
      sincosf(0.5f * (x[1].x + x[2].x), &st, &ct);
      sincosf((x[1].x - x[2].x) * Ef / (2.f * eppf), &stp, &ctp);
      st = fabsf(st); stp = fabsf(stp);        // the reference takes sqrt(1 - cos^2)
      sincospif(2.f * (x[3].x - 0.5f), &sp, &cp);
      const float sal = sph, cal = cph;        // azimuth 'al' of kinematics.py:33
      k.E[1] = (double)w; k.P[1] = w; k.pid[1] = 22;
      k.d[1] = make_float3(cal * st, sal * st, ct);
      k.E[0] = epp; k.pid[0] = pid;
      k.P[0] = sqrtf((eppf - mf) * (eppf + mf));
      const float3 v = make_float3(sal * sp * stp + cal * (ctp * st - cp * ct * stp),
                                   ctp * sal * st - (cp * ct * sal + cal * sp) * stp, ct * ctp + cp * st * stp);
      const float inv = rsqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
      k.d[0] = make_float3(v.x * inv, v.y * inv, v.z * inv);
      break;
    }
    case PT_PAIRPROD: {                       // kinematics.py:70-102
      const float wf = (float)E, span = (float)(E - 2 * kMe);
      const float eppf = fmaf(x[0].x, span, me);
      const double epm = E - (double)eppf;     // energy closes in float64
      const float epmf = (float)epm;
      float stp, ctp, stm, ctm, s2, c2;
      sincosf(wf * (x[1].x + x[2].x) / (2.f * eppf), &stp, &ctp);
      sincosf(wf * (x[1].x - x[2].x) / (2.f * epmf), &stm, &ctm);
      stp = fabsf(stp); stm = fabsf(stm);
      sincosf(2.f * (float)kPi * x[3].x + ph, &s2, &c2);
      k.E[0] = (double)eppf; k.P[0] = sqrtf((eppf - me) * (eppf + me)); k.pid[0] = -11;
      k.d[0] = make_float3(stp * cph, stp * sph, ctp);
      k.E[1] = epm; k.P[1] = sqrtf((epmf - me) * (epmf + me)); k.pid[1] = 11;
      k.d[1] = make_float3(stm * c2, stm * s2, ctm);
      break;
    }
    case PT_COMP: {                           // kinematics.py:104-132, mV = 0
      const float Eg = (float)E, s = me * me + 2.f * Eg * me, rs = sqrtf(s);
      const float Ee = (s + me * me) / (2.f * rs), EV = (s - me * me) / (2.f * rs), pF = EV;
      const float g0 = Ee / me, sq = sqrtf((g0 - 1.f) * (g0 + 1.f)), b0 = sq / g0;
      const float omb = 1.f / (g0 * (g0 + sq));                 // 1 - b0
      const float pT = pF * sqrtf(x[0].omx * x[0].opx);
      const float Eph = g0 * EV * fmaf(b0, x[0].omx, omb);      // g0 (EV - b0 pF c)
      k.E[1] = (double)Eph; k.pid[1] = 22;
      set_dir32(k, 1, pT * sph, pT * cph, g0 * EV * (x[0].omx - omb));
      k.E[0] = (E + kMe) - (double)Eph; k.pid[0] = 11;          // E_e + E_V = E_gamma + m_e
      set_dir32(k, 0, -pT * sph, -pT * cph, b0 * g0 * Ee + g0 * pF * x[0].x);
      break;
    }
    case PT_ANN: {                            // kinematics.py:301-334, mV = 0
      const float s = 2.f * me * ((float)E + me), Eg = 0.5f * sqrtf(s);
      const float g0 = Eg / me, sq = sqrtf((g0 - 1.f) * (g0 + 1.f)), b0 = sq / g0;
      const float omb = 1.f / (g0 * (g0 + sq));
      const float pT = Eg * sqrtf(x[0].omx * x[0].opx);
      const float E1 = g0 * Eg * fmaf(b0, x[0].omx, omb);
      k.E[0] = (double)E1; k.pid[0] = 22;
      set_dir32(k, 0, -pT * sph, -pT * cph, g0 * Eg * (x[0].omx - omb));
      k.E[1] = (E + kMe) - (double)E1; k.pid[1] = 22;
      set_dir32(k, 1, pT * sph, pT * cph, g0 * Eg * (b0 + x[0].x));
      break;
    }
    case PT_MOLLER: case PT_BHABHA: {         // kinematics.py:213-237 (b0 = pF/Ee0)
      const float s = 2.f * me * me + 2.f * (float)E * me, Ee0 = 0.5f * sqrtf(s);
      const float pF = sqrtf((Ee0 - me) * (Ee0 + me)), g0 = Ee0 / me;
      const float pT = pF * sqrtf(x[0].omx * x[0].opx);
      const float Eb = g0 * fmaf(pF * pF, x[0].omx, me * me) / Ee0;   // g0 (Ee0 - b0 pF c)
      k.E[1] = (double)Eb; k.pid[1] = 11;
      set_dir32(k, 1, pT * sph, pT * cph, g0 * pF * x[0].omx);
      k.E[0] = (E + kMe) - (double)Eb; k.pid[0] = pid;
      set_dir32(k, 0, -pT * sph, -pT * cph, g0 * pF * x[0].opx);
      break;
    }
    default: {                                // kinematics.py:239-265 (b0 = pe/Ee0)
      const float mm = (float)kMmu, s = me * me + mm * mm + 2.f * (float)E * me, rs = sqrtf(s);
      const float Ee0 = (s + me * me - mm * mm) / (2.f * rs), Em0 = (s + mm * mm - me * me) / (2.f * rs);
      const float pe = sqrtf((Ee0 - me) * (Ee0 + me)), pm = sqrtf((Em0 - mm) * (Em0 + mm));
      const float g0 = Ee0 / me, b0 = pe / Ee0;
      const float st = sqrtf(x[0].omx * x[0].opx);
      const float Eel = g0 * fmaf(pe * pe, x[0].omx, me * me) / Ee0;  // g0 (Ee0 - b0 pe c)
      k.E[1] = (double)Eel; k.pid[1] = 11;
      set_dir32(k, 1, -pe * st * sph, -pe * st * cph, g0 * pe * x[0].omx);
      k.E[0] = (E + kMe) - (double)Eel; k.pid[0] = pid;
      set_dir32(k, 0, pm * st * sph, pm * st * cph, b0 * g0 * Em0 + g0 * pm * x[0].x);
      break;
    }
  }
}

// An accepted proposal waiting for its final-state kinematics.
template <int PREC> struct KinEntry;
template <> struct KinEntry<0> { uint32_t i; int32_t process; double x[4]; double ph; };
template <> struct KinEntry<1> { uint32_t i; int32_t process; MapPt32 x[4]; float ph; };
constexpr int kKinQ = 64;

// Kinematics, lab rotation and daughter output for up to 32 queued accepts,
// one per lane (sample_scattering, shower.py:467-507).  All lanes call.
template <int PREC>
__device__ void run_kinematics(const WaveCtx<PREC>& c, KinEntry<PREC>* kq, int count, OutPool& opool, LocalTally& L) {
  using R = typename RingT<PREC>::R;
  const int lane = threadIdx.x & 31;
  const bool on = lane < count;
  DaughterT<R> dg[2];
  int want = 0, prim = 0, gen = 0;
  uint64_t key = 0, i = 0;
  R x0 = 0, y0 = 0, z0 = 0;
  double below = 0.0;
  if (on) {
    const KinEntry<PREC>& e = kq[lane];
    i = e.i;
    const int process = e.process;
    const Park<PREC>& P = c.park[i];                     // the parent's task record
    const double E = P.E;
    const int pid = P.pid;
    if constexpr (PREC == 0) {
      const double mass = P.mass;
      const double pf[4] = {E, P.px, P.py, P.pz};
      const double* xd = reinterpret_cast<const KinEntry<0>&>(e).x;
      const double ph = reinterpret_cast<const KinEntry<0>&>(e).ph;
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
      const KinEntry<1>& f = reinterpret_cast<const KinEntry<1>&>(e);
      KinOut k;
      kin_mixed(process, pid, E, P.mass, f.x, f.ph, k);
      const Rot32 Rm = rot32_from_momentum(P.px, P.py, P.pz);
      for (int j = 0; j < 2; ++j) {
        const float3 v = rot32_apply(Rm, k.d[j]);
        dg[j] = {k.E[j], k.P[j] * v.x, k.P[j] * v.y, k.P[j] * v.z, k.pid[j]};
      }
    }
    want = (dg[0].E > c.min_energy) + (dg[1].E > c.min_energy);
    for (int j = 0; j < 2; ++j)
      if (!(dg[j].E > c.min_energy)) { ++L.below; L.e_below += dg[j].E; below += dg[j].E; }
    prim = P.prim;
    key = P.key;
    gen = P.gen;
    x0 = P.x; y0 = P.y; z0 = P.z;
    if (below != 0.0) atomicAdd(c.tally.prim_edep + prim, below);
  }
  uint64_t slots[2] = {0, 0};
  out_take(opool, c.ctr + 2, want, slots, w_out_chunk(c));
  int slot = 0;
  for (int j = 0; j < 2; ++j) {
    if (!on || !(dg[j].E > c.min_energy)) continue;
    const uint64_t q = (w_tail(c) + slots[slot++]) & c.mask;
    ++L.pushed;
    c.q.E[q] = dg[j].E; c.q.px[q] = dg[j].px; c.q.py[q] = dg[j].py; c.q.pz[q] = dg[j].pz;
    if (PREC == 1) c.q.E32[q] = (float)dg[j].E;
    c.q.x[q] = x0; c.q.y[q] = y0; c.q.z[q] = z0;
    c.q.mass[q] = (R)table_mass(dg[j].pid);
    c.q.key[q] = daughter_key(key, j);
    c.q.pid[q] = dg[j].pid;
    c.q.prim[q] = prim;
    c.q.gen[q] = gen + 1;
  }
}

// A task of the cooperative finish: its index, process, proposals made and
// next draw.
struct CoopTask {
  uint64_t i;
  int64_t props;
  uint64_t n;
  int32_t process;
};

template <int PREC, int NW = kWarps> struct SampShared {
  unsigned long long off[9];
  KinEntry<PREC> kq[NW][kKinQ];
  CoopTask cq[NW][32];
};

// One task's sampling state, as a lane holds it.
template <int PREC> struct SampTask {
  int process = 0, d = 1, row = 0;
  uint64_t i = 0;
  int64_t props = 0, cap = 0;
  double E = 0, maxF = 0, neval = 1;
  Rng rng;
  Samp32 S32;
  const float4* g32[4] = {nullptr, nullptr, nullptr, nullptr};
  const double* g64[4] = {nullptr, nullptr, nullptr, nullptr};
  int ninc[4] = {1, 1, 1, 1};
};

// Loads task i of `process` (its parked record) and positions its stream at
// draw n.
template <int PREC>
__device__ __forceinline__ void samp_load(const WaveCtx<PREC>& c, SampTask<PREC>& k, uint64_t i, int process,
                                          uint64_t n) {
  const Tabs& T = c.T;
  k.i = i;
  k.process = process;
  k.E = c.park[i].E;
  k.row = c.park[i].row;
  k.rng.init(c.seed, c.park[i].key);
  k.rng.seek(n);
  k.neval = T.t.map_neval[k.row];
  k.d = process_dim(process);
  k.cap = c.max_n_integrators * (int64_t)k.neval;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    if (m < k.d) {
      const int64_t off = T.t.grid_offset[(int64_t)k.row * 4 + m];
      k.ninc[m] = T.t.grid_ninc[(int64_t)k.row * 4 + m];
      if (PREC == 0) k.g64[m] = T.t.grid_nodes + off;
      else k.g32[m] = reinterpret_cast<const float4*>(T.t.grid_f32x4) + off;
    }
  }
  if (PREC == 0) {
    k.maxF = T.t.map_maxF[k.row];
  } else {
    const float Ef = (float)k.E, Cr = __ldg(T.t.map_cnorm32 + k.row), a0sq = c.k32.a0sq;
    switch (process) {
      case PT_BREM: brem32_setup(k.S32, Ef, (float)kMe, c.k32.Eg_min, a0sq, Cr); break;
      case PT_MUONBREM: brem32_setup(k.S32, Ef, (float)kMmu, c.k32.Eg_min, a0sq, Cr); break;
      case PT_PAIRPROD: pair32_setup(k.S32, Ef, a0sq, Cr); break;
      case PT_COMP: comp32_setup(k.S32, Ef, Cr); break;
      case PT_ANN: ann32_setup(k.S32, Ef, c.k32.Eg_min, Cr); break;
      case PT_MOLLER: moller32_setup(k.S32, Ef, c.k32.Ee_min, Cr); break;
      case PT_BHABHA: bhabha32_setup(k.S32, Ef, c.k32.Ee_min, Cr); break;
      default: muone32_setup(k.S32, Ef, c.k32.Ee_min, Cr); break;
    }
  }
}

// One proposal (d uniforms for y, then the accept uniform; on acceptance
// the azimuth draw): true when accepted, with the sample in ent.
template <int PREC>
__device__ __forceinline__ bool samp_propose(const WaveCtx<PREC>& c, SampTask<PREC>& k, KinEntry<PREC>& ent) {
  bool accept;
  if constexpr (PREC == 0) {
    double* xd = reinterpret_cast<KinEntry<0>&>(ent).x;
    double jac = 1.0;
#pragma unroll
    for (int m = 0; m < 4; ++m)
      if (m < k.d) xd[m] = map_dim(k.g64[m], k.ninc[m], k.rng.u(), jac);
    const double f = dsigma_any(c.T, k.process, xd, k.E);
    accept = k.maxF * k.rng.u() < (jac / k.neval) * f;
    if (accept) reinterpret_cast<KinEntry<0>&>(ent).ph = 2.0 * kPi * k.rng.u();
  } else {
    MapPt32* xm = reinterpret_cast<KinEntry<1>&>(ent).x;
    float jac = 1.f;
    float ua;                      // the accept draw
    if (k.d == 4) {                // four y draws and the accept draw in three Philox blocks
      float u5[5];
      k.rng.take(u5, c.rk);
#pragma unroll
      for (int m = 0; m < 4; ++m) xm[m] = map_dim32(k.g32[m], k.ninc[m], u5[m], jac);
      ua = u5[4];
    } else {
      float u2[2];
      k.rng.take(u2, c.rk);
      xm[0] = map_dim32(k.g32[0], k.ninc[0], u2[0], jac);
      ua = u2[1];
    }
    float r;
    switch (k.process) {
      case PT_BREM: case PT_MUONBREM: r = brem32_ratio(k.S32, xm, jac); break;
      case PT_PAIRPROD: r = pair32_ratio(k.S32, xm, jac); break;
      case PT_COMP: r = comp32_ratio(k.S32, xm[0], jac); break;
      case PT_ANN: r = ann32_ratio(k.S32, xm[0], jac); break;
      case PT_MOLLER: r = moller32_ratio(k.S32, xm[0], jac); break;
      case PT_BHABHA: r = bhabha32_ratio(k.S32, xm[0], jac); break;
      default: r = muone32_ratio(k.S32, xm[0], jac); break;
    }
    accept = ua < r;
    if (accept) reinterpret_cast<KinEntry<1>&>(ent).ph = 2.f * (float)kPi * k.rng.uf(c.rk);
  }
  return accept;
}

// Queues one ballot's accepted proposals and runs their kinematics 32 at a
// time with all lanes.
template <int PREC>
__device__ __forceinline__ void samp_queue(const WaveCtx<PREC>& c, KinEntry<PREC>* kq, int& kcount, unsigned am,
                                           bool accept, const KinEntry<PREC>& ent, OutPool& opool, LocalTally& L) {
  const int lane = threadIdx.x & 31;
  if (!am) return;
  if (accept) kq[kcount + __popc(am & lanemask_lt())] = ent;
  kcount += __popc(am);
  __syncwarp();
  if (kcount >= 32) {
    run_kinematics<PREC>(c, kq, 32, opool, L);
    __syncwarp();
    KinEntry<PREC> carry;
    const int rest = kcount - 32;
    if (lane < rest) carry = kq[32 + lane];
    __syncwarp();
    if (lane < rest) kq[lane] = carry;
    kcount = rest;
    __syncwarp();
  }
}

// The cooperative finish of a warp's open tasks, once the pool is empty for
// the rest of the wave: one task at a time, lane l makes proposal p + l of
// it from draw n0 + l (d + 1) of its stream (every proposal takes d map
// draws and one accept draw), and the first accepted proposal in proposal
// order is the task's sample -- the sequential loop's sample, with its
// proposal count, later draws and PT_NO_SAMPLE cap, found up to 32 times
// sooner.  A wave ends on a few tasks with thousands of proposals (a
// muon's mu-e scattering at some energies), which the lanes' own loops run
// one lane each.  Not inlined: its registers are its own, so the main
// loop's allocation stays as it was.
template <int PREC>
__device__ __noinline__ void samp_coop_finish(const WaveCtx<PREC>& c, CoopTask* cq, int n_open, KinEntry<PREC>* kq,
                                              int& kcount, OutPool& opool, LocalTally& L) {
  const int lane = threadIdx.x & 31;
  SampTask<PREC> k;
  for (int h = 0; h < n_open;) {
    const CoopTask q = cq[h];
    samp_load(c, k, q.i, q.process, q.n + (uint64_t)lane * (uint64_t)(process_dim(q.process) + 1));
    KinEntry<PREC> ent;
    const bool mine = q.props + lane < k.cap;
    bool accept = mine && samp_propose(c, k, ent);
    const unsigned am = __ballot_sync(kFull, accept);
    const int w = am ? __ffs(am) - 1 : 32;
    accept = accept && lane == w;
    bool done = w < 32;
    if (lane == 0) {
      L.props += (unsigned long long)(w < 32 ? (int64_t)w + 1 : (k.cap - q.props < 32 ? k.cap - q.props : 32));
      if (w < 32) {
        ++L.sampled;
      } else if (q.props + 32 >= k.cap) {
        raise_status(c.status, c.err_info, PT_NO_SAMPLE, q.process, k.E, k.row - c.T.t.map_base[q.process]);
      } else {
        cq[h].props = q.props + 32;
        cq[h].n = q.n + (uint64_t)32 * (uint64_t)(k.d + 1);
      }
    }
    done = done || q.props + 32 >= k.cap;
    __syncwarp();
    if (accept) {
      ent.i = (uint32_t)q.i;
      ent.process = q.process;
    }
    samp_queue(c, kq, kcount, am ? (1u << w) : 0u, accept, ent, opool, L);
    if (done) ++h;
  }
}

template <int PREC, int NW>
__device__ __forceinline__ void sample_body(const WaveCtx<PREC>& c, SampShared<PREC, NW>& sm) {
  unsigned long long* sh_off = sm.off;
  KinEntry<PREC> (*sh_kq)[kKinQ] = sm.kq;
  if (threadIdx.x == 0) {
    unsigned long long acc = 0;            // task index space: 32 per published chunk, process by process
    for (int p = 0; p < 8; ++p) { sh_off[p] = acc; acc += (unsigned long long)kChunkTasks * __ldcg(c.ctr + 8 + p); }
    sh_off[8] = acc;
  }
  __syncthreads();
  KinEntry<PREC>* kq = sh_kq[threadIdx.x / 32];
  int kcount = 0;                      // warp-uniform
  const int64_t total = (int64_t)sh_off[8];
  const int chunk_s = wave_chunk(c.chunk[1], total);
  const int lane = threadIdx.x & 31;
  LocalTally L;
  WarpPool pool;
  OutPool opool;
  bool active = false;
  int n_open = 0;                      // tasks handed to the cooperative finish
  SampTask<PREC> k;

  for (;;) {
    __syncwarp();
    const unsigned idle = __ballot_sync(kFull, !active);   // refills in groups, as in propagation
    const bool need = !active && (__popc(idle) >= c.refill_min[1] || idle == kFull);
    const int64_t t = pool_take(pool, c.ctr + 1, total, need, chunk_s);
    const bool fresh = need && t >= 0;
    const bool drained = __any_sync(kFull, need && t < 0);   // the pool is empty for the rest of the wave
    if (__all_sync(kFull, !active && !fresh)) break;
    int32_t chunk_ent = 0;
    int process = 0;
    if (fresh) {
      while (process < 7 && (unsigned long long)t >= sh_off[process + 1]) ++process;
      chunk_ent = c.chunks[(int64_t)process * c.chunk_cap + ((t - (int64_t)sh_off[process]) >> 5)];
    }
    // a slot past a partly filled chunk's tasks holds no task: the lane asks again
    if (fresh && (int)(t & 31) <= (chunk_ent & 31)) {
      const uint64_t i = ((uint64_t)((uint32_t)chunk_ent >> 5) << 5) + (uint64_t)(t & 31);
      samp_load(c, k, i, process, c.park[i].draw);
      k.props = 0;
      active = true;
    }
    bool accept = false;
    KinEntry<PREC> ent;
    if (active) {
      accept = samp_propose(c, k, ent);
      ++k.props;
      ++L.props;
      if (accept) {
        active = false;
        ++L.sampled;
      } else if (k.props >= k.cap) {
        raise_status(c.status, c.err_info, PT_NO_SAMPLE, k.process, k.E, k.row - c.T.t.map_base[k.process]);
        active = false;
      }
    }
    if (accept) {
      ent.i = (uint32_t)k.i;
      ent.process = k.process;
    }
    samp_queue(c, kq, kcount, __ballot_sync(kFull, accept), accept, ent, opool, L);
    if (drained) {
      // hand the warp's open tasks to the cooperative finish
      CoopTask* cq = sm.cq[threadIdx.x / 32];
      const unsigned open = __ballot_sync(kFull, active);
      if (active) cq[__popc(open & lanemask_lt())] = CoopTask{k.i, k.props, k.rng.n, k.process};
      n_open = __popc(open);
      __syncwarp();
      break;
    }
  }
  if (n_open > 0) samp_coop_finish<PREC>(c, sm.cq[threadIdx.x / 32], n_open, kq, kcount, opool, L);
  if (kcount > 0) run_kinematics<PREC>(c, kq, kcount, opool, L);
  // unused slots of the warp's last output chunk become dead entries
  const uint64_t wave_tail = w_tail(c);
  for (uint64_t r = opool.next + lane; r < opool.end; r += 32) c.q.pid[(wave_tail + r) & c.mask] = 0;
  flush_tally(c.tally, L, nullptr);
}

template <int PREC, int NW>
__global__ void __launch_bounds__(NW * 32, PREC == 1 ? min_blocks32<NW>() : 1) k_sample(WaveCtx<PREC> c) {
  __shared__ SampShared<PREC, NW> sm;
  sample_body<PREC>(c, sm);
}

template <int PREC>
__global__ void k_feed(RingT<PREC> q, uint64_t mask, uint64_t tail, const double* p0, const double* r0, const int32_t* pid,
                       const double* mass, int64_t n_total, int64_t first, int64_t n, int64_t offset) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t g = first + j;
  const uint64_t i = (tail + (uint64_t)j) & mask;
  q.E[i] = p0[0 * n_total + g]; q.px[i] = p0[1 * n_total + g]; q.py[i] = p0[2 * n_total + g];
  if (PREC == 1) q.E32[i] = (float)p0[0 * n_total + g];
  q.pz[i] = p0[3 * n_total + g];
  q.x[i] = r0[0 * n_total + g]; q.y[i] = r0[1 * n_total + g]; q.z[i] = r0[2 * n_total + g];
  q.mass[i] = mass[g]; q.pid[i] = pid[g]; q.prim[i] = (int32_t)g; q.gen[i] = 0;
  q.key[i] = primary_key((uint64_t)(offset + g));
}

// ----------------------------------------------- waves planned on the GPU
constexpr long long kMaxPlannedWaves = 1ll << 20;
// plan_step: what the host loop of run_batch_impl decides between waves,
// done by one thread from the device counters: retire the last wave (its
// entries are consumed, its daughters appended), feed primaries while the
// ring is less than 1/8 full, size the next wave, clear the counters.
template <int PREC>
__device__ void plan_step(const WaveCtx<PREC>& c) {
  WavePlan& P = *c.plan;
  P.head += (unsigned long long)P.n_in;
  P.tail += __ldcg(c.ctr + 2);
  P.n_in = 0;
  P.feed_m = 0;
  for (int k = 0; k < 16; ++k) c.ctr[k] = 0;
  if (*(volatile int*)c.status != 0) { P.done = 1; return; }
  if (P.waves >= c.max_waves) {                   // a bound on the loop, far above any run's need
    raise_status(c.status, c.err_info, PT_TIMEOUT, -1, 0.0, 0);
    P.done = 1;
    return;
  }
  const int64_t cap = c.cap;
  int64_t live = (int64_t)(P.tail - P.head);
  if (P.fed >= c.n_prim && live == 0) { P.done = 1; return; }
  if (P.fed < c.n_prim && live < cap / 8) {
    int64_t m = c.n_prim - P.fed;
    if (m > cap / 8 - live) m = cap / 8 - live;
    if (m > c.feed_max) m = c.feed_max;
    P.feed_m = m;
    P.feed_at = P.tail;
    P.tail += (unsigned long long)m;
    P.fed += m;
    live += m;
  }
  int oc = kOutChunk;
  int64_t k = (cap - live - c.slack) / 2;
  if (k > live) k = live;
  if (k > c.list_cap) k = c.list_cap;
  if (k < 16 * 1024) {
    oc = 0;
    k = (cap - live) / 2;
    if (k > live) k = live;
    if (k > c.list_cap) k = c.list_cap;
  }
  if (k <= 0) {                                   // the live population filled the ring
    raise_status(c.status, nullptr, PT_OOM, 0, 0.0, 0);
    P.done = 1;
    return;
  }
  P.n_in = k;
  P.out_chunk = oc;
  P.waves += 1;
}

// The planned wave's primaries into the ring (k_feed's rows), thread j of nthr.
template <int PREC>
__device__ __forceinline__ void feed_planned(const WaveCtx<PREC>& c, int64_t j, int64_t nthr) {
  const int64_t m = __ldcg(&c.plan->feed_m);
  const uint64_t at = (uint64_t)__ldcg(&c.plan->feed_at);
  const int64_t first = __ldcg(&c.plan->fed) - m;
  const int64_t n = c.n_prim;
  for (; j < m; j += nthr) {
    const int64_t g = first + j;
    const uint64_t i = (at + (uint64_t)j) & c.mask;
    c.q.E[i] = c.in_p0[0 * n + g]; c.q.px[i] = c.in_p0[1 * n + g]; c.q.py[i] = c.in_p0[2 * n + g];
    if (PREC == 1) c.q.E32[i] = (float)c.in_p0[0 * n + g];
    c.q.pz[i] = c.in_p0[3 * n + g];
    c.q.x[i] = c.in_r0[0 * n + g]; c.q.y[i] = c.in_r0[1 * n + g]; c.q.z[i] = c.in_r0[2 * n + g];
    c.q.mass[i] = c.in_mass[g]; c.q.pid[i] = c.in_pid[g]; c.q.prim[i] = (int32_t)g; c.q.gen[i] = 0;
    c.q.key[i] = primary_key((uint64_t)(c.prim_offset + g));
  }
}

// Graph-captured loop: the body's first node plans the wave and sets the
// loop's condition (0 once the run has ended; the rest of that last body
// then finds an empty wave).
template <int PREC>
__global__ void k_plan(WaveCtx<PREC> c, cudaGraphConditionalHandle loop) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    plan_step(c);
    cudaGraphSetConditional(loop, c.plan->done ? 0u : 1u);
  }
}

template <int PREC>
__global__ void k_feed_planned(WaveCtx<PREC> c) {
  feed_planned(c, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// Grid-wide barrier of the persistent kernel, whose blocks the cooperative
// launch makes co-resident: arrivals in bar[0], the generation in bar[1].
// Bounded: a block that waits longer than bound_ns (kBarrierNs unless
// pt_batch_tuning.barrier_ns sets it) records PT_TIMEOUT and returns false,
// and every block then leaves the kernel within the same bound.
constexpr unsigned long long kBarrierNs = 20ull * 1000ull * 1000ull * 1000ull;
__device__ bool grid_barrier(unsigned int* bar, int* status, double* err_info, unsigned long long bound_ns) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = bar + 1;
    const unsigned int g = *gen;
    __threadfence();
    int good = 1;
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      while (*gen == g) {
        if (global_ns() - t0 > bound_ns) { good = 0; break; }
        __nanosleep(200);
      }
    }
    __threadfence();
    if (!good) raise_status(status, err_info, PT_TIMEOUT, -1, 0.0, 0);
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

template <int PREC> struct PropSharedOf;
template <> struct PropSharedOf<0> { using T = PropShared64; };
template <> struct PropSharedOf<1> { using T = PropSharedMixed; };

// One persistent kernel for the whole run: each wave is plan, feed,
// propagation and sampling, separated by grid barriers; the warps pull
// their work from the same device pools as the separate kernels.
template <int PREC, int BETHE>
__global__ void __launch_bounds__(kThreads, PREC == 1 ? 5 : 1) k_persistent(WaveCtx<PREC> c, unsigned int* bar) {
  union Shared {
    typename PropSharedOf<PREC>::T p;
    SampShared<PREC> s;
  };
  __shared__ Shared sm;
  for (;;) {
    if (blockIdx.x == 0 && threadIdx.x == 0) plan_step(c);
    if (!grid_barrier(bar, c.status, c.err_info, c.barrier_ns)) break;
    if (__ldcg(&c.plan->done)) break;
    feed_planned(c, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
    if (!grid_barrier(bar, c.status, c.err_info, c.barrier_ns)) break;
    if constexpr (PREC == 1) propagate_mixed_body<BETHE, false>(c, sm.p, ns_global(c.T));
    else propagate_fp64_body<BETHE>(c, sm.p);
    if (!grid_barrier(bar, c.status, c.err_info, c.barrier_ns)) break;
    sample_body<PREC, kWarps>(c, sm.s);
    if (!grid_barrier(bar, c.status, c.err_info, c.barrier_ns)) break;
  }
}

}  // namespace

// ------------------------------------------------------------- host side
struct BatchScratch {
  int64_t cap = 0;          // ring capacity (power of two)
  int64_t list_cap = 0;     // largest wave (entries)
  int64_t chunk_cap = 0;    // task chunks per wave
  void* mem = nullptr;
  void* park = nullptr;     // chunk_cap * 32 task records (sized for the float64 record)
  int32_t* chunks = nullptr;
  unsigned long long* ctr = nullptr;
  unsigned long long* h_ctr = nullptr;
  int* h_status = nullptr;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};   // around each wave's two kernels
  WavePlan* plan = nullptr;       // device-planned waves
  unsigned int* bar = nullptr;    // the persistent kernel's grid barrier
  void* rows_mem = nullptr;       // rows for a WaveRowsHook (rows_cap rows)
  int64_t rows_cap = 0;
};

#define PT_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      fprintf(stderr, "petite_gpu: %s failed: %s\n", #call, cudaGetErrorString(e_));  \
      return PT_CUDA_ERR;                                                             \
    }                                                                                 \
  } while (0)

static size_t ring_bytes(int64_t cap) { return (size_t)cap * (9 * 8 + 4 * 4) + 16 * 256; }

// Task chunks a wave can claim: one per 32 tasks of full chunks (a wave of
// k entries has at most k tasks), plus the partly filled chunk of each
// process that every propagation warp may end with.
static int64_t chunk_capacity(int64_t list_cap) {
  int dev = 0, sms = 0, threads = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&threads, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  if (sms < 1) sms = 1;
  const int warps = threads > 0 ? threads / 32 : 64;
  return (list_cap + kChunkTasks - 1) / kChunkTasks + 8 * (int64_t)sms * warps + 8;
}

pt_status batch_scratch_alloc(BatchScratch** out, int64_t cap) {
  int64_t c2 = 1 << 10;
  while (c2 < cap) c2 <<= 1;
  BatchScratch* s = *out;
  if (s && s->cap >= c2) return PT_OK;
  batch_scratch_free(s);
  *out = nullptr;
  s = new BatchScratch();
  s->cap = c2;
  s->list_cap = c2 / 2;
  s->chunk_cap = chunk_capacity(s->list_cap);
  if (cudaMalloc(&s->mem, ring_bytes(c2)) != cudaSuccess ||
      cudaMalloc(&s->park, (size_t)s->chunk_cap * kChunkTasks * sizeof(Park<0>)) != cudaSuccess ||
      cudaMalloc(&s->chunks, (size_t)8 * s->chunk_cap * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&s->ctr, 16 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&s->plan, sizeof(WavePlan)) != cudaSuccess || cudaMalloc(&s->bar, 2 * sizeof(unsigned int)) != cudaSuccess ||
      cudaMallocHost(&s->h_ctr, 16 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&s->h_status, sizeof(int)) != cudaSuccess || cudaEventCreate(&s->ev[0]) != cudaSuccess ||
      cudaEventCreate(&s->ev[1]) != cudaSuccess || cudaEventCreate(&s->ev[2]) != cudaSuccess) {
    cudaGetLastError();
    batch_scratch_free(s);
    return PT_OOM;
  }
  *out = s;
  return PT_OK;
}

// Shared memory of the PT_STAGE_SHARED propagation kernel: the three float32
// n*sigma arrays, each padded to 16 bytes; 0 (the cached path) when the
// tables exceed PT_STAGE_MAX_NODES entries or a source is not 16-byte
// aligned, as the bulk copies require.
static size_t ns_stage_bytes(const pt_tables& t) {
  int total = 0;
  for (int s = 0; s < PT_N_NSIGMA; ++s) total = std::max(total, t.ns_base[s] + t.ns_len[s]);
  if (total <= 0 || total > PT_STAGE_MAX_NODES) return 0;
  for (const float* a : {t.ns_x32, t.ns_y32, t.ns_s32})
    if (!a || (reinterpret_cast<uintptr_t>(a) & 15u)) return 0;
  return (size_t)3 * (size_t)((total + 3) & ~3) * sizeof(float);
}

template <int NW>
static const void* propagate_mixed_kernel(int bethe, bool staged) {
  if (staged) return bethe ? (const void*)k_propagate_mixed<1, true, NW> : (const void*)k_propagate_mixed<0, true, NW>;
  return bethe ? (const void*)k_propagate_mixed<1, false, NW> : (const void*)k_propagate_mixed<0, false, NW>;
}

// The kernels of one wave at nw warps per block (2, 4 or 8 for the float32
// kernels; the FP64 kernels run at kWarps).
template <int PREC>
static const void* propagate_kernel(int bethe, bool staged, int nw) {
  if constexpr (PREC == 1) {
    if (nw == 2) return propagate_mixed_kernel<2>(bethe, staged);
    if (nw == 8) return propagate_mixed_kernel<8>(bethe, staged);
    return propagate_mixed_kernel<kWarps>(bethe, staged);
  }
  return bethe ? (const void*)k_propagate_fp64<1> : (const void*)k_propagate_fp64<0>;
}

template <int PREC>
static const void* sample_kernel(int nw) {
  if constexpr (PREC == 1) {
    if (nw == 2) return (const void*)k_sample<1, 2>;
    if (nw == 8) return (const void*)k_sample<1, 8>;
  }
  return (const void*)k_sample<PREC, kWarps>;
}

// Lays out the ring arrays for one engine form in the scratch memory.
template <int PREC>
static RingT<PREC> carve_ring(BatchScratch* s) {
  using R = typename RingT<PREC>::R;
  const int64_t c2 = s->cap;
  char* p = (char*)s->mem;
  auto take = [&](size_t b) { char* r = p; p += (b + 255) & ~size_t(255); return r; };
  RingT<PREC> q;
  q.E = (double*)take(c2 * 8);
  q.E32 = (float*)take(c2 * 4);
  q.px = (R*)take(c2 * sizeof(R)); q.py = (R*)take(c2 * sizeof(R)); q.pz = (R*)take(c2 * sizeof(R));
  q.x = (R*)take(c2 * sizeof(R)); q.y = (R*)take(c2 * sizeof(R)); q.z = (R*)take(c2 * sizeof(R));
  q.mass = (R*)take(c2 * sizeof(R));
  q.key = (uint64_t*)take(c2 * 8);
  q.pid = (int32_t*)take(c2 * 4); q.prim = (int32_t*)take(c2 * 4); q.gen = (int32_t*)take(c2 * 4);
  return q;
}

void batch_scratch_free(BatchScratch* s) {
  if (!s) return;
  cudaFree(s->mem);
  cudaFree(s->park);
  cudaFree(s->chunks);
  cudaFree(s->ctr);
  cudaFree(s->plan);
  cudaFree(s->bar);
  cudaFree(s->rows_mem);
  cudaFreeHost(s->h_ctr);
  cudaFreeHost(s->h_status);
  for (cudaEvent_t e : s->ev)
    if (e) cudaEventDestroy(e);
  delete s;
}

static int resident_blocks(const void* kernel, int threads, size_t dyn_smem = 0) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, dyn_smem);
  if (per < 1) per = 1;
  return sms * per;
}

// The outcome of a run whose waves the GPU planned: its status and waves.
static pt_status finish_planned(HandleParts& hp, BatchScratch* S, cudaStream_t st, int64_t launches, float ms) {
  WavePlan P;
  PT_CUDA(cudaMemcpyAsync(&P, S->plan, sizeof(WavePlan), cudaMemcpyDeviceToHost, st));
  PT_CUDA(cudaMemcpyAsync(S->h_status, hp.status, sizeof(int), cudaMemcpyDeviceToHost, st));
  PT_CUDA(cudaStreamSynchronize(st));
  hp.launches[0] = launches;
  hp.launches[1] = P.waves;
  hp.kernel_ms[0] = ms;
  hp.kernel_ms[1] = 0.0;
  if (*S->h_status != PT_OK) {
    if (*S->h_status == PT_NO_SAMPLE || *S->h_status == PT_TIMEOUT)
      PT_CUDA(cudaMemcpy(hp.last_info, hp.err_info, 3 * sizeof(double), cudaMemcpyDeviceToHost));
    return (pt_status)*S->h_status;
  }
  return PT_OK;
}

// PT_LOOP_GRAPH: one CUDA graph whose conditional WHILE node repeats the
// wave (plan, feed, propagation, sampling) until the plan ends the run; the
// host waits once.  The kernels run at their resident grids; a wave smaller
// than that leaves the extra blocks without work.
template <int PREC>
static pt_status run_graph_loop(HandleParts& hp, BatchScratch* S, WaveCtx<PREC> c, const void* kp, size_t smem_p,
                                const void* ks, int nw, int rb_p, int rb_s, cudaStream_t st) {
  c.plan = S->plan;
  c.slack = (int64_t)rb_s * nw * kOutChunk;
  PT_CUDA(cudaMemsetAsync(S->plan, 0, sizeof(WavePlan), st));
  PT_CUDA(cudaMemsetAsync(S->ctr, 0, 16 * sizeof(unsigned long long), st));
  cudaGraph_t g = nullptr, body = nullptr;
  cudaGraphExec_t ex = nullptr;
  cudaStream_t cs = nullptr;
  pt_status rs = PT_OK;
  float ms = 0.f;
  const unsigned gf = (unsigned)((c.feed_max + 255) / 256);
#define PT_G(call)                                                                          \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      fprintf(stderr, "petite_gpu: %s failed: %s\n", #call, cudaGetErrorString(e_));         \
      rs = PT_CUDA_ERR;                                                                     \
      goto done;                                                                            \
    }                                                                                       \
  } while (0)
  {
    cudaGraphConditionalHandle loop;
    alignas(cudaGraphNodeParams) unsigned char npbuf[sizeof(cudaGraphNodeParams)] = {};
    cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(npbuf);   // zeroed, as the API requires
    cudaGraphNode_t node;
    PT_G(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    PT_G(cudaGraphCreate(&g, 0));
    PT_G(cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault));
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = loop;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    PT_G(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np));
    body = np.conditional.phGraph_out[0];
    PT_G(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    k_plan<PREC><<<1, 32, 0, cs>>>(c, loop);
    k_feed_planned<PREC><<<gf, 256, 0, cs>>>(c);
    {
      void* args[] = {&c};
      cudaLaunchKernel(kp, dim3(rb_p), dim3(nw * 32), args, smem_p, cs);
      cudaLaunchKernel(ks, dim3(rb_s), dim3(nw * 32), args, 0, cs);
    }
    PT_G(cudaStreamEndCapture(cs, &body));
    PT_G(cudaGraphInstantiate(&ex, g, 0));
    PT_G(cudaEventRecord(S->ev[0], st));
    PT_G(cudaGraphLaunch(ex, st));
    PT_G(cudaEventRecord(S->ev[1], st));
    PT_G(cudaEventSynchronize(S->ev[1]));
    PT_G(cudaEventElapsedTime(&ms, S->ev[0], S->ev[1]));
  }
done:
#undef PT_G
  if (ex) cudaGraphExecDestroy(ex);
  if (g) cudaGraphDestroy(g);
  if (cs) cudaStreamDestroy(cs);
  if (rs != PT_OK) {
    cudaGetLastError();
    return rs;
  }
  return finish_planned(hp, S, st, 1, ms);
}

// PT_LOOP_PERSISTENT: one cooperative kernel (all blocks co-resident) runs
// every wave; its warps pull work from the same device pools.
template <int PREC, int BETHE>
static pt_status run_persistent(HandleParts& hp, BatchScratch* S, WaveCtx<PREC> c, cudaStream_t st) {
  const void* kern = (const void*)k_persistent<PREC, BETHE>;
  int dev = 0, sms = 0, per = 0, coop = 0;
  PT_CUDA(cudaGetDevice(&dev));
  PT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PT_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  PT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kThreads, 0));
  if (!coop || per < 1) return PT_CUDA_ERR;
  const int grid = sms * per;
  c.plan = S->plan;
  c.slack = (int64_t)grid * kWarps * kOutChunk;
  PT_CUDA(cudaMemsetAsync(S->plan, 0, sizeof(WavePlan), st));
  PT_CUDA(cudaMemsetAsync(S->ctr, 0, 16 * sizeof(unsigned long long), st));
  PT_CUDA(cudaMemsetAsync(S->bar, 0, 2 * sizeof(unsigned int), st));
  unsigned int* bar = S->bar;
  void* args[] = {&c, &bar};
  PT_CUDA(cudaEventRecord(S->ev[0], st));
  PT_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(kThreads), args, 0, st));
  PT_CUDA(cudaEventRecord(S->ev[1], st));
  PT_CUDA(cudaEventSynchronize(S->ev[1]));
  float ms = 0.f;
  PT_CUDA(cudaEventElapsedTime(&ms, S->ev[0], S->ev[1]));
  return finish_planned(hp, S, st, 1, ms);
}

// The rows in the scratch (allocated on first use): pt_particles layout over
// rows_cap rows (at least one wave; 2^25 rows, 4 GB, so that many waves of a
// deep shower collect before the hook runs), the fields a WaveRowsHook reads.
constexpr int64_t kMinRows = (int64_t)1 << 25;
static pt_status wave_rows(BatchScratch* S, pt_particles* r) {
  const int64_t L = S->list_cap > kMinRows ? S->list_cap : kMinRows;
  S->rows_cap = L;
  const size_t bytes = (size_t)L * (13 * sizeof(double) + sizeof(int32_t) + sizeof(uint64_t)) + 8 * 256;
  if (!S->rows_mem && cudaMalloc(&S->rows_mem, bytes) != cudaSuccess) {
    // a device allocation, not the ring's capacity: PT_OOM would invite a
    // retry with a larger ring
    cudaGetLastError();
    S->rows_mem = nullptr;
    fprintf(stderr, "petite_gpu: no device memory for %zu bytes of shower rows\n", bytes);
    return PT_CUDA_ERR;
  }
  char* p = (char*)S->rows_mem;
  auto take = [&](size_t b) { char* q = p; p += (b + 255) & ~size_t(255); return q; };
  *r = pt_particles{};
  r->p0 = (double*)take(4 * L * sizeof(double));
  r->pf = (double*)take(4 * L * sizeof(double));
  r->rf = (double*)take(3 * L * sizeof(double));
  r->mass = (double*)take(L * sizeof(double));
  r->weight = (double*)take(L * sizeof(double));
  r->pid = (int32_t*)take(L * sizeof(int32_t));
  r->pkey = (uint64_t*)take(L * sizeof(uint64_t));
  r->capacity = L;
  return PT_OK;
}

// PT_LOOP_HOST with pt_batch_tuning.lanes > 1: the primaries split into
// `lanes` contiguous groups, each with its own ring, task pools and counters
// (its own scratch) and its own CUDA stream.  Each lane runs the host loop's
// waves; the host launches a lane's next wave as soon as its last one has
// ended, so one lane's kernels take the SMs that another lane's wave tail
// leaves idle (a deep shower's waves are small and end on a few long tasks).
// Every primary keeps its index and stream, and the tallies are shared
// (atomic adds), so the showers and integer tallies are those of one lane.
// A row hook runs per lane over that lane's rows, the calls ordered on the
// GPU through one event, since the hook's own scratch is shared.
template <int PREC>
static pt_status run_lanes(pt_handle* h, HandleParts& hp, int lanes, const WaveCtx<PREC>& c0, const void* kp,
                           size_t smem_p, const void* ks, int rb_p, int rb_s, int wpb, const double* p0,
                           const double* r0, const int32_t* pid, const double* mass, int64_t n, const pt_opts* o,
                           cudaStream_t st, const WaveRowsHook* hook, int64_t ring_cap) {
  struct Lane {
    BatchScratch* S = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t done = nullptr;        // after the wave's counter and status copies
    WaveCtx<PREC> c;
    int64_t first = 0, n = 0, fed = 0, k = 0, waves = 0, rows_used = 0, seq = 0;
    uint64_t head = 0, tail = 0;
    bool busy = false, over = false;
    pt_particles rows_all{};
  };
  const int nt = wpb * 32;
  if (lanes > n) lanes = (int)n;
  Lane L[kMaxLanes];
  cudaEvent_t start = nullptr, hook_ev = nullptr;
  bool hook_used = false;
  int64_t nl = 0, nw = 0, seq = 0;
  pt_status rs = PT_OK;
  hp.kernel_ms[0] = hp.kernel_ms[1] = 0.0;
#define PT_L(call)                                                                          \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      fprintf(stderr, "petite_gpu: %s failed: %s\n", #call, cudaGetErrorString(e_));         \
      rs = PT_CUDA_ERR;                                                                     \
      goto drain;                                                                           \
    }                                                                                       \
  } while (0)
#define PT_LS(expr)                                                                         \
  do {                                                                                      \
    const pt_status s_ = (expr);                                                            \
    if (s_ != PT_OK) { rs = s_; goto drain; }                                               \
  } while (0)
  PT_L(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  PT_L(cudaEventCreateWithFlags(&hook_ev, cudaEventDisableTiming));
  PT_L(cudaEventRecord(start, st));      // the inputs, tallies and status word are ready on st
  for (int l = 0; l < lanes; ++l) {
    Lane& a = L[l];
    PT_LS(batch_lane_scratch_get(h, l, &a.S, ring_cap));
    PT_L(cudaStreamCreateWithFlags(&a.s, cudaStreamNonBlocking));
    PT_L(cudaEventCreateWithFlags(&a.done, cudaEventDisableTiming));
    PT_L(cudaStreamWaitEvent(a.s, start, 0));
    a.first = n * l / lanes;
    a.n = n * (l + 1) / lanes - a.first;
    a.c = c0;
    a.c.q = carve_ring<PREC>(a.S);
    a.c.mask = (uint64_t)a.S->cap - 1;
    a.c.list_cap = a.S->list_cap;
    a.c.park = reinterpret_cast<Park<PREC>*>(a.S->park);
    a.c.chunks = a.S->chunks;
    a.c.chunk_cap = a.S->chunk_cap;
    a.c.ctr = a.S->ctr;
    a.c.cap = a.S->cap;
    if (hook) PT_LS(wave_rows(a.S, &a.rows_all));
  }
  for (;;) {
    bool launched = false, any_busy = false;
    for (int l = 0; l < lanes; ++l) {
      Lane& a = L[l];
      if (a.over) continue;
      if (a.busy) {
        const cudaError_t q = cudaEventQuery(a.done);
        if (q == cudaErrorNotReady) { any_busy = true; continue; }
        PT_L(q);
        a.busy = false;
        if (*a.S->h_status != PT_OK) {
          rs = (pt_status)*a.S->h_status;
          if (rs == PT_NO_SAMPLE || rs == PT_TIMEOUT)
            PT_L(cudaMemcpy(hp.last_info, hp.err_info, 3 * sizeof(double), cudaMemcpyDeviceToHost));
          goto drain;
        }
        float ms_p = 0.f, ms_s = 0.f;
        PT_L(cudaEventElapsedTime(&ms_p, a.S->ev[0], a.S->ev[1]));
        PT_L(cudaEventElapsedTime(&ms_s, a.S->ev[1], a.S->ev[2]));
        hp.kernel_ms[0] += ms_p;
        hp.kernel_ms[1] += ms_s;
        a.head += (uint64_t)a.k;
        a.tail += a.S->h_ctr[2];
      }
      if (a.fed >= a.n && a.tail == a.head) {           // this lane's showers are done
        if (hook && a.rows_used > 0) {
          if (hook_used) PT_L(cudaStreamWaitEvent(a.s, hook_ev, 0));
          PT_LS(hook->fn(hook->ctx, &a.rows_all, a.rows_used, a.s));
          PT_L(cudaEventRecord(hook_ev, a.s));
          hook_used = true;
          ++nl;
          a.rows_used = 0;
        }
        a.over = true;
        continue;
      }
      // the next wave of this lane: the host loop's feed and sizing
      const int64_t cap = a.S->cap;
      const int64_t feed_max = cap / 1024 > 256 ? cap / 1024 : 256;
      int64_t live = (int64_t)(a.tail - a.head);
      if (a.fed < a.n && live < cap / 8) {
        int64_t m = a.n - a.fed;
        if (m > cap / 8 - live) m = cap / 8 - live;
        if (m > feed_max) m = feed_max;
        k_feed<PREC><<<(unsigned)((m + 255) / 256), 256, 0, a.s>>>(a.c.q, a.c.mask, a.tail, p0, r0, pid, mass, n,
                                                                  a.first + a.fed, m, o->primary_offset);
        ++nl;
        a.tail += (uint64_t)m;
        a.fed += m;
        live += m;
      }
      a.c.out_chunk = kOutChunk;
      int64_t k = (cap - live - (int64_t)rb_s * wpb * kOutChunk) / 2;
      if (k > live) k = live;
      if (k > a.S->list_cap) k = a.S->list_cap;
      if (k < 16 * 1024) {
        a.c.out_chunk = 0;
        k = (cap - live) / 2;
        if (k > live) k = live;
        if (k > a.S->list_cap) k = a.S->list_cap;
      }
      if (k <= 0) { rs = PT_OOM; goto drain; }
      if (a.waves >= a.c.max_waves) {
        hp.last_info[0] = -1; hp.last_info[1] = 0.0; hp.last_info[2] = 0;
        rs = PT_TIMEOUT;
        goto drain;
      }
      PT_L(cudaMemsetAsync(a.S->ctr, 0, 16 * sizeof(unsigned long long), a.s));
      if (hook) {
        if (a.rows_used + k > a.rows_all.capacity) {
          if (hook_used) PT_L(cudaStreamWaitEvent(a.s, hook_ev, 0));
          PT_LS(hook->fn(hook->ctx, &a.rows_all, a.rows_used, a.s));
          PT_L(cudaEventRecord(hook_ev, a.s));
          hook_used = true;
          ++nl;
          a.rows_used = 0;
        }
        a.c.rows = a.rows_all;
        a.c.rows.p0 += a.rows_used; a.c.rows.pf += a.rows_used; a.c.rows.rf += a.rows_used;
        a.c.rows.mass += a.rows_used; a.c.rows.weight += a.rows_used; a.c.rows.pid += a.rows_used;
        a.c.rows.pkey += a.rows_used;
      }
      a.c.head = a.head;
      a.c.tail = a.tail;
      a.c.n_in = k;
      a.k = k;
      {
        const int64_t want_blocks = (k + nt - 1) / nt;
        const unsigned gp = (unsigned)(want_blocks < rb_p ? want_blocks : rb_p);
        const unsigned gs = (unsigned)(want_blocks < rb_s ? want_blocks : rb_s);
        void* args[] = {&a.c};
        PT_L(cudaEventRecord(a.S->ev[0], a.s));
        PT_L(cudaLaunchKernel(kp, dim3(gp), dim3(nt), args, smem_p, a.s));
        PT_L(cudaEventRecord(a.S->ev[1], a.s));
        PT_L(cudaLaunchKernel(ks, dim3(gs), dim3(nt), args, 0, a.s));
        PT_L(cudaEventRecord(a.S->ev[2], a.s));
      }
      PT_L(cudaGetLastError());
      a.rows_used += hook ? k : 0;
      PT_L(cudaMemcpyAsync(a.S->h_ctr, a.S->ctr, 16 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, a.s));
      PT_L(cudaMemcpyAsync(a.S->h_status, hp.status, sizeof(int), cudaMemcpyDeviceToHost, a.s));
      PT_L(cudaEventRecord(a.done, a.s));
      nl += 3;
      ++nw;
      ++a.waves;
      a.busy = true;
      a.seq = ++seq;
      launched = any_busy = true;
    }
    if (!any_busy) break;                              // every lane is over
    if (!launched) {
      // poll until any lane's wave ends (blocking on one lane's event would
      // hold back a lane whose wave ends first); a wave that runs far past
      // any wave's length ends the wait on the oldest lane instead
      const auto t0 = std::chrono::steady_clock::now();
      for (bool ready = false; !ready;) {
        for (int l = 0; l < lanes && !ready; ++l) {
          if (!L[l].busy) continue;
          const cudaError_t q = cudaEventQuery(L[l].done);
          if (q != cudaErrorNotReady) { PT_L(q); ready = true; }
        }
        if (!ready && std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(200)) {
          int w = -1;
          for (int l = 0; l < lanes; ++l)
            if (L[l].busy && (w < 0 || L[l].seq < L[w].seq)) w = l;
          PT_L(cudaEventSynchronize(L[w].done));
          ready = true;
        }
        if (!ready) std::this_thread::yield();
      }
    }
  }
drain:
  // every lane's work has ended before its stream goes; the caller's stream
  // then follows the lanes
  for (int l = 0; l < lanes; ++l) {
    if (!L[l].s) continue;
    if (cudaStreamSynchronize(L[l].s) != cudaSuccess && rs == PT_OK) rs = PT_CUDA_ERR;
    if (L[l].done && cudaEventRecord(L[l].done, L[l].s) == cudaSuccess) cudaStreamWaitEvent(st, L[l].done, 0);
  }
  if (rs == PT_OK) {
    int hs = PT_OK;
    if (cudaMemcpy(&hs, hp.status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) rs = PT_CUDA_ERR;
    else rs = (pt_status)hs;
  }
  for (int l = 0; l < lanes; ++l) {
    if (L[l].done) cudaEventDestroy(L[l].done);
    if (L[l].s) cudaStreamDestroy(L[l].s);
  }
  if (start) cudaEventDestroy(start);
  if (hook_ev) cudaEventDestroy(hook_ev);
#undef PT_L
#undef PT_LS
  if (rs == PT_CUDA_ERR) cudaGetLastError();
  hp.launches[0] = nl;
  hp.launches[1] = nw;
  return rs;
}

static Consts32 consts32(const Tabs& T, const pt_opts* o) {
  Consts32 k;
  k.mc[0] = (float)T.t.min_calc_photon; k.mc[1] = (float)T.t.min_calc_electron;
  k.mc[2] = (float)T.t.min_calc_positron; k.mc[3] = (float)T.t.min_calc_muon;
  k.min_energy = (float)o->min_energy;
  k.dedx = (float)T.t.dEdx_GeV_per_m;
  k.rho_cm = (float)(T.t.rho / kCmToM);
  k.A = (float)T.t.A; k.Z = (float)T.t.Z; k.Z23 = (float)T.t.Z23; k.Z13 = (float)T.t.Z13;
  k.rescale = (float)o->rescale_MCS;
  k.Eg_min = (float)T.t.Eg_min; k.Ee_min = (float)T.t.Ee_min; k.a0sq = (float)T.a0sq;
  k.ld = ld32_constants(T.t.A, T.t.Z, T.t.Z23);
  return k;
}

template <int PREC>
static pt_status run_batch_impl(pt_handle* h, BatchScratch* S, const double* p0, const double* r0, const int32_t* pid,
                                const double* mass, int64_t n, const pt_opts* o, pt_tally* tally, cudaStream_t st,
                                const WaveRowsHook* hook = nullptr) {
  HandleParts hp = handle_parts(h);
  WaveCtx<PREC> c;
  c.T = *hp.T;
  c.min_energy = o->min_energy;
  c.rescale = o->rescale_MCS;
  c.k32 = consts32(c.T, o);
  c.max_n_integrators = o->max_n_integrators;
  c.ms = o->multiple_scattering;
  c.mcs_mode = o->mcs_mode;
  c.seed = o->seed;
  c.q = carve_ring<PREC>(S);
  c.mask = (uint64_t)S->cap - 1;
  c.list_cap = S->list_cap;
  c.park = reinterpret_cast<Park<PREC>*>(S->park);
  c.chunks = S->chunks;
  c.chunk_cap = S->chunk_cap;
  c.ctr = S->ctr;
  c.status = hp.status;
  c.err_info = hp.err_info;
  c.tally = {tally->counts, tally->energy, tally->hist, tally->primary_count, tally->primary_edep,
             (float)(tally->z_max > 0 ? tally->z_max : 1.0)};
  c.rk = philox_round_keys(o->seed);
  const int32_t* tu = hp.tuning;      // 0 = default
  c.max_waves = o->loop_limit > 0 ? o->loop_limit : kMaxPlannedWaves;
  c.barrier_ns = tu[7] > 0 ? (unsigned long long)tu[7] : kBarrierNs;
  c.refill_min[0] = tu[0] ? tu[0] : kRefillMinPropagate;
  c.refill_min[1] = tu[1] ? tu[1] : kRefillMinSample;
  c.chunk[0] = tu[2] ? tu[2] : kChunkPropagate;
  c.chunk[1] = tu[3] ? tu[3] : kChunkSample;
  c.plan = nullptr;
  c.rows = pt_particles{};
  pt_particles rows_all{};        // every collected row; c.rows views it from the wave's first row
  int64_t rows_used = 0;
  if (hook) {
    const pt_status rs = wave_rows(S, &rows_all);
    if (rs != PT_OK) return rs;
  }
  c.in_p0 = p0; c.in_r0 = r0; c.in_pid = pid; c.in_mass = mass;
  c.n_prim = n;
  c.prim_offset = o->primary_offset;
  c.cap = S->cap;
  c.feed_max = S->cap / 1024 > 256 ? S->cap / 1024 : 256;
  c.slack = 0;
  const size_t smem_p = PREC == 1 && tu[5] != PT_STAGE_CACHED ? ns_stage_bytes(c.T.t) : 0;
  const int wpb = PREC == 1 && tu[6] ? tu[6] / 32 : kWarps;
  const int nt = wpb * 32;
  const void* kp = propagate_kernel<PREC>(c.mcs_mode, smem_p > 0, wpb);
  const void* ks = sample_kernel<PREC>(wpb);
  // the staged tables are dynamic shared memory on top of the kernel's
  // static share; beyond 48 KB in all, a kernel must be allowed the dynamic
  // part explicitly
  if (smem_p) PT_CUDA(cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p));
  const int rb_p = resident_blocks(kp, nt, smem_p);
  const int rb_s = resident_blocks(ks, nt);
  PT_CUDA(cudaMemsetAsync(hp.status, 0, sizeof(int), st));
  if (!hook && tu[4] == PT_LOOP_GRAPH) return run_graph_loop<PREC>(hp, S, c, kp, smem_p, ks, wpb, rb_p, rb_s, st);
  if (!hook && tu[4] == PT_LOOP_PERSISTENT)
    return c.mcs_mode ? run_persistent<PREC, 1>(hp, S, c, st) : run_persistent<PREC, 0>(hp, S, c, st);
  if (tu[8] > 1 && n > 1)
    return run_lanes<PREC>(h, hp, tu[8], c, kp, smem_p, ks, rb_p, rb_s, wpb, p0, r0, pid, mass, n, o, st, hook,
                           S->cap);
  const int64_t cap = S->cap;
  // A fed primary can grow to a few hundred live particles before its shower
  // thins out, so primaries enter in small increments while the ring is
  // mostly free.
  const int64_t feed_max = cap / 1024 > 256 ? cap / 1024 : 256;
  uint64_t head = 0, tail = 0;
  int64_t fed = 0, nl = 1, nw = 0;
  hp.kernel_ms[0] = hp.kernel_ms[1] = 0.0;
  while (fed < n || tail > head) {
    int64_t live = (int64_t)(tail - head);
    if (fed < n && live < cap / 8) {
      int64_t m = n - fed;
      if (m > cap / 8 - live) m = cap / 8 - live;
      if (m > feed_max) m = feed_max;
      k_feed<PREC><<<(unsigned)((m + 255) / 256), 256, 0, st>>>(c.q, c.mask, tail, p0, r0, pid, mass, n, fed, m,
                                                                o->primary_offset);
      ++nl;
      tail += (uint64_t)m;
      fed += m;
      live += m;
    }
    // Wave size: daughters take at most 2 slots per entry, plus at most one
    // partly used output chunk per sampler warp (bounded with the largest
    // grid); small waves reserve slots exactly and leave no dead entries.
    c.out_chunk = kOutChunk;
    int64_t k = (cap - live - (int64_t)rb_s * wpb * kOutChunk) / 2;
    if (k > live) k = live;
    if (k > S->list_cap) k = S->list_cap;
    if (k < 16 * 1024) {
      c.out_chunk = 0;
      k = (cap - live) / 2;
      if (k > live) k = live;
      if (k > S->list_cap) k = S->list_cap;
    }
    if (k <= 0) {                   // the live population filled the ring
      hp.launches[0] = nl; hp.launches[1] = nw;
      return PT_OOM;
    }
    if (nw >= c.max_waves) {        // a bound on the loop, far above any run's need
      hp.launches[0] = nl; hp.launches[1] = nw;
      hp.last_info[0] = -1; hp.last_info[1] = 0.0; hp.last_info[2] = 0;
      return PT_TIMEOUT;
    }
    PT_CUDA(cudaMemsetAsync(S->ctr, 0, 16 * sizeof(unsigned long long), st));
    if (hook) {
      // the hook runs over the collected rows when the next wave would not fit
      if (rows_used + k > rows_all.capacity) {
        const pt_status hs = hook->fn(hook->ctx, &rows_all, rows_used, st);
        if (hs != PT_OK) {
          hp.launches[0] = nl; hp.launches[1] = nw;
          return hs;
        }
        ++nl;
        rows_used = 0;
      }
      c.rows = rows_all;
      c.rows.p0 += rows_used; c.rows.pf += rows_used; c.rows.rf += rows_used;
      c.rows.mass += rows_used; c.rows.weight += rows_used; c.rows.pid += rows_used; c.rows.pkey += rows_used;
    }
    c.head = head;
    c.tail = tail;
    c.n_in = k;
    const int64_t want_blocks = (k + nt - 1) / nt;
    const unsigned gp = (unsigned)(want_blocks < rb_p ? want_blocks : rb_p);
    const unsigned gs = (unsigned)(want_blocks < rb_s ? want_blocks : rb_s);
    PT_CUDA(cudaEventRecord(S->ev[0], st));
    void* args[] = {&c};
    PT_CUDA(cudaLaunchKernel(kp, dim3(gp), dim3(nt), args, smem_p, st));
    PT_CUDA(cudaEventRecord(S->ev[1], st));
    PT_CUDA(cudaLaunchKernel(ks, dim3(gs), dim3(nt), args, 0, st));
    PT_CUDA(cudaEventRecord(S->ev[2], st));
    PT_CUDA(cudaGetLastError());
    rows_used += hook ? k : 0;
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
    float ms_p = 0.f, ms_s = 0.f;
    PT_CUDA(cudaEventElapsedTime(&ms_p, S->ev[0], S->ev[1]));
    PT_CUDA(cudaEventElapsedTime(&ms_s, S->ev[1], S->ev[2]));
    hp.kernel_ms[0] += ms_p;
    hp.kernel_ms[1] += ms_s;
    head += (uint64_t)k;
    tail += S->h_ctr[2];
  }
  if (hook && rows_used > 0) {
    const pt_status hs = hook->fn(hook->ctx, &rows_all, rows_used, st);
    ++nl;
    if (hs != PT_OK) {
      hp.launches[0] = nl; hp.launches[1] = nw;
      return hs;
    }
  }
  hp.launches[0] = nl;
  hp.launches[1] = nw;
  return PT_OK;
}

pt_status run_batch_rows(pt_handle* h, const double* p0, const double* r0, const int32_t* pid, const double* mass,
                         int64_t n, const pt_opts* o, pt_tally* tally, int64_t queue_capacity,
                         const WaveRowsHook* hook, cudaStream_t st) {
  if (!h || !o || !tally || n < 0) return PT_BAD_ARG;
  if (n == 0) return PT_OK;
  if (!p0 || !r0 || !pid || !mass || !tally->counts || !tally->energy || !tally->hist || !tally->primary_count ||
      !tally->primary_edep || (o->precision != 0 && o->precision != 1) || n > 0x7fffffff)
    return PT_BAD_ARG;
  BatchScratch* S = nullptr;
  const pt_status s = batch_scratch_get(h, &S, queue_capacity > 0 ? queue_capacity : ((int64_t)1 << 24));
  if (s != PT_OK) return s;
  if (o->precision == 1) return run_batch_impl<1>(h, S, p0, r0, pid, mass, n, o, tally, st, hook);
  return run_batch_impl<0>(h, S, p0, r0, pid, mass, n, o, tally, st, hook);
}

extern "C" pt_status pt_run_batch(pt_handle* h, const double* p0, const double* r0, const int32_t* pid,
                                  const double* mass, int64_t n, const pt_opts* o, pt_tally* tally,
                                  int64_t queue_capacity, void* stream) {
  if (!h || !o || !tally || n < 0) return PT_BAD_ARG;
  if (n == 0) return PT_OK;
  if (!p0 || !r0 || !pid || !mass || !tally->counts || !tally->energy || !tally->hist || !tally->primary_count ||
      !tally->primary_edep || (o->precision != 0 && o->precision != 1) || n > 0x7fffffff)
    return PT_BAD_ARG;
  BatchScratch* S = nullptr;
  const pt_status s = batch_scratch_get(h, &S, queue_capacity > 0 ? queue_capacity : ((int64_t)1 << 24));
  if (s != PT_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  if (o->precision == 1) return run_batch_impl<1>(h, S, p0, r0, pid, mass, n, o, tally, st);
  return run_batch_impl<0>(h, S, p0, r0, pid, mass, n, o, tally, st);
}
