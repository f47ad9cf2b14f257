// pt_train.cu -- VEGAS adaptive-map training and find_maxes on the GPU.
//
// PETITE trains one VEGAS AdaptiveMap per (process, incoming energy) with
// the vegas package (all_processes.py:1160-1245, vegas_integration in
// "Pickle" mode; utilities/generate_integrators.py:49-84) and then scans each
// map for the largest weighted integrand and the cross section
// (utilities/find_maxes.py:56-115).  Here every energy row trains at once:
//   pt_vegas_accumulate  samples each row's map (uniform y -> x, jacobian),
//                        evaluates the process's float64 differential cross
//                        section and accumulates (jac f)^2 per increment of
//                        each dimension;
//   pt_vegas_adapt       the VEGAS map adaptation (G. P. Lepage, J. Comput.
//                        Phys. 27 (1978) 192): per dimension the average
//                        (jac f)^2 of each increment, smoothed over
//                        neighbours, normalised, compressed as
//                        ((1 - d)/ln(1/d))^alpha, and the nodes moved so that
//                        every new increment holds an equal share;
//   pt_find_maxes        per row and target, n_trials batches of neval points
//                        with weight jac/neval: the largest weight*f (max_F)
//                        and the mean over trials of the summed weight*f.
// Draws come from Philox streams keyed by (row, iteration, point).
#include <cmath>
#include <cstdio>

#include "pt_dark.cuh"
#include "pt_internal.cuh"
#include "pt_physics.cuh"
#include "pt_tma.cuh"

using namespace pt;

namespace {

constexpr int kTrainThreads = 256;
constexpr int kMaxInc = 1000;
constexpr int kMaxDim = 4;
constexpr unsigned long long kStageNs = 1000ull * 1000ull * 1000ull;


// A Tabs carrying only what the SM differential cross sections read.
__device__ __forceinline__ Tabs train_tabs(const pt_train_target& t) {
  Tabs T;
  T.t.Eg_min = t.Eg_min;
  T.t.Ee_min = t.Ee_min;
  T.a0sq = t.a0sq;
  T.Z2a04 = t.Z2a04;
  return T;
}

// The differential cross section being trained: an SM process, or a dark one
// with the target's (mV, mT, Z, A) -- diff_xsection_options,
// all_processes.py:1067-1083; DarkMuonBrem takes the muon mass
// (find_maxes.py:94-97).
__device__ __forceinline__ double train_dsigma(const Tabs& T, const pt_train_target& tg, int process, const double* x,
                                               double E) {
  if (process < PT_TRAIN_DARK) return dsigma_any(T, process, x, E);
  switch (process - PT_TRAIN_DARK) {
    case PT_DARKBREM: return dsig_dark_brem<double>(x, E, tg.mV, tg.MT, kMe, tg.Z, tg.A);
    case PT_DARKMUONBREM: return dsig_dark_brem<double>(x, E, tg.mV, tg.MT, kMmu, tg.Z, tg.A);
    case PT_DARKCOMP: return dsig_dark_compton<double>(x[0], E, tg.mV);
    default: return dsig_radiative_return<double>(x[0], E, tg.mV);
  }
}

__host__ __device__ inline bool train_process_ok(int process) {
  return (process >= 0 && process < PT_N_PROCESSES) ||
         (process >= PT_TRAIN_DARK && process < PT_TRAIN_DARK + PT_N_DARK);
}

struct MapView {
  int dims;
  int ninc[kMaxDim];
  int max_nodes;
};

// A timed-out staging copy (PT_TIMEOUT), read back by the entry points.
__device__ int g_train_status;

// The block's map row (dims x max_nodes float64 nodes) in shared memory,
// staged by a TMA bulk copy; nullptr (status recorded) when it did not land.
__device__ __forceinline__ const double* stage_row(const double* g, const MapView& m) {
  extern __shared__ __align__(16) double s_row[];
  __shared__ __align__(8) uint64_t bar;
  double* out = nullptr;
  if (!stage_doubles(s_row, g, m.dims * m.max_nodes, &bar, kStageNs, &out)) {
    if (threadIdx.x == 0) atomicCAS(&g_train_status, 0, (int)PT_TIMEOUT);
    return nullptr;
  }
  return out;
}

__host__ __device__ inline size_t row_smem_bytes(int dims, int max_nodes) {
  return ((size_t)dims * max_nodes + 2) * sizeof(double);
}

// y in [0,1)^dims -> x, jacobian (AdaptiveMap.map: piecewise linear).
__device__ __forceinline__ double map_point(const MapView& m, const double* g, Rng& rng, double* x, int* inc) {
  double jac = 1.0;
  for (int d = 0; d < m.dims; ++d) {
    const int n = m.ninc[d];
    const double t = rng.u() * n;
    int i = (int)t;
    if (i > n - 1) i = n - 1;
    const double* gd = g + (size_t)d * m.max_nodes;
    const double w = gd[i + 1] - gd[i];
    x[d] = gd[i] + w * (t - i);
    jac *= n * w;
    inc[d] = i;
  }
  return jac;
}

__global__ void __launch_bounds__(kTrainThreads) k_vegas_accumulate(pt_train_target tgt, int process, const double* E,
                                                                    MapView m, const double* nodes,
                                                                    int64_t points_per_row, uint64_t seed,
                                                                    uint32_t iteration, double* acc, unsigned* cnt,
                                                                    double* sums) {
  __shared__ double s_acc[kMaxDim * kMaxInc];
  __shared__ unsigned s_cnt[kMaxDim * kMaxInc];
  for (int k = threadIdx.x; k < m.dims * kMaxInc; k += blockDim.x) { s_acc[k] = 0.0; s_cnt[k] = 0u; }
  const int row = blockIdx.y;
  const Tabs T = train_tabs(tgt);
  const double* g = stage_row(nodes + (size_t)row * m.dims * m.max_nodes, m);   // synchronises the block
  if (!g) return;
  const double Er = E[row];
  double s1 = 0.0, s2 = 0.0;
  const uint64_t base = ((uint64_t)row << 40) ^ ((uint64_t)iteration << 34);
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < points_per_row;
       p += (int64_t)gridDim.x * blockDim.x) {
    Rng rng;
    rng.init(seed, mix64(base + (uint64_t)p));
    double x[kMaxDim] = {0.0, 0.0, 0.0, 0.0};
    int inc[kMaxDim] = {0, 0, 0, 0};
    const double jac = map_point(m, g, rng, x, inc);
    double w = jac * train_dsigma(T, tgt, process, x, Er);
    if (!(w == w)) w = 0.0;
    s1 += w;
    s2 += w * w;
    for (int d = 0; d < m.dims; ++d) {
      atomicAdd(&s_acc[d * kMaxInc + inc[d]], w * w);
      atomicAdd(&s_cnt[d * kMaxInc + inc[d]], 1u);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums + 2 * row, s1);
    atomicAdd(sums + 2 * row + 1, s2);
  }
  __syncthreads();
  double* a = acc + (size_t)row * m.dims * kMaxInc;
  unsigned* c = cnt + (size_t)row * m.dims * kMaxInc;
  for (int k = threadIdx.x; k < m.dims * kMaxInc; k += blockDim.x)
    if (s_cnt[k]) {
      atomicAdd(a + k, s_acc[k]);
      atomicAdd(c + k, s_cnt[k]);
    }
}

// One block per (row, dimension); the sequential regridding runs on thread 0
// over shared arrays.
__global__ void k_vegas_adapt(MapView m, double* nodes, const double* acc, const unsigned* cnt, double alpha) {
  __shared__ double s_d[kMaxInc];
  __shared__ double s_g[kMaxInc + 1];
  const int row = blockIdx.x, d = blockIdx.y;
  const int n = m.ninc[d];
  double* g = nodes + ((size_t)row * m.dims + d) * m.max_nodes;
  const double* a = acc + ((size_t)row * m.dims + d) * kMaxInc;
  const unsigned* c = cnt + ((size_t)row * m.dims + d) * kMaxInc;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s_d[i] = c[i] ? a[i] / c[i] : 0.0;
  for (int i = threadIdx.x; i <= n; i += blockDim.x) s_g[i] = g[i];
  __syncthreads();
  if (threadIdx.x != 0 || n < 2) return;
  // smoothing over neighbours (weights 1, 6, 1; 7, 1 at the ends)
  double prev = s_d[0], total = 0.0;
  for (int i = 0; i < n; ++i) {
    const double cur = s_d[i];
    const double next = i + 1 < n ? s_d[i + 1] : cur;
    double v;
    if (i == 0) v = (7.0 * cur + next) / 8.0;
    else if (i == n - 1) v = (prev + 7.0 * cur) / 8.0;
    else v = (prev + 6.0 * cur + next) / 8.0;
    prev = cur;
    s_d[i] = v;
    total += v;
  }
  if (!(total > 0.0) || !isfinite(total)) return;                // no information: the grid stays
  // normalise and compress
  double sum = 0.0;
  for (int i = 0; i < n; ++i) {
    const double r = s_d[i] / total;
    double v = 0.0;
    if (r > 0.0) v = r < 1.0 - 1e-12 ? pow((1.0 - r) / log(1.0 / r), alpha) : 1.0;
    s_d[i] = v;
    sum += v;
  }
  if (!(sum > 0.0)) return;
  // new nodes: equal shares of the compressed weights, linear inside old increments
  const double share = sum / n;
  int j = 0;
  double below = 0.0;                        // weight of old increments before j
  g[0] = s_g[0];
  for (int k = 1; k < n; ++k) {
    const double target = k * share;
    while (j < n - 1 && below + s_d[j] < target) below += s_d[j++];
    const double f = s_d[j] > 0.0 ? (target - below) / s_d[j] : 0.0;
    const double fc = f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f);
    g[k] = s_g[j] + fc * (s_g[j + 1] - s_g[j]);
  }
  g[n] = s_g[n];
}

// One block per (row, target): n_trials batches of neval map points.
__global__ void __launch_bounds__(kTrainThreads) k_find_maxes(const pt_train_target* tg, int process, const double* E,
                                                              MapView m, const double* nodes, int neval, int n_trials,
                                                              uint64_t seed, double* max_F, double* xsec) {
  __shared__ double s_max[kTrainThreads / 32], s_sum[kTrainThreads / 32];
  const int row = blockIdx.x, t = blockIdx.y, nt = gridDim.y;
  const Tabs T = train_tabs(tg[t]);
  const double* g = stage_row(nodes + (size_t)row * m.dims * m.max_nodes, m);
  if (!g) return;
  const double Er = E[row];
  const int64_t total = (int64_t)neval * n_trials;
  double mx = 0.0, sm = 0.0;
  for (int64_t p = threadIdx.x; p < total; p += blockDim.x) {
    Rng rng;
    rng.init(seed, mix64(((uint64_t)row << 40) ^ ((uint64_t)t << 36) ^ (uint64_t)p));
    double x[kMaxDim] = {0.0, 0.0, 0.0, 0.0};
    int inc[kMaxDim];
    const double jac = map_point(m, g, rng, x, inc);
    const double MM = jac / neval * train_dsigma(T, tg[t], process, x, Er);
    if (MM > mx) mx = MM;
    if (MM == MM) sm += MM;
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    sm += __shfl_down_sync(0xffffffffu, sm, o);
  }
  if ((threadIdx.x & 31) == 0) { s_max[threadIdx.x / 32] = mx; s_sum[threadIdx.x / 32] = sm; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kTrainThreads / 32; ++w) { mx = fmax(mx, s_max[w]); sm += s_sum[w]; }
    max_F[(size_t)row * nt + t] = mx;
    xsec[(size_t)row * nt + t] = sm / n_trials;
  }
}

bool make_view(int dims, const int32_t* ninc, int max_nodes, MapView& m) {
  if (dims < 1 || dims > kMaxDim || !ninc) return false;
  m.dims = dims;
  m.max_nodes = max_nodes;
  for (int d = 0; d < kMaxDim; ++d) m.ninc[d] = 1;
  for (int d = 0; d < dims; ++d) {
    if (ninc[d] < 1 || ninc[d] > kMaxInc || ninc[d] + 1 > max_nodes) return false;
    m.ninc[d] = ninc[d];
  }
  return true;
}

#define PT_T(call)                                                                      \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      fprintf(stderr, "petite_gpu: %s failed: %s\n", #call, cudaGetErrorString(e_));    \
      return PT_CUDA_ERR;                                                               \
    }                                                                                   \
  } while (0)

int* status_word() {
  void* p = nullptr;
  cudaGetSymbolAddress(&p, g_train_status);
  return (int*)p;
}

// Waits for the stream and returns a staging timeout, if any.
pt_status read_status(cudaStream_t st) {
  int s = 0;
  PT_T(cudaMemcpyFromSymbolAsync(&s, g_train_status, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
  PT_T(cudaStreamSynchronize(st));
  return (pt_status)s;
}

}  // namespace

extern "C" pt_status pt_vegas_accumulate(int32_t process, const pt_train_target* target, const double* energy,
                                         int32_t n_rows, int32_t dims, const int32_t* ninc, const double* nodes,
                                         int32_t max_nodes, int64_t points_per_row, uint64_t seed, int32_t iteration,
                                         double* acc, uint32_t* cnt, double* sums, void* stream) {
  MapView m;
  if (!train_process_ok(process) || !target || n_rows < 1 || n_rows > 65535 || points_per_row < 1 ||
      iteration < 0 || iteration > 63 || !make_view(dims, ninc, max_nodes, m))
    return PT_BAD_ARG;
  if (!energy || !nodes || !acc || !cnt || !sums) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int64_t bx = (points_per_row + kTrainThreads * 16 - 1) / (kTrainThreads * 16);
  if (bx > 1024) bx = 1024;
  const size_t smem = row_smem_bytes(dims, max_nodes);
  PT_T(cudaFuncSetAttribute(k_vegas_accumulate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PT_T(cudaMemsetAsync(status_word(), 0, sizeof(int), st));
  k_vegas_accumulate<<<dim3((unsigned)bx, (unsigned)n_rows), kTrainThreads, smem, st>>>(
      *target, process, energy, m, nodes, points_per_row, seed, (uint32_t)iteration, acc, cnt, sums);
  PT_T(cudaGetLastError());
  return read_status(st);
}

extern "C" pt_status pt_vegas_adapt(int32_t n_rows, int32_t dims, const int32_t* ninc, double* nodes,
                                    int32_t max_nodes, const double* acc, const uint32_t* cnt, double alpha,
                                    void* stream) {
  MapView m;
  if (n_rows < 1 || n_rows > 65535 || !make_view(dims, ninc, max_nodes, m) || !(alpha >= 0.0)) return PT_BAD_ARG;
  if (!nodes || !acc || !cnt) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  k_vegas_adapt<<<dim3((unsigned)n_rows, (unsigned)dims), 128, 0, st>>>(m, nodes, acc, cnt, alpha);
  PT_T(cudaGetLastError());
  return PT_OK;
}

extern "C" pt_status pt_find_maxes(int32_t process, const pt_train_target* targets, int32_t n_targets,
                                   const double* energy, int32_t n_rows, int32_t dims, const int32_t* ninc,
                                   const double* nodes, int32_t max_nodes, int32_t neval, int32_t n_trials,
                                   uint64_t seed, double* max_F, double* xsec, void* stream) {
  MapView m;
  if (!train_process_ok(process) || !targets || n_targets < 1 || n_targets > 16 || n_rows < 1 ||
      n_rows > 65535 || neval < 1 || n_trials < 1 || !make_view(dims, ninc, max_nodes, m))
    return PT_BAD_ARG;
  if (!energy || !nodes || !max_F || !xsec) return PT_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  pt_train_target* d_t = nullptr;
  PT_T(cudaMallocAsync((void**)&d_t, sizeof(pt_train_target) * n_targets, st));
  PT_T(cudaMemcpyAsync(d_t, targets, sizeof(pt_train_target) * n_targets, cudaMemcpyHostToDevice, st));
  const size_t smem = row_smem_bytes(dims, max_nodes);
  PT_T(cudaFuncSetAttribute(k_find_maxes, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PT_T(cudaMemsetAsync(status_word(), 0, sizeof(int), st));
  k_find_maxes<<<dim3((unsigned)n_rows, (unsigned)n_targets), kTrainThreads, smem, st>>>(
      d_t, process, energy, m, nodes, neval, n_trials, seed, max_F, xsec);
  PT_T(cudaGetLastError());
  PT_T(cudaFreeAsync(d_t, st));
  return read_status(st);
}
