// pt_internal.cuh -- declarations shared by the library's translation units
// (not part of the public C ABI).
#pragma once
#include "pt_physics.cuh"

struct pt_handle;
struct BatchScratch;

// Batched-engine scratch owned by a handle (allocated on first use).
// Lanes of a batched run (pt_batch_tuning.lanes): lane 0 is the handle's
// scratch, lanes 1.. their own, kept for the next run.
constexpr int kMaxLanes = 8;
pt_status batch_scratch_get(pt_handle* h, BatchScratch** out, int64_t ring_capacity);
pt_status batch_lane_scratch_get(pt_handle* h, int lane, BatchScratch** out, int64_t ring_capacity);
pt_status batch_scratch_alloc(BatchScratch** s, int64_t ring_capacity);
void batch_scratch_free(BatchScratch* s);

// Access to a handle's tables, status word and launch counters.
struct HandleParts {
  pt::Tabs* T;
  int* status;
  double* err_info;
  double* last_info;
  int64_t* launches;   // [0] kernel launches, [1] waves of the last run
  double* kernel_ms;   // device time of the last batched run: [0] propagation, [1] sampler
  int32_t* tuning;     // batched engine: refill_min[2], chunk[2] (0 = default), loop (PT_LOOP_*)
};
HandleParts handle_parts(pt_handle* h);

// Rows of the batched engine: with a hook, the propagation kernel writes
// each particle of a wave as a row (p0 at the start of its propagation, pf
// and rf at its end, pid, mass, weight 1, pkey: the record engine's row of
// that particle; a dead entry leaves pid 0).  The rows of successive waves
// collect in one buffer; fn runs on the run's stream over the first n_rows
// rows when the next wave would not fit, and once at the end of the run.
// The host loop runs the waves of such a run.
struct WaveRowsHook {
  pt_status (*fn)(void* ctx, const pt_particles* rows, int64_t n_rows, cudaStream_t st);
  void* ctx;
};
pt_status run_batch_rows(pt_handle* h, const double* p0, const double* r0, const int32_t* pid, const double* mass,
                         int64_t n, const pt_opts* o, pt_tally* tally, int64_t queue_capacity,
                         const WaveRowsHook* hook, cudaStream_t st);
