// pt_internal.cuh -- declarations shared by the library's translation units
// (not part of the public C ABI).
#pragma once
#include "pt_physics.cuh"

struct pt_handle;
struct BatchScratch;

// Batched-engine scratch owned by a handle (allocated on first use).
pt_status batch_scratch_get(pt_handle* h, BatchScratch** out, int64_t ring_capacity);
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
