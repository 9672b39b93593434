// batch.h -- host interface of the batch kernel (kernels_batch.cu): a plan
// of phases and jobs built from the per-image dispatch schedules, its device
// copy, and the launch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "internal.h"

namespace nvpyr {

// The tunable shape of a batch launch (no influence on the bytes written).
// The default (measured on the 256-image benchmark batch: 8 warps with up to
// 255 registers beat 12 with 168 by 1.8x, whatever the unit sizes).
struct BatchTuning {
  uint32_t stripBand = 8;  // rows of level L+2 per general-pipeline strip unit
  uint32_t fastRows = 64;  // rows of level L per fast-pipeline region unit (at least 2^n, at most 64)
  uint32_t warps = 8;      // warps per CTA: 8 or 12
};

// The plan's tables in device memory (one block, written by upload).
struct BatchDevice {
  void* device = nullptr;
  const void* jobs = nullptr;
  const uint32_t* phaseJobBegin = nullptr;
  const uint32_t* phaseUnits = nullptr;
  uint32_t* counters = nullptr;  // unit counters [phases], barrier count, generation, error flag
  uint32_t phaseCount = 0;
  uint32_t warps = 8;  // CTA size of the launch
  uint64_t countersOffset = 0;
  uint64_t countersBytes = 0;
};

class BatchPlan {
 public:
  BatchPlan();
  ~BatchPlan();
  BatchPlan(const BatchPlan&) = delete;
  BatchPlan& operator=(const BatchPlan&) = delete;

  // Phases and jobs for images[i] = the dispatches of image i's schedule
  // (sRGBA8, full workgroup coverage), with units of the tuning's sizes
  // (strip band: rows of level L+2 per strip of a two-level general dispatch,
  // twice as many rows of level L+1 for one level).  cudaErrorInvalidValue if
  // a dispatch is not supported.
  cudaError_t build(const std::vector<std::vector<DispatchParams>>& images, const BatchTuning& tuning);
  uint64_t deviceBytes() const;  // upper bound of the device block
  // Copy the tables into `device` (deviceBytes() bytes) and synchronise `stream`.
  cudaError_t upload(void* device, cudaStream_t stream, BatchDevice* out) const;
  uint32_t phaseCount() const;
  uint32_t jobCount() const;
  uint64_t unitCount() const;
  uint64_t errorFlagOffset() const;  // byte offset of the error flag in the counters

 private:
  struct Tables;
  Tables* t_;
};

// Per-device set-up of the batch kernel (shared memory size, occupancy);
// done by the first launch too, but must precede a stream capture.
cudaError_t batchDeviceReady();

// Zero the unit counters and barrier words, then launch the batch kernel
// (cooperative, d.warps warps per CTA) on `stream`.
cudaError_t launchBatch(const BatchDevice& d, cudaStream_t stream, uint32_t* launches);

}  // namespace nvpyr
