// batched.h -- host-side interface of the fused batch engine (batched.cuh):
// many plumes of uneven grids advanced in lockstep, one launch per stage over
// all of them, each step one CUDA graph launch.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/plume.h"
#include "../../include/plume_batch.h"

namespace plume {

class BatchEngine {
 public:
  virtual ~BatchEngine() {}
  // Allocates every plume's device state, builds the MIC diagonals, picks the
  // tile shapes (tuning cache or autotuner) and captures the step graph.
  virtual int init(const plume_params* p, int n, const plume_batch_options& o) = 0;
  // `steps` lockstep steps (source, then step), stats instance-major.
  virtual int run(int32_t first_step, int32_t steps, double* seconds, plume_step_stats* stats) = 0;
  virtual int download(int32_t i, int32_t field, double* dst, size_t n) = 0;
  // The tile shapes in use as one JSON object.
  virtual std::string tuning_json() const = 0;
  virtual std::string& last_error() = 0;
};

BatchEngine* make_batch_engine_f32();
BatchEngine* make_batch_engine_f64();

}  // namespace plume
