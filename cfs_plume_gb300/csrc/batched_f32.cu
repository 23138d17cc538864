// batched_f32.cu -- the fused batch engine with FP32 fields (FP64 CG scalars,
// reductions and MIC diagonal), the batched-plume configuration's precision.
#include "batched.cuh"

namespace plume {

BatchEngine* make_batch_engine_f32() { return new BatchEngineT<float>(); }

}  // namespace plume
