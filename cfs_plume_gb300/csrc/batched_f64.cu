// batched_f64.cu -- the fused batch engine in FP64, compiled without
// multiply-add contraction like the FP64 single-plume engine, so each cell
// rounds as the reference's serial C++ does.
#include "batched.cuh"

namespace plume {

BatchEngine* make_batch_engine_f64() { return new BatchEngineT<double>(); }

}  // namespace plume
