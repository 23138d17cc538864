// engine_f32.cu -- FP32 engine: FP32 fields, stencils, advection and SpMV;
// FP64 CG scalars, reductions and MIC diagonal.
#include "engine.cuh"

namespace plume {

Engine* make_engine_f32() { return new EngineT<float>(); }

}  // namespace plume
