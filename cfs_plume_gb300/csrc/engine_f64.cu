// engine_f64.cu -- FP64 engine (reference-parity mode).  Built with
// -fmad=false: no multiply-add contraction, so every per-cell expression
// rounds exactly as the reference's serial C++ does.
#define PLUME_DEFINE_PRECON 1
#include "engine.cuh"

namespace plume {

cudaError_t build_mic_diagonal(const Grid& g, double* P64, double tau, double sig, cudaStream_t s) {
  for (int pl = 0; pl <= g.nx + g.ny + g.nz - 3; pl++) {
    k_mic_precon_plane<<<grid_for((long long)g.ny * g.nz), 256, 0, s>>>(g, P64, pl, tau, sig);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

Engine* make_engine_f64() { return new EngineT<double>(); }

}  // namespace plume
