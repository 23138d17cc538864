// engine.h -- host-side interface of one plume simulation on one GPU.
//
// The C ABI (plume_api.cpp) owns an Engine through this interface; the
// implementation is a template on the field type (engine.cuh), instantiated
// once for FP64 (parity mode, compiled without multiply-add contraction) and
// once for FP32 (fields in FP32, CG scalars and the MIC diagonal in FP64).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/plume.h"
#include "../../include/plume_box.h"

namespace plume {

class NetRuntime;

class Engine {
 public:
  virtual ~Engine() {}
  // Allocates device state and builds the MIC diagonal.  Returns plume_status.
  virtual int init(const plume_params& p) = 0;
  virtual int add_source(int32_t step_index) = 0;
  virtual int add_source_values(const double* values, size_t n) = 0;
  virtual int run_timed(int32_t first_step, int32_t n, double* ms, plume_step_stats* stats) = 0;
  // Enqueue one step; if stats != nullptr, wait for it and fill stats.
  virtual int step(plume_step_stats* stats) = 0;
  virtual int run(int32_t first_step, int32_t n, plume_step_stats* stats) = 0;
  // Moving box obstacle (include/plume_box.h): one stepWithMovingObstacle,
  // setInitialVelocity(BOX*), and the obstacle matrix of the last moving step
  // (inside mask and last-column values, full-grid layout).
  virtual int step_moving_box(const plume_box& box, plume_step_stats* stats) = 0;
  virtual int set_initial_velocity_box(const plume_box& box) = 0;
  virtual bool has_iop() const = 0;
  // Full-space part of the reduced step (include/plume_reduced.h) on the
  // engine's stream; kernels launched since its start.
  virtual int reduced_prestep() = 0;
  virtual int reduced_launches() const = 0;
  virtual int run_moving_timed(plume_box& box, int32_t first_step, int32_t n, double* ms,
                               plume_step_stats* stats) = 0;
  // with sweep profiling on: summed device ms and launches of the stomp kernel
  virtual int stomp_times(double* ms, int64_t* launches) = 0;
  virtual int download_iop(uint8_t* inside, double* values, size_t n) = 0;
  virtual int download(int field, double* dst, size_t n) = 0;
  virtual int upload(int field, const double* src, size_t n) = 0;
  virtual int download_obstacles(uint8_t* dst, size_t n) = 0;
  // Poisson solve on a caller right-hand side (interior of `b`), x in/out.
  virtual int solve(const double* b, double* x, plume_step_stats* stats) = 0;
  // Forward/backward MIC sweeps of the engine's preconditioner on r (FP64 in/out).
  virtual int mic_apply(const double* r, double* z, double* q) = 0;
  virtual int mic_precon(double* precon) = 0;
  virtual int sync() = 0;
  // CUDA-event timing of every MIC sweep launch: on != 0 clears the totals
  // and starts recording, 0 stops; sweep_times returns the summed device ms
  // and the number of timed launches.
  virtual int profile_sweeps(int on) = 0;
  // The divergence's solve from x = 0 stopped after at most `max_iters`
  // iterations, the iterate written into `x` (a device plane of N values of
  // the engine's field type, border 0); the step's own solver state is
  // overwritten (training pairs of the preconditioner role).
  virtual int partial_solve(int max_iters, void* x) = 0;
  // Test hook of the sweeps' bounded waits (plume_set_wait_gate).
  virtual int set_wait_gate(int closed, long long polls) = 0;
  virtual int sweep_times(double* ms, int64_t* launches) = 0;
  // Device pointer of a scalar field (field type: float or double as the
  // engine's precision), the engine's cudaStream_t, and the network used by
  // PLUME_WARM_LEARNED solves (nullptr detaches).
  virtual const void* device_field(int field) = 0;
  // The three device planes (x, y, z) of a vector field, nullptr-free only
  // when the field is kept (cached fields need cache_fields; postIOP a moving
  // step); false otherwise.
  virtual bool device_vector(int field, const void* planes[3]) = 0;
  virtual void* stream_handle() = 0;
  virtual int attach_net(NetRuntime* net) = 0;
  // CG loop as a CUDA graph (default) or driven from the host; many handles
  // stepping concurrently interleave better with the host-driven loop
  virtual void use_cg_graph(bool on) = 0;
  virtual int32_t total_steps() const = 0;
  virtual double total_time() const = 0;
  virtual double dx() const = 0;
  virtual const plume_params& params() const = 0;
  virtual std::string& last_error() = 0;
  // The step counter and time, as a state file being resumed holds them.
  virtual void set_clock(int32_t steps, double time) = 0;
};

// box.cpp: half lengths, angular and displacement velocity of a box for the
// current step; false if a parameter is non-finite or a period is zero.
void box_constants(const plume_box& b, double half[3], double omega[3], double disp[3]);
bool box_finite(const plume_box& b);

Engine* make_engine_f64();
Engine* make_engine_f32();

// C ABI helpers (plume_api.cpp): a handle's engine, and the calling thread's
// error text for calls that have no handle.
Engine* engine_of(plume_handle* h);
std::string& global_error();

}  // namespace plume
