// unet.h -- what the solver engine sees of the learned warm start.
#pragma once
#include <string>

namespace plume {

class NetRuntime {
 public:
  virtual ~NetRuntime() {}
  // Workspace for predictions on one grid (batch 1); nullptr on failure.
  virtual void* new_workspace(const int res[3], std::string& err) = 0;
  virtual void free_workspace(void* ws) = 0;
  // Interior cells of x (device grid, FP32 or FP64) = the network's initial
  // guess for A x = b; everything is queued on `stream`.  Returns plume_status.
  virtual int predict(void* ws, const void* b, void* x, int is_double, void* stream, std::string& err) = 0;
  // Kernel launches one predict() makes.
  virtual int launches_per_predict() const = 0;
  // 0: maps a right-hand side b to the solution; 1: maps the residual of the
  // previous step's pressure to the pressure change
  virtual int kind() const = 0;
  // After the caller synchronised the prediction's stream: PLUME_ERR_TIMEOUT
  // (flag cleared, err set) if a convolution's bounded wait expired, so that
  // its output is invalid; PLUME_OK otherwise.
  virtual int take_error(std::string& err) = 0;
};

}  // namespace plume
