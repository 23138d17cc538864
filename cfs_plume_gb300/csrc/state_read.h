// state_read.h -- the reference's state file read on the host, for the
// library's own callers (plume_read_state, the reduced model's ground-truth
// comparison).  The C entry points are in include/plume.h.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace plume {

struct StateField {
  int field;    // plume_field id
  double* dst;  // n doubles, reference layout
  size_t n;
};
using StateRequest = std::vector<StateField>;

// One pass over the file (FLUID_3D_MIC::readGz's order), keeping every
// requested field; res (may be null) receives the file's grid.
int read_state_fields(const std::string& path, const StateRequest& want, int32_t res[3]);

}  // namespace plume
