// snapshot.h -- host-side writers of the reference's on-disk formats.
//
//  * the full state file of FLUID_3D_MIC::writeGz (FLUID_3D_MIC.cpp:1020-1110),
//    gzip level 1, readable by FLUID_3D_MIC::readGz (1115-1246);
//  * the per-step rows of FLUID_3D_MIC::appendStreams (1329-1477) consumed by
//    svdOutOfCoreMultiple / BIG_MATRIX::outOfCoreQR and EIGEN::readRaw.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace plume {

struct StateHeader {
  int res[3];
  int total_steps;
  double dx, total_time, dt, buoyancy, vorticity_eps;
};

// The obstacle matrix N of the last moving-box step (FLUID_3D_MIC.h:246,
// built by setPeeledSparseMovingIOP, FLUID_3D_MIC.cpp:1645-1692), as an
// inside mask (N cells) and the last-column values (3N); both empty when no
// moving step has run, in which case the reference writes no matrix.
struct IopRecord {
  std::vector<uint8_t> inside;
  std::vector<double> values;
};

// fetch(field_id, dst) fills dst (N or 3N doubles, reference layout) and
// returns 0 on success; field ids are plume_field values.
using FieldFetch = std::function<int(int, std::vector<double>&)>;

// Writes the state file; `obstacles` has N bytes.  PLUME_F_POST_IOP may
// fetch an empty vector (never assigned).  Returns a plume_status.
int write_state_gz(const std::string& path, const StateHeader& h, const FieldFetch& fetch,
                   const std::vector<uint8_t>& obstacles, const IopRecord& iop, std::string& err);

// Appends one step's rows under `dir` (which must end with a path separator,
// as the reference's snapshot path does).  Returns a plume_status.
int append_streams(const std::string& dir, const int res[3], const FieldFetch& fetch,
                   const IopRecord& iop, std::string& err);

}  // namespace plume
