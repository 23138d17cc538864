// reduced_main.cpp -- the reduced3D stage (binary bin/reduced3D) without the
// GLUT window: host C++ over the C ABI of include/plume.h and
// include/plume_reduced.h.
//
// Same command line and cfg keys as the reference's
// projects/reduced3D/reduced3D.cpp (main 299-353, runEverytime 366-400):
// xRes, yRes, zRes, vorticity, the six wall flags (defaults 1 1 1 1 0 0),
// `reduced path` (the model: bases, projected operators, cubature; missing
// operators and cubature cache are built, as the reference's constructor
// does), `snapshot path` (the full-rank run that every step is compared
// against, diffGroundTruth) and `simulation snapshots` (the step count).  Per
// step: addSmokeColumn, stepReorderedCubatureStam; every 10 steps the error
// vectors are printed in the reference's form.  `iop = 1` selects the
// reference's IOP model, which this build does not provide: the binary says
// so and fails.  `device` picks the GPU.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/plume.h"
#include "../../include/plume_reduced.h"
#include "cli_config.h"

namespace {

int check(int rc, plume_handle* h, const char* what) {
  if (rc != PLUME_OK)
    std::cerr << " " << what << " failed: " << plume_strerror(rc) << " (" << plume_last_error(h) << ")"
              << std::endl;
  return rc;
}

// VECTOR's stream form, as reduced3D.cpp:381-384 prints the error vectors
void print_errors(plume_reduced* m) {
  int32_t count = 0;
  plume_reduced_errors(m, nullptr, 0, &count);
  std::vector<double> e(4 * (size_t)count);
  if (count > 0) plume_reduced_errors(m, e.data(), (int32_t)e.size(), &count);
  const char* names[4] = {"velocityAbs", "velocityRelative", "densityAbs", "densityRelative"};
  for (int k = 0; k < 4; k++) {
    std::cout << " " << names[k] << " = [";
    for (int32_t s = 0; s < count; s++) std::cout << e[4 * (size_t)s + k] << (s + 1 < count ? " " : "");
    std::cout << "];" << std::endl;
  }
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc != 2) {  // reduced3D.cpp:302-306
    std::cout << " Usage: " << argv[0] << " *.cfg" << std::endl;
    return 0;
  }
  plume_cli::Config cfg;
  std::string err;
  if (!cfg.load(argv[1], err)) {
    std::cerr << " " << err << std::endl;
    return 1;
  }
  plume_params p;
  plume_default_params(&p);
  p.res[0] = cfg.integer("xRes", 48);
  p.res[1] = cfg.integer("yRes", 64);
  p.res[2] = cfg.integer("zRes", 48);
  p.vorticity_eps = cfg.num("vorticity", 0);
  const char* names[6] = {"front", "back", "left", "right", "top", "bottom"};
  const int defaults[6] = {1, 1, 1, 1, 0, 0};
  for (int k = 0; k < 6; k++) p.bc[k] = cfg.integer(names[k], defaults[k]);
  p.device = cfg.integer("device", 0);
  const std::string reduced = cfg.str("reduced path", "./data/reduced.dummy/");
  const std::string snapshot = cfg.str("snapshot path", "./data/dummy/");
  const int steps = cfg.integer("simulation snapshots", 20);
  const bool iop = cfg.integer("iop", 0) != 0;
  std::cout << " Using resoluion: " << p.res[0] << " " << p.res[1] << " " << p.res[2] << std::endl;
  std::cout << " Using vorticity: " << p.vorticity_eps << std::endl;
  for (int k = 0; k < 6; k++)
    std::cout << " Boundary on " << names[k] << "\tis set to " << (p.bc[k] == 0 ? "Neumann " : "Dirichlet ")
              << std::endl;
  std::cout << " UsingIOP: " << iop << std::endl;
  if (iop) {
    std::cerr << " iop = 1: the IOP reduced model (initOutOfCoreIOP) is not provided by this build" << std::endl;
    return 1;
  }
  plume_handle* h = nullptr;
  if (check(plume_create(&p, &h), nullptr, "plume_create") != PLUME_OK) return 1;
  plume_reduced* m = nullptr;
  int rc = check(plume_reduced_create(h, reduced.c_str(), &m), nullptr, "loading the reduced model");
  if (rc == PLUME_OK) rc = check(plume_reduced_set_ground_truth(m, snapshot.c_str()), nullptr, "fullRankPath");
  for (int step = 0; step < steps && rc == PLUME_OK; step++) {  // reduced3D.cpp:366-400
    std::cout << " Simulation step " << 1 + step << std::endl;
    rc = check(plume_add_source(h, step), h, "addSmokeColumn");
    plume_step_stats st;
    if (rc == PLUME_OK) rc = check(plume_reduced_step(m, &st), nullptr, "stepReorderedCubatureStam");
    if (rc == PLUME_OK && (step % 10 == 0 || step == steps - 1)) print_errors(m);
  }
  if (m) plume_reduced_destroy(m);
  plume_destroy(h);
  return rc == PLUME_OK ? 0 : 1;
}
