// fluid3d_main.cpp -- `fluid3D <cfg>`: the full-rank snapshot stage of the
// pipeline, as a drop-in for the reference's projects/fluid3D/fluid3D.cpp
// (main 300-353, runEverytime 357-398) without the GLUT window and movie.
//
// Same command line, same cfg keys and defaults, same outputs:
//   <snapshot path>fluid.%04i.fluid3d.gz        FLUID_3D_MIC::writeGz format
//   <snapshot path>velocity.*.matrix.transpose  FLUID_3D_MIC::appendStreams rows
//   <snapshot path>pressure.matrix.transpose    (+ the .dims files)
// so svdOutOfCoreMultiple and cubatureGeneratorStamStaged read them unchanged.
//
// Keys read by the reference (fluid3D.cpp:313-343): xres yres zres vorticity
// front back left right top bottom, snapshot path, simulation snapshots.
// Additional keys, whose defaults reproduce the reference:
//   buoyancy (0.1f), source (column | box), source box = x0 y0 z0 x1 y1 z1,
//   source noise (0), seed (0), precision (fp64 | fp32), solver criterion
//   (reference | rel2), solver tolerance (1e-10), solver max iterations (1000),
//   mic tau (0.97), mic sigma (0.25), damping (0.9), warm start (zero |
//   previous | learned), warm start network (path of a trained network for
//   "learned"; default cfs_plume_gb300/weights/unet_warmstart.bin next to the
//   binary's ../weights), write state (1), write streams (1), device (0),
//   resume from (a state file of an earlier run of the same cfg: its fields and
//   step count are restored, plume_read_state, and the run continues from the
//   step after it; empty: start from rest), log file (append one JSON object
//   per step with the step's plume_step_stats; empty: no log).
#include <sys/stat.h>

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/plume.h"
#include "../../include/plume_net.h"
#include "cli_config.h"

namespace {

using plume_cli::Config;
using plume_cli::ensure_directory;

int check(int rc, plume_handle* h, const char* what) {
  if (rc != PLUME_OK) {
    std::cerr << " " << what << " failed: " << plume_strerror(rc) << " (" << plume_last_error(h)
              << ")" << std::endl;
  }
  return rc;
}

}  // namespace

// <dir of the binary>/../weights/unet_warmstart.bin (the package layout)
static std::string default_network_path(const char* argv0) {
  std::string d = argv0 ? argv0 : "";
  const size_t slash = d.find_last_of('/');
  d = slash == std::string::npos ? std::string(".") : d.substr(0, slash);
  return d + "/../weights/unet_warmstart.bin";
}

int main(int argc, char* argv[]) {
  if (argc != 2) {  // fluid3D.cpp:303-307
    std::cout << " Usage: " << argv[0] << " *.cfg" << std::endl;
    return 0;
  }
  Config cfg;
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
  p.buoyancy = cfg.num("buoyancy", (double)0.1f);
  const std::string source = cfg.str("source", "column");
  if (source == "box") {
    p.source = PLUME_SRC_BOX;
    std::istringstream box(cfg.str("source box", ""));
    for (int k = 0; k < 3; k++) box >> p.box_lo[k];
    for (int k = 0; k < 3; k++) box >> p.box_hi[k];
    p.source_noise = cfg.num("source noise", 0.0);
    p.seed = (uint64_t)cfg.num("seed", 0);
  } else if (source == "none") {
    p.source = PLUME_SRC_NONE;
  }
  if (cfg.str("precision", "fp64") == "fp32") p.precision = PLUME_PREC_FP32;
  if (cfg.str("solver criterion", "reference") == "rel2") {
    p.criterion = PLUME_CRIT_REL2;
    p.tol = 1e-6;
  }
  p.tol = cfg.num("solver tolerance", p.tol);
  p.max_iters = cfg.integer("solver max iterations", 1000);
  p.mic_tau = cfg.num("mic tau", 0.97);
  p.mic_sigma = cfg.num("mic sigma", 0.25);
  p.damping_w = cfg.num("damping", 0.9);
  const std::string warm = cfg.str("warm start", "zero");
  if (warm == "previous") p.warm_start = PLUME_WARM_PREVIOUS;
  if (warm == "learned") p.warm_start = PLUME_WARM_LEARNED;
  const std::string net_path = cfg.str("warm start network", default_network_path(argv[0]));
  p.device = cfg.integer("device", 0);
  const bool write_state = cfg.integer("write state", 1) != 0;
  const bool write_streams = cfg.integer("write streams", 1) != 0;
  std::string snapshot_path = cfg.str("snapshot path", "./data/dummy/");
  const int snapshots = cfg.integer("simulation snapshots", 20);
  // checkpoint / resume: a state file of an earlier run of the same cfg
  const std::string resume = cfg.str("resume from", "");
  // one JSON object per step (step_json)
  const std::string log_path = cfg.str("log file", "");
  int first_step = 0;
  if (!resume.empty()) {  // the file is checked on the host before any device work
    int32_t ints[10];
    double consts[7];
    if (check(plume_state_read_header(resume.c_str(), ints, consts), nullptr, "resume from") != PLUME_OK) return 1;
    if (ints[0] != p.res[0] || ints[1] != p.res[1] || ints[2] != p.res[2]) {
      std::cerr << " resume from: " << resume << " holds a " << ints[0] << "x" << ints[1] << "x" << ints[2]
                << " grid, the cfg a " << p.res[0] << "x" << p.res[1] << "x" << p.res[2] << " one" << std::endl;
      return 1;
    }
    first_step = ints[9];
  }
  std::FILE* log = nullptr;
  if (!log_path.empty() && !(log = std::fopen(log_path.c_str(), "a"))) {
    std::cerr << " log file: cannot open " << log_path << std::endl;
    return 1;
  }

  std::cout << " Using resoluion: " << p.res[0] << " " << p.res[1] << " " << p.res[2] << std::endl;
  std::cout << " Using vorticity: " << p.vorticity_eps << std::endl;
  for (int k = 0; k < 6; k++)
    std::cout << " Boundary on " << names[k] << "\tis set to "
              << (p.bc[k] == 0 ? "Neumann " : "Dirichlet ") << std::endl;
  ensure_directory(snapshot_path);

  plume_handle* h = nullptr;
  if (check(plume_create(&p, &h), nullptr, "plume_create") != PLUME_OK) return 1;
  plume_net* net = nullptr;
  if (p.warm_start == PLUME_WARM_LEARNED) {
    if (check(plume_net_create(0, p.device, &net), nullptr, "plume_net_create") != PLUME_OK ||
        check(plume_net_load(net, net_path.c_str()), nullptr, "plume_net_load") != PLUME_OK ||
        check(plume_attach_net(h, net), nullptr, "plume_attach_net") != PLUME_OK) {
      plume_destroy(h);
      plume_net_destroy(net);
      return 1;
    }
    std::cout << " Using learned warm start: " << net_path << std::endl;
  }
  int rc = PLUME_OK;
  if (!resume.empty()) {
    rc = check(plume_read_state(h, resume.c_str()), h, "resume from");
    if (rc == PLUME_OK) std::cout << " Resuming after step " << first_step << " from " << resume << std::endl;
  }
  for (int step = first_step; step < snapshots && rc == PLUME_OK; step++) {  // fluid3D.cpp:357-398
    std::cout << " Simulation step " << 1 + step << " of " << snapshots << std::endl;
    plume_step_stats st;
    rc = check(plume_add_source(h, step), h, "add_source");
    if (rc == PLUME_OK) rc = check(plume_step(h, &st), h, "step");
    if (rc != PLUME_OK) break;
    std::cout << "   " << st.iterations << " iterations converged to inf norm: " << st.max_residual
              << " relative two norm: " << st.rel_residual << "  (" << st.ms_total << " ms)"
              << std::endl;
    if (log) {
      const double n_int = (double)(p.res[0] - 2) * (p.res[1] - 2) * (p.res[2] - 2);
      const int S = p.precision == PLUME_PREC_FP32 ? 4 : 8;
      std::fprintf(log, "%s\n", plume_cli::step_json(step, st, n_int, S).c_str());
      std::fflush(log);
    }
    // writeGz + appendStreams (fluid3D.cpp:376-386) on the handle's writer
    // thread, overlapping the next steps
    const int what = (write_state ? 1 : 0) | (write_streams ? 2 : 0);
    if (what) rc = check(plume_snapshot_async(h, snapshot_path.c_str(), step, what), h, "snapshot");
  }
  if (rc == PLUME_OK) rc = check(plume_wait_snapshots(h), h, "snapshot");
  if (log) std::fclose(log);
  plume_destroy(h);
  plume_net_destroy(net);  // after the handle that used it
  return rc == PLUME_OK ? 0 : 1;
}
