// svd_main.cpp -- the svdOutOfCoreMultiple stage (binary bin/svdOutOfCoreMultiple):
// host C++ over the C ABI of include/plume_svd.h.
//
// Same command line and cfg keys as the reference's
// projects/svdOutOfCoreMultiple/svdOutOfCoreMultiple.cpp:87-177: for each
// snapshot stream under `snapshot path` (velocity.final, .preproject,
// .prediffuse, .preadvect, pressure, and velocity.iop when `iop` is set) it
// writes U.<name>.matrix and pca.<name>.vector under `reduced path` and the
// singular-value vector under `scratch path`, then prints the reference's
// projection check |c - U U^T c| for the first 10 snapshots.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/plume.h"
#include "../../include/plume_svd.h"
#include "cli_config.h"

int main(int argc, char* argv[]) {
  if (argc != 2) {
    std::cout << " Usage: " << argv[0] << " *.cfg" << std::endl;
    return 0;
  }
  plume_cli::Config cfg;
  std::string err;
  if (!cfg.load(argv[1], err)) {
    std::cerr << " " << err << std::endl;
    return 1;
  }
  const std::string snapshot = cfg.str("snapshot path", "./data/dummy/");
  const std::string reduced = cfg.str("reduced path", "./data/reduced.dummy/");
  const std::string scratch = cfg.str("scratch path", "./data/scratch/");
  const int simulation = cfg.integer("simulation snapshots", 20);
  const int reduced_snaps = cfg.integer("reduced snapshots", 20);
  const double threshold = cfg.num("discard threshold", 1e-9);
  const bool iop = cfg.integer("iop", 0) != 0;
  const int device = cfg.integer("device", 0);
  std::cout << (iop ? " Using IOP " : " NOT using IOP ") << std::endl;
  std::cout << " Using discard threshold: " << threshold << std::endl;
  plume_cli::ensure_directory(scratch);
  plume_cli::ensure_directory(reduced);
  if (reduced_snaps > simulation) {  // svdOutOfCoreMultiple.cpp:126-130
    std::cout << " You asked to use more snapshots than were simulated! " << std::endl;
    return 0;
  }
  std::vector<std::string> names = {"velocity.final", "velocity.preproject", "velocity.prediffuse",
                                    "velocity.preadvect", "pressure"};
  std::vector<std::string> tags = {"final", "preproject", "prediffuse", "preadvect", "pressure"};
  if (iop) {
    names.push_back("velocity.iop");
    tags.push_back("iop");
  }
  for (size_t x = 0; x < names.size(); x++) {
    const std::string prefix = snapshot + names[x] + ".matrix";
    const std::string u = reduced + "U." + tags[x] + ".matrix";
    const std::string pca = reduced + "pca." + tags[x] + ".vector";
    plume_svd_info info{};
    const int rc = plume_svd_stream(prefix.c_str(), reduced.c_str(), scratch.c_str(), threshold, u.c_str(),
                                    pca.c_str(), device, &info);
    if (rc != PLUME_OK) {
      std::cerr << " SVD of " << prefix << " failed: " << plume_strerror(rc) << " (" << plume_last_error(nullptr)
                << ")" << std::endl;
      return 1;
    }
    std::cout << " " << names[x] << ": " << info.rows << " x " << info.cols << ", keeping " << info.kept
              << " of " << info.cols << " columns; QR " << info.ms_qr << " ms, SVD " << info.ms_svd
              << " ms (" << info.sweeps << " sweeps), U " << info.ms_u << " ms, I/O " << info.ms_io
              << " ms" << std::endl;
    double diffs[10];
    const int count = info.cols < 10 ? info.cols : 10;
    if (plume_svd_verify(prefix.c_str(), u.c_str(), count, device, diffs) == PLUME_OK)
      for (int k = 0; k < count; k++) std::cout << " Diff " << k << ": " << diffs[k] << std::endl;
  }
  return 0;
}
