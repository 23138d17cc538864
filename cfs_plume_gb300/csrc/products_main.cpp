// products_main.cpp -- the buildProducts stage (binary bin/buildProducts): host
// C++ over the C ABI of include/plume.h and include/plume_reduced.h.
//
// Same command line and cfg keys as the reference's
// projects/buildProducts/buildProducts.cpp:21-80: the grid (xRes, yRes,
// zRes), the walls (front, back, left, right, top, bottom; defaults 1 1 1 1
// 0 0) and `reduced path`.  The reference constructs SUBSPACE_FLUID_3D_EIGEN
// for its side effects: initOutOfCore builds the projected operators when
// they are missing or stale (buildOutOfCoreMatrices) and readAdvectionCubature
// builds the advection cubature cache when it is missing.  Here
// plume_reduced_create does both on the GPU.  `iop = 1` selects the
// reference's IOP operators (initOutOfCoreIOP), which this build does not
// provide: the binary says so and fails.
#include <iostream>
#include <string>

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

}  // namespace

int main(int argc, char* argv[]) {
  if (argc != 2) {  // buildProducts.cpp:23-27
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
  const char* names[6] = {"front", "back", "left", "right", "top", "bottom"};
  const int defaults[6] = {1, 1, 1, 1, 0, 0};
  for (int k = 0; k < 6; k++) p.bc[k] = cfg.integer(names[k], defaults[k]);
  p.device = cfg.integer("device", 0);
  const std::string reduced = cfg.str("reduced path", "./data/reduced.dummy/");
  const bool iop = cfg.integer("iop", 0) != 0;
  for (int k = 0; k < 6; k++)
    std::cout << " Boundary on " << names[k] << "\tis set to " << (p.bc[k] == 0 ? "Neumann " : "Dirichlet ")
              << std::endl;
  std::cout << " Using iop: " << iop << std::endl;
  if (iop) {
    std::cerr << " iop = 1: the IOP reduced operators (initOutOfCoreIOP) are not provided by this build"
              << std::endl;
    return 1;
  }
  plume_handle* h = nullptr;
  if (check(plume_create(&p, &h), nullptr, "plume_create") != PLUME_OK) return 1;
  plume_reduced* m = nullptr;
  const int rc = check(plume_reduced_create(h, reduced.c_str(), &m), nullptr, "building the reduced model");
  if (rc == PLUME_OK) {
    int32_t dims[5] = {0, 0, 0, 0, 0};
    plume_reduced_dims(m, dims);
    std::cout << " Reduced model under " << reduced << ": preadvect " << dims[0] << ", prediffuse " << dims[1]
              << ", preproject " << dims[2] << ", final " << dims[3] << " columns, " << dims[4]
              << " cubature points" << std::endl;
    plume_reduced_destroy(m);
  }
  plume_destroy(h);
  return rc == PLUME_OK ? 0 : 1;
}
