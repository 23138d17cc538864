// reduced_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Headless stand-in for projects/reduced3D/reduced3D.cpp (main, lines 300-350,
// and runEverytime, lines 366-400) without GLUT: it builds the reference's own,
// unmodified SUBSPACE_FLUID_3D_EIGEN from a reduced path (the constructor
// projects the operators and the cubature cache when they are missing and
// writes them there), loads the runtime bases and runs addSmokeColumn +
// stepReorderedCubatureStam per step.
//
// usage:
//   reduced_ref res=X,Y,Z bc=f,b,l,r,t,b vorticity=E reduced=DIR/ truth=DIR/
//               steps=N out=PREFIX
//   writes PREFIX.velocity.f64, .density.f64, .heat.f64 (full grids, AoS
//   velocity), PREFIX.qdot.f64 (the last step's reduced coordinates) and
//   PREFIX.errors.f64 (per step: velocity abs, velocity rel, density abs,
//   density rel against the full-rank state files under truth=).
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "SUBSPACE_FLUID_3D_EIGEN.h"

class HeadlessReduced : public SUBSPACE_FLUID_3D_EIGEN {
 public:
  HeadlessReduced(int x, int y, int z, const std::string& path, unsigned int* bcs)
      : SUBSPACE_FLUID_3D_EIGEN(x, y, z, path, bcs, false) {}
  const VectorXd& qDot() const { return _qDot; }
  FIELD_3D& heatField() { return _heat; }
};

static std::vector<double> parse_list(const std::string& s) {
  std::vector<double> v;
  std::stringstream ss(s);
  std::string item;
  while (std::getline(ss, item, ',')) v.push_back(atof(item.c_str()));
  return v;
}

static void write_raw(const std::string& path, const void* data, size_t bytes) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) {
    perror(path.c_str());
    exit(2);
  }
  fwrite(data, 1, bytes, f);
  fclose(f);
}

int main(int argc, char** argv) {
  std::map<std::string, std::string> kv;
  for (int i = 1; i < argc; i++) {
    std::string a(argv[i]);
    size_t eq = a.find('=');
    if (eq == std::string::npos) {
      std::cerr << "bad arg " << a << "\n";
      return 1;
    }
    kv[a.substr(0, eq)] = a.substr(eq + 1);
  }
  std::vector<double> res = parse_list(kv.count("res") ? kv["res"] : "48,64,48");
  std::vector<double> bcl = parse_list(kv.count("bc") ? kv["bc"] : "1,1,1,1,0,0");
  unsigned int bcs[6];
  for (int i = 0; i < 6; i++) bcs[i] = (unsigned int)bcl[i];
  const int steps = kv.count("steps") ? atoi(kv["steps"].c_str()) : 1;
  const std::string out = kv.count("out") ? kv["out"] : "./reduced";

  HeadlessReduced fluid((int)res[0], (int)res[1], (int)res[2], kv["reduced"], bcs);
  fluid.loadReducedRuntimeBases();
  fluid.fullRankPath() = kv["truth"];
  fluid.vorticityEps() = kv.count("vorticity") ? atof(kv["vorticity"].c_str()) : 0.0;
  for (int s = 0; s < steps; s++) {
    fluid.addSmokeColumn();
    fluid.stepReorderedCubatureStam();
  }
  VECTOR3_FIELD_3D& v = fluid.velocity();
  std::vector<double> tmp(3 * (size_t)v.totalCells());
  for (int i = 0; i < v.totalCells(); i++)
    for (int c = 0; c < 3; c++) tmp[3 * i + c] = v[i][c];
  write_raw(out + ".velocity.f64", tmp.data(), tmp.size() * sizeof(double));
  write_raw(out + ".density.f64", fluid.density().data(), (size_t)fluid.density().totalCells() * sizeof(double));
  write_raw(out + ".heat.f64", fluid.heatField().data(), (size_t)fluid.heatField().totalCells() * sizeof(double));
  write_raw(out + ".qdot.f64", fluid.qDot().data(), (size_t)fluid.qDot().size() * sizeof(double));
  std::vector<double> err;
  for (size_t i = 0; i < fluid.velocityErrorAbs().size(); i++) {
    err.push_back(fluid.velocityErrorAbs()[i]);
    err.push_back(fluid.velocityErrorRelative()[i]);
    err.push_back(fluid.densityErrorAbs()[i]);
    err.push_back(fluid.densityErrorRelative()[i]);
  }
  write_raw(out + ".errors.f64", err.data(), err.size() * sizeof(double));
  return 0;
}
