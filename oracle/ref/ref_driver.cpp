// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Headless stand-in for the reference's projects/fluid3D/fluid3D.cpp main and
// runEverytime (fluid3D.cpp:300-398) without GLUT, the window or the movie.
// It drives the reference's own, unmodified FLUID_3D_MIC (compiled from the
// reference sources by oracle/Makefile) so that its outputs can pin the
// oracle restatement and the GPU implementation.
//
// usage:
//   fluid3d_ref run key=value ...     keys: res=X,Y,Z bc=f,b,l,r,t,b vorticity=E
//        buoyancy=B source=column|box|none box=x0,y0,z0,x1,y1,z1 noise=A seed=S
//        steps=N out=DIR/ gz=0|1 streams=0|1 dump=0|1
//     Per step: source, step(), then (optionally) writeGz("DIR/fluid.%04i.fluid3d")
//     and appendStreams() into DIR, as runEverytime does.  dump=1 writes the
//     final state with writeGz to DIR/final.fluid3d.gz.
//     Moving box: moving=1 boxc=cx,cy,cz boxl=lx,ly,lz period=P tperiod=T
//     [initvel=1] builds BOX(boxc, boxl, P, T) with set_dt(0.1); initvel=1
//     calls setInitialVelocity(&box) once; each step then runs
//     stepWithMovingObstacle(&box) in place of step() and afterwards
//     box.spin() and box.translate_center().
//   fluid3d_ref readgz FILE OUTPREFIX
//     Reads FILE with the reference's FLUID_3D_MIC::readGz and writes every
//     field as raw little-endian doubles to OUTPREFIX.<name>.f64 plus
//     OUTPREFIX.header.txt, so that a state file written by the GPU build can
//     be checked against the reference's own reader.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "FLUID_3D_MIC.h"

extern "C" double orc_source_value(uint64_t seed, int32_t step_index, int64_t cell, double noise);

// Gives the driver the protected state that the reference's accessors leave out
// (heat has no accessor in FLUID_3D_MIC.h).
class HeadlessFluid : public FLUID_3D_MIC {
 public:
  HeadlessFluid(int x, int y, int z, unsigned int* bcs) : FLUID_3D_MIC(x, y, z, 4, bcs) {}
  HeadlessFluid() : FLUID_3D_MIC() {}
  FIELD_3D& heatField() { return _heat; }
  FIELD_3D& densityOldField() { return _densityOld; }
  FIELD_3D& heatOldField() { return _heatOld; }
  int totalSteps() const { return _totalSteps; }
  unsigned char* obstacles() { return _obstacles; }
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
  if (!f) { perror(path.c_str()); exit(2); }
  fwrite(data, 1, bytes, f);
  fclose(f);
}

static void dump_vec(const std::string& prefix, const char* name, VECTOR3_FIELD_3D& v) {
  std::vector<double> tmp(3 * (size_t)v.totalCells());
  for (int i = 0; i < v.totalCells(); i++)
    for (int c = 0; c < 3; c++) tmp[3 * i + c] = v[i][c];
  write_raw(prefix + "." + name + ".f64", tmp.data(), tmp.size() * sizeof(double));
}
static void dump_sca(const std::string& prefix, const char* name, FIELD_3D& f) {
  write_raw(prefix + "." + name + ".f64", f.data(), (size_t)f.totalCells() * sizeof(double));
}

int main(int argc, char** argv) {
  if (argc >= 4 && std::string(argv[1]) == "readgz") {
    HeadlessFluid fluid;
    fluid.readGz(argv[2]);
    std::string pre(argv[3]);
    dump_sca(pre, "density", fluid.density());
    dump_sca(pre, "densityOld", fluid.densityOldField());
    dump_sca(pre, "heat", fluid.heatField());
    dump_sca(pre, "heatOld", fluid.heatOldField());
    dump_sca(pre, "pressure", fluid.pressure());
    dump_sca(pre, "divergence", fluid.divergence());
    dump_vec(pre, "velocity", fluid.velocity());
    dump_vec(pre, "velocityOld", fluid.velocityOld());
    dump_vec(pre, "force", fluid.force());
    dump_vec(pre, "vorticity", fluid.vorticity());
    dump_vec(pre, "preprojection", fluid.preprojection());
    dump_vec(pre, "prediffusion", fluid.prediffusion());
    dump_vec(pre, "preadvection", fluid.preadvection());
    dump_vec(pre, "cachedQuadratic", fluid.cachedQuadratic());
    dump_vec(pre, "postadvection", fluid.postadvection());
    dump_sca(pre, "cachedPressure", fluid.cachedPressure());
    dump_sca(pre, "cachedDivergence", fluid.cachedDivergence());
    dump_vec(pre, "prevorticity", fluid.prevorticity());
    write_raw(pre + ".obstacles.u8", fluid.obstacles(), (size_t)fluid.size());
    if (fluid.postIOP().totalCells() > 0) dump_vec(pre, "postIOP", fluid.postIOP());
    SPARSE_MATRIX& n = fluid.neumannIOPMatrix();
    if (n.rows() > 0) {  // the obstacle matrix as (row, col) int pairs and values
      std::vector<int> ij;
      std::vector<double> val;
      for (const auto& e : n.matrix()) {
        ij.push_back(e.first.first);
        ij.push_back(e.first.second);
        val.push_back(e.second);
      }
      write_raw(pre + ".iop_ij.i32", ij.data(), ij.size() * sizeof(int));
      write_raw(pre + ".iop_val.f64", val.data(), val.size() * sizeof(double));
      const int rc[2] = {n.rows(), n.cols()};
      write_raw(pre + ".iop_dims.i32", rc, sizeof(rc));
    }
    FILE* f = fopen((pre + ".header.txt").c_str(), "w");
    fprintf(f, "%d %d %d %d %.17g %.17g %.17g %.17g\n", fluid.xRes(), fluid.yRes(), fluid.zRes(),
            fluid.totalSteps(), fluid.dx(), fluid.dt(), fluid.buoyancy(), fluid.vorticityEps());
    fclose(f);
    return 0;
  }
  if (argc < 2 || std::string(argv[1]) != "run") {
    std::cerr << "usage: fluid3d_ref run key=value ... | readgz FILE OUTPREFIX\n";
    return 1;
  }
  std::map<std::string, std::string> kv;
  for (int i = 2; i < argc; i++) {
    std::string a(argv[i]);
    size_t eq = a.find('=');
    if (eq == std::string::npos) { std::cerr << "bad arg " << a << "\n"; return 1; }
    kv[a.substr(0, eq)] = a.substr(eq + 1);
  }
  std::vector<double> res = parse_list(kv.count("res") ? kv["res"] : "48,64,48");
  std::vector<double> bcl = parse_list(kv.count("bc") ? kv["bc"] : "1,1,1,1,0,0");
  unsigned int bcs[6];
  for (int i = 0; i < 6; i++) bcs[i] = (unsigned int)bcl[i];
  const std::string source = kv.count("source") ? kv["source"] : "column";
  std::vector<double> box = parse_list(kv.count("box") ? kv["box"] : "0,0,0,0,0,0");
  const double noise = kv.count("noise") ? atof(kv["noise"].c_str()) : 0.0;
  const uint64_t seed = kv.count("seed") ? strtoull(kv["seed"].c_str(), NULL, 10) : 0;
  const int steps = kv.count("steps") ? atoi(kv["steps"].c_str()) : 1;
  std::string out = kv.count("out") ? kv["out"] : "./";
  const bool gz = kv.count("gz") && kv["gz"] == "1";
  const bool streams = kv.count("streams") && kv["streams"] == "1";
  const bool dump = kv.count("dump") && kv["dump"] == "1";

  HeadlessFluid fluid((int)res[0], (int)res[1], (int)res[2], bcs);
  // fluid3D.cpp:346: the cfg value replaces the constructor's vorticity.
  fluid.vorticityEps() = kv.count("vorticity") ? atof(kv["vorticity"].c_str()) : 0.0;
  if (kv.count("buoyancy")) fluid.buoyancy() = atof(kv["buoyancy"].c_str());
  fluid.snapshotPath() = out;

  const bool moving = kv.count("moving") && kv["moving"] == "1";
  std::vector<double> bc3 = parse_list(kv.count("boxc") ? kv["boxc"] : "0.5,0.5,0.5");
  std::vector<double> bl3 = parse_list(kv.count("boxl") ? kv["boxl"] : "0.2,0.2,0.2");
  BOX obox(VEC3F(bc3[0], bc3[1], bc3[2]), VEC3F(bl3[0], bl3[1], bl3[2]),
          kv.count("period") ? atof(kv["period"].c_str()) : 4.0,
          kv.count("tperiod") ? atof(kv["tperiod"].c_str()) : 8.0);
  obox.set_dt(0.1);
  if (moving && kv.count("initvel") && kv["initvel"] == "1") fluid.setInitialVelocity(&obox);

  const int X = (int)res[0], Y = (int)res[1];
  for (int step = 0; step < steps; step++) {
    if (source == "column") {
      fluid.addSmokeColumn();
    } else if (source == "box") {
      for (int z = (int)box[2]; z < (int)box[5]; z++)
        for (int y = (int)box[1]; y < (int)box[4]; y++)
          for (int x = (int)box[0]; x < (int)box[3]; x++) {
            const int64_t c = x + (int64_t)y * X + (int64_t)z * X * Y;
            const double val = orc_source_value(seed, step, c, noise);
            fluid.density()[c] = val;
            fluid.heatField()[c] = val;
          }
    }
    if (moving) {
      fluid.stepWithMovingObstacle(&obox);
      obox.spin();
      obox.translate_center();
    } else {
      fluid.step();
    }
    if (gz) {
      char buffer[512];
      snprintf(buffer, sizeof(buffer), "%sfluid.%04i.fluid3d", out.c_str(), step);
      fluid.writeGz(buffer);
    }
    if (streams) fluid.appendStreams();
  }
  if (dump) fluid.writeGz(out + "final.fluid3d.gz");
  return 0;
}
