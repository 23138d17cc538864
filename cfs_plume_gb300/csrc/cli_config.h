// cli_config.h -- what the stage binaries share: the cfg reader and the
// directory helper of the reference's drivers.
#pragma once
#include <sys/stat.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <string>

namespace plume_cli {

// Config reader with the reference parser's rules (SIMPLE_PARSER.cpp:53-195):
// `key = value` lines of at most 511 characters, '#' comments only at
// column 0, keys lower-cased and trimmed, values trimmed, numbers via atof,
// unknown keys ignored, a non-empty line without '=' is an error.
class Config {
 public:
  bool load(const std::string& path, std::string& err) {
    std::ifstream f(path.c_str());
    if (!f.good()) {
      err = "Failed to open file " + path;
      return false;
    }
    char buffer[512];
    int line_no = 1;
    while (!f.eof()) {
      f.getline(buffer, 512);
      if (f.fail() && !f.eof()) f.clear();  // over-long line: keep the first 511 chars
      std::string line(buffer);
      if (line.empty() || line[0] == '#') continue;
      const size_t pos = line.find('=');
      if (pos != std::string::npos) {
        std::string lhs = trim(line.substr(0, pos));
        const std::string rhs = trim(line.substr(pos + 1));
        for (char& c : lhs) c = (char)tolower((unsigned char)c);
        vals_[lhs] = rhs;
      } else if (!trim(line).empty()) {
        err = "Unable to parse, error in line " + std::to_string(line_no) + ": '" + line + "'";
        return false;
      }
      line_no++;
    }
    return true;
  }
  bool has(const std::string& k) const { return vals_.count(lower(k)) != 0; }
  double num(const std::string& k, double def) const {
    auto it = vals_.find(lower(k));
    return it == vals_.end() ? def : atof(it->second.c_str());
  }
  int integer(const std::string& k, int def) const { return (int)num(k, def); }
  std::string str(const std::string& k, const std::string& def) const {
    auto it = vals_.find(lower(k));
    return it == vals_.end() ? def : it->second;
  }

 private:
  static std::string trim(const std::string& in) {
    size_t s = 0, e = in.size();
    while (s < in.size() && isspace((unsigned char)in[s])) s++;
    while (e > s && isspace((unsigned char)in[e - 1])) e--;
    return in.substr(s, e - s);
  }
  static std::string lower(std::string k) {
    for (char& c : k) c = (char)tolower((unsigned char)c);
    return k;
  }
  std::map<std::string, std::string> vals_;
};

// Algorithmic bytes per interior cell of each stage of the step, for field
// scalars of S bytes (the canonical model: every pass reads its operands and
// writes its results once; stencil neighbours come from cache; the wall
// flags are one byte): forces 4S (k_forces: T and u_y in, u_y out, walls),
// vorticity 18S+2 (curl pass 7S+1, confinement and axpy 11S+1), advection
// 10S, damping 6S, divergence 5S+1, gradient 7S, and the solve
// (5S+2S+2) + iterations (16S+2S+3) with the MIC diagonal stored in S bytes.
struct StageBytes {
  double forces, vorticity, advection, damping, divergence, gradient, solve0, solve_iter;
  explicit StageBytes(int S)
      : forces(4.0 * S), vorticity(18.0 * S + 2), advection(10.0 * S), damping(6.0 * S),
        divergence(5.0 * S + 1), gradient(7.0 * S), solve0(7.0 * S + 2), solve_iter(18.0 * S + 3) {}
};

// One JSON object per step for the `log file` cfg key: the step index and
// every plume_step_stats field (non-finite numbers as null).  With the
// interior cell count n_int and the field scalar size S (4 or 8 bytes), a
// "gbs" object adds each stage's algorithmic GB/s (StageBytes / its ms).
template <typename Stats>
std::string step_json(int step, const Stats& st, double n_int = 0.0, int S = 0) {
  auto num = [](double v) {
    if (!std::isfinite(v)) return std::string("null");
    char b[40];
    snprintf(b, sizeof(b), "%.17g", v);
    return std::string(b);
  };
  std::string s = "{\"step\": " + std::to_string(step);
  s += ", \"iterations\": " + std::to_string(st.iterations);
  s += ", \"converged\": " + std::to_string(st.converged);
  s += ", \"fallback\": " + std::to_string(st.fallback);
  s += ", \"launches\": " + std::to_string(st.launches);
  s += ", \"max_residual\": " + num(st.max_residual);
  s += ", \"rel_residual\": " + num(st.rel_residual);
  s += ", \"rhs_norm\": " + num(st.rhs_norm);
  s += ", \"ms_total\": " + num(st.ms_total);
  s += ", \"ms_solve\": " + num(st.ms_solve);
  s += ", \"ms_forces\": " + num(st.ms_forces);
  s += ", \"ms_vorticity\": " + num(st.ms_vorticity);
  s += ", \"ms_advection\": " + num(st.ms_advection);
  s += ", \"ms_damping\": " + num(st.ms_damping);
  s += ", \"ms_divergence\": " + num(st.ms_divergence);
  s += ", \"ms_guess\": " + num(st.ms_guess);
  s += ", \"ms_gradient\": " + num(st.ms_gradient);
  if (n_int > 0 && S > 0) {
    const StageBytes b(S);
    auto gbs = [&](double per_cell, double ms) {
      return ms > 0 ? num(per_cell * n_int / (ms * 1e6)) : std::string("null");
    };
    s += ", \"gbs\": {\"forces\": " + gbs(b.forces, st.ms_forces);
    s += ", \"vorticity\": " + gbs(b.vorticity, st.ms_vorticity);
    s += ", \"advection\": " + gbs(b.advection, st.ms_advection);
    s += ", \"damping\": " + gbs(b.damping, st.ms_damping);
    s += ", \"divergence\": " + gbs(b.divergence, st.ms_divergence);
    s += ", \"solve\": " + gbs(b.solve0 + st.iterations * b.solve_iter, st.ms_solve);
    s += ", \"gradient\": " + gbs(b.gradient, st.ms_gradient) + "}";
  }
  s += "}";
  return s;
}

// fluid3D.cpp:40-47: create every prefix of the path
inline void ensure_directory(const std::string& path) {
  std::string built;
  for (size_t i = 0; i < path.size(); i++) {
    built += path[i];
    if (path[i] == '/' || i == path.size() - 1) mkdir(built.c_str(), 0755);
  }
}

}  // namespace plume_cli
