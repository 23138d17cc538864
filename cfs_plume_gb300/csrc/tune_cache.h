// tune_cache.h -- the fused batch engine's tile shapes and their JSON cache
// (host code only: batched.cuh uses it, and the CPU tests compile it alone).
#pragma once
#include <cstdio>
#include <cstdlib>
#include <string>
#include <utility>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

namespace plume {

// Tile shapes of a batch.  cells_epb: elements per thread of the stencil and
// layout kernels; vec_epb: 16-byte groups per thread of the CG vector
// reductions; spmv_zc: planes per tile of the marching SpMV; tile_zc: planes
// per tile of the 2.5D neighbour stencils; per sweep class, bz: planes per
// CTA (slab height) and pf: TMA ring depth in 8-row blocks (2 takes a third
// less shared memory than 3, so more CTAs of the batch's clusters share an
// SM).
struct BatchTuning {
  int cells_epb = 2;
  int vec_epb = 4;
  int spmv_zc = 32;
  int tile_zc = 16;
  std::vector<int> bz, pf;
  bool from_cache = false;
  bool timed = false;
};

// The tuning cache: one JSON object whose keys are batch signatures and whose
// values are {"cells_epb": a, "vec_epb": b, "spmv_zc": c, "tile_zc": d,
// "bz": [..], "pf": [..]}.  The reader accepts exactly what the writer
// produces.
inline std::string tune_cache_path(const char* given) {
  if (given && *given) return given;
  if (const char* e = getenv("PLUME_TUNE_CACHE")) {
    if (*e) return e;
  }
  const char* home = getenv("HOME");
  if (!home || !*home) return std::string();
  return std::string(home) + "/.cache/cfs_plume_gb300/tune.json";
}

inline bool read_file(const std::string& path, std::string& out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  char buf[4096];
  size_t r;
  out.clear();
  while ((r = fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, r);
  fclose(f);
  return true;
}

// entries of the cache as (signature, value text) pairs, in file order
inline std::vector<std::pair<std::string, std::string>> parse_tune_cache(const std::string& text) {
  std::vector<std::pair<std::string, std::string>> out;
  size_t i = text.find('{');
  if (i == std::string::npos) return out;
  ++i;
  for (;;) {
    const size_t q0 = text.find('"', i);
    if (q0 == std::string::npos) break;
    const size_t q1 = text.find('"', q0 + 1);
    if (q1 == std::string::npos) break;
    const size_t b0 = text.find('{', q1);
    if (b0 == std::string::npos) break;
    const size_t b1 = text.find('}', b0);
    if (b1 == std::string::npos) break;
    out.emplace_back(text.substr(q0 + 1, q1 - q0 - 1), text.substr(b0, b1 - b0 + 1));
    i = b1 + 1;
  }
  return out;
}

inline bool json_int(const std::string& obj, const char* key, int& v) {
  const std::string k = std::string("\"") + key + "\"";
  const size_t p = obj.find(k);
  if (p == std::string::npos) return false;
  const size_t c = obj.find(':', p + k.size());
  if (c == std::string::npos) return false;
  char* end = nullptr;
  const long x = strtol(obj.c_str() + c + 1, &end, 10);
  if (end == obj.c_str() + c + 1) return false;
  v = (int)x;
  return true;
}

inline bool json_int_list(const std::string& obj, const char* key, std::vector<int>& v) {
  const std::string k = std::string("\"") + key + "\"";
  const size_t p = obj.find(k);
  if (p == std::string::npos) return false;
  const size_t a = obj.find('[', p);
  const size_t b = obj.find(']', a == std::string::npos ? p : a);
  if (a == std::string::npos || b == std::string::npos) return false;
  v.clear();
  const char* s = obj.c_str() + a + 1;
  const char* e = obj.c_str() + b;
  while (s < e) {
    char* end = nullptr;
    const long x = strtol(s, &end, 10);
    if (end == s) {
      ++s;
      continue;
    }
    v.push_back((int)x);
    s = end;
  }
  return true;
}

inline std::string tuning_value_json(const BatchTuning& t) {
  std::string s = "{\"cells_epb\": " + std::to_string(t.cells_epb) + ", \"vec_epb\": " +
                  std::to_string(t.vec_epb) + ", \"spmv_zc\": " + std::to_string(t.spmv_zc) +
                  ", \"tile_zc\": " + std::to_string(t.tile_zc) + ", \"bz\": [";
  for (size_t i = 0; i < t.bz.size(); i++) s += (i ? ", " : "") + std::to_string(t.bz[i]);
  s += "], \"pf\": [";
  for (size_t i = 0; i < t.pf.size(); i++) s += (i ? ", " : "") + std::to_string(t.pf[i]);
  return s + "]}";
}

// Merge one entry into the cache file (written whole to a temporary file,
// then renamed over the old one).
inline bool write_tune_cache(const std::string& path, const std::string& sig, const BatchTuning& t) {
  if (path.empty()) return false;
  std::string text;
  std::vector<std::pair<std::string, std::string>> entries;
  if (read_file(path, text)) entries = parse_tune_cache(text);
  bool found = false;
  for (auto& e : entries)
    if (e.first == sig) {
      e.second = tuning_value_json(t);
      found = true;
    }
  if (!found) entries.emplace_back(sig, tuning_value_json(t));
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos && slash > 0) {  // the directories on the way (EEXIST is fine)
    const std::string dir = path.substr(0, slash);
    for (size_t p = 1; p <= dir.size(); p++)
      if (p == dir.size() || dir[p] == '/') mkdir(dir.substr(0, p).c_str(), 0755);
  }
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) return false;
  fprintf(f, "{\n");
  for (size_t i = 0; i < entries.size(); i++)
    fprintf(f, "  \"%s\": %s%s\n", entries[i].first.c_str(), entries[i].second.c_str(),
            i + 1 < entries.size() ? "," : "");
  fprintf(f, "}\n");
  const bool ok = fclose(f) == 0;
  if (!ok || rename(tmp.c_str(), path.c_str()) != 0) {
    remove(tmp.c_str());
    return false;
  }
  return true;
}

}  // namespace plume
