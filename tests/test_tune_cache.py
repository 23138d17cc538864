"""The fused batch engine's tuning cache (cfs_plume_gb300/csrc/tune_cache.h),
compiled alone with the host compiler: entries are merged into one JSON
object keyed by batch signature, an entry for the same signature is replaced,
the directories on the way are created, the file is valid JSON, and the
engine's own reader gets back exactly what was written.  No GPU needed."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cfs_plume_gb300", "csrc")

DRIVER = r'''
#include <cstdio>
#include "tune_cache.h"
using namespace plume;
static BatchTuning make(int cells, int vec, int zc, int tz, std::vector<int> bz, std::vector<int> pf) {
  BatchTuning t;
  t.cells_epb = cells; t.vec_epb = vec; t.spmv_zc = zc; t.tile_zc = tz; t.bz = bz; t.pf = pf;
  return t;
}
int main(int argc, char** argv) {
  const std::string path = argv[1];
  if (!write_tune_cache(path, "GB300|sm152|fp32|g2|32x32x32*2", make(4, 8, 32, 4, {6, 5}, {2, 3}))) return 1;
  if (!write_tune_cache(path, "GB300|sm152|fp32|g1|48x64x48*1", make(2, 4, 16, 8, {4}, {3}))) return 2;
  // the same signature again: replaced in place
  if (!write_tune_cache(path, "GB300|sm152|fp32|g2|32x32x32*2", make(4, 2, 32, 4, {6, 5}, {2, 3}))) return 3;
  std::string text;
  if (!read_file(path, text)) return 4;
  for (const auto& e : parse_tune_cache(text)) {
    int a = 0, b = 0, c = 0, d = 0;
    std::vector<int> bz, pf;
    if (!json_int(e.second, "cells_epb", a) || !json_int(e.second, "vec_epb", b) ||
        !json_int(e.second, "spmv_zc", c) || !json_int(e.second, "tile_zc", d) ||
        !json_int_list(e.second, "bz", bz) || !json_int_list(e.second, "pf", pf))
      return 5;
    printf("%s %d %d %d %d", e.first.c_str(), a, b, c, d);
    for (int v : bz) printf(" b%d", v);
    for (int v : pf) printf(" p%d", v);
    printf("\n");
  }
  printf("path %s\n", tune_cache_path(nullptr).c_str());
  printf("given %s\n", tune_cache_path("/x/y.json").c_str());
  return 0;
}
'''


def test_tuning_cache_round_trip(tmp_path):
    gxx = "g++"
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    cache = tmp_path / "a" / "b" / "tune.json"  # directories created on the way
    env = dict(os.environ, PLUME_TUNE_CACHE=str(tmp_path / "env.json"))
    out = subprocess.run([str(exe), str(cache)], capture_output=True, text=True, env=env, check=True).stdout
    lines = out.strip().splitlines()
    assert lines[0] == "GB300|sm152|fp32|g2|32x32x32*2 4 2 32 4 b6 b5 p2 p3"  # replaced, kept first
    assert lines[1] == "GB300|sm152|fp32|g1|48x64x48*1 2 4 16 8 b4 p3"
    assert lines[2] == "path " + str(tmp_path / "env.json")  # $PLUME_TUNE_CACHE when none is given
    assert lines[3] == "given /x/y.json"
    with open(cache) as f:
        entries = json.load(f)  # the file is valid JSON
    assert list(entries) == ["GB300|sm152|fp32|g2|32x32x32*2", "GB300|sm152|fp32|g1|48x64x48*1"]
    assert entries["GB300|sm152|fp32|g2|32x32x32*2"] == {"cells_epb": 4, "vec_epb": 2, "spmv_zc": 32,
                                                        "tile_zc": 4, "bz": [6, 5], "pf": [2, 3]}
    assert not [p for p in os.listdir(cache.parent) if ".tmp" in p]  # written whole, then renamed


CORRUPT_DRIVER = r'''
#include <cstdio>
#include "tune_cache.h"
using namespace plume;
int main(int argc, char** argv) {
  const char* texts[] = {"", "garbage", "{", "{\"sig\"", "{\"sig\": {\"cells_epb\": }}",
                         "{\"sig\": {\"cells_epb\": 4, \"vec_epb\": 2, \"spmv_zc\": 8, \"tile_zc\": 4, \"bz\": [1,"};
  for (const char* t : texts) {
    int usable = 0;
    for (const auto& e : parse_tune_cache(t)) {
      int a = 0, b = 0, c = 0, d = 0;
      std::vector<int> bz, pf;
      if (json_int(e.second, "cells_epb", a) && json_int(e.second, "vec_epb", b) &&
          json_int(e.second, "spmv_zc", c) && json_int(e.second, "tile_zc", d) &&
          json_int_list(e.second, "bz", bz) && json_int_list(e.second, "pf", pf))
        usable++;
    }
    printf("%d\n", usable);
  }
  // a corrupt file is replaced by a valid one holding the new entry
  const std::string path = argv[1];
  FILE* f = fopen(path.c_str(), "wb");
  fputs("{\"old\": {\"cells_epb\": 4, \"bz\": [", f);
  fclose(f);
  BatchTuning t;
  t.bz = {3};
  t.pf = {2};
  return write_tune_cache(path, "NEW|sig", t) ? 0 : 1;
}
'''


def test_tuning_cache_tolerates_corrupt_files(tmp_path):
    """Empty, garbage and truncated cache files yield no usable entry (the
    engine then re-times the batch), and writing over a corrupt file leaves
    valid JSON holding the new entry."""
    src = tmp_path / "corrupt.cpp"
    src.write_text(CORRUPT_DRIVER)
    exe = tmp_path / "corrupt"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    cache = tmp_path / "tune.json"
    out = subprocess.run([str(exe), str(cache)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["0"] * 6
    with open(cache) as f:
        entries = json.load(f)
    assert "NEW|sig" in entries and entries["NEW|sig"]["bz"] == [3]
