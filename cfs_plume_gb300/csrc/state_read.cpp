// state_read.cpp -- the reference's state file read back on the host
// (plume_state_read_field) and the error norms of the reduced model's
// ground-truth comparison (plume_peeled_errors).
//
// FLUID_3D_MIC::readGz (FLUID_3D_MIC.cpp:1115-1246) reads, through zlib's
// gzread: 10 int32 (xRes, yRes, zRes, maxRes, xs, ys, zs, totalCells,
// slabSize, totalSteps), 7 doubles, 17 fields in the order of the
// plume_field ids PLUME_F_DENSITY .. PLUME_F_CACHED_DIVERGENCE (each: 3 int32
// dims, center and lengths as 6 doubles, then dims product x 1 or 3 doubles),
// the obstacle bytes (totalCells), center and lengths (6 doubles), an int32
// IOP count, then prevorticity, midMaccormack and postIOP as fields.  The
// reader walks that order and keeps the one field asked for; gzread reads
// the concatenated members of a parallel-deflated file straight through.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/plume.h"
#include "engine.h"
#include "state_read.h"

#ifdef PLUME_HAVE_ZLIB
#include <zlib.h>
#endif

namespace {

int fail(int code, const std::string& msg) {
  plume::global_error() = msg;
  return code;
}

[[maybe_unused]] bool is_vector(int field) {
  switch (field) {
    case PLUME_F_VELOCITY:
    case PLUME_F_VELOCITY_OLD:
    case PLUME_F_FORCE:
    case PLUME_F_VORTICITY:
    case PLUME_F_PREPROJECTION:
    case PLUME_F_PREDIFFUSION:
    case PLUME_F_PREADVECTION:
    case PLUME_F_CACHED_QUADRATIC:
    case PLUME_F_POSTADVECTION:
    case PLUME_F_PREVORTICITY:
    case PLUME_F_POST_IOP:
      return true;
    default:
      return false;
  }
}

#ifdef PLUME_HAVE_ZLIB
// gzread in pieces below 2^31 bytes; false on a short read.
bool read_bytes(gzFile f, void* dst, size_t bytes) {
  char* p = static_cast<char*>(dst);
  while (bytes > 0) {
    const unsigned chunk = (unsigned)std::min<size_t>(bytes, (size_t)1 << 30);
    const int got = gzread(f, p, chunk);
    if (got <= 0 || (unsigned)got != chunk) return false;
    p += chunk;
    bytes -= chunk;
  }
  return true;
}

bool skip_bytes(gzFile f, size_t bytes, std::vector<char>& scratch) {
  while (bytes > 0) {
    const size_t chunk = std::min(bytes, scratch.size());
    if (!read_bytes(f, scratch.data(), chunk)) return false;
    bytes -= chunk;
  }
  return true;
}

// One field record: dims, center, lengths, values.  Keeps the values when
// `dst` is set (n must then equal the record's count), else skips them.
int field_record(gzFile f, bool vec, double* dst, size_t n, bool keep, std::vector<char>& scratch,
                 const std::string& path) {
  int32_t dims[3];
  double geom[6];
  if (!read_bytes(f, dims, sizeof(dims)) || !read_bytes(f, geom, sizeof(geom)))
    return fail(PLUME_ERR_IO, "truncated state file " + path);
  if (dims[0] < 0 || dims[1] < 0 || dims[2] < 0) return fail(PLUME_ERR_IO, "bad field dims in " + path);
  const size_t count = (size_t)dims[0] * (size_t)dims[1] * (size_t)dims[2] * (vec ? 3 : 1);
  if (!keep) {
    if (!skip_bytes(f, count * sizeof(double), scratch)) return fail(PLUME_ERR_IO, "truncated state file " + path);
    return PLUME_OK;
  }
  if (count != n)
    return fail(PLUME_ERR_INVALID, "the field holds " + std::to_string(count) + " values in " + path + ", " +
                                       std::to_string(n) + " requested");
  if (!read_bytes(f, dst, count * sizeof(double))) return fail(PLUME_ERR_IO, "truncated state file " + path);
  return PLUME_OK;
}
#endif

}  // namespace

namespace plume {

int read_state_fields(const std::string& path, const StateRequest& want, int32_t res[3]) {
#ifndef PLUME_HAVE_ZLIB
  (void)path;
  (void)want;
  (void)res;
  return fail(PLUME_ERR_UNSUPPORTED, "built without zlib: state files cannot be read");
#else
  // readGz appends ".gz" unless the name already ends in "gz" (lines 1119-1121)
  std::string fn = path;
  if (fn.size() < 2 || fn[fn.size() - 1] != 'z' || fn[fn.size() - 2] != 'g') fn += ".gz";
  for (const StateField& w : want)
    if (w.field < 0 || w.field >= PLUME_F_COUNT || !w.dst) return fail(PLUME_ERR_INVALID, "bad field request");
  gzFile f = gzopen(fn.c_str(), "rb");
  if (!f) return fail(PLUME_ERR_IO, "could not open " + fn);
  std::vector<char> scratch((size_t)1 << 20);
  int32_t ints[10];
  double consts[7];
  int rc = PLUME_OK;
  if (!read_bytes(f, ints, sizeof(ints)) || !read_bytes(f, consts, sizeof(consts)))
    rc = fail(PLUME_ERR_IO, "truncated state file " + fn);
  if (rc == PLUME_OK && res)
    for (int k = 0; k < 3; k++) res[k] = ints[k];
  // the request for one field id, or null
  auto find = [&](int id) -> const StateField* {
    for (const StateField& w : want)
      if (w.field == id) return &w;
    return nullptr;
  };
  size_t left = want.size();
  auto record = [&](int id, bool vec) {
    const StateField* w = id >= 0 ? find(id) : nullptr;
    rc = field_record(f, vec, w ? w->dst : nullptr, w ? w->n : 0, w != nullptr, scratch, fn);
    if (w) left--;
  };
  // the main block, in plume_field order
  for (int k = PLUME_F_DENSITY; rc == PLUME_OK && left > 0 && k <= PLUME_F_CACHED_DIVERGENCE; k++)
    record(k, is_vector(k));
  if (rc == PLUME_OK && left > 0) {
    // obstacles, center and lengths, the IOP count
    int32_t iop_count = 0;
    if (ints[7] < 0 || !skip_bytes(f, (size_t)ints[7] + 6 * sizeof(double), scratch) ||
        !read_bytes(f, &iop_count, sizeof(iop_count)))
      rc = fail(PLUME_ERR_IO, "truncated state file " + fn);
    // prevorticity, midMaccormack (no plume_field), postIOP
    if (rc == PLUME_OK && left > 0) record(PLUME_F_PREVORTICITY, true);
    if (rc == PLUME_OK && left > 0) record(-1, true);
    if (rc == PLUME_OK && left > 0) record(PLUME_F_POST_IOP, true);
  }
  gzclose(f);
  return rc;
#endif
}

}  // namespace plume

extern "C" {

int plume_state_read_header(const char* path, int32_t ints[10], double consts[7]) {
  if (!path || !ints || !consts) return fail(PLUME_ERR_INVALID, "bad argument");
#ifndef PLUME_HAVE_ZLIB
  return fail(PLUME_ERR_UNSUPPORTED, "built without zlib: state files cannot be read");
#else
  std::string fn = path;
  if (fn.size() < 2 || fn[fn.size() - 1] != 'z' || fn[fn.size() - 2] != 'g') fn += ".gz";
  gzFile f = gzopen(fn.c_str(), "rb");
  if (!f) return fail(PLUME_ERR_IO, "could not open " + fn);
  const bool ok = read_bytes(f, ints, 10 * sizeof(int32_t)) && read_bytes(f, consts, 7 * sizeof(double));
  gzclose(f);
  return ok ? PLUME_OK : fail(PLUME_ERR_IO, "truncated state file " + fn);
#endif
}

int plume_state_read_field(const char* path, int32_t field, double* dst, size_t n, int32_t res[3]) {
  if (!path) return fail(PLUME_ERR_INVALID, "null path");
  if (dst && (field < 0 || field >= PLUME_F_COUNT)) return fail(PLUME_ERR_INVALID, "unknown field");
  plume::StateRequest req;
  if (dst) req.push_back({field, dst, n});
  return plume::read_state_fields(path, req, res);
}

int plume_peeled_errors(const int32_t res[3], const double* velocity, const double* density,
                        const double* truth_velocity, const double* truth_density, double errors[4]) {
  if (!res || !velocity || !density || !truth_velocity || !truth_density || !errors)
    return fail(PLUME_ERR_INVALID, "bad argument");
  const long long X = res[0], Y = res[1], Z = res[2];
  if (X < 3 || Y < 3 || Z < 3) return fail(PLUME_ERR_INVALID, "grid has no interior");
  // peelBoundary().flattenedEigen(): interior cells x fastest, velocity
  // components interleaved; the norms are sqrt of the sums of squares
  double dv = 0, nv = 0, dd = 0, nd = 0;
  for (long long z = 1; z < Z - 1; z++)
    for (long long y = 1; y < Y - 1; y++)
      for (long long x = 1; x < X - 1; x++) {
        const long long i = x + y * X + z * X * Y;
        for (int c = 0; c < 3; c++) {
          const double a = velocity[3 * i + c], d = a - truth_velocity[3 * i + c];
          dv += d * d;
          nv += a * a;
        }
        const double a = density[i], d = a - truth_density[i];
        dd += d * d;
        nd += a * a;
      }
  errors[0] = std::sqrt(dv);
  errors[1] = errors[0] / std::sqrt(nv);
  errors[2] = std::sqrt(dd);
  errors[3] = errors[2] / std::sqrt(nd);
  return PLUME_OK;
}

}  // extern "C"
