// snapshot.cpp -- reference-format state files and SVD streams (host C++).
#include "snapshot.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>

#include "../../include/plume.h"

#if defined(PLUME_HAVE_ZLIB)
#include <zlib.h>
#endif

namespace plume {

namespace {

// gzip output.  With zlib: the byte stream is cut into 16 MB pieces, each
// deflated at level 1 (the reference's "wb1") into a complete gzip member by a
// pool of host threads, and the members are written in order; concatenated
// members are one valid gzip file, which zlib's gzread (the reference's
// readGz) reads straight through.  Without zlib headers at build time: one
// gzip member of stored (uncompressed) deflate blocks.
class GzOut {
 public:
  bool open(const std::string& path) {
    f_ = fopen(path.c_str(), "wb");
    if (!f_) return false;
#if defined(PLUME_HAVE_ZLIB)
    pieces_.clear();
    pieces_.emplace_back();
    pieces_.back().reserve(kPiece);
#else
    static const unsigned char hdr[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 3};
    fwrite(hdr, 1, 10, f_);
    crc_ = 0xffffffffu;
    size_ = 0;
#endif
    return true;
  }
  bool write(const void* data, size_t n) {
    const unsigned char* p = (const unsigned char*)data;
#if defined(PLUME_HAVE_ZLIB)
    while (n > 0) {
      std::vector<unsigned char>& cur = pieces_.back();
      const size_t take = std::min(n, kPiece - cur.size());
      cur.insert(cur.end(), p, p + take);
      p += take;
      n -= take;
      if (cur.size() == kPiece) {
        pieces_.emplace_back();
        pieces_.back().reserve(kPiece);
      }
    }
    return true;
#else
    while (n > 0) {
      const size_t chunk = n > 65535 ? 65535 : n;
      const unsigned char b[5] = {0, (unsigned char)(chunk & 0xff), (unsigned char)(chunk >> 8),
                                  (unsigned char)(~chunk & 0xff),
                                  (unsigned char)((~chunk >> 8) & 0xff)};
      if (fwrite(b, 1, 5, f_) != 5 || fwrite(p, 1, chunk, f_) != chunk) return false;
      update_crc(p, chunk);
      size_ += chunk;
      p += chunk;
      n -= chunk;
    }
    return true;
#endif
  }
  bool close() {
#if defined(PLUME_HAVE_ZLIB)
    if (pieces_.back().empty() && pieces_.size() > 1) pieces_.pop_back();
    const size_t np = pieces_.size();
    std::vector<std::vector<unsigned char>> out(np);
    std::atomic<size_t> next(0);
    std::atomic<bool> ok(true);
    auto work = [&]() {
      for (size_t k = next++; k < np; k = next++) {
        if (!deflate_member(pieces_[k], out[k])) ok = false;
        std::vector<unsigned char>().swap(pieces_[k]);  // release the raw piece early
      }
    };
    unsigned hw = std::thread::hardware_concurrency();
    if (const char* env = getenv("PLUME_GZ_THREADS")) {  // deflate threads (default: all cores, <= 32)
      const int t = atoi(env);
      if (t >= 1) hw = (unsigned)t;
    }
    const size_t nt = std::min<size_t>(np, std::max(1u, std::min(hw, 32u)));
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    bool wrote = ok.load();
    for (size_t k = 0; k < np && wrote; k++)
      wrote = fwrite(out[k].data(), 1, out[k].size(), f_) == out[k].size();
    pieces_.clear();
    return (fclose(f_) == 0) && wrote;
#else
    const unsigned char last[5] = {1, 0, 0, 0xff, 0xff};  // final empty stored block
    fwrite(last, 1, 5, f_);
    const uint32_t crc = crc_ ^ 0xffffffffu;
    unsigned char tail[8];
    for (int k = 0; k < 4; k++) tail[k] = (unsigned char)(crc >> (8 * k));
    for (int k = 0; k < 4; k++) tail[4 + k] = (unsigned char)((uint32_t)size_ >> (8 * k));
    fwrite(tail, 1, 8, f_);
    return fclose(f_) == 0;
#endif
  }

 private:
  FILE* f_ = nullptr;
#if defined(PLUME_HAVE_ZLIB)
  static constexpr size_t kPiece = (size_t)16 << 20;
  std::vector<std::vector<unsigned char>> pieces_;

  // one complete gzip member (header, level-1 deflate stream, CRC-32, size)
  static bool deflate_member(const std::vector<unsigned char>& in, std::vector<unsigned char>& out) {
    z_stream z;
    memset(&z, 0, sizeof(z));
    if (deflateInit2(&z, 1, Z_DEFLATED, 15 + 16, 8, Z_DEFAULT_STRATEGY) != Z_OK) return false;
    out.resize(deflateBound(&z, (uLong)in.size()) + 64);
    z.next_in = const_cast<Bytef*>(in.data());
    z.avail_in = (uInt)in.size();
    z.next_out = out.data();
    z.avail_out = (uInt)out.size();
    const int rc = deflate(&z, Z_FINISH);
    out.resize(z.total_out);
    deflateEnd(&z);
    return rc == Z_STREAM_END;
  }
#else
  void update_crc(const unsigned char* p, size_t n) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
      for (uint32_t i = 0; i < 256; i++) {
        uint32_t c = i;
        for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        table[i] = c;
      }
      init = true;
    }
    uint32_t c = crc_;
    for (size_t i = 0; i < n; i++) c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    crc_ = c;
  }
  uint32_t crc_ = 0;
  uint64_t size_ = 0;
#endif
};

template <typename V>
bool put(GzOut& g, const V& v) {
  return g.write(&v, sizeof(V));
}

// FIELD_3D::writeGz / VECTOR3_FIELD_3D::writeGz (FIELD_3D.cpp:5993-6014,
// VECTOR3_FIELD_3D.cpp:1327-1346): 3 ints, center, lengths, doubles.
bool put_field(GzOut& g, const int res[3], const double center[3], const double lengths[3],
               const std::vector<double>& data) {
  bool ok = put(g, res[0]) && put(g, res[1]) && put(g, res[2]);
  for (int k = 0; k < 3; k++) ok = ok && put(g, center[k]);
  for (int k = 0; k < 3; k++) ok = ok && put(g, lengths[k]);
  return ok && g.write(data.data(), data.size() * sizeof(double));
}

}  // namespace

// SPARSE_MATRIX::write / writeGz (SPARSE_MATRIX.cpp:508-561) of the obstacle
// matrix: rows, cols, entry count, then (row, col, value) in (row, col)
// order.  Row i of an interior cell holds (i, i) = 1 outside the box, 0
// inside, and inside also (i, last) = the box velocity component.  Bytes go
// to `sink` in pieces of about 1 MB.
static bool put_iop_matrix(const int res[3], const IopRecord& iop,
                    const std::function<bool(const void*, size_t)>& sink) {
  const int X = res[0], Y = res[1], Z = res[2];
  const int rows = 3 * (X - 2) * (Y - 2) * (Z - 2), cols = rows + 1;
  int inside = 0;
  for (int z = 1; z < Z - 1; z++)
    for (int y = 1; y < Y - 1; y++)
      for (int x = 1; x < X - 1; x++) inside += iop.inside[x + (size_t)y * X + (size_t)z * X * Y] ? 1 : 0;
  const int total = rows + 3 * inside;
  const int head[3] = {rows, cols, total};
  if (!sink(head, sizeof(head))) return false;
  std::vector<unsigned char> buf;
  buf.reserve((1 << 20) + 64);
  auto entry = [&](int r, int c, double v) {
    unsigned char e[16];
    memcpy(e, &r, 4);
    memcpy(e + 4, &c, 4);
    memcpy(e + 8, &v, 8);
    buf.insert(buf.end(), e, e + 16);
  };
  int row = 0;
  for (int z = 1; z < Z - 1; z++)
    for (int y = 1; y < Y - 1; y++)
      for (int x = 1; x < X - 1; x++) {
        const size_t c = x + (size_t)y * X + (size_t)z * X * Y;
        for (int i = 0; i < 3; i++, row++) {
          if (iop.inside[c]) {
            entry(row, row, 0.0);
            entry(row, cols - 1, iop.values[3 * c + i]);
          } else {
            entry(row, row, 1.0);
          }
        }
        if (buf.size() >= (1u << 20)) {
          if (!sink(buf.data(), buf.size())) return false;
          buf.clear();
        }
      }
  return buf.empty() || sink(buf.data(), buf.size());
}

int write_state_gz(const std::string& path_in, const StateHeader& h, const FieldFetch& fetch,
                   const std::vector<uint8_t>& obstacles, const IopRecord& iop, std::string& err) {
  std::string path = path_in;
  const size_t n = path.size();
  if (n < 2 || path[n - 1] != 'z' || path[n - 2] != 'g') path += ".gz";  // line 1025-1027
  GzOut g;
  if (!g.open(path)) {
    err = "could not open " + path;
    return PLUME_ERR_IO;
  }
  const int X = h.res[0], Y = h.res[1], Z = h.res[2];
  int maxRes = X > Y ? X : Y;
  maxRes = Z > maxRes ? Z : maxRes;
  const int ints[10] = {X, Y, Z, maxRes, 1, X, X * Y, X * Y * Z, X * Y, h.total_steps};
  const double dbls[7] = {h.dx, h.total_time, h.dt, h.buoyancy, h.vorticity_eps, 1e-3, 1e-10};
  bool ok = g.write(ints, sizeof(ints)) && g.write(dbls, sizeof(dbls));
  const double center[3] = {0, 0, 0};
  const double lengths[3] = {h.dx * X, h.dx * Y, h.dx * Z};  // FLUID_3D_MIC.cpp:56
  std::vector<double> buf;
  // fields in the order of lines 1057-1076
  const int order[] = {PLUME_F_DENSITY,       PLUME_F_DENSITY_OLD,      PLUME_F_HEAT,
                       PLUME_F_HEAT_OLD,      PLUME_F_PRESSURE,         PLUME_F_DIVERGENCE,
                       PLUME_F_VELOCITY,      PLUME_F_VELOCITY_OLD,     PLUME_F_FORCE,
                       PLUME_F_VORTICITY,     PLUME_F_PREPROJECTION,    PLUME_F_PREDIFFUSION,
                       PLUME_F_PREADVECTION,  PLUME_F_CACHED_QUADRATIC, PLUME_F_POSTADVECTION,
                       PLUME_F_CACHED_PRESSURE, PLUME_F_CACHED_DIVERGENCE};
  for (int f : order) {
    if (!ok) break;
    int rc = fetch(f, buf);
    if (rc != PLUME_OK) {
      g.close();
      err = "field download failed while writing " + path;
      return rc;
    }
    ok = put_field(g, h.res, center, lengths, buf);
  }
  // obstacles, center, lengths, IOP count (lines 1078-1091)
  ok = ok && g.write(obstacles.data(), obstacles.size());
  for (int k = 0; k < 3; k++) ok = ok && put(g, center[k]);
  for (int k = 0; k < 3; k++) ok = ok && put(g, lengths[k]);
  const int howMany = 0;
  ok = ok && put(g, howMany);
  // prevorticity, then the never-assigned midMaccormack and postIOP fields
  // (default-constructed: zero dims, zero center and lengths, no data)
  if (ok) {
    int rc = fetch(PLUME_F_PREVORTICITY, buf);
    if (rc != PLUME_OK) {
      g.close();
      err = "field download failed while writing " + path;
      return rc;
    }
    ok = put_field(g, h.res, center, lengths, buf);
  }
  const int zres[3] = {0, 0, 0};
  const double zero3[3] = {0, 0, 0};
  const std::vector<double> empty;
  ok = ok && put_field(g, zres, zero3, zero3, empty);  // midMaccormack
  // postIOP (lines 1101-1102): empty until the first moving-box step
  if (ok) {
    int rc = fetch(PLUME_F_POST_IOP, buf);
    if (rc != PLUME_OK) {
      g.close();
      err = "field download failed while writing " + path;
      return rc;
    }
    ok = buf.empty() ? put_field(g, zres, zero3, zero3, empty) : put_field(g, h.res, center, lengths, buf);
  }
  // the obstacle matrix, only once it has rows (lines 1104-1105)
  if (ok && !iop.inside.empty())
    ok = put_iop_matrix(h.res, iop, [&](const void* d, size_t n) { return g.write(d, n); });
  const bool closed = g.close();
  if (!ok || !closed) {
    err = "write failed: " + path;
    return PLUME_ERR_IO;
  }
  return PLUME_OK;
}

namespace {

// peelBoundary + flattened (VECTOR3_FIELD_3D.cpp:3139-3151, 3222-3232;
// FIELD_3D.cpp:6679-6689, 6722-6733): interior cells, x fastest.
void peel(const int res[3], const std::vector<double>& full, int comps, std::vector<double>& out) {
  const int X = res[0], Y = res[1], Z = res[2];
  out.resize((size_t)comps * (X - 2) * (Y - 2) * (Z - 2));
  size_t o = 0;
  for (int z = 1; z < Z - 1; z++)
    for (int y = 1; y < Y - 1; y++)
      for (int x = 1; x < X - 1; x++) {
        const size_t c = (size_t)x + (size_t)y * X + (size_t)z * X * Y;
        for (int k = 0; k < comps; k++) out[o++] = full[comps * c + k];
      }
}

// VECTOR::norm2 on Linux: sqrt of the serial dot (VECTOR.cpp:426-437).
double norm2(const std::vector<double>& v) {
  double s = 0;
  for (double x : v) s += x * x;
  return sqrt(s);
}

}  // namespace

int append_streams(const std::string& dir, const int res[3], const FieldFetch& fetch,
                   const IopRecord& iop, std::string& err) {
  static const char* dims_names[6] = {"velocity.final.matrix.dims", "velocity.preproject.matrix.dims",
                                      "velocity.prediffuse.matrix.dims",
                                      "velocity.preadvect.matrix.dims", "velocity.iop.matrix.dims",
                                      "pressure.matrix.dims"};
  int rows[6] = {0, 0, 0, 0, 0, 0}, cols[6] = {0, 0, 0, 0, 0, 0};
  for (int k = 0; k < 6; k++) {  // lines 1347-1361
    FILE* f = fopen((dir + dims_names[k]).c_str(), "rb");
    if (!f) continue;
    int r = 0, c = 0;
    if (fread(&r, sizeof(int), 1, f) == 1 && fread(&c, sizeof(int), 1, f) == 1) {
      rows[k] = r;
      cols[k] = c;
    }
    fclose(f);
  }
  const int nint = (res[0] - 2) * (res[1] - 2) * (res[2] - 2);
  for (int k = 0; k < 5; k++)
    if (cols[k] == 0) cols[k] = 3 * nint;
  if (cols[5] == 0) cols[5] = nint;

  struct Row {
    const char* file;
    int field;
    int comps;
    int dims_slot;
  };
  // lines 1402-1461: four velocity streams, the postIOP stream once a
  // moving-box step has run (the IOP stream is created in any case), then
  // pressure and divergence rows into the same pressure stream.  The
  // reference never closes its IOP stream's FILE (opened at line 1385, left
  // out of the fclose list at 1458-1463), so stdio's buffered tail of each
  // row reaches its file only at process exit, after later rows; here every
  // row is appended whole, in step order.
  const bool using_iop = !iop.inside.empty();  // line 1378: _neumannIOP.rows() > 0
  std::vector<Row> rows_to_write = {
      {"velocity.final.matrix.transpose", PLUME_F_VELOCITY, 3, 0},
      {"velocity.preproject.matrix.transpose", PLUME_F_PREPROJECTION, 3, 1},
      {"velocity.prediffuse.matrix.transpose", PLUME_F_PREDIFFUSION, 3, 2},
      {"velocity.preadvect.matrix.transpose", PLUME_F_PREADVECTION, 3, 3},
  };
  if (using_iop) rows_to_write.push_back({"velocity.iop.matrix.transpose", PLUME_F_POST_IOP, 3, 4});
  rows_to_write.push_back({"pressure.matrix.transpose", PLUME_F_PRESSURE, 1, 5});
  rows_to_write.push_back({"pressure.matrix.transpose", PLUME_F_DIVERGENCE, 1, 5});
  {
    FILE* iop = fopen((dir + "velocity.iop.matrix.transpose").c_str(), "ab");
    if (!iop) {
      err = "could not open streams under " + dir;
      return PLUME_ERR_IO;
    }
    fclose(iop);
  }
  std::vector<double> full, peeled;
  for (const Row& r : rows_to_write) {
    int rc = fetch(r.field, full);
    if (rc != PLUME_OK) {
      err = "field download failed while appending streams";
      return rc;
    }
    peel(res, full, r.comps, peeled);
    FILE* f = fopen((dir + r.file).c_str(), "ab");
    if (!f) {
      err = std::string("could not open ") + dir + r.file;
      return PLUME_ERR_IO;
    }
    bool ok = true;
    if (norm2(peeled) > 1e-7) {
      ok = fwrite(peeled.data(), sizeof(double), peeled.size(), f) == peeled.size();
      rows[r.dims_slot]++;
    }
    if (fclose(f) != 0 || !ok) {
      err = std::string("write failed: ") + dir + r.file;
      return PLUME_ERR_IO;
    }
  }
  if (using_iop) {  // lines 1455-1456: the matrix itself, uncompressed
    FILE* f = fopen((dir + "neumann.iop.matrices").c_str(), "ab");
    if (!f) {
      err = "could not open " + dir + "neumann.iop.matrices";
      return PLUME_ERR_IO;
    }
    const bool ok = put_iop_matrix(res, iop, [&](const void* d, size_t n) { return fwrite(d, 1, n, f) == n; });
    if (fclose(f) != 0 || !ok) {
      err = "write failed: " + dir + "neumann.iop.matrices";
      return PLUME_ERR_IO;
    }
  }
  for (int k = 0; k < 6; k++) {  // lines 1465-1474
    FILE* f = fopen((dir + dims_names[k]).c_str(), "wb");
    if (!f) {
      err = std::string("could not write ") + dir + dims_names[k];
      return PLUME_ERR_IO;
    }
    const bool ok = fwrite(&rows[k], sizeof(int), 1, f) == 1 && fwrite(&cols[k], sizeof(int), 1, f) == 1;
    if (fclose(f) != 0 || !ok) {
      err = std::string("write failed: ") + dir + dims_names[k];
      return PLUME_ERR_IO;
    }
  }
  return PLUME_OK;
}

}  // namespace plume
