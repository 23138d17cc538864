// reduced.cu -- the reduced plume step on the GPU (include/plume_reduced.h).
//
// SUBSPACE_FLUID_3D_EIGEN::stepReorderedCubatureStam with the bases in HBM
// (FP64, column-major: column k of an n-row basis at U + k n):
//   q  = U_pa^T peel(u)                     k_red_project + k_red_reduce
//   q' = sum_points After_p * interp(U_pa q) k_red_cubature + k_red_sum
//   q  = D q'                               k_red_gemv (damping.peeled)
//   q  = P q + G q                          k_red_gemv2 (ptof, inverseProduct)
//   u  = U_f q on the interior              k_red_unproject
// after the engine's full-space stages (buoyancy, vorticity, scalar advection).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/plume.h"
#include "../../include/plume_reduced.h"
#include "engine.h"
#include "matrix_file.cuh"
#include "state_read.h"

namespace plume {
namespace reduced {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRowsPerThread = 8;
constexpr int kRowsPerBlock = kThreads * kRowsPerThread;

__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Peeled row r = 3 c + comp of the interior cell c (x fastest) -> full-grid index
__device__ inline size_t full_index(int X, int Y, int nx, int ny, long long c) {
  const long long x = c % nx, t = c / nx, y = t % ny, z = t / ny;
  return (size_t)(x + 1) + (size_t)(y + 1) * X + (size_t)(z + 1) * (size_t)X * Y;
}

// peeledProject (VECTOR3_FIELD_3D.cpp:3434-3553): partial dots of every
// basis column with the peeled velocity, per block of 2048 rows.
template <typename T>
__global__ void k_red_project(int X, int Y, int Z, const T* vx, const T* vy, const T* vz, const double* U,
                              size_t n, int r, double* partial, int nblk) {
  extern __shared__ double sm[];  // [r][kWarps]
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int nx = X - 2, ny = Y - 2;
  const size_t base = (size_t)blockIdx.x * kRowsPerBlock + threadIdx.x;
  double v[kRowsPerThread];
#pragma unroll
  for (int k = 0; k < kRowsPerThread; k++) {
    const size_t row = base + (size_t)k * kThreads;
    v[k] = 0.0;
    if (row < n) {
      const size_t cell = row / 3;
      const int comp = (int)(row - 3 * cell);
      const size_t i = full_index(X, Y, nx, ny, (long long)cell);
      const T* p = comp == 0 ? vx : (comp == 1 ? vy : vz);
      v[k] = (double)p[i];
    }
  }
  for (int j = 0; j < r; j++) {
    const double* uj = U + (size_t)j * n;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kRowsPerThread; k++) {
      const size_t row = base + (size_t)k * kThreads;
      if (row < n) s = fma(uj[row], v[k], s);
    }
    s = warp_sum(s);
    if (lane == 0) sm[j * kWarps + warp] = s;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < r; j += kThreads) {
    double t = 0.0;
    for (int w = 0; w < kWarps; w++) t += sm[j * kWarps + w];
    partial[(size_t)j * nblk + blockIdx.x] = t;
  }
}

// out[j] = sum over blocks of partial[j][.] in a fixed order, a warp per j
__global__ void k_red_reduce(const double* partial, int nblk, int cnt, double* out) {
  const int j = blockIdx.x * kWarps + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (j >= cnt) return;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += partial[(size_t)j * nblk + b];
  s = warp_sum(s);
  if (lane == 0) out[j] = s;
}

// One cubature point per warp: advectCellStamPeeled (SUBSPACE_FLUID_3D_EIGEN.cpp:
// 1106-1203) -- the cell's velocity from its Before block, the clamped
// backtrace, trilinear interpolation of the eight neighbours' U_pa q -- then
// After_p times that vector (reducedAdvectStagedStamFast, lines 1324-1352).
__global__ void k_red_cubature(const double* Upa, size_t n, int rpa, const double* q, const int* cells,
                               const double* before, const double* after, int rpd, int npts, int X, int Y,
                               int Z, double dt0, double* finals) {
  const int p = blockIdx.x * kWarps + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (p >= npts) return;
  const int nx = X - 2, ny = Y - 2, slab = nx * ny;
  const int index = cells[p];
  const int z = index / slab + 1;
  const int y = (index % slab) / nx + 1;
  const int x = (index % slab) % nx + 1;
  const double* B = before + (size_t)p * 3 * rpa;
  double v3[3];
  for (int c = 0; c < 3; c++) {
    double s = 0.0;
    for (int k = lane; k < rpa; k += 32) s = fma(B[c * rpa + k], q[k], s);
    v3[c] = __shfl_sync(0xffffffffu, warp_sum(s), 0);
  }
  double xt = x - dt0 * v3[0];
  double yt = y - dt0 * v3[1];
  double zt = z - dt0 * v3[2];
  xt = (xt < 1.5) ? 1.5 : xt;
  xt = (xt > X - 2.5) ? X - 2.5 : xt;
  yt = (yt < 1.5) ? 1.5 : yt;
  yt = (yt > Y - 2.5) ? Y - 2.5 : yt;
  zt = (zt < 1.5) ? 1.5 : zt;
  zt = (zt > Z - 2.5) ? Z - 2.5 : zt;
  const int x0 = (int)xt - 1, x1 = x0 + 1;
  const int y0 = (int)yt - 1, y1 = y0 + 1;
  const int z0 = (int)zt - 1, z1 = z0 + 1;
  const double s1 = (xt - 1) - x0, s0 = 1.0 - s1;
  const double t1 = (yt - 1) - y0, t0 = 1.0 - t1;
  const double u1 = (zt - 1) - z0, u0 = 1.0 - u1;
  const int idx[8] = {3 * (x0 + y0 * nx + z0 * slab), 3 * (x0 + y1 * nx + z0 * slab),
                      3 * (x1 + y0 * nx + z0 * slab), 3 * (x1 + y1 * nx + z0 * slab),
                      3 * (x0 + y0 * nx + z1 * slab), 3 * (x0 + y1 * nx + z1 * slab),
                      3 * (x1 + y0 * nx + z1 * slab), 3 * (x1 + y1 * nx + z1 * slab)};
  const double w[8] = {u0 * s0 * t0, u0 * s0 * t1, u0 * s1 * t0, u0 * s1 * t1,
                       u1 * s0 * t0, u1 * s0 * t1, u1 * s1 * t0, u1 * s1 * t1};
  double acc[3] = {0.0, 0.0, 0.0};
  for (int c8 = 0; c8 < 8; c8++)
    for (int c = 0; c < 3; c++) {
      double s = 0.0;
      for (int k = lane; k < rpa; k += 32) s = fma(Upa[(size_t)k * n + idx[c8] + c], q[k], s);
      s = __shfl_sync(0xffffffffu, warp_sum(s), 0);
      acc[c] += w[c8] * s;
    }
  const double* A = after + (size_t)p * rpd * 3;
  for (int k = lane; k < rpd; k += 32)
    finals[(size_t)p * rpd + k] = A[k * 3] * acc[0] + A[k * 3 + 1] * acc[1] + A[k * 3 + 2] * acc[2];
}

// final[k] = sum over points: a warp per k, lane l adding points l, l + 32, ...
// in order, then the warp's tree (a fixed order)
__global__ void k_red_sum(const double* finals, int npts, int rpd, double* out) {
  const int k = blockIdx.x * kWarps + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (k >= rpd) return;
  double s = 0.0;
  for (int p = lane; p < npts; p += 32) s += finals[(size_t)p * rpd + k];
  s = warp_sum(s);
  if (lane == 0) out[k] = s;
}

// y = M x (M rows x cols, row-major), a warp per row; with M2: y = M x + M2 x
__global__ void k_red_gemv2(const double* M, const double* M2, int rows, int cols, const double* x, double* y) {
  const int row = blockIdx.x * kWarps + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (row >= rows) return;
  double a = 0.0, b = 0.0;
  for (int k = lane; k < cols; k += 32) {
    a = fma(M[(size_t)row * cols + k], x[k], a);
    if (M2) b = fma(M2[(size_t)row * cols + k], x[k], b);
  }
  a = warp_sum(a);
  b = warp_sum(b);
  if (lane == 0) y[row] = M2 ? a + b : a;
}

// peeledUnproject (VECTOR3_FIELD_3D.cpp:3558-3605): interior velocity = U_f q
template <typename T>
__global__ void k_red_unproject(int X, int Y, int Z, T* vx, T* vy, T* vz, const double* U, size_t n, int r,
                                const double* q) {
  const int nx = X - 2, ny = Y - 2;
  const long long ncell = (long long)nx * ny * (Z - 2);
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    double s[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < r; k++) {
      const double qk = q[k];
      const double* uk = U + (size_t)k * n + 3 * (size_t)c;
      s[0] = fma(uk[0], qk, s[0]);
      s[1] = fma(uk[1], qk, s[1]);
      s[2] = fma(uk[2], qk, s[2]);
    }
    const size_t i = full_index(X, Y, nx, ny, c);
    vx[i] = (T)s[0];
    vy[i] = (T)s[1];
    vz[i] = (T)s[2];
  }
}

}  // namespace reduced
}  // namespace plume

using namespace plume::reduced;
using namespace plume::matrix_file;

struct plume_reduced {
  plume_handle* h = nullptr;
  int device = 0;
  int X = 0, Y = 0, Z = 0;
  size_t n = 0;  // 3 N_int
  int rpa = 0, rpd = 0, rpp = 0, rf = 0, npts = 0;
  double *Upa = nullptr, *Uf = nullptr, *D = nullptr, *P = nullptr, *G = nullptr;
  double *before = nullptr, *after = nullptr, *finals = nullptr, *partial = nullptr;
  double *q = nullptr, *q2 = nullptr, *q3 = nullptr;
  int* cells = nullptr;
  int nblk = 0;
  double dt0 = 0;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  std::string truth;          // full-rank state files to diff against, or empty
  std::vector<double> errors; // 4 per diffed step
};

namespace {

int fail(int code, const std::string& msg) {
  plume::global_error() = msg;
  return code;
}

// diffGroundTruth (SUBSPACE_FLUID_3D_EIGEN.cpp:804-835), the last call of
// stepReorderedCubatureStam: the full-rank state file of the frame just
// stepped, <path>fluid.%04i.fluid3d.gz with frame = total steps - 1, against
// this step's velocity and density (peeled norms, host side, as in the
// reference).
int diff_ground_truth(plume_reduced* r, plume::Engine* e) {
  const size_t N = (size_t)r->X * r->Y * r->Z;
  char name[64];
  snprintf(name, sizeof(name), "fluid.%04d.fluid3d", (int)e->total_steps() - 1);
  const std::string path = r->truth + name;
  std::vector<double> vel(3 * N), dens(N), tvel(3 * N), tdens(N);
  int rc = e->download(PLUME_F_VELOCITY, vel.data(), vel.size());
  if (rc == PLUME_OK) rc = e->download(PLUME_F_DENSITY, dens.data(), dens.size());
  if (rc != PLUME_OK) return fail(rc, e->last_error());
  int32_t res[3] = {0, 0, 0};
  rc = plume_state_read_field(path.c_str(), PLUME_F_VELOCITY, nullptr, 0, res);
  if (rc != PLUME_OK) return rc;
  if (res[0] != r->X || res[1] != r->Y || res[2] != r->Z)
    return fail(PLUME_ERR_INVALID, "ground truth " + path + " is another grid");
  rc = plume::read_state_fields(path, {{PLUME_F_DENSITY, tdens.data(), tdens.size()},
                                       {PLUME_F_VELOCITY, tvel.data(), tvel.size()}}, nullptr);
  if (rc != PLUME_OK) return rc;
  const int32_t grid[3] = {r->X, r->Y, r->Z};
  double err[4];
  rc = plume_peeled_errors(grid, vel.data(), dens.data(), tvel.data(), tdens.data(), err);
  if (rc != PLUME_OK) return rc;
  r->errors.insert(r->errors.end(), err, err + 4);
  return PLUME_OK;
}

}  // namespace

extern "C" {

void plume_reduced_destroy(plume_reduced* r) {
  if (!r) return;
  cudaSetDevice(r->device);
  for (double* b : {r->Upa, r->Uf, r->D, r->P, r->G, r->before, r->after, r->finals, r->partial, r->q, r->q2, r->q3})
    if (b) cudaFree(b);
  if (r->cells) cudaFree(r->cells);
  for (auto e : r->ev)
    if (e) cudaEventDestroy(e);
  delete r;
}

int plume_reduced_create(plume_handle* h, const char* reduced_path, plume_reduced** out) {
  if (!h || !reduced_path || !out) return fail(PLUME_ERR_INVALID, "bad argument");
  *out = nullptr;
  plume::Engine* e = plume::engine_of(h);
  const plume_params& p = e->params();
  std::unique_ptr<plume_reduced, void (*)(plume_reduced*)> r(new plume_reduced(), plume_reduced_destroy);
  r->h = h;
  r->device = p.device;
  r->X = p.res[0];
  r->Y = p.res[1];
  r->Z = p.res[2];
  const size_t nint = (size_t)(r->X - 2) * (r->Y - 2) * (r->Z - 2);
  r->n = 3 * nint;
  r->dt0 = p.dt / e->dx();  // dt0 = _dt / _dx (SUBSPACE_FLUID_3D_EIGEN.cpp:1329)
  if (cudaSetDevice(p.device) != cudaSuccess) return fail(PLUME_ERR_CUDA, "cudaSetDevice failed");
  const std::string dir = reduced_path;
  std::string err;
  // initOutOfCore (SUBSPACE_FLUID_3D_EIGEN.cpp:82-136): the six projected
  // operators make a built model unless projected.ptof no longer has a row per
  // U.final column; otherwise all six are built (buildOutOfCoreMatrices).
  {
    bool built = true;
    int rr = 0, cc = 0;
    for (const char* f : {"projected.A.matrix", "projected.ptof.matrix", "projected.vtod.matrix",
                          "damping.peeled.matrix", "projected.ptov.matrix", "inverseProduct.matrix"}) {
      FILE* t = fopen((dir + f).c_str(), "rb");
      if (!t) built = false;
      if (t) fclose(t);
    }
    int ur = 0, uc = 0;
    if (built && read_matrix_dims(dir + "U.final.matrix", ur, uc) && read_matrix_dims(dir + "projected.ptof.matrix", rr, cc) &&
        rr != uc)
      built = false;
    if (!built) {
      const int brc = plume_reduced_build_products(h, reduced_path, nullptr);
      if (brc != PLUME_OK) return brc;
    }
  }
  int rc = upload_basis(dir + "U.preadvect.matrix", r->n, r->Upa, r->rpa, err);
  if (rc == PLUME_OK) rc = upload_basis(dir + "U.final.matrix", r->n, r->Uf, r->rf, err);
  if (rc != PLUME_OK) return fail(rc, err);
  // the projected operators the step uses
  int dr = 0, dc = 0, pr = 0, pc = 0, gr = 0, gc = 0;
  std::vector<double> hd, hp, hg;
  if (!read_matrix(dir + "damping.peeled.matrix", dr, dc, hd) ||
      !read_matrix(dir + "projected.ptof.matrix", pr, pc, hp) ||
      !read_matrix(dir + "inverseProduct.matrix", gr, gc, hg))
    return fail(PLUME_ERR_IO, "missing projected operators under " + dir +
                                  " (damping.peeled, projected.ptof, inverseProduct)");
  // cubature points and weights (readAdvectionCubature, lines 1208-1245)
  std::vector<int> cells;
  std::vector<double> weights;
  {
    FILE* f = fopen((dir + "cubature").c_str(), "rb");
    if (!f) return fail(PLUME_ERR_IO, "no cubature file under " + dir);
    int size = 0;
    bool ok = fread(&size, sizeof(int), 1, f) == 1 && size > 0;
    if (ok) {
      cells.resize(size);
      weights.resize(size);
      ok = fread(cells.data(), sizeof(int), size, f) == (size_t)size &&
           fread(weights.data(), sizeof(double), size, f) == (size_t)size;
    }
    fclose(f);
    if (!ok) return fail(PLUME_ERR_IO, "bad cubature file under " + dir);
    for (int c : cells)
      if (c < 0 || (size_t)c >= nint) return fail(PLUME_ERR_IO, "cubature cell outside the grid");
  }
  r->npts = (int)cells.size();
  // the advection cubature cache: read it, or build it from U.preadvect and
  // U.prediffuse and write it (lines 1247-1318)
  std::vector<double> before, after;
  const std::string cache = dir + "advection.cubature.cache";
  FILE* cf = fopen(cache.c_str(), "rb");
  if (cf) {
    std::vector<double> m;
    int rows = 0, cols = 0;
    bool ok = true;
    for (int x = 0; ok && x < r->npts; x++) {
      ok = read_matrix_file(cf, rows, cols, m) && rows == 3 && cols == r->rpa;
      before.insert(before.end(), m.begin(), m.end());
    }
    for (int x = 0; ok && x < r->npts; x++) {
      ok = read_matrix_file(cf, rows, cols, m) && cols == 3 && (x == 0 || rows == r->rpd);
      r->rpd = rows;
      after.insert(after.end(), m.begin(), m.end());
    }
    fclose(cf);
    if (!ok) return fail(PLUME_ERR_IO, "advection cubature cache does not match the bases: " + cache);
  } else {
    int ar = 0, ac = 0, dr2 = 0, dc2 = 0;
    std::vector<double> ua, ud;
    if (!read_matrix(dir + "U.preadvect.matrix", ar, ac, ua) || !read_matrix(dir + "U.prediffuse.matrix", dr2, dc2, ud) ||
        (size_t)dr2 != r->n)
      return fail(PLUME_ERR_IO, "cannot build the cubature cache: U.prediffuse.matrix missing or mismatched");
    r->rpd = dc2;
    for (int x = 0; x < r->npts; x++)  // cellBasisPeeled (lines 860-879): rows 3 i .. 3 i + 2
      before.insert(before.end(), ua.begin() + (size_t)3 * cells[x] * ac, ua.begin() + (size_t)(3 * cells[x] + 3) * ac);
    for (int x = 0; x < r->npts; x++)  // weight * cellU^T
      for (int k = 0; k < dc2; k++)
        for (int c = 0; c < 3; c++) after.push_back(weights[x] * ud[(size_t)(3 * cells[x] + c) * dc2 + k]);
    FILE* wf = fopen(cache.c_str(), "wb");
    if (!wf) return fail(PLUME_ERR_IO, "could not write " + cache);
    bool ok = true;
    for (int x = 0; ok && x < r->npts; x++) ok = write_matrix_file(wf, 3, r->rpa, &before[(size_t)x * 3 * r->rpa]);
    for (int x = 0; ok && x < r->npts; x++) ok = write_matrix_file(wf, r->rpd, 3, &after[(size_t)x * 3 * r->rpd]);
    if (fclose(wf) != 0 || !ok) return fail(PLUME_ERR_IO, "write failed: " + cache);
  }
  r->rpp = dr;
  if (dc != r->rpd || pr != r->rf || gr != r->rf || pc != r->rpp || gc != r->rpp)
    return fail(PLUME_ERR_INVALID, "reduced operator ranks do not chain: damping " + std::to_string(dr) + "x" +
                                       std::to_string(dc) + ", ptof " + std::to_string(pr) + "x" +
                                       std::to_string(pc) + ", inverseProduct " + std::to_string(gr) + "x" +
                                       std::to_string(gc));
  r->nblk = (int)((r->n + kRowsPerBlock - 1) / kRowsPerBlock);
  const int maxr = std::max(std::max(r->rpa, r->rpd), std::max(r->rpp, r->rf));
  if (upload(r->D, hd) != cudaSuccess || upload(r->P, hp) != cudaSuccess || upload(r->G, hg) != cudaSuccess ||
      upload(r->before, before) != cudaSuccess || upload(r->after, after) != cudaSuccess ||
      upload(r->cells, cells) != cudaSuccess ||
      cudaMalloc(&r->finals, (size_t)r->npts * std::max(1, r->rpd) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&r->partial, (size_t)std::max(1, r->rpa) * r->nblk * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&r->q, std::max(1, maxr) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&r->q2, std::max(1, maxr) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&r->q3, std::max(1, maxr) * sizeof(double)) != cudaSuccess ||
      cudaEventCreate(&r->ev[0]) != cudaSuccess || cudaEventCreate(&r->ev[1]) != cudaSuccess ||
      cudaEventCreate(&r->ev[2]) != cudaSuccess)
    return fail(PLUME_ERR_OOM, "reduced model does not fit on the device");
  if ((size_t)r->rpa * kWarps * sizeof(double) > 48 * 1024 &&
      cudaFuncSetAttribute(k_red_project<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(r->rpa * kWarps * sizeof(double))) != cudaSuccess)
    return fail(PLUME_ERR_UNSUPPORTED, "U.preadvect has too many columns");
  if ((size_t)r->rpa * kWarps * sizeof(double) > 48 * 1024)
    cudaFuncSetAttribute(k_red_project<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(r->rpa * kWarps * sizeof(double)));
  *out = r.release();
  return PLUME_OK;
}

int plume_reduced_step(plume_reduced* r, plume_step_stats* stats) {
  if (!r) return fail(PLUME_ERR_INVALID, "null model");
  plume::Engine* e = plume::engine_of(r->h);
  cudaStream_t s = (cudaStream_t)e->stream_handle();
  cudaEventRecord(r->ev[2], s);
  int rc = e->reduced_prestep();
  if (rc != PLUME_OK) return fail(rc, e->last_error());
  const void* planes[3] = {nullptr, nullptr, nullptr};
  if (!e->device_vector(PLUME_F_VELOCITY, planes)) return fail(PLUME_ERR_STATE, "no velocity field");
  const bool fp32 = e->params().precision == PLUME_PREC_FP32;
  int launches = e->reduced_launches();
  cudaEventRecord(r->ev[0], s);
  // q = U_pa^T peel(u)
  const size_t smem = (size_t)r->rpa * kWarps * sizeof(double);
  if (fp32)
    k_red_project<float><<<r->nblk, kThreads, smem, s>>>(r->X, r->Y, r->Z, (const float*)planes[0],
                                                         (const float*)planes[1], (const float*)planes[2], r->Upa,
                                                         r->n, r->rpa, r->partial, r->nblk);
  else
    k_red_project<double><<<r->nblk, kThreads, smem, s>>>(r->X, r->Y, r->Z, (const double*)planes[0],
                                                          (const double*)planes[1], (const double*)planes[2],
                                                          r->Upa, r->n, r->rpa, r->partial, r->nblk);
  k_red_reduce<<<(r->rpa + kWarps - 1) / kWarps, kThreads, 0, s>>>(r->partial, r->nblk, r->rpa, r->q);
  // cubature advection into the prediffuse basis
  k_red_cubature<<<(r->npts + kWarps - 1) / kWarps, kThreads, 0, s>>>(r->Upa, r->n, r->rpa, r->q, r->cells,
                                                                       r->before, r->after, r->rpd, r->npts, r->X,
                                                                       r->Y, r->Z, r->dt0, r->finals);
  k_red_sum<<<(r->rpd + kWarps - 1) / kWarps, kThreads, 0, s>>>(r->finals, r->npts, r->rpd, r->q2);
  // reducedPeeledDiffusion (lines 606-612): q = D q
  k_red_gemv2<<<(r->rpp + kWarps - 1) / kWarps, kThreads, 0, s>>>(r->D, nullptr, r->rpp, r->rpd, r->q2, r->q);
  // reducedStagedProject (lines 700-707): q = ptof q + inverseProduct q
  k_red_gemv2<<<(r->rf + kWarps - 1) / kWarps, kThreads, 0, s>>>(r->P, r->G, r->rf, r->rpp, r->q, r->q3);
  // the interior velocity from the final basis
  const long long ncell = (long long)(r->n / 3);
  const int ug = (int)std::min<long long>((ncell + kThreads - 1) / kThreads, 152 * 16);
  if (fp32)
    k_red_unproject<float><<<ug, kThreads, 0, s>>>(r->X, r->Y, r->Z, (float*)planes[0], (float*)planes[1],
                                                   (float*)planes[2], r->Uf, r->n, r->rf, r->q3);
  else
    k_red_unproject<double><<<ug, kThreads, 0, s>>>(r->X, r->Y, r->Z, (double*)planes[0], (double*)planes[1],
                                                    (double*)planes[2], r->Uf, r->n, r->rf, r->q3);
  launches += 7;
  if (cudaGetLastError() != cudaSuccess) return fail(PLUME_ERR_CUDA, "reduced step launch failed");
  cudaEventRecord(r->ev[1], s);
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    if (cudaEventSynchronize(r->ev[1]) != cudaSuccess) return fail(PLUME_ERR_CUDA, "reduced step failed");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r->ev[0], r->ev[1]);
    stats->launches = launches;
    stats->converged = 1;
    stats->ms_solve = ms;  // the reduced part (projection through unprojection)
    cudaEventElapsedTime(&ms, r->ev[2], r->ev[1]);
    stats->ms_total = ms;
  }
  if (!r->truth.empty()) return diff_ground_truth(r, e);
  return PLUME_OK;
}

int plume_reduced_set_ground_truth(plume_reduced* r, const char* full_rank_path) {
  if (!r) return fail(PLUME_ERR_INVALID, "null model");
  r->truth = full_rank_path ? full_rank_path : "";
  return PLUME_OK;
}

int plume_reduced_errors(plume_reduced* r, double* out, int32_t n, int32_t* count) {
  if (!r || !count) return fail(PLUME_ERR_INVALID, "bad argument");
  *count = (int32_t)(r->errors.size() / 4);
  if (out && n > 0)
    std::copy(r->errors.begin(), r->errors.begin() + std::min<size_t>((size_t)n / 4 * 4, r->errors.size()), out);
  return PLUME_OK;
}

int plume_reduced_qdot(plume_reduced* r, double* q, int32_t n, int32_t* size) {
  if (!r) return fail(PLUME_ERR_INVALID, "null model");
  if (size) *size = r->rf;
  if (!q) return PLUME_OK;
  if (n < r->rf) return fail(PLUME_ERR_INVALID, "buffer too small");
  plume::Engine* e = plume::engine_of(r->h);
  cudaStream_t s = (cudaStream_t)e->stream_handle();
  if (cudaMemcpyAsync(q, r->q3, r->rf * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return fail(PLUME_ERR_CUDA, "download failed");
  return PLUME_OK;
}

int plume_reduced_dims(plume_reduced* r, int32_t dims[5]) {
  if (!r || !dims) return fail(PLUME_ERR_INVALID, "bad argument");
  dims[0] = r->rpa;
  dims[1] = r->rpd;
  dims[2] = r->rpp;
  dims[3] = r->rf;
  dims[4] = r->npts;
  return PLUME_OK;
}

}  // extern "C"
