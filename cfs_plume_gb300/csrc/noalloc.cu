// noalloc.cu -- MIC(0) preconditioner apply that allocates no device memory.
//
// Who needs it: a caller that runs its own Krylov loop on the GPU and only
// wants this library's lexicographic MIC(0) preconditioner, but cannot call
// cudaMalloc at the point of use -- for example because the call sits inside a
// region that is being captured into a CUDA graph, or because a host framework
// owns the device memory budget and forbids allocations outside its own pool.
// Such a caller passes its inputs and its output buffer; the work vectors this
// computation needs live in one file-scope device array, sized below.
//
// Built without multiply-add contraction (like the FP64 engine), so the result
// is bit-identical to plume_mic_apply on an FP64 handle.
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/plume.h"
#include "../../include/plume_noalloc.h"
#include "engine.cuh"

namespace plume {
namespace {

// Scratch: four skewed FP64 vectors (diagonal, r, forward result, z) of at
// most PLUME_NOALLOC_MAX_ELEMS values each, the solver state word block, the
// slab ticket and one progress word per plane.  Every GPU that loads the
// library holds this array until the process exits.
constexpr size_t kVecBytes = (size_t)PLUME_NOALLOC_MAX_ELEMS * sizeof(double);
constexpr size_t kStateOff = 4 * kVecBytes;
constexpr size_t kCtlOff = kStateOff + 256;
constexpr size_t kProgOff = kCtlOff + 256;
constexpr size_t kScratchBytes = kProgOff + (size_t)PLUME_NOALLOC_MAX_PLANES * sizeof(int);
static_assert(sizeof(CgState) <= 256, "CgState must fit its scratch slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the array, looked up once per device with that device
// current (in host code the symbol itself is only a host-side stand-in).
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

int scratch_address(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices) return PLUME_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      (void)cudaGetLastError();
      return PLUME_ERR_CUDA;
    }
    g_addr[dev] = p;
  }
  *out = (unsigned char*)g_addr[dev];
  return PLUME_OK;
}

// skewed result -> natural interior; if a wavefront wait expired the output
// is not valid, so every cell (border included) is set to NaN instead
__global__ void k_from_skew_checked(Grid g, Skew k, const double* sk, const CgState* st, double* nat) {
  const bool bad = st->wave_err != 0;
  if (bad) {
    PL_GRID_STRIDE(e, g.N) nat[e] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  PL_GRID_STRIDE(e, (int)k.total) {
    int ix, iy, iz;
    if (skew_cell(k, e, ix, iy, iz)) nat[(ix + 1) + (iy + 1) * g.X + (iz + 1) * g.slab] = sk[e];
  }
}

}  // namespace
}  // namespace plume

extern "C" int plume_mic_apply_noalloc(const int32_t res[3], const int32_t bc[6],
                                       const double* precon, const double* r, double* z,
                                       void* stream) {
  using namespace plume;
  if (!res || !bc || !precon || !r || !z) return PLUME_ERR_INVALID;
  for (int k = 0; k < 3; k++)
    if (res[k] < 4) return PLUME_ERR_INVALID;
  for (int k = 0; k < 6; k++)
    if (bc[k] != 0 && bc[k] != 1) return PLUME_ERR_INVALID;
  {
    // the fixed scratch bounds the grid: reject rather than overrun it (sizes
    // in 64 bits, before any of the int geometry below is formed)
    const long long nx = (long long)res[0] - 2, ny = (long long)res[1] - 2, nz = (long long)res[2] - 2;
    const long long C = (nx + 31) / 32;
    if (C > 8) return PLUME_ERR_INVALID;  // x resolution above 258 cells
    if (nz > PLUME_NOALLOC_MAX_PLANES) return PLUME_ERR_INVALID;
    const long long row = 32 * C, rows = ny + 31;
    if (rows > (long long)PLUME_NOALLOC_MAX_ELEMS / row ||
        nz * rows * row > (long long)PLUME_NOALLOC_MAX_ELEMS)
      return PLUME_ERR_INVALID;
  }
  Grid g;
  g.X = res[0];
  g.Y = res[1];
  g.Z = res[2];
  g.slab = g.X * g.Y;
  g.N = g.X * g.Y * g.Z;
  g.nx = g.X - 2;
  g.ny = g.Y - 2;
  g.nz = g.Z - 2;
  g.nint = g.nx * g.ny * g.nz;
  for (int k = 0; k < 6; k++) g.wall[k] = bc[k];
  Skew k;
  k.nx = g.nx;
  k.ny = g.ny;
  k.nz = g.nz;
  k.C = (g.nx + 31) / 32;
  k.W = 32 * k.C;
  k.R = g.ny + 31;
  k.plane = (long long)k.R * k.W;
  k.total = (long long)g.nz * k.plane;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return PLUME_ERR_CUDA;
  }
  unsigned char* base = nullptr;
  int rc = scratch_address(dev, &base);
  if (rc != PLUME_OK) return rc;
  double* sP = (double*)base;
  double* sr = (double*)(base + kVecBytes);
  double* sq = (double*)(base + 2 * kVecBytes);
  double* sz = (double*)(base + 3 * kVecBytes);
  CgState* st = (CgState*)(base + kStateOff);
  unsigned* ctl = (unsigned*)(base + kCtlOff);
  int* progress = (int*)(base + kProgOff);
  cudaStream_t s = (cudaStream_t)stream;

  // the array keeps the previous call's contents: clear what must start at 0
  if (cudaMemsetAsync(base + kStateOff, 0, kScratchBytes - kStateOff, s) != cudaSuccess)
    return PLUME_ERR_CUDA;
  const int gK = grid_for(k.total);
  k_to_skew<double, double><<<gK, 256, 0, s>>>(g, k, precon, sP);
  k_to_skew<double, double><<<gK, 256, 0, s>>>(g, k, r, sr);

  // slab configuration, chosen as the allocating path chooses it
  WaveArgs<double> a;
  a.P = sP;
  a.k = k;
  a.K = 8;
  a.ctl = ctl;
  a.progress = progress;
  a.st = st;
  // Test hook of the sweeps' bounded waits: PLUME_NOALLOC_WAIT_GATE=<polls>
  // makes each sweep CTA first poll ctl[3] (cleared above, never set) that
  // many times before it issues any copy; the wait expires and z comes back
  // NaN.  Unset in normal use.
  if (const char* gate = getenv("PLUME_NOALLOC_WAIT_GATE")) {
    const long long polls = atoll(gate);
    if (polls > 0) {
      a.gate = (const int*)(ctl + 3);
      a.gate_spins = polls;
    }
  }
  bool cluster = false;
  int bz = (g.nz + 15) / 16;
  if (bz < 4) bz = 4;
  if ((g.nz + bz - 1) / bz <= 16 && wave_smem_bytes<double>(bz, k.W) <= 227 * 1024) {
    WaveArgs<double> q = a;
    q.in = sr;
    q.out = sq;
    q.backward = 0;
    q.BZ = bz;
    q.nslabs = (g.nz + bz - 1) / bz;
    int maxc = 0;
    if (launch_wave_cl<double, true>(q, wave_smem_bytes<double>(bz, k.W), s, 1, &maxc) == cudaSuccess &&
        maxc >= 1)
      cluster = true;
    (void)cudaGetLastError();
  }
  int grid = 1;
  if (!cluster) {
    bz = 8;
    while (bz > 1 && wave_smem_bytes<double>(bz, k.W) > 200 * 1024) bz /= 2;
    int sms = 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 1;
    grid = (g.nz + bz - 1) / bz;
    if (grid > 2 * sms) grid = 2 * sms;
  }
  a.BZ = bz;
  a.nslabs = (g.nz + bz - 1) / bz;
  const size_t smem = wave_smem_bytes<double>(bz, k.W);
  cudaError_t e;
  a.in = sr;
  a.out = sq;
  a.backward = 0;
  e = cluster ? launch_wave_cl<double, true>(a, smem, s) : launch_wave<double, true>(a, grid, smem, s);
  if (e != cudaSuccess) return PLUME_ERR_CUDA;
  a.in = sq;
  a.out = sz;
  a.backward = 1;
  e = cluster ? launch_wave_cl<double, true>(a, smem, s) : launch_wave<double, true>(a, grid, smem, s);
  if (e != cudaSuccess) return PLUME_ERR_CUDA;
  // output: interior from the skewed result, zero on the border
  if (cudaMemsetAsync(z, 0, (size_t)g.N * sizeof(double), s) != cudaSuccess) return PLUME_ERR_CUDA;
  k_from_skew_checked<<<grid_for(k.total > g.N ? k.total : g.N), 256, 0, s>>>(g, k, sz, st, z);
  if (cudaGetLastError() != cudaSuccess) return PLUME_ERR_CUDA;
  return PLUME_OK;
}
