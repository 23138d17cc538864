// engine.cuh -- Engine<T>: device state and step orchestration for one plume.
//
// Included by engine_f64.cu (T = double, no multiply-add contraction) and
// engine_f32.cu (T = float).  The step follows FLUID_3D_MIC::step
// (FLUID_3D_MIC.cpp:179-223) stage for stage; the cached copies the reference
// keeps for the reduced solvers are produced as extra kernel outputs or by
// pointer rotation instead of separate full-array copies.
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"
#include "engine.h"
#include "skew_kernels.cuh"
#include "unet.h"
#include "solver_kernels.cuh"
#include "step_kernels.cuh"
#include "tile_kernels.cuh"
#include "wave.cuh"

namespace plume {

#define PL_TRY(expr)                                                          \
  do {                                                                        \
    cudaError_t e_ = (expr);                                                  \
    if (e_ != cudaSuccess) return fail_cuda(e_, #expr, __FILE__, __LINE__);   \
  } while (0)
#define PL_CHECK_LAUNCH() \
  do {                    \
    ++launches_;          \
    PL_TRY(cudaGetLastError()); \
  } while (0)

// NVTX range around the host code that enqueues one stage of the step, named
// after the reference's TIMER bucket for it (src/util/TIMER.cpp:33-149 keys
// its buckets by function name, FLUID_3D_MIC.cpp:316-1253); a profiler maps
// the kernels launched inside onto the range.  No cost without a tool.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

inline int grid_for(long long n, int threads = 256, int cap = 152 * 32) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

// Column source cells of FLUID_3D_MIC::addSmokeTestCase (FLUID_3D_MIC.cpp:
// 674-700), evaluated with the reference's float sqrtf and float literals.
inline std::vector<int> column_cells(int X, int Y, int Z) {
  std::vector<int> cells;
  int maxRes = X;
  if (Y > maxRes) maxRes = Y;
  if (Z > maxRes) maxRes = Z;
  const double dx = 1.0f / (double)maxRes;
  const double xTotal = dx * X, zTotal = dx * Z;
  const double heighMin = 0.05, heighMax = 0.10;
  for (int z = 0; z < Z; z++)
    for (int y = (int)(heighMin * Y); y <= (int)(heighMax * Y); y++)
      for (int x = 0; x < X; x++) {
        const double xLength = x * dx - xTotal * 0.4f;
        const double zLength = z * dx - zTotal * 0.5f;
        const double radius = sqrtf((float)(xLength * xLength + zLength * zLength));
        if (radius < 0.075f * xTotal) cells.push_back(x + y * X + z * X * Y);
      }
  return cells;
}

// Field download into host memory the GPU can address (pageable memory on a
// system with coherent host access): dst[o], o = cell * ncomp + component, in
// FP64 (the reference's AoS layout); consecutive threads write consecutive
// doubles.
template <typename T>
__global__ void k_planes_to_host(const T* a, const T* b, const T* c, int ncomp, long long N, double* dst) {
  const long long n = N * ncomp;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n;
       o += (long long)gridDim.x * blockDim.x) {
    const long long cell = ncomp == 1 ? o : o / 3;
    const int comp = ncomp == 1 ? 0 : (int)(o - cell * 3);
    const T* src = comp == 0 ? a : (comp == 1 ? b : c);
    dst[o] = (double)src[cell];
  }
}

// Runs `set` (a kernel's cudaFuncSetAttribute calls) once per device: the
// attributes belong to the current device, so a flag per process would leave
// a second GPU without them.  `done` holds one bit per device ordinal below
// 64 (higher ordinals set the attributes on every launch); threads that race
// on a device's first launch may both set them, which is harmless.
template <typename F>
inline cudaError_t once_per_device(std::atomic<unsigned long long>& done, F&& set) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = set();
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

// The same for a vector field, two cells per thread: the 6 doubles of a cell
// pair are 48 contiguous bytes, written as three 16-byte stores (dst 16-byte
// aligned); an odd last cell is written by one thread.
template <typename T>
__global__ void k_vec_to_host2(const T* a, const T* b, const T* c, long long N, double* dst) {
  const long long np = N / 2;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np;
       p += (long long)gridDim.x * blockDim.x) {
    const long long c0 = 2 * p;
    double2* o = reinterpret_cast<double2*>(dst + 6 * p);
    o[0] = make_double2((double)a[c0], (double)b[c0]);
    o[1] = make_double2((double)c[c0], (double)a[c0 + 1]);
    o[2] = make_double2((double)b[c0 + 1], (double)c[c0 + 1]);
  }
  if ((N & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const long long l = N - 1;
    dst[3 * l] = (double)a[l];
    dst[3 * l + 1] = (double)b[l];
    dst[3 * l + 2] = (double)c[l];
  }
}

template <typename T, int C, bool EXACT>
cudaError_t launch_wave_c(const WaveArgs<T>& a, int grid, size_t smem, cudaStream_t s) {
  void (*kf)(WaveArgs<T>) = a.backward ? k_mic_wave<T, C, EXACT, true> : k_mic_wave<T, C, EXACT, false>;
  static std::atomic<unsigned long long> attr_done[2];
  cudaError_t ea = once_per_device(attr_done[a.backward ? 1 : 0], [&] {
    return cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  });
  if (ea != cudaSuccess) return ea;
  // launched as explicit one-CTA clusters: the ring hand-off uses
  // shared::cluster forms (st.async, cluster-scope barrier waits)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(32 * (a.BZ + 2), 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 1;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kf, a);
}

template <typename T, int C, bool EXACT>
cudaError_t launch_wave_cl_c(const WaveArgs<T>& a, size_t smem, cudaStream_t s, int query,
                             int* max_clusters) {
  void (*kf)(WaveArgs<T>) =
      a.backward ? k_mic_wave_cl<T, C, EXACT, true> : k_mic_wave_cl<T, C, EXACT, false>;
  static std::atomic<unsigned long long> attr_done[2];
  cudaError_t ea = once_per_device(attr_done[a.backward ? 1 : 0], [&] {
    cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kf, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
  });
  if (ea != cudaSuccess) return ea;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nslabs, 1, 1);
  cfg.blockDim = dim3(32 * a.BZ, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = a.nslabs;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (query) return cudaOccupancyMaxActiveClusters(max_clusters, (void*)kf, &cfg);
  return cudaLaunchKernelEx(&cfg, kf, a);
}

// Cluster wavefront (one cluster holds every slab of the plume); query != 0
// only asks how many such clusters fit on the device.
template <typename T, bool EXACT>
cudaError_t launch_wave_cl(const WaveArgs<T>& a, size_t smem, cudaStream_t s, int query = 0,
                           int* max_clusters = nullptr) {
  switch (a.k.C) {
    case 1: return launch_wave_cl_c<T, 1, EXACT>(a, smem, s, query, max_clusters);
    case 2: return launch_wave_cl_c<T, 2, EXACT>(a, smem, s, query, max_clusters);
    case 3: return launch_wave_cl_c<T, 3, EXACT>(a, smem, s, query, max_clusters);
    case 4: return launch_wave_cl_c<T, 4, EXACT>(a, smem, s, query, max_clusters);
    case 5: return launch_wave_cl_c<T, 5, EXACT>(a, smem, s, query, max_clusters);
    case 6: return launch_wave_cl_c<T, 6, EXACT>(a, smem, s, query, max_clusters);
    case 7: return launch_wave_cl_c<T, 7, EXACT>(a, smem, s, query, max_clusters);
    case 8: return launch_wave_cl_c<T, 8, EXACT>(a, smem, s, query, max_clusters);
    default: return cudaErrorInvalidValue;
  }
}

// MIC sweep dispatch on the cells-per-lane count C (1..8: up to 256 cells per row).
template <typename T, bool EXACT>
cudaError_t launch_wave(const WaveArgs<T>& a, int grid, size_t smem, cudaStream_t s) {
  switch (a.k.C) {
    case 1: return launch_wave_c<T, 1, EXACT>(a, grid, smem, s);
    case 2: return launch_wave_c<T, 2, EXACT>(a, grid, smem, s);
    case 3: return launch_wave_c<T, 3, EXACT>(a, grid, smem, s);
    case 4: return launch_wave_c<T, 4, EXACT>(a, grid, smem, s);
    case 5: return launch_wave_c<T, 5, EXACT>(a, grid, smem, s);
    case 6: return launch_wave_c<T, 6, EXACT>(a, grid, smem, s);
    case 7: return launch_wave_c<T, 7, EXACT>(a, grid, smem, s);
    case 8: return launch_wave_c<T, 8, EXACT>(a, grid, smem, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
class EngineT : public Engine {
 public:
  EngineT() {}
  ~EngineT() override { release(); }

  // ------------------------------------------------------------------ init
  int init(const plume_params& p) override {
    p_ = p;
    for (int k = 0; k < 3; k++)
      if (p.res[k] < 4) return fail(PLUME_ERR_INVALID, "every grid dimension must be >= 4");
    const long long N = (long long)p.res[0] * p.res[1] * p.res[2];
    if (N > (1ll << 30)) return fail(PLUME_ERR_INVALID, "grid larger than 2^30 cells");
    for (int k = 0; k < 6; k++)
      if (p.bc[k] != 0 && p.bc[k] != 1) return fail(PLUME_ERR_INVALID, "bc flags must be 0 or 1");
    if (p.criterion != PLUME_CRIT_REFERENCE && p.criterion != PLUME_CRIT_REL2)
      return fail(PLUME_ERR_INVALID, "unknown criterion");
    if (p.source == PLUME_SRC_BOX)
      for (int k = 0; k < 3; k++)
        if (p.box_lo[k] < 0 || p.box_hi[k] > p.res[k] || p.box_lo[k] > p.box_hi[k])
          return fail(PLUME_ERR_INVALID, "source box outside the grid");
    if (p.warm_start != PLUME_WARM_ZERO && p.warm_start != PLUME_WARM_PREVIOUS &&
        p.warm_start != PLUME_WARM_LEARNED)
      return fail(PLUME_ERR_INVALID, "unknown warm start");
    if (p.preconditioner != PLUME_PRECOND_MIC && p.preconditioner != PLUME_PRECOND_NET)
      return fail(PLUME_ERR_INVALID, "unknown preconditioner");
    g_.X = p.res[0];
    g_.Y = p.res[1];
    g_.Z = p.res[2];
    g_.slab = g_.X * g_.Y;
    g_.N = (int)N;
    g_.nx = g_.X - 2;
    g_.ny = g_.Y - 2;
    g_.nz = g_.Z - 2;
    g_.nint = g_.nx * g_.ny * g_.nz;
    for (int k = 0; k < 6; k++) g_.wall[k] = p.bc[k];
    int maxRes = g_.X > g_.Y ? g_.X : g_.Y;
    maxRes = g_.Z > maxRes ? g_.Z : maxRes;
    dx_ = 1.0f / (double)maxRes;  // FLUID_3D_MIC.cpp:46
    set_consts();

    PL_TRY(cudaSetDevice(p.device));
    {  // the GPU writes downloads straight into the caller's (pageable) buffer
       // when it can access host memory coherently (Grace + Blackwell over C2C)
      int pageable = 0;
      if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, p.device) != cudaSuccess)
        pageable = 0;
      const char* off = getenv("PLUME_NO_HOST_DIRECT");
      host_direct_ = pageable == 1 && !(off && atoi(off) != 0);
      (void)cudaGetLastError();
    }
    PL_TRY(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
    for (auto* e : {&ev_[0], &ev_[1], &ev_[2], &ev_[3]}) PL_TRY(cudaEventCreate(e));
    for (auto& e : evs_) PL_TRY(cudaEventCreate(&e));

    // one pool: 13 scalar planes + 8 vector fields (24 planes) of T, the FP64
    // MIC diagonal, the obstacle bytes, solver state and reduction partials.
    const size_t n = (size_t)g_.N;
    const size_t aT = align(n * sizeof(T));
    const size_t bytes = 36 * aT + align(n * sizeof(double)) + align(n) +
                         align(sizeof(CgState)) + align(8 * kRedBlocks * sizeof(double));
    cudaError_t e = cudaMalloc(&pool_, bytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(PLUME_ERR_OOM, "device allocation of the field pool failed");
    }
    PL_TRY(cudaMemsetAsync(pool_, 0, bytes, s_));
    char* cur = pool_;
    auto take = [&](size_t b) { char* r = cur; cur += align(b); return r; };
    T** scal[] = {&dens_, &dens_old_, &heat_, &heat_old_, &pres_, &div_, &mag_,
                  &r_,    &d_,        &q_ad_, &z_,        &qf_};
    for (T** s : scal) *s = (T*)take(n * sizeof(T));
    V3<T>* vecs[] = {&vel_, &vel_old_, &spare_, &prevort_, &postadv_, &preproj_, &force_, &vort_};
    for (V3<T>* v : vecs) {
      v->x = (T*)take(n * sizeof(T));
      v->y = (T*)take(n * sizeof(T));
      v->z = (T*)take(n * sizeof(T));
    }
    P64_ = (double*)take(n * sizeof(double));
    obst_ = (uint8_t*)take(n);
    st_ = (CgState*)take(sizeof(CgState));
    part_ = (double*)take(8 * kRedBlocks * sizeof(double));

    // obstacle slabs (FLUID_3D_MIC.cpp:105-159), kept for download and the
    // state file; kernels derive walls from the flags.
    std::vector<uint8_t> ob(n, 0);
    for (int z = 0; z < g_.Z; z++)
      for (int y = 0; y < g_.Y; y++)
        for (int x = 0; x < g_.X; x++) {
          const bool w = (z == 0 && p.bc[0] == 1) || (z == g_.Z - 1 && p.bc[1] == 1) ||
                         (y == 0 && p.bc[5] == 1) || (y == g_.Y - 1 && p.bc[4] == 1) ||
                         (x == 0 && p.bc[2] == 1) || (x == g_.X - 1 && p.bc[3] == 1);
          ob[x + y * g_.X + z * g_.slab] = w ? 1 : 0;
        }
    PL_TRY(cudaMemcpyAsync(obst_, ob.data(), n, cudaMemcpyHostToDevice, s_));

    if (p.source == PLUME_SRC_COLUMN) {
      std::vector<int> cells = column_cells(g_.X, g_.Y, g_.Z);
      n_col_ = (int)cells.size();
      if (n_col_ > 0) {
        PL_TRY(cudaMalloc(&col_cells_, cells.size() * sizeof(int)));
        PL_TRY(cudaMemcpyAsync(col_cells_, cells.data(), cells.size() * sizeof(int),
                               cudaMemcpyHostToDevice, s_));
      }
    }
    PL_TRY(cudaMallocHost(&st_host_, sizeof(CgState)));
    PL_TRY(cudaMallocHost(&stage_, n * 3 * sizeof(double)));

    // MIC(0) diagonal, built once: the reference rebuilds an identical one at
    // every solve (FLUID_3D_MIC.cpp:921-922) since the walls never change.
    PL_TRY(build_mic_diagonal(g_, P64_, p.mic_tau, p.mic_sigma, s_));
    int rc = init_solver();
    if (rc != PLUME_OK) return rc;
    PL_TRY(cudaStreamSynchronize(s_));
    return PLUME_OK;
  }

  // --------------------------------------------------------------- sources
  int add_source(int32_t step_index) override {
    if (p_.source == PLUME_SRC_COLUMN && n_col_ > 0) {
      k_source_list<T><<<grid_for(n_col_), 256, 0, s_>>>(dens_, heat_, col_cells_, n_col_);
      PL_CHECK_LAUNCH();
    } else if (p_.source == PLUME_SRC_BOX) {
      const int bx = p_.box_hi[0] - p_.box_lo[0], by = p_.box_hi[1] - p_.box_lo[1],
                bz = p_.box_hi[2] - p_.box_lo[2];
      if (bx > 0 && by > 0 && bz > 0) {
        k_source_box<T><<<grid_for((long long)bx * by * bz), 256, 0, s_>>>(
            dens_, heat_, g_, p_.box_lo[0], p_.box_lo[1], p_.box_lo[2], bx, by, bz, p_.seed,
            step_index, p_.source_noise);
        PL_CHECK_LAUNCH();
      }
    }
    return PLUME_OK;
  }

  int add_source_values(const double* values, size_t n) override {
    if (p_.source != PLUME_SRC_BOX) return fail(PLUME_ERR_STATE, "source values need a box source");
    const int bx = p_.box_hi[0] - p_.box_lo[0], by = p_.box_hi[1] - p_.box_lo[1],
              bz = p_.box_hi[2] - p_.box_lo[2];
    const size_t nb = (size_t)bx * by * bz;
    if (!values || n != nb) return fail(PLUME_ERR_INVALID, "values must cover the source box");
    if (nb == 0) return PLUME_OK;
    if (src_dev_ == nullptr) {
      PL_TRY(cudaMalloc(&src_dev_, nb * sizeof(T)));
      PL_TRY(cudaMallocHost(&src_host_, nb * sizeof(T)));
    }
    PL_TRY(cudaStreamSynchronize(s_));  // src_host_ may still feed a previous copy
    for (size_t k = 0; k < nb; k++) src_host_[k] = (T)values[k];
    PL_TRY(cudaMemcpyAsync(src_dev_, src_host_, nb * sizeof(T), cudaMemcpyHostToDevice, s_));
    k_source_box_values<T><<<grid_for((long long)nb), 256, 0, s_>>>(
        dens_, heat_, g_, p_.box_lo[0], p_.box_lo[1], p_.box_lo[2], bx, by, bz, src_dev_);
    PL_CHECK_LAUNCH();
    return PLUME_OK;
  }

  int run_timed(int32_t first_step, int32_t n, double* ms, plume_step_stats* stats) override {
    return timed([&] { return run(first_step, n, stats); }, ms);
  }

  // n moving-box steps, the box spun and translated on the host after each
  int run_moving_timed(plume_box& box, int32_t first_step, int32_t n, double* ms,
                       plume_step_stats* stats) override {
    return timed(
        [&] {
          for (int k = 0; k < n; k++) {
            int rc = add_source(first_step + k);
            if (rc == PLUME_OK) rc = step_moving_box(box, stats ? stats + k : nullptr);
            if (rc != PLUME_OK) return rc;
            plume_box_spin(&box);
            plume_box_translate(&box);
          }
          return (int)PLUME_OK;
        },
        ms);
  }

  int stomp_times(double* ms, int64_t* launches) override {
    PL_TRY(cudaStreamSynchronize(s_));
    *ms = stomp_ms_;
    *launches = stomp_n_;
    return PLUME_OK;
  }

  // CUDA events on the library stream around body()
  template <typename F>
  int timed(F&& body, double* ms) {
    cudaEvent_t a, b;
    PL_TRY(cudaEventCreate(&a));
    PL_TRY(cudaEventCreate(&b));
    PL_TRY(cudaEventRecord(a, s_));
    int rc = body();
    if (rc == PLUME_OK) {
      PL_TRY(cudaEventRecord(b, s_));
      PL_TRY(cudaEventSynchronize(b));
      float f = 0.f;
      PL_TRY(cudaEventElapsedTime(&f, a, b));
      *ms = f;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
  }

  // ------------------------------------------------------------------ step
  int step(plume_step_stats* stats) override { return step_impl(nullptr, stats); }

  // FLUID_3D_MIC::stepWithMovingObstacle (FLUID_3D_MIC.cpp:236-310): the
  // step without buoyancy, with the obstacle stomp between damping and
  // projection.
  int step_moving_box(const plume_box& box, plume_step_stats* stats) override {
    BoxDev b;
    if (!box_dev(box, b)) return fail(PLUME_ERR_INVALID, "box with non-finite or zero parameters");
    if (!iop_in_) {
      const size_t N = (size_t)g_.N;
      PL_TRY(cudaMalloc(&iop_in_, N));
      PL_TRY(cudaMemsetAsync(iop_in_, 0, N, s_));  // border cells stay 0
      PL_TRY(cudaMalloc(&iop_val_, 3 * N * sizeof(double)));
      if (p_.cache_fields) {
        PL_TRY(cudaMalloc(&iop_post_pool_, 3 * N * sizeof(T)));
        PL_TRY(cudaMemsetAsync(iop_post_pool_, 0, 3 * N * sizeof(T), s_));
        post_iop_ = V3<T>{iop_post_pool_, iop_post_pool_ + N, iop_post_pool_ + 2 * N};
      }
    }
    return step_impl(&b, stats);
  }

  // FLUID_3D_MIC::setInitialVelocity(BOX*) (FLUID_3D_MIC.cpp:744-764)
  int set_initial_velocity_box(const plume_box& box) override {
    BoxDev b;
    if (!box_dev(box, b)) return fail(PLUME_ERR_INVALID, "box with non-finite or zero parameters");
    launches_ = 0;
    k_box_stomp<T><<<grid_for(box_cells(b)), 256, 0, s_>>>(g_, b, vel_, vel_, 0, nullptr, nullptr, 1);
    PL_CHECK_LAUNCH();
    PL_TRY(cudaStreamSynchronize(s_));
    return PLUME_OK;
  }

  bool has_iop() const override { return has_iop_; }

  // The full-space stages of SUBSPACE_FLUID_3D_EIGEN::stepReorderedCubatureStam
  // (SUBSPACE_FLUID_3D_EIGEN.cpp:247-266): velocity walls (density is left
  // as it is), buoyancy, vorticity confinement, then advectHeatAndDensityStam
  // (lines 573-601): the velocity's face conditions, density and heat advected
  // with it, their borders zeroed.  The velocity itself is advected in reduced
  // coordinates by the caller.
  int reduced_prestep() override {
    const int gN = grid_for(g_.N);
    const int nfaces = 2 * (g_.Y * g_.Z + g_.X * g_.Z + g_.X * g_.Y);
    const int gF = grid_for(nfaces);
    launches_ = 0;
    PL_TRY(cudaEventRecord(ev_[0], s_));
    k_forces<T><<<gN, 256, 0, s_>>>(g_, vel_, nullptr, heat_, prevort_, c_, 0);
    PL_CHECK_LAUNCH();
    const int gT = tile_blocks(g_);
    if (c_.has_vort) {
      k_vort1_t<T><<<gT, kTileThreads, 0, s_>>>(g_, vel_, vort_, mag_, c_);
      PL_CHECK_LAUNCH();
      k_vort2_t<T><<<gT, kTileThreads, 0, s_>>>(g_, vel_, vort_, mag_, force_, c_, 0);
      PL_CHECK_LAUNCH();
    }
    const int ox = p_.bc[2] == 0, oy = p_.bc[4] == 0, oz = p_.bc[0] == 0;
    k_face_bc<T><<<gF, 256, 0, s_>>>(g_, vel_, ox ? 1 : 0, oy ? 1 : 0, oz ? 1 : 0);
    PL_CHECK_LAUNCH();
    std::swap(dens_, dens_old_);
    std::swap(heat_, heat_old_);
    k_advect<T><<<gN, 256, 0, s_>>>(g_, c_, vel_, dens_old_, heat_old_, vel_, dens_, heat_, postadv_, 0, ox,
                                    oy, oz, 0);
    PL_CHECK_LAUNCH();
    total_time_ += 0.1;  // SUBSPACE_FLUID_3D_EIGEN.cpp:298
    total_steps_ += 1;
    return PLUME_OK;
  }
  int reduced_launches() const override { return launches_; }

  int download_iop(uint8_t* inside, double* values, size_t n) override {
    const size_t N = (size_t)g_.N;
    if (n != N) return fail(PLUME_ERR_INVALID, "the obstacle matrix needs N cells");
    if (!has_iop_) return fail(PLUME_ERR_STATE, "no moving-box step has run");
    std::vector<uint8_t> in(N);
    PL_TRY(cudaMemcpyAsync(in.data(), iop_in_, N, cudaMemcpyDeviceToHost, s_));
    if (values) PL_TRY(cudaMemcpyAsync(values, iop_val_, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    if (values)  // only inside cells are written on the device
      for (size_t c = 0; c < N; c++)
        if (!in[c]) values[3 * c] = values[3 * c + 1] = values[3 * c + 2] = 0.0;
    if (inside) memcpy(inside, in.data(), N);
    return PLUME_OK;
  }

  int step_impl(const BoxDev* box, plume_step_stats* stats) {
    const int cache = p_.cache_fields ? 1 : 0;
    const int gN = grid_for(g_.N);
    const int gI = grid_for(g_.nint);
    const int nfaces = 2 * (g_.Y * g_.Z + g_.X * g_.Z + g_.X * g_.Y);
    const int gF = grid_for(nfaces);
    const int gT = tile_blocks(g_);  // 2.5D stencil tiles (tile_kernels.cuh)
    launches_ = 0;
    NvtxRange step_range(box ? "stepWithMovingObstacle" : "step");
    PL_TRY(cudaEventRecord(ev_[0], s_));
    // forces: walls, buoyancy, prevorticity (FLUID_3D_MIC.cpp:188-199)
    StepConsts<T> cf = c_;
    if (box) cf.has_beta = 0;  // the moving step adds no buoyancy (lines 247-254)
    {
      NvtxRange r("addBuoyancy");
      k_forces<T><<<gN, 256, 0, s_>>>(g_, vel_, dens_, heat_, prevort_, cf, cache);
      PL_CHECK_LAUNCH();
    }
    PL_TRY(cudaEventRecord(evs_[0], s_));
    if (c_.has_vort) {  // addVorticity returns early when eps <= 0 (line 527)
      NvtxRange r("addVorticity");
      k_vort1_t<T><<<gT, kTileThreads, 0, s_>>>(g_, vel_, vort_, mag_, c_);
      PL_CHECK_LAUNCH();
      k_vort2_t<T><<<gT, kTileThreads, 0, s_>>>(g_, vel_, vort_, mag_, force_, c_, cache);
      PL_CHECK_LAUNCH();
    }
    PL_TRY(cudaEventRecord(evs_[1], s_));
    // advectStam (lines 595-650): boundary copy, swap, advect + fix-up
    const int ox = p_.bc[2] == 0, oy = p_.bc[4] == 0, oz = p_.bc[0] == 0;
    {
      NvtxRange r("advectStam");
      k_face_bc<T><<<gF, 256, 0, s_>>>(g_, vel_, ox ? 1 : 0, oy ? 1 : 0, oz ? 1 : 0);
      PL_CHECK_LAUNCH();
      std::swap(vel_, vel_old_);
      std::swap(dens_, dens_old_);
      std::swap(heat_, heat_old_);
      k_advect<T><<<gN, 256, 0, s_>>>(g_, c_, vel_old_, dens_old_, heat_old_, vel_, dens_, heat_,
                                      postadv_, cache, ox, oy, oz);
      PL_CHECK_LAUNCH();
    }
    PL_TRY(cudaEventRecord(evs_[2], s_));
    // damping (lines 209-212); the input buffer becomes `prediffusion`
    {
      NvtxRange r("buildPeeledDampingMatrixFull");
      k_damping_t<T><<<gT, kTileThreads, 0, s_>>>(g_, c_, vel_, spare_, preproj_, cache);
      PL_CHECK_LAUNCH();
    }
    std::swap(vel_, spare_);
    PL_TRY(cudaEventRecord(evs_[3], s_));
    NvtxRange project_range("project");
    if (box) {
      // the IOP stomp u <- N [u; 1], cached as postIOP (lines 276-284)
      if (prof_on_) PL_TRY(cudaEventRecord(stomp_ev_[0], s_));
      const int cache_post = post_iop_.x ? 1 : 0;
      k_box_post<T><<<gN, 256, 0, s_>>>(g_, vel_, post_iop_, cache_post, iop_in_);
      PL_CHECK_LAUNCH();
      k_box_stomp<T><<<grid_for(box_cells(*box)), 256, 0, s_>>>(g_, *box, vel_, post_iop_, cache_post,
                                                                 iop_in_, iop_val_, 0);
      PL_CHECK_LAUNCH();
      if (prof_on_) PL_TRY(cudaEventRecord(stomp_ev_[1], s_));
      has_iop_ = true;
    }
    // project (lines 314-399)
    k_face_bc<T><<<gF, 256, 0, s_>>>(g_, vel_, ox ? 2 : 0, oy ? 2 : 0, oz ? 2 : 0);
    PL_CHECK_LAUNCH();
    const bool learned = p_.warm_start == PLUME_WARM_LEARNED;
    // the learned start also uses the previous step's pressure
    const int keep_p = (p_.warm_start == PLUME_WARM_PREVIOUS || learned) ? 1 : 0;
    k_divergence_t<T><<<gT, kTileThreads, 0, s_>>>(g_, c_, vel_, div_, pres_, keep_p);
    PL_CHECK_LAUNCH();
    if (!learned) {
      k_copy_border_all<T><<<gF, 256, 0, s_>>>(g_, pres_);
      PL_CHECK_LAUNCH();
    }
    PL_TRY(cudaEventRecord(evs_[4], s_));
    last_fallback_ = 0;
    if (learned) {
      NvtxRange r("learned initial guess");
      // x0 = p_prev + g c with c = net(r0), r0 = b - A p_prev: the network
      // (an approximate inverse of A) applied to the previous pressure's
      // residual, scaled by the 1-D A-norm Galerkin factor g = c.r0 / c.A c;
      // border 0, as the reference's p = 0 leaves it
      // (a network trained on solve pairs maps b itself: x0 = g c, c = net(b))
      if (!net_) return fail(PLUME_ERR_STATE, "learned warm start without an attached network");
      const bool corr = net_->kind() != 0;  // correction and iterate networks map a residual
      k_zero_border<T><<<gF, 256, 0, s_>>>(g_, pres_);
      PL_CHECK_LAUNCH();
      if (corr) {
        k_residual<T><<<gN, 256, 0, s_>>>(g_, div_, pres_, r_);
        PL_CHECK_LAUNCH();
      }
      const T* rhs = corr ? r_ : div_;
      const int prc = net_->predict(net_ws_, rhs, z_, std::is_same<T, double>::value ? 1 : 0, s_, err_);
      if (prc != PLUME_OK) return prc;
      launches_ += net_->launches_per_predict();
      k_zero_border<T><<<gF, 256, 0, s_>>>(g_, z_);
      PL_CHECK_LAUNCH();
      k_guess_dots<T><<<kRedBlocks, kRedThreads, 0, s_>>>(g_, z_, z_, rhs, st_, part_);
      PL_CHECK_LAUNCH();
      k_guess_apply<T><<<gI, 256, 0, s_>>>(g_, corr ? pres_ : nullptr, z_, z_, st_, pres_);
      PL_CHECK_LAUNCH();
    }
    PL_TRY(cudaEventRecord(ev_[1], s_));
    NvtxRange solve_range("solvePoisson");
    // a learned-start or network-preconditioned solve gets at most twice the
    // previous step's iterations: a network that does not pay off falls back
    // early
    const bool flex = p_.preconditioner == PLUME_PRECOND_NET;
    if (flex && !net_) return fail(PLUME_ERR_STATE, "network preconditioner without an attached network");
    const bool uses_net = learned || flex;
    int cap = p_.max_iters;
    if (uses_net && last_iters_ > 0) cap = std::min(p_.max_iters, std::max(20, 2 * last_iters_));
    int rc = flex ? solve_fcg(div_, pres_, cap, !learned && keep_p == 0)
                  : solve_device(div_, pres_, cap, !learned && keep_p == 0);
    if (rc != PLUME_OK) return rc;
    // a convolution whose bounded wait expired left the guess or a
    // preconditioner output invalid (the solve above has synchronised the
    // stream): treat it as a rejected solve
    const bool net_failed = uses_net && net_->take_error(err_) != PLUME_OK;
    if (uses_net && (!st_host_->converged || net_failed)) {
      // the guess did not lead to convergence: plain MIC-PCG from p = 0
      last_fallback_ = 1;
      PL_TRY(cudaMemsetAsync(pres_, 0, (size_t)g_.N * sizeof(T), s_));
      rc = solve_device(div_, pres_, -1, true);
      if (rc != PLUME_OK) return rc;
    }
    last_iters_ = st_host_->iter;
    PL_TRY(cudaEventRecord(ev_[2], s_));
    k_gradient_t<T><<<gT, kTileThreads, 0, s_>>>(g_, c_, vel_, pres_);
    PL_CHECK_LAUNCH();
    PL_TRY(cudaEventRecord(ev_[3], s_));
    stages_valid_ = true;
    total_time_ += 0.1;  // FLUID_3D_MIC.cpp:221 (goalTime)
    total_steps_ += 1;
    if (box && prof_on_) {
      PL_TRY(cudaEventSynchronize(stomp_ev_[1]));
      float f = 0.f;
      PL_TRY(cudaEventElapsedTime(&f, stomp_ev_[0], stomp_ev_[1]));
      stomp_ms_ += f;
      stomp_n_ += 1;
    }
    if (stats) return fill_stats(stats);
    return PLUME_OK;
  }

  int run(int32_t first_step, int32_t n, plume_step_stats* stats) override {
    for (int k = 0; k < n; k++) {
      int rc = add_source(first_step + k);
      if (rc == PLUME_OK) rc = step(stats ? stats + k : nullptr);
      if (rc != PLUME_OK) return rc;
    }
    return PLUME_OK;
  }

  // ------------------------------------------------------------- transfer
  int download(int field, double* dst, size_t n) override {
    const size_t N = (size_t)g_.N;
    if (!dst) return fail(PLUME_ERR_INVALID, "null destination");
    const bool cached = (field == PLUME_F_PREVORTICITY || field == PLUME_F_POSTADVECTION ||
                         field == PLUME_F_PREPROJECTION || field == PLUME_F_CACHED_QUADRATIC ||
                         field == PLUME_F_FORCE);
    if (cached && !p_.cache_fields)
      return fail(PLUME_ERR_STATE, "field is not kept when cache_fields = 0");
    if (field == PLUME_F_POST_IOP && !p_.cache_fields)
      return fail(PLUME_ERR_STATE, "postIOP is not kept when cache_fields = 0");
    if (field == PLUME_F_POST_IOP && !has_iop_)
      return fail(PLUME_ERR_STATE, "postIOP: no moving-box step has run");
    const T* s = scalar_ptr(field);
    if (s) {
      if (n != N) return fail(PLUME_ERR_INVALID, "scalar field needs N doubles");
      return fetch_plane(s, dst, 1, 0);
    }
    V3<T> v;
    if (field == PLUME_F_CACHED_QUADRATIC) {
      if (n != 3 * N) return fail(PLUME_ERR_INVALID, "vector field needs 3N doubles");
      // _cachedQuadratic = velocity - velocityOld right after advection
      // (FLUID_3D_MIC.cpp:627) = postadvection - velocityOld.
      std::vector<double> a(3 * N), b(3 * N);
      int rc = fetch_vec(postadv_, a.data());
      if (rc == PLUME_OK) rc = fetch_vec(vel_old_, b.data());
      if (rc != PLUME_OK) return rc;
      if (std::is_same<T, float>::value) {
        for (size_t k = 0; k < 3 * N; k++) dst[k] = (double)((float)a[k] - (float)b[k]);
      } else {
        for (size_t k = 0; k < 3 * N; k++) dst[k] = a[k] - b[k];
      }
      return PLUME_OK;
    }
    if (!vector_ref(field, v)) return fail(PLUME_ERR_INVALID, "unknown field");
    if (n != 3 * N) return fail(PLUME_ERR_INVALID, "vector field needs 3N doubles");
    return fetch_vec(v, dst);
  }

  int upload(int field, const double* src, size_t n) override {
    const size_t N = (size_t)g_.N;
    if (!src) return fail(PLUME_ERR_INVALID, "null source");
    T* s = nullptr;
    switch (field) {
      case PLUME_F_DENSITY: s = dens_; break;
      case PLUME_F_DENSITY_OLD: s = dens_old_; break;
      case PLUME_F_HEAT: s = heat_; break;
      case PLUME_F_HEAT_OLD: s = heat_old_; break;
      case PLUME_F_PRESSURE: s = pres_; break;
      default: break;
    }
    if (s) {
      if (n != N) return fail(PLUME_ERR_INVALID, "scalar field needs N doubles");
      return put_plane(s, src, 1, 0);
    }
    V3<T> v;
    switch (field) {
      case PLUME_F_VELOCITY: v = vel_; break;
      case PLUME_F_VELOCITY_OLD: v = vel_old_; break;
      case PLUME_F_VORTICITY: v = vort_; break;
      default: return fail(PLUME_ERR_UNSUPPORTED, "field is derived and cannot be uploaded");
    }
    if (n != 3 * N) return fail(PLUME_ERR_INVALID, "vector field needs 3N doubles");
    int rc = put_plane(v.x, src, 3, 0);
    if (rc == PLUME_OK) rc = put_plane(v.y, src, 3, 1);
    if (rc == PLUME_OK) rc = put_plane(v.z, src, 3, 2);
    return rc;
  }

  int download_obstacles(uint8_t* dst, size_t n) override {
    if (!dst || n != (size_t)g_.N) return fail(PLUME_ERR_INVALID, "obstacles need N bytes");
    PL_TRY(cudaMemcpyAsync(dst, obst_, n, cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    return PLUME_OK;
  }

  // -------------------------------------------------------- solver access
  int solve(const double* b, double* x, plume_step_stats* stats) override {
    if (!b || !x) return fail(PLUME_ERR_INVALID, "null buffer");
    // uses the divergence/pressure planes as right-hand side and unknown
    int rc = put_plane(div_, b, 1, 0);
    if (rc == PLUME_OK) rc = put_plane(pres_, x, 1, 0);
    if (rc != PLUME_OK) return rc;
    stages_valid_ = false;
    PL_TRY(cudaEventRecord(ev_[1], s_));
    if (p_.preconditioner == PLUME_PRECOND_NET) {
      if (!net_) return fail(PLUME_ERR_STATE, "network preconditioner without an attached network");
      rc = solve_fcg(div_, pres_, -1, false);
      if (rc == PLUME_OK && net_->take_error(err_) != PLUME_OK) return PLUME_ERR_TIMEOUT;
    } else {
      rc = solve_device(div_, pres_);
    }
    if (rc != PLUME_OK) return rc;
    PL_TRY(cudaEventRecord(ev_[2], s_));
    PL_TRY(cudaEventRecord(ev_[0], s_));
    PL_TRY(cudaEventRecord(ev_[3], s_));
    rc = fetch_plane(pres_, x, 1, 0);
    if (rc == PLUME_OK && stats) rc = fill_stats(stats);
    return rc;
  }

  int mic_apply(const double* r, double* z, double* q) override {
    int rc = put_plane(r_, r, 1, 0);
    if (rc != PLUME_OK) return rc;
    // a fresh solver state so the sweeps are not skipped
    PL_TRY(cudaMemsetAsync(st_, 0, sizeof(CgState), s_));
    const int gK = grid_for(k_.total);
    k_to_skew<T, T><<<gK, 256, 0, s_>>>(g_, k_, r_, sr_);
    PL_CHECK_LAUNCH();
    prof_it_ = -1;
    rc = mic_sweeps(sr_, sqf_, sz_);
    if (rc != PLUME_OK) return rc;
    PL_TRY(cudaMemsetAsync(z_, 0, (size_t)g_.N * sizeof(T), s_));
    PL_TRY(cudaMemsetAsync(qf_, 0, (size_t)g_.N * sizeof(T), s_));
    k_from_skew<T><<<gK, 256, 0, s_>>>(g_, k_, sz_, z_);
    PL_CHECK_LAUNCH();
    k_from_skew<T><<<gK, 256, 0, s_>>>(g_, k_, sqf_, qf_);
    PL_CHECK_LAUNCH();
    if (!std::is_same<T, double>::value) {  // the FP32 forward sweep writes P q
      k_fwd_unscale<T><<<grid_for(g_.N), 256, 0, s_>>>(g_.N, P64_, qf_);
      PL_CHECK_LAUNCH();
    }
    PL_TRY(cudaMemcpyAsync(st_host_, st_, sizeof(CgState), cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    if (prof_on_) {
      rc = prof_harvest(prof_cur_);
      if (rc != PLUME_OK) return rc;
    }
    if (st_host_->wave_err) return fail(PLUME_ERR_TIMEOUT, "MIC wavefront wait expired");
    rc = fetch_plane(z_, z, 1, 0);
    if (rc == PLUME_OK && q) rc = fetch_plane(qf_, q, 1, 0);
    return rc;
  }

  int mic_precon(double* precon) override {
    PL_TRY(cudaMemcpyAsync(stage_, P64_, (size_t)g_.N * sizeof(double), cudaMemcpyDeviceToHost,
                           s_));
    PL_TRY(cudaStreamSynchronize(s_));
    memcpy(precon, stage_, (size_t)g_.N * sizeof(double));
    return PLUME_OK;
  }

  int sync() override {
    PL_TRY(cudaStreamSynchronize(s_));
    return PLUME_OK;
  }

  void use_cg_graph(bool on) override { no_cg_graph_ = !on; }
  const void* device_field(int field) override { return scalar_ptr(field); }
  bool device_vector(int field, const void* planes[3]) override {
    const bool cached = field == PLUME_F_PREVORTICITY || field == PLUME_F_POSTADVECTION ||
                        field == PLUME_F_PREPROJECTION || field == PLUME_F_FORCE ||
                        field == PLUME_F_POST_IOP;
    if (cached && !p_.cache_fields) return false;
    if (field == PLUME_F_POST_IOP && !has_iop_) return false;
    V3<T> v;
    if (!vector_ref(field, v) || !v.x) return false;
    planes[0] = v.x;
    planes[1] = v.y;
    planes[2] = v.z;
    return true;
  }
  void* stream_handle() override { return (void*)s_; }
  int attach_net(NetRuntime* net) override {
    PL_TRY(cudaStreamSynchronize(s_));
    if (net_ws_) net_->free_workspace(net_ws_);
    net_ = nullptr;
    net_ws_ = nullptr;
    if (!net) return PLUME_OK;
    net_ws_ = net->new_workspace(p_.res, err_);
    if (!net_ws_) return fail(PLUME_ERR_INVALID, err_.empty() ? "network workspace" : err_.c_str());
    net_ = net;
    return PLUME_OK;
  }
  void set_clock(int32_t steps, double time) override {
    total_steps_ = steps;
    total_time_ = time;
  }
  int32_t total_steps() const override { return total_steps_; }
  double total_time() const override { return total_time_; }
  double dx() const override { return dx_; }
  const plume_params& params() const override { return p_; }
  std::string& last_error() override { return err_; }

 private:
  static size_t align(size_t b) { return (b + 255) & ~(size_t)255; }

  void set_consts() {
    const double dt = p_.dt, dx = dx_;
    c_.dt = (T)dt;
    c_.beta = (T)p_.buoyancy;
    c_.eps = (T)p_.vorticity_eps;
    c_.dx = (T)dx;
    c_.gridSize = (T)(0.5 / dx);
    c_.oneOverDx = (T)(1.0 / dx);
    c_.dt0 = (T)(dt / dx);
    c_.divc = (T)(-dx * 0.5);
    c_.wMinus = (T)(1.0 - p_.damping_w);
    c_.sixth = (T)((1. / 6.) * p_.damping_w);
    c_.xHi = (T)(g_.X - 2.5);
    c_.yHi = (T)(g_.Y - 2.5);
    c_.zHi = (T)(g_.Z - 2.5);
    c_.has_vort = p_.vorticity_eps > 0.0 ? 1 : 0;
    c_.has_beta = p_.buoyancy != 0.0 ? 1 : 0;
  }

  // ---------------------------------------------------------------- solver
  // Skewed interior layout and wavefront configuration (wave.cuh).
  int init_solver() {
    k_.nx = g_.nx;
    k_.ny = g_.ny;
    k_.nz = g_.nz;
    k_.C = (g_.nx + 31) / 32;
    if (k_.C > 8) return fail(PLUME_ERR_UNSUPPORTED, "x resolution above 258 cells");
    k_.W = 32 * k_.C;
    k_.R = g_.ny + 31;
    k_.plane = (long long)k_.R * k_.W;
    k_.total = (long long)g_.nz * k_.plane;
    if (k_.total >= (1ll << 31)) return fail(PLUME_ERR_UNSUPPORTED, "grid too large for the solver");
    const size_t vb = align((size_t)k_.total * sizeof(T));
    const size_t bytes = 9 * vb + align(4 * sizeof(unsigned)) + align((size_t)g_.nz * sizeof(int));
    cudaError_t e = cudaMalloc(&spool_, bytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(PLUME_ERR_OOM, "device allocation of the solver vectors failed");
    }
    PL_TRY(cudaMemsetAsync(spool_, 0, bytes, s_));
    char* cur = spool_;
    T** v[] = {&sr_, &sd_, &sq_, &sz_, &sqf_, &sx_, &sb_, &sP_, &sd2_};
    for (T** p : v) {
      *p = (T*)cur;
      cur += vb;
    }
    wave_ctl_ = (unsigned*)cur;
    cur += align(4 * sizeof(unsigned));
    wave_prog_ = (int*)cur;
    k_diag_to_skew<T><<<grid_for(k_.total), 256, 0, s_>>>(g_, k_, P64_, sP_, std::is_same<T, double>::value ? 0 : 1);
    PL_CHECK_LAUNCH();
    // slab height: as many planes per CTA as shared memory allows, up to 8
    int dev = 0;
    PL_TRY(cudaGetDevice(&dev));
    PL_TRY(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
    bz_ = 8;
    while (bz_ > 1 && wave_smem_bytes<T>(bz_, k_.W) > 200 * 1024) bz_ /= 2;
    if (const char* env = getenv("PLUME_WAVE_BZ")) {
      const int b = atoi(env);
      if (b >= 1 && b <= 16 && wave_smem_bytes<T>(b, k_.W) <= 227 * 1024) bz_ = b;
    }
    wave_k_ = 8;
    if (const char* env = getenv("PLUME_WAVE_K")) {
      const int kk = atoi(env);
      if (kk >= 1 && kk <= 1024) wave_k_ = kk;
    }
    // cluster path: every slab of the plume in one cluster of <= 16 CTAs
    use_cluster_ = false;
    {
      int bzc = (g_.nz + 15) / 16;
      if (bzc < 4) bzc = 4;
      if (const char* env = getenv("PLUME_WAVE_CL_BZ")) {
        const int b = atoi(env);
        if (b >= 1 && b <= 16) bzc = b;
      }
      const char* off = getenv("PLUME_WAVE_NO_CLUSTER");
      if (!(off && atoi(off) != 0) && bzc <= 16 && (g_.nz + bzc - 1) / bzc <= 16 &&
          wave_smem_bytes<T>(bzc, k_.W) <= 227 * 1024) {
        WaveArgs<T> q = wave_args(sr_, sqf_, 0);
        q.BZ = bzc;
        q.nslabs = (g_.nz + bzc - 1) / bzc;
        int maxc = 0;
        constexpr bool exact = std::is_same<T, double>::value;
        cudaError_t e = launch_wave_cl<T, exact>(q, wave_smem_bytes<T>(bzc, k_.W), s_, 1, &maxc);
        if (e == cudaSuccess && maxc >= 1) {
          use_cluster_ = true;
          bz_ = bzc;
        }
        (void)cudaGetLastError();
      }
    }
    nslabs_ = (g_.nz + bz_ - 1) / bz_;
    wave_smem_ = wave_smem_bytes<T>(bz_, k_.W);
    wave_grid_ = nslabs_;  // slabs are handed out by ticket, so any grid size is safe
    if (wave_grid_ > 2 * num_sms_) wave_grid_ = 2 * num_sms_;
    if (const char* env = getenv("PLUME_WAVE_GRID")) {  // fewer CTAs than slabs: ticket loop
      const int gcap = atoi(env);
      if (gcap >= 1 && gcap < wave_grid_) wave_grid_ = gcap;
    }
    return PLUME_OK;
  }

  // fused direction update + SpMV (skew_kernels.cuh), dispatched on C
  int launch_spmv_dir(const T* z, const T* d_old, T* d_new, T* q) {
    // 16-byte groups where the cells per lane divide into them
    constexpr int NV = Vec16<T>::n;
    if (k_.C % NV == 0) {
      switch (k_.C) {
#define PL_SPMV_V_CASE(CC)                                                                              \
  case CC:                                                                                              \
    k_cgs_spmv_dir_v<T, (CC % NV == 0 ? CC : NV)><<<kRedBlocks, kRedThreads, 0, s_>>>(g_, k_, z, d_old, \
                                                                                      d_new, q, st_,  \
                                                                                      part_);         \
    PL_CHECK_LAUNCH();                                                                                  \
    return PLUME_OK;
        PL_SPMV_V_CASE(2)
        PL_SPMV_V_CASE(4)
        PL_SPMV_V_CASE(6)
        PL_SPMV_V_CASE(8)
#undef PL_SPMV_V_CASE
        default:
          break;
      }
    }
    switch (k_.C) {
#define PL_SPMV_CASE(CC)                                                                         \
  case CC:                                                                                       \
    k_cgs_spmv_dir<T, CC><<<kRedBlocks, SkewRows<CC>::THREADS, 0, s_>>>(g_, k_, z, d_old, d_new, q, \
                                                                       st_, part_);             \
    break;
      PL_SPMV_CASE(1)
      PL_SPMV_CASE(2)
      PL_SPMV_CASE(3)
      PL_SPMV_CASE(4)
      PL_SPMV_CASE(5)
      PL_SPMV_CASE(6)
      PL_SPMV_CASE(7)
      PL_SPMV_CASE(8)
#undef PL_SPMV_CASE
      default:
        return fail(PLUME_ERR_UNSUPPORTED, "cells per lane");
    }
    PL_CHECK_LAUNCH();
    return PLUME_OK;
  }

  WaveArgs<T> wave_args(const T* in, T* out, int backward) {
    WaveArgs<T> a;
    a.P = sP_;
    a.in = in;
    a.out = out;
    a.k = k_;
    a.BZ = bz_;
    a.nslabs = nslabs_;
    a.K = wave_k_;
    a.backward = backward;
    a.ctl = wave_ctl_;
    a.progress = wave_prog_;
    a.st = st_;
    a.gate = gate_closed_ ? (const int*)(wave_ctl_ + 3) : nullptr;  // ctl[3]: never written
    a.gate_spins = gate_spins_;
    return a;
  }

  int partial_solve(int max_iters, void* xv) override {
    if (max_iters < 1) return fail(PLUME_ERR_INVALID, "partial solve needs at least one iteration");
    T* x = (T*)xv;
    PL_TRY(cudaMemsetAsync(x, 0, (size_t)g_.N * sizeof(T), s_));
    return solve_device(div_, x, max_iters, true);
  }

  int set_wait_gate(int closed, long long polls) override {
    if (closed && polls <= 0) return fail(PLUME_ERR_INVALID, "the gate's poll limit must be positive");
    PL_TRY(cudaStreamSynchronize(s_));
    gate_closed_ = closed != 0;
    gate_spins_ = closed ? polls : 0;
    // the CG-loop graph holds the sweeps' arguments by value: build it anew
    if (cg_exec_) cudaGraphExecDestroy(cg_exec_);
    cg_exec_ = nullptr;
    return PLUME_OK;
  }

  // MIC forward then backward sweep on skewed vectors (wavefront kernels).
  // With sweep profiling on, CUDA events on the handle's stream bracket each
  // of the two launches.
  int mic_sweeps(const T* r, T* q, T* z) {
    constexpr bool exact = std::is_same<T, double>::value;
    cudaEvent_t* ev = nullptr;
    if (prof_on_ && prof_n_[prof_cur_] + 3 <= kProfEvents) {
      ev = &prof_ev_[prof_cur_][prof_n_[prof_cur_]];
      prof_idx_[prof_cur_][prof_n_[prof_cur_] / 3] = prof_it_;
      prof_n_[prof_cur_] += 3;
      PL_TRY(cudaEventRecord(ev[0], s_));
    }
    cudaError_t e = use_cluster_ ? launch_wave_cl<T, exact>(wave_args(r, q, 0), wave_smem_, s_)
                                 : launch_wave<T, exact>(wave_args(r, q, 0), wave_grid_, wave_smem_, s_);
    PL_TRY(e);
    ++launches_;
    if (ev) PL_TRY(cudaEventRecord(ev[1], s_));
    e = use_cluster_ ? launch_wave_cl<T, exact>(wave_args(q, z, 1), wave_smem_, s_)
                     : launch_wave<T, exact>(wave_args(q, z, 1), wave_grid_, wave_smem_, s_);
    PL_TRY(e);
    ++launches_;
    if (ev) PL_TRY(cudaEventRecord(ev[2], s_));
    return PLUME_OK;
  }

  // Adds up the sweep timings recorded in event buffer b, counting only the
  // pairs of PCG iterations below `ran` (later launches of a chunk return at
  // once because the solve had finished); every event in the buffer must have
  // completed (the stream was synchronized after they were queued).
  int prof_harvest(int b, int ran = 1 << 30) {
    for (int i = 0; i + 2 < prof_n_[b]; i += 3) {
      if (prof_idx_[b][i / 3] >= ran) continue;
      float f = 0.f, g = 0.f;
      PL_TRY(cudaEventElapsedTime(&f, prof_ev_[b][i], prof_ev_[b][i + 1]));
      PL_TRY(cudaEventElapsedTime(&g, prof_ev_[b][i + 1], prof_ev_[b][i + 2]));
      prof_ms_ += (double)f + (double)g;
      prof_launches_ += 2;
    }
    prof_n_[b] = 0;
    return PLUME_OK;
  }

  int profile_sweeps(int on) override {
    PL_TRY(cudaStreamSynchronize(s_));
    if (on && !prof_ev_[0][0]) {
      for (auto& buf : prof_ev_)
        for (auto& e : buf) PL_TRY(cudaEventCreate(&e));
      for (auto& e : stomp_ev_) PL_TRY(cudaEventCreate(&e));
    }
    prof_on_ = on != 0;
    stomp_ms_ = 0;
    stomp_n_ = 0;
    prof_n_[0] = prof_n_[1] = 0;
    prof_ms_ = 0;
    prof_launches_ = 0;
    return PLUME_OK;
  }

  int sweep_times(double* ms, int64_t* launches) override {
    PL_TRY(cudaStreamSynchronize(s_));
    int rc = prof_harvest(0);
    if (rc == PLUME_OK) rc = prof_harvest(1);
    if (ms) *ms = prof_ms_;
    if (launches) *launches = prof_launches_;
    return rc;
  }

  // MIC-PCG (FLUID_3D_MIC.cpp:918-1015); x (natural layout) holds the initial
  // guess on entry and the solution on return, b is the natural right side.
  // x_zero: the caller knows x = 0 on the interior (r = b without A x)
  int solve_device(const T* b, T* x, int max_iters = -1, bool x_zero = false) {
    if (max_iters < 0) max_iters = p_.max_iters;
    const int gK = grid_for(k_.total);
    k_to_skew<T, T><<<gK, 256, 0, s_>>>(g_, k_, b, sb_);
    PL_CHECK_LAUNCH();
    k_to_skew<T, T><<<gK, 256, 0, s_>>>(g_, k_, x, sx_);
    PL_CHECK_LAUNCH();
    k_cgs_init<T><<<kRedBlocks, kRedThreads, 0, s_>>>(g_, k_, sb_, sx_, sr_, st_, part_, p_.tol,
                                                      max_iters, p_.criterion, x_zero ? 1 : 0);
    PL_CHECK_LAUNCH();
    prof_it_ = -1;
    int rc = mic_sweeps(sr_, sqf_, sz_);
    if (rc != PLUME_OK) return rc;
    k_cgs_init2<T><<<kRedBlocks, kRedThreads, 0, s_>>>(k_, sr_, sz_, (T*)nullptr, st_, part_);
    PL_CHECK_LAUNCH();
    // zeroed so that 0 * d_old on the first iteration can never see stale
    // non-finite values
    PL_TRY(cudaMemsetAsync(sd_, 0, (size_t)k_.total * sizeof(T), s_));
    if (!prof_on_ && !no_cg_graph_ && cg_graph_ready()) {
      // the whole iteration loop as one graph launch (conditional while node)
      PL_TRY(cudaMemsetAsync(&st_->bodies, 0, sizeof(int), s_));
      PL_TRY(cudaGraphLaunch(cg_exec_, s_));
      return finish_solve(x, true);
    }
    int chunk = 4;
    T* dcur = sd_;  // direction of the previous iteration (beta = 0 on the first)
    T* dnext = sd2_;
    for (int it = 0; it < max_iters + chunk;) {
      for (int kk = 0; kk < chunk; kk++) {
        rc = launch_spmv_dir(sz_, dcur, dnext, sq_);
        if (rc != PLUME_OK) return rc;
        k_cgs_axpy_v<T><<<kRedBlocks, kRedThreads, 0, s_>>>(k_, dnext, sq_, sx_, sr_, st_, part_);
        PL_CHECK_LAUNCH();
        prof_it_ = it + kk;
        rc = mic_sweeps(sr_, sqf_, sz_);
        if (rc != PLUME_OK) return rc;
        k_cgs_rz_v<T><<<kRedBlocks, kRedThreads, 0, s_>>>(k_, sr_, sz_, st_, part_);
        PL_CHECK_LAUNCH();
        std::swap(dcur, dnext);
      }
      it += chunk;
      // the other event buffer was filled before the last synchronize: read
      // it while this chunk runs, then fill the other one next
      if (prof_on_) {
        rc = prof_harvest(prof_cur_ ^ 1);
        if (rc != PLUME_OK) return rc;
      }
      PL_TRY(cudaMemcpyAsync(st_host_, st_, sizeof(CgState), cudaMemcpyDeviceToHost, s_));
      PL_TRY(cudaStreamSynchronize(s_));
      prof_cur_ ^= 1;
      if (st_host_->done) break;
      if (chunk < 16) chunk *= 2;
    }
    return finish_solve(x, false);
  }

  // The network as the preconditioner stage: z = net(r) on skewed vectors
  // (through the natural-layout planes r_ and z_, whose borders the network
  // neither reads nor writes).
  int precondition_net(const T* rs, T* zs) {
    const int gK = grid_for(k_.total);
    k_from_skew<T><<<gK, 256, 0, s_>>>(g_, k_, rs, r_);
    PL_CHECK_LAUNCH();
    const int prc = net_->predict(net_ws_, r_, z_, std::is_same<T, double>::value ? 1 : 0, s_, err_);
    if (prc != PLUME_OK) return prc;
    launches_ += net_->launches_per_predict();
    k_to_skew<T, T><<<gK, 256, 0, s_>>>(g_, k_, z_, zs);
    PL_CHECK_LAUNCH();
    return PLUME_OK;
  }

  // Flexible CG (FCG(1), k_cgs_rz_fcg) with the network as the
  // preconditioner stage, the reference's loop (FLUID_3D_MIC.cpp:951-1013)
  // with z = net(r) in place of applyMICPreconditioner and the direction
  // update made A-orthogonal.  The same set-up, stop tests and state as
  // solve_device.  Host-driven: one synchronisation per iteration, after the
  // update, so that no network pass runs once the stop test is met (a pass
  // costs several MIC-PCG iterations).
  int solve_fcg(const T* b, T* x, int max_iters, bool x_zero) {
    if (max_iters < 0) max_iters = p_.max_iters;
    const int gK = grid_for(k_.total);
    k_to_skew<T, T><<<gK, 256, 0, s_>>>(g_, k_, b, sb_);
    PL_CHECK_LAUNCH();
    k_to_skew<T, T><<<gK, 256, 0, s_>>>(g_, k_, x, sx_);
    PL_CHECK_LAUNCH();
    k_cgs_init<T><<<kRedBlocks, kRedThreads, 0, s_>>>(g_, k_, sb_, sx_, sr_, st_, part_, p_.tol,
                                                      max_iters, p_.criterion, x_zero ? 1 : 0);
    PL_CHECK_LAUNCH();
    int rc = precondition_net(sr_, sz_);
    if (rc != PLUME_OK) return rc;
    k_cgs_init2<T><<<kRedBlocks, kRedThreads, 0, s_>>>(k_, sr_, sz_, (T*)nullptr, st_, part_);
    PL_CHECK_LAUNCH();
    PL_TRY(cudaMemsetAsync(sd_, 0, (size_t)k_.total * sizeof(T), s_));
    T* dcur = sd_;
    T* dnext = sd2_;
    for (int it = 0; it <= max_iters; it++) {
      rc = launch_spmv_dir(sz_, dcur, dnext, sq_);
      if (rc != PLUME_OK) return rc;
      k_cgs_axpy_v<T><<<kRedBlocks, kRedThreads, 0, s_>>>(k_, dnext, sq_, sx_, sr_, st_, part_);
      PL_CHECK_LAUNCH();
      PL_TRY(cudaMemcpyAsync(st_host_, st_, sizeof(CgState), cudaMemcpyDeviceToHost, s_));
      PL_TRY(cudaStreamSynchronize(s_));
      if (st_host_->done) break;
      rc = precondition_net(sr_, sz_);
      if (rc != PLUME_OK) return rc;
      k_cgs_rz_fcg<T><<<kRedBlocks, kRedThreads, 0, s_>>>(k_, sr_, sz_, sq_, dnext, st_, part_);
      PL_CHECK_LAUNCH();
      std::swap(dcur, dnext);
    }
    return finish_solve(x, false);
  }

  // The CG iteration loop as a CUDA graph: a conditional while node whose
  // body is 16 iterations (SpMV + direction, update, forward and backward MIC
  // sweeps, r.z) followed by k_cg_continue, which sets the loop condition from
  // the device-side state.  Built on first use by capturing the body on the
  // handle's stream; if any step fails, the host-driven loop is used instead.
  static constexpr int kCgBody = 16;  // even: the direction buffers swap back
  static constexpr int kCgBodyLaunches = kCgBody * 5 + 1;
  bool cg_graph_ready() {
    if (cg_exec_) return true;
    if (cg_graph_failed_) return false;
    const int saved = launches_;
    cudaGraph_t graph = nullptr;
    cudaGraphConditionalHandle h = 0;
    bool capturing = false;
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};  // every other byte zero
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
    if (e == cudaSuccess)
      e = cudaStreamBeginCaptureToGraph(s_, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed);
    capturing = e == cudaSuccess;
    int rc = PLUME_OK;
    T* dcur = sd_;
    T* dnext = sd2_;
    for (int kk = 0; kk < kCgBody && e == cudaSuccess && rc == PLUME_OK; kk++) {
      rc = launch_spmv_dir(sz_, dcur, dnext, sq_);
      if (rc == PLUME_OK) {
        k_cgs_axpy_v<T><<<kRedBlocks, kRedThreads, 0, s_>>>(k_, dnext, sq_, sx_, sr_, st_, part_);
        e = cudaGetLastError();
      }
      if (rc == PLUME_OK && e == cudaSuccess) rc = mic_sweeps(sr_, sqf_, sz_);
      if (rc == PLUME_OK && e == cudaSuccess) {
        k_cgs_rz_v<T><<<kRedBlocks, kRedThreads, 0, s_>>>(k_, sr_, sz_, st_, part_);
        e = cudaGetLastError();
      }
      std::swap(dcur, dnext);
    }
    if (e == cudaSuccess && rc == PLUME_OK) {
      k_cg_continue<<<1, 32, 0, s_>>>(h, st_);
      e = cudaGetLastError();
    }
    if (capturing) {
      cudaGraph_t body = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(s_, &body);
      if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess && rc == PLUME_OK) e = cudaGraphInstantiate(&cg_exec_, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    launches_ = saved;  // captured launches ran nothing
    err_.clear();
    (void)cudaGetLastError();
    if (e != cudaSuccess || rc != PLUME_OK || !cg_exec_) {
      if (cg_exec_) cudaGraphExecDestroy(cg_exec_);
      cg_exec_ = nullptr;
      cg_graph_failed_ = true;
      return false;
    }
    return true;
  }

  // Solution back to the natural layout and the solver state to the host
  // (one synchronisation).
  int finish_solve(T* x, bool graph) {
    const int gK = grid_for(k_.total);
    int rc = PLUME_OK;
    k_from_skew<T><<<gK, 256, 0, s_>>>(g_, k_, sx_, x);
    PL_CHECK_LAUNCH();
    PL_TRY(cudaMemcpyAsync(st_host_, st_, sizeof(CgState), cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    if (graph) launches_ += st_host_->bodies * kCgBodyLaunches;
    if (prof_on_) {
      // iterations whose sweeps ran: all counted ones, less the last when the
      // rel-L2 test stopped the solve before its sweeps (k_cgs_axpy_v)
      int ran = st_host_->iter;
      if (st_host_->criterion == 1 && st_host_->converged) ran -= 1;
      rc = prof_harvest(prof_cur_ ^ 1, ran);
      if (rc != PLUME_OK) return rc;
    }
    if (st_host_->wave_err) {
      char buf[128];
      snprintf(buf, sizeof(buf), "MIC wavefront wait expired (code %d)", st_host_->wave_err);
      return fail(PLUME_ERR_TIMEOUT, buf);
    }
    return PLUME_OK;
  }

  int fill_stats(plume_step_stats* st) {
    PL_TRY(cudaMemcpyAsync(st_host_, st_, sizeof(CgState), cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    memset(st, 0, sizeof(*st));
    st->iterations = st_host_->iter;
    st->launches = launches_;
    st->converged = st_host_->converged;
    st->fallback = last_fallback_;
    st->max_residual = st_host_->maxR;
    st->rhs_norm = sqrt(st_host_->bb);
    st->rel_residual = st_host_->bb > 0 ? sqrt(st_host_->rr) / sqrt(st_host_->bb) : 0.0;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev_[0], ev_[3]) == cudaSuccess) st->ms_total = ms;
    if (cudaEventElapsedTime(&ms, ev_[1], ev_[2]) == cudaSuccess) st->ms_solve = ms;
    if (stages_valid_) {
      // stage boundaries in step order: start, forces, vorticity, advection,
      // damping, divergence (guess start), guess (solve start), ..., end
      const cudaEvent_t b[8] = {ev_[0], evs_[0], evs_[1], evs_[2], evs_[3], evs_[4], ev_[1], ev_[2]};
      double* out[6] = {&st->ms_forces, &st->ms_vorticity, &st->ms_advection, &st->ms_damping,
                        &st->ms_divergence, &st->ms_guess};
      for (int k = 0; k < 6; k++)
        if (cudaEventElapsedTime(&ms, b[k], b[k + 1]) == cudaSuccess) *out[k] = ms;
      if (cudaEventElapsedTime(&ms, ev_[2], ev_[3]) == cudaSuccess) st->ms_gradient = ms;
    }
    (void)cudaGetLastError();
    return PLUME_OK;
  }

  // The per-step constants of the stomp (box.cpp) and a cell range that
  // certainly contains every inside cell: the circumscribed sphere of the box,
  // widened by two cells, when R is a rotation; the whole interior otherwise.
  bool box_dev(const plume_box& box, BoxDev& b) const {
    if (!box_finite(box)) return false;
    box_constants(box, b.half, b.omega, b.disp);
    const int res[3] = {g_.X, g_.Y, g_.Z};
    for (int k = 0; k < 3; k++) {
      b.center[k] = box.center[k];
      b.axis[k] = k == 2 ? 1.0 : 0.0;
      b.d[k] = 1.0 / res[k];
      b.lo[k] = 1;
      b.hi[k] = res[k] - 1;
    }
    for (int k = 0; k < 9; k++) b.R[k] = box.rotation[k];
    double dev = 0;  // max |R^T R - I|
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double s = 0;
        for (int k = 0; k < 3; k++) s += b.R[3 * k + i] * b.R[3 * k + j];
        dev = std::max(dev, std::fabs(s - (i == j ? 1.0 : 0.0)));
      }
    if (dev <= 1e-9) {
      // R is a rotation: inside cells satisfy u = R^T q with |q_k| <= half_k,
      // so |u_i| <= sum_k |R_ki| |half_k|; widened by 1e-6 and two cells
      for (int k = 0; k < 3; k++) {
        double ext = 0;
        for (int j = 0; j < 3; j++) ext += std::fabs(b.R[3 * j + k]) * std::fabs(b.half[j]);
        ext *= 1.0 + 1e-6;
        const double n = res[k];
        const double lo = std::floor((b.center[k] - ext) * n - 0.5) - 2.0;
        const double hi = std::ceil((b.center[k] + ext) * n - 0.5) + 3.0;
        b.lo[k] = (int)std::max(1.0, std::min(n - 1.0, lo));
        b.hi[k] = (int)std::max(1.0, std::min(n - 1.0, hi));
      }
    }
    double rmax = 0;
    for (int k = 0; k < 9; k++) {
      b.fR[k] = (float)b.R[k];
      rmax = std::max(rmax, std::fabs(b.R[k]));
    }
    for (int k = 0; k < 3; k++) {
      b.fc[k] = (float)b.center[k];
      b.fh[k] = (float)b.half[k];
      b.fd[k] = (float)b.d[k];
    }
    b.ftol = (float)(1e-5 * (1.0 + rmax));
    return true;
  }

  static long long box_cells(const BoxDev& b) {
    return std::max(1LL, (long long)(b.hi[0] - b.lo[0]) * (b.hi[1] - b.lo[1]) * (b.hi[2] - b.lo[2]));
  }

  const T* scalar_ptr(int field) const {
    switch (field) {
      case PLUME_F_DENSITY: return dens_;
      case PLUME_F_DENSITY_OLD: return dens_old_;
      case PLUME_F_HEAT: return heat_;
      case PLUME_F_HEAT_OLD: return heat_old_;
      case PLUME_F_PRESSURE: return pres_;
      case PLUME_F_DIVERGENCE: return div_;
      case PLUME_F_CACHED_PRESSURE: return pres_;      // solvePoisson leaves it untouched after
      case PLUME_F_CACHED_DIVERGENCE: return div_;  // the copy (FLUID_3D_MIC.cpp:364,369)
      default: return nullptr;
    }
  }
  bool vector_ref(int field, V3<T>& v) const {
    switch (field) {
      case PLUME_F_VELOCITY: v = vel_; return true;
      case PLUME_F_VELOCITY_OLD: v = vel_old_; return true;
      case PLUME_F_FORCE: v = force_; return true;
      case PLUME_F_VORTICITY: v = vort_; return true;
      case PLUME_F_PREPROJECTION: v = preproj_; return true;
      case PLUME_F_PREDIFFUSION: v = spare_; return true;
      case PLUME_F_PREADVECTION: v = vel_old_; return true;  // same data after the swap (line 617)
      case PLUME_F_POSTADVECTION: v = postadv_; return true;
      case PLUME_F_PREVORTICITY: v = prevort_; return true;
      case PLUME_F_POST_IOP: v = post_iop_; return post_iop_.x != nullptr;
      default: return false;
    }
  }

  // device plane -> host doubles at dst[k*stride + off]
  int fetch_plane(const T* src, double* dst, int stride, int off) {
    const size_t N = (size_t)g_.N;
    if (host_direct_ && stride == 1) {
      k_planes_to_host<T><<<grid_for((long long)N), 256, 0, s_>>>(src, src, src, 1, (long long)N, dst);
      PL_CHECK_LAUNCH();
      PL_TRY(cudaStreamSynchronize(s_));
      return PLUME_OK;
    }
    PL_TRY(cudaMemcpyAsync(stage_, src, N * sizeof(T), cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    const T* h = (const T*)stage_;
    for (size_t k = 0; k < N; k++) dst[k * stride + off] = (double)h[k];
    return PLUME_OK;
  }
  int fetch_vec(const V3<T>& v, double* dst) {
    if (host_direct_) {
      const long long N = g_.N;
      if (((uintptr_t)dst & 15) == 0)
        k_vec_to_host2<T><<<grid_for(N / 2 + 1), 256, 0, s_>>>(v.x, v.y, v.z, N, dst);
      else
        k_planes_to_host<T><<<grid_for(3 * N), 256, 0, s_>>>(v.x, v.y, v.z, 3, N, dst);
      PL_CHECK_LAUNCH();
      PL_TRY(cudaStreamSynchronize(s_));
      return PLUME_OK;
    }
    int rc = fetch_plane(v.x, dst, 3, 0);
    if (rc == PLUME_OK) rc = fetch_plane(v.y, dst, 3, 1);
    if (rc == PLUME_OK) rc = fetch_plane(v.z, dst, 3, 2);
    return rc;
  }
  int put_plane(T* dst, const double* src, int stride, int off) {
    const size_t N = (size_t)g_.N;
    PL_TRY(cudaStreamSynchronize(s_));
    T* h = (T*)stage_;
    for (size_t k = 0; k < N; k++) h[k] = (T)src[k * stride + off];
    PL_TRY(cudaMemcpyAsync(dst, stage_, N * sizeof(T), cudaMemcpyHostToDevice, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    return PLUME_OK;
  }

  int fail(int code, const char* msg) {
    err_ = msg;
    return code;
  }
  int fail_cuda(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
    err_ = buf;
    (void)cudaGetLastError();
    return (e == cudaErrorMemoryAllocation) ? PLUME_ERR_OOM : PLUME_ERR_CUDA;
  }

  void release() {
    if (s_) cudaStreamSynchronize(s_);
    if (cg_exec_) cudaGraphExecDestroy(cg_exec_);
    cg_exec_ = nullptr;
    if (net_ws_) net_->free_workspace(net_ws_);
    net_ws_ = nullptr;
    if (pool_) cudaFree(pool_);
    if (spool_) cudaFree(spool_);
    if (iop_in_) cudaFree(iop_in_);
    if (iop_val_) cudaFree(iop_val_);
    if (iop_post_pool_) cudaFree(iop_post_pool_);
    iop_in_ = nullptr;
    iop_val_ = nullptr;
    iop_post_pool_ = nullptr;
    if (col_cells_) cudaFree(col_cells_);
    if (src_dev_) cudaFree(src_dev_);
    if (src_host_) cudaFreeHost(src_host_);
    if (st_host_) cudaFreeHost(st_host_);
    if (stage_) cudaFreeHost(stage_);
    for (auto e : ev_)
      if (e) cudaEventDestroy(e);
    for (auto e : evs_)
      if (e) cudaEventDestroy(e);
    for (auto& buf : prof_ev_)
      for (auto e : buf)
        if (e) cudaEventDestroy(e);
    for (auto e : stomp_ev_)
      if (e) cudaEventDestroy(e);
    if (s_) cudaStreamDestroy(s_);
    pool_ = nullptr;
    s_ = nullptr;
  }

  plume_params p_{};
  Grid g_{};
  StepConsts<T> c_{};
  double dx_ = 0, total_time_ = 0;
  int total_steps_ = 0;
  int launches_ = 0;
  cudaStream_t s_ = nullptr;
  cudaEvent_t ev_[4] = {nullptr, nullptr, nullptr, nullptr};
  // stage boundaries inside a step: after forces, vorticity, advection,
  // damping and the divergence (plume_step_stats' per-stage times)
  cudaEvent_t evs_[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  bool stages_valid_ = false;
  char* pool_ = nullptr;
  T *dens_ = nullptr, *dens_old_ = nullptr, *heat_ = nullptr, *heat_old_ = nullptr;
  T *pres_ = nullptr, *div_ = nullptr, *mag_ = nullptr;
  T *r_ = nullptr, *d_ = nullptr, *q_ad_ = nullptr, *z_ = nullptr, *qf_ = nullptr;
  V3<T> vel_{}, vel_old_{}, spare_{}, prevort_{}, postadv_{}, preproj_{}, force_{}, vort_{};
  double* P64_ = nullptr;
  // moving box: inside mask (N), last-column values (3N doubles) and postIOP,
  // allocated at the first moving step
  uint8_t* iop_in_ = nullptr;
  double* iop_val_ = nullptr;
  T* iop_post_pool_ = nullptr;
  V3<T> post_iop_{};
  bool has_iop_ = false;
  // skewed solver vectors and wavefront configuration
  Skew k_{};
  char* spool_ = nullptr;
  T *sr_ = nullptr, *sd_ = nullptr, *sq_ = nullptr, *sz_ = nullptr, *sqf_ = nullptr, *sx_ = nullptr,
    *sb_ = nullptr, *sP_ = nullptr, *sd2_ = nullptr;
  unsigned* wave_ctl_ = nullptr;  // [0] slab ticket, [1] exited CTAs, [3] the test gate (0)
  int* wave_prog_ = nullptr;
  bool gate_closed_ = false;  // plume_set_wait_gate
  long long gate_spins_ = 0;
  int bz_ = 8, wave_k_ = 8, nslabs_ = 1, wave_grid_ = 1, num_sms_ = 1;
  bool use_cluster_ = false;
  size_t wave_smem_ = 0;
  uint8_t* obst_ = nullptr;
  CgState* st_ = nullptr;
  double* part_ = nullptr;
  int* col_cells_ = nullptr;
  T* src_dev_ = nullptr;
  T* src_host_ = nullptr;
  int n_col_ = 0;
  CgState* st_host_ = nullptr;
  void* stage_ = nullptr;
  // sweep profiling: two event buffers, one filled while the other is read
  // (three events per forward+backward pair; a chunk holds at most 17 pairs)
  NetRuntime* net_ = nullptr;
  void* net_ws_ = nullptr;
  int last_fallback_ = 0;
  int last_iters_ = 0;  // iterations of the last accepted step solve
  cudaGraphExec_t cg_exec_ = nullptr;  // CG loop graph (cg_graph_ready)
  bool no_cg_graph_ = false;
  bool cg_graph_failed_ = getenv("PLUME_NO_CG_GRAPH") != nullptr;
  bool host_direct_ = false;  // downloads written by a kernel into host memory
  static constexpr int kProfEvents = 64;
  bool prof_on_ = false;
  cudaEvent_t stomp_ev_[2] = {nullptr, nullptr};  // around the moving-box stomp
  double stomp_ms_ = 0;
  int64_t stomp_n_ = 0;
  cudaEvent_t prof_ev_[2][kProfEvents] = {};
  int prof_n_[2] = {0, 0};
  int prof_idx_[2][kProfEvents / 3] = {};  // PCG iteration of each pair (-1: set-up)
  int prof_cur_ = 0;
  int prof_it_ = -1;
  double prof_ms_ = 0;
  int64_t prof_launches_ = 0;
  std::string err_;
};

}  // namespace plume
