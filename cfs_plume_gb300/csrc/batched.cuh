// batched.cuh -- the fused batch engine: many plumes of uneven grids advanced
// in lockstep on one GPU (include/plume_batch.h, PLUME_BATCH_FUSED).
//
// Layout.  Every plume keeps the single-plume engine's natural-layout planes
// (SoA, x fastest) and skewed solver vectors (wave.cuh); the solver vectors of
// one kind (all plumes' r, all plumes' d, ...) are one contiguous region, so
// one memset clears a kind for the whole batch.
//
// Launches.  A stage kernel's grid is the concatenation of the plumes'
// shares: plume i gets count[i] blocks, chosen from its own element count and
// the tuned elements per thread.  A block reads its plume and its index
// within that share from the stage's table (two loads) and runs the kernel
// body the single-plume engine runs (step_kernels.cuh, skew_kernels.cuh), so
// each cell evaluates the same expression as in the single-plume step
// (FLUID_3D_MIC::step, FLUID_3D_MIC.cpp:179-223).  A reduction's partial sums
// and last-block ticket are per plume.  The MIC sweeps (wave.cuh: one
// thread-block cluster per plume) have their cells per lane and cluster shape
// fixed at launch, so they launch once per shape class -- plumes with the
// same cells per lane and depth -- and the classes run as parallel branches
// of the graph.
//
// Lockstep CG.  Every plume runs its own MIC-PCG (its own scalars in its own
// CgState); an iteration is one launch of each kernel over all plumes, and a
// plume whose stop test has been met returns at the top of its blocks.  The
// loop is a conditional-while node that ends when every plume is done.
//
// Graph.  A whole step -- box source, forces, vorticity, advection, damping,
// projection set-up, the CG loop, gradient and the per-plume statistics row --
// is captured once into a CUDA graph; the density/heat buffer parity, the
// source's step index and the statistics row live in device memory, so the
// same graph serves every step.
#pragma once
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

#include "batched.h"
#include "engine.cuh"
#include "tune_cache.h"

namespace plume {

// One plume of the batch as the kernels see it (device memory).
template <typename T>
struct BPlume {
  Grid g;
  Skew k;
  StepConsts<T> c;
  V3<T> vel, tmp, vort;  // velocity; advection target; vorticity
  T* dens[2];            // density, current = dens[parity]
  T* heat[2];
  T* pres;
  T* div;
  T* mag;
  T *sb, *sx, *sr, *sq, *sqf, *sz, *sP;  // skewed solver vectors
  T* sd[2];                              // CG direction, double-buffered
  CgState* st;
  double* part;          // reduction partials (4 * kRedBlocks)
  int src_lo[3], src_n[3];
  uint64_t seed;
  double noise;
  int open[3];           // open x / y / z faces (copy-out boundary)
  int keep_p;            // previous pressure as the initial guess
  double tol;
  int max_iters, criterion;
};

// Per-step statistics row of one plume.
struct BStat {
  int iter, converged, done, broke, wave_err, bodies;
  double rr, bb, maxR;
};

constexpr int kMaxGroups = 4;  // CG groups: independent lockstep loops, parallel graph branches

// Batch-wide control word (device memory).
struct BCtl {
  int parity;                 // which density/heat buffer is current
  int step_index;             // noise key of the next step's source
  int step_local;             // statistics row of the next step
  int bodies[kMaxGroups];     // CG-loop bodies each group ran in this step
  int max_iters;              // largest per-plume iteration cap (loop bound)
  int n;
  BStat* stats;               // [rows][n]
  const int* group_of;        // [n] each plume's CG group
};

// A stage's block table: virtual block v of the stage belongs to plume
// inst[v] and is block (v - first[inst[v]]) of that plume's count[inst[v]];
// `total` virtual blocks in all.
struct DomMap {
  const int* inst;
  const int* first;
  const int* count;
  int total;
};

template <typename T>
__device__ __forceinline__ const BPlume<T>& locate(const BPlume<T>* P, const DomMap& m, int v, Blk& b) {
  const int i = __ldg(m.inst + v);
  b.id = v - __ldg(m.first + i);
  b.n = __ldg(m.count + i);
  return P[i];
}

// Every stage kernel walks the stage's virtual blocks in strides of its grid,
// running the kernel body for each exactly as one block of a launch with one
// block per virtual block would (the bodies keep their block-level barriers
// and per-plume reductions).  So the same kernels run either with one block
// per virtual block or as a persistent launch whose grid holds as many blocks
// as stay resident (plume_batch_options.persistent).

// ------------------------------------------------------------ stage kernels
template <typename T>
__global__ void kb_source(const BPlume<T>* P, DomMap m, const BCtl* ctl) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    const int par = ctl->parity;
    source_box_body<T>(b, p.dens[par], p.heat[par], p.g, p.src_lo[0], p.src_lo[1], p.src_lo[2], p.src_n[0],
                       p.src_n[1], p.src_n[2], p.seed, ctl->step_index, p.noise);
  }
}

template <typename T>
__global__ void kb_forces(const BPlume<T>* P, DomMap m, const BCtl* ctl) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    const int par = ctl->parity;
    forces_body<T>(b, p.g, p.vel, p.dens[par], p.heat[par], V3<T>{}, p.c, 0);
  }
}

// the neighbour stencils: 2.5D tiles of zc planes (tile_kernels.cuh)
template <typename T>
__global__ void __launch_bounds__(kTileThreads) kb_vort1(const BPlume<T>* P, DomMap m, int zc) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    if (!p.c.has_vort) continue;  // addVorticity returns early when eps <= 0
    vort1_tile_body<T>(b, p.g, p.vel, p.vort, p.mag, p.c, zc);
  }
}

template <typename T>
__global__ void __launch_bounds__(kTileThreads) kb_vort2(const BPlume<T>* P, DomMap m, int zc) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    if (!p.c.has_vort) continue;
    vort2_tile_body<T>(b, p.g, p.vel, p.vort, p.mag, V3<T>{}, p.c, 0, zc);
  }
}

// mode 1 before advection (copyBorder on open axes), 2 before projection
// (setNeumann on open axes); closed axes are zeroed
template <typename T>
__global__ void kb_face_bc(const BPlume<T>* P, DomMap m, int mode) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    face_bc_body<T>(b, p.g, p.vel, p.open[0] ? mode : 0, p.open[1] ? mode : 0, p.open[2] ? mode : 0);
  }
}

// velocity, density and heat advected from the current buffers into tmp and
// the other density/heat buffers
template <typename T>
__global__ void kb_advect(const BPlume<T>* P, DomMap m, const BCtl* ctl) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    const int par = ctl->parity;
    advect_body<T>(b, p.g, p.c, p.vel, p.dens[par], p.heat[par], p.tmp, p.dens[par ^ 1], p.heat[par ^ 1],
                   V3<T>{}, 0, p.open[0], p.open[1], p.open[2], 1);
  }
}

// damping from tmp back into the velocity planes
template <typename T>
__global__ void __launch_bounds__(kTileThreads) kb_damping(const BPlume<T>* P, DomMap m, int zc) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    damping_tile_body<T>(b, p.g, p.c, p.tmp, p.vel, V3<T>{}, 0, zc);
  }
}

template <typename T>
__global__ void __launch_bounds__(kTileThreads) kb_divergence(const BPlume<T>* P, DomMap m, int zc) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    divergence_tile_body<T>(b, p.g, p.c, p.vel, p.div, p.pres, p.keep_p, zc);
  }
}

template <typename T>
__global__ void kb_copy_border(const BPlume<T>* P, DomMap m) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    copy_border_all_body<T>(b, p.g, p.pres);
  }
}

// right side and initial guess into the skewed layout
template <typename T>
__global__ void kb_to_skew(const BPlume<T>* P, DomMap m) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    to_skew_body<T, T>(b, p.g, p.k, p.div, p.sb);
    to_skew_body<T, T>(b, p.g, p.k, p.pres, p.sx);
  }
}

template <typename T>
__global__ void kb_cgs_init(const BPlume<T>* P, DomMap m) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    cgs_init_body<T>(b, p.g, p.k, p.sb, p.sx, p.sr, p.st, p.part, p.tol, p.max_iters, p.criterion,
                     p.keep_p ? 0 : 1);
  }
}

template <typename T>
__global__ void kb_cgs_init2(const BPlume<T>* P, DomMap m) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    cgs_init2_body<T>(b, p.k, p.sr, p.sz, (T*)nullptr, p.st, p.part);
  }
}

// CG iteration j: direction d[j+1 mod 2] = z + beta d[j mod 2], q = A d,
// marching tiles of zc planes
template <typename T>
__global__ void __launch_bounds__(256, 4) kb_spmv_dir(const BPlume<T>* P, DomMap m, int flip, int zc) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    cgs_spmv_dir_march_body<T>(b, p.g, p.k, p.sz, p.sd[flip], p.sd[flip ^ 1], p.sq, p.st, p.part, zc);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) kb_axpy(const BPlume<T>* P, DomMap m, int flip) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    cgs_axpy_v_body<T>(b, p.k, p.sd[flip ^ 1], p.sq, p.sx, p.sr, p.st, p.part);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) kb_rz(const BPlume<T>* P, DomMap m) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    cgs_rz_v_body<T>(b, p.k, p.sr, p.sz, p.st, p.part);
  }
}

template <typename T>
__global__ void kb_from_skew(const BPlume<T>* P, DomMap m) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    from_skew_body<T>(b, p.g, p.k, p.sx, p.pres);
  }
}

template <typename T>
__global__ void __launch_bounds__(kTileThreads) kb_gradient(const BPlume<T>* P, DomMap m, int zc) {
  for (int v = (int)blockIdx.x; v < m.total; v += (int)gridDim.x) {
    Blk b;
    const BPlume<T>& p = locate(P, m, v, b);
    gradient_tile_body<T>(b, p.g, p.c, p.vel, p.pres, zc);
  }
}

// MIC sweep of one shape class: cluster c (nslabs CTAs) sweeps plume
// tab[c]'s vectors, exactly as k_mic_wave_cl does for a single plume.
template <typename T, int C, bool EXACT, bool BWD>
__global__ void __launch_bounds__(32 * 16) kb_wave(const WaveArgs<T>* tab, int nslabs) {
  mic_wave_cl_body<T, C, EXACT, BWD>(tab[blockIdx.x / nslabs]);
}

// Last node of a CG group's loop body: loop again while any of the group's
// plumes (`members`, `nm` of them) is not done.  The body count bounds the
// loop on the device as in the single-plume graph.
static __global__ void kb_continue(cudaGraphConditionalHandle h, const CgState* st, const int* members, int nm,
                                   BCtl* ctl, int group, int body) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int k = threadIdx.x; k < nm; k += blockDim.x)
    if (!st[members[k]].done) any = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->bodies[group] += 1;
    const bool more = any && ctl->bodies[group] * body <= ctl->max_iters + 64;
    cudaGraphSetConditional(h, more ? 1u : 0u);
  }
}

// End of a step: one statistics row, then flip the buffer parity and advance
// the source's step index.
static __global__ void kb_end_step(const CgState* st, BCtl* ctl) {
  const int n = ctl->n;
  BStat* row = ctl->stats + (size_t)ctl->step_local * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const CgState& s = st[i];
    BStat o;
    o.iter = s.iter;
    o.converged = s.converged;
    o.done = s.done;
    o.broke = s.broke;
    o.wave_err = s.wave_err;
    o.bodies = ctl->bodies[ctl->group_of[i]];
    o.rr = s.rr;
    o.bb = s.bb;
    o.maxR = s.maxR;
    row[i] = o;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->parity ^= 1;
    ctl->step_index += 1;
    ctl->step_local += 1;
    for (int g = 0; g < kMaxGroups; g++) ctl->bodies[g] = 0;
  }
}

// ------------------------------------------------------------- sweep launch
template <typename T, int C, bool EXACT, bool BWD>
cudaError_t launch_bwave_c(const WaveArgs<T>* tab, int nplumes, int nslabs, int BZ, size_t smem,
                           cudaStream_t s, int query, int* max_clusters) {
  void (*kf)(const WaveArgs<T>*, int) = kb_wave<T, C, EXACT, BWD>;
  static std::atomic<unsigned long long> attr_done;
  cudaError_t ea = once_per_device(attr_done, [&] {
    cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kf, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
  });
  if (ea != cudaSuccess) return ea;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nplumes * nslabs, 1, 1);
  cfg.blockDim = dim3(32 * BZ, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = nslabs;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (query) return cudaOccupancyMaxActiveClusters(max_clusters, (void*)kf, &cfg);
  return cudaLaunchKernelEx(&cfg, kf, tab, nslabs);
}

template <typename T, bool EXACT, bool BWD>
cudaError_t launch_bwave(int C, const WaveArgs<T>* tab, int nplumes, int nslabs, int BZ, size_t smem,
                         cudaStream_t s, int query = 0, int* max_clusters = nullptr) {
  switch (C) {
#define PL_BW_CASE(CC) \
  case CC: return launch_bwave_c<T, CC, EXACT, BWD>(tab, nplumes, nslabs, BZ, smem, s, query, max_clusters);
    PL_BW_CASE(1)
    PL_BW_CASE(2)
    PL_BW_CASE(3)
    PL_BW_CASE(4)
    PL_BW_CASE(5)
    PL_BW_CASE(6)
    PL_BW_CASE(7)
    PL_BW_CASE(8)
#undef PL_BW_CASE
    default: return cudaErrorInvalidValue;
  }
}

// ------------------------------------------------------------------ engine
template <typename T>
class BatchEngineT : public BatchEngine {
 public:
  BatchEngineT() {}
  ~BatchEngineT() override { release(); }
  std::string& last_error() override { return err_; }

  int init(const plume_params* ps, int n, const plume_batch_options& o) override {
    if (!ps || n < 1) return fail(PLUME_ERR_INVALID, "bad argument");
    opt_ = o;
    n_ = n;
    dev_ = ps[0].device;
    const int prec = std::is_same<T, double>::value ? PLUME_PREC_FP64 : PLUME_PREC_FP32;
    hp_.resize(n);
    for (int i = 0; i < n; i++) {
      int rc = plan_plume(i, ps[i], prec);
      if (rc != PLUME_OK) return rc;
    }
    PL_TRY(cudaSetDevice(dev_));
    PL_TRY(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev_));
    // measured on the 64-plume configuration: 1 / 2 / 3 / 4 groups gave
    // 3.96 / 4.38 / 4.39 / 4.51e8 cell-steps/s
    ngroups_ = opt_.groups > 0 ? std::min(opt_.groups, kMaxGroups) : (n >= 32 ? 4 : (n >= 8 ? 2 : 1));
    ngroups_ = std::max(1, std::min(ngroups_, n));
    persistent_ = opt_.persistent != 0;
    PL_TRY(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
    for (int g = 0; g < kMaxGroups; g++) {
      PL_TRY(cudaStreamCreateWithFlags(&sg_[g], cudaStreamNonBlocking));
      PL_TRY(cudaStreamCreateWithFlags(&sbody_[g], cudaStreamNonBlocking));
      PL_TRY(cudaEventCreateWithFlags(&gjoin_[g], cudaEventDisableTiming));
    }
    PL_TRY(cudaEventCreateWithFlags(&gfork_, cudaEventDisableTiming));
    for (auto* e : {&ev_[0], &ev_[1]}) PL_TRY(cudaEventCreate(e));
    int rc = allocate();
    if (rc == PLUME_OK) rc = build_diagonals();
    if (rc == PLUME_OK) rc = plan_classes();
    if (rc != PLUME_OK) return rc;
    // tile shapes: the cache, else timed on this GPU, else defaults
    tune_ = default_tuning();
    rc = apply_tuning(tune_);
    if (rc != PLUME_OK) return rc;
    if (opt_.tune) {
      cache_path_ = tune_cache_path(opt_.tune_cache);
      BatchTuning t;
      if (load_cached(t) && apply_tuning(t) == PLUME_OK) {
        tune_ = t;
      } else {
        err_.clear();  // a cache entry that no longer fits is re-timed
        rc = apply_tuning(tune_);
        if (rc == PLUME_OK) rc = autotune();
        if (rc != PLUME_OK) return rc;
        cache_written_ = write_tune_cache(cache_path_, signature(), tune_);
      }
    }
    PL_TRY(cudaStreamSynchronize(s_));
    if (opt_.graph) {
      graph_ok_ = build_graph();
      if (!graph_ok_) {
        graph_note_ = err_;
        err_.clear();
        (void)cudaGetLastError();
      }
    }
    return PLUME_OK;
  }

  int run(int32_t first_step, int32_t steps, double* seconds, plume_step_stats* stats) override {
    if (steps < 0) return fail(PLUME_ERR_INVALID, "negative step count");
    PL_TRY(cudaSetDevice(dev_));
    const auto t0 = std::chrono::steady_clock::now();
    if (steps == 0) {
      if (seconds) *seconds = 0.0;
      return PLUME_OK;
    }
    if (steps > stats_cap_) {
      if (stats_dev_) cudaFree(stats_dev_);
      stats_dev_ = nullptr;
      stats_cap_ = 0;
      cudaError_t e = cudaMalloc(&stats_dev_, (size_t)steps * n_ * sizeof(BStat));
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(PLUME_ERR_OOM, "device allocation of the statistics rows failed");
      }
      stats_cap_ = steps;
    }
    BCtl c = {};
    c.parity = parity_;
    c.step_index = first_step;
    c.step_local = 0;
    for (int g = 0; g < kMaxGroups; g++) c.bodies[g] = 0;
    c.max_iters = max_iters_all_;
    c.n = n_;
    c.stats = stats_dev_;
    c.group_of = group_of_dev_;
    *ctl_host_ = c;
    PL_TRY(cudaMemcpyAsync(ctl_, ctl_host_, sizeof(BCtl), cudaMemcpyHostToDevice, s_));
    PL_TRY(cudaEventRecord(ev_[0], s_));
    std::vector<int> host_launches;
    for (int k = 0; k < steps; k++) {
      if (graph_ok_) {
        PL_TRY(cudaGraphLaunch(exec_, s_));
      } else {
        int launched = 0;
        int rc = host_step(&launched);
        if (rc != PLUME_OK) return rc;
        host_launches.push_back(launched);
      }
    }
    PL_TRY(cudaEventRecord(ev_[1], s_));
    std::vector<BStat> rows((size_t)steps * n_);
    PL_TRY(cudaMemcpyAsync(rows.data(), stats_dev_, rows.size() * sizeof(BStat), cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaMemcpyAsync(ctl_host_, ctl_, sizeof(BCtl), cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    float ms = 0.f;
    PL_TRY(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    parity_ = ctl_host_->parity;
    total_steps_ += steps;
    last_ms_ = ms;
    int rc = PLUME_OK;
    for (int k = 0; k < steps; k++) {
      int launched = host_launches.empty() ? 0 : host_launches[k];
      if (graph_ok_) {  // the stencils, each group's set-up and loop bodies, the tail
        launched = prefix_launches_ + suffix_launches_;
        for (int g = 0; g < ngroups_; g++) {
          const int bodies = rows[(size_t)k * n_ + gmembers_[g][0]].bodies;
          launched += setup_launches_[g] + bodies * (kBody * iter_launches_[g] + 1);
        }
      }
      for (int i = 0; i < n_; i++) {
        const BStat& r = rows[(size_t)k * n_ + i];
        if (stats) {
          plume_step_stats& o = stats[(size_t)i * steps + k];
          memset(&o, 0, sizeof(o));
          o.iterations = r.iter;
          o.converged = r.converged;
          o.fallback = 0;
          o.launches = launched;
          o.max_residual = r.maxR;
          o.rel_residual = r.bb > 0.0 ? sqrt(r.rr) / sqrt(r.bb) : 0.0;
          o.rhs_norm = sqrt(r.bb);
          o.ms_total = ms / steps;
        }
        if (r.wave_err && rc == PLUME_OK) {
          char buf[160];
          snprintf(buf, sizeof(buf), "plume %d, step %d: MIC wavefront wait expired (code %d)", i,
                   first_step + k, r.wave_err);
          rc = fail(PLUME_ERR_TIMEOUT, buf);
        }
      }
    }
    return rc;
  }

  int download(int32_t i, int32_t field, double* dst, size_t n) override {
    if (i < 0 || i >= n_ || !dst) return fail(PLUME_ERR_INVALID, "bad instance or destination");
    PL_TRY(cudaSetDevice(dev_));
    const Host& h = hp_[i];
    const BPlume<T>& p = plumes_[i];
    const size_t N = (size_t)h.g.N;
    const T* planes[3] = {nullptr, nullptr, nullptr};
    int nc = 1;
    switch (field) {
      case PLUME_F_DENSITY: planes[0] = p.dens[parity_]; break;
      case PLUME_F_DENSITY_OLD: planes[0] = p.dens[parity_ ^ 1]; break;
      case PLUME_F_HEAT: planes[0] = p.heat[parity_]; break;
      case PLUME_F_HEAT_OLD: planes[0] = p.heat[parity_ ^ 1]; break;
      case PLUME_F_PRESSURE: planes[0] = p.pres; break;
      case PLUME_F_DIVERGENCE: planes[0] = p.div; break;
      case PLUME_F_VELOCITY:
        planes[0] = p.vel.x;
        planes[1] = p.vel.y;
        planes[2] = p.vel.z;
        nc = 3;
        break;
      default:
        return fail(PLUME_ERR_STATE, "the fused batch keeps density, heat, pressure, divergence and velocity");
    }
    if (n != N * nc) return fail(PLUME_ERR_INVALID, nc == 3 ? "vector field needs 3N doubles" : "scalar field needs N doubles");
    std::vector<T> buf(N * nc);
    for (int c = 0; c < nc; c++)
      PL_TRY(cudaMemcpyAsync(buf.data() + c * N, planes[c], N * sizeof(T), cudaMemcpyDeviceToHost, s_));
    PL_TRY(cudaStreamSynchronize(s_));
    for (size_t cell = 0; cell < N; cell++)
      for (int c = 0; c < nc; c++) dst[cell * nc + c] = (double)buf[c * N + cell];
    return PLUME_OK;
  }

  std::string tuning_json() const override {
    std::string s = "{\"signature\": \"" + signature() + "\", \"cells_epb\": " + std::to_string(tune_.cells_epb) +
                    ", \"vec_epb\": " + std::to_string(tune_.vec_epb) + ", \"spmv_zc\": " +
                    std::to_string(tune_.spmv_zc) + ", \"tile_zc\": " + std::to_string(tune_.tile_zc) +
                    ", \"classes\": [";
    for (size_t c = 0; c < cls_.size(); c++) {
      const Class& k = cls_[c];
      s += (c ? ", " : "");
      s += "{\"group\": " + std::to_string(k.group) + ", \"cells_per_lane\": " + std::to_string(k.C) +
           ", \"nz\": " + std::to_string(k.nz) +
           ", \"plumes\": " + std::to_string(k.members.size()) + ", \"bz\": " + std::to_string(k.BZ) +
           ", \"pf\": " + std::to_string(k.PF) + ", \"slabs\": " + std::to_string(k.nslabs) +
           ", \"smem\": " + std::to_string(k.smem) + ", \"shape_candidates\": [";
      for (size_t j = 0; j < k.shapes.size(); j++)
        s += (j ? ", [" : "[") + std::to_string(k.shapes[j].first) + ", " + std::to_string(k.shapes[j].second) +
             ", " + std::to_string(k.resident[j]) + "]";
      s += "]}";
    }
    s += "], \"from_cache\": " + std::string(tune_.from_cache ? "true" : "false") +
         ", \"timed\": " + std::string(tune_.timed ? "true" : "false") +
         ", \"cache_written\": " + std::string(cache_written_ ? "true" : "false") +
         ", \"graph\": " + std::string(graph_ok_ ? "true" : "false") + ", \"groups\": " + std::to_string(ngroups_) +
         ", \"persistent\": " + std::string(persistent_ ? "true" : "false") +
         ", \"launches_per_step\": {\"stencils\": " + std::to_string(prefix_launches_) + ", \"per_cg_iteration\": [";
    for (int g = 0; g < ngroups_; g++) s += (g ? ", " : "") + std::to_string(iter_launches_[g]);
    s += "], \"suffix\": " + std::to_string(suffix_launches_) + "}";
    if (!graph_note_.empty()) s += ", \"graph_note\": \"" + sanitize(graph_note_) + "\"";
    if (!tune_log_.empty()) s += ", \"timings\": {" + tune_log_ + "}";
    return s + "}";
  }

 private:
  enum { D_CELLS, D_FACES, D_SRC, D_SKEW, D_RED, D_VEC, D_ROWS, D_TILES, D_COUNT };
  static constexpr int kThreads = 256;
  static constexpr int kBody = 16;  // CG iterations per graph-loop body (even: directions swap back)
  static constexpr int kKinds = 9;  // skewed vectors per plume
  static constexpr int kPlanes = 16;  // natural-layout planes per plume

  struct Host {
    plume_params p;
    Grid g;
    Skew k;
    StepConsts<T> c;
    int cls = 0;
    int group = 0;  // CG group
  };
  struct Class {
    int group = 0;
    int C = 1, nz = 1, W = 32;
    std::vector<int> members;
    // (slab height, ring depth) pairs that fit: nslabs <= 16, shared memory,
    // at least one cluster resident
    std::vector<std::pair<int, int>> shapes;
    std::vector<int> resident;  // clusters of each shape resident at once (occupancy query)
    int BZ = 4, PF = kWavePF, nslabs = 1;
    size_t smem = 0;
    WaveArgs<T>* tab = nullptr;  // [2][members]: forward, then backward
  };

  static std::string sanitize(const std::string& in) {
    std::string s = in;
    for (char& ch : s)
      if (ch == '"' || ch == '\\' || (unsigned char)ch < 32) ch = '_';
    return s;
  }
  static size_t align(size_t b) { return (b + 255) & ~(size_t)255; }

  int fail(int code, const std::string& msg) {
    err_ = msg;
    return code;
  }
  int fail_cuda(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    (void)cudaGetLastError();
    return fail(PLUME_ERR_CUDA, buf);
  }

  // Grid, solver layout and step constants of plume i, as the single-plume
  // engine derives them (EngineT::init, set_consts, init_solver).
  int plan_plume(int i, const plume_params& p, int prec) {
    char pre[48];
    snprintf(pre, sizeof(pre), "plume %d: ", i);
    const std::string P = pre;
    if (p.abi_version != PLUME_ABI_VERSION) return fail(PLUME_ERR_INVALID, P + "abi_version mismatch");
    if (p.device != dev_) return fail(PLUME_ERR_UNSUPPORTED, P + "every plume of a fused batch must be on one device");
    if (p.precision != prec) return fail(PLUME_ERR_UNSUPPORTED, P + "every plume of a fused batch must have one precision");
    for (int k = 0; k < 3; k++)
      if (p.res[k] < 4) return fail(PLUME_ERR_INVALID, P + "every grid dimension must be >= 4");
    const long long N = (long long)p.res[0] * p.res[1] * p.res[2];
    if (N > (1ll << 30)) return fail(PLUME_ERR_INVALID, P + "grid larger than 2^30 cells");
    for (int k = 0; k < 6; k++)
      if (p.bc[k] != 0 && p.bc[k] != 1) return fail(PLUME_ERR_INVALID, P + "bc flags must be 0 or 1");
    if (p.criterion != PLUME_CRIT_REFERENCE && p.criterion != PLUME_CRIT_REL2)
      return fail(PLUME_ERR_INVALID, P + "unknown criterion");
    if (p.source != PLUME_SRC_BOX && p.source != PLUME_SRC_NONE)
      return fail(PLUME_ERR_UNSUPPORTED, P + "the fused batch takes a box source or none");
    if (p.source == PLUME_SRC_BOX)
      for (int k = 0; k < 3; k++)
        if (p.box_lo[k] < 0 || p.box_hi[k] > p.res[k] || p.box_lo[k] > p.box_hi[k])
          return fail(PLUME_ERR_INVALID, P + "source box outside the grid");
    if (p.warm_start != PLUME_WARM_ZERO && p.warm_start != PLUME_WARM_PREVIOUS)
      return fail(PLUME_ERR_UNSUPPORTED, P + "the fused batch takes warm start ZERO or PREVIOUS");
    if (p.preconditioner != PLUME_PRECOND_MIC)
      return fail(PLUME_ERR_UNSUPPORTED, P + "the fused batch uses the MIC preconditioner");
    if (p.max_iters < 0) return fail(PLUME_ERR_INVALID, P + "negative iteration cap");
    Host& h = hp_[i];
    h.p = p;
    Grid& g = h.g;
    g.X = p.res[0];
    g.Y = p.res[1];
    g.Z = p.res[2];
    g.slab = g.X * g.Y;
    g.N = (int)N;
    g.nx = g.X - 2;
    g.ny = g.Y - 2;
    g.nz = g.Z - 2;
    g.nint = g.nx * g.ny * g.nz;
    for (int k = 0; k < 6; k++) g.wall[k] = p.bc[k];
    Skew& k = h.k;
    k.nx = g.nx;
    k.ny = g.ny;
    k.nz = g.nz;
    k.C = (g.nx + 31) / 32;
    if (k.C > 8) return fail(PLUME_ERR_UNSUPPORTED, P + "x resolution above 258 cells");
    if (g.nz > 256) return fail(PLUME_ERR_UNSUPPORTED, P + "z resolution above 258 cells");
    k.W = 32 * k.C;
    k.R = g.ny + 31;
    k.plane = (long long)k.R * k.W;
    k.total = (long long)g.nz * k.plane;
    if (k.total >= (1ll << 31)) return fail(PLUME_ERR_UNSUPPORTED, P + "grid too large for the solver");
    int maxRes = g.X > g.Y ? g.X : g.Y;
    maxRes = g.Z > maxRes ? g.Z : maxRes;
    const double dx = 1.0f / (double)maxRes;  // FLUID_3D_MIC.cpp:46
    const double dt = p.dt;
    StepConsts<T>& c = h.c;
    c.dt = (T)dt;
    c.beta = (T)p.buoyancy;
    c.eps = (T)p.vorticity_eps;
    c.dx = (T)dx;
    c.gridSize = (T)(0.5 / dx);
    c.oneOverDx = (T)(1.0 / dx);
    c.dt0 = (T)(dt / dx);
    c.divc = (T)(-dx * 0.5);
    c.wMinus = (T)(1.0 - p.damping_w);
    c.sixth = (T)((1. / 6.) * p.damping_w);
    c.xHi = (T)(g.X - 2.5);
    c.yHi = (T)(g.Y - 2.5);
    c.zHi = (T)(g.Z - 2.5);
    c.has_vort = p.vorticity_eps > 0.0 ? 1 : 0;
    c.has_beta = p.buoyancy != 0.0 ? 1 : 0;
    max_iters_all_ = std::max(max_iters_all_, p.max_iters);
    return PLUME_OK;
  }

  // One pool: natural planes of every plume, then the skewed vectors kind by
  // kind, the CG states and the reduction partials.
  int allocate() {
    size_t nat = 0, sk = 0;
    std::vector<size_t> nat_off(n_), sk_off(n_);
    for (int i = 0; i < n_; i++) {
      nat_off[i] = nat;
      nat += (size_t)kPlanes * align((size_t)hp_[i].g.N * sizeof(T));
      sk_off[i] = sk;  // elements; every plume's total is a multiple of 32
      sk += (size_t)hp_[i].k.total;
    }
    const size_t kind_bytes = align(sk * sizeof(T));
    const size_t bytes = align(nat) + kKinds * kind_bytes + align((size_t)n_ * sizeof(CgState)) +
                         align((size_t)n_ * 4 * kRedBlocks * sizeof(double)) + align(sizeof(BCtl));
    cudaError_t e = cudaMalloc(&pool_, bytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(PLUME_ERR_OOM, "device allocation of the batch pool failed");
    }
    PL_TRY(cudaMemsetAsync(pool_, 0, bytes, s_));
    char* skb = pool_ + align(nat);
    kind_base_ = skb;
    kind_bytes_ = kind_bytes;
    st_ = (CgState*)(skb + kKinds * kind_bytes);
    part_ = (double*)((char*)st_ + align((size_t)n_ * sizeof(CgState)));
    ctl_ = (BCtl*)((char*)part_ + align((size_t)n_ * 4 * kRedBlocks * sizeof(double)));
    PL_TRY(cudaMallocHost(&ctl_host_, sizeof(BCtl)));
    plumes_.resize(n_);
    for (int i = 0; i < n_; i++) {
      const Host& h = hp_[i];
      BPlume<T>& p = plumes_[i];
      p.g = h.g;
      p.k = h.k;
      p.c = h.c;
      char* cur = pool_ + nat_off[i];
      auto plane = [&]() {
        T* r = (T*)cur;
        cur += align((size_t)h.g.N * sizeof(T));
        return r;
      };
      p.vel = V3<T>{plane(), plane(), plane()};
      p.tmp = V3<T>{plane(), plane(), plane()};
      p.vort = V3<T>{plane(), plane(), plane()};
      p.dens[0] = plane();
      p.dens[1] = plane();
      p.heat[0] = plane();
      p.heat[1] = plane();
      p.pres = plane();
      p.div = plane();
      p.mag = plane();
      T** kinds[kKinds] = {&p.sb, &p.sx, &p.sr, &p.sq, &p.sqf, &p.sz, &p.sP, &p.sd[0], &p.sd[1]};
      for (int k = 0; k < kKinds; k++) *kinds[k] = (T*)(skb + k * kind_bytes) + sk_off[i];
      p.st = st_ + i;
      p.part = part_ + (size_t)i * 4 * kRedBlocks;
      const plume_params& q = h.p;
      const bool box = q.source == PLUME_SRC_BOX;
      for (int k = 0; k < 3; k++) {
        p.src_lo[k] = box ? q.box_lo[k] : 0;
        p.src_n[k] = box ? q.box_hi[k] - q.box_lo[k] : 0;
      }
      p.seed = q.seed;
      p.noise = q.source_noise;
      p.open[0] = q.bc[2] == 0;
      p.open[1] = q.bc[4] == 0;
      p.open[2] = q.bc[0] == 0;
      p.keep_p = q.warm_start == PLUME_WARM_PREVIOUS ? 1 : 0;
      p.tol = q.tol;
      p.max_iters = q.max_iters;
      p.criterion = q.criterion;
    }
    e = cudaMalloc(&P_dev_, (size_t)n_ * sizeof(BPlume<T>));
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(PLUME_ERR_OOM, "device allocation of the plume table failed");
    }
    PL_TRY(cudaMemcpyAsync(P_dev_, plumes_.data(), (size_t)n_ * sizeof(BPlume<T>), cudaMemcpyHostToDevice, s_));
    return PLUME_OK;
  }

  // Every plume's MIC(0) diagonal, built in FP64 once (the walls never
  // change) and stored skewed: P for the FP64 sweeps, P^2 rounded once for the
  // FP32 sweeps (k_diag_to_skew).
  int build_diagonals() {
    int maxN = 0;
    for (const Host& h : hp_) maxN = std::max(maxN, h.g.N);
    double* P64 = nullptr;
    cudaError_t e = cudaMalloc(&P64, (size_t)maxN * sizeof(double));
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(PLUME_ERR_OOM, "device allocation of the diagonal scratch failed");
    }
    int rc = PLUME_OK;
    for (int i = 0; i < n_ && rc == PLUME_OK; i++) {
      const Host& h = hp_[i];
      const BPlume<T>& p = plumes_[i];
      e = cudaMemsetAsync(P64, 0, (size_t)h.g.N * sizeof(double), s_);
      if (e == cudaSuccess) e = build_mic_diagonal(h.g, P64, h.p.mic_tau, h.p.mic_sigma, s_);
      if (e == cudaSuccess) {
        k_diag_to_skew<T><<<grid_for(h.k.total), 256, 0, s_>>>(h.g, h.k, P64, p.sP,
                                                               std::is_same<T, double>::value ? 0 : 1);
        e = cudaGetLastError();
      }
      if (e != cudaSuccess) rc = fail_cuda(e, "MIC diagonal", __FILE__, __LINE__);
    }
    cudaError_t e2 = cudaStreamSynchronize(s_);
    cudaFree(P64);
    if (rc == PLUME_OK && e2 != cudaSuccess) rc = fail_cuda(e2, "MIC diagonal", __FILE__, __LINE__);
    return rc;
  }

  // CG groups and the shape classes of the sweeps.  The plumes of each shape
  // (cells per lane, depth) are dealt to the groups in turn, so every group
  // holds a like share of every shape; a class is the plumes of one shape in
  // one group.
  int plan_classes() {
    std::map<std::pair<int, int>, int> dealt;
    for (int i = 0; i < n_; i++) hp_[i].group = dealt[std::make_pair(hp_[i].k.C, hp_[i].g.nz)]++ % ngroups_;
    std::map<std::array<int, 3>, int> idx;
    for (int i = 0; i < n_; i++) {
      const std::array<int, 3> key = {hp_[i].group, hp_[i].k.C, hp_[i].g.nz};
      auto it = idx.find(key);
      if (it == idx.end()) {
        it = idx.emplace(key, (int)cls_.size()).first;
        Class c;
        c.group = key[0];
        c.C = key[1];
        c.nz = key[2];
        c.W = 32 * c.C;
        cls_.push_back(c);
      }
      hp_[i].cls = it->second;
      cls_[it->second].members.push_back(i);
    }
    std::vector<int> group_of(n_), members;
    for (int g = 0; g < ngroups_; g++) {
      gmembers_[g].clear();
      gcls_[g].clear();
      gmem_off_[g] = (int)members.size();
      for (int i = 0; i < n_; i++)
        if (hp_[i].group == g) {
          gmembers_[g].push_back(i);
          members.push_back(i);
        }
      for (size_t ci = 0; ci < cls_.size(); ci++)
        if (cls_[ci].group == g) gcls_[g].push_back((int)ci);
    }
    for (int i = 0; i < n_; i++) group_of[i] = hp_[i].group;
    cudaError_t ea = cudaMalloc(&gidx_dev_, 2 * (size_t)n_ * sizeof(int));
    if (ea != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(PLUME_ERR_OOM, "device allocation of the group tables failed");
    }
    group_of_dev_ = gidx_dev_;
    gmem_dev_ = gidx_dev_ + n_;
    PL_TRY(cudaMemcpyAsync(group_of_dev_, group_of.data(), (size_t)n_ * sizeof(int), cudaMemcpyHostToDevice, s_));
    PL_TRY(cudaMemcpyAsync(gmem_dev_, members.data(), (size_t)n_ * sizeof(int), cudaMemcpyHostToDevice, s_));
    constexpr bool exact = std::is_same<T, double>::value;
    for (size_t ci = 0; ci < cls_.size(); ci++) {
      Class& c = cls_[ci];
      cudaError_t e = cudaMalloc(&c.tab, 2 * c.members.size() * sizeof(WaveArgs<T>));
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(PLUME_ERR_OOM, "device allocation of the sweep tables failed");
      }
      for (int pf : {kWavePF, 2}) {
        int last_ns = -1;
        for (int bz = (c.nz + 15) / 16; bz <= 16; bz++) {
          const int ns = (c.nz + bz - 1) / bz;
          // a taller slab that leaves the slab count unchanged only idles warps
          if (ns > 16 || ns == last_ns) continue;
          const size_t sm = wave_smem_bytes<T>(bz, c.W, pf);
          if (sm > 227 * 1024) continue;
          int maxc = 0;
          e = launch_bwave<T, exact, false>(c.C, c.tab, 1, ns, bz, sm, s_, 1, &maxc);
          (void)cudaGetLastError();
          if (e != cudaSuccess || maxc < 1) continue;
          c.shapes.emplace_back(bz, pf);
          c.resident.push_back(maxc);
          last_ns = ns;
        }
      }
      if (c.shapes.empty()) {
        char buf[160];
        snprintf(buf, sizeof(buf),
                 "plume %d: no cluster shape fits its MIC sweep (cells per lane %d, depth %d)", c.members[0],
                 c.C, c.nz);
        return fail(PLUME_ERR_UNSUPPORTED, buf);
      }
    }
    // parallel branches for every class but the first
    side_.resize(cls_.size());
    for (auto& set : side_)
      for (auto& st : set) {
        PL_TRY(cudaStreamCreateWithFlags(&st.s, cudaStreamNonBlocking));
        PL_TRY(cudaEventCreateWithFlags(&st.join, cudaEventDisableTiming));
      }
    for (auto& set : fork_)
      for (auto& e : set) PL_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return PLUME_OK;
  }

  BatchTuning default_tuning() const {
    BatchTuning t;
    for (const Class& c : cls_) {
      // the single-plume engine's shape: ring depth 3, slab height at least
      // 4 planes, at most 16 slabs
      const int want = std::max(4, (c.nz + 15) / 16);
      std::pair<int, int> pick = c.shapes.front();
      for (const auto& sh : c.shapes)
        if (sh.second == kWavePF && (pick.second != kWavePF || pick.first < want)) {
          pick = sh;
          if (sh.first >= want) break;
        }
      t.bz.push_back(pick.first);
      t.pf.push_back(pick.second);
    }
    return t;
  }

  // Block tables of every stage for tuning t, and the sweep classes' slab
  // heights and argument tables.
  int apply_tuning(const BatchTuning& t) {
    if (t.bz.size() != cls_.size() || t.pf.size() != cls_.size() || t.cells_epb < 1 || t.vec_epb < 1 ||
        t.spmv_zc < 1 || t.tile_zc < 1)
      return fail(PLUME_ERR_INVALID, "tuning does not match the batch");
    for (size_t ci = 0; ci < cls_.size(); ci++) {
      const auto& sh = cls_[ci].shapes;
      if (std::find(sh.begin(), sh.end(), std::make_pair(t.bz[ci], t.pf[ci])) == sh.end())
        return fail(PLUME_ERR_INVALID, "tuned sweep shape does not fit");
    }
    constexpr int NV = Vec16<T>::n;
    auto cdiv = [](long long a, long long b) { return (int)((a + b - 1) / b); };
    std::vector<int> host;
    // table gi = 0 covers every plume, gi = 1 + g the plumes of CG group g
    for (int gi = 0; gi <= ngroups_; gi++)
    for (int d = 0; d < D_COUNT; d++) {
      std::vector<int> cnt(n_), first(n_);
      int tot = 0;
      for (int i = 0; i < n_; i++) {
        const Grid& g = hp_[i].g;
        const Skew& k = hp_[i].k;
        long long c = 0;
        if (gi > 0 && hp_[i].group != gi - 1) {  // not in this table's group
          cnt[i] = 0;
          first[i] = tot;
          continue;
        }
        switch (d) {
          case D_CELLS: c = cdiv(g.N, (long long)kThreads * t.cells_epb); break;
          case D_FACES: c = cdiv(2ll * (g.Y * g.Z + g.X * g.Z + g.X * g.Y), kThreads); break;
          case D_SRC: {
            const BPlume<T>& p = plumes_[i];
            const long long nb = (long long)p.src_n[0] * p.src_n[1] * p.src_n[2];
            c = nb > 0 ? cdiv(nb, kThreads) : 0;
            break;
          }
          case D_SKEW: c = cdiv(k.total, (long long)kThreads * t.cells_epb); break;
          case D_RED: c = std::min<long long>(kRedBlocks, cdiv(k.total, (long long)kThreads * NV * t.vec_epb)); break;
          case D_VEC: c = std::min<long long>(kRedBlocks, cdiv(k.total / NV, (long long)kThreads * t.vec_epb)); break;
          case D_TILES: c = tile_grid(g, t.tile_zc).count(); break;
          case D_ROWS: {  // marching tiles: rows of the plane layout x zc planes
            const int rpb = kThreads / k.W;
            c = std::min<long long>(kRedBlocks, (long long)cdiv(k.R, rpb) * cdiv(k.nz, t.spmv_zc));
            break;
          }
        }
        if (d >= D_RED && c < 1) c = 1;  // every plume's reduction needs its last block
        cnt[i] = (int)c;
        first[i] = tot;
        tot += (int)c;
      }
      dom_total_[gi][d] = tot;
      dom_off_[gi][d][0] = (int)host.size();
      for (int i = 0; i < n_; i++)
        for (int b = 0; b < cnt[i]; b++) host.push_back(i);
      dom_off_[gi][d][1] = (int)host.size();
      host.insert(host.end(), first.begin(), first.end());
      dom_off_[gi][d][2] = (int)host.size();
      host.insert(host.end(), cnt.begin(), cnt.end());
    }
    if (dom_buf_) cudaFree(dom_buf_);
    dom_buf_ = nullptr;
    cudaError_t e = cudaMalloc(&dom_buf_, host.size() * sizeof(int));
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return fail(PLUME_ERR_OOM, "device allocation of the block tables failed");
    }
    PL_TRY(cudaMemcpyAsync(dom_buf_, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice, s_));
    dom_host_ = std::move(host);
    // sweep argument tables
    for (size_t ci = 0; ci < cls_.size(); ci++) {
      Class& c = cls_[ci];
      c.BZ = t.bz[ci];
      c.PF = t.pf[ci];
      c.nslabs = (c.nz + c.BZ - 1) / c.BZ;
      c.smem = wave_smem_bytes<T>(c.BZ, c.W, c.PF);
      std::vector<WaveArgs<T>> a(2 * c.members.size());
      for (size_t j = 0; j < c.members.size(); j++) {
        const BPlume<T>& p = plumes_[c.members[j]];
        for (int bwd = 0; bwd < 2; bwd++) {
          WaveArgs<T>& w = a[bwd * c.members.size() + j];
          w.P = p.sP;
          w.in = bwd ? p.sqf : p.sr;
          w.out = bwd ? p.sz : p.sqf;
          w.k = p.k;
          w.BZ = c.BZ;
          w.pf = c.PF;
          w.nslabs = c.nslabs;
          w.K = 8;
          w.backward = bwd;
          w.ctl = nullptr;       // the cluster path hands off inside the cluster
          w.progress = nullptr;  // and keeps no global flags
          w.st = p.st;
          w.gate = nullptr;
          w.gate_spins = 0;
        }
      }
      PL_TRY(cudaMemcpyAsync(c.tab, a.data(), a.size() * sizeof(WaveArgs<T>), cudaMemcpyHostToDevice, s_));
    }
    PL_TRY(cudaStreamSynchronize(s_));
    count_launches();
    return PLUME_OK;
  }

  DomMap dom(int d, int gi = 0) const {
    DomMap m;
    m.inst = dom_buf_ + dom_off_[gi][d][0];
    m.first = dom_buf_ + dom_off_[gi][d][1];
    m.count = dom_buf_ + dom_off_[gi][d][2];
    m.total = dom_total_[gi][d];
    return m;
  }

  // Blocks of kernel `f` resident on the whole GPU at kThreads per block
  // (the persistent grid), from the occupancy calculator, once per kernel.
  int resident_blocks(const void* f) {
    auto it = resident_.find(f);
    if (it != resident_.end()) return it->second;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, kThreads, 0) != cudaSuccess || per_sm < 1) {
      (void)cudaGetLastError();
      per_sm = 1;
    }
    const int r = per_sm * num_sms_;
    resident_[f] = r;
    return r;
  }

  void count_launches() {
    bool any_vort = false;
    for (const Host& h : hp_) any_vort = any_vort || h.c.has_vort;
    // source, forces, vorticity (two passes), face conditions, advection,
    // damping, face conditions, divergence, border copy, layout change
    prefix_launches_ = (dom_total_[0][D_SRC] > 0 ? 1 : 0) + 1 + (any_vort ? 2 : 0) + 7;
    for (int g = 0; g < ngroups_; g++) {
      const int ncls = (int)gcls_[g].size();
      setup_launches_[g] = 2 + 2 * ncls;  // two set-up kernels, the first sweeps
      iter_launches_[g] = 3 + 2 * ncls;
    }
    suffix_launches_ = 3;
  }

  // --------------------------------------------------------- launch helpers
  // one launch of `kern` over the plumes of table gi (0: all, 1 + g: group g)
  template <typename... K, typename... A>
  int launch_in(int gi, int d, void (*kern)(const BPlume<T>*, DomMap, K...), cudaStream_t s, A... args) {
    const int total = dom_total_[gi][d];
    if (total == 0) return PLUME_OK;
    // one block per virtual block, or (persistent) the resident blocks walking
    // them: measured on the 64-plume configuration the persistent grid was
    // 4-7 % slower (3.69 / 4.32e8 against 3.96 / 4.51e8 cell-steps/s with one
    // and four CG groups; a persistent grid per group left the groups' kernels
    // less room to interleave, and one sized to a share of the GPU per group
    // lost bandwidth: 3.68e8)
    const int grid = persistent_ ? std::min(total, resident_blocks((const void*)kern)) : total;
    kern<<<grid, kThreads, 0, s>>>(P_dev_, dom(d, gi), args...);
    PL_TRY(cudaGetLastError());
    return PLUME_OK;
  }
  template <typename... K, typename... A>
  int launch(int d, void (*kern)(const BPlume<T>*, DomMap, K...), cudaStream_t s, A... args) {
    return launch_in(0, d, kern, s, args...);
  }

  // One sweep direction for the classes `cls`: the first on stream s, the
  // others on their own streams forked from s and joined back (parallel
  // branches when captured).  `set` picks the side streams and fork event
  // (0: the step and timing, 1: the CG loop body), `slot` the group.
  int sweeps(cudaStream_t s, int bwd, int set, const std::vector<int>& cls, int slot) {
    constexpr bool exact = std::is_same<T, double>::value;
    const int ncls = (int)cls.size();
    const bool fork = ncls > 1;
    if (fork) PL_TRY(cudaEventRecord(fork_[set][slot], s));
    for (int j = 0; j < ncls; j++) {
      const int ci = cls[j];
      const Class& c = cls_[ci];
      cudaStream_t cs = s;
      if (fork && j > 0) {
        cs = side_[ci][set].s;
        PL_TRY(cudaStreamWaitEvent(cs, fork_[set][slot], 0));
      }
      const WaveArgs<T>* tab = c.tab + (bwd ? c.members.size() : 0);
      cudaError_t e = bwd ? launch_bwave<T, exact, true>(c.C, tab, (int)c.members.size(), c.nslabs, c.BZ, c.smem, cs)
                          : launch_bwave<T, exact, false>(c.C, tab, (int)c.members.size(), c.nslabs, c.BZ, c.smem, cs);
      PL_TRY(e);
      if (fork && j > 0) PL_TRY(cudaEventRecord(side_[ci][set].join, cs));
    }
    if (fork)
      for (int j = 1; j < ncls; j++) PL_TRY(cudaStreamWaitEvent(s, side_[cls[j]][set].join, 0));
    return PLUME_OK;
  }
  int sweep_class(cudaStream_t s, int bwd, int ci) { return sweeps(s, bwd, 0, std::vector<int>{ci}, 0); }

  // source .. projection's right side in the solver layout, every plume
  int enqueue_stencils(cudaStream_t s) {
    int rc = launch(D_SRC, kb_source<T>, s, (const BCtl*)ctl_);
    if (rc == PLUME_OK) rc = launch(D_CELLS, kb_forces<T>, s, (const BCtl*)ctl_);
    bool any_vort = false;
    for (const Host& h : hp_) any_vort = any_vort || h.c.has_vort;
    const int zt = tune_.tile_zc;
    if (rc == PLUME_OK && any_vort) rc = launch(D_TILES, kb_vort1<T>, s, zt);
    if (rc == PLUME_OK && any_vort) rc = launch(D_TILES, kb_vort2<T>, s, zt);
    if (rc == PLUME_OK) rc = launch(D_FACES, kb_face_bc<T>, s, 1);
    if (rc == PLUME_OK) rc = launch(D_CELLS, kb_advect<T>, s, (const BCtl*)ctl_);
    if (rc == PLUME_OK) rc = launch(D_TILES, kb_damping<T>, s, zt);
    if (rc == PLUME_OK) rc = launch(D_FACES, kb_face_bc<T>, s, 2);
    if (rc == PLUME_OK) rc = launch(D_TILES, kb_divergence<T>, s, zt);
    if (rc == PLUME_OK) rc = launch(D_FACES, kb_copy_border<T>, s);
    if (rc == PLUME_OK) rc = launch(D_SKEW, kb_to_skew<T>, s);
    if (rc != PLUME_OK) return rc;
    // the first direction is z itself: d_old = 0 with beta = 0
    PL_TRY(cudaMemsetAsync(plumes_[0].sd[0], 0, kind_bytes_, s));
    return PLUME_OK;
  }

  // CG set-up of group g: r = b - A x, the first preconditioner application, r.z
  int enqueue_setup(cudaStream_t s, int g) {
    int rc = launch_in(1 + g, D_RED, kb_cgs_init<T>, s);
    if (rc == PLUME_OK) rc = sweeps(s, 0, 0, gcls_[g], g);
    if (rc == PLUME_OK) rc = sweeps(s, 1, 0, gcls_[g], g);
    if (rc == PLUME_OK) rc = launch_in(1 + g, D_RED, kb_cgs_init2<T>, s);
    return rc;
  }

  // CG iteration j of group g (directions alternate between the two buffers)
  int enqueue_iter(cudaStream_t s, int j, int set, int g) {
    const int flip = j & 1, gi = 1 + g;
    int rc = launch_in(gi, D_ROWS, kb_spmv_dir<T>, s, flip, tune_.spmv_zc);
    if (rc == PLUME_OK) rc = launch_in(gi, D_VEC, kb_axpy<T>, s, flip);
    if (rc == PLUME_OK) rc = sweeps(s, 0, set, gcls_[g], g);
    if (rc == PLUME_OK) rc = sweeps(s, 1, set, gcls_[g], g);
    if (rc == PLUME_OK) rc = launch_in(gi, D_VEC, kb_rz<T>, s);
    return rc;
  }

  int enqueue_suffix(cudaStream_t s) {
    int rc = launch(D_SKEW, kb_from_skew<T>, s);
    if (rc == PLUME_OK) rc = launch(D_TILES, kb_gradient<T>, s, tune_.tile_zc);
    if (rc != PLUME_OK) return rc;
    kb_end_step<<<1, 256, 0, s>>>(st_, ctl_);
    PL_TRY(cudaGetLastError());
    return PLUME_OK;
  }

  // One step with the CG loops driven from the host (no graph): the groups
  // one after another on the main stream.  Each plume's arithmetic does not
  // depend on its group or on when its loop stops, so the results equal the
  // graph's bit for bit.
  int host_step(int* launched) {
    int rc = enqueue_stencils(s_);
    if (rc != PLUME_OK) return rc;
    *launched = prefix_launches_ + suffix_launches_;
    std::vector<CgState> hs(n_);
    for (int g = 0; g < ngroups_; g++) {
      rc = enqueue_setup(s_, g);
      if (rc != PLUME_OK) return rc;
      int j = 0, chunk = 4;
      for (;;) {
        for (int kk = 0; kk < chunk; kk++, j++) {
          rc = enqueue_iter(s_, j, 0, g);
          if (rc != PLUME_OK) return rc;
        }
        PL_TRY(cudaMemcpyAsync(hs.data(), st_, (size_t)n_ * sizeof(CgState), cudaMemcpyDeviceToHost, s_));
        PL_TRY(cudaStreamSynchronize(s_));
        bool all = true;
        for (int i : gmembers_[g]) all = all && hs[i].done;
        if (all || j > max_iters_all_ + 64) break;
        if (chunk < 16) chunk *= 2;
      }
      *launched += setup_launches_[g] + j * iter_launches_[g];
    }
    return enqueue_suffix(s_);
  }

  // Group g's CG set-up and loop on stream s (captured): the set-up kernels,
  // then a conditional-while node whose body -- kBody iterations and
  // kb_continue -- is captured on the group's body stream.
  cudaError_t capture_group(cudaStream_t s, int g, int* rc) {
    *rc = enqueue_setup(s, g);
    if (*rc != PLUME_OK) return cudaSuccess;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &nd);
    cudaGraphConditionalHandle h = 0;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &cp);
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCaptureToGraph(sbody_[g], cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return e;
    for (int j = 0; j < kBody && *rc == PLUME_OK; j++) *rc = enqueue_iter(sbody_[g], j, 1, g);
    if (*rc == PLUME_OK) {
      kb_continue<<<1, 256, 0, sbody_[g]>>>(h, st_, gmem_dev_ + gmem_off_[g], (int)gmembers_[g].size(), ctl_, g,
                                            kBody);
      e = cudaGetLastError();
    }
    cudaGraph_t body = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(sbody_[g], &body);
    return e == cudaSuccess ? e2 : e;
  }

  // The whole step as one graph: the stencils over every plume, the CG groups
  // as parallel branches (each its set-up and its own conditional-while
  // loop, so one group's latency-bound sweeps can run beside the other's
  // bandwidth-bound vector kernels), then the tail over every plume.
  bool build_graph() {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s_, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
      fail_cuda(e, "graph capture", __FILE__, __LINE__);
      return false;
    }
    int rc = enqueue_stencils(s_);
    if (rc == PLUME_OK && ngroups_ == 1) {
      e = capture_group(s_, 0, &rc);
    } else if (rc == PLUME_OK) {
      e = cudaEventRecord(gfork_, s_);
      for (int g = 0; g < ngroups_ && e == cudaSuccess && rc == PLUME_OK; g++) {
        e = cudaStreamWaitEvent(sg_[g], gfork_, 0);
        if (e == cudaSuccess) e = capture_group(sg_[g], g, &rc);
        if (e == cudaSuccess && rc == PLUME_OK) e = cudaEventRecord(gjoin_[g], sg_[g]);
      }
      for (int g = 0; g < ngroups_ && e == cudaSuccess && rc == PLUME_OK; g++) e = cudaStreamWaitEvent(s_, gjoin_[g], 0);
    }
    if (rc == PLUME_OK && e == cudaSuccess) rc = enqueue_suffix(s_);
    const cudaError_t e3 = cudaStreamEndCapture(s_, &graph);
    if (e == cudaSuccess) e = e3;
    if (rc == PLUME_OK && e == cudaSuccess) e = cudaGraphInstantiate(&exec_, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (rc != PLUME_OK) return false;
    if (e != cudaSuccess) {
      fail_cuda(e, "step graph", __FILE__, __LINE__);
      if (exec_) cudaGraphExecDestroy(exec_);
      exec_ = nullptr;
      return false;
    }
    return true;
  }

  // ----------------------------------------------------------- autotuning
  std::string signature() const {
    cudaDeviceProp prop;
    std::string name = "device";
    if (cudaGetDeviceProperties(&prop, dev_) == cudaSuccess) name = prop.name;
    std::map<std::string, int> grids;
    for (const Host& h : hp_)
      grids[std::to_string(h.g.X) + "x" + std::to_string(h.g.Y) + "x" + std::to_string(h.g.Z)] += 1;
    std::string s = sanitize(name) + "|sm" + std::to_string(num_sms_) + "|" +
                    (std::is_same<T, double>::value ? "fp64" : "fp32") + "|g" + std::to_string(ngroups_) + "|";
    bool first = true;
    for (const auto& g : grids) {
      s += (first ? "" : ",") + g.first + "*" + std::to_string(g.second);
      first = false;
    }
    return s;
  }

  bool load_cached(BatchTuning& t) {
    std::string text;
    if (cache_path_.empty() || !read_file(cache_path_, text)) return false;
    const std::string sig = signature();
    for (const auto& e : parse_tune_cache(text)) {
      if (e.first != sig) continue;
      BatchTuning c;
      if (!json_int(e.second, "cells_epb", c.cells_epb) || !json_int(e.second, "vec_epb", c.vec_epb) ||
          !json_int(e.second, "spmv_zc", c.spmv_zc) || !json_int(e.second, "tile_zc", c.tile_zc) ||
          !json_int_list(e.second, "bz", c.bz) ||
          !json_int_list(e.second, "pf", c.pf))
        return false;
      c.from_cache = true;
      t = c;
      return true;
    }
    return false;
  }

  // Best of `reps` event-timed runs of body() on the main stream, each after
  // the CG states are cleared (so no plume's kernels return early).
  template <typename F>
  int time_min(F&& body, int reps, float* best) {
    *best = 1e30f;
    for (int r = 0; r <= reps; r++) {  // the first run warms up
      PL_TRY(cudaMemsetAsync(st_, 0, (size_t)n_ * sizeof(CgState), s_));
      PL_TRY(cudaEventRecord(ev_[0], s_));
      const int rc = body();
      if (rc != PLUME_OK) return rc;
      PL_TRY(cudaEventRecord(ev_[1], s_));
      PL_TRY(cudaEventSynchronize(ev_[1]));
      float ms = 0.f;
      PL_TRY(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
      if (r > 0) *best = std::min(*best, ms);
    }
    return PLUME_OK;
  }

  // Times the candidates of each knob on this batch's own (all-zero) fields,
  // one knob at a time, and keeps the fastest.  The fields stay zero: every
  // timed stage maps zero to zero.
  int autotune() {
    BatchTuning t = tune_;
    std::string log;
    auto note = [&](const std::string& k, int v, float ms) {
      char buf[96];
      snprintf(buf, sizeof(buf), "%s\"%s=%d\": %.4f", log.empty() ? "" : ", ", k.c_str(), v, ms);
      log += buf;
    };
    const int reps = 3;
    // stencil and layout kernels
    {
      int best_v = t.cells_epb;
      float best = 1e30f;
      for (int v : {1, 2, 4}) {
        BatchTuning c = t;
        c.cells_epb = v;
        int rc = apply_tuning(c);
        if (rc != PLUME_OK) return rc;
        float ms = 0.f;
        rc = time_min(
            [&] {
              int r = launch(D_CELLS, kb_forces<T>, s_, (const BCtl*)ctl_);
              if (r == PLUME_OK) r = launch(D_CELLS, kb_advect<T>, s_, (const BCtl*)ctl_);
              if (r == PLUME_OK) r = launch(D_SKEW, kb_to_skew<T>, s_);
              return r;
            },
            reps, &ms);
        if (rc != PLUME_OK) return rc;
        note("cells_epb", v, ms);
        if (ms < best) {
          best = ms;
          best_v = v;
        }
      }
      t.cells_epb = best_v;
    }
    // neighbour stencils: planes per tile
    {
      int best_v = t.tile_zc;
      float best = 1e30f;
      for (int v : {2, 4, 8, 16}) {
        BatchTuning c = t;
        c.tile_zc = v;
        int rc = apply_tuning(c);
        if (rc != PLUME_OK) return rc;
        float ms = 0.f;
        rc = time_min(
            [&] {
              int r = launch(D_TILES, kb_vort1<T>, s_, v);
              if (r == PLUME_OK) r = launch(D_TILES, kb_vort2<T>, s_, v);
              if (r == PLUME_OK) r = launch(D_TILES, kb_damping<T>, s_, v);
              if (r == PLUME_OK) r = launch(D_TILES, kb_divergence<T>, s_, v);
              if (r == PLUME_OK) r = launch(D_TILES, kb_gradient<T>, s_, v);
              return r;
            },
            reps, &ms);
        if (rc != PLUME_OK) return rc;
        note("tile_zc", v, ms);
        if (ms < best) {
          best = ms;
          best_v = v;
        }
      }
      t.tile_zc = best_v;
    }
    // CG vector kernels
    {
      int best_v = t.vec_epb;
      float best = 1e30f;
      for (int v : {1, 2, 4, 8}) {
        BatchTuning c = t;
        c.vec_epb = v;
        int rc = apply_tuning(c);
        if (rc != PLUME_OK) return rc;
        float ms = 0.f;
        rc = time_min(
            [&] {
              int r = launch(D_VEC, kb_axpy<T>, s_, 0);
              if (r == PLUME_OK) r = launch(D_VEC, kb_rz<T>, s_);
              return r;
            },
            reps, &ms);
        if (rc != PLUME_OK) return rc;
        note("vec_epb", v, ms);
        if (ms < best) {
          best = ms;
          best_v = v;
        }
      }
      t.vec_epb = best_v;
    }
    {
      int best_v = t.spmv_zc;
      float best = 1e30f;
      for (int v : {8, 16, 32, 64}) {
        BatchTuning c = t;
        c.spmv_zc = v;
        int rc = apply_tuning(c);
        if (rc != PLUME_OK) return rc;
        float ms = 0.f;
        rc = time_min([&] { return launch(D_ROWS, kb_spmv_dir<T>, s_, 0, v); }, reps, &ms);
        if (rc != PLUME_OK) return rc;
        note("spmv_zc", v, ms);
        if (ms < best) {
          best = ms;
          best_v = v;
        }
      }
      t.spmv_zc = best_v;
    }
    // each sweep class's shape, the class timed alone
    for (size_t ci = 0; ci < cls_.size(); ci++) {
      std::pair<int, int> best_v(t.bz[ci], t.pf[ci]);
      float best = 1e30f;
      for (const auto& v : cls_[ci].shapes) {
        BatchTuning c = t;
        c.bz[ci] = v.first;
        c.pf[ci] = v.second;
        int rc = apply_tuning(c);
        if (rc != PLUME_OK) return rc;
        float ms = 0.f;
        rc = time_min(
            [&] {
              int r = sweep_class(s_, 0, (int)ci);
              if (r == PLUME_OK) r = sweep_class(s_, 1, (int)ci);
              return r;
            },
            reps, &ms);
        if (rc != PLUME_OK) return rc;
        note("class" + std::to_string(ci) + "_bz" + std::to_string(v.first) + "_pf", v.second, ms);
        if (ms < best) {
          best = ms;
          best_v = v;
        }
      }
      t.bz[ci] = best_v.first;
      t.pf[ci] = best_v.second;
    }
    t.timed = true;
    t.from_cache = false;
    int rc = apply_tuning(t);
    if (rc != PLUME_OK) return rc;
    PL_TRY(cudaMemsetAsync(st_, 0, (size_t)n_ * sizeof(CgState), s_));
    PL_TRY(cudaStreamSynchronize(s_));
    tune_ = t;
    tune_log_ = log;
    return PLUME_OK;
  }

  void release() {
    if (dev_ >= 0) cudaSetDevice(dev_);
    if (s_) cudaStreamSynchronize(s_);
    if (exec_) cudaGraphExecDestroy(exec_);
    for (Class& c : cls_)
      if (c.tab) cudaFree(c.tab);
    for (auto& set : side_)
      for (auto& st : set) {
        if (st.s) cudaStreamDestroy(st.s);
        if (st.join) cudaEventDestroy(st.join);
      }
    for (auto& set : fork_)
      for (auto& e : set)
        if (e) cudaEventDestroy(e);
    for (auto& e : ev_)
      if (e) cudaEventDestroy(e);
    if (dom_buf_) cudaFree(dom_buf_);
    if (stats_dev_) cudaFree(stats_dev_);
    if (P_dev_) cudaFree(P_dev_);
    if (pool_) cudaFree(pool_);
    if (ctl_host_) cudaFreeHost(ctl_host_);
    for (int g = 0; g < kMaxGroups; g++) {
      if (sbody_[g]) cudaStreamDestroy(sbody_[g]);
      if (sg_[g]) cudaStreamDestroy(sg_[g]);
      if (gjoin_[g]) cudaEventDestroy(gjoin_[g]);
      sbody_[g] = sg_[g] = nullptr;
      gjoin_[g] = nullptr;
    }
    if (gfork_) cudaEventDestroy(gfork_);
    gfork_ = nullptr;
    if (gidx_dev_) cudaFree(gidx_dev_);
    gidx_dev_ = nullptr;
    if (s_) cudaStreamDestroy(s_);
    exec_ = nullptr;
    cls_.clear();
    side_.clear();
    dom_buf_ = nullptr;
    stats_dev_ = nullptr;
    P_dev_ = nullptr;
    pool_ = nullptr;
    ctl_host_ = nullptr;
    s_ = nullptr;
  }

  struct Side {
    cudaStream_t s = nullptr;
    cudaEvent_t join = nullptr;
  };

  plume_batch_options opt_ = {};
  int n_ = 0, dev_ = -1, num_sms_ = 1;
  int max_iters_all_ = 0;
  int parity_ = 0;
  long long total_steps_ = 0;
  float last_ms_ = 0.f;
  std::vector<Host> hp_;
  std::vector<BPlume<T>> plumes_;
  std::vector<Class> cls_;
  std::vector<std::array<Side, 2>> side_;
  cudaEvent_t fork_[2][kMaxGroups] = {};
  cudaEvent_t ev_[2] = {nullptr, nullptr};
  cudaStream_t s_ = nullptr;
  // CG groups: the plumes and classes of each, their branch and body streams
  int ngroups_ = 1;
  std::vector<int> gmembers_[kMaxGroups], gcls_[kMaxGroups];
  int gmem_off_[kMaxGroups] = {};
  int* gidx_dev_ = nullptr;      // [2n]: each plume's group, then the groups' member lists
  int* group_of_dev_ = nullptr;
  int* gmem_dev_ = nullptr;
  cudaStream_t sg_[kMaxGroups] = {}, sbody_[kMaxGroups] = {};
  cudaEvent_t gfork_ = nullptr, gjoin_[kMaxGroups] = {};
  char* pool_ = nullptr;
  char* kind_base_ = nullptr;
  size_t kind_bytes_ = 0;
  CgState* st_ = nullptr;
  double* part_ = nullptr;
  BCtl* ctl_ = nullptr;
  BCtl* ctl_host_ = nullptr;
  BPlume<T>* P_dev_ = nullptr;
  int* dom_buf_ = nullptr;
  std::map<const void*, int> resident_;  // persistent grid per stage kernel
  bool persistent_ = false;
  std::vector<int> dom_host_;
  int dom_off_[kMaxGroups + 1][D_COUNT][3] = {};
  int dom_total_[kMaxGroups + 1][D_COUNT] = {};
  BStat* stats_dev_ = nullptr;
  int stats_cap_ = 0;
  cudaGraphExec_t exec_ = nullptr;
  bool graph_ok_ = false;
  std::string graph_note_;
  BatchTuning tune_;
  std::string tune_log_;
  std::string cache_path_;
  bool cache_written_ = false;
  int prefix_launches_ = 0, suffix_launches_ = 0;
  int setup_launches_[kMaxGroups] = {}, iter_launches_[kMaxGroups] = {};
  std::string err_;
};

}  // namespace plume
