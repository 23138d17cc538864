// wave.cuh -- persistent wavefront kernels for the MIC(0) triangular sweeps of
// FLUID_3D_MIC::applyMICPreconditioner (FLUID_3D_MIC.cpp:864-899), keeping the
// reference's lexicographic ordering (the same operator, not a red-black
// substitute).
//
// Skewed storage.  The solver's vectors hold only the interior cells.  Plane
// iz is stored as R = ny + 31 rows of W = 32*C values, cell (ix, iy) at row
// s = iy + ix/C, column ix.  A warp owns one plane; lane l owns the C cells
// ix in [l*C, l*C + C) and, at warp step t, the row iy = t - l (forward
// sweep).  Every dependency of the lexicographic recurrence is then local:
//   -x : the lane's previous cell, or lane l-1's last cell of the previous
//        step (one shuffle);
//   -y : the same lane's previous step (registers);
//   -z : the warp of plane iz-1 at the same step (a shared-memory ring, or the
//        slab's courier warp when iz-1 belongs to another CTA);
// and every step reads and writes exactly one contiguous row, streamed in by
// 1-D TMA bulk copies.  Padding cells (iy outside [0, ny), ix >= nx) hold
// zero input and zero diagonal, so they compute zero and stay zero.
//
// With EXACT, each cell evaluates the reference's expression in its order,
// ((r - (A.P).q) - (A.P).q) - (A.P).q times P, so the FP64 result is
// bit-identical to the serial sweep.  Without it (FP32 mode) the sum is
// reassociated so that only one multiply-add per cell lies on the x-chain.
//
// Slabs of BZ planes are handed out to CTAs in sweep order by a ticket, so a
// CTA only ever waits for slabs that are already running: no deadlock for any
// grid size.  Every wait is bounded; on expiry the kernel records an error
// word, waits (bounded) for its own copies in flight and returns.
#pragma once
#include <type_traits>
#include "common.cuh"
#include "solver_kernels.cuh"

namespace plume {

struct Skew {
  int C, W, R;   // cells per lane, row width (32*C), rows (ny + 31)
  int nx, ny, nz;
  long long plane;  // R*W
  long long total;  // nz*plane
};

__host__ __device__ inline long long skew_index(const Skew& k, int ix, int iy, int iz) {
  return (long long)iz * k.plane + (long long)(iy + ix / k.C) * k.W + ix;
}

constexpr int kWaveKB = 8;     // rows per TMA block (contiguous in the skewed layout)
constexpr int kWavePF = 3;     // TMA ring depth (blocks) of a single plume's sweep
constexpr int kWaveD = 8;      // inter-warp ring depth (steps)
static_assert(kWaveD == kWaveKB, "sweep_plane maps step u of a TMA block to ring slot u");
constexpr long long kSpinLimit = 1ll << 24;     // shared-memory polls (~0.3 s)
constexpr long long kSpinLimitSlow = 1ll << 21; // global-flag polls and TMA waits (~2 s)

enum WaveError {
  WAVE_OK = 0,
  WAVE_TIMEOUT_RING = 1,
  WAVE_TIMEOUT_TMA = 2,
  WAVE_TIMEOUT_FLAG = 3,
  WAVE_TIMEOUT_GATE = 4
};

template <typename T>
struct WaveArgs {
  const T* P;       // MIC diagonal, skewed
  const T* in;      // r (forward) or q (backward), skewed
  T* out;           // q (forward) or z (backward), skewed
  Skew k;
  int BZ;           // planes per slab (= compute warps per CTA)
  int nslabs;
  int K;            // rows per published progress step across slabs
  int backward;
  unsigned* ctl;    // [0] slab ticket, [1] exited CTAs
  int* progress;    // [nz] steps completed, for planes read by another slab
  CgState* st;      // skip when st->done; wave_err recorded here
  int pf = kWavePF; // TMA ring depth in blocks (2 or 3): 2 needs a third less
                    // shared memory, so more CTAs share an SM
  // Test hook for the bounded waits: when `gate` is set, one thread per CTA
  // first polls *gate (a device word that nothing sets) at most gate_spins
  // times, before any copy is issued; on expiry the CTA records
  // WAVE_TIMEOUT_GATE and skips its planes, so the sweep ends with nothing in
  // flight.  Null in normal runs.
  const int* gate = nullptr;
  long long gate_spins = 0;
};

// The entry gate of a sweep CTA (see WaveArgs::gate); false when it expired.
template <typename T>
__device__ inline bool wave_pass_gate(const WaveArgs<T>& a, int* failed) {
  if (!a.gate) return true;
  if (threadIdx.x == 0) {
    long long spins = 0;
    while (*((volatile const int*)a.gate) == 0) {
      if (++spins > a.gate_spins) {
        atomicCAS(&a.st->wave_err, 0, (int)WAVE_TIMEOUT_GATE);
        *((volatile int*)failed) = 1;
        break;
      }
    }
  }
  __syncthreads();
  return *((volatile int*)failed) == 0;
}

// ------------------------------------------------------------- PTX helpers
__device__ inline unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ inline void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ inline void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ inline bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}" : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ inline void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ inline void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ inline int ld_vol(const int* p) { return *((volatile const int*)p); }
__device__ inline void st_vol(int* p, int v) { *((volatile int*)p) = v; }

// Extra PTX for the ring hand-off: st.async writes a value into (possibly
// another CTA's) shared memory and signals that CTA's mbarrier with the bytes
// written (complete_tx).  The consumer arms each of its slot barriers itself
// -- one arrival with the expected byte count, at start and again right after
// each use of the slot -- and waits on the phase; a phase completes once the
// arrival and the bytes are both in, in either order.  So the producer's
// step sends nothing but the data, and no fence sits on its side either (a
// step never waits for its own global stores to drain).
__device__ inline void mbar_arm(uint64_t* bar, unsigned bytes) { mbar_expect_tx(bar, bytes); }

// Single-lane operations of the sweep step as predicated instructions rather
// than `if (lane == 0)` branches, so the warp never diverges and reconverges
// inside the step: arm a slot barrier; publish a counter to shared memory;
// issue one TMA block (arm its barrier with the bytes of both copies, then
// the two bulk copies).
__device__ inline void mbar_arm_if(bool pred, uint64_t* bar, unsigned bytes) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %2, 0;\n"
      " @p mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n}" ::"r"(smem_u32(bar)),
      "r"(bytes), "r"((int)pred)
      : "memory");
}
__device__ inline void st_shared_if(bool pred, int* dst, int v) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %2, 0;\n @p st.volatile.shared.u32 [%0], %1;\n}" ::"r"(
                   smem_u32(dst)),
               "r"(v), "r"((int)pred)
               : "memory");
}
__device__ inline void tma_pair_if(bool pred, uint64_t* bar, void* d0, const void* s0, void* d1, const void* s1,
                                   unsigned bytes) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %0, 0;\n"
      " @p mbarrier.arrive.expect_tx.shared::cta.b64 _, [%1], %2;\n"
      " @p cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%3], [%4], %6, [%1];\n"
      " @p cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%5], [%7], %6, [%1];\n}" ::"r"(
          (int)pred),
      "r"(smem_u32(bar)), "r"(2u * bytes), "r"(smem_u32(d0)), "l"(s0), "r"(smem_u32(d1)), "r"(bytes), "l"(s1)
      : "memory");
}
__device__ inline bool mbar_try_wait_cluster(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ inline void st_async(unsigned addr, float v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f32 [%0], %1, [%2];" ::"r"(addr),
               "f"(v), "r"(bar)
               : "memory");
}
__device__ inline void st_async(unsigned addr, double v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f64 [%0], %1, [%2];" ::"r"(addr),
               "d"(v), "r"(bar)
               : "memory");
}
__device__ inline void st_async4(unsigned addr, float a, float b, float c, float d, unsigned bar) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(addr),
      "f"(a), "f"(b), "f"(c), "f"(d), "r"(bar)
      : "memory");
}
__device__ inline void st_async2(unsigned addr, double a, double b, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, [%3];" ::"r"(addr),
               "d"(a), "d"(b), "r"(bar)
               : "memory");
}
__device__ inline void st_async2f(unsigned addr, float a, float b, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(addr),
               "f"(a), "f"(b), "r"(bar)
               : "memory");
}

// Values a lane keeps per ring row: C rounded up so that the lane's hand-off
// is whole vector stores (16 bytes, or 8 for a pair of floats, or one value),
// which is what the consumer's slot barrier counts per step; the padding is
// written as zero and never read.  The ring is internal to the sweep: the
// global vectors keep their W = 32*C rows.
__host__ __device__ constexpr int ring_cp(int C, int tsize) {
  return C == 1 ? 1 : (tsize == 4 ? (C == 2 ? 2 : ((C + 3) / 4) * 4) : ((C + 1) / 2) * 2);
}

// lane's C values -> its padded ring slice at shared::cluster address `dst`
// (aligned to the slice size)
template <typename T, int C>
__device__ inline void st_async_ring(unsigned dst, const T (&v)[C], unsigned bar) {
  constexpr int CP = ring_cp(C, sizeof(T));
  T w[CP];
#pragma unroll
  for (int j = 0; j < CP; j++) w[j] = j < C ? v[j] : T(0);
  if (sizeof(T) == 4 && CP % 4 == 0) {
#pragma unroll
    for (int j = 0; j < CP; j += 4)
      st_async4(dst + j * 4, (float)w[j], (float)w[j + 1], (float)w[j + 2], (float)w[j + 3], bar);
  } else if (sizeof(T) == 4 && CP == 2) {
    st_async2f(dst, (float)w[0], (float)w[1], bar);
  } else if (sizeof(T) == 8 && CP % 2 == 0) {
#pragma unroll
    for (int j = 0; j < CP; j += 2) st_async2(dst + j * 8, (double)w[j], (double)w[j + 1], bar);
  } else {
#pragma unroll
    for (int j = 0; j < CP; j++) st_async(dst + j * sizeof(T), w[j], bar);
  }
}

__device__ inline unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ inline void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ inline unsigned mapa_u32(const void* p, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ inline int ld_remote_relaxed(unsigned raddr) {
  int v;
  asm volatile("ld.relaxed.cluster.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(raddr) : "memory");
  return v;
}

// Shared-memory layout of one CTA (dynamic): see wave_smem_bytes().
template <typename T>
struct WaveSmem {
  T* tma;          // [BZ][PF][2][KB][W]  KB input rows, then KB diagonal rows
  uint64_t* bar;   // [BZ][PF]        TMA slot barriers
  T* ring;         // [BZ][D][32*CP]  ring r is read by compute warp r (CP = ring_cp)
  uint64_t* rbar;  // [BZ][D]         ring slot barriers (armed by the reader)
  int* prog;       // [BZ + 1]        steps consumed per compute warp; [BZ] courier fetch count
  int* misc;       // [4]             slab, failed
};

// Every region starts on a 128-byte boundary (16-byte vector accesses and
// bulk copies need at least 16; mbarrier counts differ in size per region).
__host__ __device__ inline size_t wave_al(size_t b) { return (b + 127) & ~(size_t)127; }

template <typename T>
__host__ __device__ inline size_t wave_smem_bytes(int BZ, int W, int pf = kWavePF) {
  size_t b = wave_al((size_t)BZ * pf * 2 * kWaveKB * W * sizeof(T));
  b += wave_al((size_t)BZ * pf * sizeof(uint64_t));
  b += wave_al((size_t)BZ * kWaveD * 32 * ring_cp(W / 32, (int)sizeof(T)) * sizeof(T));
  b += wave_al((size_t)BZ * kWaveD * sizeof(uint64_t));
  b += wave_al((size_t)(BZ + 1 + 4) * sizeof(int));
  return b;
}

template <typename T>
__device__ inline WaveSmem<T> wave_carve(char* base, int BZ, int W, int pf) {
  WaveSmem<T> s;
  s.tma = (T*)base;
  base += wave_al((size_t)BZ * pf * 2 * kWaveKB * W * sizeof(T));
  s.bar = (uint64_t*)base;
  base += wave_al((size_t)BZ * pf * sizeof(uint64_t));
  s.ring = (T*)base;
  base += wave_al((size_t)BZ * kWaveD * 32 * ring_cp(W / 32, (int)sizeof(T)) * sizeof(T));
  s.rbar = (uint64_t*)base;
  base += wave_al((size_t)BZ * kWaveD * sizeof(uint64_t));
  s.prog = (int*)base;
  s.misc = s.prog + BZ + 1;
  return s;
}

__device__ inline void wave_fail(CgState* st, int code, int* failed) {
  atomicCAS(&st->wave_err, 0, code);
  st_vol(failed, 1);
}

// A lane's C consecutive values from shared memory (16-byte loads when the
// row slice allows it).
template <typename T, int C>
__device__ inline void lds_row(const T* src, T (&v)[C]) {
  if (sizeof(T) == 4 && C % 4 == 0) {
#pragma unroll
    for (int j = 0; j < C; j += 4) {
      const float4 f = *reinterpret_cast<const float4*>(src + j);
      v[j] = (T)f.x;
      v[j + 1] = (T)f.y;
      v[j + 2] = (T)f.z;
      v[j + 3] = (T)f.w;
    }
  } else if (sizeof(T) == 8 && C % 2 == 0) {
#pragma unroll
    for (int j = 0; j < C; j += 2) {
      const double2 d = *reinterpret_cast<const double2*>(src + j);
      v[j] = (T)d.x;
      v[j + 1] = (T)d.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < C; j++) v[j] = src[j];
  }
}

// A lane's C values from its padded ring slice (ring_cp values, vector loads).
template <typename T, int C>
__device__ inline void lds_ring(const T* src, T (&v)[C]) {
  constexpr int CP = ring_cp(C, sizeof(T));
  T w[CP];
  if (sizeof(T) == 4 && CP == 2) {
    const float2 f = *reinterpret_cast<const float2*>(src);
    w[0] = (T)f.x;
    w[1] = (T)f.y;
  } else {
    lds_row<T, CP>(src, w);
  }
#pragma unroll
  for (int j = 0; j < C; j++) v[j] = w[j];
}

// Explicitly typed multiply-add: the generic overload set must never pick the
// FP64 form for FP32 operands (FP64 is a small fraction of FP32 on GB300).
__device__ inline float madd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ inline double madd(double a, double b, double c) { return __fma_rn(a, b, c); }

// One cell of the sweep.  With EXACT (FP64) p = P and the reference's
// expressions: forward t = ((r + wx) + wy) + wz, q = t*P, and the value
// handed to the +x/+y/+z neighbours is w = P*q, because the reference forms
// (A+ . P) . q = (-P) . q; backward t = ((q + P zx) + P zy) + P zz, z = t*P,
// and neighbours receive z itself.  Without EXACT (FP32) p = P^2 (the skewed
// diagonal holds the square) and the forward sweep writes w = P q in place of
// q: forward w = P^2 (r + wy + wz + wx); backward, from z = P (q + P S) with
// S = zx + zy + zz, z = w + P^2 S, summed in the order the neighbour values
// arrive (y from the lane's previous step, z from the ring, x last).  Either way one multiply-add per cell lies
// on the x-chain and P itself is never needed.
template <typename T, bool EXACT, bool BWD>
__device__ inline void sweep_cell(T in, T p, T cx, T cy, T cz, T& out, T& pass) {
  if (!BWD) {
    if (EXACT) {
      const T t = ((in + cx) + cy) + cz;
      out = t * p;
      pass = p * out;
    } else {  // p (in + cy) does not wait for the ring; cz, then cx, each one multiply-add
      pass = madd(p, cx, madd(p, cz, p * (in + cy)));
      out = pass;
    }
  } else {
    if (EXACT) {
      const T t = ((in + p * cx) + p * cy) + p * cz;
      out = t * p;
    } else {
      out = madd(p, cx, madd(p, cz, madd(p, cy, in)));
    }
    pass = out;
  }
}

// Where a compute warp sends its per-step values: into ring slot barriers of
// a consumer in this CTA or in another CTA of the cluster (shared::cluster
// addresses), whose consumed-step counter gives the back-pressure.
struct RingDst {
  unsigned ring;   // shared::cluster address of the consumer ring (slot 0)
  unsigned rbar;   // shared::cluster address of the consumer's slot barriers
  unsigned prog;   // shared::cluster address of the consumer's consumed-step counter
  bool remote;     // counter lives in another CTA
};

// The per-plane body shared by both kernels: R steps of one compute warp.
// ring_in/rbar_in: this warp's input ring (zeros and no waiting when
// `no_input`).  Returns false after a bounded wait expired.
template <typename T, int C, bool EXACT, bool BWD>
__device__ __forceinline__ bool sweep_plane(const WaveArgs<T>& a, WaveSmem<T>& sm, int warp, int lane, int z,
                            bool no_input, const RingDst dst, bool has_dst, int* failed,
                            unsigned& tparity, unsigned& rparity, int feed_K, bool feed_fence) {
  constexpr int W = 32 * C;  // == a.k.W: row offsets below are compile-time constants
  const int R = a.k.R;
  constexpr unsigned rowb = (unsigned)(W * sizeof(T));
  constexpr int CP = ring_cp(C, sizeof(T));
  constexpr unsigned ringb = 32u * CP * sizeof(T);  // bytes of one ring row
  const int nblocks = (R + kWaveKB - 1) / kWaveKB;
  const T* inp = a.in + (long long)z * a.k.plane;
  const T* Pp = a.P + (long long)z * a.k.plane;
  T* outp = a.out + (long long)z * a.k.plane;
  const int PF = a.pf;
  T* tma = sm.tma + (size_t)warp * PF * 2 * kWaveKB * W;
  uint64_t* bar = sm.bar + warp * PF;
  const T* ring_in = sm.ring + (size_t)warp * kWaveD * 32 * CP;
  uint64_t* rbar_in = sm.rbar + warp * kWaveD;
  // block j = steps [j*KB, j*KB+KB); its rows are contiguous, so one bulk
  // copy per array per block (rows stored ascending in the slot).
  // (lane 0 issues; the other lanes pass through the predicated copy)
  auto issue = [&](int j) {
    const int t0 = j * kWaveKB;
    const int n = min(kWaveKB, R - t0);
    const int row0 = BWD ? (R - t0 - n) : t0;
    T* d = tma + (size_t)(j % PF) * 2 * kWaveKB * W;
    tma_pair_if(lane == 0, &bar[j % PF], d, inp + (size_t)row0 * W, d + (size_t)kWaveKB * W,
                Pp + (size_t)row0 * W, (unsigned)n * rowb);
  };
  int issued = min(PF - 1, nblocks), consumed = 0;
  for (int j = 0; j < issued; j++) issue(j);
  bool ok = true;
  const T* din = tma;
  // make block j current (issue the block PF - 1 ahead, wait for j's
  // copies); false on timeout
  auto enter_block = [&](int j) -> bool {
    if (j + PF - 1 < nblocks) {
      issue(j + PF - 1);
      issued = j + PF;
    }
    const int slot = j % PF;
    long long spins = 0;
    while (!mbar_try_wait(&bar[slot], (tparity >> slot) & 1u)) {
      if (++spins > kSpinLimitSlow) {
        if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_TMA, failed);
        return false;
      }
    }
    tparity ^= 1u << slot;
    consumed = j + 1;
    din = tma + (size_t)slot * 2 * kWaveKB * W;
    return true;
  };
  T cy[C];
#pragma unroll
  for (int j = 0; j < C; j++) cy[j] = T(0);
  T edge = T(0);
  int next_seen = 0;
  // Step t, the u-th of its block (the block's rows at `blk`, n_blk of
  // them); false after an expired wait.  Blocks start at multiples of
  // kWaveKB == kWaveD, so the ring slot of step t is u: in a full block,
  // which the caller unrolls, every slot index, row offset and bookkeeping
  // test below is a compile-time constant.
  // The warp's two roles -- whether it hands its values on (kDst) and whether
  // it has ring input (kNoIn: the plume's first plane has none) -- are
  // compile-time constants of the step: the block loop below is instantiated
  // once per combination, so no step tests them.  kTail: the block may hold
  // the plane's last row (only the last block does).
  auto step = [&](auto kDst, auto kNoIn, auto kTail, const int t, const int u, const T* blk,
                  const int n_blk) -> bool {
    constexpr bool HAS_DST = decltype(kDst)::value;
    constexpr bool NO_INPUT = decltype(kNoIn)::value;
    constexpr bool TAIL = decltype(kTail)::value;
    const int rs = u;
    if constexpr (HAS_DST) {
      // the consumer may be at most D steps behind.  Its consumed-step
      // counter moves in fours, so the test is made for four steps at a
      // time: before steps t .. t+3 the consumer must have consumed step
      // t + 3 - D (it re-arms each slot itself once it has read it).
      if ((u & 3) == 0 && next_seen <= t + 3 - kWaveD) {
        long long spins = 0;
        for (;;) {
          next_seen = ld_remote_relaxed(dst.prog);  // a shared::cta address is valid here too
          if (next_seen > t + 3 - kWaveD) break;
          if (++spins > kSpinLimit || ld_vol(failed)) {
            if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_RING, failed);
            return false;
          }
        }
      }
    }
    // this step's inputs from the block's TMA slot
    const int rib = BWD ? (n_blk - 1 - u) : u;
    T vin[C], vp[C];
    lds_row<T, C>(blk + (size_t)rib * W + lane * C, vin);
    lds_row<T, C>(blk + (size_t)(kWaveKB + rib) * W + lane * C, vp);
    // ---- critical chain: neighbour value -> cell updates -> hand-off ----
    T cz[C];
    if constexpr (NO_INPUT) {
#pragma unroll
      for (int j = 0; j < C; j++) cz[j] = T(0);
    } else {
      long long spins = 0;
      while (!mbar_try_wait_cluster(&rbar_in[rs], (rparity >> rs) & 1u)) {
        if (++spins > kSpinLimit || ld_vol(failed)) {
          if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_RING, failed);
          return false;
        }
      }
      rparity ^= 1u << rs;
      lds_ring<T, C>(ring_in + (size_t)(rs * 32 + lane) * CP, cz);
      mbar_arm_if(lane == 0, &rbar_in[rs], ringb);  // the slot's next use
    }
    T cx = BWD ? __shfl_down_sync(0xffffffffu, edge, 1) : __shfl_up_sync(0xffffffffu, edge, 1);
    if (BWD ? (lane == 31) : (lane == 0)) cx = T(0);
    T vout[C], pass[C];
    if (!BWD) {
#pragma unroll
      for (int j = 0; j < C; j++) {
        sweep_cell<T, EXACT, false>(vin[j], vp[j], cx, cy[j], cz[j], vout[j], pass[j]);
        cx = pass[j];
      }
      edge = pass[C - 1];
    } else {
#pragma unroll
      for (int j = C - 1; j >= 0; j--) {
        sweep_cell<T, EXACT, true>(vin[j], vp[j], cx, cy[j], cz[j], vout[j], pass[j]);
        cx = pass[j];
      }
      edge = pass[0];
    }
    if constexpr (HAS_DST) {
      const unsigned off = (unsigned)((size_t)(rs * 32 + lane) * CP * sizeof(T));
      st_async_ring<T, C>(dst.ring + off, pass, dst.rbar + (unsigned)(rs * sizeof(uint64_t)));
    }
    // ---- off the chain: output and bookkeeping ----
#pragma unroll
    for (int j = 0; j < C; j++) cy[j] = pass[j];
    T* orow = outp + (size_t)(BWD ? (R - 1 - t) : t) * W + lane * C;
    if (sizeof(T) == 4 && C % 4 == 0) {
#pragma unroll
      for (int j = 0; j < C; j += 4)
        *reinterpret_cast<float4*>(orow + j) = make_float4(vout[j], vout[j + 1], vout[j + 2], vout[j + 3]);
    } else {
#pragma unroll
      for (int j = 0; j < C; j++) orow[j] = vout[j];
    }
    if ((u & 3) == 3 || (TAIL && t + 1 == R)) {  // report consumed ring steps (back-pressure)
      __syncwarp();
      st_shared_if(lane == 0, &sm.prog[warp], t + 1);
    }
    if (feed_fence && ((t + 1) % feed_K == 0 || t + 1 == R)) {
      // boundary plane of the courier path: rows visible GPU-wide every K
      __threadfence();
      __syncwarp();
      if (lane == 0) st_vol(&sm.misc[2], t + 1);
    }
    return true;
  };
  using Yes = std::true_type;
  using No = std::false_type;
  auto run_blocks = [&](auto kDst, auto kNoIn) {
    for (int j = 0; j < nblocks && ok; j++) {
      if (!enter_block(j)) {
        ok = false;
        break;
      }
      const int t0 = j * kWaveKB;
      const int n = min(kWaveKB, R - t0);
      const T* blk = din;
      if (t0 + kWaveKB < R) {  // a full block before the last: unrolled
#pragma unroll
        for (int u = 0; u < kWaveKB; u++)
          if (!step(kDst, kNoIn, No{}, t0 + u, u, blk, kWaveKB)) {
            ok = false;
            break;
          }
      } else {  // the last block, full or not
        for (int u = 0; u < n; u++)
          if (!step(kDst, kNoIn, Yes{}, t0 + u, u, blk, n)) {
            ok = false;
            break;
          }
      }
    }
  };
  if (has_dst)
    no_input ? run_blocks(Yes{}, Yes{}) : run_blocks(Yes{}, No{});
  else
    no_input ? run_blocks(No{}, Yes{}) : run_blocks(No{}, No{});
  // every issued TMA block must land before its slot is reused or the CTA exits
  for (int j = consumed; j < issued; j++) {
    const int k = j % PF;
    long long spins = 0;
    while (!mbar_try_wait(&bar[k], (tparity >> k) & 1u)) {
      if (++spins > kSpinLimitSlow) {
        if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_TMA, failed);
        break;
      }
    }
    tparity ^= 1u << k;
  }
  __syncwarp();
  return ok;
}

// ------------------------------------------------------------ cluster path
// One thread-block cluster per plume: CTA rank r owns slab r (BZ planes), so
// the plume's whole z-extent lives in one cluster (nslabs <= 16).  The last
// compute warp of a slab st.async-writes its per-step values into ring 0 of
// the next slab's CTA over distributed shared memory.  No global flags.
template <typename T, int C, bool EXACT, bool BWD>
__device__ __forceinline__ void mic_wave_cl_body(const WaveArgs<T>& a) {
  if (a.st->done) return;
  extern __shared__ __align__(128) char smem_raw[];
  const int BZ = a.BZ, W = a.k.W;
  WaveSmem<T> sm = wave_carve<T>(smem_raw, BZ, W, a.pf);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned rank = cluster_rank();
  const int z0 = (int)rank * BZ;
  const int zend = min(z0 + BZ, a.k.nz);
  const int nw = max(zend - z0, 0);
  const bool has_up = BWD ? (zend < a.k.nz) : (z0 > 0);
  const bool has_down = BWD ? (z0 > 0) : (zend < a.k.nz);
  const unsigned down_rank = BWD ? rank - 1 : rank + 1;
  int* failed = &sm.misc[1];
  if (lane == 0 && warp < BZ) {
    for (int k = 0; k < a.pf; k++) mbar_init(&sm.bar[warp * a.pf + k], 1);
    for (int k = 0; k < kWaveD; k++) mbar_init(&sm.rbar[warp * kWaveD + k], 1);
    // every ring slot armed for its first use (the consumer re-arms after each)
    for (int k = 0; k < kWaveD; k++)
      mbar_arm(&sm.rbar[warp * kWaveD + k], 32u * ring_cp(C, sizeof(T)) * sizeof(T));
  }
  if (threadIdx.x == 0) {
    sm.misc[1] = 0;
    for (int w = 0; w <= BZ; w++) sm.prog[w] = 0;
  }
  fence_mbar_init();
  __syncthreads();
  cluster_sync_all();  // every CTA's barriers exist before any remote st.async
  const bool gate_ok = wave_pass_gate(a, failed);
  if (warp < nw && gate_ok) {
    const int z = BWD ? (zend - 1 - warp) : (z0 + warp);
    RingDst d{0u, 0u, 0u, false};
    bool has_dst = false;
    if (warp + 1 < nw) {
      d.ring = smem_u32(sm.ring + (size_t)(warp + 1) * kWaveD * 32 * ring_cp(C, sizeof(T)));
      d.rbar = smem_u32(sm.rbar + (warp + 1) * kWaveD);
      d.prog = smem_u32(&sm.prog[warp + 1]);
      has_dst = true;
    } else if (has_down) {
      d.ring = mapa_u32(sm.ring, down_rank);
      d.rbar = mapa_u32(sm.rbar, down_rank);
      d.prog = mapa_u32(&sm.prog[0], down_rank);
      d.remote = true;
      has_dst = true;
    }
    unsigned tpar = 0u, rpar = 0u;
    sweep_plane<T, C, EXACT, BWD>(a, sm, warp, lane, z, warp == 0 && !has_up, d, has_dst, failed, tpar,
                                  rpar, 1, false);
  }
  __syncthreads();
  cluster_sync_all();  // no CTA leaves while a neighbour may still write into it
}
template <typename T, int C, bool EXACT, bool BWD>
__global__ void __launch_bounds__(32 * 16) k_mic_wave_cl(WaveArgs<T> a) {
  mic_wave_cl_body<T, C, EXACT, BWD>(a);
}

// ------------------------------------------------------------ courier path
// For plumes too tall for one cluster: slabs are handed to CTAs in sweep
// order by a ticket (a CTA only waits on slabs already running, so any grid
// size is deadlock-free); per CTA a fetch courier feeds ring 0 from the
// upstream slab's boundary plane in global memory, and a publish courier
// advertises this slab's boundary progress every K steps.
template <typename T, int C, bool EXACT, bool BWD>
__global__ void __launch_bounds__(32 * 18) k_mic_wave(WaveArgs<T> a) {
  if (a.st->done) return;
  extern __shared__ __align__(128) char smem_raw[];
  const int BZ = a.BZ, W = a.k.W, R = a.k.R;
  WaveSmem<T> sm = wave_carve<T>(smem_raw, BZ, W, a.pf);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* failed = &sm.misc[1];
  if (lane == 0 && warp < BZ) {
    for (int k = 0; k < a.pf; k++) mbar_init(&sm.bar[warp * a.pf + k], 1);
    for (int k = 0; k < kWaveD; k++) mbar_init(&sm.rbar[warp * kWaveD + k], 1);
    // every ring slot armed for its first use (the consumer re-arms after each)
    for (int k = 0; k < kWaveD; k++)
      mbar_arm(&sm.rbar[warp * kWaveD + k], 32u * ring_cp(C, sizeof(T)) * sizeof(T));
  }
  if (threadIdx.x == 0) sm.misc[1] = 0;
  fence_mbar_init();
  __syncthreads();
  (void)wave_pass_gate(a, failed);  // on expiry the ticket loop below exits at once
  unsigned tpar = 0u, rpar = 0u;  // barrier phases carry over between slabs
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned tk = atomicAdd(&a.ctl[0], 1u);
      sm.misc[0] = (tk < (unsigned)a.nslabs) ? (int)tk : -1;
      sm.misc[2] = 0;
      for (int w = 0; w <= BZ; w++) sm.prog[w] = 0;
    }
    __syncthreads();
    const int ticket = sm.misc[0];
    if (ticket < 0 || ld_vol(failed) || ld_vol(&a.st->wave_err)) break;
    const int slab = a.backward ? (a.nslabs - 1 - ticket) : ticket;
    const int z0 = slab * BZ;
    const int zend = min(z0 + BZ, a.k.nz);
    const int nw = zend - z0;
    const bool has_up = a.backward ? (zend < a.k.nz) : (z0 > 0);
    const bool has_down = a.backward ? (z0 > 0) : (zend < a.k.nz);
    const int z_up = a.backward ? zend : z0 - 1;
    const int z_last = a.backward ? z0 : zend - 1;
    if (warp == BZ) {
      // fetch courier: upstream boundary plane -> ring 0 (st.async, local)
      if (has_up) {
        // the value a plane hands on is its output, except in the exact
        // forward sweep, which writes q and hands on P q (the FP32 forward
        // sweep writes P q itself; see sweep_cell)
        constexpr bool kScaleOut = EXACT && !BWD;
        int in_next = 0;
        long long spins = 0;
        const unsigned ring0 = smem_u32(sm.ring), rbar0 = smem_u32(sm.rbar);
        while (in_next < R && !ld_vol(failed)) {
          const int avail = ld_vol(&a.progress[z_up]);
          const int space = ld_vol(&sm.prog[0]) + kWaveD - in_next;
          const int n = min(min(avail - in_next, space), 4);
          if (n <= 0) {
            if (++spins > kSpinLimitSlow) {
              if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_FLAG, failed);
              break;
            }
            __nanosleep(32);
            continue;
          }
          spins = 0;
          __threadfence();
          T o[4][C], pv[4][C];
#pragma unroll
          for (int i = 0; i < 4; i++) {
            if (i < n) {
              const int t = in_next + i;
              const int row = a.backward ? (R - 1 - t) : t;
              const long long base = (long long)z_up * a.k.plane + (long long)row * W + lane * C;
#pragma unroll
              for (int j = 0; j < C; j++) {
                o[i][j] = __ldcg(a.out + base + j);
                pv[i][j] = kScaleOut ? __ldcg(a.P + base + j) : T(1);
              }
            }
          }
#pragma unroll
          for (int i = 0; i < 4; i++) {
            if (i < n) {
              const int rs = (in_next + i) % kWaveD;
              T v[C];
#pragma unroll
              for (int j = 0; j < C; j++) v[j] = kScaleOut ? pv[i][j] * o[i][j] : o[i][j];
              constexpr int CP = ring_cp(C, sizeof(T));
              st_async_ring<T, C>(ring0 + (unsigned)((size_t)(rs * 32 + lane) * CP * sizeof(T)), v,
                                  rbar0 + (unsigned)(rs * sizeof(uint64_t)));
            }
          }
          in_next += n;
        }
      }
    } else if (warp == BZ + 1) {
      // publish courier: this slab's boundary progress -> global flag
      if (has_down) {
        int pub = 0;
        long long spins = 0;
        while (pub < R && !ld_vol(failed)) {
          const int p = ld_vol(&sm.misc[2]);  // rows the boundary warp has fenced
          if (p > pub) {
            if (lane == 0) st_vol(&a.progress[z_last], p);
            pub = p;
            spins = 0;
          } else if (++spins > kSpinLimitSlow) {
            if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_FLAG, failed);
            break;
          } else {
            __nanosleep(32);
          }
        }
      }
    } else if (warp < nw) {
      const int z = a.backward ? (zend - 1 - warp) : (z0 + warp);
      RingDst d{0u, 0u, 0u, false};
      const bool has_dst = warp + 1 < nw;
      if (has_dst) {
        d.ring = smem_u32(sm.ring + (size_t)(warp + 1) * kWaveD * 32 * ring_cp(C, sizeof(T)));
        d.rbar = smem_u32(sm.rbar + (warp + 1) * kWaveD);
        d.prog = smem_u32(&sm.prog[warp + 1]);
      }
      const bool boundary = has_down && warp == nw - 1;
      sweep_plane<T, C, EXACT, BWD>(a, sm, warp, lane, z, warp == 0 && !has_up, d, has_dst, failed,
                                    tpar, rpar, a.K, boundary);
    }
    __syncthreads();
    if (ld_vol(failed)) break;
  }
  // exit: the last CTA out resets the ticket, exit counter and progress flags
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned e = atomicAdd(&a.ctl[1], 1u);
    if (e == gridDim.x - 1) {
      for (int zz = 0; zz < a.k.nz; zz++) a.progress[zz] = 0;
      a.ctl[0] = 0;
      __threadfence();
      a.ctl[1] = 0;
    }
  }
}

}  // namespace plume
