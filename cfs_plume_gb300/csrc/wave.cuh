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

constexpr int kWavePF = 8;     // TMA prefetch ring depth (rows)
constexpr int kWaveD = 8;      // inter-warp ring depth (steps)
constexpr long long kSpinLimit = 1ll << 24;     // shared-memory polls (~0.3 s)
constexpr long long kSpinLimitSlow = 1ll << 21; // global-flag polls and TMA waits (~2 s)

enum WaveError { WAVE_OK = 0, WAVE_TIMEOUT_RING = 1, WAVE_TIMEOUT_TMA = 2, WAVE_TIMEOUT_FLAG = 3 };

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
};

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
__device__ inline void tma_row(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
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

// Shared-memory layout of one CTA (dynamic): see wave_smem_bytes().
template <typename T>
struct WaveSmem {
  T* tma;          // [BZ][PF][2][W]  in-row, P-row per slot
  uint64_t* bar;   // [BZ][PF]
  T* ring;         // [BZ][D][W]      ring r is read by compute warp r
  int* prog;       // [BZ + 1]        steps completed: warps 0..BZ-1, courier (ring 0) at BZ
  int* misc;       // [4]             slab, failed
};

template <typename T>
__host__ __device__ inline size_t wave_smem_bytes(int BZ, int W) {
  size_t b = (size_t)BZ * kWavePF * 2 * W * sizeof(T);
  b += (size_t)BZ * kWavePF * sizeof(uint64_t);
  b += (size_t)BZ * kWaveD * W * sizeof(T);
  b += (size_t)(BZ + 1 + 4) * sizeof(int);
  return b;
}

template <typename T>
__device__ inline WaveSmem<T> wave_carve(char* base, int BZ, int W) {
  WaveSmem<T> s;
  s.tma = (T*)base;
  base += (size_t)BZ * kWavePF * 2 * W * sizeof(T);
  s.bar = (uint64_t*)base;
  base += (size_t)BZ * kWavePF * sizeof(uint64_t);
  s.ring = (T*)base;
  base += (size_t)BZ * kWaveD * W * sizeof(T);
  s.prog = (int*)base;
  s.misc = s.prog + BZ + 1;
  return s;
}

__device__ inline void wave_fail(CgState* st, int code, int* failed) {
  atomicCAS(&st->wave_err, 0, code);
  st_vol(failed, 1);
}

// One cell of the sweep.  Forward: t = ((r + wx) + wy) + wz, q = t*P, and the
// value handed to the +x/+y/+z neighbours is w = P*q, because the reference
// forms (A+ . P) . q = (-P) . q.  Backward: t = ((q + P zx) + P zy) + P zz,
// z = t*P; neighbours receive z itself.
template <typename T, bool EXACT, bool BWD>
__device__ inline void sweep_cell(T in, T p, T cx, T cy, T cz, T& out, T& pass) {
  if (!BWD) {
    T t;
    if (EXACT)
      t = ((in + cx) + cy) + cz;
    else
      t = (in + cy + cz) + cx;
    out = t * p;
    pass = p * out;
  } else {
    T t;
    if (EXACT)
      t = ((in + p * cx) + p * cy) + p * cz;
    else
      t = (in + p * (cy + cz)) + p * cx;
    out = t * p;
    pass = out;
  }
}

template <typename T, int C, bool EXACT, bool BWD>
__global__ void __launch_bounds__(32 * 17) k_mic_wave(WaveArgs<T> a) {
  if (a.st->done) return;
  extern __shared__ __align__(128) char smem_raw[];
  const int BZ = a.BZ, W = a.k.W, R = a.k.R;
  WaveSmem<T> sm = wave_carve<T>(smem_raw, BZ, W);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool courier = (warp == BZ);
  int* failed = &sm.misc[1];
  const unsigned rowb = (unsigned)(W * sizeof(T));

  // per-warp TMA slot barriers, initialised once per CTA
  if (!courier && lane == 0)
    for (int k = 0; k < kWavePF; k++) mbar_init(&sm.bar[warp * kWavePF + k], 1);
  if (threadIdx.x == 0) sm.misc[1] = 0;
  fence_mbar_init();
  __syncthreads();
  // bit k = phase parity expected next on TMA slot k (same in every lane)
  unsigned parity = 0u;

  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned tk = atomicAdd(&a.ctl[0], 1u);
      sm.misc[0] = (tk < (unsigned)a.nslabs) ? (int)tk : -1;
      for (int w = 0; w <= BZ; w++) sm.prog[w] = 0;
    }
    __syncthreads();
    const int ticket = sm.misc[0];
    if (ticket < 0 || ld_vol(failed) || ld_vol(&a.st->wave_err)) break;
    const int slab = a.backward ? (a.nslabs - 1 - ticket) : ticket;
    const int z0 = slab * BZ;
    const int zend = min(z0 + BZ, a.k.nz);  // planes [z0, zend)
    const int nw = zend - z0;                // compute warps with a plane
    const bool has_up = a.backward ? (zend < a.k.nz) : (z0 > 0);
    const bool has_down = a.backward ? (z0 > 0) : (zend < a.k.nz);
    const int z_up = a.backward ? zend : z0 - 1;  // neighbour plane feeding warp 0
    const int z_last = a.backward ? z0 : zend - 1;  // plane the next slab reads

    if (courier) {
      // ---------------- courier: bridge to the neighbouring slabs ----------
      int in_next = 0;  // steps of plane z_up copied into ring 0
      int pub = has_down ? 0 : R;  // steps of plane z_last published
      if (!has_up) {
        // no neighbour plane: ring 0 holds zeros for the whole slab
        for (int e = lane; e < kWaveD * W; e += 32) sm.ring[e] = T(0);
        __syncwarp();
        __threadfence_block();
        in_next = R;
        if (lane == 0) st_vol(&sm.prog[BZ], R);
      }
      long long spins = 0;
      while ((in_next < R || pub < R) && !ld_vol(failed)) {
        bool moved = false;
        if (in_next < R) {
          const int avail = ld_vol(&a.progress[z_up]);
          const int space = ld_vol(&sm.prog[0]) + kWaveD - in_next;
          const int n = min(min(avail - in_next, space), 4);
          if (n > 0) {
            __threadfence();
            for (int i = 0; i < n; i++) {
              const int t = in_next + i;
              const int row = a.backward ? (R - 1 - t) : t;
              const long long base = (long long)z_up * a.k.plane + (long long)row * W;
              T* slot = sm.ring + (size_t)(t % kWaveD) * W;  // ring 0
#pragma unroll
              for (int j = 0; j < C; j++) {
                const int c = lane * C + j;
                const T o = __ldcg(a.out + base + c);
                slot[c] = BWD ? o : (__ldcg(a.P + base + c) * o);
              }
            }
            __syncwarp();
            __threadfence_block();
            in_next += n;
            if (lane == 0) st_vol(&sm.prog[BZ], in_next);
            moved = true;
          }
        }
        if (pub < R) {
          const int p = ld_vol(&sm.prog[nw - 1]);
          if (p >= min(pub + a.K, R)) {
            __threadfence();
            if (lane == 0) st_vol(&a.progress[z_last], p);
            pub = p;
            moved = true;
          }
        }
        if (moved) {
          spins = 0;
        } else if (++spins > kSpinLimitSlow) {
          if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_FLAG, failed);
          break;
        } else {
          __nanosleep(32);
        }
      }
    } else if (warp < nw) {
      // ---------------- compute warp: one plane, R steps -------------------
      const int z = a.backward ? (zend - 1 - warp) : (z0 + warp);
      const T* inp = a.in + (long long)z * a.k.plane;
      const T* Pp = a.P + (long long)z * a.k.plane;
      T* outp = a.out + (long long)z * a.k.plane;
      T* tma = sm.tma + (size_t)warp * kWavePF * 2 * W;
      uint64_t* bar = sm.bar + warp * kWavePF;
      const T* ring_in = sm.ring + (size_t)warp * kWaveD * W;   // filled by warp-1 / courier
      T* ring_out = sm.ring + (size_t)(warp + 1) * kWaveD * W;  // read by warp+1
      const int* prog_in = (warp == 0) ? &sm.prog[BZ] : &sm.prog[warp - 1];
      const bool has_next = (warp + 1 < nw);
      const int* prog_next = &sm.prog[warp + 1];
      // the boundary warp makes its rows visible GPU-wide before counting them
      const bool feeds_slab = has_down && (warp == nw - 1);
      int issued = 0, consumed = 0;
      auto issue = [&](int tn) {  // lane 0 only
        uint64_t* b = &bar[tn % kWavePF];
        T* d = tma + (size_t)(tn % kWavePF) * 2 * W;
        const int row = a.backward ? (R - 1 - tn) : tn;
        fence_proxy_async();
        mbar_expect_tx(b, 2 * rowb);
        tma_row(d, inp + (size_t)row * W, rowb, b);
        tma_row(d + W, Pp + (size_t)row * W, rowb, b);
      };
      const int prime = min(kWavePF - 1, R);
      if (lane == 0)
        for (int t = 0; t < prime; t++) issue(t);
      issued = prime;
      T cy[C];  // value from the previous step (the -y / +y neighbour)
#pragma unroll
      for (int j = 0; j < C; j++) cy[j] = T(0);
      T edge = T(0);  // this lane's outermost value of the previous step
      bool ok = true;
      for (int t = 0; t < R && ok; t++) {
        const int slot = t % kWavePF;
        // issue step t+PF-1 into the slot consumed at step t-1
        if (t + kWavePF - 1 < R) {
          if (lane == 0) issue(t + kWavePF - 1);
          issued = t + kWavePF;
        }
        // neighbour plane values for this step
        long long spins = 0;
        while (ld_vol(prog_in) <= t) {
          if (++spins > kSpinLimit || ld_vol(failed)) {
            if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_RING, failed);
            ok = false;
            break;
          }
        }
        if (!ok) break;
        __threadfence_block();
        const T* rin = ring_in + (size_t)(t % kWaveD) * W;
        T cz[C];
#pragma unroll
        for (int j = 0; j < C; j++) cz[j] = rin[lane * C + j];
        // this step's input row and diagonal
        spins = 0;
        while (!mbar_try_wait(&bar[slot], (parity >> slot) & 1u)) {
          if (++spins > kSpinLimitSlow) {
            if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_TMA, failed);
            ok = false;
            break;
          }
        }
        if (!ok) break;
        parity ^= 1u << slot;
        consumed = t + 1;
        const T* din = tma + (size_t)slot * 2 * W;
        T vin[C], vp[C];
#pragma unroll
        for (int j = 0; j < C; j++) {
          vin[j] = din[lane * C + j];
          vp[j] = din[W + lane * C + j];
        }
        // x-neighbour across the lane boundary: previous step of lane-1
        // (forward) or lane+1 (backward)
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
        // output row
        T* orow = outp + (size_t)(a.backward ? (R - 1 - t) : t) * W + lane * C;
#pragma unroll
        for (int j = 0; j < C; j++) {
          orow[j] = vout[j];
          cy[j] = pass[j];
        }
        // hand this step to the next warp (bounded back-pressure on its ring)
        if (has_next) {
          spins = 0;
          while (ld_vol(prog_next) <= t - kWaveD) {
            if (++spins > kSpinLimit || ld_vol(failed)) {
              if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_RING, failed);
              ok = false;
              break;
            }
          }
          if (!ok) break;
          T* rout = ring_out + (size_t)(t % kWaveD) * W;
#pragma unroll
          for (int j = 0; j < C; j++) rout[lane * C + j] = pass[j];
        }
        if (feeds_slab && ((t + 1) % a.K == 0 || t + 1 == R)) __threadfence();
        __syncwarp();
        __threadfence_block();
        if (lane == 0) st_vol(&sm.prog[warp], t + 1);
      }
      // every issued copy must land before its slot is reused by the next
      // slab or the CTA exits: wait (bounded) for steps consumed..issued-1
      for (int t = consumed; t < issued; t++) {
        const int k = t % kWavePF;
        long long spins = 0;
        while (!mbar_try_wait(&bar[k], (parity >> k) & 1u)) {
          if (++spins > kSpinLimitSlow) {
            if (lane == 0) wave_fail(a.st, WAVE_TIMEOUT_TMA, failed);
            break;
          }
        }
        parity ^= 1u << k;
      }
      __syncwarp();
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
