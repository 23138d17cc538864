// unet_tc.cuh -- the U-Net's 3x3x3 convolution on the 5th-generation tensor
// cores (tcgen05, sm_103a): implicit GEMM with the accumulators in TMEM.
//
// A work item is a 16 (x) x 8 (y) x 2 (z) brick of output cells.  Its input
// halo (18 x 10 x 4 cells) and the layer's whole weight tensor are staged in
// shared memory in the no-swizzle K-major canonical layout of the tensor-core
// operands (8 x 16-byte "core matrices"):
//   halo    [channel group g of 8][hz][hx][hy] x 16 bytes: for a fixed (g, hz,
//           hx), 8 consecutive hy cells form one core matrix, so the A operand
//           of output z-plane t and tap (dx, dy, dz) -- 128 cells, x-major and
//           y-minor -- is 16 core matrices at a stride of HY * 16 bytes (SBO),
//           and the two channel groups of a 16-channel K step lie one plane
//           apart (LBO);
//   weights [tap][16-channel step][cout block of 8][k half][8 cout][8 cin]:
//           the B operand (N = COUT, K = 16) of every (tap, step).
// One thread issues the 27 * CIN/16 tcgen05.mma (M = 128, N = COUT, K = 16,
// BF16 inputs, FP32 accumulation) per z-plane into TMEM columns [t COUT,
// (t+1) COUT) of the item's accumulator buffer, commits to an mbarrier, and
// the 8 warps read the accumulators back with tcgen05.ld (warp w: z-plane
// w / 4, TMEM lanes 32 (w % 4) ...).
// Every wait is bounded: on expiry the CTA records an error, waits (bounded,
// much longer) for the MMAs it issued to retire, frees its TMEM and returns.
#pragma once
#include "unet_kernels.cuh"

namespace plume {
namespace unet {

template <int CIN, int COUT>
struct TcCfg {
  static constexpr int BZ = 2, BY = 8, BX = 16;
  static constexpr int HX = BX + 2, HY = BY + 2, HZ = BZ + 2;
  static constexpr int G = CIN / 8, KC = CIN / 16;
  static constexpr int PLANE = HZ * HX * HY * 16;  // bytes of one channel group
  static constexpr int BRICK = G * PLANE;
  static constexpr int WTILE = COUT * 32;  // bytes of one (tap, step) B operand
  static constexpr int WBYTES = 27 * KC * WTILE;
  // accumulation chains: each z-plane's taps are split by dz into P partial
  // accumulators (summed in the epilogue) when TMEM has room, so that up to
  // 2 P MMAs in a row are independent
  static constexpr int P = 2 * BZ * 3 * COUT <= 512 ? 3 : 1;
  static constexpr int ACC = BZ * P * COUT;  // TMEM columns of one accumulator buffer
  static constexpr int NCOLS = 2 * ACC <= 32 ? 32 : (2 * ACC <= 64 ? 64 : (2 * ACC <= 128 ? 128 : 256));
  static constexpr int SMEM = WBYTES + 2 * BRICK + 64;
  static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 128, "channel counts");
};

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of sm_100-class parts; no swizzle, base offset 0
  return d;
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major
template <int M, int N>
__host__ __device__ constexpr uint32_t tc_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mbar_init(uint32_t bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool tc_mbar_wait(uint32_t bar, unsigned parity, long long limit) {
  for (long long i = 0; i < limit; i++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
      "%14, %15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

constexpr long long kTcSpinLimit = 1ll << 22;
constexpr long long kTcDrainLimit = 1ll << 26;  // MMAs still in flight after an expired wait

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Issue the copies of one brick's halo (channel group fastest, then x:
// coalesced global reads) into a shared-memory buffer.
template <int CIN, int COUT>
__device__ __forceinline__ void tc_stage(const Dims& d, const View& in, long long item, int nbricks,
                                         unsigned char* buf) {
  using C = TcCfg<CIN, COUT>;
  const int nbx = (d.X + C::BX - 1) / C::BX, nby = (d.Y + C::BY - 1) / C::BY;
  const long long b = item / nbricks;
  int bi = (int)(item - b * nbricks);
  const int bx = bi % nbx;
  bi /= nbx;
  const int x0 = bx * C::BX, y0 = (bi % nby) * C::BY, z0 = (bi / nby) * C::BZ;
  const bf16* src = in.p + b * in.bs + in.co;
  constexpr int NCH = C::G * C::HX * C::HY * C::HZ;
  for (int i = threadIdx.x; i < NCH; i += blockDim.x) {
    const int g = i % C::G;
    int t = i / C::G;
    const int hx = t % C::HX;
    t /= C::HX;
    const int hy = t % C::HY, hz = t / C::HY;
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
    const bool ok = gx >= 0 && gx < d.X && gy >= 0 && gy < d.Y && gz >= 0 && gz < d.Z;
    const long long cell = ok ? ((long long)gz * d.Y + gy) * d.X + gx : 0;
    const int dst = (((g * C::HZ + hz) * C::HX + hx) * C::HY + hy) * 16;
    cp_async16(smem_u32addr(buf + dst), src + cell * in.cs + g * 8, ok ? 16 : 0);
  }
}

// out = act(conv3(in, W) + bias) [* (mask > 0)]
//   wpack : weights in the B-operand layout above (k_prep_tc)
//   err   : set to 1 if a wait expired (host-mapped: plain stores, read by
//           the host after it synchronises the stream)
// Persistent: CTA c takes work items (brick, sample) c, c + gridDim.x, ...;
// the weights are staged once, the halo in two buffers: while one item's
// MMAs and epilogue run, the next item's halo is in flight.  The two TMEM
// accumulator buffers (BZ * COUT columns each) alternate with the halo
// buffers, each with its own completion mbarrier.
// grid: min(items, resident CTAs); block 256; dynamic smem TcCfg::SMEM
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv3_tc(Dims d, int batch, View in, const bf16* __restrict__ wpack,
                                                  const float* __restrict__ bias, View out, View mask, int relu,
                                                  int* err) {
  using C = TcCfg<CIN, COUT>;
  extern __shared__ __align__(128) unsigned char tsm[];
  unsigned char* wsm = tsm;
  unsigned char* bufs = tsm + C::WBYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(tsm + C::WBYTES + 2 * C::BRICK);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + C::WBYTES + 2 * C::BRICK + 16);
  const int nbx = (d.X + C::BX - 1) / C::BX, nby = (d.Y + C::BY - 1) / C::BY,
            nbz = (d.Z + C::BZ - 1) / C::BZ;
  const int nbricks = nbx * nby * nbz;
  const long long items = (long long)nbricks * batch;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (int i = threadIdx.x; i < C::WBYTES / 16; i += blockDim.x)
    cp_async16(smem_u32addr(wsm + i * 16), wpack + i * 8, 16);
  if ((long long)blockIdx.x < items) tc_stage<CIN, COUT>(d, in, blockIdx.x, nbricks, bufs);
  cp_async_commit();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32addr(tslot)),
                 "r"(C::NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 32) {
    tc_mbar_init(smem_u32addr(&bars[0]), 1);
    tc_mbar_init(smem_u32addr(&bars[1]), 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;
  const uint32_t ws = smem_u32addr(wsm);
  constexpr uint32_t idesc = tc_idesc<128, COUT>();

  int j = 0;
  int fail_bar = -1;  // commit barrier and phase of an item whose wait expired
  unsigned fail_parity = 0;
  for (long long item = blockIdx.x; item < items; item += gridDim.x, j++) {
    const int cur = j & 1;
    const long long next = item + gridDim.x;
    // the next item's halo goes to the other buffer, free since its MMAs
    // completed before the previous epilogue
    if (next < items) tc_stage<CIN, COUT>(d, in, next, nbricks, bufs + (cur ^ 1) * C::BRICK);
    cp_async_commit();
    cp_async_wait<1>();  // this item's halo (and, first time, the weights)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tacc = tbase + (uint32_t)(cur * C::ACC);
    if (threadIdx.x == 0) {
      // fully unrolled: every operand address is the buffer's base descriptor
      // plus a compile-time offset (the start-address field holds bytes / 16
      // and the brick stays far below the field's 256 KB range); the z-planes'
      // accumulations are interleaved so that consecutive MMAs are independent
      const uint64_t a0 = tc_desc(smem_u32addr(bufs + cur * C::BRICK), C::PLANE, C::HY * 16);
      const uint64_t b0 = tc_desc(ws, 128, 256);
#pragma unroll
      for (int off = 0; off < 27; off++) {
        const int dz = off / 9 - 1, dy = (off / 3) % 3 - 1, dx = off % 3 - 1;
#pragma unroll
        for (int kc = 0; kc < C::KC; kc++)
#pragma unroll
          for (int t = 0; t < C::BZ; t++) {
            const uint32_t ao = (uint32_t)((((2 * kc * C::HZ + t + 1 + dz) * C::HX + 1 + dx) * C::HY + 1 + dy) * 16);
            const uint32_t bo = (uint32_t)((off * C::KC + kc) * C::WTILE);
            const int part = C::P == 3 ? dz + 1 : 0;
            const bool first = C::P == 3 ? (off % 9 == 0 && kc == 0) : (off == 0 && kc == 0);
            tc_mma(tacc + (uint32_t)((t * C::P + part) * COUT), a0 + (ao >> 4), b0 + (bo >> 4), idesc,
                   first ? 0u : 1u);
          }
      }
      tc_commit(smem_u32addr(&bars[cur]));
    }
    const unsigned parity = (unsigned)((j >> 1) & 1);
    bool ok = tc_mbar_wait(smem_u32addr(&bars[cur]), parity, kTcSpinLimit);
    if (!ok) ok = tc_mbar_wait(smem_u32addr(&bars[cur]), parity, kTcSpinLimit);
    ok = __syncthreads_and(ok) != 0;  // the TMEM loads below are warp-collective
    tc_fence_after();
    if (!ok) {
      if (threadIdx.x == 0) *(volatile int*)err = 1;
      fail_bar = cur;
      fail_parity = parity;
      break;
    }
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. of z-plane w / 4
    const long long b = item / nbricks;
    int bi = (int)(item - b * nbricks);
    const int bx = bi % nbx;
    bi /= nbx;
    const int x0 = bx * C::BX, y0 = (bi % nby) * C::BY, z0 = (bi / nby) * C::BZ;
    const int t = warp >> 2, q = warp & 3;
    const int m = 32 * q + lane;
    const int gx = x0 + m / 8, gy = y0 + m % 8, gz = z0 + t;
    const bool inside = gx < d.X && gy < d.Y && gz < d.Z;
    const long long cell = ((long long)gz * d.Y + gy) * d.X + gx;
    bf16* dst = out.p + b * out.bs + out.co + cell * out.cs;
    const bf16* msk = mask.p ? mask.p + b * mask.bs + mask.co + cell * mask.cs : nullptr;
#pragma unroll
    for (int c16 = 0; c16 < COUT / 16; c16++) {
      float v[16];
      tc_ld16(tacc + ((uint32_t)(32 * q) << 16) + (uint32_t)(t * C::P * COUT + c16 * 16), v);
#pragma unroll
      for (int pp = 1; pp < C::P; pp++) {
        float w[16];
        tc_ld16(tacc + ((uint32_t)(32 * q) << 16) + (uint32_t)((t * C::P + pp) * COUT + c16 * 16), w);
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] += w[k];
      }
      if (!inside) continue;
      uint32_t packed[8];
#pragma unroll
      for (int k = 0; k < 16; k += 2) {
        const int n = c16 * 16 + k;
        float v0 = v[k], v1 = v[k + 1];
        if (bias) {
          v0 += bias[n];
          v1 += bias[n + 1];
        }
        if (relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (msk) {
          const __nv_bfloat162 mm = *reinterpret_cast<const __nv_bfloat162*>(msk + n);
          if (!(__low2float(mm) > 0.f)) v0 = 0.f;
          if (!(__high2float(mm) > 0.f)) v1 = 0.f;
        }
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v0, v1);
        packed[k / 2] = *reinterpret_cast<const uint32_t*>(&h2);
      }
      uint4* d4 = reinterpret_cast<uint4*>(dst + c16 * 16);
      d4[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
      d4[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
    }
  }
  cp_async_wait<0>();
  // the accumulators must not be freed under MMAs that are still running
  if (fail_bar >= 0 && threadIdx.x == 0)
    (void)tc_mbar_wait(smem_u32addr(&bars[fail_bar]), fail_parity, kTcDrainLimit);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(C::NCOLS) : "memory");
}

// FP32 master W[27][cin][cout] -> the B-operand layout of k_conv3_tc:
// [tap][16-channel step kc][cout block nb][k half kb][8 cout][8 cin]
__global__ void k_prep_tc(const float* W, int cin, int cout, bf16* out) {
  const int KC = cin / 16, NB = cout / 8;
  const long long total = 27LL * cin * cout;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long t = i;
    const int k = (int)(t % 8);
    t /= 8;
    const int n = (int)(t % 8);
    t /= 8;
    const int kb = (int)(t % 2);
    t /= 2;
    const int nb = (int)(t % NB);
    t /= NB;
    const int kc = (int)(t % KC);
    const int off = (int)(t / KC);
    const int ci = kc * 16 + kb * 8 + k, co = nb * 8 + n;
    out[i] = __float2bfloat16_rn(W[((size_t)off * cin + ci) * cout + co]);
  }
}

}  // namespace unet
}  // namespace plume
