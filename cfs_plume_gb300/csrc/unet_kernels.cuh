// unet_kernels.cuh -- device code of the learned pressure warm start: a 3-level
// 3-D U-Net (channels 16/32/64, 3x3x3 convolutions) on BF16 activations with
// FP32 accumulation, forward and backward.
//
// Tensors are channels-last BF16: element (sample b, cell, channel c) at
// p[b*bs + cell*cs + co + c], cell = x + X*(y + Y*z).  `cs` and `co` let a
// layer read or write a channel slice of a wider buffer (the U-Net's skip
// concatenations are slices, never copies).
//
// The 3x3x3 convolution is an implicit GEMM on the tensor cores
// (mma.sync m16n8k16, BF16 in, FP32 accumulate): M = output cells of a brick
// (rows of 16 cells along x), N = output channels, K = 27 offsets x input
// channels.  A CTA stages its brick plus a one-cell halo in shared memory
// (cp.async, zero fill outside the grid = zero padding) and reads the A
// fragments of every offset from there with ldmatrix; B fragments come from a
// weight copy pre-arranged in fragment order.  The input-gradient pass is the
// same kernel on flipped, transposed weights; the weight gradient is a second
// implicit GEMM (M = input channels, N = output channels, K = cells) whose
// per-CTA partial sums are reduced in a fixed order, so training is
// deterministic.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace plume {
namespace unet {

typedef __nv_bfloat16 bf16;

struct Dims {
  int X, Y, Z;
  long long cells;
};

struct View {
  bf16* p;
  int cs;        // elements from one cell to the next
  int co;        // first channel of the slice
  long long bs;  // elements from one sample to the next
};

__device__ __forceinline__ float bf2f(bf16 v) { return __bfloat162float(v); }

__device__ __forceinline__ uint32_t smem_u32addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// 16-byte global -> shared copy; nbytes = 0 writes zeros (no global read)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int nbytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(nbytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t* r) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t* r) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

// d += a (16x16, row) * b (16x8, col), BF16 in, FP32 accumulate
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

// ------------------------------------------------------------- convolution
// Brick shape: 16 cells along x, BY x BZ rows; 8 warps, MF row fragments
// (16-cell rows) each.  MF in {1, 2, 4, 8} is the tile-shape knob the
// autotuner picks per layer and grid (unet.cu); every shape accumulates each
// output in the same order, so the choice never changes a result.
template <int CIN, int COUT, int MF_>
struct ConvCfg {
  static constexpr int NF = COUT / 8;
  static constexpr int KC = CIN / 16;
  static constexpr int MF = MF_;
  static constexpr int WARPS = 8;
  static constexpr int ROWS = WARPS * MF;
  static constexpr int BY = (MF >= 4) ? 8 : 4;
  static constexpr int BZ = ROWS / BY;
  static constexpr int HX = 18, HY = BY + 2, HZ = BZ + 2;
  static constexpr int HCELLS = HX * HY * HZ;
  static constexpr int CSE = CIN + 8;  // padded cell stride in shared memory (conflict-free ldmatrix)
  static constexpr int SMEM = HCELLS * CSE * 2;
  static_assert(CIN % 16 == 0 && COUT % 8 == 0, "channel counts");
  static_assert(ROWS % BY == 0, "brick rows");
};

template <int CIN, int COUT, int MF>
inline int conv_bricks(const Dims& d) {
  using C = ConvCfg<CIN, COUT, MF>;
  return ((d.X + 15) / 16) * ((d.Y + C::BY - 1) / C::BY) * ((d.Z + C::BZ - 1) / C::BZ);
}

// Stage the (BX+2) x (BY+2) x (BZ+2) halo brick of CIN channels starting at
// grid cell (x0-1, y0-1, z0-1); cells outside the grid read as zero.
template <int CIN, int HX, int HY, int HZ, int CSE>
__device__ __forceinline__ void load_halo(const Dims& d, const bf16* src, int cs, int x0, int y0, int z0,
                                          bf16* hb) {
  constexpr int CH = CIN / 8;
  constexpr int N = HX * HY * HZ * CH;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const int q = i % CH;
    const int h = i / CH;
    const int hx = h % HX, hy = (h / HX) % HY, hz = h / (HX * HY);
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
    const bool ok = gx >= 0 && gx < d.X && gy >= 0 && gy < d.Y && gz >= 0 && gz < d.Z;
    const long long cell = ok ? ((long long)gz * d.Y + gy) * d.X + gx : 0;
    cp_async16(smem_u32addr(hb + h * CSE + q * 8), src + cell * cs + q * 8, ok ? 16 : 0);
  }
}

// out = act(conv3(in, W) + bias) [* (mask > 0)]
//   wf   : weights in B-fragment order, [27][KC][NF][32 lanes] x uint2
//   bias : COUT floats or nullptr
//   relu : clamp at 0
//   mask : if mask.p, zero every output whose mask element is not > 0
// grid: (bricks, batch); block 256; dynamic smem ConvCfg::SMEM
template <int CIN, int COUT, int MF>
__global__ void __launch_bounds__(256) k_conv3(Dims d, View in, const uint2* __restrict__ wf,
                                               const float* __restrict__ bias, View out, View mask,
                                               int relu) {
  using C = ConvCfg<CIN, COUT, MF>;
  extern __shared__ __align__(128) unsigned char conv_smem[];
  bf16* hb = reinterpret_cast<bf16*>(conv_smem);
  const int nbx = (d.X + 15) / 16, nby = (d.Y + C::BY - 1) / C::BY;
  int bi = blockIdx.x;
  const int bx = bi % nbx;
  bi /= nbx;
  const int by = bi % nby, bz = bi / nby;
  const int x0 = bx * 16, y0 = by * C::BY, z0 = bz * C::BZ;
  const long long b = blockIdx.y;

  load_halo<CIN, C::HX, C::HY, C::HZ, C::CSE>(d, in.p + b * in.bs + in.co, in.cs, x0, y0, z0, hb);
  cp_async_wait_all();
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float acc[C::MF][C::NF][4];
#pragma unroll
  for (int i = 0; i < C::MF; i++)
#pragma unroll
    for (int j = 0; j < C::NF; j++)
#pragma unroll
      for (int k = 0; k < 4; k++) acc[i][j][k] = 0.f;

  const uint32_t hbase = smem_u32addr(hb);
  // B fragments are loaded one k-chunk ahead of their use (register double
  // buffer), so the weight loads overlap the previous chunk's MMAs
  constexpr int NSTEP = 27 * C::KC;
  uint2 bnext[C::NF];
#pragma unroll
  for (int nf = 0; nf < C::NF; nf++) bnext[nf] = __ldg(&wf[nf * 32 + lane]);
  for (int off = 0; off < 27; off++) {
    const int dz = off / 9 - 1, dy = (off / 3) % 3 - 1, dx = off % 3 - 1;
#pragma unroll
    for (int kc = 0; kc < C::KC; kc++) {
      uint2 bw[C::NF];
#pragma unroll
      for (int nf = 0; nf < C::NF; nf++) bw[nf] = bnext[nf];
      const int step = off * C::KC + kc + 1;
      if (step < NSTEP) {
#pragma unroll
        for (int nf = 0; nf < C::NF; nf++) bnext[nf] = __ldg(&wf[(step * C::NF + nf) * 32 + lane]);
      }
#pragma unroll
      for (int mf = 0; mf < C::MF; mf++) {
        const int row = warp * C::MF + mf;
        const int ty = row % C::BY, tz = row / C::BY;
        const int h = ((tz + 1 + dz) * C::HY + (ty + 1 + dy)) * C::HX + 1 + dx + (lane & 15);
        uint32_t a[4];
        ldsm_x4(hbase + (uint32_t)(h * C::CSE + kc * 16 + (lane >> 4) * 8) * 2u, a);
#pragma unroll
        for (int nf = 0; nf < C::NF; nf++) mma16816(acc[mf][nf], a, bw[nf].x, bw[nf].y);
      }
    }
  }

  bf16* dst = out.p + b * out.bs + out.co;
  const bf16* msk = mask.p ? mask.p + b * mask.bs + mask.co : nullptr;
#pragma unroll
  for (int mf = 0; mf < C::MF; mf++) {
    const int row = warp * C::MF + mf;
    const int gy = y0 + row % C::BY, gz = z0 + row / C::BY;
    if (gy >= d.Y || gz >= d.Z) continue;
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int gx = x0 + (lane >> 2) + half * 8;
      if (gx >= d.X) continue;
      const long long cell = ((long long)gz * d.Y + gy) * d.X + gx;
#pragma unroll
      for (int nf = 0; nf < C::NF; nf++) {
        const int n = nf * 8 + (lane & 3) * 2;
        float v0 = acc[mf][nf][half * 2], v1 = acc[mf][nf][half * 2 + 1];
        if (bias) {
          v0 += bias[n];
          v1 += bias[n + 1];
        }
        if (relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (msk) {
          const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162*>(msk + cell * mask.cs + n);
          if (!(__low2float(m) > 0.f)) v0 = 0.f;
          if (!(__high2float(m) > 0.f)) v1 = 0.f;
        }
        *reinterpret_cast<__nv_bfloat162*>(dst + cell * out.cs + n) = __floats2bfloat162_rn(v0, v1);
      }
    }
  }
}

// ----------------------------------------------------------- weight gradient
// dW[off][cin][cout] = sum over samples and cells p of x(p + off)[cin] * g(p)[cout]
// Brick 16 x 4 x 2 cells; GO offsets per CTA group (grid.y groups), the CTA's
// (offset, 16-input-channel) combinations spread over its 8 warps.  Each CTA
// walks bricks blockIdx.x, +gridDim.x, ... and writes its partial sums to
// part[blockIdx.x][off][cin][cout] (every slot written by exactly one CTA).
template <int CIN, int COUT, int GO>
struct WgCfg {
  static constexpr int NF = COUT / 8;
  static constexpr int KC = CIN / 16;
  static constexpr int WARPS = 8;
  static constexpr int BY = 4, BZ = 2, ROWS = 8;
  static constexpr int HX = 18, HY = BY + 2, HZ = BZ + 2;
  static constexpr int HCELLS = HX * HY * HZ;
  static constexpr int CSX = CIN + 8, CSG = COUT + 8;
  static constexpr int COMBOS = GO * KC;
  static constexpr int CPW = (COMBOS + WARPS - 1) / WARPS;
  static constexpr int NGROUPS = (27 + GO - 1) / GO;
  static constexpr int XBYTES = HCELLS * CSX * 2;
  static constexpr int SMEM = XBYTES + 16 * ROWS * CSG * 2;
  static_assert(NF % 2 == 0, "output channels must be a multiple of 16");
};

template <int CIN, int COUT, int GO>
__global__ void __launch_bounds__(256) k_conv3_wgrad(Dims d, int batch, View x, View g, float* part) {
  using C = WgCfg<CIN, COUT, GO>;
  extern __shared__ __align__(128) unsigned char wg_smem[];
  bf16* xb = reinterpret_cast<bf16*>(wg_smem);
  bf16* gb = reinterpret_cast<bf16*>(wg_smem + C::XBYTES);
  const int nbx = (d.X + 15) / 16, nby = (d.Y + C::BY - 1) / C::BY, nbz = (d.Z + C::BZ - 1) / C::BZ;
  const int nbricks = nbx * nby * nbz;
  const long long nitems = (long long)nbricks * batch;
  const int group = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  float acc[C::CPW][C::NF][4];
#pragma unroll
  for (int i = 0; i < C::CPW; i++)
#pragma unroll
    for (int j = 0; j < C::NF; j++)
#pragma unroll
      for (int k = 0; k < 4; k++) acc[i][j][k] = 0.f;

  const uint32_t xbase = smem_u32addr(xb), gbase = smem_u32addr(gb);
  for (long long item = blockIdx.x; item < nitems; item += gridDim.x) {
    const long long b = item / nbricks;
    int bi = (int)(item % nbricks);
    const int bx = bi % nbx;
    bi /= nbx;
    const int by = bi % nby, bz = bi / nby;
    const int x0 = bx * 16, y0 = by * C::BY, z0 = bz * C::BZ;
    __syncthreads();  // the previous brick's shared-memory reads are done
    load_halo<CIN, C::HX, C::HY, C::HZ, C::CSX>(d, x.p + b * x.bs + x.co, x.cs, x0, y0, z0, xb);
    {
      constexpr int CH = COUT / 8;
      const bf16* gs = g.p + b * g.bs + g.co;
      for (int i = threadIdx.x; i < 16 * C::ROWS * CH; i += blockDim.x) {
        const int q = i % CH, c = i / CH;
        const int gx = x0 + (c & 15), gy = y0 + (c >> 4) % C::BY, gz = z0 + (c >> 4) / C::BY;
        const bool ok = gx < d.X && gy < d.Y && gz < d.Z;
        const long long cell = ok ? ((long long)gz * d.Y + gy) * d.X + gx : 0;
        cp_async16(smem_u32addr(gb + c * C::CSG + q * 8), gs + cell * g.cs + q * 8, ok ? 16 : 0);
      }
    }
    cp_async_wait_all();
    __syncthreads();

    for (int row = 0; row < C::ROWS; row++) {
      const int ty = row % C::BY, tz = row / C::BY;
      uint32_t bq[C::NF][2];
#pragma unroll
      for (int np = 0; np < C::NF / 2; np++) {
        const int cell = row * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;
        const int ch = (np * 2 + (lane >> 4)) * 8;
        uint32_t r[4];
        ldsm_x4_t(gbase + (uint32_t)(cell * C::CSG + ch) * 2u, r);
        bq[2 * np][0] = r[0];
        bq[2 * np][1] = r[1];
        bq[2 * np + 1][0] = r[2];
        bq[2 * np + 1][1] = r[3];
      }
#pragma unroll
      for (int j = 0; j < C::CPW; j++) {
        const int combo = warp + C::WARPS * j;
        if (combo >= C::COMBOS) continue;
        const int off = group * GO + combo / C::KC, mi = combo % C::KC;
        if (off >= 27) continue;
        const int dz = off / 9 - 1, dy = (off / 3) % 3 - 1, dx = off % 3 - 1;
        const int h = ((tz + 1 + dz) * C::HY + (ty + 1 + dy)) * C::HX + 1 + dx + (lane & 7) +
                      ((lane >> 4) & 1) * 8;
        const int cin = mi * 16 + ((lane >> 3) & 1) * 8;
        uint32_t a[4];
        ldsm_x4_t(xbase + (uint32_t)(h * C::CSX + cin) * 2u, a);
#pragma unroll
        for (int nf = 0; nf < C::NF; nf++) mma16816(acc[j][nf], a, bq[nf][0], bq[nf][1]);
      }
    }
  }

  float* dst = part + (size_t)blockIdx.x * 27 * CIN * COUT;
#pragma unroll
  for (int j = 0; j < C::CPW; j++) {
    const int combo = warp + C::WARPS * j;
    if (combo >= C::COMBOS) continue;
    const int off = group * GO + combo / C::KC, mi = combo % C::KC;
    if (off >= 27) continue;
    const int r0 = mi * 16 + (lane >> 2);
#pragma unroll
    for (int nf = 0; nf < C::NF; nf++) {
      const int n = nf * 8 + (lane & 3) * 2;
      float* o = dst + ((size_t)off * CIN + r0) * COUT + n;
      o[0] = acc[j][nf][0];
      o[1] = acc[j][nf][1];
      o[8 * COUT] = acc[j][nf][2];
      o[8 * COUT + 1] = acc[j][nf][3];
    }
  }
}

// out[i] (+)= sum over k < nparts of part[k*n + i], in order of k
__global__ void k_sum_parts(const float* part, int nparts, long long n, float* out, int accumulate) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < nparts; k++) s += part[(long long)k * n + i];
    out[i] = accumulate ? out[i] + s : s;
  }
}

// *acc += *v (a single-thread accumulation kept on the device)
__global__ void k_add_to_double(const float* v, double* acc) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *acc += (double)*v;
}

// per-block channel sums of g over every sample and cell: part[block][C]
__global__ void k_chan_sum(View g, int C, long long cells, int batch, float* part) {
  __shared__ float sh[256];
  const int R = blockDim.x / C;
  const int c = threadIdx.x % C, r = threadIdx.x / C;
  float s = 0.f;
  if (r < R) {
    const long long rows = cells * batch;
    for (long long i = (long long)blockIdx.x * R + r; i < rows; i += (long long)gridDim.x * R) {
      const long long b = i / cells, cell = i % cells;
      s += bf2f(g.p[b * g.bs + cell * g.cs + g.co + c]);
    }
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < C) {
    float t = 0.f;
    for (int k = 0; k < R; k++) t += sh[k * C + threadIdx.x];
    part[(long long)blockIdx.x * C + threadIdx.x] = t;
  }
}

// ------------------------------------------------------- weight re-layouts
// FP32 master W[27][cin][cout] -> B fragments of the forward convolution
__global__ void k_prep_fwd(const float* W, int cin, int cout, uint2* wf) {
  const int KC = cin / 16, NF = cout / 8;
  const int total = 27 * KC * NF * 32;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int lane = i % 32, nf = (i / 32) % NF, kc = (i / (32 * NF)) % KC, off = i / (32 * NF * KC);
    const int k0 = kc * 16 + (lane & 3) * 2, n = nf * 8 + (lane >> 2);
    const float* w = W + (size_t)off * cin * cout;
    wf[i] = make_uint2(pack_bf2(w[k0 * cout + n], w[(k0 + 1) * cout + n]),
                       pack_bf2(w[(k0 + 8) * cout + n], w[(k0 + 9) * cout + n]));
  }
}

// ... and of the input-gradient convolution: CIN' = cout, COUT' = cin,
// W'[off][co][ci] = W[26 - off][ci][co] (offsets mirrored)
__global__ void k_prep_bwd(const float* W, int cin, int cout, uint2* wf) {
  const int KC = cout / 16, NF = cin / 8;
  const int total = 27 * KC * NF * 32;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int lane = i % 32, nf = (i / 32) % NF, kc = (i / (32 * NF)) % KC, off = i / (32 * NF * KC);
    const int k0 = kc * 16 + (lane & 3) * 2, n = nf * 8 + (lane >> 2);
    const float* w = W + (size_t)(26 - off) * cin * cout;
    wf[i] = make_uint2(pack_bf2(w[n * cout + k0], w[n * cout + k0 + 1]),
                       pack_bf2(w[n * cout + k0 + 8], w[n * cout + k0 + 9]));
  }
}

// --------------------------------------------------------- pool / upsample
// 8 channels (16 bytes) per thread; fine grid = 2 x coarse grid on every axis
struct Chunk8 {
  float v[8];
};
__device__ __forceinline__ Chunk8 ld8(const bf16* p) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
  Chunk8 c;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    c.v[2 * k] = __low2float(h[k]);
    c.v[2 * k + 1] = __high2float(h[k]);
  }
  return c;
}
__device__ __forceinline__ void st8(bf16* p, const Chunk8& c) {
  uint4 u;
  u.x = pack_bf2(c.v[0], c.v[1]);
  u.y = pack_bf2(c.v[2], c.v[3]);
  u.z = pack_bf2(c.v[4], c.v[5]);
  u.w = pack_bf2(c.v[6], c.v[7]);
  *reinterpret_cast<uint4*>(p) = u;
}
__device__ __forceinline__ long long child_cell(const Dims& f, long long qc, const Dims& c, int k) {
  const int qx = (int)(qc % c.X), qy = (int)((qc / c.X) % c.Y), qz = (int)(qc / ((long long)c.X * c.Y));
  return ((long long)(2 * qz + (k >> 2)) * f.Y + (2 * qy + ((k >> 1) & 1))) * f.X + 2 * qx + (k & 1);
}
__device__ __forceinline__ long long parent_cell(const Dims& f, long long pc, const Dims& c) {
  const int px = (int)(pc % f.X), py = (int)((pc / f.X) % f.Y), pz = (int)(pc / ((long long)f.X * f.Y));
  return ((long long)(pz >> 1) * c.Y + (py >> 1)) * c.X + (px >> 1);
}

// out(coarse) = mean of the 8 children of in(fine)
__global__ void k_pool(Dims f, Dims c, int batch, int C, View in, View out) {
  const int CH = C / 8;
  const long long n = c.cells * CH * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(i % CH);
    const long long r = i / CH, b = r / c.cells, qc = r % c.cells;
    Chunk8 s;
#pragma unroll
    for (int k = 0; k < 8; k++) s.v[k] = 0.f;
    for (int k = 0; k < 8; k++) {
      const Chunk8 v = ld8(in.p + b * in.bs + child_cell(f, qc, c, k) * in.cs + in.co + q * 8);
#pragma unroll
      for (int e = 0; e < 8; e++) s.v[e] += v.v[e];
    }
#pragma unroll
    for (int e = 0; e < 8; e++) s.v[e] *= 0.125f;
    st8(out.p + b * out.bs + qc * out.cs + out.co + q * 8, s);
  }
}

// out(fine) = [mask > 0] * (g(coarse parent) / 8 + add(fine))
__global__ void k_pool_bwd(Dims f, Dims c, int batch, int C, View g, View add, View mask, View out) {
  const int CH = C / 8;
  const long long n = f.cells * CH * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(i % CH);
    const long long r = i / CH, b = r / f.cells, pc = r % f.cells;
    Chunk8 s = ld8(g.p + b * g.bs + parent_cell(f, pc, c) * g.cs + g.co + q * 8);
#pragma unroll
    for (int e = 0; e < 8; e++) s.v[e] *= 0.125f;
    if (add.p) {
      const Chunk8 a = ld8(add.p + b * add.bs + pc * add.cs + add.co + q * 8);
#pragma unroll
      for (int e = 0; e < 8; e++) s.v[e] += a.v[e];
    }
    if (mask.p) {
      const Chunk8 m = ld8(mask.p + b * mask.bs + pc * mask.cs + mask.co + q * 8);
#pragma unroll
      for (int e = 0; e < 8; e++)
        if (!(m.v[e] > 0.f)) s.v[e] = 0.f;
    }
    st8(out.p + b * out.bs + pc * out.cs + out.co + q * 8, s);
  }
}

// out(fine) = in(coarse parent)
__global__ void k_upsample(Dims f, Dims c, int batch, int C, View in, View out) {
  const int CH = C / 8;
  const long long n = f.cells * CH * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(i % CH);
    const long long r = i / CH, b = r / f.cells, pc = r % f.cells;
    const uint4 v =
        *reinterpret_cast<const uint4*>(in.p + b * in.bs + parent_cell(f, pc, c) * in.cs + in.co + q * 8);
    *reinterpret_cast<uint4*>(out.p + b * out.bs + pc * out.cs + out.co + q * 8) = v;
  }
}

// out(coarse) = [mask > 0] * sum of g over the 8 children
__global__ void k_upsample_bwd(Dims f, Dims c, int batch, int C, View g, View mask, View out) {
  const int CH = C / 8;
  const long long n = c.cells * CH * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(i % CH);
    const long long r = i / CH, b = r / c.cells, qc = r % c.cells;
    Chunk8 s;
#pragma unroll
    for (int k = 0; k < 8; k++) s.v[k] = 0.f;
    for (int k = 0; k < 8; k++) {
      const Chunk8 v = ld8(g.p + b * g.bs + child_cell(f, qc, c, k) * g.cs + g.co + q * 8);
#pragma unroll
      for (int e = 0; e < 8; e++) s.v[e] += v.v[e];
    }
    if (mask.p) {
      const Chunk8 m = ld8(mask.p + b * mask.bs + qc * mask.cs + mask.co + q * 8);
#pragma unroll
      for (int e = 0; e < 8; e++)
        if (!(m.v[e] > 0.f)) s.v[e] = 0.f;
    }
    st8(out.p + b * out.bs + qc * out.cs + out.co + q * 8, s);
  }
}

// ------------------------------------------------------------ output layer
// y = w[16] + sum_c w[c] x[c]   (1x1x1 convolution 16 -> 1, FP32 weights)
__global__ void k_out_fwd(long long cells, int batch, View x, const float* __restrict__ w, float* y) {
  const long long n = cells * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const bf16* p = x.p + (i / cells) * x.bs + (i % cells) * x.cs + x.co;
    const Chunk8 a = ld8(p), b = ld8(p + 8);
    float s = w[16];
#pragma unroll
    for (int e = 0; e < 8; e++) s += w[e] * a.v[e];
#pragma unroll
    for (int e = 0; e < 8; e++) s += w[8 + e] * b.v[e];
    y[i] = s;
  }
}

__device__ __forceinline__ bool interior(const Dims& d, long long cell) {
  const int x = (int)(cell % d.X), y = (int)((cell / d.X) % d.Y), z = (int)(cell / ((long long)d.X * d.Y));
  return x > 0 && x < d.X - 1 && y > 0 && y < d.Y - 1 && z > 0 && z < d.Z - 1;
}

template <int BLOCK>
__device__ __forceinline__ float block_sum_f(float v, float* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x == 0)
    for (int k = 0; k < BLOCK / 32; k++) t += sh[k];
  __syncthreads();
  return t;  // valid in thread 0
}

// squared error over interior cells; gy = d loss / d y with loss = sum / count
__global__ void __launch_bounds__(256) k_loss(Dims d, int batch, const float* y, const float* t, float* gy,
                                              float inv_count, float* part) {
  __shared__ float sh[8];
  const long long n = d.cells * batch;
  float s = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float g = 0.f;
    if (interior(d, i % d.cells)) {
      const float e = y[i] - t[i];
      s += e * e;
      g = 2.f * e * inv_count;
    }
    gy[i] = g;
  }
  const float tot = block_sum_f<256>(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// e = y - t on interior cells, 0 elsewhere
__global__ void k_err(Dims d, int batch, const float* y, const float* t, float* e) {
  const long long n = d.cells * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    e[i] = interior(d, i % d.cells) ? y[i] - t[i] : 0.f;
}

// Energy norm of the error, the quantity CG's error bound starts from:
// loss = (e^T A e + w e^T e) / count with A the 7-point operator of a closed
// box (diagonal = number of interior neighbours, -1 per interior neighbour);
// gy = 2 (A e + w e) / count.  e must be 0 outside the interior.
__global__ void __launch_bounds__(256) k_loss_energy(Dims d, int batch, const float* e, float* gy, float inv_count,
                                                     float w, float* part) {
  __shared__ float sh[8];
  const long long n = d.cells * batch;
  const long long sy = d.X, sz = (long long)d.X * d.Y;
  float s = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long cell = i % d.cells;
    const int x = (int)(cell % d.X), y = (int)((cell / d.X) % d.Y), z = (int)(cell / sz);
    float g = 0.f;
    if (x > 0 && x < d.X - 1 && y > 0 && y < d.Y - 1 && z > 0 && z < d.Z - 1) {
      const float ei = e[i];
      float q = 0.f;
      int cnt = 0;
      if (x > 1) { q -= e[i - 1]; cnt++; }
      if (x < d.X - 2) { q -= e[i + 1]; cnt++; }
      if (y > 1) { q -= e[i - sy]; cnt++; }
      if (y < d.Y - 2) { q -= e[i + sy]; cnt++; }
      if (z > 1) { q -= e[i - sz]; cnt++; }
      if (z < d.Z - 2) { q -= e[i + sz]; cnt++; }
      q += (float)cnt * ei;
      s += ei * q + w * ei * ei;
      g = 2.f * (q + w * ei) * inv_count;
    }
    gy[i] = g;
  }
  const float tot = block_sum_f<256>(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// output-layer backward: gx = [x > 0] * w * gy (BF16); per-block partial
// sums of dW (16) and db (1) in part[block][17]
__global__ void __launch_bounds__(256) k_out_bwd(long long cells, int batch, View x, const float* __restrict__ w,
                                                 const float* gy, View gx, float* part) {
  __shared__ float sh[8];
  float acc[17];
#pragma unroll
  for (int k = 0; k < 17; k++) acc[k] = 0.f;
  const long long n = cells * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / cells, cell = i % cells;
    const bf16* p = x.p + b * x.bs + cell * x.cs + x.co;
    const Chunk8 a = ld8(p), c = ld8(p + 8);
    const float g = gy[i];
    Chunk8 oa, oc;
#pragma unroll
    for (int e = 0; e < 8; e++) {
      acc[e] += a.v[e] * g;
      acc[8 + e] += c.v[e] * g;
      oa.v[e] = a.v[e] > 0.f ? w[e] * g : 0.f;
      oc.v[e] = c.v[e] > 0.f ? w[8 + e] * g : 0.f;
    }
    acc[16] += g;
    bf16* q = gx.p + b * gx.bs + cell * gx.cs + gx.co;
    st8(q, oa);
    st8(q + 8, oc);
  }
#pragma unroll
  for (int k = 0; k < 17; k++) {
    const float t = block_sum_f<256>(acc[k], sh);
    if (threadIdx.x == 0) part[(long long)blockIdx.x * 17 + k] = t;
  }
}

// ------------------------------------------------------------------ Adam
__global__ void k_adam(long long n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2,
                       float eps, float bc1, float bc2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// ------------------------------------------------------- network inputs
// 16-channel input: channel 0 = src value, channels 1..15 = 0
__global__ void k_input16(long long cells, int batch, const float* src, View xin) {
  const long long n = cells * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    bf16* q = xin.p + (i / cells) * xin.bs + (i % cells) * xin.cs + xin.co;
    uint4 u = make_uint4(pack_bf2(src[i], 0.f), 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(q) = u;
    *reinterpret_cast<uint4*>(q + 8) = make_uint4(0u, 0u, 0u, 0u);
  }
}

// training batch from the pair store: sample k of the batch is pair idx[k]
__global__ void k_gather_batch(long long cells, int batch, const bf16* in_store, const float* tgt_store,
                               const int* idx, float inv_scale, View xin, float* tgt) {
  const long long n = cells * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / cells, cell = i % cells;
    const long long src = (long long)idx[b] * cells + cell;
    bf16* q = xin.p + b * xin.bs + cell * xin.cs + xin.co;
    const float v = bf2f(in_store[src]);
    *reinterpret_cast<uint4*>(q) = make_uint4(pack_bf2(v, 0.f), 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(q + 8) = make_uint4(0u, 0u, 0u, 0u);
    tgt[i] = tgt_store[src] * inv_scale;
  }
}

// sum of squares of b over interior cells, per block (FP64)
template <typename T>
__global__ void __launch_bounds__(256) k_sumsq_interior(Dims d, const T* b, double* part) {
  __shared__ double sh[8];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.cells;
       i += (long long)gridDim.x * blockDim.x)
    if (interior(d, i)) {
      const double v = (double)b[i];
      s += v * v;
    }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < 8; k++) t += sh[k];
    part[blockIdx.x] = t;
  }
}

// scale[0] = rms over `count` interior cells (0 when the field is all zero)
// (one block of 256 threads: strided partial sums, then a fixed-order tree)
__global__ void __launch_bounds__(256) k_rms_scale(const double* part, int nparts, double count, float* scale) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int k = threadIdx.x; k < nparts; k += 256) s += part[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) scale[0] = (float)sqrt(sh[0] / count);
}

// network input from a right-hand side: interior b / scale, 0 elsewhere
template <typename T>
__global__ void k_input_from_rhs(Dims d, const T* b, const float* scale, View xin) {
  const float s = scale[0];
  const float inv = s > 0.f ? 1.f / s : 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.cells;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = interior(d, i) ? (float)b[i] * inv : 0.f;
    bf16* q = xin.p + i * xin.cs + xin.co;
    *reinterpret_cast<uint4*>(q) = make_uint4(pack_bf2(v, 0.f), 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(q + 8) = make_uint4(0u, 0u, 0u, 0u);
  }
}

// initial guess x = scale * c * y on interior cells (border left as is)
template <typename T>
__global__ void k_guess_from_output(Dims d, const float* y, const float* scale, float c, T* x) {
  const float s = scale[0] * c;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.cells;
       i += (long long)gridDim.x * blockDim.x)
    if (interior(d, i)) x[i] = (T)(s * y[i]);
}

// one (right-hand side, solution) pair into the store: b / s (BF16) and p / s
template <typename T>
__global__ void k_store_pair(Dims d, const T* b, const T* p, const float* scale, bf16* in_slot,
                             float* tgt_slot) {
  const float s = scale[0];
  const float inv = s > 0.f ? 1.f / s : 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.cells;
       i += (long long)gridDim.x * blockDim.x) {
    const bool in = interior(d, i);
    in_slot[i] = __float2bfloat16_rn(in ? (float)b[i] * inv : 0.f);
    tgt_slot[i] = in ? (float)p[i] * inv : 0.f;
  }
}

// r = b - A x on interior cells for a closed box (A: number of interior
// neighbours on the diagonal, -1 per interior neighbour), FP64 accumulation;
// 0 on the border
template <typename T>
__global__ void k_closed_box_residual(Dims d, const T* b, const T* x, float* r) {
  const long long sy = d.X, sz = (long long)d.X * d.Y;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.cells;
       i += (long long)gridDim.x * blockDim.x) {
    const int cx = (int)(i % d.X), cy = (int)((i / d.X) % d.Y), cz = (int)(i / sz);
    float v = 0.f;
    if (cx > 0 && cx < d.X - 1 && cy > 0 && cy < d.Y - 1 && cz > 0 && cz < d.Z - 1) {
      double s = 0.0;
      int cnt = 0;
      if (cx > 1) { s += (double)x[i - 1]; cnt++; }
      if (cx < d.X - 2) { s += (double)x[i + 1]; cnt++; }
      if (cy > 1) { s += (double)x[i - sy]; cnt++; }
      if (cy < d.Y - 2) { s += (double)x[i + sy]; cnt++; }
      if (cz > 1) { s += (double)x[i - sz]; cnt++; }
      if (cz < d.Z - 2) { s += (double)x[i + sz]; cnt++; }
      v = (float)((double)b[i] - ((double)cnt * (double)x[i] - s));
    }
    r[i] = v;
  }
}

// one correction pair into the store: r0 / s (BF16) and (p - p_prev) / s
template <typename T>
__global__ void k_store_correction(Dims d, const float* r0, const T* p, const float* p_prev,
                                   const float* scale, bf16* in_slot, float* tgt_slot) {
  const float s = scale[0];
  const float inv = s > 0.f ? 1.f / s : 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.cells;
       i += (long long)gridDim.x * blockDim.x) {
    const bool in = interior(d, i);
    in_slot[i] = __float2bfloat16_rn(in ? r0[i] * inv : 0.f);
    tgt_slot[i] = in ? ((float)p[i] - p_prev[i]) * inv : 0.f;
  }
}

// sum of squares of a float array, per block (FP64)
__global__ void __launch_bounds__(256) k_sumsq_f(long long n, const float* a, double* part) {
  __shared__ double sh[8];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = a[i];
    s += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < 8; k++) t += sh[k];
    part[blockIdx.x] = t;
  }
}

}  // namespace unet
}  // namespace plume
