// common.cuh -- device-side helpers shared by the plume kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace plume {

#define PL_GRID_STRIDE(i, n) \
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += blockDim.x * gridDim.x)

// The block a kernel body runs as: its index among the blocks that share one
// plume's work, and their count.  A launch for one plume passes
// {blockIdx.x, gridDim.x} (hw_blk); a batched launch over many plumes
// (batched.cu) gives each plume a contiguous range of the grid, so the same
// body serves both and visits the same elements per block for the same count.
struct Blk {
  int id, n;
};
__device__ inline Blk hw_blk() { return Blk{(int)blockIdx.x, (int)gridDim.x}; }
#define PL_BLK_STRIDE(i, count, blk) \
  for (int i = (blk).id * (int)blockDim.x + (int)threadIdx.x; i < (count); i += (int)blockDim.x * (blk).n)

// Grid geometry.  Index = x + y*X + z*X*Y (x fastest), the reference layout
// (src/geometry/FIELD_3D.h:54-57).  `wall` holds the six BC flags in the
// reference order front(z=0), back(z=Z-1), left(x=0), right(x=X-1),
// top(y=Y-1), bottom(y=0); 1 = obstacle slab (FLUID_3D_MIC.cpp:105-159).
struct Grid {
  int X, Y, Z;
  int slab;        // X*Y
  int N;           // X*Y*Z
  int nx, ny, nz;  // interior extents (X-2, Y-2, Z-2)
  int nint;        // nx*ny*nz
  int wall[6];
};

__host__ __device__ inline bool on_border(const Grid& g, int x, int y, int z) {
  return x == 0 || y == 0 || z == 0 || x == g.X - 1 || y == g.Y - 1 || z == g.Z - 1;
}

// Full-grid index of interior cell number i (interior cells enumerated x fastest).
__device__ inline int interior_cell(const Grid& g, int i, int& x, int& y, int& z) {
  const int t = i / g.nx;
  x = 1 + (i - t * g.nx);
  y = 1 + (t % g.ny);
  z = 1 + t / g.ny;
  return x + y * g.X + z * g.slab;
}

// Is the face neighbour of an interior cell an obstacle?  Only the wall slabs
// are obstacles, so the neighbour across a face is a wall exactly when the
// cell touches that face and the face's flag is set.
__device__ inline bool wall_xm(const Grid& g, int x) { return x == 1 && g.wall[2] == 1; }
__device__ inline bool wall_xp(const Grid& g, int x) { return x == g.X - 2 && g.wall[3] == 1; }
__device__ inline bool wall_ym(const Grid& g, int y) { return y == 1 && g.wall[5] == 1; }
__device__ inline bool wall_yp(const Grid& g, int y) { return y == g.Y - 2 && g.wall[4] == 1; }
__device__ inline bool wall_zm(const Grid& g, int z) { return z == 1 && g.wall[0] == 1; }
__device__ inline bool wall_zp(const Grid& g, int z) { return z == g.Z - 2 && g.wall[1] == 1; }

// Explicitly typed square root for the field type (the FP32 path must not
// widen to FP64).
__device__ inline float sqrt_t(float v) { return sqrtf(v); }
__device__ inline double sqrt_t(double v) { return sqrt(v); }

// Deterministic block reduction (fixed shuffle tree, fixed smem order).
template <typename A>
__device__ inline A warp_sum(A v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
template <typename A>
__device__ inline A warp_max(A v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    A w = __shfl_down_sync(0xffffffffu, v, o);
    v = (w > v) ? w : v;
  }
  return v;
}

// Sum over the block; result valid in thread 0.  `sh` needs blockDim/32 slots.
template <typename A>
__device__ inline A block_sum(A v, A* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  A r = 0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : A(0);
    r = warp_sum(r);
  }
  return r;
}
template <typename A>
__device__ inline A block_max(A v, A* sh, A ident) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  A r = ident;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : ident;
    r = warp_max(r);
  }
  return r;
}

// Block sum of per-thread T values with the warp-level tree in T and the
// warps' sums in double (result valid in thread 0).  For T = double it is
// block_sum; for float it keeps the shuffle tree off the FP64 pipe, which
// issues at 1/64 of the FP32 rate on this part.  (The CG dot products use
// DotAcc below instead.)
template <typename T>
__device__ inline double block_sum_w(T v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = (double)v;
  __syncthreads();
  double r = 0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;
}
// Compensated FP32 dot-product accumulation: algorithm Dot2 of Ogita, Rump and
// Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005).
// Each product a*b is split exactly into p + e by one FMA (TwoProduct) and p
// is added with Knuth's TwoSum, so the pair (s, c) holds the sum as if it had
// been accumulated in twice the working precision (about 48 significand
// bits), at a few FP32 operations per element instead of an FP64 operation.
// The _rn intrinsics keep the compiler from contracting or reassociating.
__device__ inline void ff_add(float& s, float& c, float p) {
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z)));
  s = t;
}
__device__ inline void ff_prod(float& s, float& c, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  ff_add(s, c, p);
  c = __fadd_rn(c, e);
}

// Per-thread dot-product accumulator of the CG reductions.  FP64 fields
// accumulate in FP64 in the plain order (bit-for-bit the serial expression
// r += a*b); FP32 fields use the compensated pair above, so the FP32 engine's
// dot products carry FP64-class precision.  block() sums over the block
// (result valid in thread 0); the float pairs stay pairs through the warp
// tree and become doubles per warp.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ void prod(double a, double b) { s += a * b; }
  __device__ double block(double* sh) { return block_sum_w(s, sh); }
};
template <>
struct DotAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ void prod(float a, float b) { ff_prod(s, c, a, b); }
  __device__ double block(double* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float s2 = __shfl_down_sync(0xffffffffu, s, o);
      const float c2 = __shfl_down_sync(0xffffffffu, c, o);
      ff_add(s, c, s2);
      c = __fadd_rn(c, c2);
    }
    __syncthreads();
    if (lane == 0) sh[wid] = (double)s + (double)c;
    __syncthreads();
    double r = 0;
    if (wid == 0) {
      r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
      r = warp_sum(r);
    }
    return r;
  }
};

template <typename T>
__device__ inline double block_max_w(T v, double* sh, double ident) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sh[wid] = (double)v;
  __syncthreads();
  double r = ident;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : ident;
    r = warp_max(r);
  }
  return r;
}

// SplitMix64 finaliser; identical integer recipe on host (oracle) and device.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Seeded plume source value 1 + noise*(2u - 1), u in [0,1) from (seed, step, cell).
__host__ __device__ inline double source_value(uint64_t seed, int32_t step, int64_t cell,
                                               double noise) {
  uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ull);
  h = mix64(h + (uint64_t)(uint32_t)step * 0xD1B54A32D192ED03ull);
  h = mix64(h + (uint64_t)cell);
  const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
#ifdef __CUDA_ARCH__
  // explicit rounding: no multiply-add contraction, same bits as the host
  return __dadd_rn(1.0, __dmul_rn(noise, __dadd_rn(__dmul_rn(2.0, u), -1.0)));
#else
  return 1.0 + noise * (2.0 * u - 1.0);
#endif
}

}  // namespace plume
