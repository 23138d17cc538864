// skew_kernels.cuh -- the PCG loop of FLUID_3D_MIC::solvePoisson
// (FLUID_3D_MIC.cpp:918-1015) as vector kernels on the skewed interior layout
// of the wavefront MIC sweeps (wave.cuh); threads run over the stored
// elements row by row, so loads and stores are contiguous; padding elements
// are kept at zero.
#pragma once
#include <type_traits>
#include "solver_kernels.cuh"
#include "wave.cuh"

namespace plume {

// Dot products accumulate per thread in DotAcc<T> (common.cuh): plain FP64 for
// FP64 fields; for FP32 fields a compensated FP32 pair (Dot2), which carries
// FP64-class precision at FP32 cost (GB300's FP64 rate is a small fraction of
// its FP32 rate, so one FP64 operation per element would bound these
// kernels).  Block and grid reductions run in FP64 in a fixed order.
// Stored element e -> interior cell (ix, iy, iz); false for padding.
__device__ inline bool skew_cell(const Skew& k, int e, int& ix, int& iy, int& iz) {
  iz = e / (int)k.plane;
  const int rem = e - iz * (int)k.plane;
  const int s = rem / k.W;
  ix = rem - s * k.W;
  iy = s - ix / k.C;
  return ix < k.nx && iy >= 0 && iy < k.ny;
}

__device__ inline int skew_at(const Skew& k, int ix, int iy, int iz) {
  return iz * (int)k.plane + (iy + ix / k.C) * k.W + ix;
}

// multA (FLUID_3D_MIC.cpp:811-822) at interior cell (ix,iy,iz) in skewed
// storage; neighbours outside the interior are border cells, which hold 0.
template <typename T>
__device__ inline T mult_a_skew(const Grid& g, const Skew& k, const T* v, int e, int ix, int iy,
                                int iz) {
  const int x = ix + 1, y = iy + 1, z = iz + 1;
  const T vxm = ix > 0 ? v[skew_at(k, ix - 1, iy, iz)] : T(0);
  const T vxp = ix + 1 < k.nx ? v[skew_at(k, ix + 1, iy, iz)] : T(0);
  const T vym = iy > 0 ? v[e - k.W] : T(0);
  const T vyp = iy + 1 < k.ny ? v[e + k.W] : T(0);
  const T vzm = iz > 0 ? v[e - (int)k.plane] : T(0);
  const T vzp = iz + 1 < k.nz ? v[e + (int)k.plane] : T(0);
  return adiag<T>(g, x, y, z) * v[e] + vxm * coef<T>(wall_xm(g, x)) + vxp * coef<T>(wall_xp(g, x)) +
         vym * coef<T>(wall_ym(g, y)) + vyp * coef<T>(wall_yp(g, y)) +
         vzm * coef<T>(wall_zm(g, z)) + vzp * coef<T>(wall_zp(g, z));
}

// mult_a_skew with every product and sum in FP64
template <typename T>
__device__ inline double mult_a_skew_d(const Grid& g, const Skew& k, const T* v, int e, int ix, int iy,
                                       int iz) {
  const int x = ix + 1, y = iy + 1, z = iz + 1;
  const double vxm = ix > 0 ? (double)v[skew_at(k, ix - 1, iy, iz)] : 0.0;
  const double vxp = ix + 1 < k.nx ? (double)v[skew_at(k, ix + 1, iy, iz)] : 0.0;
  const double vym = iy > 0 ? (double)v[e - k.W] : 0.0;
  const double vyp = iy + 1 < k.ny ? (double)v[e + k.W] : 0.0;
  const double vzm = iz > 0 ? (double)v[e - (int)k.plane] : 0.0;
  const double vzp = iz + 1 < k.nz ? (double)v[e + (int)k.plane] : 0.0;
  return adiag<double>(g, x, y, z) * (double)v[e] + vxm * coef<double>(wall_xm(g, x)) +
         vxp * coef<double>(wall_xp(g, x)) + vym * coef<double>(wall_ym(g, y)) +
         vyp * coef<double>(wall_yp(g, y)) + vzm * coef<double>(wall_zm(g, z)) +
         vzp * coef<double>(wall_zp(g, z));
}

// natural full grid -> skewed interior (padding zero)
template <typename S, typename T>
__device__ __forceinline__ void to_skew_body(Blk blk_, Grid g, Skew k, const S* nat, T* sk) {
  PL_BLK_STRIDE(e, (int)k.total, blk_) {
    int ix, iy, iz;
    T v = T(0);
    if (skew_cell(k, e, ix, iy, iz)) v = (T)nat[(ix + 1) + (iy + 1) * g.X + (iz + 1) * g.slab];
    sk[e] = v;
  }
}
template <typename S, typename T>
__global__ void k_to_skew(Grid g, Skew k, const S* nat, T* sk) {
  to_skew_body<S, T>(hw_blk(), g, k, nat, sk);
}

// The MIC(0) diagonal in the sweeps' skewed layout.  The exact (FP64) sweeps
// take P itself; the FP32 sweeps only ever multiply by P^2 (see sweep_cell),
// so for them the square is formed in FP64 and rounded once.
template <typename T>
__global__ void k_diag_to_skew(Grid g, Skew k, const double* P64, T* sk, int square) {
  const Blk b = hw_blk();
  PL_BLK_STRIDE(e, (int)k.total, b) {
    int ix, iy, iz;
    double v = 0.0;
    if (skew_cell(k, e, ix, iy, iz)) v = P64[(ix + 1) + (iy + 1) * g.X + (iz + 1) * g.slab];
    sk[e] = (T)(square ? v * v : v);
  }
}

// The FP32 forward sweep hands back w = P q (natural layout, in place); q
// itself is w / P, and zero where P is (those cells compute zero).
template <typename T>
__global__ void k_fwd_unscale(int n, const double* P64, T* w) {
  PL_GRID_STRIDE(i, n) {
    const double p = P64[i];
    w[i] = p != 0.0 ? (T)((double)w[i] / p) : T(0);
  }
}

// skewed interior -> natural full grid (interior cells only)
template <typename T>
__device__ __forceinline__ void from_skew_body(Blk blk_, Grid g, Skew k, const T* sk, T* nat) {
  PL_BLK_STRIDE(e, (int)k.total, blk_) {
    int ix, iy, iz;
    if (skew_cell(k, e, ix, iy, iz)) nat[(ix + 1) + (iy + 1) * g.X + (iz + 1) * g.slab] = sk[e];
  }
}
template <typename T>
__global__ void k_from_skew(Grid g, Skew k, const T* sk, T* nat) {
  from_skew_body<T>(hw_blk(), g, k, sk, nat);
}

// set-up part 1: r = b - A x, b.b
template <typename T>
__device__ __forceinline__ void cgs_init_body(Blk blk_, Grid g, Skew k, const T* b, const T* x, T* r,
                                              CgState* st, double* part, double tol, int max_iters,
                                              int criterion, int x_zero) {
  __shared__ double sh[32];
  DotAcc<T> bb;
  PL_BLK_STRIDE(e, (int)k.total, blk_) {
    int ix, iy, iz;
    T v = T(0);
    if (skew_cell(k, e, ix, iy, iz)) {
      const T bi = b[e];
      if (x_zero) {
        v = bi;  // the guess is zero: r = b exactly
      } else if (std::is_same<T, float>::value) {
        // FP32 fields: b - A x accumulated in FP64, so a large initial guess
        // (|x| ~ N^2 |b| for the smoothest modes) does not leave rounding
        // noise above the stop test in r; x = 0 gives r = b as before
        v = (T)((double)bi - mult_a_skew_d(g, k, x, e, ix, iy, iz));
      } else {
        v = bi - mult_a_skew(g, k, x, e, ix, iy, iz);
      }
      bb.prod(bi, bi);
    }
    r[e] = v;
  }
  const double s = bb.block(sh);
  if (threadIdx.x == 0) part[blk_.id] = s;
  if (arrive_last(&st->ticket[0], blk_.n)) {
    const double tot = sum_partials(part, sh, blk_.n);
    if (threadIdx.x == 0) {
      st->bb = tot;
      st->tol = tol;
      st->max_iters = max_iters;
      st->criterion = criterion;
      st->iter = 0;
      st->done = 0;
      st->converged = 0;
      st->broke = 0;
      st->wave_err = 0;
      st->ticket[0] = 0;
    }
  }
}
template <typename T>
__global__ void k_cgs_init(Grid g, Skew k, const T* b, const T* x, T* r, CgState* st, double* part,
                           double tol, int max_iters, int criterion, int x_zero) {
  cgs_init_body<T>(hw_blk(), g, k, b, x, r, st, part, tol, max_iters, criterion, x_zero);
}

// set-up part 2: d = z, deltaNew = r.z, loop entry test
template <typename T>
__device__ __forceinline__ void cgs_init2_body(Blk blk_, Skew k, const T* r, const T* z, T* d, CgState* st,
                                               double* part) {
  __shared__ double sh[32];
  DotAcc<T> rz, rr;
  PL_BLK_STRIDE(e, (int)k.total, blk_) {
    const T zi = z[e], ri = r[e];
    if (d) d[e] = zi;
    rz.prod(ri, zi);
    rr.prod(ri, ri);
  }
  const double s1 = rz.block(sh);
  if (threadIdx.x == 0) part[blk_.id] = s1;
  const double s2 = rr.block(sh);
  if (threadIdx.x == 0) part[blk_.n + blk_.id] = s2;
  if (arrive_last(&st->ticket[0], blk_.n)) {
    const double trz = sum_partials(part, sh, blk_.n);
    const double trr = sum_partials(part + blk_.n, sh, blk_.n);
    if (threadIdx.x == 0) {
      st->deltaNew = trz;
      st->rr = trr;
      st->beta = 0.0;  // the first direction is z itself
      if (st->wave_err) st->done = 3;
      if (st->criterion == 0) {
        st->maxR = 2.0 * st->tol;
        if (!(st->maxR > st->tol) || st->max_iters <= 0) st->done = st->done ? st->done : 1;
      } else {
        if (sqrt(trr) <= st->tol * sqrt(st->bb)) {
          st->done = st->done ? st->done : 1;
          st->converged = 1;
        }
        if (st->max_iters <= 0) st->done = st->done ? st->done : 1;
      }
      st->ticket[0] = 0;
    }
  }
}
template <typename T>
__global__ void k_cgs_init2(Skew k, const T* r, const T* z, T* d, CgState* st, double* part) {
  cgs_init2_body<T>(hw_blk(), k, r, z, d, st, part);
}

// ----------------------------------------------------- fused fast path
// Rows of the skewed layout are walked whole: thread (row, ix) with the row
// width W = 32*C known at compile time, so no per-element division.
template <int C>
struct SkewRows {
  static constexpr int W = 32 * C;
  static constexpr int RPB = (256 / W) > 0 ? (256 / W) : 1;  // rows per block pass
  static constexpr int THREADS = RPB * W;
};

// Iteration part 1 with the direction update folded in:
//   d = z + beta * d_old   (FLUID_3D_MIC.cpp:995-996, `_direction *= beta;
//                           _direction += _z`, same rounding order)
//   q = A d, d.q, alpha = deltaNew / d.q
// Each cell rebuilds its neighbours' new direction values instead of reading
// a separately written d, so the update costs no extra pass.  beta = 0 on the
// first iteration (d = z).  d is double-buffered: reads d_old, writes d_new.
template <typename T, int C>
__global__ void __launch_bounds__(SkewRows<C>::THREADS) k_cgs_spmv_dir(Grid g, Skew k, const T* z,
                                                                        const T* d_old, T* d_new,
                                                                        T* q, CgState* st,
                                                                        double* part) {
  if (st->done) return;
  __shared__ double sh[32];
  constexpr int W = SkewRows<C>::W, RPB = SkewRows<C>::RPB;
  const int ix = threadIdx.x % W, lr = threadIdx.x / W;
  const int lb = ix / C, jb = ix - lb * C;
  const T beta = (T)st->beta;
  const int plane = (int)k.plane;
  const int nrows = k.nz * k.R;
  DotAcc<T> dq;
  for (int row = blockIdx.x * RPB + lr; row < nrows; row += gridDim.x * RPB) {
    const int iz = row / k.R;
    const int sr = row - iz * k.R;
    const int iy = sr - lb;
    const int e = row * W + ix;
    T dn = T(0), qq = T(0);
    if (ix < k.nx && iy >= 0 && iy < k.ny) {
      const int x = ix + 1, y = iy + 1, zz = iz + 1;
      dn = d_old[e] * beta + z[e];
      const T vxm = ix > 0 ? (jb > 0 ? d_old[e - 1] * beta + z[e - 1]
                                     : d_old[e - W - 1] * beta + z[e - W - 1])
                           : T(0);
      const T vxp = ix + 1 < k.nx ? (jb < C - 1 ? d_old[e + 1] * beta + z[e + 1]
                                                : d_old[e + W + 1] * beta + z[e + W + 1])
                                  : T(0);
      const T vym = iy > 0 ? d_old[e - W] * beta + z[e - W] : T(0);
      const T vyp = iy + 1 < k.ny ? d_old[e + W] * beta + z[e + W] : T(0);
      const T vzm = iz > 0 ? d_old[e - plane] * beta + z[e - plane] : T(0);
      const T vzp = iz + 1 < k.nz ? d_old[e + plane] * beta + z[e + plane] : T(0);
      qq = adiag<T>(g, x, y, zz) * dn + vxm * coef<T>(wall_xm(g, x)) + vxp * coef<T>(wall_xp(g, x)) +
           vym * coef<T>(wall_ym(g, y)) + vyp * coef<T>(wall_yp(g, y)) +
           vzm * coef<T>(wall_zm(g, zz)) + vzp * coef<T>(wall_zp(g, zz));
      dq.prod(dn, qq);
    }
    d_new[e] = dn;
    q[e] = qq;
  }
  const double sblk = dq.block(sh);
  if (threadIdx.x == 0) part[blockIdx.x] = sblk;
  if (arrive_last(&st->ticket[0])) {
    const double t = sum_partials(part, sh);
    if (threadIdx.x == 0) {
      st->dq = t;
      if (fabs(t) > 0.0) {
        st->alpha = st->deltaNew / t;
      } else {  // "PCG alpha broke down! Bailing." (FLUID_3D_MIC.cpp:962-969)
        st->done = 1;
        st->broke = 1;
      }
      st->ticket[0] = 0;
    }
  }
}

// The same fused direction update + SpMV with the row width W = 32*C read at
// run time (the batched launch covers plumes of several widths in one grid):
// blockDim.x / W rows per block pass (blockDim.x >= W), threads past them
// idle.  Per cell the expression of k_cgs_spmv_dir.
template <typename T>
__device__ __forceinline__ void cgs_spmv_dir_rows_body(Blk blk_, Grid g, Skew k, const T* z, const T* d_old,
                                                       T* d_new, T* q, CgState* st, double* part) {
  if (st->done) return;
  __shared__ double sh[32];
  const int W = k.W, C = k.C;
  const int rpb = (int)blockDim.x / W;
  const int lr = (int)threadIdx.x / W, ix = (int)threadIdx.x - lr * W;
  const int lb = ix / C, jb = ix - lb * C;
  const T beta = (T)st->beta;
  const int plane = (int)k.plane;
  const int nrows = k.nz * k.R;
  DotAcc<T> dq;
  if (lr < rpb) {
    for (int row = blk_.id * rpb + lr; row < nrows; row += blk_.n * rpb) {
      const int iz = row / k.R;
      const int sr = row - iz * k.R;
      const int iy = sr - lb;
      const int e = row * W + ix;
      T dn = T(0), qq = T(0);
      if (ix < k.nx && iy >= 0 && iy < k.ny) {
        const int x = ix + 1, y = iy + 1, zz = iz + 1;
        dn = d_old[e] * beta + z[e];
        const T vxm = ix > 0 ? (jb > 0 ? d_old[e - 1] * beta + z[e - 1]
                                       : d_old[e - W - 1] * beta + z[e - W - 1])
                             : T(0);
        const T vxp = ix + 1 < k.nx ? (jb < C - 1 ? d_old[e + 1] * beta + z[e + 1]
                                                  : d_old[e + W + 1] * beta + z[e + W + 1])
                                    : T(0);
        const T vym = iy > 0 ? d_old[e - W] * beta + z[e - W] : T(0);
        const T vyp = iy + 1 < k.ny ? d_old[e + W] * beta + z[e + W] : T(0);
        const T vzm = iz > 0 ? d_old[e - plane] * beta + z[e - plane] : T(0);
        const T vzp = iz + 1 < k.nz ? d_old[e + plane] * beta + z[e + plane] : T(0);
        qq = adiag<T>(g, x, y, zz) * dn + vxm * coef<T>(wall_xm(g, x)) + vxp * coef<T>(wall_xp(g, x)) +
             vym * coef<T>(wall_ym(g, y)) + vyp * coef<T>(wall_yp(g, y)) +
             vzm * coef<T>(wall_zm(g, zz)) + vzp * coef<T>(wall_zp(g, zz));
        dq.prod(dn, qq);
      }
      d_new[e] = dn;
      q[e] = qq;
    }
  }
  const double sblk = dq.block(sh);
  if (threadIdx.x == 0) part[blk_.id] = sblk;
  if (arrive_last(&st->ticket[0], blk_.n)) {
    const double t = sum_partials(part, sh, blk_.n);
    if (threadIdx.x == 0) {
      st->dq = t;
      if (fabs(t) > 0.0) {
        st->alpha = st->deltaNew / t;
      } else {  // "PCG alpha broke down! Bailing." (FLUID_3D_MIC.cpp:962-969)
        st->done = 1;
        st->broke = 1;
      }
      st->ticket[0] = 0;
    }
  }
}

// The fused direction update + SpMV marching along z.  A tile is `rpb` rows
// (blockDim.x / W of them) of the plane layout times `zc` planes; each thread
// owns one (row, column) position of the tile and walks it down the planes,
// keeping the direction values of the planes below, at and above in
// registers, so a cell's z neighbours cost nothing and its wall coefficients,
// x-neighbour offsets and validity are worked out once per tile instead of
// once per cell.  Per cell the expression of k_cgs_spmv_dir (same order).
// Tiles are handed to the plume's blocks round-robin.
template <typename T>
__device__ __forceinline__ void cgs_spmv_dir_march_body(Blk blk_, Grid g, Skew k, const T* z, const T* d_old,
                                                        T* d_new, T* q, CgState* st, double* part, int zc) {
  if (st->done) return;
  __shared__ double sh[32];
  const int W = k.W, C = k.C;
  const int rpb = (int)blockDim.x / W;
  const int lr = (int)threadIdx.x / W, ix = (int)threadIdx.x - lr * W;
  const int lb = ix / C, jb = ix - lb * C;
  const T beta = (T)st->beta;
  const int plane = (int)k.plane;
  const int nrg = (k.R + rpb - 1) / rpb, nzc = (k.nz + zc - 1) / zc;
  const int ntiles = nrg * nzc;
  // per-thread constants of the x direction
  const int x = ix + 1;
  const bool hxm = ix > 0, hxp = ix + 1 < k.nx;
  const int oxm = jb > 0 ? -1 : -W - 1, oxp = jb < C - 1 ? 1 : W + 1;
  const T cxm = coef<T>(wall_xm(g, x)), cxp = coef<T>(wall_xp(g, x));
  DotAcc<T> dq;
  if (lr < rpb) {
    for (int tile = blk_.id; tile < ntiles; tile += blk_.n) {
      const int rg = tile % nrg, zi = tile / nrg;
      const int s = rg * rpb + lr;
      if (s >= k.R) continue;
      const int z0 = zi * zc, z1 = min(z0 + zc, k.nz);
      const int iy = s - lb;
      const bool valid = ix < k.nx && iy >= 0 && iy < k.ny;
      int e = z0 * plane + s * W + ix;
      if (!valid) {  // padding stays zero
        for (int iz = z0; iz < z1; iz++, e += plane) {
          d_new[e] = T(0);
          q[e] = T(0);
        }
        continue;
      }
      const int y = iy + 1;
      const bool hym = iy > 0, hyp = iy + 1 < k.ny;
      const T cym = coef<T>(wall_ym(g, y)), cyp = coef<T>(wall_yp(g, y));
      // the diagonal's x and y part (counts of open neighbours: exact in T,
      // so the sum equals adiag's whatever the order)
      const T axy = T((wall_xp(g, x) ? 0 : 1) + (wall_xm(g, x) ? 0 : 1) + (wall_yp(g, y) ? 0 : 1) +
                      (wall_ym(g, y) ? 0 : 1));
      auto dn = [&](int i) { return d_old[i] * beta + z[i]; };
      T dprev = z0 > 0 ? dn(e - plane) : T(0);
      T dcur = dn(e);
#pragma unroll 2
      for (int iz = z0; iz < z1; iz++, e += plane) {
        const int zz = iz + 1;
        const T dnext = iz + 1 < k.nz ? dn(e + plane) : T(0);
        const T vxm = hxm ? dn(e + oxm) : T(0);
        const T vxp = hxp ? dn(e + oxp) : T(0);
        const T vym = hym ? dn(e - W) : T(0);
        const T vyp = hyp ? dn(e + W) : T(0);
        const T vzm = iz > 0 ? dprev : T(0);
        const bool wzm = wall_zm(g, zz), wzp = wall_zp(g, zz);
        const T diag = axy + T((wzp ? 0 : 1) + (wzm ? 0 : 1));
        const T qq = diag * dcur + vxm * cxm + vxp * cxp + vym * cym + vyp * cyp + vzm * coef<T>(wzm) +
                     dnext * coef<T>(wzp);
        dq.prod(dcur, qq);
        d_new[e] = dcur;
        q[e] = qq;
        dprev = dcur;
        dcur = dnext;
      }
    }
  }
  const double sblk = dq.block(sh);
  if (threadIdx.x == 0) part[blk_.id] = sblk;
  if (arrive_last(&st->ticket[0], blk_.n)) {
    const double t = sum_partials(part, sh, blk_.n);
    if (threadIdx.x == 0) {
      st->dq = t;
      if (fabs(t) > 0.0) {
        st->alpha = st->deltaNew / t;
      } else {  // "PCG alpha broke down! Bailing." (FLUID_3D_MIC.cpp:962-969)
        st->done = 1;
        st->broke = 1;
      }
      st->ticket[0] = 0;
    }
  }
}
template <typename T>
__global__ void __launch_bounds__(256, 4) k_cgs_spmv_dir_march(Grid g, Skew k, const T* z, const T* d_old, T* d_new,
                                                            T* q, CgState* st, double* part, int zc) {
  cgs_spmv_dir_march_body<T>(hw_blk(), g, k, z, d_old, d_new, q, st, part, zc);
}

// 16-byte vector type of T
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  typedef float4 type;
  static constexpr int n = 4;
};
template <>
struct Vec16<double> {
  typedef double2 type;
  static constexpr int n = 2;
};
template <typename T>
__device__ inline T vget(const typename Vec16<T>::type& v, int i);
template <>
__device__ inline float vget<float>(const float4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}
template <>
__device__ inline double vget<double>(const double2& v, int i) {
  return i == 0 ? v.x : v.y;
}
template <typename T>
__device__ inline void vset(typename Vec16<T>::type& v, int i, T x);
template <>
__device__ inline void vset<float>(float4& v, int i, float x) {
  if (i == 0) v.x = x; else if (i == 1) v.y = x; else if (i == 2) v.z = x; else v.w = x;
}
template <>
__device__ inline void vset<double>(double2& v, int i, double x) {
  if (i == 0) v.x = x; else v.y = x;
}

// k_cgs_spmv_dir on 16-byte groups: a thread takes NV consecutive values of
// one lane's segment of a row (4 FP32 or 2 FP64 cells; C % NV == 0, so a group
// never straddles two lanes) and loads the group, its y and z neighbour
// groups as vectors; the x neighbours inside the group come from registers,
// the two at its ends as scalars (the previous or next lane's cell sits one
// row up or down in the skewed layout).  Each cell evaluates the same
// expression as k_cgs_spmv_dir (bit for bit in FP64, which is compiled
// without multiply-add contraction); the order in which d.q is summed
// differs.
template <typename T, int C>
__global__ void __launch_bounds__(kRedThreads) k_cgs_spmv_dir_v(Grid g, Skew k, const T* z, const T* d_old,
                                                                T* d_new, T* q, CgState* st, double* part) {
  if (st->done) return;
  typedef typename Vec16<T>::type V;
  constexpr int NV = Vec16<T>::n;
  constexpr int W = 32 * C, GPR = W / NV;  // groups per row
  static_assert(C % NV == 0, "a group must lie in one lane's segment");
  __shared__ double sh[32];
  const T beta = (T)st->beta;
  const int plane = (int)k.plane;
  const int ngroups = k.nz * k.R * GPR;
  DotAcc<T> dq;
  PL_GRID_STRIDE(gi, ngroups) {
    const int row = gi / GPR;
    const int ix0 = (gi - row * GPR) * NV;
    const int lane = ix0 / C, jb0 = ix0 - lane * C;
    const int iz = row / k.R;
    const int iy = row - iz * k.R - lane;
    const int e0 = row * W + ix0;
    V dnv, qv;
    if (iy >= 0 && iy < k.ny && ix0 < k.nx) {
      const int y = iy + 1, zz = iz + 1;
      auto dirv = [&](int e) {  // z + beta d_old at e, as a vector
        const V a = *reinterpret_cast<const V*>(z + e), b = *reinterpret_cast<const V*>(d_old + e);
        V r;
#pragma unroll
        for (int j = 0; j < NV; j++) vset<T>(r, j, vget<T>(b, j) * beta + vget<T>(a, j));
        return r;
      };
      const V dc = dirv(e0);
      const V dym = iy > 0 ? dirv(e0 - W) : V{};
      const V dyp = iy + 1 < k.ny ? dirv(e0 + W) : V{};
      const V dzm = iz > 0 ? dirv(e0 - plane) : V{};
      const V dzp = iz + 1 < k.nz ? dirv(e0 + plane) : V{};
      // x neighbours at the group's ends
      const int el = jb0 > 0 ? e0 - 1 : e0 - W - 1;
      const int er = jb0 + NV < C ? e0 + NV : e0 + NV - 1 + W + 1;
      const T xl = ix0 > 0 ? d_old[el] * beta + z[el] : T(0);
      const T xr = ix0 + NV < k.nx ? d_old[er] * beta + z[er] : T(0);
#pragma unroll
      for (int j = 0; j < NV; j++) {
        const int ix = ix0 + j, x = ix + 1;
        T dn = T(0), qq = T(0);
        if (ix < k.nx) {
          dn = vget<T>(dc, j);
          const T vxm = ix > 0 ? (j > 0 ? vget<T>(dc, j - 1) : xl) : T(0);
          const T vxp = ix + 1 < k.nx ? (j + 1 < NV ? vget<T>(dc, j + 1) : xr) : T(0);
          const T vym = iy > 0 ? vget<T>(dym, j) : T(0);
          const T vyp = iy + 1 < k.ny ? vget<T>(dyp, j) : T(0);
          const T vzm = iz > 0 ? vget<T>(dzm, j) : T(0);
          const T vzp = iz + 1 < k.nz ? vget<T>(dzp, j) : T(0);
          qq = adiag<T>(g, x, y, zz) * dn + vxm * coef<T>(wall_xm(g, x)) + vxp * coef<T>(wall_xp(g, x)) +
               vym * coef<T>(wall_ym(g, y)) + vyp * coef<T>(wall_yp(g, y)) +
               vzm * coef<T>(wall_zm(g, zz)) + vzp * coef<T>(wall_zp(g, zz));
          dq.prod(dn, qq);
        }
        vset<T>(dnv, j, dn);
        vset<T>(qv, j, qq);
      }
    } else {
#pragma unroll
      for (int j = 0; j < NV; j++) {
        vset<T>(dnv, j, T(0));
        vset<T>(qv, j, T(0));
      }
    }
    *reinterpret_cast<V*>(d_new + e0) = dnv;
    *reinterpret_cast<V*>(q + e0) = qv;
  }
  const double sblk = dq.block(sh);
  if (threadIdx.x == 0) part[blockIdx.x] = sblk;
  if (arrive_last(&st->ticket[0])) {
    const double t = sum_partials(part, sh);
    if (threadIdx.x == 0) {
      st->dq = t;
      if (fabs(t) > 0.0) {
        st->alpha = st->deltaNew / t;
      } else {  // "PCG alpha broke down! Bailing." (FLUID_3D_MIC.cpp:962-969)
        st->done = 1;
        st->broke = 1;
      }
      st->ticket[0] = 0;
    }
  }
}

// Iteration part 2, vectorised: x += alpha d, r -= alpha q, signed max(r), r.r
// (the PCG loop of FLUID_3D_MIC::solvePoisson, FLUID_3D_MIC.cpp:951-1013)
template <typename T>
__device__ __forceinline__ void cgs_axpy_v_body(Blk blk_, Skew k, const T* d, const T* q, T* x, T* r,
                                                CgState* st, double* part) {
  if (st->done) return;
  typedef typename Vec16<T>::type V;
  constexpr int NV = Vec16<T>::n;
  __shared__ double sh[32];
  const T alpha = (T)st->alpha;
  T mx = T(-3.0e38);
  DotAcc<T> rr;
  const int nvec = (int)(k.total / NV);
  const V* dv = reinterpret_cast<const V*>(d);
  const V* qv = reinterpret_cast<const V*>(q);
  V* xv = reinterpret_cast<V*>(x);
  V* rv = reinterpret_cast<V*>(r);
  PL_BLK_STRIDE(i, nvec, blk_) {
    const V dd = dv[i], qq = qv[i];
    V xx = xv[i], ri = rv[i];
#pragma unroll
    for (int c = 0; c < NV; c++) {
      vset<T>(xx, c, vget<T>(xx, c) + alpha * vget<T>(dd, c));
      const T rn = vget<T>(ri, c) + (-alpha) * vget<T>(qq, c);
      vset<T>(ri, c, rn);
      mx = (rn > mx) ? rn : mx;
      rr.prod(rn, rn);
    }
    xv[i] = xx;
    rv[i] = ri;
  }
  const double s1 = block_max_w(mx, sh, -1.0e308);
  if (threadIdx.x == 0) part[blk_.id] = s1;
  const double s2 = rr.block(sh);
  if (threadIdx.x == 0) part[blk_.n + blk_.id] = s2;
  if (arrive_last(&st->ticket[0], blk_.n)) {
    const double tm = max_partials(part, sh, blk_.n);
    const double trr = sum_partials(part + blk_.n, sh, blk_.n);
    if (threadIdx.x == 0) {
      st->oldMaxR = st->maxR;
      st->maxR = tm > 0.0 ? tm : 0.0;  // FIELD_3D::max starts at a border cell (0)
      st->rr = trr;
      if (st->criterion == 1 && sqrt(trr) <= st->tol * sqrt(st->bb)) {
        st->iter += 1;
        st->done = 1;
        st->converged = 1;
      }
      st->ticket[0] = 0;
    }
  }
}
template <typename T>
__global__ void k_cgs_axpy_v(Skew k, const T* d, const T* q, T* x, T* r, CgState* st, double* part) {
  cgs_axpy_v_body<T>(hw_blk(), k, d, q, x, r, st, part);
}

// Iteration part 3, vectorised: deltaNew = r.z, beta, exit tests
template <typename T>
__device__ __forceinline__ void cgs_rz_v_body(Blk blk_, Skew k, const T* r, const T* z, CgState* st,
                                              double* part) {
  if (st->done) return;
  typedef typename Vec16<T>::type V;
  constexpr int NV = Vec16<T>::n;
  __shared__ double sh[32];
  DotAcc<T> rz;
  const int nvec = (int)(k.total / NV);
  const V* rv = reinterpret_cast<const V*>(r);
  const V* zv = reinterpret_cast<const V*>(z);
  PL_BLK_STRIDE(i, nvec, blk_) {
    const V a = rv[i], b = zv[i];
#pragma unroll
    for (int c = 0; c < NV; c++) rz.prod(vget<T>(a, c), vget<T>(b, c));
  }
  const double s = rz.block(sh);
  if (threadIdx.x == 0) part[blk_.id] = s;
  if (arrive_last(&st->ticket[0], blk_.n)) {
    const double t = sum_partials(part, sh, blk_.n);
    if (threadIdx.x == 0) {
      st->deltaOld = st->deltaNew;
      st->deltaNew = t;
      st->beta = t / st->deltaOld;
      st->iter += 1;
      if (st->wave_err) st->done = 3;
      if (st->criterion == 0) {
        const double relative = fabs((st->maxR - st->oldMaxR) / st->oldMaxR);
        if (relative < 1e-7) st->done = st->done ? st->done : 2;  // stagnation bail
        if (!(st->maxR > st->tol)) st->converged = 1;
      }
      if (st->converged || st->iter >= st->max_iters) st->done = st->done ? st->done : 1;
      st->ticket[0] = 0;
    }
  }
}
template <typename T>
__global__ void k_cgs_rz_v(Skew k, const T* r, const T* z, CgState* st, double* part) {
  cgs_rz_v_body<T>(hw_blk(), k, r, z, st, part);
}

// Flexible CG, iteration part 3 (Notay, "Flexible conjugate gradients",
// SIAM J. Sci. Comput. 22(4), 2000: FCG(1)).  After z = M(r) with a
// preconditioner M that may change from one application to the next (the
// network), the next direction d' = z + beta d is made A-orthogonal to the
// last one: beta = -(z.q) / (d.q) with q = A d of the iteration that just
// ended (st->dq).  deltaNew = d'.r = z.r + beta (d.r), so that the next
// k_cgs_spmv_dir takes alpha = d'.r / d'.q, the exact line search along d',
// which never increases the A-norm error whatever M returned.  With a fixed
// SPD M and exact arithmetic d.r = 0 and this is the PCG iteration.  The
// exit tests are those of k_cgs_rz_v.
template <typename T>
__global__ void k_cgs_rz_fcg(Skew k, const T* r, const T* z, const T* q, const T* d, CgState* st,
                             double* part) {
  if (st->done) return;
  typedef typename Vec16<T>::type V;
  constexpr int NV = Vec16<T>::n;
  __shared__ double sh[32];
  DotAcc<T> zr, zq, dr;
  const int nvec = (int)(k.total / NV);
  const V* rv = reinterpret_cast<const V*>(r);
  const V* zv = reinterpret_cast<const V*>(z);
  const V* qv = reinterpret_cast<const V*>(q);
  const V* dv = reinterpret_cast<const V*>(d);
  PL_GRID_STRIDE(i, nvec) {
    const V a = rv[i], b = zv[i], c = qv[i], e = dv[i];
#pragma unroll
    for (int j = 0; j < NV; j++) {
      zr.prod(vget<T>(b, j), vget<T>(a, j));
      zq.prod(vget<T>(b, j), vget<T>(c, j));
      dr.prod(vget<T>(e, j), vget<T>(a, j));
    }
  }
  const double s1 = zr.block(sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s1;
  const double s2 = zq.block(sh);
  if (threadIdx.x == 0) part[kRedBlocks + blockIdx.x] = s2;
  const double s3 = dr.block(sh);
  if (threadIdx.x == 0) part[2 * kRedBlocks + blockIdx.x] = s3;
  if (arrive_last(&st->ticket[0])) {
    const double tzr = sum_partials(part, sh);
    const double tzq = sum_partials(part + kRedBlocks, sh);
    const double tdr = sum_partials(part + 2 * kRedBlocks, sh);
    if (threadIdx.x == 0) {
      const double beta = st->dq != 0.0 ? -tzq / st->dq : 0.0;
      st->deltaOld = st->deltaNew;
      st->deltaNew = tzr + beta * tdr;
      st->beta = beta;
      st->iter += 1;
      if (st->wave_err) st->done = 3;
      if (st->criterion == 0) {
        const double relative = fabs((st->maxR - st->oldMaxR) / st->oldMaxR);
        if (relative < 1e-7) st->done = st->done ? st->done : 2;
        if (!(st->maxR > st->tol)) st->converged = 1;
      }
      if (st->converged || st->iter >= st->max_iters) st->done = st->done ? st->done : 1;
      st->ticket[0] = 0;
    }
  }
}

}  // namespace plume
